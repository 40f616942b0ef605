// Vertex-phase derivatives of the triangle form factor (device math of the
// triangle adjoint, shared with host-side numerical checks).
#pragma once
#include "dfmath.cuh"

namespace pi {

// A_tri = -2 gamma F with gamma = khat . S and F = e[pa, pb, pc] (second
// divided difference of e^{iz} at the vertex phases).  With D_v = dF/dp_v =
// e[.., p_v, p_v, ..] (one node repeated) and dp_v/dv = k:
//   dA/dv = -2 ( grad_v(gamma) F + gamma k D_v ),
// grad_v0 gamma = khat x (e2 - e1)/2, grad_v1 gamma = -khat x e2/2,
// grad_v2 gamma = khat x e1/2 (reference formula,
// cpp/src/dof/triangle_mesh_dof.cpp:119-133).  D_a + D_b + D_c = i F.
//
// Small spread (D < 2): expansion about the centroid phase pm,
//   F   = e^{i pm} sum_m i^{m+2} h_m / (m+2)!,
//   D_v = e^{i pm} sum_m i^{m+3} h_m^(v) / (m+3)!,  h_m^(v) = h_m + d_v h_{m-1}^(v),
// truncated after m = 12.
// Large spread: with (P, Q) the pair with the largest gap, R the middle
// vertex, and G(h) = (e^{ih}-1-ih)/h^2,
//   f[u,u,v] = e^{iu} G(v-u),
//   D_Q = (f[R,Q,Q] - F) / (Q-P),  D_P = (F - f[P,P,R]) / (Q-P),
//   D_R = i F - D_P - D_Q.
struct TriDer { cf F, Da, Db, Dc; };

__device__ __forceinline__ cf imul(cf a) { return {-a.im, a.re}; }  // i a

// Terms up to h_MM: MM = 12 for k sp < 2; MM = 8 where k |e|max < 1 (|e|max
// the longest edge), where the dropped terms of F, D_b, D_c stay below 1e-8 of
// the leading ones (FP64 evaluation over icosphere and box triangles at the
// bound).
template <int MM>
__device__ __forceinline__ TriDer tri_series_der(cf P, float al, float be) {
  static_assert(MM >= 4 && MM <= 12, "tri_series_der: order out of range");
  const float da = -(al + be) * (1.0f / 3.0f);
  const float db = al + da, dc = be + da;
  const float me2 = 0.5f * (da * da + db * db + dc * dc);
  const float e3 = da * db * dc;
  float h[13];
  h[0] = 1.f; h[1] = 0.f; h[2] = me2; h[3] = e3;
#pragma unroll
  for (int m = 4; m <= MM; ++m) h[m] = fmaf(me2, h[m - 2], e3 * h[m - 3]);
  // i^{m+2}/(m+2)!  and  i^{m+3}/(m+3)!  split into real / imaginary parts
  const float inv_fact[16] = {1.f, 1.f, 0.5f, 1.f / 6, 1.f / 24, 1.f / 120, 1.f / 720, 1.f / 5040, 1.f / 40320,
                              1.f / 362880, 1.f / 3628800, 1.f / 39916800, 1.f / 479001600, 1.f / 6227020800.f,
                              1.f / 87178291200.f, 1.f / 1307674368000.f};
  float Fre = 0.f, Fim = 0.f;
#pragma unroll
  for (int m = 0; m <= MM; ++m) {
    const int p = (m + 2) & 3;  // i^p: 0 -> 1, 1 -> i, 2 -> -1, 3 -> -i
    const float t = h[m] * inv_fact[m + 2];
    if (p == 0) Fre += t; else if (p == 1) Fim += t; else if (p == 2) Fre -= t; else Fim -= t;
  }
  float hb = 1.f, hc = 1.f;  // h^(v)_0
  float Bre = 0.f, Bim = 0.f, Cre = 0.f, Cim = 0.f;
#pragma unroll
  for (int m = 0; m <= MM; ++m) {
    if (m > 0) { hb = fmaf(db, hb, h[m]); hc = fmaf(dc, hc, h[m]); }
    const int p = (m + 3) & 3;
    const float f = inv_fact[m + 3];
    const float tb = hb * f, tc = hc * f;
    if (p == 0) { Bre += tb; Cre += tc; } else if (p == 1) { Bim += tb; Cim += tc; }
    else if (p == 2) { Bre -= tb; Cre -= tc; } else { Bim -= tb; Cim -= tc; }
  }
  TriDer d;
  d.F = cmul(P, cf{Fre, Fim});
  d.Db = cmul(P, cf{Bre, Bim});
  d.Dc = cmul(P, cf{Cre, Cim});
  const cf iF = imul(d.F);
  d.Da = {iF.re - d.Db.re - d.Dc.re, iF.im - d.Db.im - d.Dc.im};
  return d;
}

// The small-spread series of F, D_b and D_c as polynomials in the radius k
// for one element and direction, so that each radius costs a few Horner
// chains instead of the recurrences of tri_series_der.  With the centred
// direction dots d_v (centred phases k d_v), h_m = k^m H_m and
// h^(v)_m = k^m H^(v)_m, H^(v)_m = H_m + d_v H^(v)_{m-1}, H^(v)_0 = 1, so with
// u = k^2 (P = e^{i pm} applied outside):
//   Re F/P = sum_j fa_j u^j,        fa_j = (-1)^(j+1) H_2j / (2j+2)!
//   Im F/P = k^3 sum_j fb_j u^j,    fb_j = (-1)^j H_(2j+3) / (2j+5)!
//   Im D_v/P = sum_j va_j u^j,      va_j = (-1)^(j+1) H^(v)_2j / (2j+3)!
//   Re D_v/P = k sum_j vb_j u^j,    vb_j = (-1)^j H^(v)_(2j+1) / (2j+4)!
// (m <= 12 as in tri_series_der.)
struct TriDerPoly { float fa[7], fb[5], ba[7], bb[6], ca[7], cb[6]; };

// c_0 + c_1 u + ... + c_{N-1} u^{N-1} by Horner's rule.
template <int N>
__device__ __forceinline__ float poly_u(const float (&c)[N], float u) {
  float r = c[N - 1];
#pragma unroll
  for (int i = N - 2; i >= 0; --i) r = fmaf(r, u, c[i]);
  return r;
}

// The same for the first N of the M coefficients (the series cut after h_8
// where k |e|max < 1: 5, 3, 5, 4, 5, 4 terms of fa, fb, ba, bb, ca, cb).
template <int N, int M>
__device__ __forceinline__ float poly_first(const float (&c)[M], float u) {
  static_assert(N >= 1 && N <= M, "poly_first: N out of range");
  float r = c[N - 1];
#pragma unroll
  for (int i = N - 2; i >= 0; --i) r = fmaf(r, u, c[i]);
  return r;
}

__device__ __forceinline__ TriDerPoly tri_der_coeffs(float s1, float s2) {
  const float da = -(s1 + s2) * (1.0f / 3.0f);
  const float db = s1 + da, dc = s2 + da;
  const float mu = 0.5f * (da * da + db * db + dc * dc);
  const float nu = da * db * dc;
  float H[13];
  H[0] = 1.f; H[1] = 0.f; H[2] = mu; H[3] = nu;
#pragma unroll
  for (int m = 4; m <= 12; ++m) H[m] = fmaf(mu, H[m - 2], nu * H[m - 3]);
  // 1/n! for n = 0..15
  const float inv_fact[16] = {1.f, 1.f, 0.5f, 1.f / 6, 1.f / 24, 1.f / 120, 1.f / 720, 1.f / 5040, 1.f / 40320,
                              1.f / 362880, 1.f / 3628800, 1.f / 39916800, 1.f / 479001600, 1.f / 6227020800.f,
                              1.f / 87178291200.f, 1.f / 1307674368000.f};
  TriDerPoly c;
#pragma unroll
  for (int j = 0; j <= 6; ++j) c.fa[j] = ((j & 1) ? H[2 * j] : -H[2 * j]) * inv_fact[2 * j + 2];
#pragma unroll
  for (int j = 0; j <= 4; ++j) c.fb[j] = ((j & 1) ? -H[2 * j + 3] : H[2 * j + 3]) * inv_fact[2 * j + 5];
  float hb = 1.f, hc = 1.f;  // H^(b)_m, H^(c)_m
#pragma unroll
  for (int m = 0; m <= 12; ++m) {
    if (m > 0) { hb = fmaf(db, hb, H[m]); hc = fmaf(dc, hc, H[m]); }
    const int j = m >> 1;
    if ((m & 1) == 0) {
      const float f = ((j & 1) ? 1.f : -1.f) * inv_fact[m + 3];
      c.ba[j] = hb * f;
      c.ca[j] = hc * f;
    } else {
      const float f = ((j & 1) ? -1.f : 1.f) * inv_fact[m + 3];
      c.bb[j] = hb * f;
      c.cb[j] = hc * f;
    }
  }
  return c;
}

// G(h) = (e^{ih} - 1 - ih)/h^2 given E = e^{ih}: the direct form for
// |h| >= 1/2, otherwise the series sum_m i^{m+2} h^m/(m+2)!, m = 0..9:
//   Re = -1/2 + h^2/24 - h^4/720 + h^6/40320 - h^8/3628800
//   Im = h (-1/6 + h^2/120 - h^4/5040 + h^6/362880 - h^8/39916800)
// Both are evaluated and one is selected (no divergent branch).
__device__ __forceinline__ cf Gfun(cf E, float h) {
  const float h2 = h * h;
  const float ih2 = rcp_fast(h2);  // inf for h = 0, where the series is taken
  const float re = fmaf(h2, fmaf(h2, fmaf(h2, fmaf(h2, -1.0f / 3628800.0f, 1.0f / 40320.0f), -1.0f / 720.0f),
                                 1.0f / 24.0f), -0.5f);
  const float im = h * fmaf(h2, fmaf(h2, fmaf(h2, fmaf(h2, -1.0f / 39916800.0f, 1.0f / 362880.0f), -1.0f / 5040.0f),
                                     1.0f / 120.0f), -1.0f / 6.0f);
  const bool big = fabsf(h) >= 0.5f;
  return {big ? (E.re - 1.0f) * ih2 : re, big ? (E.im - h) * ih2 : im};
}

__device__ __forceinline__ cf conjmul(cf a, cf b) { return {a.re * b.re + a.im * b.im, a.im * b.re - a.re * b.im}; }  // a conj(b)

__device__ __forceinline__ cf csel(bool c, cf a, cf b) { return {c ? a.re : b.re, c ? a.im : b.im}; }

// The roles (P, Q the pair with the largest gap, R the middle vertex) are
// chosen by selects, so lanes of a warp that pick different pairs do not split.
__device__ __forceinline__ TriDer tri_generic_der(cf Pa, cf Pb, cf Pc, float al, float be) {
  TriDer d;
  d.F = tri_generic(Pa, Pb, Pc, al, be);
  const float gab = al, gac = be, gbc = be - al;
  const float aab = fabsf(gab), aac = fabsf(gac), abc = fabsf(gbc);
  const bool c1 = aab >= aac && aab >= abc;  // P = a, Q = b, R = c
  const bool c2 = !c1 && aac >= abc;         // P = a, Q = c, R = b; else P = b, Q = c, R = a
  // vertices as (phasor, relative phase): a = 0, b = al, c = be
  const cf phP = csel(c1 || c2, Pa, Pb), phQ = csel(c1, Pb, Pc), phR = csel(c1, Pc, csel(c2, Pb, Pa));
  const float zP = c1 || c2 ? 0.f : al, zQ = c1 ? al : be, zR = c1 ? be : (c2 ? al : 0.f);
  const float iden = rcp_fast(zQ - zP);
  // f[u,u,v] = e^{iu} G(v - u), e^{i(v-u)} = Pv conj(Pu)
  const cf fQQR = cmul(phQ, Gfun(conjmul(phR, phQ), zR - zQ));
  const cf fPPR = cmul(phP, Gfun(conjmul(phR, phP), zR - zP));
  const cf DQ = cscale(csub(fQQR, d.F), iden);
  const cf DP = cscale(csub(d.F, fPPR), iden);
  // D_R from D_P + D_Q + D_R = i F (translation invariance) instead of its
  // own two G terms: |F| <= 1/2 and |D| <= 1/6, so the subtraction costs
  // ~1e-7 absolute, the level of the other terms' rounding
  const cf DR = {-d.F.im - DP.re - DQ.re, d.F.re - DP.im - DQ.im};
  d.Da = csel(c1 || c2, DP, DR);
  d.Db = csel(c1, DQ, csel(c2, DR, DP));
  d.Dc = csel(c1, DR, DQ);
  return d;
}

// The large-spread derivatives from the vertex phases, as an out-of-line call:
// a kernel whose hot radius loop inlines this rarely taken path as well as the
// series outgrows the instruction cache (the loop then stalls on instruction
// fetch), while the call costs little on the few nodes that take it.
// The vertex phasors come from the phasor table (cis_tab_df): tab is the
// 256-entry table, kt the radius in 1/256 turns per unit length.
static __device__ __noinline__ TriDer tri_generic_der_at(const float2* tab, float2 kt, df sa, df sb, df sc, float al,
                                                         float be) {
  return tri_generic_der(cis_tab_df(tab, kt, sa), cis_tab_df(tab, kt, sb), cis_tab_df(tab, kt, sc), al, be);
}

}  // namespace pi
