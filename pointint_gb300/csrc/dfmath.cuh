// Device arithmetic for the FP32 form-factor kernels.
//
// Phases k.x reach 1e4-1e5 rad on the configs' k-grids (k up to ~7e3, centres
// up to ~14 from the origin).  A plain FP32 phase would carry ~1e-2 rad of
// error there, so phases are formed as double-float (hi + lo FP32 pair) products
// and reduced modulo pi/2 by the Cody-Waite method (W. J. Cody and W. Waite,
// "Software Manual for the Elementary Functions", 1980) with a two-part split
// of pi/2 computed from its decimal expansion below, then sin and cos come
// from short polynomials on [-pi/4, pi/4].  Error-free product / sum
// transformations follow Dekker (1971) and Knuth (TAOCP vol. 2, 4.2.2).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

namespace pi {

struct df { float hi, lo; };

__device__ __forceinline__ df two_prod(float a, float b) {
  float p = a * b;
  return {p, fmaf(a, b, -p)};
}

__device__ __forceinline__ df two_sum(float a, float b) {
  float s = a + b;
  float bb = s - a;
  float e = (a - (s - bb)) + (b - bb);
  return {s, e};
}

// Fixed-order compensated FP32 sum (Kahan-Babuska / Neumaier): the running
// sum and the sum of its rounding errors; hi + lo keeps ~48 bits.  Used for
// the split-K reductions, where FP64 adds (1/64 of the FP32 rate on GB300)
// would cost more than reading the partial tiles.
struct kbsum {
  float hi, lo;
  __device__ __forceinline__ void add(float x) {
    const df t = two_sum(hi, x);
    hi = t.hi;
    lo += t.lo;
  }
  __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};

__device__ __forceinline__ df quick_two_sum(float a, float b) {  // requires |a| >= |b|
  float s = a + b;
  return {s, b - (s - a)};
}

__device__ __forceinline__ df df_add(df a, df b) {
  df s = two_sum(a.hi, b.hi);
  return quick_two_sum(s.hi, s.lo + a.lo + b.lo);
}

__device__ __forceinline__ df df_mul(df a, df b) {
  df p = two_prod(a.hi, b.hi);
  float lo = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, p.lo));
  return quick_two_sum(p.hi, lo);
}

__device__ __forceinline__ df operator*(df a, float s) {  // a * s for s = +-1 or a power of two
  return {a.hi * s, a.lo * s};
}

// a * b as an unnormalised pair (hi, lo) -- enough for cis, which treats hi
// and lo separately.
__device__ __forceinline__ df df_mul_un(df a, df b) {
  const float p = a.hi * b.hi;
  return {p, fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, fmaf(a.hi, b.hi, -p)))};
}

// (dh + dl) . x in double-float, x in FP32.
__device__ __forceinline__ df cdot(float3 dh, float3 dl, float3 x) {
  df p0 = two_prod(dh.x, x.x), p1 = two_prod(dh.y, x.y), p2 = two_prod(dh.z, x.z);
  df s = two_sum(p0.hi, p1.hi);
  df t = two_sum(s.hi, p2.hi);
  float lo = s.lo + t.lo + p0.lo + p1.lo + p2.lo + (dl.x * x.x + dl.y * x.y + dl.z * x.z);
  return quick_two_sum(t.hi, lo);
}

// (dh + dl) . (xh + xl) in double-float, the dl . xl term (~2^-48 relative)
// dropped, without the final renormalisation: (hi, lo) with |lo| a few ulp of
// hi, enough for df_mul_un and cis, which treat the two parts separately.
__device__ __forceinline__ df cdot2_un(float3 dh, float3 dl, float3 xh, float3 xl) {
  df p0 = two_prod(dh.x, xh.x), p1 = two_prod(dh.y, xh.y), p2 = two_prod(dh.z, xh.z);
  df s = two_sum(p0.hi, p1.hi);
  df t = two_sum(s.hi, p2.hi);
  return {t.hi, s.lo + t.lo + p0.lo + p1.lo + p2.lo + (dl.x * xh.x + dl.y * xh.y + dl.z * xh.z) +
                    (dh.x * xl.x + dh.y * xl.y + dh.z * xl.z)};
}

// (dh + dl) . (xh + xl) in double-float; the dl . xl term (~2^-48 relative)
// is dropped.
__device__ __forceinline__ df cdot2(float3 dh, float3 dl, float3 xh, float3 xl) {
  df p0 = two_prod(dh.x, xh.x), p1 = two_prod(dh.y, xh.y), p2 = two_prod(dh.z, xh.z);
  df s = two_sum(p0.hi, p1.hi);
  df t = two_sum(s.hi, p2.hi);
  float lo = s.lo + t.lo + p0.lo + p1.lo + p2.lo + (dl.x * xh.x + dl.y * xh.y + dl.z * xh.z) +
             (dh.x * xl.x + dh.y * xl.y + dh.z * xl.z);
  return quick_two_sum(t.hi, lo);
}

// pi/2 = 1.57079632679489661923132169163975144209858...
//   PIO2_A = FP32(pi/2)            = 1.5707963705062866
//   PIO2_B = FP32(pi/2 - PIO2_A)   = -4.371138828673793e-08
// |pi/2 - A - B| < 2e-15, so n (pi/2 - A - B) < 2e-10 for |n| < 1e5.
#define PI_PIO2_A 1.5707963705062866f
#define PI_PIO2_B (-4.371138828673793e-08f)
#define PI_TWO_OVER_PI 0.6366197466850281f

struct cf { float re, im; };

// 1/x by the hardware approximation (rcp.approx.ftz: about 1 ulp, inf at 0).
// Used where the result scales a difference that already carries far more
// rounding error than that, as in the divided differences below.
__device__ __forceinline__ float rcp_fast(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// sqrt(x) by the hardware approximation (sqrt.approx.ftz: about 1 ulp), for
// arguments of Bessel functions and the like, where an IEEE square root's
// multi-instruction sequence buys nothing.
__device__ __forceinline__ float sqrt_fast(float x) {
  float r;
  asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// e^{i (r + q pi/2)} for r in [-pi/4, pi/4]: this project's own least-squares
// polynomials for sin(r)/r (degree 3 in r^2) and cos(r) (degree 4 in r^2),
// fitted on Chebyshev-spaced samples of [-pi/4, pi/4].  Their approximation
// errors (2.4e-9, 4.7e-11) sit far below FP32 rounding, so the FP32
// evaluation error is the rounding's, <= 6e-8 each (emulated), about 5x below
// the hardware sin/cos approximation; one degree more changes nothing.  The
// quadrant q mod 4 rotates the result.
__device__ __forceinline__ cf cis_quadrant(float r, int q) {
  const float t = r * r;
  const float sn = r * fmaf(t, fmaf(t, fmaf(t, -1.950395963e-04f, 8.332036436e-03f), -1.666665077e-01f), 1.0f);
  const float cs = fmaf(t, fmaf(t, fmaf(t, fmaf(t, 2.437987678e-05f, -1.388661913e-03f), 4.166661575e-02f), -0.5f),
                        1.0f);
  const float s1 = (q & 1) ? cs : sn;   // sin(r + q pi/2) up to sign
  const float c1 = (q & 1) ? sn : cs;   // cos(r + q pi/2) up to sign
  // signs: cos(r + q pi/2) < 0 for q mod 4 = 1, 2 and sin for q mod 4 = 2, 3
  // ((q + 1) & 2) = (q & 2) ^ ((q & 1) << 1), so the cosine's sign bit is the
  // sine's flipped by q's low bit
  const unsigned sim = (unsigned)(q & 2) << 30, sre = sim ^ ((unsigned)q << 31);
  return {__uint_as_float(__float_as_uint(c1) ^ sre), __uint_as_float(__float_as_uint(s1) ^ sim)};
}

// Round-to-nearest integer of a * b + c, |result| < 2^22, by the 1.5 * 2^23
// shift: the FMA rounds the exact a * b + c to an integer, returned as a float
// in *n, and the low bits of the shifted float are that integer modulo 4.
#define PI_ROUND_SHIFT 12582912.0f
__device__ __forceinline__ int round_fma(float a, float b, float c, float* n) {
  const float t = fmaf(a, b, c + PI_ROUND_SHIFT);
  *n = t - PI_ROUND_SHIFT;
  return __float_as_int(t);
}

// e^{i x} for a double-float phase x (|x| < ~1e5): Cody-Waite reduction by
// pi/2 to r in [-pi/4, pi/4] (n = x.hi 2/pi rounded; fmaf(-n, A, x) is exact:
// the result needs at most 23 significant bits), then cis_quadrant.
__device__ __forceinline__ cf cis(df x) {
  float n;
  const int q = round_fma(x.hi, PI_TWO_OVER_PI, 0.0f, &n);
  float r = fmaf(-n, PI_PIO2_A, x.hi);
  r = fmaf(-n, PI_PIO2_B, r);
  r += x.lo;
  return cis_quadrant(r, q);
}

// e^{i x} for an FP64 phase of any size FP64 holds, such as the origin phase
// e^{i k.o} of an object far from the frame's origin (cis above wants
// |x| < ~1e5): Cody-Waite reduction by pi/2 in FP64, pi/2 = A + B with
// A = 1.5707963267948966, B = 6.123233995736766e-17 (|pi/2 - A - B| < 2e-33),
// then cis_quadrant.  A handful of FP64 operations, so it is used once per
// output, not in element loops.
__device__ __forceinline__ cf cis_f64(double x) {
  const double n = rint(x * 0.6366197723675814);
  double r = fma(-n, 1.5707963267948966, x);
  r = fma(-n, 6.123233995736766e-17, r);
  return cis_quadrant((float)r, (int)(long long)n);
}

// ---------------------------------------------------------------------------
// Table phasors.  A phase given in units of 1/256 turn, y = 256 x / (2 pi),
// is split as y = n + f with n = round(y) (the 1.5 * 2^23 shift: |y| < 2^22,
// so |x| < 1.0e5 rad) and |f| <= 1/2; then
//   e^{i x} = tab[n mod 256] e^{i c f},  c = 2 pi / 256,
// with tab[j] = e^{2 pi i j / 256} rounded once from FP64 (per component
// error <= 2^-25) and, on |c f| <= pi / 256 = 0.0123, cos(c f) = 1 - (c f)^2 / 2
// and sin(c f) = c f - (c f)^3 / 6 (truncation 9.4e-10 and 2.4e-12; Taylor
// series, whose next terms bound the error on so short an interval).  About
// 7e-8 per component overall, the same order as FP32 rounding of the phasor.
#define PI_TURN256 0.024543692606170259f  // 2 pi / 256
#define PI_TURN256_C2 0.00030119642337308832f  // c^2 / 2
#define PI_TURN256_C3 2.4641574764489986e-06f  // c^3 / 6

// e^{i c f} times tab[idx] (idx already reduced mod 256).
// cos = 1 + cm with cm = -(c f)^2 / 2 tiny: tab (cos + i sin) is formed as
// tab + tab cm + i tab sin, so both roundings happen at the phasor's scale.
__device__ __forceinline__ cf cis_tab_frac(const float2* tab, int idx, float f) {
  const float f2 = f * f;
  const float cm = f2 * -PI_TURN256_C2;
  const float sn = f * fmaf(f2, -PI_TURN256_C3, PI_TURN256);
  const float2 t = tab[idx];
  return {fmaf(t.x, cm, fmaf(-t.y, sn, t.x)), fmaf(t.y, cm, fmaf(t.x, sn, t.y))};
}

// e^{i x} with x = 2 pi (kt.hi + kt.lo) (sm.hi + sm.lo) / 256: kt is a radius
// in units of 1/256 turn per unit length (double-float), sm a direction dot
// product (double-float, unnormalised).  The leading product's rounding is
// recovered by an FMA against the rounded integer, so f carries the full
// product to ~2^-25 of a unit; the cross terms are added to it (the lo.lo
// term, ~2^-48 relative, is dropped).
__device__ __forceinline__ cf cis_tab_df(const float2* tab, float2 kt, df sm) {
  const float t = fmaf(kt.x, sm.hi, PI_ROUND_SHIFT);  // rounds the exact product to an integer
  const float n = t - PI_ROUND_SHIFT;
  float f = fmaf(kt.x, sm.hi, -n);
  f = fmaf(kt.x, sm.lo, f);
  f = fmaf(kt.y, sm.hi, f);
  return cis_tab_frac(tab, __float_as_int(t) & 255, f);
}

// The same for an FP32 dot product d (kt still double-float).
__device__ __forceinline__ cf cis_tab_f(const float2* tab, float2 kt, float d) {
  const float t = fmaf(kt.x, d, PI_ROUND_SHIFT);
  const float n = t - PI_ROUND_SHIFT;
  float f = fmaf(kt.x, d, -n);
  f = fmaf(kt.y, d, f);
  return cis_tab_frac(tab, __float_as_int(t) & 255, f);
}

// Two phasors at once with packed FP32 (sm_100 family): radii a, b in the
// halves of kth = (kt_a.hi, kt_b.hi), ktl = (kt_a.lo, kt_b.lo), the same dot
// product in both halves of smh, sml.  Every packed operation is an operation
// of cis_tab_df on each half, so each half gives cis_tab_df's result.
struct cf2 { float2 re, im; };

__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 dup2(float a) { return make_float2(a, a); }

__device__ __forceinline__ cf2 cis_tab_df2(const float2* tab, float2 kth, float2 ktl, float2 smh, float2 sml) {
  const float2 t = __ffma2_rn(kth, smh, dup2(PI_ROUND_SHIFT));
  const float2 mn = __ffma2_rn(t, dup2(-1.0f), dup2(PI_ROUND_SHIFT));  // -n, exact
  float2 f = __ffma2_rn(kth, smh, mn);
  f = __ffma2_rn(kth, sml, f);
  f = __ffma2_rn(ktl, smh, f);
  const float2 f2 = __fmul2_rn(f, f);
  const float2 cm = __fmul2_rn(f2, dup2(-PI_TURN256_C2));
  const float2 sn = __fmul2_rn(f, __ffma2_rn(f2, dup2(-PI_TURN256_C3), dup2(PI_TURN256)));
  const float2* ta = tab + (__float_as_int(t.x) & 255);
  const float2* tb = tab + (__float_as_int(t.y) & 255);
  const float2 tx = make_float2(ta->x, tb->x), ty = make_float2(ta->y, tb->y);
  return {__ffma2_rn(tx, cm, __ffma2_rn(neg2(ty), sn, tx)), __ffma2_rn(ty, cm, __ffma2_rn(tx, sn, ty))};
}

__device__ __forceinline__ cf cmul(cf a, cf b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
__device__ __forceinline__ cf csub(cf a, cf b) { return {a.re - b.re, a.im - b.im}; }
__device__ __forceinline__ cf cscale(cf a, float s) { return {a.re * s, a.im * s}; }

// Exact-ish division of a double-float by 3 (the FP32 quotient's remainder is
// formed exactly with an FMA).
__device__ __forceinline__ df df_div3(df a) {
  const float q = a.hi * (1.0f / 3.0f);
  const float r = fmaf(-q, 3.0f, a.hi);
  return quick_two_sum(q, (r + a.lo) * (1.0f / 3.0f));
}

// The triangle form factor is e^{ik.a} Phi(al, be) (k.S)/|k| with Phi as in the
// reference's Triangle_Phi_ab (cpp/src/element_functions.cpp:63-70), and
// Phi = -2 e[0, al, be] for the divided differences e[..] of e(z) = e^{iz}.
// Shifting by the vertex phase, e^{ik.a} Phi = -2 e[pa, pb, pc] with the vertex
// phases pa = k.a, pb = k.b, pc = k.c.  Two evaluations are used, both without
// the common factor -2:
//
// tri_series: spread D = max(|al|, |be|, |be-al|) < 3.  Taylor series about
//   the centroid phase pm = k.m, m = (a+b+c)/3 (no cancellation):
//     e[pa,pb,pc] = e^{i pm} S,  S = sum_m i^{m+2} h_m / (m+2)!
//   with h_m the complete homogeneous symmetric polynomials of the centred
//   points (|centred point| <= 2D/3), h_m = -e2 h_{m-2} + e3 h_{m-3} (e1 = 0),
//   truncated after h_13: the remainder stays below 7e-10 of the leading
//   term 1/2 (40-digit divided differences over random triangles at D up to
//   3; the cut after h_12 leaves 5e-9 there, 3e-11 at D < 2).

// The same series as a polynomial in the radius k for a fixed element and
// direction: with the centred direction dots d (so the centred phases are k d),
// -e2 = k^2 mu and e3 = k^3 nu, hence h_m = k^m H_m with H_m = mu H_{m-2} +
// nu H_{m-3}, and
//   Re S = sum_j a_j u^j (u = k^2),   Im S = k^3 sum_j b_j u^j.
// tri_series_coeffs returns g * a_0..a_6 and g * b_0..b_5 so that one radius
// costs two Horner chains.  The factorials enter as constant reciprocals
// (1.0f / c folds at compile time): g / c would be an IEEE division per
// coefficient.
struct TriPoly { float a[7], b[6]; };

__device__ __forceinline__ TriPoly tri_series_coeffs(float s1, float s2, float g) {
  const float da = -(s1 + s2) * (1.0f / 3.0f);
  const float db = s1 + da, dc = s2 + da;
  const float mu = 0.5f * (da * da + db * db + dc * dc);
  const float nu = da * db * dc;
  // G_m = g H_m: the recurrence is linear, so starting it from g H_2, g H_3
  // leaves one constant multiply per coefficient
  const float G2 = mu * g, G3 = nu * g, G4 = mu * G2;
  const float G5 = fmaf(mu, G3, nu * G2);
  const float G6 = fmaf(mu, G4, nu * G3);
  const float G7 = fmaf(mu, G5, nu * G4);
  const float G8 = fmaf(mu, G6, nu * G5);
  const float G9 = fmaf(mu, G7, nu * G6);
  const float G10 = fmaf(mu, G8, nu * G7);
  const float G11 = fmaf(mu, G9, nu * G8);
  const float G12 = fmaf(mu, G10, nu * G9);
  const float G13 = fmaf(mu, G11, nu * G10);
  TriPoly t;
  t.a[0] = -0.5f * g;
  t.a[1] = G2 * (1.0f / 24.0f);
  t.a[2] = G4 * (-1.0f / 720.0f);
  t.a[3] = G6 * (1.0f / 40320.0f);
  t.a[4] = G8 * (-1.0f / 3628800.0f);
  t.a[5] = G10 * (1.0f / 479001600.0f);
  t.a[6] = G12 * (-1.0f / 87178291200.0f);
  t.b[0] = G3 * (1.0f / 120.0f);
  t.b[1] = G5 * (-1.0f / 5040.0f);
  t.b[2] = G7 * (1.0f / 362880.0f);
  t.b[3] = G9 * (-1.0f / 39916800.0f);
  t.b[4] = G11 * (1.0f / 6227020800.0f);
  t.b[5] = G13 * (-1.0f / 1307674368000.0f);
  return t;
}

// u = k^2, k3 = k^3.
__device__ __forceinline__ cf tri_series_eval(const TriPoly& t, float u, float k3) {
  const float re = fmaf(u, fmaf(u, fmaf(u, fmaf(u, fmaf(u, fmaf(u, t.a[6], t.a[5]), t.a[4]), t.a[3]), t.a[2]), t.a[1]), t.a[0]);
  const float im =
      k3 * fmaf(u, fmaf(u, fmaf(u, fmaf(u, fmaf(u, t.b[5], t.b[4]), t.b[3]), t.b[2]), t.b[1]), t.b[0]);
  return {re, im};
}

// The coefficients that tri_series_eval_short reads (a[0..3], b[0..2]) alone.
struct TriPolyShort { float a[4], b[3]; };

__device__ __forceinline__ TriPolyShort tri_series_coeffs_short(float s1, float s2, float g) {
  const float da = -(s1 + s2) * (1.0f / 3.0f);
  const float db = s1 + da, dc = s2 + da;
  const float mu = 0.5f * (da * da + db * db + dc * dc);
  const float nu = da * db * dc;
  const float G2 = mu * g, G3 = nu * g, G4 = mu * G2;
  const float G5 = fmaf(mu, G3, nu * G2);
  const float G6 = fmaf(mu, G4, nu * G3);
  const float G7 = fmaf(mu, G5, nu * G4);
  TriPolyShort t;
  t.a[0] = -0.5f * g;
  t.a[1] = G2 * (1.0f / 24.0f);
  t.a[2] = G4 * (-1.0f / 720.0f);
  t.a[3] = G6 * (1.0f / 40320.0f);
  t.b[0] = G3 * (1.0f / 120.0f);
  t.b[1] = G5 * (-1.0f / 5040.0f);
  t.b[2] = G7 * (1.0f / 362880.0f);
  return t;
}

// tri_series_eval_short for two radii (u = k^2, k3 = k^3 per half) with packed FP32.
__device__ __forceinline__ cf2 tri_series_eval_short2(const TriPolyShort& t, float2 u, float2 k3) {
  const float2 re = __ffma2_rn(u, __ffma2_rn(u, __ffma2_rn(u, dup2(t.a[3]), dup2(t.a[2])), dup2(t.a[1])), dup2(t.a[0]));
  const float2 im = __fmul2_rn(k3, __ffma2_rn(u, __ffma2_rn(u, dup2(t.b[2]), dup2(t.b[1])), dup2(t.b[0])));
  return {re, im};
}

// The same series cut after a[3] and b[2], for k |e|max < 1 (|e|max the longest
// edge, so k sp < 1): the dropped terms stay below 6.2e-9 of |a[0]| (FP64
// evaluation over icosphere and box triangles at the bound).
template <class Poly>
__device__ __forceinline__ cf tri_series_eval_short(const Poly& t, float u, float k3) {
  const float re = fmaf(u, fmaf(u, fmaf(u, t.a[3], t.a[2]), t.a[1]), t.a[0]);
  const float im = k3 * fmaf(u, fmaf(u, t.b[2], t.b[1]), t.b[0]);
  return {re, im};
}

// First divided difference of f(z) = e^{iz} at two points u, v = u + g, given
// Pu = e^{iu}, Pv = e^{iv}: (Pv - Pu)/g for |g| >= 1/2, otherwise the
// cancellation-free form i e^{i(u+v)/2} sinc(g/2) with short Taylor series of
// cos, sin and sinc on |g/2| < 1/4 (truncation < 1e-9).  Both forms are
// evaluated and one is selected, so the lanes of a warp never split on |g|.
__device__ __forceinline__ cf dd1(cf Pu, cf Pv, float g) {
  const float ig = rcp_fast(g);  // inf for g = 0, where the series form is taken
  const cf big = cscale(csub(Pv, Pu), ig);
  const float x = 0.5f * g, x2 = x * x;
  const float c = fmaf(x2, fmaf(x2, fmaf(x2, -1.0f / 720.0f, 1.0f / 24.0f), -0.5f), 1.0f);
  const float sc = fmaf(x2, fmaf(x2, fmaf(x2, -1.0f / 5040.0f, 1.0f / 120.0f), -1.0f / 6.0f), 1.0f);
  const cf m = cmul(Pu, cf{c, x * sc});
  const bool b = fabsf(g) >= 0.5f;
  return {b ? big.re : -m.im * sc, b ? big.im : m.re * sc};
}

// tri_generic: spread D >= 2 (the form-factor kernel takes it for D >= 3,
// the adjoint's tri_generic_der for D >= 2).
// e[u, v, w] = (f[v, w] - f[u, v]) / (w - u) with (u, v) the pair of
// vertices with the smallest gap.  The two gaps to w
// are then the middle one and D, both at least D / 2 >= 1, so f[v, w] takes
// the direct form (Pw - Pv) / (w - v) and the final division is by at least
// D / 2 (at most a factor 2 more FP32 rounding than a division by D), while
// f[u, v] takes dd1 (its gap may be anything up to D / 2).  Returns
// e[pa, pb, pc] given the vertex phasors and al = pb - pa, be = pc - pa.  The
// roles are chosen by selects, not a three-way branch: the lanes of a warp
// hold different directions and pick different pairs, and a branch would run
// all three cases for the warp.
__device__ __forceinline__ cf tri_generic(cf Pa, cf Pb, cf Pc, float al, float be) {
  const float aab = fabsf(al), aac = fabsf(be), abc = fabsf(be - al);
  const bool nab = aab <= aac && aab <= abc;  // near pair (a, b), w = c
  const bool nac = !nab && aac <= abc;        // near pair (a, c), w = b; else (b, c), w = a
  // vertices as (phasor, phase relative to a)
  const bool ua = nab || nac;
  const cf Pu = ua ? Pa : Pb;
  const cf Pv = nab ? Pb : Pc;
  const cf Pw = nab ? Pc : (nac ? Pb : Pa);
  const float zu = ua ? 0.f : al, zv = nab ? al : be, zw = nab ? be : (nac ? al : 0.f);
  const cf fuv = dd1(Pu, Pv, zv - zu);
  const float ivw = rcp_fast(zw - zv);
  const cf fvw = {(Pw.re - Pv.re) * ivw, (Pw.im - Pv.im) * ivw};
  const float s = rcp_fast(zw - zu);
  return {(fvw.re - fuv.re) * s, (fvw.im - fuv.im) * s};
}

}  // namespace pi
