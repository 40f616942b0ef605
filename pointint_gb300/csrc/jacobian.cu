// Jacobian of the form factors with respect to the DoFs, and from it the
// Gauss-Newton Hessian blocks.
//
//   G[d][q] = sqrt|w_q| dA_n(k_q)/dtheta_{n,d}
//
// for every object n and DoF d, rows in the order of the concatenated DoF
// vector, FP32 complex, q-major like J.  The reference's Gauss-Newton blocks
// (hessian_ij of compute_intersection_volume_multi_object.cpp:236-292 / K16
// cpp/src/compute_intersection_volume_multi_object.cu:189-229; hessian_geom1,
// geom2, cross of compute_intersection_volume_cpu.cpp:153-186 / K11
// cpp/src/compute_intersection_volume.cu:109-157) are blocks of
//
//   H = Re(G diag(sign w) G^H) / (8 pi^3),
//
// which the volume contraction forms from G's rows exactly as it forms V from
// J's.  The per-element derivatives are the adjoint's (adjoint.cu); here they
// are summed over elements at every k-node (forward mode) instead of over
// k-nodes for every element.
//
//  * AffineDoF triangles (x = A x0 + t): dA/dt_r = i k_r A; dA/dA_rc =
//    sum_e sum_s (df_e/dv_s)_r x0_{s,c} with df/dv_s = -2 (c_s F + gamma k d D_s),
//    so each thread accumulates sum_e F N0_e (from which sum_e F U_e,
//    U_rc = sum_s c_{s,r} x0_{s,c}, follows per node) and
//    sum_e gamma sum_s D_s x0_s.
//  * AffineDoF disks / Gaussians (c = A c0 + t, n' = A n0, M = A A^T):
//    dA/dA_rc = i k d_r Z_c + khat_r N_c + k^2 d_r (A^T d)_c Y with
//    Z = sum P S a c0, N = sum P (S - k^2 s_n^2 S_r) n0, Y = sum P a S_r.
//  * TriangleMeshDoF: dA/dv_p = sum over the triangles at vertex p of
//    df_e/dv_p (a gather over the batch's vertex adjacency, no atomics).
//
// Thread layouts: the affine-triangle kernel as ff_kernel (a warp owns 32
// directions x JAC_R neighbouring radii); the others one radius per thread (a
// warp owns 32 directions at one radius).  The origin phase e^{ik.o} and
// sqrt|w| are applied once per output.
#include <cuda_runtime.h>
#include <algorithm>
#include <cstdint>
#include <vector>
#include "pi_internal.h"
#include "dfmath.cuh"
#include "bessel.cuh"
#include "tri_adjoint.cuh"

namespace pi {

namespace {

constexpr int JAC_THREADS = 128;
constexpr int JAC_WARPS = JAC_THREADS / 32;
constexpr int JAC_TILE = 128;

enum { JAC_AFFINE_TRI = 0, JAC_AFFINE_SURF = 1, JAC_MESH_TRI = 2 };

struct JacObj {
  int32_t obj, kind;
  int64_t row0;                    // first row of G
  int64_t vstart, nverts;          // TriangleMeshDoF: vertex range in the batch's adjacency
  const unsigned char* src;        // reference-layout source elements
  const double* dofs;              // device DoF vector
};

struct TriSrcJ { double a[3], e1[3], e2[3], S[3]; int32_t vid0, vid1, vid2, pad; };
struct SurfSrcJ { double c[3], n[3], p0, p1; };

// FP32 sum with chunked partials and a compensated running total (complex).
struct kcf {
  float pr = 0.f, pi = 0.f, sr = 0.f, si = 0.f, cr = 0.f, ci = 0.f;
  __device__ __forceinline__ void fma_add(cf a, float s) { pr = fmaf(a.re, s, pr); pi = fmaf(a.im, s, pi); }
  __device__ __forceinline__ void flush() {
    float y = pr - cr, t = sr + y;
    cr = (t - sr) - y; sr = t;
    y = pi - ci; t = si + y;
    ci = (t - si) - y; si = t;
    pr = pi = 0.f;
  }
  __device__ __forceinline__ cf value() const { return cf{sr, si}; }
};

struct JacThread {
  int j, jm, r;  // direction j evaluated, its antipode jm written from it (or -1)
  bool active;
  float3 dh, dl;
  float inv_norm, dnorm;
  df k;
  float2 kt;  // |k| in 1/256 turns per unit length (double-float), for the table phasors
};

__device__ __forceinline__ JacThread jac_thread(const KGridDev& kg) {
  JacThread t;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int item = blockIdx.x * JAC_WARPS + warp;
  const int dt = item / kg.L;
  t.r = item - dt * kg.L;
  const int ei = dt * 32 + lane;
  t.active = dt < (kg.Me + 31) / 32 && ei < kg.Me;
  t.j = 0;
  t.jm = -1;
  if (t.active) { const int2 pr = kg.dpair[ei]; t.j = pr.x; t.jm = pr.y; }
  t.dh = t.dl = make_float3(0.f, 0.f, 0.f);
  t.inv_norm = t.dnorm = 0.f;
  t.k = df{0.f, 0.f};
  t.kt = make_float2(0.f, 0.f);
  if (t.active) {
    const float4 h = kg.dir_hi[t.j], l = kg.dir_lo[t.j];
    t.dh = make_float3(h.x, h.y, h.z);
    t.dl = make_float3(l.x, l.y, l.z);
    t.inv_norm = h.w;
    t.dnorm = l.w;
    const float2 km = kg.kmag[t.r];
    t.k = df{km.x, km.y};
    t.kt = kg.kt256[t.r];
  }
  return t;
}

// The 256-entry phasor table of cis_tab_df in shared memory; every thread of
// the CTA calls this before its first use (it ends in __syncthreads).
__device__ __forceinline__ void stage_cis_tab(const KGridDev& kg, float2* ctab) {
  for (int i = threadIdx.x; i < 256; i += blockDim.x) ctab[i] = kg.cis_tab[i];
  __syncthreads();
}

// e^{ik.o} for this thread's node (0 at k = 0, where A = 0 by definition).
__device__ __forceinline__ cf jac_origin_phase(const JacThread& t, const ObjDev& od) {
  const double so_d = ((double)t.dh.x + t.dl.x) * od.origin[0] + ((double)t.dh.y + t.dl.y) * od.origin[1] +
                      ((double)t.dh.z + t.dl.z) * od.origin[2];
  const cf e = cis_f64(((double)t.k.hi + (double)t.k.lo) * so_d);
  return (t.k.hi * t.dnorm < 1e-10f) ? cf{0.f, 0.f} : e;
}

// The node of radius r and direction j, and that of its antipode jm: a
// derivative of a real solid's form factor obeys dA(-k) = -conj dA(k) like A,
// so one evaluation gives both outputs, each scaled by its own sqrt|w|.
struct JacOut {
  int64_t q, qm;  // qm < 0: no antipode
  float sw, swm;
  __device__ __forceinline__ void put(float2* row, cf v) const {
    row[q] = make_float2(v.re * sw, v.im * sw);
    if (qm >= 0) row[qm] = make_float2(-v.re * swm, v.im * swm);
  }
};

__device__ __forceinline__ JacOut jac_out(const KGridDev& kg, int r, int j, int jm) {
  JacOut o;
  o.q = (int64_t)r * kg.M + j;
  o.qm = jm >= 0 ? (int64_t)r * kg.M + jm : -1;
  o.sw = kg.sqrtw[o.q];
  o.swm = jm >= 0 ? kg.sqrtw[o.qm] : 0.f;
  return o;
}

// Triangle derivative pieces at one node: F, D_a, D_b, D_c (tri_adjoint.cuh),
// gamma = khat.S and the gradient vectors c_s of gamma with respect to the vertices.
struct TriNode {
  TriDer d;
  float gam;
  float3 c[3];
};

// ml: the centroid's low word, and in .w the longest edge (the series-length bound).
__device__ __forceinline__ TriNode tri_node(const JacThread& t, const float2* ctab, float3 m, float4 ml, float3 e1,
                                            float3 e2, float3 S) {
  TriNode o;
  const df sm = cdot2(t.dh, t.dl, m, make_float3(ml.x, ml.y, ml.z)), d1 = cdot(t.dh, t.dl, e1),
           d2 = cdot(t.dh, t.dl, e2);
  const float sp = fmaxf(fmaxf(fabsf(d1.hi), fabsf(d2.hi)), fabsf(d2.hi - d1.hi));
  const float al = t.k.hi * d1.hi, be = t.k.hi * d2.hi;
  if (t.k.hi * sp < 2.0f) {
    const cf P = cis_tab_df(ctab, t.kt, sm);
    // the lanes of a warp share the radius and the element: a uniform branch
    if (t.k.hi * t.dnorm * ml.w < 1.0f)
      o.d = tri_series_der<8>(P, al, be);
    else
      o.d = tri_series_der<12>(P, al, be);
  } else {
    const df sa = df_add(sm, df_div3(df_add(d1, d2)) * -1.0f);
    const df sb = df_add(sa, d1), sc = df_add(sa, d2);
    o.d = tri_generic_der(cis_tab_df(ctab, t.kt, sa), cis_tab_df(ctab, t.kt, sb), cis_tab_df(ctab, t.kt, sc), al, be);
  }
  o.gam = (t.dh.x * S.x + t.dh.y * S.y + t.dh.z * S.z) * t.inv_norm;
  const float3 kh = make_float3(t.dh.x * t.inv_norm, t.dh.y * t.inv_norm, t.dh.z * t.inv_norm);
  const float3 w0 = make_float3(e2.x - e1.x, e2.y - e1.y, e2.z - e1.z);
  o.c[0] = make_float3(0.5f * (kh.y * w0.z - kh.z * w0.y), 0.5f * (kh.z * w0.x - kh.x * w0.z),
                       0.5f * (kh.x * w0.y - kh.y * w0.x));
  o.c[1] = make_float3(-0.5f * (kh.y * e2.z - kh.z * e2.y), -0.5f * (kh.z * e2.x - kh.x * e2.z),
                       -0.5f * (kh.x * e2.y - kh.y * e2.x));
  o.c[2] = make_float3(0.5f * (kh.y * e1.z - kh.z * e1.y), 0.5f * (kh.z * e1.x - kh.x * e1.z),
                       0.5f * (kh.x * e1.y - kh.y * e1.x));
  return o;
}

__device__ __forceinline__ float comp(float3 v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }

// ---- AffineDoF triangles -------------------------------------------------------------
// A thread owns one direction and R neighbouring radii (the warp 32
// directions, the CTA 4 neighbouring direction blocks of one radial block).
// R = 4 (three CTAs per SM: 168 registers, 74 KB of shared memory each)
// where the launch has at least two waves of CTAs; fewer radii per thread
// for small launches (one moving mesh of the alignment caller), which
// would otherwise leave SMs idle.
// Per element and direction the small-spread series of F, D_b and D_c are
// formed once as polynomials in k (tri_der_coeffs), so a radius costs a table
// phasor, the Horner chains (cut after h_8 where k |e|max < 1, a test that is
// the same for the whole warp on a tensor grid) and three complex products.
// Radial blocks run heavy-first and the CTA order is re-mapped so that every
// object's heavy blocks start first, as in ff_kernel.  Per radius and node
// seven complex sums, chunked in FP32 and Kahan-compensated in shared memory:
//   A  += -2 gamma F                                   (translations: i k d A)
//   NF += F N0,  N0 = E1 x E2 (reference edges)        (see MF below)
//   W  += gamma (i F a0 + D_b E1 + D_c E2)             (sum_s D_s x0_s, D_a + D_b + D_c = i F)
constexpr int JAC_NSUM = 14;  // floats per radius: A, NF[3], W[3] (complex)

template <int R>
__global__ void __launch_bounds__(JAC_THREADS, 3)
jac_affine_tri_kernel(KGridDev kg, BatchDev b, const JacObj* __restrict__ jobs, float2* __restrict__ G) {
  const unsigned lin = blockIdx.y * gridDim.x + blockIdx.x;
  const int slot = (int)(lin % gridDim.y), cta = (int)(lin / gridDim.y);
  const JacObj jo = jobs[slot];
  const ObjDev od = b.objs[jo.obj];
  const int nrb = (kg.L + R - 1) / R, ndt = (kg.Me + 31) / 32;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int item = cta * JAC_WARPS + warp;
  const int ib = item / ndt, dt = item - ib * ndt;
  const int rb = ib < nrb ? nrb - 1 - ib : 0;
  const int ei = dt * 32 + lane;
  const bool active = item < ndt * nrb && ei < kg.Me;
  int j = 0, jm = -1;  // direction evaluated, its antipode written from it (or -1)
  if (active) { const int2 pr = kg.dpair[ei]; j = pr.x; jm = pr.y; }
  float3 dh = make_float3(0.f, 0.f, 0.f), dl = dh;
  float inv_norm = 0.f, dnorm = 0.f;
  if (active) {
    const float4 h = kg.dir_hi[j], l = kg.dir_lo[j];
    dh = make_float3(h.x, h.y, h.z);
    dl = make_float3(l.x, l.y, l.z);
    inv_norm = h.w;
    dnorm = l.w;
  }
  __shared__ float4 tile[7 * JAC_TILE];
  __shared__ float2 ctab[256];
  __shared__ float4 krad[JAC_WARPS][R];  // (|k| hi, lo, |k| 256 / 2 pi hi, lo)
  __shared__ float run[2 * JAC_NSUM * R * JAC_THREADS];  // running sums, then compensations
  for (int t = threadIdx.x; t < 256; t += JAC_THREADS) ctab[t] = kg.cis_tab[t];
  if (lane < R) {
    const int r = rb * R + lane;
    const bool ok = item < ndt * nrb && r < kg.L;
    const float2 km = ok ? kg.kmag[r] : make_float2(0.f, 0.f);
    const float2 kt = ok ? kg.kt256[r] : make_float2(0.f, 0.f);
    krad[warp][lane] = make_float4(km.x, km.y, kt.x, kt.y);
  }
  for (int v = 0; v < 2 * JAC_NSUM * R; ++v) run[v * JAC_THREADS + threadIdx.x] = 0.f;
  float acc[R][JAC_NSUM];
#pragma unroll
  for (int i = 0; i < R; ++i)
#pragma unroll
    for (int v = 0; v < JAC_NSUM; ++v) acc[i][v] = 0.f;
  // adds the chunk's partials to the compensated running sums
  auto flush = [&]() {
#pragma unroll
    for (int i = 0; i < R; ++i)
#pragma unroll
      for (int v = 0; v < JAC_NSUM; ++v) {
        float* ps = run + (i * JAC_NSUM + v) * JAC_THREADS + threadIdx.x;
        float* pc = ps + JAC_NSUM * R * JAC_THREADS;
        const float sum = *ps, y = acc[i][v] - *pc, t = sum + y;
        *pc = (t - sum) - y;
        *ps = t;
        acc[i][v] = 0.f;
      }
  };
  const float4* pool = b.tri_pool + 3 * od.elem_off;
  const float4* pool_lo = b.tri_lo + od.elem_off;
  const TriSrcJ* src = reinterpret_cast<const TriSrcJ*>(jo.src);
  for (int base = 0; base < od.n_elems; base += JAC_TILE) {
    const int cnt = min(JAC_TILE, od.n_elems - base);
    __syncthreads();
    for (int e = threadIdx.x; e < cnt; e += JAC_THREADS) {
      tile[6 * e] = pool[3 * (int64_t)(base + e)];
      tile[6 * e + 1] = pool[3 * (int64_t)(base + e) + 1];
      tile[6 * e + 2] = pool[3 * (int64_t)(base + e) + 2];
      // the reference vertex a0 and edges E1, E2; in .w the reference
      // doubled area vector N0 = E1 x E2
      const TriSrcJ& s = src[base + e];
      const double n0x = s.e1[1] * s.e2[2] - s.e1[2] * s.e2[1], n0y = s.e1[2] * s.e2[0] - s.e1[0] * s.e2[2],
                   n0z = s.e1[0] * s.e2[1] - s.e1[1] * s.e2[0];
      tile[6 * e + 3] = make_float4((float)s.a[0], (float)s.a[1], (float)s.a[2], (float)n0x);
      tile[6 * e + 4] = make_float4((float)s.e1[0], (float)s.e1[1], (float)s.e1[2], (float)n0y);
      tile[6 * e + 5] = make_float4((float)s.e2[0], (float)s.e2[1], (float)s.e2[2], (float)n0z);
      tile[6 * JAC_TILE + e] = pool_lo[base + e];  // centroid low word, longest edge
    }
    __syncthreads();
    if (!active) continue;
    for (int e = 0; e < cnt; ++e) {
      const float4 q0 = tile[6 * e], q1 = tile[6 * e + 1], q2 = tile[6 * e + 2], ql = tile[6 * JAC_TILE + e];
      const float3 m = make_float3(q0.x, q0.y, q0.z), e1 = make_float3(q1.x, q1.y, q1.z),
                   e2 = make_float3(q2.x, q2.y, q2.z);
      const df sm = cdot2(dh, dl, m, make_float3(ql.x, ql.y, ql.z)), d1 = cdot(dh, dl, e1), d2 = cdot(dh, dl, e2);
      const float sp = fmaxf(fmaxf(fabsf(d1.hi), fabsf(d2.hi)), fabsf(d2.hi - d1.hi));
      const float kthr = __fdividef(2.0f, sp);           // the series for k sp < 2 (inf when sp = 0)
      const float kshort = rcp_fast(ql.w * dnorm);       // cut after h_8 for k |e|max < 1
      const float gam = (dh.x * q0.w + dh.y * q1.w + dh.z * q2.w) * inv_norm;
      const TriDerPoly cp = tri_der_coeffs(d1.hi, d2.hi);
#pragma unroll
      for (int i = 0; i < R; ++i) {
        const float4 kr = krad[warp][i];
        const float k = kr.x;
        cf F, Db, Dc;
        if (k < kthr) {
          const cf P = cis_tab_df(ctab, make_float2(kr.z, kr.w), sm);
          const float u = k * k;
          float fre, fim, bre, bim, cre, cim;
          if (k < kshort) {
            fre = poly_first<5>(cp.fa, u); fim = poly_first<3>(cp.fb, u);
            bim = poly_first<5>(cp.ba, u); bre = poly_first<4>(cp.bb, u);
            cim = poly_first<5>(cp.ca, u); cre = poly_first<4>(cp.cb, u);
          } else {
            fre = poly_u(cp.fa, u); fim = poly_u(cp.fb, u);
            bim = poly_u(cp.ba, u); bre = poly_u(cp.bb, u);
            cim = poly_u(cp.ca, u); cre = poly_u(cp.cb, u);
          }
          F = cmul(P, cf{fre, u * k * fim});
          Db = cmul(P, cf{k * bre, bim});
          Dc = cmul(P, cf{k * cre, cim});
        } else {
          const df sa = df_add(sm, df_div3(df_add(d1, d2)) * -1.0f);
          const TriDer d = tri_generic_der_at(ctab, make_float2(kr.z, kr.w), sa, df_add(sa, d1), df_add(sa, d2),
                                              k * d1.hi, k * d2.hi);
          F = d.F;
          Db = d.Db;
          Dc = d.Dc;
        }
        const float4 ta = tile[6 * e + 3], tb = tile[6 * e + 4], tc = tile[6 * e + 5];
        const float g2 = -2.0f * gam;
        acc[i][0] = fmaf(F.re, g2, acc[i][0]);
        acc[i][1] = fmaf(F.im, g2, acc[i][1]);
        acc[i][2] = fmaf(F.re, ta.w, acc[i][2]);
        acc[i][3] = fmaf(F.im, ta.w, acc[i][3]);
        acc[i][4] = fmaf(F.re, tb.w, acc[i][4]);
        acc[i][5] = fmaf(F.im, tb.w, acc[i][5]);
        acc[i][6] = fmaf(F.re, tc.w, acc[i][6]);
        acc[i][7] = fmaf(F.im, tc.w, acc[i][7]);
        const cf gF = cscale(F, gam), gB = cscale(Db, gam), gC = cscale(Dc, gam);
        const float a0[3] = {ta.x, ta.y, ta.z}, E1[3] = {tb.x, tb.y, tb.z}, E2[3] = {tc.x, tc.y, tc.z};
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          acc[i][8 + 2 * c] = fmaf(-gF.im, a0[c], fmaf(gB.re, E1[c], fmaf(gC.re, E2[c], acc[i][8 + 2 * c])));
          acc[i][9 + 2 * c] = fmaf(gF.re, a0[c], fmaf(gB.im, E1[c], fmaf(gC.im, E2[c], acc[i][9 + 2 * c])));
        }
      }
      if ((e & 15) == 15) flush();
    }
    flush();
  }
  if (!active) return;
  // MF[r][c] = sum_e F_e sum_s grad_s(gamma)_r x0_s[c] = ((khat / 2) x (A (e_c x N~)))_r, N~ = sum_e F_e N0_e
  const double* Am = jo.dofs + 3;  // A row-major
  float Af[9];
#pragma unroll
  for (int a = 0; a < 9; ++a) Af[a] = (float)Am[a];
  const float3 kh = make_float3(0.5f * dh.x * inv_norm, 0.5f * dh.y * inv_norm, 0.5f * dh.z * inv_norm);
  const double so_d = ((double)dh.x + dl.x) * od.origin[0] + ((double)dh.y + dl.y) * od.origin[1] +
                      ((double)dh.z + dl.z) * od.origin[2];
#pragma unroll
  for (int i = 0; i < R; ++i) {
    const int r = rb * R + i;
    if (r >= kg.L) continue;
    const float4 kr = krad[warp][i];
    const float k = kr.x;
    const JacOut o = jac_out(kg, r, j, jm);
    // e^{ik.o} (0 at k = 0, where A = 0 by definition); sqrt|w| at the store
    const cf eo = cis_f64(((double)kr.x + (double)kr.y) * so_d);
    const cf sc = (k * dnorm < 1e-10f) ? cf{0.f, 0.f} : eo;
    float sv[JAC_NSUM];
#pragma unroll
    for (int v = 0; v < JAC_NSUM; ++v) sv[v] = run[(i * JAC_NSUM + v) * JAC_THREADS + threadIdx.x];
    const cf a = cmul(cf{sv[0], sv[1]}, sc);
    float2* out = G + jo.row0 * kg.Q;
#pragma unroll
    for (int rr = 0; rr < 3; ++rr) {  // dA/dt_r = i k d_r A
      const float kd = k * comp(dh, rr);
      o.put(out + (int64_t)rr * kg.Q, cf{-kd * a.im, kd * a.re});
    }
    const cf Nt[3] = {cf{sv[2], sv[3]}, cf{sv[4], sv[5]}, cf{sv[6], sv[7]}};
    cf MF[9];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      cf v[3];  // e_c x N~
      v[c] = cf{0.f, 0.f};
      v[(c + 1) % 3] = cf{-Nt[(c + 2) % 3].re, -Nt[(c + 2) % 3].im};
      v[(c + 2) % 3] = Nt[(c + 1) % 3];
      cf mv[3];  // A v
#pragma unroll
      for (int a3 = 0; a3 < 3; ++a3) {
        const float x0 = Af[3 * a3], x1 = Af[3 * a3 + 1], x2 = Af[3 * a3 + 2];
        mv[a3] = cf{fmaf(x0, v[0].re, fmaf(x1, v[1].re, x2 * v[2].re)), fmaf(x0, v[0].im, fmaf(x1, v[1].im, x2 * v[2].im))};
      }
      MF[c] = cf{kh.y * mv[2].re - kh.z * mv[1].re, kh.y * mv[2].im - kh.z * mv[1].im};
      MF[3 + c] = cf{kh.z * mv[0].re - kh.x * mv[2].re, kh.z * mv[0].im - kh.x * mv[2].im};
      MF[6 + c] = cf{kh.x * mv[1].re - kh.y * mv[0].re, kh.x * mv[1].im - kh.y * mv[0].im};
    }
#pragma unroll
    for (int rr = 0; rr < 3; ++rr)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const cf mf = MF[3 * rr + c], w = cf{sv[8 + 2 * c], sv[9 + 2 * c]};
        const float kd = k * comp(dh, rr);
        const cf v = cmul(cf{-2.0f * (mf.re + kd * w.re), -2.0f * (mf.im + kd * w.im)}, sc);
        o.put(out + (int64_t)(3 + 3 * rr + c) * kg.Q, v);
      }
  }
}

// ---- AffineDoF disks / Gaussians --------------------------------------------------------
__global__ void __launch_bounds__(JAC_THREADS)
jac_affine_surf_kernel(KGridDev kg, BatchDev b, const JacObj* __restrict__ jobs, float2* __restrict__ G) {
  const JacObj jo = jobs[blockIdx.y];
  const ObjDev od = b.objs[jo.obj];
  const JacThread t = jac_thread(kg);
  const bool disk = od.type == PI_GEOM_DISK;
  __shared__ float4 tile[6 * JAC_TILE];
  __shared__ float2 ctab[256];
  stage_cis_tab(kg, ctab);
  // v = A^T dir (k' = |k| v), qd = |v|^2
  const float* Af = od.A;
  const float3 v = make_float3(Af[0] * t.dh.x + Af[3] * t.dh.y + Af[6] * t.dh.z,
                               Af[1] * t.dh.x + Af[4] * t.dh.y + Af[7] * t.dh.z,
                               Af[2] * t.dh.x + Af[5] * t.dh.y + Af[8] * t.dh.z);
  const float qd = fmaf(v.x, v.x, fmaf(v.y, v.y, v.z * v.z));
  kcf A, Z[3], N[3], Y;
  const float4* pool = b.surf_pool + 2 * od.elem_off;
  const float4* pool_lo = b.surf_lo + od.elem_off;
  const float4* pool_nref = b.surf_nref + od.elem_off;
  const SurfSrcJ* src = reinterpret_cast<const SurfSrcJ*>(jo.src);
  const float k = t.k.hi, k2 = k * k;
  for (int base = 0; base < od.n_elems; base += JAC_TILE) {
    const int cnt = min(JAC_TILE, od.n_elems - base);
    __syncthreads();
    for (int e = threadIdx.x; e < cnt; e += JAC_THREADS) {
      tile[4 * e] = pool[2 * (int64_t)(base + e)];
      tile[4 * e + 1] = pool[2 * (int64_t)(base + e) + 1];
      const SurfSrcJ& s = src[base + e];  // reference centre c0 and normal n0
      tile[4 * e + 2] = make_float4((float)s.c[0], (float)s.c[1], (float)s.c[2], 0.f);
      tile[4 * e + 3] = make_float4((float)s.n[0], (float)s.n[1], (float)s.n[2], 0.f);
      tile[4 * JAC_TILE + e] = pool_lo[base + e];  // centre low word
      tile[5 * JAC_TILE + e] = pool_nref[base + e];  // (n / |n|, 1 - |n|^2)
    }
    __syncthreads();
    if (!t.active) continue;
    for (int e = 0; e < cnt; ++e) {
      const float4 q0 = tile[4 * e], q1 = tile[4 * e + 1], c0 = tile[4 * e + 2], n0 = tile[4 * e + 3];
      const float4 cl = tile[4 * JAC_TILE + e];
      const df sc = cdot2(t.dh, t.dl, make_float3(q0.x, q0.y, q0.z), make_float3(cl.x, cl.y, cl.z));
      const float sn = t.dh.x * q1.x + t.dh.y * q1.y + t.dh.z * q1.z;
      // |k'_perp|^2 / |k|^2 = qd (1 - |n|^2) + |n|^2 |v x n/|n||^2 (no cancellation near the normal)
      const float4 nr = tile[5 * JAC_TILE + e];
      const float cx = fmaf(v.y, nr.z, -v.z * nr.y), cy = fmaf(v.z, nr.x, -v.x * nr.z),
                  cz = fmaf(v.x, nr.y, -v.y * nr.x);
      const float perp = fmaxf(fmaf(qd, nr.w, (1.0f - nr.w) * fmaf(cx, cx, fmaf(cy, cy, cz * cz))), 0.f);
      const float amp = sn * t.inv_norm;
      const cf P = cis_tab_df(ctab, t.kt, sc);
      float S, Sr;
      if (disk) {
        const float x = k * q0.w * sqrt_fast(perp);
        S = q1.w * ((x < 1e-10f) ? 1.0f : 2.0f * j1x(x));
        Sr = -2.0f * q1.w * q0.w * q0.w * j2x2(x);
      } else {
        S = q1.w * __expf(-0.5f * q0.w * q0.w * k2 * perp);
        Sr = -q0.w * q0.w * S;
      }
      const float sa = S * amp, sn_t = S - k2 * sn * sn * Sr;
      A.fma_add(P, sa);
      Z[0].fma_add(P, sa * c0.x); Z[1].fma_add(P, sa * c0.y); Z[2].fma_add(P, sa * c0.z);
      N[0].fma_add(P, sn_t * n0.x); N[1].fma_add(P, sn_t * n0.y); N[2].fma_add(P, sn_t * n0.z);
      Y.fma_add(P, amp * Sr);
      if ((e & 15) == 15) {
        A.flush(); Y.flush();
#pragma unroll
        for (int a = 0; a < 3; ++a) { Z[a].flush(); N[a].flush(); }
      }
    }
    A.flush(); Y.flush();
#pragma unroll
    for (int a = 0; a < 3; ++a) { Z[a].flush(); N[a].flush(); }
  }
  if (!t.active) return;
  const JacOut o = jac_out(kg, t.r, t.j, t.jm);
  const cf scl = jac_origin_phase(t, od);
  const double* Am = jo.dofs + 3;  // A row-major
  float atd[3];  // (A^T d)_c = sum_p d_p A_pc
#pragma unroll
  for (int c = 0; c < 3; ++c)
    atd[c] = (float)(t.dh.x * Am[c] + t.dh.y * Am[3 + c] + t.dh.z * Am[6 + c]);
  const cf a = cmul(A.value(), scl), y = Y.value();
  float2* out = G + jo.row0 * kg.Q;
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    const float kr = k * comp(t.dh, r);
    o.put(out + (int64_t)r * kg.Q, cf{-kr * a.im, kr * a.re});
  }
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float dr = comp(t.dh, r);
      const cf z = Z[c].value(), nn = N[c].value();
      // i k d_r Z_c + khat_r N_c + k^2 d_r (A^T d)_c Y
      const float f = k2 * dr * atd[c], g = dr * t.inv_norm, kd = k * dr;
      const cf v = cmul(cf{-kd * z.im + g * nn.re + f * y.re, kd * z.re + g * nn.im + f * y.im}, scl);
      o.put(out + (int64_t)(3 + 3 * r + c) * kg.Q, v);
    }
}

// ---- TriangleMeshDoF: vertex gather --------------------------------------------------------
__global__ void __launch_bounds__(JAC_THREADS)
jac_mesh_kernel(KGridDev kg, BatchDev b, const JacObj* __restrict__ jobs, const int64_t* __restrict__ vrow,
                const int64_t* __restrict__ vent, const int64_t* __restrict__ vmap, float2* __restrict__ G) {
  const JacObj jo = jobs[blockIdx.y];
  const ObjDev od = b.objs[jo.obj];
  const JacThread t = jac_thread(kg);
  __shared__ float2 ctab[256];
  stage_cis_tab(kg, ctab);
  if (!t.active) return;
  const JacOut o = jac_out(kg, t.r, t.j, t.jm);
  const cf scl = jac_origin_phase(t, od);
  const float k = t.k.hi;
  for (int64_t v = jo.vstart; v < jo.vstart + jo.nverts; ++v) {
    float gr[3] = {0.f, 0.f, 0.f}, gi[3] = {0.f, 0.f, 0.f};
    for (int64_t p = vrow[v]; p < vrow[v + 1]; ++p) {
      const int64_t te = vent[p];  // pool triangle * 3 + slot
      const int64_t tri = te / 3;
      const int slot = (int)(te - 3 * tri);
      const float4 q0 = b.tri_pool[3 * tri], q1 = b.tri_pool[3 * tri + 1], q2 = b.tri_pool[3 * tri + 2];
      const float4 ql = b.tri_lo[tri];
      const TriNode o = tri_node(t, ctab, make_float3(q0.x, q0.y, q0.z), ql, make_float3(q1.x, q1.y, q1.z),
                                 make_float3(q2.x, q2.y, q2.z), make_float3(q0.w, q1.w, q2.w));
      const cf D = slot == 0 ? o.d.Da : (slot == 1 ? o.d.Db : o.d.Dc);
      const float3 cs = o.c[slot];
#pragma unroll
      for (int r = 0; r < 3; ++r) {  // df/dv = -2 (c_s F + gamma k d D_s)
        const float cr = comp(cs, r), gk = o.gam * k * comp(t.dh, r);
        gr[r] += -2.0f * (cr * o.d.F.re + gk * D.re);
        gi[r] += -2.0f * (cr * o.d.F.im + gk * D.im);
      }
    }
    const int64_t row = vmap[v];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      o.put(G + (row + r) * kg.Q, cmul(cf{gr[r], gi[r]}, scl));
    }
  }
}

}  // namespace

int launch_jacobian(const pi_kgrid_impl* kg, const pi_batch_impl* b, float2* G, cudaStream_t s) {
  std::vector<JacObj> tri, surf, mesh;
  int64_t row = 0, vstart = 0;
  for (int i = 0; i < b->n_obj; ++i) {
    const HostObjInfo& in = b->info[i];
    JacObj o{};
    o.obj = i;
    o.row0 = row;
    o.src = static_cast<const unsigned char*>(b->d_src) + in.src_off;
    o.dofs = b->d_dofs + in.dof_off;
    if (in.dof_type == PI_DOF_TRIANGLE_MESH) {
      o.kind = JAC_MESH_TRI;
      o.vstart = vstart;
      o.nverts = in.n_dofs / 3;
      vstart += o.nverts;
      mesh.push_back(o);
    } else if (in.n_dofs != 12) {
      return fail(PI_ERR_UNSUPPORTED, "the Jacobian supports AffineDoF (12) and TriangleMeshDoF objects");
    } else if (in.geom_type == PI_GEOM_TRIANGLE) {
      o.kind = JAC_AFFINE_TRI;
      tri.push_back(o);
    } else {
      o.kind = JAC_AFFINE_SURF;
      surf.push_back(o);
    }
    row += in.n_dofs;
  }
  if (!mesh.empty() && !b->d_vrow) return fail(PI_ERR_UNSUPPORTED, "vertex adjacency missing for TriangleMeshDoF objects");
  const size_t nj = tri.size() + surf.size() + mesh.size();
  if (nj == 0) return PI_OK;
  if (nj > 65535) return fail(PI_ERR_UNSUPPORTED, "more than 65535 objects in one Jacobian");
  std::vector<JacObj> all(tri);
  all.insert(all.end(), surf.begin(), surf.end());
  all.insert(all.end(), mesh.begin(), mesh.end());
  JacObj* d = nullptr;
  PI_CUDA(cudaMallocAsync((void**)&d, nj * sizeof(JacObj), s));
  PI_CUDA(cudaMemcpyAsync(d, all.data(), nj * sizeof(JacObj), cudaMemcpyHostToDevice, s));
  const KGridDev K = kg->dev;
  const BatchDev B = b->dev();
  const unsigned gx = (unsigned)(((int64_t)((K.Me + 31) / 32) * K.L + JAC_WARPS - 1) / JAC_WARPS);
  if (!tri.empty()) {
    // the most radii per thread that still gives two waves of CTAs
    const int n_sm = current_sm_count();
    auto ctas = [&](int R) {
      return (int64_t)(((int64_t)((K.L + R - 1) / R) * ((K.Me + 31) / 32) + JAC_WARPS - 1) / JAC_WARPS);
    };
    const int64_t wave = (int64_t)n_sm * 3;
    const int R = ctas(4) * (int64_t)tri.size() >= 2 * wave ? 4 : ctas(2) * (int64_t)tri.size() >= 2 * wave ? 2 : 1;
    const dim3 grid((unsigned)ctas(R), (unsigned)tri.size());
    if (R == 4) jac_affine_tri_kernel<4><<<grid, JAC_THREADS, 0, s>>>(K, B, d, G);
    else if (R == 2) jac_affine_tri_kernel<2><<<grid, JAC_THREADS, 0, s>>>(K, B, d, G);
    else jac_affine_tri_kernel<1><<<grid, JAC_THREADS, 0, s>>>(K, B, d, G);
    PI_LAUNCHED("jac_affine_tri_kernel");
  }
  if (!surf.empty()) {
    jac_affine_surf_kernel<<<dim3(gx, (unsigned)surf.size()), JAC_THREADS, 0, s>>>(K, B, d + tri.size(), G);
    PI_LAUNCHED("jac_affine_surf_kernel");
  }
  if (!mesh.empty()) {
    jac_mesh_kernel<<<dim3(gx, (unsigned)mesh.size()), JAC_THREADS, 0, s>>>(K, B, d + tri.size() + surf.size(),
                                                                             b->d_vrow, b->d_vent, b->d_vmap, G);
    PI_LAUNCHED("jac_mesh_kernel");
  }
  PI_CUDA(cudaFreeAsync(d, s));
  return PI_OK;
}

}  // namespace pi
