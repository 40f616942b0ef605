// Adjoint of the Fourier intersection volume: gradients of L = sum_ij C_ij V_ij.
//
// dL/dtheta_n = (1/8 pi^3) sum_q w_q Re( dA_n(k_q)/dtheta_n  conj(B_n(k_q)) ),
// B_n = sum_j W_nj A_j  (the cotangent).  For L = sum_ij C_ij V_ij, W = C + C^T;
// W = e_j 1^T-style single columns give the reference's per-pair gradients
// dV_ij/dtheta_i (B_i = A_j for every i).
//
// Replaces the reference's gradient kernels K4-K6, K8, K10 and K15
// (cpp/src/dof/cuda/affine_dof_cuda.cu:254-576, 693-849;
//  cpp/src/dof/cuda/triangle_mesh_dof_cuda.cu:147-310;
//  cpp/src/compute_intersection_volume.cu:60-101;
//  cpp/src/compute_intersection_volume_multi_object.cu:124-176), which
// materialised dA/dtheta for every k-node (Q x 3V complex doubles for a mesh:
// ~9.5 GB for an icosphere-4 at N_k = 76,928) and reduced it with FP64
// atomics.  Here nothing of size Q x (parameters) exists:
//
//  * cotangent_kernel: B^ = W J^ on the sqrt|w|-scaled J (one pass over J);
//  * adj_surf_kernel / adj_tri_kernel: one thread per element; the CTA's
//    elements share one object, so the cotangent of a tile of directions is
//    staged once in shared memory (with the object's origin phase and the
//    quadrature weight folded in) and read as broadcasts, while every thread
//    recomputes its element's form factor and derivatives at each k-node and
//    accumulates the element's parameter gradient in registers; of two
//    antipodal directions only one is evaluated, the other's cotangent folded
//    into it (stage_tile);
//  * chain kernels turn element gradients into AffineDoF gradients (fixed
//    order FP64 block reduction per object) or TriangleMeshDoF vertex
//    gradients (CSR gather per vertex, no atomics): results are bitwise
//    reproducible.
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

constexpr int ADJ_THREADS = 128;
constexpr int ADJ_DT = 8;        // directions staged per shared-memory tile
constexpr int ADJ_LMAX = 256;    // radii per direction held in shared memory
constexpr double INV8PI3 = 1.0 / (8.0 * 3.14159265358979323846 * 3.14159265358979323846 * 3.14159265358979323846);

// Kahan-compensated FP32 accumulator.
struct kf {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float x) {
    const float y = x - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
  }
};

// B^[n][q] = sum_j W[n][j] J^[j][q]; grid (q blocks, n blocks of 16).
__global__ void cotangent_kernel(const float2* __restrict__ Jw, const float* __restrict__ Cs, int n, int64_t Q,
                                 float2* __restrict__ Bw) {
  __shared__ float cs[16][64];
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int n0 = blockIdx.y * 16;
  float2 acc[16];
#pragma unroll
  for (int a = 0; a < 16; ++a) acc[a] = make_float2(0.f, 0.f);
  for (int j0 = 0; j0 < n; j0 += 64) {
    __syncthreads();
    for (int t = threadIdx.x; t < 16 * 64; t += blockDim.x) {
      const int a = t / 64, jj = t % 64;
      cs[a][jj] = (n0 + a < n && j0 + jj < n) ? Cs[(int64_t)(n0 + a) * n + j0 + jj] : 0.f;
    }
    __syncthreads();
    if (q < Q) {
      const int jn = min(64, n - j0);
      for (int jj = 0; jj < jn; ++jj) {
        const float2 v = Jw[(int64_t)(j0 + jj) * Q + q];
#pragma unroll
        for (int a = 0; a < 16; ++a) {
          acc[a].x = fmaf(cs[a][jj], v.x, acc[a].x);
          acc[a].y = fmaf(cs[a][jj], v.y, acc[a].y);
        }
      }
    }
  }
  if (q < Q)
#pragma unroll
    for (int a = 0; a < 16; ++a)
      if (n0 + a < n) Bw[(int64_t)(n0 + a) * Q + q] = acc[a];
}

struct AdjWork { int32_t obj, first; };

// Shared staging of one direction tile: cotangent with sign(w) sqrt|w| and the
// origin phase e^{-ik.o} folded in (zero at k = 0 nodes, where A = 0 by
// definition), plus the directions.
struct AdjStage {
  float2 B[ADJ_DT * ADJ_LMAX];
  float4 dh[ADJ_DT], dl[ADJ_DT];
  float4 va[ADJ_DT];  // v = A^T dir and qd = |v|^2 (disks/Gaussians: k' = |k| v)
  double so[ADJ_DT];  // dir . origin
  int2 jp[ADJ_DT];    // (direction, its antipode or -1); -1, -1 past the last direction
};

// Per-CTA copies of the radii (double-float |k|, and |k| in 1/256 turns per
// unit length for the table phasors) and of the phasor table; the first
// __syncthreads of the direction loop publishes them.
__device__ __forceinline__ void stage_radii(const KGridDev& kg, float2* km, float2* kt, float2* ctab) {
  for (int r = threadIdx.x; r < kg.L; r += blockDim.x) {
    km[r] = kg.kmag[r];
    kt[r] = kg.kt256[r];
  }
  for (int t = threadIdx.x; t < 256; t += blockDim.x) ctab[t] = kg.cis_tab[t];
}

// The tile holds evaluated directions e0 .. e0 + ADJ_DT - 1 (KGridDev::dpair).
// A direction's antipode contributes Re(conj(B') dA(-k)) with
// dA(-k) = -conj dA(k) for every real parameter, which is
// Re(conj(-conj B') dA(k)): the staged cotangent is B - conj(B') (each with
// its own weight and origin phase) and the antipode is never evaluated.
__device__ __forceinline__ void stage_tile(AdjStage& st, const KGridDev& kg, const ObjDev& od, const float2* Bw_obj,
                                           const float2* km, int e0) {
  const int tid = threadIdx.x;
  if (tid < ADJ_DT) {
    const int e = e0 + tid;
    float4 h = make_float4(0.f, 0.f, 0.f, 0.f), l = h;
    int2 jp = make_int2(-1, -1);
    if (e < kg.Me) { jp = kg.dpair[e]; h = kg.dir_hi[jp.x]; l = kg.dir_lo[jp.x]; }
    st.jp[tid] = jp;
    st.dh[tid] = h;
    st.dl[tid] = l;
    const float* Am = od.A;
    const float vx = Am[0] * h.x + Am[3] * h.y + Am[6] * h.z, vy = Am[1] * h.x + Am[4] * h.y + Am[7] * h.z,
                vz = Am[2] * h.x + Am[5] * h.y + Am[8] * h.z;
    st.va[tid] = make_float4(vx, vy, vz, fmaf(vx, vx, fmaf(vy, vy, vz * vz)));
    const double so = ((double)h.x + l.x) * od.origin[0] + ((double)h.y + l.y) * od.origin[1] +
                      ((double)h.z + l.z) * od.origin[2];
    st.so[tid] = so;
  }
  __syncthreads();
  for (int t = tid; t < ADJ_DT * kg.L; t += blockDim.x) {
    const int jj = t / kg.L, r = t % kg.L;
    const int2 jp = st.jp[jj];
    float2 v = make_float2(0.f, 0.f);
    if (jp.x >= 0) {
      const int64_t q = (int64_t)r * kg.M + jp.x;
      const df k = df{km[r].x, km[r].y};
      if (k.hi * st.dl[jj].w >= 1e-10f) {
        const float2 b = Bw_obj[q];
        const float s = kg.sqrtw[q] * (kg.sign ? kg.sign[q] : 1.f);
        const cf e = cis_f64(((double)k.hi + (double)k.lo) * st.so[jj]);  // e^{ik.o}
        // B e^{-ik.o} scaled: (b.x + i b.y)(e.re - i e.im)
        v = make_float2(s * (b.x * e.re + b.y * e.im), s * (b.y * e.re - b.x * e.im));
        if (jp.y >= 0) {  // minus conj of the antipode's B' e^{+ik.o}, scaled
          const int64_t qm = (int64_t)r * kg.M + jp.y;
          const float2 bm = Bw_obj[qm];
          const float sm = kg.sqrtw[qm] * (kg.sign ? kg.sign[qm] : 1.f);
          v.x -= sm * (bm.x * e.re - bm.y * e.im);
          v.y += sm * (bm.y * e.re + bm.x * e.im);
        }
      }
    }
    st.B[jj * ADJ_LMAX + r] = v;
  }
  __syncthreads();
}

// Per disk / Gaussian: 12 outputs dL/dc (3), dL/dn' (3), dL/dM (6, M = A A^T,
// entries xx xy xz yy yz zz of a symmetric gradient).
//   A = e^{ik.c} S(r) (k.n')/|k|,  r^2 = k^T M k - (k.n')^2,
//   dA/dc  = i k A
//   dA/dn' = e^{ik.c} khat [S - (k.n')^2 (dS/dr)/r]
//   dA/dM  = e^{ik.c} (k.n')/|k| (dS/dr)/(2r) k k^T
// Disk S = area 2 J1(rho r)/(rho r), (dS/dr)/r = -2 area rho^2 J2(x)/x^2;
// Gaussian S = w exp(-sigma^2 r^2/2), (dS/dr)/r = -sigma^2 S.
__global__ void __launch_bounds__(ADJ_THREADS)
adj_surf_kernel(KGridDev kg, BatchDev b, const AdjWork* __restrict__ work, const float2* __restrict__ Bw,
                float* __restrict__ out) {
  __shared__ AdjStage st;
  __shared__ float2 km[ADJ_LMAX], kt[ADJ_LMAX], ctab[256];
  const AdjWork wk = work[blockIdx.x];
  const ObjDev od = b.objs[wk.obj];
  const int e = wk.first + threadIdx.x;
  const bool valid = e < od.n_elems;
  const bool disk = od.type == PI_GEOM_DISK;
  stage_radii(kg, km, kt, ctab);
  float4 q0 = make_float4(0.f, 0.f, 0.f, 0.f), q1 = q0, ql = q0, nr = q0;
  if (valid) {
    q0 = b.surf_pool[2 * (od.elem_off + e)];
    q1 = b.surf_pool[2 * (od.elem_off + e) + 1];
    ql = b.surf_lo[od.elem_off + e];
    nr = b.surf_nref[od.elem_off + e];
  }
  const float3 c = make_float3(q0.x, q0.y, q0.z), nn = make_float3(q1.x, q1.y, q1.z);
  const float3 cl = make_float3(ql.x, ql.y, ql.z);  // centre low word
  const float p0 = q0.w, p1 = q1.w;
  kf gc[3], gn[3], gm[6];
  const float2* Bw_obj = Bw + (int64_t)wk.obj * kg.Q;
  for (int j0 = 0; j0 < kg.Me; j0 += ADJ_DT) {
    __syncthreads();
    stage_tile(st, kg, od, Bw_obj, km, j0);
    if (!valid) continue;
    const int jn = min(ADJ_DT, kg.Me - j0);
    for (int jj = 0; jj < jn; ++jj) {
      const float4 h = st.dh[jj], l = st.dl[jj];
      const float3 dh = make_float3(h.x, h.y, h.z), dl = make_float3(l.x, l.y, l.z);
      const float inv_norm = h.w;
      const df sc = cdot2(dh, dl, c, cl);
      const float sn = dh.x * nn.x + dh.y * nn.y + dh.z * nn.z;
      // |k'_perp|^2 / |k|^2 = qd (1 - |n|^2) + |n|^2 |v x n/|n||^2 (no cancellation near the normal)
      const float4 va = st.va[jj];
      const float cx = fmaf(va.y, nr.z, -va.z * nr.y), cy = fmaf(va.z, nr.x, -va.x * nr.z),
                  cz = fmaf(va.x, nr.y, -va.y * nr.x);
      const float perp = fmaxf(fmaf(va.w, nr.w, (1.0f - nr.w) * fmaf(cx, cx, fmaf(cy, cy, cz * cz))), 0.f);
      const float rr = p0 * sqrt_fast(perp);
      const float amp = sn * inv_norm;
      float s_c = 0.f, s_n = 0.f, s_m = 0.f;
      const float2* Bj = st.B + jj * ADJ_LMAX;
#pragma unroll 2
      for (int r = 0; r < kg.L; ++r) {
        const float2 Bv = Bj[r];
        const df k = df{km[r].x, km[r].y};
        const cf P = cis_tab_df(ctab, kt[r], sc);
        const float ure = Bv.x * P.re + Bv.y * P.im;  // Re(conj(B) P)
        const float uim = Bv.x * P.im - Bv.y * P.re;  // Im(conj(B) P)
        const float k2 = k.hi * k.hi;
        float S, Sr;
        if (disk) {
          const float x = k.hi * rr;
          S = p1 * ((x < 1e-10f) ? 1.0f : 2.0f * j1x(x));
          Sr = -2.0f * p1 * p0 * p0 * j2x2(x);
        } else {
          S = p1 * __expf(-0.5f * p0 * p0 * k2 * perp);
          Sr = -p0 * p0 * S;
        }
        s_c = fmaf(-k.hi * uim, S * amp, s_c);
        s_n = fmaf(ure, fmaf(-k2 * sn * sn, Sr, S), s_n);
        s_m = fmaf(k2 * ure, 0.5f * amp * Sr, s_m);
      }
      gc[0].add(dh.x * s_c); gc[1].add(dh.y * s_c); gc[2].add(dh.z * s_c);
      const float sn2 = s_n * inv_norm;
      gn[0].add(dh.x * sn2); gn[1].add(dh.y * sn2); gn[2].add(dh.z * sn2);
      gm[0].add(dh.x * dh.x * s_m); gm[1].add(dh.x * dh.y * s_m); gm[2].add(dh.x * dh.z * s_m);
      gm[3].add(dh.y * dh.y * s_m); gm[4].add(dh.y * dh.z * s_m); gm[5].add(dh.z * dh.z * s_m);
    }
  }
  if (!valid) return;
  float* o = out + 12 * (od.elem_off + e);
  const float sc8 = (float)INV8PI3;
  for (int a = 0; a < 3; ++a) { o[a] = gc[a].s * sc8; o[3 + a] = gn[a].s * sc8; }
  for (int a = 0; a < 6; ++a) o[6 + a] = gm[a].s * sc8;
}

// Per triangle: 9 outputs dL/dv0, dL/dv1, dL/dv2 (world-frame vertex positions).
__global__ void __launch_bounds__(ADJ_THREADS, 4)
adj_tri_kernel(KGridDev kg, BatchDev b, const AdjWork* __restrict__ work, const float2* __restrict__ Bw,
               float* __restrict__ out) {
  __shared__ AdjStage st;
  __shared__ float2 km[ADJ_LMAX], kt[ADJ_LMAX], ctab[256];
  const AdjWork wk = work[blockIdx.x];
  const ObjDev od = b.objs[wk.obj];
  const int e = wk.first + threadIdx.x;
  const bool valid = e < od.n_elems;
  stage_radii(kg, km, kt, ctab);
  float4 q0 = make_float4(0.f, 0.f, 0.f, 0.f), q1 = q0, q2 = q0, ql = q0;
  if (valid) {
    q0 = b.tri_pool[3 * (od.elem_off + e)];
    q1 = b.tri_pool[3 * (od.elem_off + e) + 1];
    q2 = b.tri_pool[3 * (od.elem_off + e) + 2];
    ql = b.tri_lo[od.elem_off + e];
  }
  const float3 ml = make_float3(ql.x, ql.y, ql.z);  // centroid low word
  const float3 m = make_float3(q0.x, q0.y, q0.z), e1 = make_float3(q1.x, q1.y, q1.z),
               e2 = make_float3(q2.x, q2.y, q2.z), S = make_float3(q0.w, q1.w, q2.w);
  kf g[9];
  const float2* Bw_obj = Bw + (int64_t)wk.obj * kg.Q;
  for (int j0 = 0; j0 < kg.Me; j0 += ADJ_DT) {
    __syncthreads();
    stage_tile(st, kg, od, Bw_obj, km, j0);
    if (!valid) continue;
    const int jn = min(ADJ_DT, kg.Me - j0);
    for (int jj = 0; jj < jn; ++jj) {
      const float4 h = st.dh[jj], l = st.dl[jj];
      const float3 dh = make_float3(h.x, h.y, h.z), dl = make_float3(l.x, l.y, l.z);
      const float inv_norm = h.w;
      const df sm = cdot2(dh, dl, m, ml), d1 = cdot(dh, dl, e1), d2 = cdot(dh, dl, e2);
      const df sa = df_add(sm, df_div3(df_add(d1, d2)) * -1.0f);
      const df sb = df_add(sa, d1), sc = df_add(sa, d2);
      const float sp = fmaxf(fmaxf(fabsf(d1.hi), fabsf(d2.hi)), fabsf(d2.hi - d1.hi));
      const float kthr = __fdividef(2.0f, sp);  // the series for k sp < 2 (inf when sp = 0)
      const float gam = (dh.x * S.x + dh.y * S.y + dh.z * S.z) * inv_norm;
      const TriDerPoly cp = tri_der_coeffs(d1.hi, d2.hi);
      float t0 = 0.f, ta = 0.f, tb = 0.f, tc = 0.f;
      const float2* Bj = st.B + jj * ADJ_LMAX;
      for (int r = 0; r < kg.L; ++r) {
        const float2 Bv = Bj[r];
        const df k = df{km[r].x, km[r].y};
        if (k.hi < kthr) {
          // F = P SF, D_v = P SV with the series as polynomials in k; with
          // BP = conj(B) P, Re(conj(B) X) = Re(BP SX) and D_a = i F - D_b - D_c
          const cf P = cis_tab_df(ctab, kt[r], sm);
          const float u = k.hi * k.hi, k3 = u * k.hi;
          const float fre = poly_u(cp.fa, u), fim = k3 * poly_u(cp.fb, u);
          const float bim = poly_u(cp.ba, u), bre = k.hi * poly_u(cp.bb, u);
          const float cim = poly_u(cp.ca, u), cre = k.hi * poly_u(cp.cb, u);
          const float pr = fmaf(Bv.x, P.re, Bv.y * P.im), pi = fmaf(Bv.x, P.im, -Bv.y * P.re);
          const float f_re = fmaf(pr, fre, -pi * fim), f_im = fmaf(pr, fim, pi * fre);
          const float b_re = fmaf(pr, bre, -pi * bim), c_re = fmaf(pr, cre, -pi * cim);
          t0 += f_re;
          ta = fmaf(k.hi, -f_im - b_re - c_re, ta);
          tb = fmaf(k.hi, b_re, tb);
          tc = fmaf(k.hi, c_re, tc);
        } else {
          const TriDer d = tri_generic_der_at(ctab, kt[r], sa, sb, sc, k.hi * d1.hi, k.hi * d2.hi);
          // Re(conj(B) X) = B.re X.re + B.im X.im
          t0 = fmaf(Bv.x, d.F.re, fmaf(Bv.y, d.F.im, t0));
          ta = fmaf(k.hi, fmaf(Bv.x, d.Da.re, Bv.y * d.Da.im), ta);
          tb = fmaf(k.hi, fmaf(Bv.x, d.Db.re, Bv.y * d.Db.im), tb);
          tc = fmaf(k.hi, fmaf(Bv.x, d.Dc.re, Bv.y * d.Dc.im), tc);
        }
      }
      // khat x u / 2 terms for grad gamma
      const float3 kh = make_float3(dh.x * inv_norm, dh.y * inv_norm, dh.z * inv_norm);
      const float3 w0 = make_float3(e2.x - e1.x, e2.y - e1.y, e2.z - e1.z);
      const float3 c0 = make_float3(0.5f * (kh.y * w0.z - kh.z * w0.y), 0.5f * (kh.z * w0.x - kh.x * w0.z),
                                    0.5f * (kh.x * w0.y - kh.y * w0.x));
      const float3 c1 = make_float3(-0.5f * (kh.y * e2.z - kh.z * e2.y), -0.5f * (kh.z * e2.x - kh.x * e2.z),
                                    -0.5f * (kh.x * e2.y - kh.y * e2.x));
      const float3 c2 = make_float3(0.5f * (kh.y * e1.z - kh.z * e1.y), 0.5f * (kh.z * e1.x - kh.x * e1.z),
                                    0.5f * (kh.x * e1.y - kh.y * e1.x));
      // dL/dv = -2 (grad gamma t0 + gamma dir t_v)
      g[0].add(-2.f * (c0.x * t0 + gam * dh.x * ta)); g[1].add(-2.f * (c0.y * t0 + gam * dh.y * ta));
      g[2].add(-2.f * (c0.z * t0 + gam * dh.z * ta));
      g[3].add(-2.f * (c1.x * t0 + gam * dh.x * tb)); g[4].add(-2.f * (c1.y * t0 + gam * dh.y * tb));
      g[5].add(-2.f * (c1.z * t0 + gam * dh.z * tb));
      g[6].add(-2.f * (c2.x * t0 + gam * dh.x * tc)); g[7].add(-2.f * (c2.y * t0 + gam * dh.y * tc));
      g[8].add(-2.f * (c2.z * t0 + gam * dh.z * tc));
    }
  }
  if (!valid) return;
  float* o = out + 9 * (od.elem_off + e);
  const float sc8 = (float)INV8PI3;
#pragma unroll
  for (int a = 0; a < 9; ++a) o[a] = g[a].s * sc8;
}

// ---- chain rule to DoF gradients ---------------------------------------------------
struct ChainObj {
  int32_t geom_type, dof_type;
  int64_t n_elems, pool_off, grad_off;   // grad_off: offset (doubles) of this object's DoF gradient
  const unsigned char* src;             // reference-layout packed source
  const double* dofs;
};

struct TriSrcC { double a[3], e1[3], e2[3], S[3]; int32_t vid0, vid1, vid2, pad; };
struct SurfSrcC { double c[3], n[3], p0, p1; };

// AffineDoF: one CTA per object, fixed-order FP64 reduction.
//   triangles: dL/dt = sum_v g_v, dL/dA = sum_v g_v v_ref^T  (v = A v_ref + t)
//   surfels:   dL/dt = sum g_c, dL/dA = sum g_c c_ref^T + g_n n_ref^T + 2 G_M A
__global__ void chain_affine_kernel(const ChainObj* objs, const float* __restrict__ tri_g,
                                    const float* __restrict__ surf_g, double* __restrict__ grad) {
  const ChainObj o = objs[blockIdx.x];
  if (o.dof_type != PI_DOF_AFFINE) return;
  __shared__ double red[18][128];
  double acc[18];
#pragma unroll
  for (int a = 0; a < 18; ++a) acc[a] = 0.0;
  for (int64_t e = threadIdx.x; e < o.n_elems; e += blockDim.x) {
    if (o.geom_type == PI_GEOM_TRIANGLE) {
      const TriSrcC& t = reinterpret_cast<const TriSrcC*>(o.src)[e];
      const float* g = tri_g + 9 * (o.pool_off + e);
      const double v[3][3] = {{t.a[0], t.a[1], t.a[2]},
                              {t.a[0] + t.e1[0], t.a[1] + t.e1[1], t.a[2] + t.e1[2]},
                              {t.a[0] + t.e2[0], t.a[1] + t.e2[1], t.a[2] + t.e2[2]}};
      for (int s = 0; s < 3; ++s)
        for (int r = 0; r < 3; ++r) {
          const double gv = g[3 * s + r];
          acc[r] += gv;
          for (int c = 0; c < 3; ++c) acc[3 + 3 * r + c] += gv * v[s][c];
        }
    } else {
      const SurfSrcC& s = reinterpret_cast<const SurfSrcC*>(o.src)[e];
      const float* g = surf_g + 12 * (o.pool_off + e);
      for (int r = 0; r < 3; ++r) {
        acc[r] += g[r];
        for (int c = 0; c < 3; ++c) acc[3 + 3 * r + c] += (double)g[r] * s.c[c] + (double)g[3 + r] * s.n[c];
      }
      for (int a = 0; a < 6; ++a) acc[12 + a] += g[6 + a];
    }
  }
  for (int a = 0; a < 18; ++a) red[a][threadIdx.x] = acc[a];
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w)
      for (int a = 0; a < 18; ++a) red[a][threadIdx.x] += red[a][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    double* out = grad + o.grad_off;
    for (int a = 0; a < 12; ++a) out[a] = red[a][0];
    if (o.geom_type != PI_GEOM_TRIANGLE) {
      // + 2 G A with G symmetric (xx xy xz yy yz zz)
      const double G[3][3] = {{red[12][0], red[13][0], red[14][0]},
                              {red[13][0], red[15][0], red[16][0]},
                              {red[14][0], red[16][0], red[17][0]}};
      const double* A = o.dofs + 3;
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c)
          out[3 + 3 * r + c] += 2.0 * (G[r][0] * A[c] + G[r][1] * A[3 + c] + G[r][2] * A[6 + c]);
    }
  }
}

// TriangleMeshDoF: one thread per vertex, CSR gather of (triangle, slot) gradients.
__global__ void chain_mesh_kernel(const int64_t* __restrict__ row, const int64_t* __restrict__ ent,
                                  const float* __restrict__ tri_g, int64_t nv_total, const int64_t* __restrict__ vmap,
                                  double* __restrict__ grad) {
  const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv_total) return;
  double s[3] = {0.0, 0.0, 0.0};
  for (int64_t p = row[v]; p < row[v + 1]; ++p) {
    const int64_t te = ent[p];  // pool triangle * 3 + slot
    const float* g = tri_g + 9 * (te / 3) + 3 * (te % 3);
    s[0] += g[0]; s[1] += g[1]; s[2] += g[2];
  }
  double* o = grad + vmap[v];
  o[0] = s[0]; o[1] = s[1]; o[2] = s[2];
}

}  // namespace

// ---- host side ------------------------------------------------------------------------
int64_t dof_gradient_size(const pi_batch_impl* b) {
  int64_t s = 0;
  for (const HostObjInfo& in : b->info) s += in.n_dofs;
  return s;
}

size_t adjoint_ws_bytes(const pi_kgrid_impl* kg, const pi_batch_impl* b) {
  const size_t nb = (size_t)b->n_obj * kg->Q * sizeof(float2);            // cotangent
  const size_t cs = (size_t)b->n_obj * b->n_obj * sizeof(float);           // C + C^T
  const size_t tg = (size_t)b->n_tri * 9 * sizeof(float), sg = (size_t)b->n_surf * 12 * sizeof(float);
  return 256 + nb + 256 + cs + 256 + tg + 256 + sg + 256;
}

static size_t up256(size_t x) { return (x + 255) & ~size_t(255); }

int launch_adjoint_elements(const pi_kgrid_impl* kg, const pi_batch_impl* b, const float2* Jw, const double* W_host,
                            float** tri_g_out, float** surf_g_out, void* ws, size_t ws_bytes, cudaStream_t s) {
  if (kg->L > ADJ_LMAX) return fail(PI_ERR_UNSUPPORTED, "adjoint supports at most 256 radial nodes");
  if (ws_bytes < adjoint_ws_bytes(kg, b) || !ws) return fail(PI_ERR_WORKSPACE_TOO_SMALL, "adjoint workspace too small");
  const int n = b->n_obj;
  unsigned char* p = static_cast<unsigned char*>(ws);
  float2* Bw = reinterpret_cast<float2*>(p);
  p += up256((size_t)n * kg->Q * sizeof(float2));
  float* Cs = reinterpret_cast<float*>(p);
  p += up256((size_t)n * n * sizeof(float));
  float* tri_g = reinterpret_cast<float*>(p);
  p += up256((size_t)b->n_tri * 9 * sizeof(float));
  float* surf_g = reinterpret_cast<float*>(p);
  std::vector<float> cs((size_t)n * n);
  for (size_t t = 0; t < cs.size(); ++t) cs[t] = (float)W_host[t];
  PI_CUDA(cudaMemcpyAsync(Cs, cs.data(), cs.size() * sizeof(float), cudaMemcpyHostToDevice, s));
  dim3 cg((unsigned)((kg->Q + 255) / 256), (unsigned)((n + 15) / 16));
  cotangent_kernel<<<cg, 256, 0, s>>>(Jw, Cs, n, kg->Q, Bw);
  PI_LAUNCHED("cotangent_kernel");
  std::vector<AdjWork> wt, ws2;
  for (int i = 0; i < n; ++i) {
    const HostObjInfo& in = b->info[i];
    for (int64_t f = 0; f < in.n_elems; f += ADJ_THREADS)
      (in.geom_type == PI_GEOM_TRIANGLE ? wt : ws2).push_back(AdjWork{i, (int32_t)f});
  }
  AdjWork* dw = nullptr;
  const size_t nw = wt.size() + ws2.size();
  if (nw) {
    PI_CUDA(cudaMallocAsync((void**)&dw, nw * sizeof(AdjWork), s));
    std::vector<AdjWork> all(wt);
    all.insert(all.end(), ws2.begin(), ws2.end());
    PI_CUDA(cudaMemcpyAsync(dw, all.data(), nw * sizeof(AdjWork), cudaMemcpyHostToDevice, s));
    if (!wt.empty()) {
      adj_tri_kernel<<<(unsigned)wt.size(), ADJ_THREADS, 0, s>>>(kg->dev, b->dev(), dw, Bw, tri_g);
      PI_LAUNCHED("adj_tri_kernel");
    }
    if (!ws2.empty()) {
      adj_surf_kernel<<<(unsigned)ws2.size(), ADJ_THREADS, 0, s>>>(kg->dev, b->dev(), dw + wt.size(), Bw, surf_g);
      PI_LAUNCHED("adj_surf_kernel");
    }
    PI_CUDA(cudaFreeAsync(dw, s));
  }
  *tri_g_out = tri_g;
  *surf_g_out = surf_g;
  return PI_OK;
}

int launch_dof_gradients(const pi_kgrid_impl* kg, pi_batch_impl* b, const float2* Jw, const double* W_host,
                         double* grad, void* ws, size_t ws_bytes, cudaStream_t s) {
  float *tri_g = nullptr, *surf_g = nullptr;
  int rc = launch_adjoint_elements(kg, b, Jw, W_host, &tri_g, &surf_g, ws, ws_bytes, s);
  if (rc) return rc;
  const int n = b->n_obj;
  std::vector<ChainObj> co(n);
  int64_t goff = 0;
  bool any_mesh = false;
  for (int i = 0; i < n; ++i) {
    const HostObjInfo& in = b->info[i];
    co[i] = ChainObj{in.geom_type, in.dof_type, in.n_elems, in.pool_off, goff,
                     static_cast<const unsigned char*>(b->d_src) + in.src_off, b->d_dofs + in.dof_off};
    goff += in.n_dofs;
    any_mesh |= in.dof_type == PI_DOF_TRIANGLE_MESH;
  }
  ChainObj* dco = nullptr;
  PI_CUDA(cudaMallocAsync((void**)&dco, n * sizeof(ChainObj), s));
  PI_CUDA(cudaMemcpyAsync(dco, co.data(), n * sizeof(ChainObj), cudaMemcpyHostToDevice, s));
  chain_affine_kernel<<<n, 128, 0, s>>>(dco, tri_g, surf_g, grad);
  PI_LAUNCHED("chain_affine_kernel");
  PI_CUDA(cudaFreeAsync(dco, s));
  if (any_mesh) {
    if (!b->d_vrow) return fail(PI_ERR_UNSUPPORTED, "vertex adjacency missing for TriangleMeshDoF objects");
    chain_mesh_kernel<<<(unsigned)((b->n_mesh_verts + 255) / 256), 256, 0, s>>>(b->d_vrow, b->d_vent, tri_g,
                                                                               b->n_mesh_verts, b->d_vmap, grad);
    PI_LAUNCHED("chain_mesh_kernel");
  }
  return PI_OK;
}

}  // namespace pi
