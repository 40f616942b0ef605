// Per-object form factors A_n(k_q) on the device.
//
// Replaces the reference kernels K1-K3 (cpp/src/dof/cuda/affine_dof_cuda.cu:43-250,
// 580-689) and K7 (cpp/src/dof/cuda/triangle_mesh_dof_cuda.cu:34-143), whose
// grid was one CTA per k-node looping over every element in FP64 with a shared
// memory tree reduction.  Here:
//
//  * prepare_*: each object's elements are transformed once per DoF change by
//    its AffineDoF / TriangleMeshDoF into an FP32 object-local frame (origin =
//    centroid of the transformed anchors), centroids (centres) as FP32 hi + lo;
//    the origin phase e^{ik.o} is formed and reduced in FP64 per output.
//  * ff_kernel: one CTA = one object x 4 warps; a warp owns 32 directions
//    (one per lane) x R neighbouring radial nodes of the factored k-grid, so
//    each element's direction dot products and series coefficients are
//    formed once and reused for R radii; where all R radii take the short
//    series, two radii share each packed FP32 instruction.  On a centrally
//    symmetric direction set a lane evaluates one direction of an antipodal
//    pair and writes both (A(-k) = -conj A(k) for a real solid: half the
//    evaluations), and a warp's 32 directions form a compact cluster.  Radial
//    blocks start largest-k first, for all objects.  Elements are staged
//    through shared memory and read as broadcasts; each thread accumulates
//    its own outputs (no reduction across threads), 32-element partials in
//    registers and compensated running sums in shared memory; each output
//    element is written once, in the contraction's operand layout.
#include <cuda_runtime.h>
#include <cstdint>
#include <algorithm>
#include "pi_internal.h"
#include "dfmath.cuh"
#include "bessel.cuh"

namespace pi {

namespace {

struct TriSrc { double a[3], e1[3], e2[3], S[3]; int32_t vid0, vid1, vid2, pad; };
struct SurfSrc { double c[3], n[3], p0, p1; };

struct PrepObj {
  int32_t geom_type, dof_type;
  int64_t n_elems, n_dofs;
  const unsigned char* src;
  const double* dofs;
  int64_t pool_off;
};

__device__ __forceinline__ void affine_apply(const double* d, const double* x, double* y, bool translate) {
  for (int r = 0; r < 3; ++r) {
    double v = d[3 + 3 * r] * x[0] + d[3 + 3 * r + 1] * x[1] + d[3 + 3 * r + 2] * x[2];
    y[r] = translate ? v + d[r] : v;
  }
}

// Anchor point of element e after the DoF transform (first vertex / centre).
__device__ __forceinline__ void anchor(const PrepObj& o, int64_t e, double* y) {
  if (o.geom_type == PI_GEOM_TRIANGLE) {
    const TriSrc& t = reinterpret_cast<const TriSrc*>(o.src)[e];
    if (o.dof_type == PI_DOF_TRIANGLE_MESH) {
      int64_t nv = o.n_dofs / 3;
      if (t.vid0 < 0 || t.vid0 >= nv) { y[0] = y[1] = y[2] = 0.0; return; }
      y[0] = o.dofs[3 * t.vid0]; y[1] = o.dofs[3 * t.vid0 + 1]; y[2] = o.dofs[3 * t.vid0 + 2];
    } else {
      affine_apply(o.dofs, t.a, y, true);
    }
  } else {
    const SurfSrc& s = reinterpret_cast<const SurfSrc*>(o.src)[e];
    affine_apply(o.dofs, s.c, y, true);
  }
}

// One CTA per object: fixed-order mean of the anchors (deterministic), plus
// the object's A for the surfel k' = A^T k rule.
__global__ void prepare_origin_kernel(const PrepObj* objs, ObjDev* out, int only) {
  const int oi = only >= 0 ? only : blockIdx.x;
  const PrepObj o = objs[oi];
  __shared__ double red[3][256];
  double s[3] = {0.0, 0.0, 0.0};
  int64_t valid = 0;
  for (int64_t e = threadIdx.x; e < o.n_elems; e += blockDim.x) {
    double y[3];
    anchor(o, e, y);
    s[0] += y[0]; s[1] += y[1]; s[2] += y[2];
    ++valid;
  }
  for (int c = 0; c < 3; ++c) red[c][threadIdx.x] = s[c];
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w)
      for (int c = 0; c < 3; ++c) red[c][threadIdx.x] += red[c][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    ObjDev d;
    double inv = o.n_elems > 0 ? 1.0 / (double)o.n_elems : 0.0;
    for (int c = 0; c < 3; ++c) d.origin[c] = red[c][0] * inv;
    if (o.dof_type == PI_DOF_AFFINE) {
      const double* A = o.dofs + 3;
      for (int i = 0; i < 9; ++i) d.A[i] = (float)A[i];
    } else {
      for (int i = 0; i < 9; ++i) d.A[i] = (i % 4 == 0) ? 1.f : 0.f;
    }
    d.type = o.geom_type;
    d.n_elems = (int32_t)o.n_elems;
    d.elem_off = o.pool_off;
    out[oi] = d;
  }
}

// grid (x: element blocks, y: object).  Writes the FP32 local-frame pools.
__global__ void prepare_elems_kernel(const PrepObj* objs, const ObjDev* od, float4* tri_pool, float4* surf_pool,
                                     float4* tri_lo, float4* surf_lo, float4* surf_nref, int only) {
  const int oi = only >= 0 ? only : blockIdx.y;
  const PrepObj o = objs[oi];
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= o.n_elems) return;
  const double* org = od[oi].origin;
  if (o.geom_type == PI_GEOM_TRIANGLE) {
    const TriSrc& t = reinterpret_cast<const TriSrc*>(o.src)[e];
    double a[3], e1[3], e2[3];
    bool ok = true;
    if (o.dof_type == PI_DOF_TRIANGLE_MESH) {
      int64_t nv = o.n_dofs / 3;
      ok = t.vid0 >= 0 && t.vid1 >= 0 && t.vid2 >= 0 && t.vid0 < nv && t.vid1 < nv && t.vid2 < nv;
      if (ok) {
        const double* v0 = o.dofs + 3 * t.vid0;
        const double* v1 = o.dofs + 3 * t.vid1;
        const double* v2 = o.dofs + 3 * t.vid2;
        for (int c = 0; c < 3; ++c) { a[c] = v0[c]; e1[c] = v1[c] - v0[c]; e2[c] = v2[c] - v0[c]; }
      }
    } else {
      affine_apply(o.dofs, t.a, a, true);
      affine_apply(o.dofs, t.e1, e1, false);
      affine_apply(o.dofs, t.e2, e2, false);
    }
    float4* dst = tri_pool + 3 * (o.pool_off + e);
    if (!ok) {  // unset vertex ids contribute nothing (triangle_mesh_dof.cpp:44-45)
      dst[0] = make_float4(0.f, 0.f, 0.f, 0.f); dst[1] = dst[0]; dst[2] = dst[0];
      tri_lo[o.pool_off + e] = dst[0];
      return;
    }
    double S[3] = {0.5 * (e1[1] * e2[2] - e1[2] * e2[1]), 0.5 * (e1[2] * e2[0] - e1[0] * e2[2]),
                   0.5 * (e1[0] * e2[1] - e1[1] * e2[0])};
    // centroid m = a + (e1 + e2)/3 relative to the object origin, FP32 hi + lo;
    // beside its low word the longest edge (the series-length bound k |e|max)
    const double l1 = e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2];
    const double l2 = e2[0] * e2[0] + e2[1] * e2[1] + e2[2] * e2[2];
    const double l3 = (e2[0] - e1[0]) * (e2[0] - e1[0]) + (e2[1] - e1[1]) * (e2[1] - e1[1]) +
                      (e2[2] - e1[2]) * (e2[2] - e1[2]);
    const float lmax = (float)sqrt(fmax(fmax(l1, l2), l3));
    float mh[3], ml[3];
    for (int c = 0; c < 3; ++c) {
      const double m = a[c] + (e1[c] + e2[c]) / 3.0 - org[c];
      mh[c] = (float)m;
      ml[c] = (float)(m - (double)mh[c]);
    }
    dst[0] = make_float4(mh[0], mh[1], mh[2], (float)S[0]);
    tri_lo[o.pool_off + e] = make_float4(ml[0], ml[1], ml[2], lmax);
    dst[1] = make_float4((float)e1[0], (float)e1[1], (float)e1[2], (float)S[1]);
    dst[2] = make_float4((float)e2[0], (float)e2[1], (float)e2[2], (float)S[2]);
  } else {
    const SurfSrc& s = reinterpret_cast<const SurfSrc*>(o.src)[e];
    double c[3], n[3];
    affine_apply(o.dofs, s.c, c, true);
    affine_apply(o.dofs, s.n, n, false);  // n' = A n so that k'.n = k.(A n) with k' = A^T k
    float4* dst = surf_pool + 2 * (o.pool_off + e);
    float ch[3], cl[3];
    for (int a = 0; a < 3; ++a) {
      const double r = c[a] - org[a];
      ch[a] = (float)r;
      cl[a] = (float)(r - (double)ch[a]);
    }
    dst[0] = make_float4(ch[0], ch[1], ch[2], (float)s.p0);
    surf_lo[o.pool_off + e] = make_float4(cl[0], cl[1], cl[2], 0.f);
    const double nn = s.n[0] * s.n[0] + s.n[1] * s.n[1] + s.n[2] * s.n[2];
    const double in = nn > 0.0 ? 1.0 / sqrt(nn) : 0.0;
    surf_nref[o.pool_off + e] =
        make_float4((float)(s.n[0] * in), (float)(s.n[1] * in), (float)(s.n[2] * in), (float)(1.0 - nn));
    dst[1] = make_float4((float)n[0], (float)n[1], (float)n[2], (float)s.p1);
  }
}

constexpr int FF_THREADS = 128;
constexpr int FF_WARPS = FF_THREADS / 32;
constexpr int FF_TILE = 256;  // elements staged per shared-memory tile (a multiple of FF_CHUNK)
constexpr int FF_CHUNK = 32;  // elements summed in FP32 before the compensated outer sum
static_assert(FF_TILE % FF_CHUNK == 0, "element chunks must not straddle tiles");

// Sums over thousands of elements: each thread adds FF_CHUNK element terms into
// a fresh FP32 partial, then adds the partial to a Kahan-compensated running
// sum, so rounding does not grow with the element count (a plain FP32 sum over
// 1,280 triangles measured ~1e-6 of max|A| per node).  The partials live in
// registers; the running sums and compensations live in shared memory, where
// they are touched once per FF_CHUNK elements, which leaves the registers for
// five CTAs per SM.
// A float4 from shared memory, loaded where it is written in the source: the
// element loop reads its radius constants each time instead of keeping them
// in registers across the loop.
__device__ __forceinline__ float4 ld_shared_f4(const float4* p) {
  float4 v;
  asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
               : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
               : "r"((unsigned)__cvta_generic_to_shared(p)));
  return v;
}

template <int R>
struct Acc {
  static_assert(R % 2 == 0, "radii are paired for packed FP32");
  // current chunk; radii (2p, 2p + 1) in one float2, the operand of packed FP32
  float2 re2[R / 2], im2[R / 2];
  float* run;  // run[(4 i + v) FF_THREADS]: v = sum re, sum im, compensation re, im
  __device__ __forceinline__ float& re(int i) { return (i & 1) ? re2[i >> 1].y : re2[i >> 1].x; }
  __device__ __forceinline__ float& im(int i) { return (i & 1) ? im2[i >> 1].y : im2[i >> 1].x; }
  __device__ __forceinline__ void init(float* base) {
    run = base + threadIdx.x;
#pragma unroll
    for (int i = 0; i < R; ++i) {
      re(i) = im(i) = 0.f;
#pragma unroll
      for (int v = 0; v < 4; ++v) run[(4 * i + v) * FF_THREADS] = 0.f;
    }
  }
  __device__ __forceinline__ void flush() {
#pragma unroll
    for (int i = 0; i < R; ++i) {
      float* p = run + 4 * i * FF_THREADS;
      float sre = p[0], sim = p[FF_THREADS], cre = p[2 * FF_THREADS], cim = p[3 * FF_THREADS];
      float y = re(i) - cre, t = sre + y;
      cre = (t - sre) - y;
      sre = t;
      y = im(i) - cim;
      t = sim + y;
      cim = (t - sim) - y;
      sim = t;
      p[0] = sre; p[FF_THREADS] = sim; p[2 * FF_THREADS] = cre; p[3 * FF_THREADS] = cim;
      re(i) = 0.f;
      im(i) = 0.f;
    }
  }
  __device__ __forceinline__ float sre(int i) const { return run[4 * i * FF_THREADS]; }
  __device__ __forceinline__ float sim(int i) const { return run[(4 * i + 1) * FF_THREADS]; }
};

// The grid is (CTAs per object) x (objects or evaluations); the CTAs are
// taken in the order the hardware dispatches them (x fastest, then y) and
// re-mapped so that the object slot varies fastest and the CTA index within
// the object slowest: every object's first CTAs (its largest-k radial block,
// below) run before any object's later ones.
// SERVE: the object slot indexes `evals` (serving evaluations: optional rotation of
// the k directions, local-frame direction-major output, row maximum);
// otherwise it indexes the batch's objects (largest first) and J is written
// q-major with the origin phase.
template <int R, bool SERVE>
__global__ void __launch_bounds__(FF_THREADS, 5)
ff_kernel(KGridDev kg, BatchDev b, float2* __restrict__ J, int scale_sqrt_w, const EvalDev* __restrict__ evals,
          unsigned* __restrict__ row_amax) {
  const unsigned lin = blockIdx.y * gridDim.x + blockIdx.x;
  const int slot = (int)(lin % gridDim.y), cta = (int)(lin / gridDim.y);
  const int oi = SERVE ? evals[slot].obj : b.order[slot];
  const ObjDev od = b.objs[oi];
  const int nrb = (kg.L + R - 1) / R;
  const int ndt = (kg.Me + 31) / 32;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // Warps of a CTA take neighbouring direction blocks at the same radial
  // block: they see the same radii, so they take the large-spread branch at
  // the same points of the element loop and reach the tile barriers together.
  // Radial blocks run in descending order of k: on a grid of ascending radii
  // the blocks of large k, whose elements take the long branches, start
  // first (for all objects, by the re-mapping above) and the launch ends on
  // light blocks (with neighbouring radii per warp the blocks differ
  // several-fold in cost).
  // A lane evaluates direction j = dpair[.].x and also writes its antipode
  // jm = dpair[.].y (A(-k) = -conj A(k)), when the grid has one.
  const int item = cta * FF_WARPS + warp;
  const int ib = item / ndt, dt = item - ib * ndt;
  const int rb = ib < nrb ? nrb - 1 - ib : 0;
  const int ei = dt * 32 + lane;
  const bool active = item < ndt * nrb && ei < kg.Me;
  int j = 0, jm = -1;
  if (active) { const int2 pr = kg.dpair[ei]; j = pr.x; jm = pr.y; }

  float3 dh = make_float3(0.f, 0.f, 0.f), dl = dh;
  float inv_norm = 0.f, dnorm = 0.f;
  if (active) {
    float4 h = kg.dir_hi[j], l = kg.dir_lo[j];
    dh = make_float3(h.x, h.y, h.z); dl = make_float3(l.x, l.y, l.z);
    inv_norm = h.w; dnorm = l.w;
    if (SERVE && evals[slot].rotate) {
      // rotated object: its form factor at k is the unrotated one's at R^T k
      // (|R^T k| = |k|); the direction is turned in FP64 and re-split.
      const double* Rm = evals[slot].R;
      const double d0 = (double)h.x + (double)l.x, d1 = (double)h.y + (double)l.y, d2 = (double)h.z + (double)l.z;
      double e[3];
#pragma unroll
      for (int a = 0; a < 3; ++a) e[a] = Rm[a] * d0 + Rm[3 + a] * d1 + Rm[6 + a] * d2;
      dh = make_float3((float)e[0], (float)e[1], (float)e[2]);
      dl = make_float3((float)(e[0] - (double)dh.x), (float)(e[1] - (double)dh.y), (float)(e[2] - (double)dh.z));
    }
  }
  // radii r = rb R + i: a warp's radii are neighbours, so warps at small k
  // take the short series for every radius of most elements (the lean loop
  // below, chosen once per element for the whole warp), and the branches of
  // the others are taken together more often.
  // The warp's radii as (k 256 / 2 pi hi, lo, k^2, k^3), in shared memory:
  // every lane reads the same entry (a broadcast), once per element and
  // radius, which keeps them out of the registers the element loop needs.
  __shared__ float4 krad[FF_WARPS][R];
  // e^{2 pi i j / 256}, j = 0..255: the phasor table of cis_tab_*
  __shared__ float2 ctab[256];
  for (int t = threadIdx.x; t < 256; t += FF_THREADS) ctab[t] = kg.cis_tab[t];
  if (lane < R) {
    const int r = rb * R + lane;
    const bool ok = item < ndt * nrb && r < kg.L;
    const float2 k = ok ? kg.kmag[r] : make_float2(0.f, 0.f);
    const float2 k2 = ok ? kg.kt256[r] : make_float2(0.f, 0.f);
    krad[warp][lane] = make_float4(k2.x, k2.y, k.x * k.x, k.x * k.x * k.x);
  }
  // the same constants paired for packed FP32: radii (2p, 2p + 1) as
  // (kt.hi, kt.hi', kt.lo, kt.lo') and (k^2, k^2', k^3, k^3')
  __shared__ float4 kpair[FF_WARPS][R];
  if (lane < R / 2) {
    float v[2][4];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int r = rb * R + 2 * lane + h;
      const bool ok = item < ndt * nrb && r < kg.L;
      const float2 k = ok ? kg.kmag[r] : make_float2(0.f, 0.f);
      const float2 k2 = ok ? kg.kt256[r] : make_float2(0.f, 0.f);
      v[h][0] = k2.x; v[h][1] = k2.y; v[h][2] = k.x * k.x; v[h][3] = k.x * k.x * k.x;
    }
    kpair[warp][2 * lane] = make_float4(v[0][0], v[1][0], v[0][1], v[1][1]);
    kpair[warp][2 * lane + 1] = make_float4(v[0][2], v[1][2], v[0][3], v[1][3]);
  }
  __syncthreads();
  const float4* kw = krad[warp];
  const float4* kp = kpair[warp];
  float kmax2 = 0.f;  // the warp's largest k^2
#pragma unroll
  for (int i = 0; i < R; ++i) kmax2 = fmaxf(kmax2, kw[i].z);
  __shared__ float run_sm[4 * R * FF_THREADS];
  Acc<R> acc;
  acc.init(run_sm);

  // tile[0, 3 FF_TILE): the elements' pool entries (surfels use the first
  // 2 FF_TILE and put their unit normals at tile[2 FF_TILE + e]);
  // tile[3 FF_TILE + e]: the low word of element e's centroid (centre).
  __shared__ float4 tile[4 * FF_TILE];
  const int n = od.n_elems;

  if (od.type == PI_GEOM_TRIANGLE) {
    const float4* src = b.tri_pool + 3 * od.elem_off;
    const float4* lo = b.tri_lo + od.elem_off;
    for (int base = 0; base < n; base += FF_TILE) {
      const int cnt = min(FF_TILE, n - base);
      __syncthreads();
      for (int t = threadIdx.x; t < 3 * cnt; t += FF_THREADS) tile[t] = src[3 * (int64_t)base + t];
      for (int t = threadIdx.x; t < cnt; t += FF_THREADS) tile[3 * FF_TILE + t] = lo[base + t];
      __syncthreads();
      if (active) {
        // chunks of FF_CHUNK elements (tiles hold a multiple of FF_CHUNK)
        for (int e0 = 0; e0 < cnt; e0 += FF_CHUNK) {
        const int e1 = min(e0 + FF_CHUNK, cnt);
        for (int e = e0; e < e1; ++e) {
          const float4 q0 = tile[3 * e], q1 = tile[3 * e + 1], q2 = tile[3 * e + 2];
          const float3 m = make_float3(q0.x, q0.y, q0.z);  // centroid, object frame
          const float3 e1 = make_float3(q1.x, q1.y, q1.z);
          const float3 e2 = make_float3(q2.x, q2.y, q2.z);
          // -2 (khat . S): gamma of the reference times the -2 of Phi = -2 e[..]
          const float g = -2.0f * (dh.x * q0.w + dh.y * q1.w + dh.z * q2.w) * inv_norm;
          const float4 ml = tile[3 * FF_TILE + e];
          const df sm = cdot2_un(dh, dl, m, make_float3(ml.x, ml.y, ml.z));
          const float kl = ml.w * dnorm;  // k kl bounds k sp: the short series below k kl = 1
          const float slim = rcp_fast(kl * kl);  // the short series for k^2 < 1 / kl^2 (inf when kl = 0)
          const float s1 = fmaf(dh.x, e1.x, fmaf(dh.y, e1.y, dh.z * e1.z));
          const float s2 = fmaf(dh.x, e2.x, fmaf(dh.y, e2.y, dh.z * e2.z));
          if (kmax2 < slim) {
            // every radius of this thread takes the short series (the same for
            // all lanes on a tensor grid: unit directions)
            // two radii per packed FP32 instruction: the same operations,
            // roundings and results as the scalar loop below
            const TriPolyShort tp = tri_series_coeffs_short(s1, s2, g);
            const float2 smh = make_float2(sm.hi, sm.hi), sml = make_float2(sm.lo, sm.lo);
#pragma unroll
            for (int p = 0; p < R / 2; ++p) {
              const float4 kx = ld_shared_f4(kp + 2 * p), ku = ld_shared_f4(kp + 2 * p + 1);
              const cf2 P = cis_tab_df2(ctab, make_float2(kx.x, kx.y), make_float2(kx.z, kx.w), smh, sml);
              const cf2 T = tri_series_eval_short2(tp, make_float2(ku.x, ku.y), make_float2(ku.z, ku.w));
              acc.re2[p] = __ffma2_rn(P.re, T.re, __ffma2_rn(neg2(P.im), T.im, acc.re2[p]));
              acc.im2[p] = __ffma2_rn(P.re, T.im, __ffma2_rn(P.im, T.re, acc.im2[p]));
            }
            continue;
          }
          const float sp = fmaxf(fmaxf(fabsf(s1), fabsf(s2)), fabsf(s2 - s1));
          const float kthr2 = __fdividef(9.0f, sp * sp);  // the series for (k sp)^2 < 9 (inf when sp = 0)
          const TriPoly tp = tri_series_coeffs(s1, s2, g);
          // vertex phases relative to the centroid (a = m - (e1 + e2)/3, b = a + e1, c = a + e2)
          const float da = -(s1 + s2) * (1.0f / 3.0f), db = da + s1, dc = da + s2;
#pragma unroll
          for (int i = 0; i < R; ++i) {
            const float4 kr = ld_shared_f4(kw + i);
            const float2 kt = make_float2(kr.x, kr.y);
            const cf P = cis_tab_df(ctab, kt, sm);  // centroid phase
            cf T;
            if (kr.z < slim) {  // the same for all lanes on a tensor grid (unit directions)
              T = tri_series_eval_short(tp, kr.z, kr.w);
            } else if (kr.z < kthr2) {
              T = tri_series_eval(tp, kr.z, kr.w);  // centroid Taylor series, gamma folded in
            } else {
              // Large spread: e[pa, pb, pc] = e^{i k.m} e[k da, k db, k dc].  The
              // relative phases are FP32 dot products times the double-float
              // radius: their error |k d| 6e-8 rad multiplies a term of size
              // ~1/|k d|^2 here.
              const float k = kr.x * PI_TURN256;
              const cf v = tri_generic(cis_tab_f(ctab, kt, da), cis_tab_f(ctab, kt, db), cis_tab_f(ctab, kt, dc),
                                       k * s1, k * s2);
              T = cf{g * v.re, g * v.im};
            }
            acc.re(i) = fmaf(P.re, T.re, fmaf(-P.im, T.im, acc.re(i)));
            acc.im(i) = fmaf(P.re, T.im, fmaf(P.im, T.re, acc.im(i)));
          }
        }
        if (e1 - e0 == FF_CHUNK) acc.flush();
        }
      }
    }
  } else {
    const float4* src = b.surf_pool + 2 * od.elem_off;
    const float4* lo = b.surf_lo + od.elem_off;
    const bool disk = od.type == PI_GEOM_DISK;
    // v = A^T dir, so k' = kmag v and |k'|^2 = kmag^2 qd
    const float* Am = od.A;
    const float3 v = make_float3(Am[0] * dh.x + Am[3] * dh.y + Am[6] * dh.z, Am[1] * dh.x + Am[4] * dh.y + Am[7] * dh.z,
                                 Am[2] * dh.x + Am[5] * dh.y + Am[8] * dh.z);
    const float qd = fmaf(v.x, v.x, fmaf(v.y, v.y, v.z * v.z));
    const float4* nref = b.surf_nref + od.elem_off;
    for (int base = 0; base < n; base += FF_TILE) {
      const int cnt = min(FF_TILE, n - base);
      __syncthreads();
      for (int t = threadIdx.x; t < 2 * cnt; t += FF_THREADS) tile[t] = src[2 * (int64_t)base + t];
      for (int t = threadIdx.x; t < cnt; t += FF_THREADS) {
        tile[2 * FF_TILE + t] = nref[base + t];
        tile[3 * FF_TILE + t] = lo[base + t];
      }
      __syncthreads();
      if (active) {
        for (int e0 = 0; e0 < cnt; e0 += FF_CHUNK) {
        const int e1 = min(e0 + FF_CHUNK, cnt);
        for (int e = e0; e < e1; ++e) {
          const float4 q0 = tile[2 * e], q1 = tile[2 * e + 1], nr = tile[2 * FF_TILE + e];
          const float4 cl = tile[3 * FF_TILE + e];
          const df sc = cdot2_un(dh, dl, make_float3(q0.x, q0.y, q0.z), make_float3(cl.x, cl.y, cl.z));
          const float sn = dh.x * q1.x + dh.y * q1.y + dh.z * q1.z;  // dir . (A n)
          // |k'_perp|^2 / kmag^2 = qd (1 - |n|^2) + |n|^2 |v x n/|n||^2: its rounding
          // shrinks with the angle to the normal, where qd - sn^2 would leave ~1e-7
          // (a Bessel argument off by (k rho)^2 1e-7 / (2 x) rad).
          const float cx = fmaf(v.y, nr.z, -v.z * nr.y), cy = fmaf(v.z, nr.x, -v.x * nr.z),
                      cz = fmaf(v.x, nr.y, -v.y * nr.x);
          const float perp = fmaf(qd, nr.w, (1.0f - nr.w) * fmaf(cx, cx, fmaf(cy, cy, cz * cz)));
          const float amp = sn * inv_norm * q1.w;                   // area|w * (k'.n)/|k|
          // two radii per packed FP32 phasor and accumulation (cis_tab_df2)
          const float2 sch = make_float2(sc.hi, sc.hi), scl = make_float2(sc.lo, sc.lo);
          if (disk) {
            const float rr = q0.w * sqrt_fast(fmaxf(perp, 0.f)) * PI_TURN256;  // rho |k'_perp| / kmag, per 1/256 turn
#pragma unroll
            for (int p = 0; p < R / 2; ++p) {
              const float4 kx = ld_shared_f4(kp + 2 * p);
              const float xa = kx.x * rr, xb = kx.y * rr;
              const float Sa = (xa < 1e-10f) ? 1.0f : 2.0f * j1x(xa);
              const float Sb = (xb < 1e-10f) ? 1.0f : 2.0f * j1x(xb);
              const cf2 P = cis_tab_df2(ctab, make_float2(kx.x, kx.y), make_float2(kx.z, kx.w), sch, scl);
              const float2 m = make_float2(Sa * amp, Sb * amp);
              acc.re2[p] = __ffma2_rn(m, P.re, acc.re2[p]);
              acc.im2[p] = __ffma2_rn(m, P.im, acc.im2[p]);
            }
          } else {
            const float hs = -0.5f * q0.w * q0.w * perp;
#pragma unroll
            for (int p = 0; p < R / 2; ++p) {
              const float4 kx = ld_shared_f4(kp + 2 * p), ku = ld_shared_f4(kp + 2 * p + 1);
              const float2 m = make_float2(__expf(hs * ku.x) * amp, __expf(hs * ku.y) * amp);
              const cf2 P = cis_tab_df2(ctab, make_float2(kx.x, kx.y), make_float2(kx.z, kx.w), sch, scl);
              acc.re2[p] = __ffma2_rn(m, P.re, acc.re2[p]);
              acc.im2[p] = __ffma2_rn(m, P.im, acc.im2[p]);
            }
          }
        }
        if (e1 - e0 == FF_CHUNK) acc.flush();
        }
      }
    }
  }

  if (!active) return;
  acc.flush();
  if (SERVE) {
    const EvalDev& ev = evals[slot];
    float m = 0.f;
#pragma unroll
    for (int i = 0; i < R; ++i) {
      const int r = rb * R + i;
      if (r < kg.L) {
        const int64_t q = (int64_t)r * kg.M + j;
        cf v{acc.sre(i), acc.sim(i)};
        if (kw[i].x * PI_TURN256 * dnorm < 1e-10f) v = cf{0.f, 0.f};  // A(0) = 0 (affine_dof.cpp:64-65)
        const float sw = kg.sqrtw[q];
        ev.dst[(int64_t)j * kg.L + r] = make_float2(v.re * sw, v.im * sw);
        m = fmaxf(m, fmaxf(fabsf(v.re * sw), fabsf(v.im * sw)));
        if (jm >= 0) {  // the antipode: -conj
          const float swm = kg.sqrtw[(int64_t)r * kg.M + jm];
          ev.dst[(int64_t)jm * kg.L + r] = make_float2(-v.re * swm, v.im * swm);
          m = fmaxf(m, fmaxf(fabsf(v.re * swm), fabsf(v.im * swm)));
        }
      }
    }
    atomicMax(reinterpret_cast<unsigned*>(ev.amax), __float_as_uint(m));
    return;
  }
  // origin phase e^{i k.o}: formed and reduced in FP64 once per output, so
  // objects far from the frame's origin keep their accuracy.
  const double dox = (double)dh.x + (double)dl.x, doy = (double)dh.y + (double)dl.y,
               doz = (double)dh.z + (double)dl.z;
  const double so_d = dox * od.origin[0] + doy * od.origin[1] + doz * od.origin[2];
  const int64_t Jrow = (int64_t)oi * kg.Q;
  float m = 0.f;
#pragma unroll
  for (int i = 0; i < R; ++i) {
    const int r = rb * R + i;
    if (r < kg.L) {
      const int64_t q = (int64_t)r * kg.M + j;
      const double kd = ((double)kw[i].x + (double)kw[i].y) * (6.283185307179586476925 / 256.0);
      cf v = cmul(cis_f64(kd * so_d), cf{acc.sre(i), acc.sim(i)});
      if (kw[i].x * PI_TURN256 * dnorm < 1e-10f) v = cf{0.f, 0.f};  // A(0) = 0 (affine_dof.cpp:64-65)
      if (jm >= 0) {  // the antipode: -conj (the origin phase included)
        const int64_t qm = (int64_t)r * kg.M + jm;
        const float s = scale_sqrt_w ? kg.sqrtw[qm] : 1.0f;
        const float2 u = make_float2(-v.re * s, v.im * s);
        J[Jrow + qm] = u;
        m = fmaxf(m, fmaxf(fabsf(u.x), fabsf(u.y)));
      }
      if (scale_sqrt_w) { const float s = kg.sqrtw[q]; v.re *= s; v.im *= s; }
      J[Jrow + q] = make_float2(v.re, v.im);
      m = fmaxf(m, fmaxf(fabsf(v.re), fabsf(v.im)));
    }
  }
  if (row_amax) {  // the row's largest |Re|, |Im| (FP32 bits order like the non-negative floats)
    const unsigned mask = __activemask();
    const unsigned mb = __reduce_max_sync(mask, __float_as_uint(m));
    if (lane == __ffs(mask) - 1) atomicMax(row_amax + oi, mb);
  }
}

__global__ void to_double2_kernel(const float2* __restrict__ J, int64_t n, double2* __restrict__ out) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) { float2 v = J[i]; out[i] = make_double2(v.x, v.y); }
}

}  // namespace

static int radii_per_thread(int L) { return L >= 32 ? 8 : L >= 4 ? 4 : 2; }  // even: radii are paired

int launch_prepare(pi_batch_impl* b, int only_index, cudaStream_t s) {
  std::vector<PrepObj> h(b->n_obj);
  int64_t max_elems = 0;
  for (int i = 0; i < b->n_obj; ++i) {
    const HostObjInfo& in = b->info[i];
    PrepObj& p = h[i];
    p.geom_type = in.geom_type; p.dof_type = in.dof_type; p.n_elems = in.n_elems; p.n_dofs = in.n_dofs;
    p.src = static_cast<const unsigned char*>(b->d_src) + in.src_off;
    p.dofs = b->d_dofs + in.dof_off;
    p.pool_off = in.pool_off;
    if (only_index < 0 || only_index == i) max_elems = std::max(max_elems, in.n_elems);
  }
  if (b->n_obj == 0) return PI_OK;
  PrepObj* d = nullptr;
  PI_CUDA(cudaMallocAsync((void**)&d, sizeof(PrepObj) * h.size(), s));
  PI_CUDA(cudaMemcpyAsync(d, h.data(), sizeof(PrepObj) * h.size(), cudaMemcpyHostToDevice, s));
  const int nobj_launch = only_index >= 0 ? 1 : b->n_obj;
  prepare_origin_kernel<<<nobj_launch, 256, 0, s>>>(d, b->d_objs, only_index);
  PI_LAUNCHED("prepare_origin_kernel");
  if (max_elems > 0) {
    dim3 grid((unsigned)((max_elems + 255) / 256), (unsigned)nobj_launch);
    prepare_elems_kernel<<<grid, 256, 0, s>>>(d, b->d_objs, b->d_tri_pool, b->d_surf_pool, b->d_tri_lo,
                                              b->d_surf_lo, b->d_surf_nref, only_index);
    PI_LAUNCHED("prepare_elems_kernel");
  }
  // The host staging array `h` has been consumed by the copy above once the
  // stream reaches it; cudaMemcpyAsync from pageable memory is synchronous
  // with respect to the host buffer, so it may go out of scope here.
  PI_CUDA(cudaFreeAsync(d, s));
  return PI_OK;
}

int launch_form_factors(const pi_kgrid_impl* kg, const pi_batch_impl* b, int scale_sqrt_w, float2* J,
                        cudaStream_t s, float* row_amax) {
  if (b->n_obj == 0) return PI_OK;
  if (row_amax) PI_CUDA(cudaMemsetAsync(row_amax, 0, (size_t)b->n_obj * sizeof(float), s));
  unsigned* ra = reinterpret_cast<unsigned*>(row_amax);
  const KGridDev K = kg->dev;
  const BatchDev B = b->dev();
  int R = radii_per_thread(K.L);
  const int ndt = (K.Me + 31) / 32;
  auto ctas = [&](int r) { return ((int64_t)((K.L + r - 1) / r) * ndt + FF_WARPS - 1) / FF_WARPS; };
  // a launch of fewer than two CTAs per SM at 8 radii per thread, such as
  // one moving mesh of the alignment caller (76 CTAs), takes 4, which fills
  // twice the SMs; above that 8 radii share the per-element work better
  // (the 8-object surfel sample, 608 CTAs: 64.1 ms at 8, 68.6 ms at 4)
  const int n_sm = current_sm_count();
  if (R == 8 && ctas(8) * b->n_obj < 2 * (int64_t)n_sm) R = 4;
  dim3 grid((unsigned)ctas(R), (unsigned)b->n_obj);
  if (grid.y > 65535) return fail(PI_ERR_UNSUPPORTED, "more than 65535 objects in one batch");
  switch (R) {
    case 8: ff_kernel<8, false><<<grid, FF_THREADS, 0, s>>>(K, B, J, scale_sqrt_w, nullptr, ra); break;
    case 4: ff_kernel<4, false><<<grid, FF_THREADS, 0, s>>>(K, B, J, scale_sqrt_w, nullptr, ra); break;
    default: ff_kernel<2, false><<<grid, FF_THREADS, 0, s>>>(K, B, J, scale_sqrt_w, nullptr, ra); break;
  }
  PI_LAUNCHED("ff_kernel");
  return PI_OK;
}

int ff_serve_threads() { return FF_THREADS; }

int ff_serve_grid_x(const pi_kgrid_impl* kg) {
  const int R = radii_per_thread(kg->dev.L);
  const int64_t items = (int64_t)((kg->dev.L + R - 1) / R) * ((kg->dev.Me + 31) / 32);
  return (int)((items + FF_WARPS - 1) / FF_WARPS);
}

const void* ff_serve_fn(const pi_kgrid_impl* kg) {
  switch (radii_per_thread(kg->dev.L)) {
    case 8: return reinterpret_cast<const void*>(ff_kernel<8, true>);
    case 4: return reinterpret_cast<const void*>(ff_kernel<4, true>);
    default: return reinterpret_cast<const void*>(ff_kernel<2, true>);
  }
}

int launch_form_factors_serve(const pi_kgrid_impl* kg, const pi_batch_impl* lib, const EvalDev* evals, int n_evals,
                              cudaStream_t s) {
  if (n_evals <= 0) return PI_OK;
  if (n_evals > 65535) return fail(PI_ERR_UNSUPPORTED, "more than 65535 evaluations in one launch");
  KGridDev K = kg->dev;
  BatchDev B = lib->dev();
  float2* none = nullptr;
  int scale = 1;
  unsigned* no_amax = nullptr;
  void* args[6] = {&K, &B, &none, &scale, const_cast<EvalDev**>(&evals), &no_amax};
  PI_CUDA(cudaLaunchKernel(ff_serve_fn(kg), dim3((unsigned)ff_serve_grid_x(kg), (unsigned)n_evals), dim3(FF_THREADS),
                           args, 0, s));
  count_launch();
  return PI_OK;
}

namespace {
__global__ void amax_commit_kernel(const EvalDev* __restrict__ evals, const int32_t* __restrict__ n_evals) {
  const int n = *n_evals;
  for (int e = threadIdx.x; e < n; e += blockDim.x) *evals[e].amax_keep = *evals[e].amax;
}
}  // namespace

const void* amax_commit_fn() { return reinterpret_cast<const void*>(amax_commit_kernel); }
int amax_commit_threads() { return 256; }

int launch_amax_commit(const EvalDev* evals, const int32_t* n_evals, cudaStream_t s) {
  amax_commit_kernel<<<1, 256, 0, s>>>(evals, n_evals);
  PI_LAUNCHED("amax_commit_kernel");
  return PI_OK;
}

int launch_to_double2(const float2* J, int64_t n, double* out, cudaStream_t s) {
  if (n == 0) return PI_OK;
  to_double2_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(J, n, reinterpret_cast<double2*>(out));
  PI_LAUNCHED("to_double2_kernel");
  return PI_OK;
}

}  // namespace pi
