// Volume contraction V = Re(J^H diag(w) J) / (8 pi^3), plain FP32 form.
//
// Replaces K9 (cpp/src/compute_intersection_volume.cu:33-50: one global FP64
// atomicAdd per k-node) and K14 (cpp/src/compute_intersection_volume_multi_object.cu:74-116:
// one thread per (i,j) streaming all of J with no tiling).  With the operand
// X = [Re sqrt|w| J ; Im sqrt|w| J] (n x 2Q real, the layout the form-factor
// kernel writes), V is the SYRK X diag(sign) X^T on FP32 CUDA cores.
//
// syrk_fp32_kernel: one CTA = one 128 x 128 output tile of the upper triangle
// x one K range.  256 threads, each owning an 8 x 8 register block (rows
// 4 ty + {0..3} and 64 + 4 ty + {0..3}, columns likewise with tx), fed from
// K-major shared-memory slabs of 32 k values, double-buffered through
// registers.  A diagonal tile skips its lower-left 64 x 64 quadrant (it lies
// below the diagonal) and takes 4/3 of an off-diagonal tile's K range, so the
// CTAs finish together and 80% of the multiply-adds are upper-triangle work at
// 256 objects.  Each thread sums 64 k values into a fresh register block
// (packed FP32 multiply-adds) and then adds it, Kahan-compensated, to a
// running sum held in shared memory: off-diagonal entries are small
// differences of large partial sums.  Over the 256-object matrix the fold
// length trades time for error against an FP64 contraction of the same J:
// 32 k 0.376 ms / 4.4e-6, 64 k 0.338 ms / 5.5e-6, 96 k 0.324 ms / 6.9e-6,
// 256 k 0.305 ms / 2.1e-5 (conditioned with the 1e-3 floor).
// Per-CTA partial tiles are reduced in a fixed order (compensated FP32,
// ~48 bits) by a second kernel: results are bitwise reproducible run to run.
#include <cuda_runtime.h>
#include <cstdint>
#include <algorithm>
#include <mutex>
#include "pi_internal.h"
#include "dfmath.cuh"

namespace pi {

namespace {

constexpr int TB = 128;              // output tile edge
constexpr int BK = 32;               // k values per shared-memory slab (a power of two)
constexpr int LDM = TB + 4;          // padded slab row (floats)
#ifndef PI_SYRK_FOLD
#define PI_SYRK_FOLD 2
#endif
constexpr int FOLD = PI_SYRK_FOLD;   // slabs per compensated fold
constexpr int NT = 256;              // threads per CTA
constexpr int SLAB_FLOATS = BK * LDM;
constexpr size_t SYRK_SMEM = (size_t)(4 * SLAB_FLOATS + 128 * NT) * sizeof(float);  // 2 x (A, B) slabs + running sums
constexpr double INV8PI3 = 1.0 / (8.0 * 3.14159265358979323846 * 3.14159265358979323846 * 3.14159265358979323846);

// Work split: CTAs [0, nt s_d) are diagonal tiles (s_d K ranges of kc_d each),
// then the nt (nt - 1) / 2 off-diagonal tiles in row-major upper order
// (s_o K ranges of kc_o each).  A CTA's partial tile is partials[blockIdx.x].
struct SyrkGeom {
  int n, nt, s_d, s_o;
  int64_t K, kc_d, kc_o;
};

// Off-diagonal tile o (row-major over bi < bj) -> (bi, bj).
__host__ __device__ __forceinline__ void off_tile_of(int o, int nt, int* bi, int* bj) {
  int i = 0, rem = o;
  while (rem >= nt - 1 - i) { rem -= nt - 1 - i; ++i; }
  *bi = i; *bj = i + 1 + rem;
}

// 4 k values (kk .. kk + 3) of one row; zero past kend or for rows past n.
__device__ __forceinline__ float4 load4(const float* __restrict__ row, int64_t kk, int64_t kend, bool vec) {
  if (vec && kk + 3 < kend) return __ldg(reinterpret_cast<const float4*>(row + kk));
  float4 v;
  v.x = kk < kend ? __ldg(row + kk) : 0.f;
  v.y = kk + 1 < kend ? __ldg(row + kk + 1) : 0.f;
  v.z = kk + 2 < kend ? __ldg(row + kk + 2) : 0.f;
  v.w = kk + 3 < kend ? __ldg(row + kk + 3) : 0.f;
  return v;
}

// A 32-k slab of one 128-row tile: thread t loads row t % 128 at k quads
// t / 128 + 2 l (a warp reads 32 consecutive rows, so its transposed stores
// into the K-major slab hit 32 consecutive words).
struct SlabRegs { float4 v[4]; };

__device__ __forceinline__ void slab_load(SlabRegs& r, const float* __restrict__ X, int row0, int n, int64_t K,
                                          int64_t k, int64_t kend, bool vec, const float* __restrict__ sign) {
  const int row = threadIdx.x & (TB - 1);
  const int gr = row0 + row;
  const float* src = X + (int64_t)gr * K;
#pragma unroll
  for (int l = 0; l < 4; ++l) {
    const int64_t kk = k + 4 * ((threadIdx.x >> 7) + 2 * l);
    float4 v = gr < n ? load4(src, kk, kend, vec) : make_float4(0.f, 0.f, 0.f, 0.f);
    if (sign) {  // V = X diag(sign) X^T: one operand carries the signs; kk is a multiple of 4
      const float s0 = kk < K ? __ldg(sign + (kk >> 1)) : 0.f, s1 = kk + 2 < K ? __ldg(sign + ((kk + 2) >> 1)) : 0.f;
      v.x *= s0; v.y *= s0; v.z *= s1; v.w *= s1;
    }
    r.v[l] = v;
  }
}

__device__ __forceinline__ void slab_store(const SlabRegs& r, float* __restrict__ slab) {
  const int row = threadIdx.x & (TB - 1);
#pragma unroll
  for (int l = 0; l < 4; ++l) {
    const int k4 = 4 * ((threadIdx.x >> 7) + 2 * l);
    slab[(k4 + 0) * LDM + row] = r.v[l].x;
    slab[(k4 + 1) * LDM + row] = r.v[l].y;
    slab[(k4 + 2) * LDM + row] = r.v[l].z;
    slab[(k4 + 3) * LDM + row] = r.v[l].w;
  }
}

// part[i][jj] += sum over the slab's 32 k of A[k][row i] (B[k][col 2 jj], B[k][col 2 jj + 1]),
// with packed FP32 FMAs (two multiply-adds per instruction, each rounded
// like fmaf), which halves the issue slots the multiply-adds take.  DIAG
// skips the lower-left quadrant (rows 64.., columns ..63 of a diagonal tile).
// The next k step's operands are read from shared memory before this step's
// multiply-adds (the last step re-reads row 0: in bounds, unused), and the
// loop is unrolled by 8 so that its body stays inside the instruction cache.
template <bool DIAG>
__device__ __forceinline__ void slab_fma(float2 (&part)[8][4], const float* __restrict__ As,
                                         const float* __restrict__ Bs, int ty, int tx) {
  float4 na0 = *reinterpret_cast<const float4*>(As + 4 * ty);
  float4 na1 = *reinterpret_cast<const float4*>(As + 64 + 4 * ty);
  float4 nb0 = *reinterpret_cast<const float4*>(Bs + 4 * tx);
  float4 nb1 = *reinterpret_cast<const float4*>(Bs + 64 + 4 * tx);
#pragma unroll 8
  for (int kk = 0; kk < BK; ++kk) {
    const float a[8] = {na0.x, na0.y, na0.z, na0.w, na1.x, na1.y, na1.z, na1.w};
    const float2 b[4] = {make_float2(nb0.x, nb0.y), make_float2(nb0.z, nb0.w), make_float2(nb1.x, nb1.y),
                         make_float2(nb1.z, nb1.w)};
    const int kn = ((kk + 1) & (BK - 1)) * LDM;
    na0 = *reinterpret_cast<const float4*>(As + kn + 4 * ty);
    na1 = *reinterpret_cast<const float4*>(As + kn + 64 + 4 * ty);
    nb0 = *reinterpret_cast<const float4*>(Bs + kn + 4 * tx);
    nb1 = *reinterpret_cast<const float4*>(Bs + kn + 64 + 4 * tx);
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const float2 ai = make_float2(a[i], a[i]);
#pragma unroll
      for (int jj = 0; jj < 4; ++jj) {
        if (DIAG && i >= 4 && jj < 2) continue;
        part[i][jj] = __ffma2_rn(ai, b[jj], part[i][jj]);
      }
    }
  }
}

// Kahan step of every register-block entry into the running sums in shared
// memory: run4[g NT + tid] (g = 0..15) holds the sums of entries
// (i, 4h .. 4h + 3), g = 2 i + h, and run4[(16 + g) NT + tid] their
// compensations; 16-byte accesses, consecutive across a warp.  Zeroes part.
// Kahan step on pairs with packed FP32 arithmetic; a - b is formed as
// fma(b, -1, a), exact in the product, so each step rounds like its scalar form.
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }

__device__ __forceinline__ void kahan2(float2& acc, float2& cmp, float2 v) {
  const float2 y = sub2(v, cmp);
  const float2 t = __fadd2_rn(acc, y);
  cmp = sub2(sub2(t, acc), y);
  acc = t;
}

template <bool DIAG>
__device__ __forceinline__ void fold(float2 (&part)[8][4], float4* __restrict__ run4) {
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      if (DIAG && i >= 4 && h == 0) continue;  // the skipped quadrant stays zero
      float4* pa = run4 + (2 * i + h) * NT + threadIdx.x;
      float4* pc = pa + 16 * NT;
      const float4 a4 = *pa, c4 = *pc;
      float2 a0 = make_float2(a4.x, a4.y), a1 = make_float2(a4.z, a4.w);
      float2 c0 = make_float2(c4.x, c4.y), c1 = make_float2(c4.z, c4.w);
      kahan2(a0, c0, part[i][2 * h]);
      kahan2(a1, c1, part[i][2 * h + 1]);
      *pa = make_float4(a0.x, a0.y, a1.x, a1.y);
      *pc = make_float4(c0.x, c0.y, c1.x, c1.y);
      part[i][2 * h] = make_float2(0.f, 0.f);
      part[i][2 * h + 1] = make_float2(0.f, 0.f);
    }
}

template <bool DIAG>
__device__ __forceinline__ void syrk_tile(const float* __restrict__ X, const SyrkGeom& g, int bi, int bj, int64_t k0,
                                          int64_t k1, const float* __restrict__ sign, bool vec,
                                          float* __restrict__ out) {
  extern __shared__ __align__(16) float sm[];
  // buffer b: A slab at sm + 2 b SLAB_FLOATS, B slab right after it
  float4* run4 = reinterpret_cast<float4*>(sm + 4 * SLAB_FLOATS);
  const int tid = threadIdx.x, ty = tid >> 4, tx = tid & 15;
  // a diagonal tile reads one operand tile, unless the weights' signs make B differ from A
  const bool sep_b = !DIAG || sign != nullptr;
  for (int g = 0; g < 32; ++g) run4[g * NT + tid] = make_float4(0.f, 0.f, 0.f, 0.f);
  float2 part[8][4];
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) part[i][j] = make_float2(0.f, 0.f);

  SlabRegs ra, rb;
  const int64_t nslab = (k1 - k0 + BK - 1) / BK;
  if (nslab > 0) {
    slab_load(ra, X, bi * TB, g.n, g.K, k0, k1, vec, nullptr);
    if (sep_b) slab_load(rb, X, bj * TB, g.n, g.K, k0, k1, vec, sign);
    slab_store(ra, sm);
    if (sep_b) slab_store(rb, sm + SLAB_FLOATS);
  }
  __syncthreads();
  for (int64_t s = 0; s < nslab; ++s) {
    const int buf = (int)(s & 1);
    const bool more = s + 1 < nslab;
    if (more) {  // next slab in flight while this one is multiplied
      const int64_t kn = k0 + (s + 1) * BK;
      slab_load(ra, X, bi * TB, g.n, g.K, kn, k1, vec, nullptr);
      if (sep_b) slab_load(rb, X, bj * TB, g.n, g.K, kn, k1, vec, sign);
    }
    const float* As = sm + 2 * buf * SLAB_FLOATS;
    slab_fma<DIAG>(part, As, sep_b ? As + SLAB_FLOATS : As, ty, tx);
    if ((s + 1) % FOLD == 0 || !more) fold<DIAG>(part, run4);
    if (more) {
      float* An = sm + 2 * (buf ^ 1) * SLAB_FLOATS;
      slab_store(ra, An);
      if (sep_b) slab_store(rb, An + SLAB_FLOATS);
    }
    __syncthreads();
  }
  // partial tile: running sum minus its compensation
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int r = (i < 4 ? 0 : 64) + 4 * ty + (i & 3);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      if (DIAG && i >= 4 && h == 0) continue;  // below the diagonal: never read
      const float4 a = run4[(2 * i + h) * NT + tid], c = run4[(16 + 2 * i + h) * NT + tid];
      *reinterpret_cast<float4*>(out + r * TB + 64 * h + 4 * tx) = make_float4(a.x - c.x, a.y - c.y, a.z - c.z, a.w - c.w);
    }
  }
}

__global__ void __launch_bounds__(NT, 1)
syrk_fp32_kernel(const float* __restrict__ X, const SyrkGeom g, const float* __restrict__ sign, bool vec,
                 float* __restrict__ partials) {
  const int c = blockIdx.x;
  const int nd = g.nt * g.s_d;
  float* out = partials + (int64_t)c * (TB * TB);
  if (c < nd) {
    const int b = c / g.s_d, sp = c - b * g.s_d;
    const int64_t k0 = (int64_t)sp * g.kc_d, k1 = min(g.K, k0 + g.kc_d);
    syrk_tile<true>(X, g, b, b, k0, k1, sign, vec, out);
  } else {
    const int o = (c - nd) / g.s_o, sp = (c - nd) - o * g.s_o;
    int bi, bj;
    off_tile_of(o, g.nt, &bi, &bj);
    const int64_t k0 = (int64_t)sp * g.kc_o, k1 = min(g.K, k0 + g.kc_o);
    syrk_tile<false>(X, g, bi, bj, k0, k1, sign, vec, out);
  }
}

// Fixed-order compensated sum of a tile's partials, scaled by 1/(8 pi^3),
// mirrored; one thread per (i, j), i <= j.
__global__ void reduce_tiles_kernel(const float* __restrict__ partials, const SyrkGeom g, double* __restrict__ V) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)g.n * g.n) return;
  const int i = (int)(t / g.n), j = (int)(t - (int64_t)i * g.n);
  if (i > j) return;
  const int ti = i / TB, tj = j / TB;
  int64_t base;
  int cnt;
  if (ti == tj) {
    base = (int64_t)ti * g.s_d;
    cnt = g.s_d;
  } else {
    const int o = ti * (g.nt - 1) - ti * (ti - 1) / 2 + (tj - ti - 1);
    base = (int64_t)g.nt * g.s_d + (int64_t)o * g.s_o;
    cnt = g.s_o;
  }
  // compensated FP32 sum in split order (FP64 adds run at 1/64 of the FP32 rate)
  kbsum acc{0.f, 0.f};
  const float* src = partials + base * (TB * TB) + (i % TB) * TB + (j % TB);
  int sp = 0;
  for (; sp + 16 <= cnt; sp += 16) {  // sixteen loads in flight ahead of their adds
    float v[16];
#pragma unroll
    for (int u = 0; u < 16; ++u) v[u] = __ldcs(src + (int64_t)(sp + u) * (TB * TB));
#pragma unroll
    for (int u = 0; u < 16; ++u) acc.add(v[u]);
  }
  for (; sp < cnt; ++sp) acc.add(__ldcs(src + (int64_t)sp * (TB * TB)));
  const double s = acc.value() * INV8PI3;
  V[(int64_t)i * g.n + j] = s;
  V[(int64_t)j * g.n + i] = s;
}

int sm_count() { return current_sm_count(); }

// K ranges: a diagonal tile's 3 quadrants get 4/3 of an off-diagonal tile's
// k per CTA (s_d : s_o = 3 : 4), with as many CTAs as fit in one wave of one
// CTA per SM (capped at max_tiles partial tiles when max_tiles > 0), or one
// CTA per tile when the tiles alone fill the GPU.  Returns false when
// max_tiles cannot hold one partial tile per tile.
bool plan_syrk(int64_t Q, int n, SyrkGeom* g, int64_t max_tiles = 0) {
  g->n = n;
  g->K = 2 * Q;
  g->nt = (n + TB - 1) / TB;
  const int64_t noff = (int64_t)g->nt * (g->nt - 1) / 2;
  const int64_t units = 3LL * g->nt + 4 * noff;
  int64_t slots = sm_count();
  if (max_tiles > 0) slots = std::min<int64_t>(slots, max_tiles);
  const int64_t m = slots / units;
  int64_t sd = m >= 1 ? 3 * m : 1, so = m >= 1 ? 4 * m : 1;
  const int64_t nslab = (g->K + BK - 1) / BK;
  sd = std::max<int64_t>(1, std::min(sd, nslab));
  so = std::max<int64_t>(1, std::min(so, nslab));
  g->kc_d = (nslab + sd - 1) / sd * BK;
  g->kc_o = (nslab + so - 1) / so * BK;
  g->s_d = (int)((g->K + g->kc_d - 1) / g->kc_d);  // no empty K ranges
  g->s_o = (int)((g->K + g->kc_o - 1) / g->kc_o);
  return max_tiles <= 0 || (int64_t)g->nt * g->s_d + noff * g->s_o <= max_tiles;
}

int64_t syrk_tiles(const SyrkGeom& g) {
  return (int64_t)g.nt * g.s_d + (int64_t)g.nt * (g.nt - 1) / 2 * g.s_o;
}

// float4 loads of the rows need 16-byte aligned rows: K % 4 == 0 and a
// 16-byte aligned base (a complex64 pointer is only 8-byte aligned in general).
bool vector_loads_ok(const void* X, int64_t K) {
  return (K & 3) == 0 && (reinterpret_cast<uintptr_t>(X) & 15) == 0;
}

int launch_syrk(const float* X, const SyrkGeom& g, const float* sign, float* partials, double* V, cudaStream_t s) {
  const int attr = ensure_smem_limit(reinterpret_cast<const void*>(syrk_fp32_kernel), (int)SYRK_SMEM,
                                     "cudaFuncSetAttribute(syrk_fp32_kernel)");
  if (attr != PI_OK) return attr;
  const int64_t ctas = syrk_tiles(g);
  if (ctas > 0x7fffffffLL) return fail(PI_ERR_UNSUPPORTED, "too many objects for the FP32 contraction");
  syrk_fp32_kernel<<<(unsigned)ctas, NT, SYRK_SMEM, s>>>(X, g, sign, vector_loads_ok(X, g.K), partials);
  PI_LAUNCHED("syrk_fp32_kernel");
  const int64_t total = (int64_t)g.n * g.n;
  reduce_tiles_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(partials, g, V);
  PI_LAUNCHED("reduce_tiles_kernel");
  return PI_OK;
}

}  // namespace

size_t contract_fp32_ws_bytes(int64_t Q, int n) {
  if (n <= 0 || Q <= 0) return 0;
  SyrkGeom g;
  plan_syrk(Q, n, &g);
  return (size_t)syrk_tiles(g) * TB * TB * sizeof(float);
}

int launch_contract_fp32(const pi_kgrid_impl* kg, const float2* Jw, int n, double* V, void* ws, size_t ws_bytes,
                         cudaStream_t s) {
  if (n <= 0) return PI_OK;
  SyrkGeom g;
  plan_syrk(kg->Q, n, &g);
  const size_t need = (size_t)syrk_tiles(g) * TB * TB * sizeof(float);
  if (ws_bytes < need || (need && !ws)) return fail(PI_ERR_WORKSPACE_TOO_SMALL, "contraction workspace too small");
  return launch_syrk(reinterpret_cast<const float*>(Jw), g, kg->all_positive ? nullptr : kg->dev.sign,
                     static_cast<float*>(ws), V, s);
}

// ---------------------------------------------------------------------------
// Allocation-free variant of the FP32 contraction (pi_contract_fp32_static).
//
// Some callers cannot call cudaMalloc: applications whose device memory is
// owned by a host framework (a pool or arena reserved up front, from which a
// library may not allocate), and latency-critical loops in which a
// cudaMalloc / cudaFree would synchronise the device.  For them the split-K
// partial tiles live in this file-scope device array instead of a caller
// workspace.  Every GPU that loads the library holds these 8 MiB until the
// process exits.  All calls share the array: two calls whose kernels overlap
// on the GPU (different streams, or different host threads) race on it and
// must be ordered by the caller.  The partial tiles are fully written by the
// first kernel before the second kernel reads them, so nothing in the array
// needs to start at zero and what the previous call left there is never read.
// The plan caps the partial tiles at the array's 128 tiles of 128 x 128
// floats by lowering the K split, so every object count up to 15 tiles of
// 128 (n <= 1920: 120 tiles of the upper triangle, one CTA each) fits on any
// GPU and only larger ones are rejected.
// The array's device address is looked up once per device and kept for the
// life of the process: the entry point must not be used across a
// cudaDeviceReset (or any teardown of the device's primary context), after
// which that address is stale.
// ---------------------------------------------------------------------------
constexpr size_t PI_STATIC_SCRATCH_BYTES = size_t(8) << 20;  // 8 MiB of partial tiles
constexpr int64_t PI_STATIC_MAX_TILES = PI_STATIC_SCRATCH_BYTES / (TB * TB * sizeof(float));  // 128
static __device__ __align__(256) float g_static_partials[PI_STATIC_SCRATCH_BYTES / sizeof(float)];

namespace {
std::mutex g_static_mu;
float* g_static_ptr[256] = {};  // per device: device address of g_static_partials
}  // namespace

}  // namespace pi

extern "C" int pi_contract_fp32_static(const void* d_Jw, int64_t Q, int n, const float* d_sign, double* d_V,
                                       pi_stream stream) {
  using namespace pi;
  if (n < 0 || Q <= 0 || (n > 0 && (!d_Jw || !d_V)))
    return fail(PI_ERR_INVALID_ARGUMENT, "pi_contract_fp32_static: bad arguments");
  if (n == 0) return PI_OK;
  int dev = 0;
  PI_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 256) return fail(PI_ERR_UNSUPPORTED, "pi_contract_fp32_static: device index beyond 255");
  SyrkGeom g;
  if (!plan_syrk(Q, n, &g, PI_STATIC_MAX_TILES)) {
    char buf[200];
    snprintf(buf, sizeof buf,
             "pi_contract_fp32_static: %d objects need %lld partial tiles of 64 KiB, above the fixed %zu-byte "
             "device array (at most 1920 objects); use pi_contract with a caller workspace",
             n, (long long)syrk_tiles(g), PI_STATIC_SCRATCH_BYTES);
    return fail(PI_ERR_WORKSPACE_TOO_SMALL, buf);
  }
  float* scratch = nullptr;
  {
    // First call on a device: look up the array's device address with that
    // device current (host code cannot use the symbol itself as a pointer).
    std::lock_guard<std::mutex> lock(g_static_mu);
    if (!g_static_ptr[dev]) {
      void* ptr = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&ptr, g_static_partials);
      if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_static_partials)");
      g_static_ptr[dev] = static_cast<float*>(ptr);
    }
    scratch = g_static_ptr[dev];
  }
  return launch_syrk(static_cast<const float*>(d_Jw), g, d_sign, scratch, d_V, reinterpret_cast<cudaStream_t>(stream));
}
