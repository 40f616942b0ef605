// Volume contraction V = Re(J^H diag(w) J) / (8 pi^3), plain FP32 form.
//
// Replaces K9 (cpp/src/compute_intersection_volume.cu:33-50: one global FP64
// atomicAdd per k-node) and K14 (cpp/src/compute_intersection_volume_multi_object.cu:74-116:
// one thread per (i,j) streaming all of J with no tiling).  With the operand
// X = [Re sqrt|w| J ; Im sqrt|w| J] (n x 2Q real, the layout the form-factor
// kernel writes), V is the SYRK X diag(sign) X^T.  Upper-triangle 64x64 output
// tiles x split-K; each thread owns a 4x4 register block and sums every 32-wide
// K slab into a fresh block before adding it, Kahan-compensated, to its
// running sum (off-diagonal entries are small differences of large slab sums).
// Per-split partial tiles are
// reduced in a fixed order (compensated FP32, ~48 bits) by a second kernel:
// results are bitwise reproducible run to run.
#include <cuda_runtime.h>
#include <cstdint>
#include <algorithm>
#include <mutex>
#include "pi_internal.h"
#include "dfmath.cuh"

namespace pi {

namespace {

constexpr int TB = 64;   // output tile edge
constexpr int KT = 32;   // K slab staged in shared memory
constexpr int PAD = 4;
constexpr double INV8PI3 = 1.0 / (8.0 * 3.14159265358979323846 * 3.14159265358979323846 * 3.14159265358979323846);

__device__ __forceinline__ void tile_of(int p, int nt, int* bi, int* bj) {
  int i = 0, rem = p;
  while (rem >= nt - i) { rem -= nt - i; ++i; }
  *bi = i; *bj = i + rem;
}

__device__ __forceinline__ float4 load4(const float* __restrict__ row, int64_t kk, int64_t kend, bool vec) {
  if (vec && kk + 3 < kend) return *reinterpret_cast<const float4*>(row + kk);
  float4 v;
  v.x = kk < kend ? row[kk] : 0.f;
  v.y = kk + 1 < kend ? row[kk + 1] : 0.f;
  v.z = kk + 2 < kend ? row[kk + 2] : 0.f;
  v.w = kk + 3 < kend ? row[kk + 3] : 0.f;
  return v;
}

__global__ void __launch_bounds__(256, 2)
syrk_fp32_kernel(const float* __restrict__ X, int n, int64_t K, const float* __restrict__ sign, int nt,
                 int64_t kchunk, float* __restrict__ partials) {
  int bi, bj;
  tile_of(blockIdx.x, nt, &bi, &bj);
  const int64_t k0 = (int64_t)blockIdx.y * kchunk;
  const int64_t k1 = min(K, k0 + kchunk);
  __shared__ __align__(16) float As[KT][TB + PAD];
  __shared__ __align__(16) float Bs[KT][TB + PAD];
  const int tid = threadIdx.x, ty = tid >> 4, tx = tid & 15;
  const bool vec = (K & 3) == 0;
  float acc[4][4], cmp[4][4];  // running sum + Kahan compensation
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int c = 0; c < 4; ++c) { acc[a][c] = 0.f; cmp[a][c] = 0.f; }

  for (int64_t k = k0; k < k1; k += KT) {
#pragma unroll
    for (int l = 0; l < 2; ++l) {
      const int idx = tid + 256 * l;
      const int row = idx >> 3, c4 = idx & 7;
      const int64_t kk = k + 4 * c4;
      const int gi = bi * TB + row, gj = bj * TB + row;
      float4 va = gi < n ? load4(X + (int64_t)gi * K, kk, k1, vec) : make_float4(0.f, 0.f, 0.f, 0.f);
      float4 vb = gj < n ? load4(X + (int64_t)gj * K, kk, k1, vec) : make_float4(0.f, 0.f, 0.f, 0.f);
      if (sign) {  // negative quadrature weights: V = X diag(sign) X^T; kk is a multiple of 4
        if (kk < K) { const float sg = sign[kk >> 1]; vb.x *= sg; vb.y *= sg; }
        if (kk + 2 < K) { const float sg = sign[(kk + 2) >> 1]; vb.z *= sg; vb.w *= sg; }
      }
      As[4 * c4 + 0][row] = va.x; As[4 * c4 + 1][row] = va.y; As[4 * c4 + 2][row] = va.z; As[4 * c4 + 3][row] = va.w;
      Bs[4 * c4 + 0][row] = vb.x; Bs[4 * c4 + 1][row] = vb.y; Bs[4 * c4 + 2][row] = vb.z; Bs[4 * c4 + 3][row] = vb.w;
    }
    __syncthreads();
    float part[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int c = 0; c < 4; ++c) part[a][c] = 0.f;
#pragma unroll 8
    for (int kk = 0; kk < KT; ++kk) {
      const float4 av = *reinterpret_cast<const float4*>(&As[kk][ty * 4]);
      const float4 bv = *reinterpret_cast<const float4*>(&Bs[kk][tx * 4]);
      const float ar[4] = {av.x, av.y, av.z, av.w}, br[4] = {bv.x, bv.y, bv.z, bv.w};
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int c = 0; c < 4; ++c) part[a][c] = fmaf(ar[a], br[c], part[a][c]);
    }
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int c = 0; c < 4; ++c) {  // Kahan: the slab sums of an off-diagonal entry cancel
        const float y = part[a][c] - cmp[a][c];
        const float t = acc[a][c] + y;
        cmp[a][c] = (t - acc[a][c]) - y;
        acc[a][c] = t;
      }
    __syncthreads();
  }
  float* out = partials + ((int64_t)blockIdx.y * gridDim.x + blockIdx.x) * (TB * TB);
#pragma unroll
  for (int a = 0; a < 4; ++a)
    *reinterpret_cast<float4*>(&out[(ty * 4 + a) * TB + tx * 4]) = make_float4(acc[a][0], acc[a][1], acc[a][2], acc[a][3]);
}

// Fixed-order compensated sum of the split partials, scaled by 1/(8 pi^3), mirrored;
// one thread per output element of the upper-triangle tiles.
__global__ void reduce_tiles_kernel(const float* __restrict__ partials, int nsplit, int npairs, int nt, int n,
                                    double* __restrict__ V) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)npairs * TB * TB) return;
  const int p = (int)(t / (TB * TB)), e = (int)(t % (TB * TB));
  int bi, bj;
  tile_of(p, nt, &bi, &bj);
  const int r = e / TB, c = e % TB;
  const int i = bi * TB + r, j = bj * TB + c;
  if (i >= n || j >= n || (bi == bj && r > c)) return;
  // compensated FP32 sum in split order (FP64 adds run at 1/64 of the FP32 rate)
  kbsum acc{0.f, 0.f};
  const float* src = partials + (int64_t)p * (TB * TB) + e;
  const int64_t stride = (int64_t)npairs * (TB * TB);
  int sp = 0;
  for (; sp + 16 <= nsplit; sp += 16) {  // sixteen loads in flight ahead of their adds
    float v[16];
#pragma unroll
    for (int u = 0; u < 16; ++u) v[u] = __ldcs(src + (sp + u) * stride);
#pragma unroll
    for (int u = 0; u < 16; ++u) acc.add(v[u]);
  }
  for (; sp < nsplit; ++sp) acc.add(__ldcs(src + sp * stride));
  const double s = acc.value() * INV8PI3;
  V[(int64_t)i * n + j] = s;
  V[(int64_t)j * n + i] = s;
}

struct SyrkPlan { int nt, npairs, nsplit; int64_t K, kchunk; };

SyrkPlan plan_syrk(int64_t Q, int n) {
  SyrkPlan p;
  p.K = 2 * Q;
  p.nt = (n + TB - 1) / TB;
  p.npairs = p.nt * (p.nt + 1) / 2;
  int dev = 0, sms = 148;
  if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int64_t target = 2LL * sms;
  int64_t nsplit = (target + p.npairs - 1) / p.npairs;
  const int64_t max_split = std::max<int64_t>(1, p.K / (8 * KT));
  nsplit = std::max<int64_t>(1, std::min<int64_t>(nsplit, max_split));
  int64_t chunk = (p.K + nsplit - 1) / nsplit;
  chunk = (chunk + KT - 1) / KT * KT;
  p.kchunk = std::max<int64_t>(chunk, KT);
  p.nsplit = (int)((p.K + p.kchunk - 1) / p.kchunk);
  return p;
}

}  // namespace

size_t contract_fp32_ws_bytes(int64_t Q, int n) {
  if (n <= 0 || Q <= 0) return 0;
  SyrkPlan p = plan_syrk(Q, n);
  return (size_t)p.nsplit * p.npairs * TB * TB * sizeof(float);
}

int launch_contract_fp32(const pi_kgrid_impl* kg, const float2* Jw, int n, double* V, void* ws, size_t ws_bytes,
                         cudaStream_t s) {
  if (n <= 0) return PI_OK;
  SyrkPlan p = plan_syrk(kg->Q, n);
  const size_t need = (size_t)p.nsplit * p.npairs * TB * TB * sizeof(float);
  if (ws_bytes < need || (need && !ws)) return fail(PI_ERR_WORKSPACE_TOO_SMALL, "contraction workspace too small");
  if (p.npairs > 65535 * 64) return fail(PI_ERR_UNSUPPORTED, "too many objects for the FP32 contraction");
  dim3 grid((unsigned)p.npairs, (unsigned)p.nsplit);
  syrk_fp32_kernel<<<grid, 256, 0, s>>>(reinterpret_cast<const float*>(Jw), n, p.K,
                                        kg->all_positive ? nullptr : kg->dev.sign, p.nt, p.kchunk,
                                        static_cast<float*>(ws));
  PI_LAUNCHED("syrk_fp32_kernel");
  const int64_t total = (int64_t)p.npairs * TB * TB;
  reduce_tiles_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(static_cast<const float*>(ws), p.nsplit,
                                                                      p.npairs, p.nt, n, V);
  PI_LAUNCHED("reduce_tiles_kernel");
  return PI_OK;
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
// ---------------------------------------------------------------------------
constexpr size_t PI_STATIC_SCRATCH_BYTES = size_t(8) << 20;  // 8 MiB of partial tiles
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
  SyrkPlan p = plan_syrk(Q, n);
  const size_t need = (size_t)p.nsplit * p.npairs * TB * TB * sizeof(float);
  if (need > PI_STATIC_SCRATCH_BYTES) {
    char buf[200];
    snprintf(buf, sizeof buf,
             "pi_contract_fp32_static: %d objects need %zu bytes of partial tiles, above the fixed %zu-byte "
             "device array; use pi_contract with a caller workspace",
             n, need, PI_STATIC_SCRATCH_BYTES);
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
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  dim3 grid((unsigned)p.npairs, (unsigned)p.nsplit);
  syrk_fp32_kernel<<<grid, 256, 0, s>>>(static_cast<const float*>(d_Jw), n, p.K, d_sign, p.nt, p.kchunk, scratch);
  PI_LAUNCHED("syrk_fp32_kernel");
  const int64_t total = (int64_t)p.npairs * TB * TB;
  reduce_tiles_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(scratch, p.nsplit, p.npairs, p.nt, n, d_V);
  PI_LAUNCHED("reduce_tiles_kernel");
  return PI_OK;
}
