// Volume contraction on tcgen05 tensor cores: hi+lo split operands (BF16 or
// TF32), FP32 accumulation.
//
// V = X X^T with X = [Re sqrt|w| J ; Im sqrt|w| J] (n x 2Q, the FP32 layout the
// form-factor kernel writes).  Each FP32 operand value x is split into
// h = bf16(x) and l = bf16(x - h) while it is staged, and every output tile
// accumulates  H_i H_j^T + H_i L_j^T + L_i H_j^T  (the l.l term, ~2^-16
// relative, is dropped) in a 128x128 FP32 accumulator in tensor memory.
//
// CTA = 8 producer warps + 1 MMA warp.  Work unit = (upper-triangle pair of
// 128-row object blocks, K range).  Producers load 8 FP32 values per thread
// per step (coalesced 32-byte rows), split them, and store both halves into a
// 3-stage ring of 128-byte-swizzled K-major tiles (the canonical layout of
// the UMMA shared-memory descriptors); an elected thread of the MMA warp
// issues tcgen05.mma (M = N = 128, K = 16) three times per K step and commits
// each stage back to the producers through an mbarrier.  The epilogue reads
// the accumulator with tcgen05.ld and writes a per-unit FP32 partial tile;
// a second kernel sums the partials in a fixed order (compensated FP32).
//
// Every wait is bounded (~2 s of SM clock); on expiry the kernel records an
// error code in the workspace, stops issuing work, drains its outstanding
// MMAs, frees its tensor memory and returns; the reduction then writes NaN to
// V so a failure can never read as a volume.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cstdint>
#include <algorithm>
#include <mutex>
#include "pi_internal.h"
#include "dfmath.cuh"
#include "tc_ptx.cuh"

namespace pi {

namespace {

using namespace tc;

constexpr int TC_M = 128;                       // tile edge (objects)
constexpr int TC_STAGES = 3;
constexpr int TC_MAX_CHUNKS = 16;                // K stages per CTA (accumulation-error bound)
constexpr int TC_PWARPS = 8;                    // converter warps
constexpr int TC_TMA_WARP = TC_PWARPS;          // lane 0 issues the TMA loads
constexpr int TC_MMA_WARP = TC_PWARPS + 1;      // lane 0 issues the MMAs; the warp owns TMEM
constexpr int TC_THREADS = (TC_PWARPS + 2) * 32;
constexpr int BLK_BYTES = TC_M * 128;           // 16 KB: one operand block, 128-byte K rows
constexpr int STAGE_BYTES = 4 * BLK_BYTES;      // A hi, A lo, B hi, B lo
constexpr int SMEM_BYTES = TC_STAGES * STAGE_BYTES + 1024;  // + alignment slack
constexpr double INV8PI3 = 1.0 / (8.0 * 3.14159265358979323846 * 3.14159265358979323846 * 3.14159265358979323846);

// Operand kinds.  A 128-byte K row holds 64 BF16 or 32 TF32 values; each
// 16-byte chunk of it is produced from EPC FP32 inputs (EPC = 8 or 4).
enum { KIND_BF16 = 0, KIND_TF32 = 1 };
template <int KIND> struct Kind;
template <> struct Kind<KIND_BF16> { static constexpr int EPC = 8; static constexpr uint32_t FMT = 1; };
template <> struct Kind<KIND_TF32> { static constexpr int EPC = 4; static constexpr uint32_t FMT = 2; };

// Instruction descriptor (kind::f16 / kind::tf32): D = F32 (bits 4-5 = 1), A and
// B format at bits 7-9 / 10-12 (1 = BF16, 2 = TF32), both K-major, N >> 3 at
// bits 17-22, M >> 4 at bits 24-28.
template <int KIND>
__host__ __device__ constexpr uint32_t idesc() { return tc::idesc(Kind<KIND>::FMT, TC_M, TC_M); }

enum { ERR_PRODUCER_WAIT = 1, ERR_MMA_WAIT = 2, ERR_EPILOGUE_WAIT = 3, ERR_TMA_WAIT = 4 };

template <int KIND>
__device__ __forceinline__ void umma(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t accumulate) {
  if (KIND == KIND_BF16) umma_f16(tmem_d, a, b, idesc<KIND_BF16>(), accumulate);
  else umma_tf32(tmem_d, a, b, idesc<KIND_TF32>(), accumulate);
}

__device__ __forceinline__ bool converters_any(bool pred) { return bar_any(1, TC_PWARPS * 32, pred); }

__device__ __forceinline__ void tile_of(int p, int nt, int* bi, int* bj) {
  int i = 0, rem = p;
  while (rem >= nt - i) { rem -= nt - i; ++i; }
  *bi = i; *bj = i + rem;
}

template <int KIND>
__global__ void __launch_bounds__(TC_THREADS, 1)
syrk_split3_kernel(const __grid_constant__ CUtensorMap xmap, int n, int64_t K, int nt, int64_t nchunks, int64_t cps,
                   float* __restrict__ partials, int* __restrict__ err) {
  extern __shared__ uint8_t smem_raw[];
  __shared__ __align__(8) uint64_t tma_bar[TC_STAGES];
  __shared__ __align__(8) uint64_t full_bar[TC_STAGES];
  __shared__ __align__(8) uint64_t empty_bar[TC_STAGES];
  __shared__ __align__(8) uint64_t done_bar;
  __shared__ uint32_t tmem_slot;

  uint8_t* smem = smem_raw + ((1024 - (smem_u32(smem_raw) & 1023)) & 1023);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  int bi, bj;
  tile_of(blockIdx.x, nt, &bi, &bj);
  const bool diag = bi == bj;
  const int64_t c0 = (int64_t)blockIdx.y * cps;
  const int64_t nc = max((int64_t)0, min(nchunks, c0 + cps) - c0);

  if (tid == 0) {
    for (int s = 0; s < TC_STAGES; ++s) {
      mbar_init(smem_u32(&tma_bar[s]), 1);
      mbar_init(smem_u32(&full_bar[s]), TC_PWARPS);
      mbar_init(smem_u32(&empty_bar[s]), 1);
    }
    mbar_init(smem_u32(&done_bar), 1);
    fence_mbar_init();
  }
  if (warp == TC_MMA_WARP) {
    tmem_alloc(smem_u32(&tmem_slot), 2 * TC_M);
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = tmem_slot;          // main accumulator (hi.hi)
  const uint32_t tmem_c = tmem + TC_M;      // correction accumulator (hi.lo + lo.hi)

  constexpr int EPC = Kind<KIND>::EPC;
  constexpr int KC = 8 * EPC;                              // K elements per stage
  constexpr uint32_t BOX_BYTES = TC_M * KC * 4;            // FP32 box of one 128-row block
  // BF16: the 32 KB FP32 box fills the block's 32 KB hi+lo region; TF32: the
  // 16 KB box lands in the upper half.  Either way the split is done in place.
  constexpr uint32_t BOX_OFF = 2 * BLK_BYTES - BOX_BYTES;
  if (warp == TC_TMA_WARP) {
    // ---------------- TMA: FP32 J tiles into the stage ring ----------------
    if (lane == 0) {
      int64_t issued = 0;
      for (int64_t c = 0; c < nc; ++c) {
        const int s = (int)(c % TC_STAGES);
        const int64_t r = c / TC_STAGES;
        if (r > 0 && !mbar_wait(smem_u32(&empty_bar[s]), (uint32_t)((r - 1) & 1), err, ERR_TMA_WAIT)) break;
        const uint32_t st = smem_u32(smem + s * STAGE_BYTES);
        const int x = (int)((c0 + c) * KC);
        mbar_expect_tx(smem_u32(&tma_bar[s]), diag ? BOX_BYTES : 2 * BOX_BYTES);
        tma_load_2d(st + BOX_OFF, &xmap, x, bi * TC_M, smem_u32(&tma_bar[s]));
        if (!diag) tma_load_2d(st + 2 * BLK_BYTES + BOX_OFF, &xmap, x, bj * TC_M, smem_u32(&tma_bar[s]));
        issued = c + 1;
      }
      // Never leave this CTA with a copy still landing in its shared memory:
      // wait (bounded) for the last load issued into every stage.
      for (int64_t c = max((int64_t)0, issued - TC_STAGES); c < issued; ++c)
        mbar_drain(smem_u32(&tma_bar[c % TC_STAGES]), (uint32_t)((c / TC_STAGES) & 1));
    }
  } else if (warp < TC_PWARPS) {
    // ---------------- converters: FP32 box -> hi/lo split, 128-byte swizzled K-major ----------------
    constexpr int UPT = 2 * TC_M * 8 / (TC_PWARPS * 32);  // 16-byte output chunks per thread (off-diagonal pair)
    const int upt = diag ? UPT / 2 : UPT;
    for (int64_t c = 0; c < nc; ++c) {
      const int s = (int)(c % TC_STAGES);
      const int64_t r = c / TC_STAGES;
      bool ok = mbar_wait(smem_u32(&tma_bar[s]), (uint32_t)(r & 1), err, ERR_PRODUCER_WAIT);
      uint8_t* st = smem + s * STAGE_BYTES;
      float x[UPT][EPC];
      if (ok) {
#pragma unroll
        for (int i = 0; i < UPT; ++i) {
          if (i >= upt) break;
          const int u = tid + i * TC_PWARPS * 32;
          const int blk = u >= TC_M * 8;
          const int uu = u - blk * TC_M * 8;
          const int row = uu >> 3, ch = uu & 7;
          const float4* src = reinterpret_cast<const float4*>(st + blk * 2 * BLK_BYTES + BOX_OFF + row * (KC * 4) +
                                                             ch * (EPC * 4));
#pragma unroll
          for (int v = 0; v < EPC / 4; ++v) {
            const float4 a = src[v];
            x[i][4 * v] = a.x; x[i][4 * v + 1] = a.y; x[i][4 * v + 2] = a.z; x[i][4 * v + 3] = a.w;
          }
        }
      }
      // every converter has read its inputs before any output overwrites the
      // box; all converters leave together if any of them saw an error
      if (converters_any(!ok)) break;
#pragma unroll
      for (int i = 0; i < UPT; ++i) {
        if (i >= upt) break;
        const int u = tid + i * TC_PWARPS * 32;
        const int blk = u >= TC_M * 8;
        const int uu = u - blk * TC_M * 8;
        const int row = uu >> 3, ch = uu & 7;
        uint4 hi, lo;
        if (KIND == KIND_BF16) split8(x[i], &hi, &lo);
        else split4_tf32(x[i], &hi, &lo);
        const uint32_t off = (uint32_t)((row >> 3) * 1024 + (row & 7) * 128 + ((ch ^ (row & 7)) << 4));
        uint8_t* base = st + (blk ? 2 * BLK_BYTES : 0);
        *reinterpret_cast<uint4*>(base + off) = hi;
        *reinterpret_cast<uint4*>(base + BLK_BYTES + off) = lo;
      }
      fence_proxy_async();
      __syncwarp();
      if (lane == 0) mbar_arrive(smem_u32(&full_bar[s]));
    }
  } else if (warp == TC_MMA_WARP && lane == 0) {
    // ---------------- MMA issuer ----------------
    for (int64_t c = 0; c < nc; ++c) {
      const int s = (int)(c % TC_STAGES);
      const int64_t r = c / TC_STAGES;
      if (!mbar_wait(smem_u32(&full_bar[s]), (uint32_t)(r & 1), err, ERR_MMA_WAIT)) break;
      fence_after();
      const uint32_t st = smem_u32(smem + s * STAGE_BYTES);
      const uint64_t aH = desc_sw128(st), aL = desc_sw128(st + BLK_BYTES);
      const uint64_t bH = diag ? aH : desc_sw128(st + 2 * BLK_BYTES);
      const uint64_t bL = diag ? aL : desc_sw128(st + 3 * BLK_BYTES);
#pragma unroll
      for (int k = 0; k < 4; ++k) {  // one MMA covers 32 bytes of K (16 BF16 / 8 TF32)
        const uint64_t adv = (uint64_t)(k * 32) >> 4;  // +32 bytes along K inside the swizzled row
        const uint32_t acc = (c > 0 || k > 0) ? 1u : 0u;
        umma<KIND>(tmem, aH + adv, bH + adv, acc);
        umma<KIND>(tmem_c, aH + adv, bL + adv, acc);
        umma<KIND>(tmem_c, aL + adv, bH + adv, 1u);
      }
      umma_commit(smem_u32(&empty_bar[s]));
    }
    umma_commit(smem_u32(&done_bar));  // arrives once every issued MMA has completed
  }

  // ---------------- epilogue: TMEM -> FP32 partial tile ----------------
  if (warp < 4) {
    // every lane takes the same decision before the warp-collective tensor-memory loads
    const bool ok = __all_sync(0xffffffffu, mbar_wait(smem_u32(&done_bar), 0u, err, ERR_EPILOGUE_WAIT));
    fence_after();
    const int row = warp * 32 + lane;
    float* out = partials + ((int64_t)blockIdx.y * gridDim.x + blockIdx.x) * (TC_M * TC_M) + (int64_t)row * TC_M;
#pragma unroll 1
    for (int cb = 0; cb < TC_M / 32; ++cb) {
      float v[32];
      if (ok && nc > 0) {
        float cc[32];
        tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(cb * 32), v);
        tmem_ld32(tmem_c + ((uint32_t)(warp * 32) << 16) + (uint32_t)(cb * 32), cc);
#pragma unroll
        for (int i = 0; i < 32; ++i) v[i] += cc[i];
      } else {
#pragma unroll
        for (int i = 0; i < 32; ++i) v[i] = 0.f;
      }
#pragma unroll
      for (int i = 0; i < 32; i += 4)
        *reinterpret_cast<float4*>(out + cb * 32 + i) = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
    }
  }
  fence_before();
  __syncthreads();
  if (warp == TC_MMA_WARP) {
    __syncwarp();
    fence_after();
    tmem_dealloc(tmem, 2 * TC_M);
  }
}

// One thread per output element of the upper-triangle tiles.
__global__ void reduce_tc_tiles_kernel(const float* __restrict__ partials, int nsplit, int npairs, int nt, int n,
                                       const int* __restrict__ err, double* __restrict__ V) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)npairs * TC_M * TC_M) return;
  const int p = (int)(t / (TC_M * TC_M)), e = (int)(t % (TC_M * TC_M));
  int bi, bj;
  tile_of(p, nt, &bi, &bj);
  const int r = e / TC_M, c = e % TC_M;
  const int i = bi * TC_M + r, j = bj * TC_M + c;
  if (i >= n || j >= n || (bi == bj && r > c)) return;
  // compensated FP32 sum in split order (FP64 adds run at 1/64 of the FP32 rate)
  kbsum acc{0.f, 0.f};
  const float* src = partials + (int64_t)p * (TC_M * TC_M) + e;
  const int64_t stride = (int64_t)npairs * (TC_M * TC_M);
  int sp = 0;
  for (; sp + 16 <= nsplit; sp += 16) {  // sixteen loads in flight ahead of their adds
    float v[16];
#pragma unroll
    for (int u = 0; u < 16; ++u) v[u] = __ldcs(src + (sp + u) * stride);
#pragma unroll
    for (int u = 0; u < 16; ++u) acc.add(v[u]);
  }
  for (; sp < nsplit; ++sp) acc.add(__ldcs(src + sp * stride));
  const double s = (*err != 0) ? __longlong_as_double(0x7ff8000000000000LL) : acc.value() * INV8PI3;
  V[(int64_t)i * n + j] = s;
  V[(int64_t)j * n + i] = s;
}

struct TcPlan { int nt, npairs, nsplit; int64_t K, nchunks, cps; };

TcPlan plan_tc(int64_t Q, int n, int kind) {
  TcPlan p;
  p.K = 2 * Q;
  p.nt = (n + TC_M - 1) / TC_M;
  p.npairs = p.nt * (p.nt + 1) / 2;
  const int64_t kc = kind == KIND_BF16 ? 64 : 32;
  p.nchunks = (p.K + kc - 1) / kc;
  const int sms = current_sm_count();
  // At least one CTA per SM, and at most TC_MAX_CHUNKS chunks (48-96 MMAs
  // each) per accumulator: the tensor cores' FP32 accumulation error grows
  // with the number of MMAs summed into one accumulator.
  int64_t nsplit = std::max<int64_t>(1, sms / p.npairs);
  nsplit = std::max<int64_t>(nsplit, (p.nchunks + TC_MAX_CHUNKS - 1) / TC_MAX_CHUNKS);
  nsplit = std::min<int64_t>(nsplit, p.nchunks);
  p.cps = (p.nchunks + nsplit - 1) / nsplit;
  p.nsplit = (int)((p.nchunks + p.cps - 1) / p.cps);
  return p;
}

}  // namespace

size_t contract_tc_ws_bytes(int64_t Q, int n, int kind) {
  if (n <= 0 || Q <= 0) return 0;
  TcPlan p = plan_tc(Q, n, kind);
  return 256 + (size_t)p.nsplit * p.npairs * TC_M * TC_M * sizeof(float);
}

namespace {
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn encode_tiled() {
  static std::once_flag once;
  static EncodeTiledFn fn = nullptr;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  });
  return fn;
}
}  // namespace

int launch_contract_tc(const pi_kgrid_impl* kg, const float2* Jw, int n, int kind, double* V, void* ws,
                       size_t ws_bytes, cudaStream_t s) {
  if (n <= 0) return PI_OK;
  TcPlan p = plan_tc(kg->Q, n, kind);
  if (p.K % 4 != 0) return fail(PI_ERR_UNSUPPORTED, "tensor-core contraction needs an even node count");
  EncodeTiledFn enc = encode_tiled();
  if (!enc) return fail(PI_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
  CUtensorMap xmap;
  const cuuint64_t gdim[2] = {(cuuint64_t)p.K, (cuuint64_t)n};
  const cuuint64_t gstride[1] = {(cuuint64_t)p.K * sizeof(float)};
  const cuuint32_t box[2] = {(cuuint32_t)(kind == KIND_BF16 ? 64 : 32), (cuuint32_t)TC_M};
  const cuuint32_t estride[2] = {1, 1};
  CUresult cr = enc(&xmap, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float2*>(Jw), gdim, gstride, box, estride,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (cr != CUDA_SUCCESS) return fail(PI_ERR_CUDA, "cuTensorMapEncodeTiled failed for J");
  const size_t need = 256 + (size_t)p.nsplit * p.npairs * TC_M * TC_M * sizeof(float);
  if (ws_bytes < need || !ws) return fail(PI_ERR_WORKSPACE_TOO_SMALL, "tensor-core contraction workspace too small");
  if ((reinterpret_cast<uintptr_t>(Jw) & 15) != 0) return fail(PI_ERR_INVALID_ARGUMENT, "J must be 16-byte aligned");
  {
    const void* fn = kind == KIND_BF16 ? reinterpret_cast<const void*>(syrk_split3_kernel<KIND_BF16>)
                                       : reinterpret_cast<const void*>(syrk_split3_kernel<KIND_TF32>);
    const int rc = ensure_smem_limit(fn, (int)SMEM_BYTES, "cudaFuncSetAttribute(syrk_split3_kernel)");
    if (rc != PI_OK) return rc;
  }
  int* err = static_cast<int*>(ws);
  float* partials = reinterpret_cast<float*>(static_cast<unsigned char*>(ws) + 256);
  PI_CUDA(cudaMemsetAsync(err, 0, sizeof(int), s));
  dim3 grid((unsigned)p.npairs, (unsigned)p.nsplit);
  if (kind == KIND_BF16)
    syrk_split3_kernel<KIND_BF16><<<grid, TC_THREADS, SMEM_BYTES, s>>>(xmap, n, p.K, p.nt, p.nchunks, p.cps,
                                                                      partials, err);
  else
    syrk_split3_kernel<KIND_TF32><<<grid, TC_THREADS, SMEM_BYTES, s>>>(xmap, n, p.K, p.nt, p.nchunks, p.cps,
                                                                      partials, err);
  PI_LAUNCHED("syrk_split3_kernel");
  const int64_t total = (int64_t)p.npairs * TC_M * TC_M;
  reduce_tc_tiles_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(partials, p.nsplit, p.npairs, p.nt, n, err, V);
  PI_LAUNCHED("reduce_tc_tiles_kernel");
  return PI_OK;
}

}  // namespace pi
