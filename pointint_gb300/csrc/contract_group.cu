// Grouped split-precision volume contraction on tcgen05 tensor cores.
//
// Replaces the reference's per-pair FP64 sum K14
// (cpp/src/compute_intersection_volume_multi_object.cu:74-116, one thread per
// (i, j) streaming all Q nodes) for any number of volume matrices at once.
//
// V_ij = sum_q Re(conj(X_iq) X_jq) / (8 pi^3) with X_iq = sqrt(w_q) A_i(k_q)
// e^{i k_q . c_i}.  Rows are read as 64 FP32 values per 32-column chunk; each
// value x (times the row's power-of-two scale s for FP16 operands) is split
// into h = f16(x s) and l = f16(x s - h) (or the BF16 pair, unscaled), and an
// output tile accumulates H_i H_j^T + H_i L_j^T + L_i H_j^T (the l.l term is
// dropped).  The tensor cores' FP32 accumulation error grows with the number
// of MMAs summed into one accumulator, so each accumulator chain spans only
// CHAIN k chunks; the epilogue folds every finished chain into a running FP32
// sum kept in tensor memory (round-to-nearest adds), and a work item can then
// cover a long k range with one partial tile.
//
// Persistent CTA (one per SM) of 23 warps:
//   warps 16-17 loaders.  Rows contiguous in memory (one volume matrix over a
//               caller's J): one lane issues 2D TMA boxes of 128 rows x 32
//               FP32 values, two per tile and chunk.  Rows gathered from
//               anywhere (the serving pool): 16-byte cp.async copies, one
//               warp per tile.  Either way a 3-stage ring of 64 KB stages
//               receives the FP32 values in the 128-byte-swizzled layout of
//               the TMA (16-byte unit u of row r at r * 128 + ((u ^ r % 8) * 16)
//               within each 16 KB half-box), which keeps the converters'
//               reads free of bank conflicts;
//   warps 0-15  converters: each thread takes 8 complex values of one row of
//               each tile, applies the translation phase (direction-major rows:
//               the direction is fixed over the 8 values, so d.c is formed
//               once in double-float and each value needs one product with
//               kmag / 2 pi and a quarter-turn reduction), splits hi/lo and
//               writes both halves back in place as 128-byte-swizzled K-major
//               UMMA operands;
//   warp 18     MMA issuer (one lane) and tensor-memory owner: columns 0-255
//               hold two chain accumulators (double-buffered), 256-383 the
//               running sum;
//   warps 19-22 epilogue: chain -> running sum; at the end of an item the sum
//               goes to the item's FP32 partial tile.
// Every wait is bounded (~2 s of SM clock); on expiry the kernel records an
// error code, every role leaves its loop, in-flight copies and MMAs are
// drained, tensor memory is freed, and the reduction writes NaN.
#include <cuda_runtime.h>
#include <cstdint>
#include <algorithm>
#include <atomic>
#include <mutex>
#include <cstring>
#include "pi_internal.h"
#include "group.h"
#include "dfmath.cuh"
#include "tc_ptx.cuh"

namespace pi {

namespace {

using namespace tc;

constexpr int GM = GROUP_TILE;
constexpr int CK = GROUP_CHUNK;
#ifndef PI_GROUP_CHAIN
#define PI_GROUP_CHAIN 2
#endif
constexpr int CHAIN = PI_GROUP_CHAIN;            // k chunks per tensor-memory accumulation chain
constexpr int OPB = GM * 128;                    // 16,384 B: one 128 x 64 16-bit operand block
constexpr int HALF = GM * 128;                   // 16,384 B: 128 rows x 32 FP32 values (one TMA box)
constexpr int BOXB = 2 * HALF;                   // 32 KB: one tile's FP32 chunk
constexpr int STAGE = 2 * BOXB;                  // 64 KB: two tiles = four operand blocks
constexpr int NST = 3;
constexpr int SMEM = NST * STAGE + 1024;         // + alignment slack
constexpr int CWARPS = 16, LWARP0 = 16, MWARP = 18, EWARP0 = 19, NWARPS = 23;
constexpr int CV = 8;                            // complex values of one row per converter thread and tile
static_assert(CWARPS * 32 * CV == GM * CK, "converters cover a tile's chunk exactly once");
static_assert(LWARP0 + 2 == MWARP && MWARP + 1 == EWARP0 && EWARP0 + 4 == NWARPS, "warp roles");
constexpr int NTHREADS = NWARPS * 32;
constexpr int TMEM_COLS = 512;
constexpr uint32_t SUM_COL = 256;                // running sum columns 256..383
constexpr int RED_THREADS = 256;
static_assert(STAGE % 1024 == 0, "stage base must keep 1024-byte operand alignment");
static_assert(STAGE == 4 * OPB && BOXB == 2 * OPB, "in-place split: a tile's FP32 chunk becomes its hi and lo blocks");

// Byte offset of 16-byte unit u (0..15) of row r in a tile's staged chunk.
__device__ __forceinline__ uint32_t stage_off(int r, int u) {
  return (uint32_t)((u >> 3) * HALF + r * 128 + (((u & 7) ^ (r & 7)) << 4));
}

// kind::f16 operand format: 0 = F16, 1 = BF16.
template <int OP> constexpr uint32_t op_idesc() { return idesc(OP == GROUP_OP_F16 ? 0u : 1u, GM, GM); }

enum { ERR_LOAD = 1, ERR_CONVERT = 2, ERR_MMA = 3, ERR_EPILOGUE = 4, ERR_CAPACITY = 5 };

// x[0..2 NV - 1] = NV complex values of one row of a direction-major row
// (col = j L + r), at radii r0 .. r0 + NV - 1 of one direction (L is a
// multiple of 16).  Multiplies them by e^{2 pi i kturn_r (d_j . c)}.
// d: the direction's staged hi, lo pair.
template <int NV>
__device__ __forceinline__ void apply_phase(float* x, int r0, float3 ch, float3 cl, const float2* kt, const float4* d) {
  const float4 h = d[0], l = d[1];
  const df s = cdot2(make_float3(h.x, h.y, h.z), make_float3(l.x, l.y, l.z), ch, cl);
#pragma unroll
  for (int i = 0; i < NV; ++i) {
    const float2 k = kt[r0 + i];
    // turns = kturn * s: the integer part of the leading product is removed
    // exactly; the rounding error of that product and the small cross terms
    // are added back to the fraction.
    const float p = k.x * s.hi;
    const float e = fmaf(k.x, s.hi, -p);
    const float t = (p - rintf(p)) + fmaf(k.y, s.hi, fmaf(k.x, s.lo, e));  // |t| <= 1/2 + 2^-20
    // Each value is rotated once, so the hardware sine/cosine on |2 pi t| <= pi
    // (absolute error ~4e-7) enters V as independent per-value noise, far
    // below the split contraction's 1e-4; it is a third of the polynomial's
    // instructions on the converters' critical path.
    float sn, cs;
    __sincosf(6.283185307179586f * t, &sn, &cs);
    const float re = x[2 * i], im = x[2 * i + 1];
    x[2 * i] = fmaf(re, cs, -im * sn);
    x[2 * i + 1] = fmaf(re, sn, im * cs);
  }
}

// Split 8 NU FP32 values (part q of a 64-value K row), times the row scale,
// into 16-bit hi and lo and store both, 128-byte swizzled: K chunk (16 B) u of
// row r lives at (r / 8) * 1024 + (r % 8) * 128 + ((u ^ (r % 8)) * 16), and
// part q covers units NU q .. NU q + NU - 1.
template <int OP, int NU>
__device__ __forceinline__ void store_split(uint8_t* op, int row, int q, const float* x, float scale) {
  const uint32_t rb = (uint32_t)((row >> 3) * 1024 + (row & 7) * 128);
#pragma unroll
  for (int p = 0; p < NU; ++p) {
    uint32_t hi[4], lo[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const float a = x[8 * p + 2 * i], b = x[8 * p + 2 * i + 1];
      if (OP == GROUP_OP_F16) split2_f16(a * scale, b * scale, &hi[i], &lo[i]);
      else split2_bf16(a, b, &hi[i], &lo[i]);
    }
    const uint32_t off = rb + ((uint32_t)((NU * q + p) ^ (row & 7)) << 4);
    *reinterpret_cast<uint4*>(op + off) = make_uint4(hi[0], hi[1], hi[2], hi[3]);
    *reinterpret_cast<uint4*>(op + OPB + off) = make_uint4(lo[0], lo[1], lo[2], lo[3]);
  }
}

__device__ __forceinline__ float row_scale(const GRow& r, int op) {
  return (op == GROUP_OP_F16 && r.amax) ? group_row_scale(*r.amax) : 1.f;
}

template <int OP, bool PHASE, bool TMA>
__global__ void __launch_bounds__(NTHREADS, 1)
group_split3_kernel(const GroupDev g, const __grid_constant__ CUtensorMap xmap) {
  extern __shared__ uint8_t smem_raw[];
  __shared__ __align__(8) uint64_t load_bar[NST];
  __shared__ __align__(8) uint64_t full_bar[NST];
  __shared__ __align__(8) uint64_t empty_bar[NST];
  __shared__ __align__(8) uint64_t chf_bar[2];     // chain accumulator b is complete
  __shared__ __align__(8) uint64_t che_bar[2];     // chain accumulator b has been read
  __shared__ __align__(8) uint64_t fin_bar;
  __shared__ uint32_t tmem_slot;
  __shared__ float2 kt[PHASE ? GROUP_MAX_L : 1];
  __shared__ __align__(16) float4 sdir[PHASE ? NST : 1][4];  // per stage: hi, lo of the chunk's (up to) two directions

  uint8_t* smem = smem_raw + ((1024 - (smem_u32(smem_raw) & 1023)) & 1023);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  int* err = g.err;
  const long long wlim = g.wait_cycles > 0 ? (long long)g.wait_cycles : WAIT_CYCLES;
  int n_items = g.hdr->n_items;
  if (n_items > g.max_items) {  // descriptor inconsistent with the partial arena: do no work
    if (threadIdx.x == 0 && blockIdx.x == 0) atomicCAS(err, 0, ERR_CAPACITY);
    n_items = 0;
  }

  if (tid == 0) {
    for (int s = 0; s < NST; ++s) {
      mbar_init(smem_u32(&load_bar[s]), TMA ? 1 : 64);  // expect_tx arrival, or one cp.async arrival per loader lane
      mbar_init(smem_u32(&full_bar[s]), CWARPS);
      mbar_init(smem_u32(&empty_bar[s]), 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(smem_u32(&chf_bar[b]), 1);
      mbar_init(smem_u32(&che_bar[b]), 4);
    }
    mbar_init(smem_u32(&fin_bar), 1);
    fence_mbar_init();
  }
  if (PHASE)
    for (int r = tid; r < g.L; r += NTHREADS) kt[r] = g.kturn[r];
  if (warp == MWARP) tmem_alloc(smem_u32(&tmem_slot), TMEM_COLS);
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = tmem_slot;

  if (warp == LWARP0 || warp == LWARP0 + 1) {
    // ---------------- loaders ----------------
    const int box = warp - LWARP0;
    int64_t gc = 0, issued = 0;
    bool ok = true;
    if (TMA) {
      if (box == 0 && lane == 0) {
        for (int it = blockIdx.x; it < n_items && ok; it += gridDim.x) {
          const GItem w = group_item(g, it);
          const bool diag = w.row_a == w.row_b;
          for (int c = 0; c < w.nchunks; ++c, ++gc) {
            const int s = (int)(gc % NST);
            const int64_t rnd = gc / NST;
            if (rnd > 0 && !mbar_wait(smem_u32(&empty_bar[s]), (uint32_t)((rnd - 1) & 1), err, ERR_LOAD, wlim)) {
              ok = false;
              break;
            }
            if (g.starve_plus1 > 0 && blockIdx.x == 0 && gc + 1 == g.starve_plus1) continue;  // testing: never loaded
            const int x = (int)(((int64_t)w.chunk0 + (int64_t)c * w.cstride) * (2 * CK));  // FP32 column
            const uint32_t st = smem_u32(smem + s * STAGE), bar = smem_u32(&load_bar[s]);
            mbar_expect_tx(bar, diag ? BOXB : 2 * BOXB);  // out-of-range rows and columns arrive as zeros
            tma_load_2d(st, &xmap, x, w.row_a, bar);
            tma_load_2d(st + HALF, &xmap, x + CK, w.row_a, bar);
            if (!diag) {
              tma_load_2d(st + BOXB, &xmap, x, w.row_b, bar);
              tma_load_2d(st + BOXB + HALF, &xmap, x + CK, w.row_b, bar);
            }
            issued = gc + 1;
          }
        }
        for (int64_t c = max((int64_t)0, issued - NST); c < issued; ++c)
          mbar_drain(smem_u32(&load_bar[c % NST]), (uint32_t)((c / NST) & 1), wlim);
      }
    } else {
      const int piece = lane & 15, rpar = lane >> 4;
      for (int it = blockIdx.x; it < n_items && ok; it += gridDim.x) {
        const GItem w = group_item(g, it);
        const bool diag = w.row_a == w.row_b;
        const int nrows = box == 0 ? w.na : (diag ? 0 : w.nb);
        const int rbase = box == 0 ? w.row_a : w.row_b;
        // a tile whose rows are consecutive rows of the map loads by TMA
        const int tma_row = (g.tile_tma && nrows > 0) ? g.rows[rbase].tma_row : -1;
        // lane l holds the row pointers of rows l, l+32, l+64, l+96
        unsigned long long myrow[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const int r = lane + 32 * k;
          myrow[k] = (tma_row < 0 && r < nrows) ? reinterpret_cast<unsigned long long>(g.rows[rbase + r].J) : 0ull;
        }
        for (int c = 0; c < w.nchunks; ++c, ++gc) {
          const int s = (int)(gc % NST);
          const int64_t rnd = gc / NST;
          // every lane acquires the stage itself before writing into it
          if (rnd > 0) ok = mbar_wait(smem_u32(&empty_bar[s]), (uint32_t)((rnd - 1) & 1), err, ERR_LOAD, wlim);
          ok = __all_sync(0xffffffffu, ok);
          if (!ok) break;
          const int64_t col0 = ((int64_t)w.chunk0 + (int64_t)c * w.cstride) * CK;
          const uint32_t st = smem_u32(smem + s * STAGE) + (uint32_t)(box * BOXB);
          const uint32_t bar = smem_u32(&load_bar[s]);
          if (PHASE && box == 0 && lane >= 1 && lane <= 4) {
            // the chunk's directions for the converters' phases (lanes 1-4;
            // their cp.async arrival below covers these copies)
            const int64_t j = (col0 + (lane >= 3 ? 16 : 0)) / g.L;
            if (j < g.M)
              cp_async16(smem_u32(&sdir[s][lane - 1]), (lane & 1) ? (const void*)(g.dir_hi + j) : (const void*)(g.dir_lo + j));
          }
          if (tma_row >= 0) {
            // one arrival per lane as in the gather: lane 0's carries the bytes
            if (lane == 0) {
              mbar_expect_tx(bar, BOXB);
              tma_load_2d(st, &xmap, (int)(col0 * 2), tma_row, bar);
              tma_load_2d(st + HALF, &xmap, (int)(col0 * 2) + CK, tma_row, bar);
            } else {
              cp_async_arrive(bar);
            }
          } else {
            const int npieces = (int)min((int64_t)CK, g.ncols - col0) / 2;  // 16-byte pieces (2 complex)
            const int64_t coff = (col0 + 2 * piece) * (int64_t)sizeof(float2);
            const bool active = piece < npieces;
            // Half-warp h copies row 2m + h: 16 lanes x 16 B = the row's 256-byte
            // chunk.  The row pointer comes from its owner lane by shuffle.
#pragma unroll
            for (int k = 0; k < 4; ++k) {
              if (32 * k >= nrows) break;  // warp-uniform
#pragma unroll 4
              for (int m = 0; m < 16; ++m) {
                const int r = 32 * k + 2 * m + rpar;
                const unsigned long long base = __shfl_sync(0xffffffffu, myrow[k], (2 * m + rpar) & 31);
                if (active && r < nrows)
                  cp_async16(st + stage_off(r, piece), reinterpret_cast<const void*>(base + coff));
              }
            }
            cp_async_arrive(bar);
          }
          issued = gc + 1;
        }
      }
      // Never leave with a copy still landing in shared memory.
      cp_async_wait_all();
      for (int64_t c = max((int64_t)0, issued - NST); c < issued; ++c)
        mbar_drain(smem_u32(&load_bar[c % NST]), (uint32_t)((c / NST) & 1), wlim);
    }
  } else if (warp < CWARPS) {
    // ---------------- converters ----------------
    // thread (row, q): 8 complex values (quarter q of the chunk's 32 columns)
    // of one row of each tile; a warp owns all four quarters of 8 rows.  The
    // hi and lo operand rows of row r occupy exactly the bytes of row r's
    // FP32 input (first and second half-box), so a warp overwrites only
    // inputs it has read itself and needs no barrier with the other warps.
    const int row = warp * 8 + (lane >> 2), q = lane & 3;
    int64_t gc = 0;
    bool ok = true;
    for (int it = blockIdx.x; it < n_items && ok; it += gridDim.x) {
      const GItem w = group_item(g, it);
      const bool diag = w.row_a == w.row_b;
      const bool va = row < w.na, vb = !diag && row < w.nb;
      float3 cah = make_float3(0.f, 0.f, 0.f), cal = cah, cbh = cah, cbl = cah;
      float sa = 1.f, sb = 1.f;
      if (va) {
        const GRow R = g.rows[w.row_a + row];
        sa = row_scale(R, OP);
        if (PHASE) { cah = make_float3(R.c_hi[0], R.c_hi[1], R.c_hi[2]); cal = make_float3(R.c_lo[0], R.c_lo[1], R.c_lo[2]); }
      }
      if (vb) {
        const GRow R = g.rows[w.row_b + row];
        sb = row_scale(R, OP);
        if (PHASE) { cbh = make_float3(R.c_hi[0], R.c_hi[1], R.c_hi[2]); cbl = make_float3(R.c_lo[0], R.c_lo[1], R.c_lo[2]); }
      }
      for (int c = 0; c < w.nchunks; ++c, ++gc) {
        const int s = (int)(gc % NST);
        const int64_t rnd = gc / NST;
        ok = mbar_wait(smem_u32(&load_bar[s]), (uint32_t)(rnd & 1), err, ERR_CONVERT, wlim);
        ok = __all_sync(0xffffffffu, ok);
        if (!ok) break;
        uint8_t* st = smem + s * STAGE;
        const int64_t col0 = ((int64_t)w.chunk0 + (int64_t)c * w.cstride) * CK + CV * q;
        const int64_t nvalid = g.ncols - col0;  // < CV only in the last chunk of a ragged row
        // Direction and first radius of this thread's values: the chunk starts
        // at radius rc of direction jc, and with L a multiple of 16 the
        // thread's 8 values sit in direction jc or jc + 1 (32-bit arithmetic:
        // phase launches have rows of fewer than 2^31 columns).
        bool phase_ok = false;
        int r0 = 0, dslot = 0;
        if (PHASE) {
          const uint32_t cbase = (uint32_t)(((int64_t)w.chunk0 + (int64_t)c * w.cstride) * CK);
          const uint32_t jc = cbase / (uint32_t)g.L;
          r0 = (int)(cbase - jc * (uint32_t)g.L) + CV * q;
          uint32_t j = jc;
          if (r0 >= g.L) { r0 -= g.L; ++j; dslot = 2; }
          phase_ok = j < (uint32_t)g.M;  // padding columns past the last direction hold zeros
        }
        // One tile at a time (fewer live registers).  Every lane of the warp
        // has read a tile's inputs before any of its outputs overwrites them.
#pragma unroll
        for (int t = 0; t < 2; ++t) {
          const bool v = t == 0 ? va : vb;
          float x[2 * CV];
          if (v) {
#pragma unroll
            for (int m = 0; m < CV / 2; ++m) {
              const float4 u = *reinterpret_cast<const float4*>(st + t * BOXB + stage_off(row, (CV / 2) * q + m));
              x[4 * m] = u.x; x[4 * m + 1] = u.y; x[4 * m + 2] = u.z; x[4 * m + 3] = u.w;
            }
          }
          __syncwarp();
          if (v) {
            if (nvalid < CV) {
#pragma unroll
              for (int i = 0; i < CV; ++i)
                if (i >= nvalid) x[2 * i] = x[2 * i + 1] = 0.f;
            }
            if (PHASE && phase_ok)
              apply_phase<CV>(x, r0, t == 0 ? cah : cbh, t == 0 ? cal : cbl, kt, &sdir[PHASE ? s : 0][dslot]);
            store_split<OP, CV / 4>(st + t * 2 * OPB, row, q, x, t == 0 ? sa : sb);
          }
        }
        fence_proxy_async();
        __syncwarp();
        if (lane == 0) mbar_arrive(smem_u32(&full_bar[s]));
      }
    }
  } else if (warp == MWARP) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      constexpr uint32_t ID = op_idesc<OP>();
      int64_t gc = 0, gch = 0;
      bool ok = true;
      for (int it = blockIdx.x; it < n_items && ok; it += gridDim.x) {
        const GItem w = group_item(g, it);
        const bool diag = w.row_a == w.row_b;
        for (int c = 0; c < w.nchunks; ++c, ++gc) {
          const int b = (int)(gch & 1);
          const bool first = (c % CHAIN) == 0;
          if (first && gch >= 2) {
            if (!mbar_wait(smem_u32(&che_bar[b]), (uint32_t)(((gch >> 1) - 1) & 1), err, ERR_MMA, wlim)) { ok = false; break; }
          }
          const int s = (int)(gc % NST);
          const int64_t rnd = gc / NST;
          if (!mbar_wait(smem_u32(&full_bar[s]), (uint32_t)(rnd & 1), err, ERR_MMA, wlim)) { ok = false; break; }
          fence_after();
          const uint32_t st = smem_u32(smem + s * STAGE);
          const uint64_t aH = desc_sw128(st), aL = desc_sw128(st + OPB);
          const uint64_t bH = diag ? aH : desc_sw128(st + 2 * OPB);
          const uint64_t bL = diag ? aL : desc_sw128(st + 3 * OPB);
          const uint32_t d = tmem + (uint32_t)(b * GM);
#pragma unroll
          for (int k = 0; k < 4; ++k) {  // one MMA covers 32 bytes (16 values) of K
            const uint64_t adv = (uint64_t)(k * 32) >> 4;
            umma_f16(d, aH + adv, bH + adv, ID, (first && k == 0) ? 0u : 1u);
            umma_f16(d, aH + adv, bL + adv, ID, 1u);
            umma_f16(d, aL + adv, bH + adv, ID, 1u);
          }
          umma_commit(smem_u32(&empty_bar[s]));
          if ((c % CHAIN) == CHAIN - 1 || c == w.nchunks - 1) {
            umma_commit(smem_u32(&chf_bar[b]));
            ++gch;
          }
        }
      }
      // every MMA issued by this thread has completed before tensor memory is freed
      umma_commit(smem_u32(&fin_bar));
      mbar_drain(smem_u32(&fin_bar), 0u, wlim);
    }
    __syncwarp();
  } else {
    // ---------------- epilogue ----------------
    const int q4 = warp & 3;  // this warp may access tensor-memory lanes 32 q4 .. 32 q4 + 31
    const int row = q4 * 32 + lane;
    const uint32_t tl = tmem + ((uint32_t)(q4 * 32) << 16);
    int64_t gch = 0;
    bool ok = true;
    for (int it = blockIdx.x; it < n_items && ok; it += gridDim.x) {
      const GItem w = group_item(g, it);
      const int nch = (w.nchunks + CHAIN - 1) / CHAIN;
      const int ncb = (w.nb + 15) >> 4;
      float* out = g.partials + (int64_t)it * (GM * GM) + (int64_t)row * GM;
      for (int ch = 0; ch < nch; ++ch, ++gch) {
        const int b = (int)(gch & 1);
        // every lane takes the same decision before the warp-collective tensor-memory loads
        ok = __all_sync(0xffffffffu, mbar_wait(smem_u32(&chf_bar[b]), (uint32_t)((gch >> 1) & 1), err, ERR_EPILOGUE, wlim));
        if (!ok) break;
        fence_after();
        const bool first = ch == 0, last = ch == nch - 1;
#pragma unroll 1
        for (int cb = 0; cb < 8; ++cb) {
          if (cb >= ncb) break;  // warp-uniform
          float v[16];
          tmem_ld16(tl + (uint32_t)(b * GM + cb * 16), v);
          if (!first) {
            float r[16];
            tmem_ld16(tl + SUM_COL + (uint32_t)(cb * 16), r);
#pragma unroll
            for (int i = 0; i < 16; ++i) v[i] += r[i];
          }
          if (!last) {
            tmem_st16(tl + SUM_COL + (uint32_t)(cb * 16), v);
          } else if (row < w.na) {
#pragma unroll
            for (int i = 0; i < 16; i += 4)
              *reinterpret_cast<float4*>(out + cb * 16 + i) = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
          }
        }
        fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(smem_u32(&che_bar[b]));
      }
    }
  }

  fence_before();
  __syncthreads();
  if (warp == MWARP) {
    fence_after();
    tmem_dealloc(tmem, TMEM_COLS);
  }
}

// Fixed-order compensated sum of the partial tiles; one thread per (query, i, j) with
// i <= j, mirrored.  Grid-stride, so one fixed grid serves every batch.
__global__ void __launch_bounds__(RED_THREADS) group_reduce_kernel(const GroupDev g) {
  const int64_t n_elems = g.hdr->n_elems;
  const int nq = g.hdr->n_queries;
  const bool bad = *reinterpret_cast<volatile int*>(g.err) != 0;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n_elems;
       e += (int64_t)gridDim.x * blockDim.x) {
    int lo = 0, hi = nq - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (g.elem0[mid] <= e) lo = mid; else hi = mid - 1;
    }
    const GQuery q = g.queries[lo];
    const int64_t le = e - g.elem0[lo];
    const int i = (int)(le / q.n), j = (int)(le - (int64_t)i * q.n);
    if (i > j) continue;
    const int ta = i / GM, tb = j / GM;
    const int npairs = q.nt * (q.nt + 1) / 2;
    const int p = ta * q.nt - ta * (ta - 1) / 2 + (tb - ta);
    const int64_t off = (int64_t)(i % GM) * GM + (j % GM);
    double s = __longlong_as_double(0x7ff8000000000000LL);  // NaN unless the contraction succeeded
    if (!bad) {
      // compensated FP32 sum in split order; sixteen loads in flight ahead of their adds
      const float* src = g.partials + (q.item0 + p) * (GM * GM) + off;
      const int64_t stride = (int64_t)npairs * (GM * GM);
      kbsum acc{0.f, 0.f};
      int sp = 0;
      for (; sp + 16 <= q.nsplit; sp += 16) {
        float v[16];
#pragma unroll
        for (int u = 0; u < 16; ++u) v[u] = __ldcs(src + (sp + u) * stride);
#pragma unroll
        for (int u = 0; u < 16; ++u) acc.add(v[u]);
      }
      for (; sp < q.nsplit; ++sp) acc.add(__ldcs(src + sp * stride));
      s = acc.value() * g.scale / ((double)row_scale(g.rows[q.row0 + i], g.op) * (double)row_scale(g.rows[q.row0 + j], g.op));
    }
    g.out[q.out_off + (int64_t)i * q.n + j] = s;
    g.out[q.out_off + (int64_t)j * q.n + i] = s;
  }
}

// max |x| over each row of n contiguous rows of 2Q floats, as FP32 bit
// patterns (non-negative floats order like their bits) via atomicMax.
__global__ void row_amax_kernel(const float4* __restrict__ X, int64_t q4_per_row, int n, unsigned* __restrict__ amax) {
  const int row = blockIdx.y;
  float m = 0.f;
  const float4* r = X + (int64_t)row * q4_per_row;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < q4_per_row; i += (int64_t)gridDim.x * blockDim.x) {
    const float4 v = r[i];
    m = fmaxf(m, fmaxf(fmaxf(fabsf(v.x), fabsf(v.y)), fmaxf(fabsf(v.z), fabsf(v.w))));
  }
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0 && row < n) atomicMax(amax + row, __float_as_uint(m));
}

// Descriptors of one query over contiguous rows J + i * Q.
__global__ void group_single_setup_kernel(GRow* rows, GQuery* query, GHeader* hdr, int64_t* elem0, const float2* J,
                                          const float* amax, int64_t Q, int n, int nt, int nsplit) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) {
    GRow r;
    r.J = J + t * Q;
    r.amax = amax ? amax + t : nullptr;
    for (int c = 0; c < 3; ++c) { r.c_hi[c] = 0.f; r.c_lo[c] = 0.f; }
    r.tma_row = -1;
    r.reserved_ = 0;
    rows[t] = r;
  }
  if (t == 0) {
    GQuery q;
    q.row0 = 0; q.n = n; q.nt = nt; q.nsplit = nsplit; q.item0 = 0; q.out_off = 0;
    *query = q;
    GHeader h;
    h.n_items = nt * (nt + 1) / 2 * nsplit; h.n_queries = 1; h.n_elems = (int64_t)n * n;
    h.n_evals = 0; h.reserved_ = 0;
    *hdr = h;
    elem0[0] = 0;
  }
}

// Testing hooks (pi_test_set_contract_faults): the wait limit and the chunk
// that CTA 0's loader skips, read when a single-matrix contraction is set up.
std::atomic<long long> g_test_wait_cycles{0};
std::atomic<long long> g_test_starve_chunk{-1};
int sms() { return current_sm_count(); }

struct SinglePlan {
  int nt, npairs, nsplit, nchunks, items;
  size_t off_hdr, off_q, off_e, off_amax, off_rows, off_part, total;
};

// Items of one query: up to two per SM (rounded down, so that no CTA gets a
// third item and sets the kernel's length), otherwise as long as possible
// (one partial tile per item).
SinglePlan plan_single(int64_t Q, int n) {
  SinglePlan p;
  p.nt = (n + GM - 1) / GM;
  p.npairs = p.nt * (p.nt + 1) / 2;
  p.nchunks = (int)((Q + CK - 1) / CK);
  const int nsplit = std::max(1, (2 * sms()) / p.npairs);
  p.nsplit = std::min(nsplit, p.nchunks);
  p.items = p.npairs * p.nsplit;
  auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
  p.off_hdr = 256;                                   // [0, 256): error flag
  p.off_q = p.off_hdr + 256;
  p.off_e = p.off_q + 256;
  p.off_amax = p.off_e + 256;
  p.off_rows = al(p.off_amax + (size_t)n * sizeof(float));
  p.off_part = al(p.off_rows + (size_t)n * sizeof(GRow));
  p.total = p.off_part + (size_t)p.items * GM * GM * sizeof(float);
  return p;
}

template <int OP, bool PHASE, bool TMA>
const void* fn() { return reinterpret_cast<const void*>(group_split3_kernel<OP, PHASE, TMA>); }

const void* fn_of(int op, int phase, int tma) {
  if (op == GROUP_OP_F16) {
    if (phase) return tma ? fn<GROUP_OP_F16, true, true>() : fn<GROUP_OP_F16, true, false>();
    return tma ? fn<GROUP_OP_F16, false, true>() : fn<GROUP_OP_F16, false, false>();
  }
  if (phase) return tma ? fn<GROUP_OP_BF16, true, true>() : fn<GROUP_OP_BF16, true, false>();
  return tma ? fn<GROUP_OP_BF16, false, true>() : fn<GROUP_OP_BF16, false, false>();
}

}  // namespace

size_t group_smem_bytes() { return SMEM; }
int group_threads() { return NTHREADS; }
int group_reduce_threads() { return RED_THREADS; }
int group_grid() { return sms(); }
const void* group_contract_fn(int op, int phase, int all_tma) { return fn_of(op, phase, all_tma); }
const void* group_reduce_fn() { return reinterpret_cast<const void*>(group_reduce_kernel); }

int group_prepare_attributes() {
  for (int v = 0; v < 8; ++v) {
    const int rc = ensure_smem_limit(fn_of(v & 1, (v >> 1) & 1, v >> 2), (int)SMEM, "cudaFuncSetAttribute(group_split3_kernel)");
    if (rc != PI_OK) return rc;
  }
  return PI_OK;
}

int launch_group_contract(const GroupDev& g, const CUtensorMap* xmap, bool all_tma, int grid, cudaStream_t s) {
  int rc = group_prepare_attributes();
  if (rc) return rc;
  if (g.phase && (g.L <= 0 || g.L > GROUP_MAX_L || g.L % 16 != 0))
    return fail(PI_ERR_UNSUPPORTED, "translation phases need 16 | L <= 512 radial nodes per direction");
  if (g.phase && g.ncols >= (int64_t(1) << 31))
    return fail(PI_ERR_UNSUPPORTED, "translation phases support rows of fewer than 2^31 columns");
  if ((all_tma || g.tile_tma) && !xmap) return fail(PI_ERR_INVALID_ARGUMENT, "TMA loads need a tensor map");
  CUtensorMap none;
  std::memset(&none, 0, sizeof(none));
  const CUtensorMap& map = xmap ? *xmap : none;
  void* args[2] = {const_cast<GroupDev*>(&g), const_cast<CUtensorMap*>(&map)};
  PI_CUDA(cudaLaunchKernel(fn_of(g.op, g.phase, all_tma ? 1 : 0), dim3(grid), dim3(NTHREADS), args, SMEM, s));
  count_launch();
  return PI_OK;
}

int launch_group_reduce(const GroupDev& g, int grid, cudaStream_t s) {
  group_reduce_kernel<<<grid, RED_THREADS, 0, s>>>(g);
  PI_LAUNCHED("group_reduce_kernel");
  return PI_OK;
}

namespace {
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn encode_fn() {
  static std::once_flag once;
  static EncodeTiledFn f = nullptr;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      f = reinterpret_cast<EncodeTiledFn>(p);
  });
  return f;
}
}  // namespace

int encode_row_map(CUtensorMap* map, const void* base, int64_t row_floats, int64_t n_rows) {
  EncodeTiledFn enc = encode_fn();
  if (!enc) return fail(PI_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
  if ((reinterpret_cast<uintptr_t>(base) & 15) != 0 || (row_floats * 4) % 16 != 0)
    return fail(PI_ERR_INVALID_ARGUMENT, "tensor map: rows must start 16-byte aligned");
  const cuuint64_t gdim[2] = {(cuuint64_t)row_floats, (cuuint64_t)n_rows};
  const cuuint64_t gstride[1] = {(cuuint64_t)row_floats * sizeof(float)};
  const cuuint32_t box[2] = {(cuuint32_t)GROUP_CHUNK, (cuuint32_t)GROUP_TILE};  // 32 FP32 = 128 B per row
  const cuuint32_t estride[2] = {1, 1};
  CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void*>(base), gdim, gstride, box, estride,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? PI_OK : fail(PI_ERR_CUDA, "cuTensorMapEncodeTiled failed for the contraction rows");
}

size_t group_single_ws_bytes(int64_t Q, int n, int op) {
  (void)op;
  if (n <= 0 || Q <= 0) return 0;
  return plan_single(Q, n).total;
}

int launch_group_single(const float2* Jw, int64_t Q, int n, int op, double* V, void* ws, size_t ws_bytes,
                        double scale, cudaStream_t s, const float* row_amax) {
  if (n <= 0) return PI_OK;
  if (Q % 2 != 0) return fail(PI_ERR_UNSUPPORTED, "tensor-core contraction needs an even node count");
  if ((reinterpret_cast<uintptr_t>(Jw) & 15) != 0) return fail(PI_ERR_INVALID_ARGUMENT, "J must be 16-byte aligned");
  const SinglePlan p = plan_single(Q, n);
  if (!ws || ws_bytes < p.total) return fail(PI_ERR_WORKSPACE_TOO_SMALL, "tensor-core contraction workspace too small");
  unsigned char* base = static_cast<unsigned char*>(ws);
  GroupDev g{};
  g.hdr = reinterpret_cast<const GHeader*>(base + p.off_hdr);
  g.queries = reinterpret_cast<const GQuery*>(base + p.off_q);
  g.elem0 = reinterpret_cast<const int64_t*>(base + p.off_e);
  g.rows = reinterpret_cast<const GRow*>(base + p.off_rows);
  g.partials = reinterpret_cast<float*>(base + p.off_part);
  g.max_items = p.items;
  g.err = reinterpret_cast<int*>(base);
  g.out = V;
  g.ncols = Q;
  g.op = op;
  g.phase = 0;
  g.scale = scale;
  g.wait_cycles = g_test_wait_cycles.load();
  const long long starve = g_test_starve_chunk.load();
  g.starve_plus1 = starve >= 0 && starve < 0x7ffffffeLL ? (int32_t)(starve + 1) : 0;
  const float* amax = nullptr;
  if (op == GROUP_OP_F16 && row_amax) {
    amax = row_amax;  // the form-factor kernel's row maxima: no second pass over J
  } else if (op == GROUP_OP_F16) {
    float* ws_amax = reinterpret_cast<float*>(base + p.off_amax);
    amax = ws_amax;
    PI_CUDA(cudaMemsetAsync(ws_amax, 0, (size_t)n * sizeof(float), s));
    const int64_t q4 = Q / 2;  // whole float4s per row (2 complex each); rows start 16-byte aligned
    const int bx = (int)std::max<int64_t>(1, std::min<int64_t>((q4 + 255) / 256, 4 * sms() / n));
    if (q4 > 0) {
      row_amax_kernel<<<dim3((unsigned)bx, (unsigned)n), 256, 0, s>>>(reinterpret_cast<const float4*>(Jw), q4, n,
                                                                      reinterpret_cast<unsigned*>(ws_amax));
      PI_LAUNCHED("row_amax_kernel");
    }
  }
  PI_CUDA(cudaMemsetAsync(g.err, 0, sizeof(int), s));
  group_single_setup_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(
      const_cast<GRow*>(g.rows), const_cast<GQuery*>(g.queries), const_cast<GHeader*>(g.hdr),
      const_cast<int64_t*>(g.elem0), Jw, amax, Q, n, p.nt, p.nsplit);
  PI_LAUNCHED("group_single_setup_kernel");
  CUtensorMap xmap;
  int rc = encode_row_map(&xmap, Jw, 2 * Q, n);
  if (rc) return rc;
  rc = launch_group_contract(g, &xmap, true, std::min(p.items, sms()), s);
  if (rc) return rc;
  const int64_t red_blocks = std::min<int64_t>(((int64_t)n * n + RED_THREADS - 1) / RED_THREADS, 4 * sms());
  return launch_group_reduce(g, (int)std::max<int64_t>(1, red_blocks), s);
}

void group_test_set_faults(long long wait_cycles, long long starve_chunk) {
  g_test_wait_cycles.store(wait_cycles > 0 ? wait_cycles : 0);
  g_test_starve_chunk.store(starve_chunk);
}

}  // namespace pi
