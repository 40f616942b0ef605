// Grouped volume contraction: many independent volume matrices (one per
// query) in one persistent launch.
//
// Every query is a list of operand rows.  A row is one object's sqrt|w|-scaled
// form factors J (ncols complex values), optionally the maximum |x| over the
// row's real and imaginary parts (which sets the power-of-two scale of the
// FP16 split), and a translation c whose phase e^{i k.c} is applied as the row
// is staged (direction-major rows only).  A query with n rows owns the
// upper-triangle pairs of its 128-row tiles; each pair is cut along k into
// nsplit work items, item s taking the chunks (32 complex columns each)
// s, s + nsplit, s + 2 nsplit, ...  Items are ordered split-major, so CTAs
// running at the same time read the same chunks of a tile (one DRAM read, the
// other pairs hit L2) and neighbouring chunks of each row (long DRAM runs).
// Each work item writes a 128 x 128 FP32 partial tile, and the reduction sums
// the partials of every pair in a fixed order (compensated FP32): a query's
// result does not depend on which other queries share the launch.
//
// All counts live in device memory (GHeader), so a launch sequence captured
// once in a CUDA graph serves every batch.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <cstdint>

namespace pi {

constexpr int GROUP_TILE = 128;        // rows per tile
constexpr int GROUP_CHUNK = 32;        // complex columns per k chunk
constexpr int GROUP_MAX_L = 512;       // radial nodes per direction supported by the phase path

enum { GROUP_OP_BF16 = 0, GROUP_OP_F16 = 1 };

struct GRow {                          // 48 bytes
  const float2* J;                     // ncols complex values, 16-byte aligned
  const float* amax;                   // max |Re|, |Im| over the row (FP16 operands), or null
  float c_hi[3], c_lo[3];              // translation c = c_hi + c_lo
  int32_t tma_row;                     // first row of a tile whose rows are consecutive rows tma_row,
                                       // tma_row + 1, ... of the loader's tensor map; -1 otherwise
  int32_t reserved_;
};

struct GItem {                         // one work item, derived on the device from the query table
  int32_t row_a, row_b;                // first row of each tile (absolute row index)
  int32_t na, nb;                      // valid rows in each tile (1..128)
  int32_t chunk0, nchunks;             // k chunks chunk0 + c * cstride, c < nchunks
  int32_t cstride;                     // = the query's nsplit: the splits of a pair interleave, so the
                                       // CTAs running at one time read neighbouring chunks of each row
  int32_t query;
};

struct GQuery {                        // 32 bytes
  int32_t row0, n;                     // rows [row0, row0 + n)
  int32_t nt, nsplit;                  // tiles, k splits per tile pair
  int64_t item0;                       // first work item; item0 + split * npairs + pair
  int64_t out_off;                     // V (n x n, FP64) at out + out_off
};

struct GHeader {                       // 24 bytes
  int32_t n_items, n_queries;
  int64_t n_elems;                     // sum of n^2 over queries
  int32_t n_evals, reserved_;          // form-factor evaluations of the batch (serving)
};

struct GroupDev {                      // kernel argument; pointers fixed for the life of a graph
  const GHeader* hdr;
  const GRow* rows;
  const GQuery* queries;
  const int64_t* elem0;                // per query: prefix sum of n^2
  int64_t ncols;                       // complex columns per row
  int32_t op;                          // GROUP_OP_*
  int32_t phase;                       // 1: rows are direction-major (col = j * L + r) and get e^{i k.c}
  int32_t tile_tma;                    // gather loader: tiles with rows[first].tma_row >= 0 load by TMA
  int32_t reserved_;
  int32_t L, M;                        // radial nodes per direction, directions
  const float4* dir_hi;                // directions (double-float), M entries
  const float4* dir_lo;
  const float2* kturn;                 // kmag / 2 pi (double-float), L entries
  float* partials;                     // n_items x 128 x 128
  int64_t max_items;                   // capacity of `partials`; a launch with more items records an error
  int* err;                            // 0 = ok
  double* out;                         // output arena
  double scale;                        // 1 / (8 pi^3)
  int64_t wait_cycles;                 // limit of every bounded wait in SM clocks; <= 0: the built-in ~2 s
  int32_t starve_plus1;                // testing: > 0 makes CTA 0's loader skip its chunk starve_plus1 - 1
  int32_t reserved2_;
};

// Power-of-two operand scale of a row with maximum |x| = amax: the scaled
// maximum lies in [2^14, 2^15), inside FP16's range with its full precision.
__host__ __device__ inline float group_row_scale(float amax) {
  if (!(amax > 0.f) || !(amax < 3.0e38f)) return 1.f;
  int e;
  (void)frexpf(amax, &e);  // amax = m 2^e, m in [0.5, 1)
  return ldexpf(1.f, 15 - e);
}

size_t group_smem_bytes();
int group_threads();
int group_grid();                      // persistent grid on the current device
const void* group_contract_fn(int op, int phase, int all_tma);
const void* group_reduce_fn();
int group_reduce_threads();
int group_prepare_attributes();

#ifdef __CUDACC__
// Work item `it` (split-major within its query: it - item0 = split * npairs + pair).
__device__ __forceinline__ GItem group_item(const GroupDev& g, int it) {
  int lo = 0, hi = g.hdr->n_queries - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (g.queries[mid].item0 <= it) lo = mid; else hi = mid - 1;
  }
  const GQuery q = g.queries[lo];
  const int npairs = q.nt * (q.nt + 1) / 2;
  const int local = (int)(it - q.item0);
  const int sp = local / npairs;
  int a = 0, rem = local - sp * npairs;
  while (rem >= q.nt - a) { rem -= q.nt - a; ++a; }
  const int b = a + rem;
  const int nch = (int)((g.ncols + GROUP_CHUNK - 1) / GROUP_CHUNK);
  GItem w;
  w.row_a = q.row0 + a * GROUP_TILE;
  w.row_b = q.row0 + b * GROUP_TILE;
  w.na = min(GROUP_TILE, q.n - a * GROUP_TILE);
  w.nb = min(GROUP_TILE, q.n - b * GROUP_TILE);
  w.chunk0 = sp;
  w.cstride = q.nsplit;
  w.nchunks = (nch - sp + q.nsplit - 1) / q.nsplit;
  w.query = lo;
  return w;
}
#endif

// 2D tensor map over n_rows contiguous rows of row_floats FP32 values, in the
// contraction's 128-row x 32-value boxes, 128-byte swizzled.
int encode_row_map(CUtensorMap* map, const void* base, int64_t row_floats, int64_t n_rows);

// Direct launches (not captured).  all_tma: every tile loads by TMA and row
// indices are row coordinates of xmap (one query over contiguous rows).
// Otherwise rows are gathered through g.rows[].J (cp.async), except tiles
// marked with tma_row when g.tile_tma and xmap are set.
int launch_group_contract(const GroupDev& g, const CUtensorMap* xmap, bool all_tma, int grid, cudaStream_t s);
int launch_group_reduce(const GroupDev& g, int grid, cudaStream_t s);

// One query over n contiguous rows Jw + i * Q (the pi_contract layout): the
// descriptors (and, for FP16 operands, the row maxima) are formed on the
// device inside the workspace.
size_t group_single_ws_bytes(int64_t Q, int n, int op);
// Testing: every later single-matrix contraction waits at most wait_cycles SM
// clocks per barrier (<= 0: the built-in ~2 s), and CTA 0's loader skips its
// chunk starve_chunk (< 0: none), so that a wait runs out.
void group_test_set_faults(long long wait_cycles, long long starve_chunk);
// row_amax (optional, FP16 operands only): each row's largest |Re|, |Im| (or
// any upper bound of it), as written by the form-factor kernel; without it
// the maxima are found by a pass over J.
int launch_group_single(const float2* Jw, int64_t Q, int n, int op, double* V, void* ws, size_t ws_bytes,
                        double scale, cudaStream_t s, const float* row_amax = nullptr);

}  // namespace pi
