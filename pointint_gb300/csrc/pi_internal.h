// Internal structures shared by the translation units of libpointint_gb300.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <string>
#include <vector>
#include "pointint_gb300.h"

namespace pi {

// ---- error handling ---------------------------------------------------------
void set_error(const std::string& msg);
int fail(int status, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);
void count_launch(int n = 1);

// ---- per-device launch set-up (a process may drive several GPUs) ------------
// SM count of the current device (148 when the query fails).
int current_sm_count();
// Raises fn's dynamic shared-memory limit to `bytes` on the current device,
// once per (function, device): the attribute belongs to the device's context.
// Returns PI_OK or the first attempt's error status.
int ensure_smem_limit(const void* fn, int bytes, const char* what);

#define PI_CUDA(call)                                        \
  do {                                                       \
    cudaError_t e_ = (call);                                 \
    if (e_ != cudaSuccess) return ::pi::cuda_fail(e_, #call); \
  } while (0)

#define PI_LAUNCHED(what)                                           \
  do {                                                              \
    cudaError_t e_ = cudaGetLastError();                            \
    if (e_ != cudaSuccess) return ::pi::cuda_fail(e_, what);        \
    ::pi::count_launch();                                           \
  } while (0)

// ---- device k-grid ------------------------------------------------------------
// Factored layout: node q = r * M + j has k_q = kmag[r] * dir[j].  Directions
// are stored as FP32 hi/lo pairs so that phases k.x can be formed to ~2^-44
// relative accuracy; radii likewise.  A grid without tensor structure is
// stored with M = Q, L = 1, dir[j] = k_j and kmag = 1.
struct KGridDev {
  int64_t Q;
  int M, L;
  const float4* dir_hi;   // M: (hx, hy, hz, 1/|dir|)
  const float4* dir_lo;   // M: (lx, ly, lz, |dir|)
  const float2* kmag;     // L: (hi, lo)
  const float* sqrtw;     // Q: sqrt(|w_q|)
  const float* sign;      // Q: sign(w_q), or nullptr when every weight is >= 0
  const float2* kturn;    // L: kmag / 2 pi (hi, lo)
  const float2* kt256;    // L: kmag 256 / 2 pi (hi, lo): phases in units of 1/256 turn
  const float2* cis_tab;  // 256: e^{2 pi i j / 256} (cos, sin), rounded once from FP64
  // Evaluated directions: Me entries (j, j'), j' the direction antipodal to j
  // (d_j' = -d_j) or -1.  The form factor of a real solid satisfies
  // A(-k) = -conj A(k), so the kernels that produce per-node outputs evaluate
  // direction j only and write j' from it.  On a centrally symmetric
  // direction set (every Lebedev rule) Me = M / 2, the entries grouped 32 at
  // a time into compact clusters of directions; otherwise (j, -1) in order.
  const int2* dpair;
  int Me;
};

struct pi_kgrid_impl {
  KGridDev dev;
  void* d_mem = nullptr;        // single allocation behind the pointers above
  std::vector<double> w;        // host copy of weights
  int64_t Q = 0;
  int M = 0, L = 0;
  int Me = 0;                   // evaluated directions (dev.dpair)
  bool tensor = false;
  bool all_positive = true;
};

// ---- device object batch -----------------------------------------------------
struct ObjDev {
  double origin[3];       // local-frame origin (transformed element centroid)
  float A[9];             // A, row-major (identity without AffineDoF): k' = A^T k
  int32_t type;           // PI_GEOM_*
  int32_t n_elems;
  int64_t elem_off;       // offset (in elements) into the pool of its type
};

// Pools in the kernels' layout, object-local frame, FP32:
//   triangles: 3 x float4 per element  (m.xyz, S.x) (e1.xyz, S.y) (e2.xyz, S.z), m the centroid
//   disks/Gaussians: 2 x float4        (c.xyz, rho|sigma) (n'.xyz, area|w)
// plus one float4 per element in tri_lo / surf_lo: the FP32 remainder of the
// centroid (centre) m - (float)m, so that the phase k.m keeps ~48 bits at
// k |m| of thousands of radians; and for disks/Gaussians one float4 in
// surf_nref: (n / |n|, 1 - |n|^2) of the reference-frame normal n, for
// |k'_perp|^2 = |k'|^2 - (k'.n)^2 = |k'|^2 (1 - |n|^2) + |n|^2 |k' x n/|n||^2
// without the cancellation of the difference form near the normal.
struct BatchDev {
  int n_obj;
  const ObjDev* objs;
  const int32_t* order;      // CTA y-index -> object (largest first)
  const float4* tri_pool;
  const float4* surf_pool;
  const float4* tri_lo;
  const float4* surf_lo;
  const float4* surf_nref;
};

// One form-factor evaluation of the serving path: library object `obj`,
// optionally rotated (its form factors at k are the unrotated object's at
// R^T k), written in the object-local frame (no origin phase), sqrt|w|-scaled
// and direction-major (column j * L + r) to dst; the largest |Re|, |Im| goes
// to *amax (FP32 bits, atomicMax) for the FP16 operand scale.
struct EvalDev {          // 104 bytes
  int32_t obj;
  int32_t rotate;
  float2* dst;
  float* amax;            // zeroed before the launch; atomicMax target
  float* amax_keep;       // the row's persistent maximum, copied from *amax after the evaluation
  double R[9];            // row-major
};

struct HostObjInfo {
  int32_t geom_type, dof_type;
  int64_t n_elems, n_dofs;
  int64_t src_off;           // byte offset of its packed source in the source arena
  int64_t dof_off;           // offset (doubles) into the dof arena
  int64_t pool_off;          // element offset in its pool
};

struct pi_batch_impl {
  int n_obj = 0;
  std::vector<HostObjInfo> info;
  std::vector<int32_t> order;
  int64_t n_tri = 0, n_surf = 0;
  // device allocations: one block (d_block) carved into the buffers below
  void* d_block = nullptr;
  void* d_src = nullptr;     // packed reference-layout elements of all objects
  double* d_dofs = nullptr;  // all DoF vectors
  float4* d_tri_pool = nullptr;
  float4* d_surf_pool = nullptr;
  float4* d_tri_lo = nullptr;
  float4* d_surf_lo = nullptr;
  float4* d_surf_nref = nullptr;
  ObjDev* d_objs = nullptr;
  int32_t* d_order = nullptr;
  // TriangleMeshDoF vertex adjacency (CSR over every mesh object's vertices):
  // row[v]..row[v+1] index ent[] = pool triangle * 3 + slot; vmap[v] = offset of
  // the vertex's 3 gradient entries in the concatenated DoF-gradient vector.
  int64_t n_mesh_verts = 0;
  int64_t* d_vrow = nullptr;
  int64_t* d_vent = nullptr;
  int64_t* d_vmap = nullptr;
  BatchDev dev() const {
    BatchDev b;
    b.n_obj = n_obj; b.objs = d_objs; b.order = d_order; b.tri_pool = d_tri_pool; b.surf_pool = d_surf_pool;
    b.tri_lo = d_tri_lo; b.surf_lo = d_surf_lo; b.surf_nref = d_surf_nref;
    return b;
  }
};

// ---- launchers (formfactor.cu / contract.cu) ------------------------------------
int launch_prepare(pi_batch_impl* b, int only_index, cudaStream_t s);
// row_amax (optional, n_objects floats): each row's largest |Re|, |Im| of the
// written values, for the FP16 operand scales of the split contraction.
int launch_form_factors(const pi_kgrid_impl* kg, const pi_batch_impl* b, int scale_sqrt_w, float2* J,
                        cudaStream_t s, float* row_amax = nullptr);
size_t contract_fp32_ws_bytes(int64_t Q, int n);
int launch_contract_fp32(const pi_kgrid_impl* kg, const float2* Jw, int n, double* V, void* ws, size_t ws_bytes,
                         cudaStream_t s);
size_t contract_tc_ws_bytes(int64_t Q, int n, int kind);  // kind 0 = BF16 split, 1 = TF32 split
int launch_contract_tc(const pi_kgrid_impl* kg, const float2* Jw, int n, int kind, double* V, void* ws,
                       size_t ws_bytes, cudaStream_t s);
int64_t dof_gradient_size(const pi_batch_impl* b);
size_t adjoint_ws_bytes(const pi_kgrid_impl* kg, const pi_batch_impl* b);
int launch_adjoint_elements(const pi_kgrid_impl* kg, const pi_batch_impl* b, const float2* Jw, const double* W_host,
                            float** tri_g, float** surf_g, void* ws, size_t ws_bytes, cudaStream_t s);
int launch_dof_gradients(const pi_kgrid_impl* kg, pi_batch_impl* b, const float2* Jw, const double* W_host,
                         double* grad, void* ws, size_t ws_bytes, cudaStream_t s);
int launch_to_double2(const float2* J, int64_t n, double* out, cudaStream_t s);
// G[d][q] = sqrt|w_q| dA(k_q)/dtheta_d for the concatenated DoF vector
// (dof_gradient_size(b) rows of Q complex64), origin phase included.
int launch_jacobian(const pi_kgrid_impl* kg, const pi_batch_impl* b, float2* G, cudaStream_t s);
// Serving evaluations: grid (ff_serve_grid_x(kg), n_evals), ff_serve_threads().
int ff_serve_grid_x(const pi_kgrid_impl* kg);
int ff_serve_threads();
const void* ff_serve_fn(const pi_kgrid_impl* kg);
int launch_form_factors_serve(const pi_kgrid_impl* kg, const pi_batch_impl* lib, const EvalDev* evals, int n_evals,
                              cudaStream_t s);
// After the serving evaluations: *amax_keep = *amax for the first *n_evals evals
// (one CTA of amax_commit_threads()).
const void* amax_commit_fn();
int amax_commit_threads();
int launch_amax_commit(const EvalDev* evals, const int32_t* n_evals, cudaStream_t s);

}  // namespace pi

struct pi_kgrid_s : pi::pi_kgrid_impl {};
struct pi_batch_s : pi::pi_batch_impl {};
