/*
 * pointint_gb300 -- C ABI of the GB300-native Fourier intersection-volume path.
 *
 * Drop-in boundary for PoIntInt's Fourier path (reference paths are inside the
 * PoIntInt project).  Every entry point returns an int status (PI_OK == 0);
 * pi_last_error() gives the message of the last failure on the calling thread.
 * Nothing is ever silently zeroed: the reference printed CUDA errors and
 * returned zeros (cpp/src/compute_intersection_volume.cu:243-262, 473-486);
 * here the caller always sees a status.
 *
 * Memory: entry points named *_host take host buffers and do their own
 * uploads/downloads (the reference's calling convention).  All other entry
 * points take caller-owned DEVICE buffers, run on the given stream and never
 * synchronize the device implicitly.
 *
 * Element layouts are byte-identical to the reference's TriPacked / DiskPacked /
 * GaussianPacked (cpp/include/geometry/types.hpp:9-37), so a C++ caller can
 * pass geom.tris.data() / geom.disks.data() / geom.gaussians.data() as is.
 * K-grids are passed as the three arrays of the reference's KGrid
 * (cpp/include/quadrature/kgrid.hpp:9-13): dirs (Q x 3), kmag (Q), w (Q).
 * Volumes carry the 1/(8 pi^3) factor; k-grid weights do not.
 */
#ifndef POINTINT_GB300_H
#define POINTINT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* cudaStream_t without pulling in the CUDA headers. */
typedef struct CUstream_st* pi_stream;

/* ---- status codes -------------------------------------------------------- */
enum {
  PI_OK = 0,
  PI_ERR_INVALID_ARGUMENT = 1,
  PI_ERR_CUDA = 2,
  PI_ERR_UNSUPPORTED = 3,
  PI_ERR_OUT_OF_MEMORY = 4,
  PI_ERR_NOT_FOUND = 5,
  PI_ERR_WORKSPACE_TOO_SMALL = 6,
  PI_ERR_IO = 7,
  PI_ERR_TIMEOUT = 8
};

/* Geometry types: reference GeometryType (cpp/include/geometry/types.hpp:40-44). */
enum { PI_GEOM_TRIANGLE = 0, PI_GEOM_DISK = 1, PI_GEOM_GAUSSIAN = 2 };
/* DoF parameterizations: AffineDoF (cpp/include/dof/affine_dof.hpp:8-14) and
 * TriangleMeshDoF (cpp/include/dof/triangle_mesh_dof.hpp). */
enum { PI_DOF_AFFINE = 0, PI_DOF_TRIANGLE_MESH = 1 };
/* ComputationFlags (cpp/include/computation_flags.hpp:12-40). */
enum { PI_VOLUME_ONLY = 1, PI_GRADIENT = 2, PI_HESSIAN = 4, PI_ALL = 7 };
/* Contraction precision for V = Re(J^H diag(w) J). */
enum {
  PI_CONTRACT_FP32 = 0,      /* FP32 SIMT (the plain drop-in)                                    */
  PI_CONTRACT_BF16X3 = 1,    /* BF16 hi+lo split on tcgen05 tensor cores, FP32 accumulation      */
  PI_CONTRACT_TF32X3 = 2,    /* TF32 hi+lo split on tcgen05 tensor cores (~21 bits), FP32 accum. */
  PI_CONTRACT_FP16X3 = 3     /* FP16 hi+lo split of each row scaled by a power of two (~22 bits),
                                tcgen05 tensor cores, FP32 accumulation                           */
};

/* ---- packed element layouts (reference cpp/include/geometry/types.hpp:9-37) */
typedef struct { double a[3], e1[3], e2[3], S[3]; int32_t vid0, vid1, vid2, pad_; } pi_tri_packed;     /* 112 B */
typedef struct { double c[3], n[3]; double rho, area; } pi_disk_packed;                              /* 64 B  */
typedef struct { double c[3], n[3]; double sigma, w; } pi_gaussian_packed;                           /* 64 B  */

/* One object: packed elements + DoF parameterization + DoF vector.  AffineDoF
 * vectors are [tx,ty,tz, A00..A22 row-major] (cpp/src/dof/affine_dof.cpp:17-29);
 * TriangleMeshDoF vectors are 3V vertex coordinates indexed by vid0..2.
 * Whether `elems` / `dofs` are host or device pointers is stated by each
 * entry point. */
typedef struct {
  int32_t geom_type;
  int32_t dof_type;
  int64_t n_elems;
  const void* elems;
  int64_t n_dofs;
  const double* dofs;
} pi_object;

/* ---- errors / version ------------------------------------------------------ */
const char* pi_status_string(int status);
const char* pi_last_error(void);
int pi_version(void);
/* Number of device-side launches the library issued on this thread (for
 * instrumentation of benchmarks). */
int64_t pi_launch_count(void);

/* ---- host-side quadrature and geometry helpers (no GPU needed) ------------- */
/* gauss_legendre_interval (cpp/include/quadrature/gauss_legendre.hpp:16-62) */
int pi_gauss_legendre(int n, double a, double b, double* x, double* w);
/* load_lebedev_txt (cpp/include/quadrature/lebedev_io.hpp:24-59); returns the
 * row count in *n_rows and fills up to `cap` rows (dirs: cap x 3). */
int pi_load_lebedev(const char* path, double* dirs, double* w, int64_t cap, int64_t* n_rows);
/* build_kgrid (cpp/include/quadrature/kgrid.hpp:17-47); outputs Q = M*n_radial nodes. */
int pi_build_kgrid(const double* leb_dirs, const double* leb_w, int64_t M, int n_radial,
                   double* dirs, double* kmag, double* w);
/* pack_tris / pack_disks / pack_gaussians (cpp/src/geometry/packing.cpp:10-112) */
int pi_pack_tris(const double* V, int64_t n_verts, const int32_t* F, int64_t n_faces, pi_tri_packed* out);
int pi_pack_disks(const double* P, const double* N, const double* radii_or_areas, int64_t n, int is_radius,
                  pi_disk_packed* out);
int pi_pack_gaussians(const double* P, const double* N, const double* sigmas, const double* weights, int64_t n,
                      pi_gaussian_packed* out);
/* create_unit_cube_mesh / create_sphere_pointcloud / create_sphere_gaussians
 * (cpp/src/geometry/geometry_helpers.cpp:16-131) */
int pi_create_unit_cube_mesh(double* V /*8x3*/, int32_t* F /*12x3*/);
int pi_create_sphere_pointcloud(int n, double* P, double* N, double* radii);
int pi_create_sphere_gaussians(int n, double* P, double* N, double* sigmas, double* weights);
/* box_box / sphere_sphere_intersection_volume (cpp/src/analytical_intersection.cpp:15-60) */
double pi_box_box_intersection_volume(const double* c1, const double* h1, const double* c2, const double* h2);
double pi_sphere_sphere_intersection_volume(const double* c1, double r1, const double* c2, double r2);
/* DoFParameterization::compute_volume -- divergence theorem (cpp/src/compute_volume.cpp:17-73,
 * cpp/src/dof/affine_dof.cpp:324-384, cpp/src/dof/triangle_mesh_dof.cpp:145-179). Host object. */
int pi_self_volume(const pi_object* obj, double* volume);

/* ---- device-resident k-grid -------------------------------------------------- */
/* Uploads a KGrid once (the reference re-uploaded it for every object on every
 * call, cpp/src/dof/cuda/affine_dof_cuda.cu:895-914).  Host arrays.  A grid in
 * the reference's tensor order (q = ir*M + j) is detected and stored factored
 * as M directions x L radii; any other grid is stored node by node. */
typedef struct pi_kgrid_s* pi_kgrid;
int pi_kgrid_create(const double* dirs, const double* kmag, const double* w, int64_t Q, pi_kgrid* out);
int pi_kgrid_destroy(pi_kgrid kg);
int pi_kgrid_info(pi_kgrid kg, int64_t* Q, int64_t* n_dirs, int64_t* n_radial);
/* Host only, no counterpart in the reference.  The directions a k-grid's
 * kernels evaluate: the form factor of a real solid obeys A(-k) = -conj A(k),
 * so of two antipodal directions (d' = -d to 1e-10 |d|; every Lebedev rule is
 * made of such pairs) one is evaluated and the other written from it.  Writes
 * *n_eval pairs (j, j') as 2 int32 each into out (j' = -1 for a direction
 * without an antipode): on a tensor grid with pairs, in groups of 32 compact
 * clusters of directions; otherwise (j, -1) in index order.  The pairing
 * pi_kgrid_create stores.  PI_ERR_WORKSPACE_TOO_SMALL when cap < *n_eval. */
int pi_kgrid_direction_pairs(const double* dirs, const double* kmag, int64_t Q, int32_t* out, int64_t cap,
                             int64_t* n_eval);

/* ---- device-resident object batch ------------------------------------------- */
/* A set of objects transformed by their DoFs into the kernels' FP32 local-frame
 * layout.  `on_device` says whether elems/dofs in `objs` are device (1) or host
 * (0) pointers; the batch keeps its own copies.  Replaces the per-object,
 * per-call uploads of the reference's registry wrappers. */
typedef struct pi_batch_s* pi_batch;
int pi_batch_create(const pi_object* objs, int n_objects, int on_device, pi_stream stream, pi_batch* out);
/* Replace the DoF vector of object `index` (device pointer, same length) and
 * re-transform it, stream-ordered. */
int pi_batch_set_dofs(pi_batch b, int index, const double* d_dofs, pi_stream stream);
/* Replace every object's DoF vector at once: d_dofs holds the vectors
 * concatenated in object order (device doubles); re-transforms all objects. */
int pi_batch_set_all_dofs(pi_batch b, const double* d_dofs, pi_stream stream);
/* Re-run the DoF transform of every object from the batch's current DoF
 * vectors (stream-ordered). */
int pi_batch_prepare(pi_batch b, pi_stream stream);
int pi_batch_destroy(pi_batch b);
int pi_batch_count(pi_batch b, int* n_objects);

/* ---- form factors: J[n][q] = A_n(k_q) (complex64, n_objects x Q) ------------ */
/* Replaces kernels K1-K3, K7 and K12 (cpp/src/dof/cuda/affine_dof_cuda.cu:43-250,
 * 580-689; cpp/src/dof/cuda/triangle_mesh_dof_cuda.cu:34-143;
 * cpp/src/compute_intersection_volume_multi_object.cu:33-46).  If
 * scale_sqrt_w != 0 every row q is multiplied by sqrt(|w_q|) (the contraction's
 * operand form).  d_J: device, n_objects*Q*8 bytes. */
int pi_form_factors(pi_kgrid kg, pi_batch b, int scale_sqrt_w, void* d_J, pi_stream stream);
/* pi_form_factors that also writes each row's largest |Re|, |Im| of the values
 * written (d_row_amax: device, n_objects floats), which pi_contract_rowmax
 * takes as the FP16 operand scales of PI_CONTRACT_FP16X3 instead of reading J
 * a second time to find them.  No reference counterpart. */
int pi_form_factors_rowmax(pi_kgrid kg, pi_batch b, int scale_sqrt_w, void* d_J, float* d_row_amax,
                           pi_stream stream);

/* ---- contraction V = Re(J^H diag(w) J)/(8 pi^3) -------------------------------- */
/* Replaces K9 and K14 (cpp/src/compute_intersection_volume.cu:33-50;
 * cpp/src/compute_intersection_volume_multi_object.cu:74-116).  d_Jw is the
 * sqrt(|w|)-scaled J from pi_form_factors(scale_sqrt_w=1).  d_V: device
 * n x n doubles (full symmetric matrix).  d_ws: device workspace of at least
 * the size reported by pi_contract_workspace_size. */
int pi_contract_workspace_size(pi_kgrid kg, int n_objects, int precision, size_t* bytes);
int pi_contract(pi_kgrid kg, const void* d_Jw, int n_objects, int precision, double* d_V, void* d_ws,
                size_t ws_bytes, pi_stream stream);
/* pi_contract with the rows' maxima given (d_row_amax: device, n_objects
 * floats, each row's largest |Re|, |Im| or any upper bound of it, e.g. from
 * pi_form_factors_rowmax on the same J), used by PI_CONTRACT_FP16X3; NULL
 * finds them with a pass over J like pi_contract.  Other precisions ignore it. */
int pi_contract_rowmax(pi_kgrid kg, const void* d_Jw, const float* d_row_amax, int n_objects, int precision,
                       double* d_V, void* d_ws, size_t ws_bytes, pi_stream stream);
/* Device-side status of the last tensor-core contraction that used d_ws:
 * synchronises `stream`, then PI_OK, or PI_ERR_TIMEOUT when one of the
 * kernel's bounded waits (~2 s of SM clock each) ran out -- the kernel then
 * left every loop, drained its copies and tensor-core operations, freed its
 * tensor memory and wrote NaN to V, and the context stays usable.
 * PI_CONTRACT_FP32 has no waits and always reports PI_OK.  No reference
 * counterpart (the reference printed CUDA errors and returned zeros). */
int pi_contract_error(int precision, const void* d_ws, pi_stream stream);

/* Testing hook, not for production use: every later single-matrix FP16 / BF16
 * split contraction (pi_contract) waits at most wait_cycles SM clocks per
 * barrier (<= 0 restores the built-in ~2 s) and, when starve_chunk >= 0, the
 * loader of its first CTA never loads that chunk, so that a wait runs out
 * without any fault.  Process-wide; call (0, -1) to undo. */
int pi_test_set_contract_faults(int64_t wait_cycles, int64_t starve_chunk);

/* Replace the packed elements of object `index` (device pointer, same count and
 * layout) and re-transform it; used by optimisation loops that move elements. */
int pi_batch_set_elements(pi_batch b, int index, const void* d_elems, pi_stream stream);
/* Where object `index` sits in the batch's element pool of its type and in the
 * concatenated DoF-gradient vector. */
int pi_batch_layout(pi_batch b, int index, int64_t* pool_offset, int64_t* n_elems, int64_t* dof_offset);

/* ---- adjoint: gradients of L = sum_ij C_ij V_ij ------------------------------- */
/* The cotangent of object i is B_i = sum_j W_ij A_j (host W, n x n doubles):
 * pass W = C + C^T for a loss L = sum_ij C_ij V_ij, or W with a single column
 * of ones (W_ij = [j == j0]) for the reference's per-pair gradients
 * dV_{i j0}/dtheta_i (grad_matrix[i][j0], cpp/include/compute_intersection_volume_multi_object.hpp:21-26).
 * d_Jw is the sqrt(|w|)-scaled J of the batch (pi_form_factors with
 * scale_sqrt_w = 1).  Replaces K4-K6, K8, K10, K15
 * (cpp/src/dof/cuda/affine_dof_cuda.cu:254-576, 693-849; cpp/src/dof/cuda/triangle_mesh_dof_cuda.cu:147-310;
 *  cpp/src/compute_intersection_volume.cu:60-101; cpp/src/compute_intersection_volume_multi_object.cu:124-176)
 * without materialising dA/dtheta per k-node. */
int pi_adjoint_workspace_size(pi_kgrid kg, pi_batch b, size_t* bytes);
/* Per-element gradients (device float outputs in pool order, either may be NULL):
 *   triangles: 9 per element = dL/dv0, dL/dv1, dL/dv2 (world-frame vertex positions);
 *   disks / Gaussians: 12 per element = dL/dc (3), dL/dn' (3, n' = A n), dL/dM (6: xx xy xz yy yz zz, M = A A^T). */
int pi_element_gradients(pi_kgrid kg, pi_batch b, const void* d_Jw, const double* W, float* d_tri_grad,
                         float* d_surf_grad, void* d_ws, size_t ws_bytes, pi_stream stream);
/* DoF gradients of every object concatenated in object order (device doubles):
 * 12 per AffineDoF object ([t, A row-major], affine_dof.cpp:172-322 chain rule),
 * 3V per TriangleMeshDoF object (triangle_mesh_dof.cpp:76-143). */
int pi_dof_gradients(pi_kgrid kg, pi_batch b, const void* d_Jw, const double* W, double* d_grad, void* d_ws,
                     size_t ws_bytes, pi_stream stream);

/* Allocation-free FP32 contraction.  No counterpart in the reference.
 * For callers that cannot call cudaMalloc -- an application whose device
 * memory belongs to a host framework's pre-reserved pool, or a latency-
 * critical loop where an allocation would synchronise the device -- this entry
 * point allocates nothing: its split-K scratch is a fixed 8 MiB device array
 * inside the library, held on every GPU that loads the library until the
 * process exits.  The first call on a device looks up that array's address
 * with the device current; make that first call before any stream capture.
 * Inputs and output are caller-owned device buffers: d_Jw is the
 * sqrt(|w|)-scaled J (complex64, n x Q), d_sign the Q signs of the quadrature
 * weights or NULL when all are >= 0, d_V the n x n double output (1/(8 pi^3)
 * applied).  d_Jw needs no particular alignment (8-byte aligned complex64
 * rows are read element-wise).  Up to 1,920 objects fit the array on any GPU
 * (the K split is lowered to stay inside it); more return
 * PI_ERR_WORKSPACE_TOO_SMALL.  All calls share the array, so calls whose
 * kernels overlap on the GPU race.  The array's address is looked up once per
 * device: do not use this entry point across a cudaDeviceReset. */
int pi_contract_fp32_static(const void* d_Jw, int64_t Q, int n_objects, const float* d_sign, double* d_V,
                            pi_stream stream);

/* ---- one-shot host-buffer drop-ins ------------------------------------------ */
/* compute_intersection_volume_matrix_cuda (cpp/include/compute_intersection_volume_multi_object.hpp:51-59).
 * Host objects and k-grid; V_out: host n x n.  flags: PI_VOLUME_ONLY only in
 * this entry point (gradients go through the adjoint entry points).  Objects
 * whose elems point at the same array (same count and kind) share one upload
 * of it; the arrays are read during the call only. */
int pi_volume_matrix_host(const pi_object* objs, int n_objects, const double* dirs, const double* kmag,
                          const double* w, int64_t Q, int flags, int precision, double* V_out);
/* compute_intersection_volume_cuda (cpp/include/compute_intersection_volume.hpp:48-59), volume. */
int pi_pair_volume_host(const pi_object* o1, const pi_object* o2, const double* dirs, const double* kmag,
                        const double* w, int64_t Q, double* volume);
/* compute_intersection_volume_cuda with ComputationFlags::GRADIENT
 * (cpp/include/compute_intersection_volume.hpp:48-59): volume and the DoF
 * gradients grad_geom1 (o1->n_dofs) / grad_geom2 (o2->n_dofs), host buffers. */
int pi_pair_volume_grad_host(const pi_object* o1, const pi_object* o2, const double* dirs, const double* kmag,
                             const double* w, int64_t Q, double* volume, double* grad1, double* grad2);
/* compute_intersection_volume_matrix_cuda with GRADIENT
 * (cpp/include/compute_intersection_volume_multi_object.hpp:51-59): V (n x n)
 * and grad_matrix packed as blocks (i, j) = dV_ij/dtheta_i of n_dofs[i] doubles
 * at offset n * sum_{m<i} n_dofs[m] + j * n_dofs[i]. */
int pi_volume_matrix_grad_host(const pi_object* objs, int n_objects, const double* dirs, const double* kmag,
                               const double* w, int64_t Q, double* V_out, double* grad_out);
/* ---- Gauss-Newton Hessian -------------------------------------------------------- */
/* DoF Jacobian of the form factors: d_G[d][q] = sqrt(|w_q|) dA_n(k_q)/dtheta_{n,d},
 * rows in the order of the concatenated DoF vector (12 per AffineDoF object,
 * 3V per TriangleMeshDoF object; pi_batch_layout gives each object's first
 * row), Q complex64 per row, the object's position phase included.  This is
 * the reference's per-k dA/dtheta (compute_A_gradient, affine_dof.cpp:172-322,
 * triangle_mesh_dof.cpp:76-143; K4/K5/K8 cpp/src/dof/cuda/affine_dof_cuda.cu:254-576,
 * cpp/src/dof/cuda/triangle_mesh_dof_cuda.cu:147-310) in the contraction's
 * operand form: the Gauss-Newton Hessian blocks are Re(G_i diag(sign w) G_j^H)/(8 pi^3),
 * which pi_contract forms from the stacked rows. */
int pi_dof_jacobian(pi_kgrid kg, pi_batch b, void* d_G, pi_stream stream);
/* compute_intersection_volume_matrix_cuda with GRADIENT | HESSIAN
 * (cpp/include/compute_intersection_volume_multi_object.hpp:21-59;
 * hessian_ij, cpp/src/compute_intersection_volume_multi_object.cu:189-229):
 * V (n x n), grad_out (may be NULL; packed as in pi_volume_matrix_grad_host)
 * and hess_out = hessian_ij[i][j] for every (i, j): blocks of n_dofs[i] x n_dofs[j]
 * doubles (row-major) in (i, j) row-major order.  hessian_ii and hessian_jj
 * are zero in the reference's Gauss-Newton form and are not returned. */
int pi_volume_matrix_hessian_host(const pi_object* objs, int n_objects, const double* dirs, const double* kmag,
                                  const double* w, int64_t Q, double* V_out, double* grad_out, double* hess_out);
/* compute_intersection_volume_cuda with GRADIENT | HESSIAN
 * (cpp/include/compute_intersection_volume.hpp:24-59; K11,
 * cpp/src/compute_intersection_volume.cu:109-157): volume, grad_geom1/2 (may be
 * NULL), hessian_geom1 (d1 x d1), hessian_geom2 (d2 x d2), hessian_cross (d1 x d2). */
int pi_pair_volume_hessian_host(const pi_object* o1, const pi_object* o2, const double* dirs, const double* kmag,
                                const double* w, int64_t Q, double* volume, double* grad1, double* grad2,
                                double* H11, double* H22, double* H12);

/* CudaComputeAkFunc registry plugin (cpp/include/dof/cuda/dof_cuda_interface.hpp:24-30):
 * host object and k-grid, output d_A_out = Q complex doubles (double2) on the device. */
int pi_compute_Ak(const pi_object* obj, const double* dirs, const double* kmag, int64_t Q, double* d_A_out,
                  int block_size);
/* compute_Ak_cuda (cpp/include/compute_intersection_volume.hpp:120-126): A at one
 * k-vector, host in and out (out = re, im). */
int pi_compute_Ak_single(const pi_object* obj, const double* k, double* out);
/* The registry's gradient function (CudaComputeAkGradientFunc,
 * cpp/include/dof/cuda/dof_cuda_interface.hpp:32-40): host object and k-grid,
 * output d_grad_out = Q x D complex doubles (double2), row-major, q-major, on the
 * device, D = obj->n_dofs: dA(k_q)/dtheta_d with the object's position phase
 * (affine_dof.cpp:172-322, triangle_mesh_dof.cpp:76-143).  Synchronous like the
 * reference wrapper. */
int pi_compute_Ak_gradient(const pi_object* obj, const double* dirs, const double* kmag, int64_t Q,
                           double* d_grad_out, int block_size);
/* compute_Ak_gradient_cuda (cpp/include/compute_intersection_volume.hpp:129-135):
 * dA(k)/dtheta at one k-vector, host in and out (out = D pairs re, im; zeros
 * at |k| < 1e-10 like the reference). */
int pi_compute_Ak_gradient_single(const pi_object* obj, const double* k, double* out);

/* ---- serving: resident form factors, rigid-transform queries ----------------
 * No reference counterpart: the reference evaluates every object's form
 * factors from scratch on every call (compute_intersection_volume_multi_object.cu:234-713).
 *
 * A server owns a library of objects (elements + DoFs, uploaded once) and a
 * pool of resident form-factor rows in HBM.  A query is a scene: a list of
 * library objects, each under a rigid transform x' = R x + t applied on top of
 * its DoFs; the result is the scene's volume matrix (n x n, FP64, 1/(8 pi^3)
 * applied).  Translations never re-evaluate form factors: the phase
 * e^{i k . c} of each object's centre c = R o + t is applied inside the
 * contraction.  A rotation evaluates the object's form factors at R^T k into a
 * row owned by that query.  A worker thread admits pending queries, in arrival
 * order, into up to `inflight_batches` batches on the device at once, as long
 * as the resident pool (LRU, within hbm_budget_bytes) and the batch arenas have
 * room; each batch runs as one CUDA graph (descriptor upload, form factors of
 * the new rows, one persistent tensor-core contraction over every query of the
 * batch, the split-K reduction, result download).  Each query's result depends on
 * that query alone, not on the batch it ran in. */
typedef struct pi_server_s* pi_server;

typedef struct {
  int64_t hbm_budget_bytes;  /* resident rows + batch arenas; 0 = a quarter of the free device memory */
  int32_t max_batch_queries; /* 0 = 64 */
  int32_t max_batch_rows;    /* object rows (sum of n over the batch's queries); 0 = 4096 */
  int32_t max_batch_evals;   /* form-factor evaluations per batch; 0 = 256 */
  int32_t inflight_batches;  /* 1..4; 0 = 4 */
  int32_t precision;         /* PI_CONTRACT_FP16X3 (0 = default) or PI_CONTRACT_BF16X3 */
  int32_t use_graphs;        /* 1: each batch is one CUDA graph launch; 0: plain stream launches; -1 = 1 */
  int32_t autotune;          /* 1: time work-item sizes at creation; 0: built-in sizes; -1 = 1 */
  int32_t items_per_sm_x4;   /* > 0: work items per SM for every scene size, in quarters (overrides autotune) */
} pi_server_config;

typedef struct {
  int32_t n_objects;         /* rows of the scene (a library object may appear more than once) */
  int32_t reserved_;
  const int32_t* objects;    /* library indices */
  const double* rotations;   /* n x 9 row-major proper rotations, or NULL (no rotation) */
  const double* translations;/* n x 3, or NULL (no translation) */
} pi_query;

enum { PI_QUERY_PENDING = 0, PI_QUERY_RUNNING = 1, PI_QUERY_DONE = 2, PI_QUERY_FAILED = 3, PI_QUERY_CANCELLED = 4 };

typedef struct {
  int64_t submitted, completed, failed, cancelled;
  int64_t batches, evaluations, resident_hits, resident_misses, evictions;
  int64_t pool_rows, resident_rows, graph_launches;
  int32_t tuned_items_per_sm[4];  /* autotuned work items per SM for scenes of <= 16, <= 128, <= 512, > 512 objects, x 1/4 */
  int32_t tuned_k_splits[4];      /* the K splits per tile pair that this sets for scenes of 16, 128, 512, 1024 objects */
} pi_server_stats;

/* Zero config fields take the defaults above. */
int pi_server_create(pi_kgrid kg, const pi_object* library, int n_library, const pi_server_config* cfg,
                     pi_server* out);
/* Queue a scene.  V_out (host, n x n row-major) is written before the ticket
 * reads as done; it must stay valid until then. */
int pi_server_submit(pi_server s, const pi_query* q, double* V_out, uint64_t* ticket);
int pi_server_poll(pi_server s, uint64_t ticket, int32_t* state);
/* Block until the ticket is done (PI_OK), failed (its error), cancelled, or
 * timeout_s elapses (PI_ERR_TIMEOUT; timeout_s < 0 waits forever). */
int pi_server_wait(pi_server s, uint64_t ticket, double timeout_s);
/* Cancels a query that has not been admitted to a batch yet (PI_OK); a
 * running or finished query is left alone (PI_ERR_UNSUPPORTED). */
int pi_server_cancel(pi_server s, uint64_t ticket);
/* Host steady-clock nanoseconds: submitted, admitted to a batch, result written. */
int pi_server_times(pi_server s, uint64_t ticket, int64_t* submit_ns, int64_t* start_ns, int64_t* done_ns);
/* Forget a finished ticket. */
int pi_server_release(pi_server s, uint64_t ticket);
int pi_server_stats_get(pi_server s, pi_server_stats* st);
/* Waits for the queries already admitted, fails the pending ones, frees everything. */
int pi_server_destroy(pi_server s);

/* ---- alignment caller: similarity measures, damped Newton, warm start ---------
 * cpp/app/align (similarity_measure.hpp:10-48, optimizer.hpp:11-33,
 * warm_start.hpp:9-34), headless.  Geometry 1 is fixed at the identity,
 * geometry 2 moves under an AffineDoF (12 DoFs [t, A row-major]); the
 * objective is -log(similarity). */
enum { PI_SIM_OCHIAI = 0, PI_SIM_JACCARD = 1, PI_SIM_DICE = 2 };
enum { PI_SIM_FUNC_ONLY = 1, PI_SIM_GRADIENT = 2, PI_SIM_HESSIAN = 4, PI_SIM_FUNC_GRAD = 3, PI_SIM_ALL = 7 };

/* OptimizationState (optimizer.hpp:12-19) plus two counters. */
typedef struct {
  double dofs[12];
  double similarity;       /* similarity at the last gradient evaluation */
  double similarity_loss;  /* -log(similarity) there */
  int32_t iteration;
  int32_t converged;
  int32_t steps;           /* accepted Newton steps */
  int32_t evaluations;     /* similarity evaluations (gradient + line search) */
  char status[64];
} pi_optimization_state;

typedef struct pi_aligner_s* pi_aligner;

/* Holds the k-grid and both geometries on the device (host inputs; the DoF
 * fields of geom1/geom2 are ignored), and evaluates geometry 1's form factors
 * once. */
int pi_aligner_create(const pi_object* geom1, const pi_object* geom2, const double* dirs, const double* kmag,
                      const double* w, int64_t Q, pi_aligner* out);
int pi_aligner_destroy(pi_aligner a);
/* Fourier self-volume of geometry 1 on the aligner's grid: the V1 that the
 * reference app passes in (compute_intersection_volume_cuda(geom1, geom1),
 * cpp/app/align/main.cpp:224-230). */
int pi_aligner_fixed_volume(pi_aligner a, double* V1);
/* compute_similarity (similarity_measure.hpp:37-48): value = -log(max(s, 1e-10)),
 * similarity = s; grad (12) and hess (12 x 12 row-major) of the value when the
 * flags ask for them (else may be NULL).  The Hessian is the reference's
 * Gauss-Newton form (zero Hessian of the intersection volume). */
int pi_similarity(pi_aligner a, const double* dofs2, int measure, double V1, int flags, double* value,
                  double* similarity, double* grad, double* hess);
/* optimize_alignment (optimizer.hpp:22-33): Newton steps on the PSD projection
 * of the Hessian plus damping I, Armijo backtracking (c = 0.1, factor 0.5, at
 * most 20 halvings, alpha_min = 1e-10); stops when |grad| < tolerance.  Like the
 * reference, a run that stops without converging reports "Reached max iterations". */
int pi_optimize_alignment(pi_aligner a, const double* initial_dofs, int measure, double V1, double tolerance,
                          int max_iterations, double damping, pi_optimization_state* state);
/* compute_moments (warm_start.hpp:17-24) under the AffineDoF dofs (host
 * geometry): volume, centroid (3), covariance (3 x 3 row-major).  No GPU. */
int pi_compute_moments(const pi_object* geom, const double* dofs, double* volume, double* centroid,
                       double* covariance);
/* compute_warm_start (warm_start.hpp:26-34): the 12 AffineDoF parameters of
 * the similarity transform matching geometry 2's moments to geometry 1's.
 * Principal axes are taken with ascending eigenvalues and each axis's
 * largest-magnitude component positive (the reference leaves these signs to
 * its eigen-solver).  No GPU. */
int pi_compute_warm_start(const pi_object* geom1, const pi_object* geom2, double* dofs_out);

#ifdef __cplusplus
}
#endif
#endif /* POINTINT_GB300_H */
