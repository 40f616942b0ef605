// Alignment caller of the volume path: similarity measures of a fixed
// geometry and an affinely moved one, their gradients and Gauss-Newton
// Hessians, the damped Newton optimiser and the moment-matching warm start.
//
// Reference: cpp/app/align/similarity_measure.cpp:9-157 (measures and the
// -log transform), optimizer.cpp:8-133 (PSD-projected, damped Newton with
// Armijo backtracking), warm_start.cpp:8-243 (moments, similarity warm start).
//
// The reference evaluates every similarity through a fresh
// compute_intersection_volume_matrix_cuda call (k-grid, elements and DoFs
// uploaded, FP64 per-pair kernels).  Here an aligner holds the k-grid, both
// objects and one operand buffer resident on the device:
//   row 0        J_1  (geometry 1 at the identity; evaluated once),
//   row 1        J_2  (geometry 2 at the current DoFs),
//   rows 2..13   G_2  (d J_2 / d theta_2, the forward-mode DoF Jacobian),
// all sqrt|w|-scaled, and one FP32 contraction of the first 2 (function only)
// or 14 rows gives V_12, V_22, dV_21/dtheta_2 (row 2 + a, column 0),
// dV_22/dtheta_2 / 2 (column 1) and the Gauss-Newton block
// hessian_ij[1][1] (rows and columns 2..13).  In the reference's
// Gauss-Newton form hessian_ii and hessian_jj are zero, so the Hessian of the
// intersection term is zero and H_V2 = 2 hessian_ij[1][1].
#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <vector>
#include "pi_internal.h"

using pi::fail;

namespace {

constexpr int ND = 12;            // AffineDoF parameters
constexpr int ROWS = 2 + ND;      // J_1, J_2, G_2

struct DevMem {
  void* p = nullptr;
  ~DevMem() { if (p) cudaFree(p); }
};

// Cyclic Jacobi eigen-decomposition of a symmetric n x n matrix (row-major):
// eigenvalues in `lam`, eigenvectors in the columns of `V`.
void jacobi_eigen(std::vector<double> A, int n, std::vector<double>& lam, std::vector<double>& V) {
  V.assign((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) V[(size_t)i * n + i] = 1.0;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0, diag = 0.0;
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) (i == j ? diag : off) += A[(size_t)i * n + j] * A[(size_t)i * n + j];
    if (off <= 1e-30 * std::max(diag, 1e-300)) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double apq = A[(size_t)p * n + q];
        if (apq == 0.0) continue;
        const double app = A[(size_t)p * n + p], aqq = A[(size_t)q * n + q];
        const double theta = (aqq - app) / (2.0 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; ++k) {  // A <- A J (columns p, q)
          const double akp = A[(size_t)k * n + p], akq = A[(size_t)k * n + q];
          A[(size_t)k * n + p] = c * akp - s * akq;
          A[(size_t)k * n + q] = s * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {  // A <- J^T A (rows p, q)
          const double apk = A[(size_t)p * n + k], aqk = A[(size_t)q * n + k];
          A[(size_t)p * n + k] = c * apk - s * aqk;
          A[(size_t)q * n + k] = s * apk + c * aqk;
        }
        for (int k = 0; k < n; ++k) {
          const double vkp = V[(size_t)k * n + p], vkq = V[(size_t)k * n + q];
          V[(size_t)k * n + p] = c * vkp - s * vkq;
          V[(size_t)k * n + q] = s * vkp + c * vkq;
        }
      }
  }
  lam.resize(n);
  for (int i = 0; i < n; ++i) lam[i] = A[(size_t)i * n + i];
  // ascending eigenvalues; each eigenvector's largest-magnitude component positive
  std::vector<int> idx(n);
  for (int i = 0; i < n; ++i) idx[i] = i;
  std::sort(idx.begin(), idx.end(), [&](int a, int b) { return lam[a] < lam[b]; });
  std::vector<double> l2(n), V2((size_t)n * n);
  for (int c = 0; c < n; ++c) {
    const int o = idx[c];
    l2[c] = lam[o];
    int imax = 0;
    for (int r = 1; r < n; ++r)
      if (std::fabs(V[(size_t)r * n + o]) > std::fabs(V[(size_t)imax * n + o])) imax = r;
    const double sg = V[(size_t)imax * n + o] < 0 ? -1.0 : 1.0;
    for (int r = 0; r < n; ++r) V2[(size_t)r * n + c] = sg * V[(size_t)r * n + o];
  }
  lam.swap(l2);
  V.swap(V2);
}

// LDL^T solve of a symmetric positive definite system; false when a pivot is
// not positive and finite.
bool ldlt_solve(std::vector<double> A, int n, const double* b, double* x) {
  std::vector<double> d(n);
  for (int j = 0; j < n; ++j) {
    double dj = A[(size_t)j * n + j];
    for (int k = 0; k < j; ++k) dj -= A[(size_t)j * n + k] * A[(size_t)j * n + k] * d[k];
    if (!(dj > 0.0) || !std::isfinite(dj)) return false;
    d[j] = dj;
    for (int i = j + 1; i < n; ++i) {
      double lij = A[(size_t)i * n + j];
      for (int k = 0; k < j; ++k) lij -= A[(size_t)i * n + k] * A[(size_t)j * n + k] * d[k];
      A[(size_t)i * n + j] = lij / dj;
    }
  }
  std::vector<double> y(b, b + n);
  for (int i = 0; i < n; ++i)
    for (int k = 0; k < i; ++k) y[i] -= A[(size_t)i * n + k] * y[k];
  for (int i = 0; i < n; ++i) y[i] /= d[i];
  for (int i = n - 1; i >= 0; --i) {
    for (int k = i + 1; k < n; ++k) y[i] -= A[(size_t)k * n + i] * y[k];
    x[i] = y[i];
  }
  return true;
}

double det3(const double* A) {
  return A[0] * (A[4] * A[8] - A[5] * A[7]) - A[1] * (A[3] * A[8] - A[5] * A[6]) + A[2] * (A[3] * A[7] - A[4] * A[6]);
}

const double IDENTITY_DOFS[ND] = {0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0, 1};

}  // namespace

struct pi_aligner_s {
  pi_kgrid kg = nullptr;
  pi_batch b1 = nullptr, b2 = nullptr;
  int64_t Q = 0;
  cudaStream_t s = nullptr;
  DevMem X, ws, H, dofs;
  size_t ws_bytes = 0;
  double V11 = 0.0;
  ~pi_aligner_s() {
    if (b1) pi_batch_destroy(b1);
    if (b2) pi_batch_destroy(b2);
    if (kg) pi_kgrid_destroy(kg);
    if (s) cudaStreamDestroy(s);
  }
};

namespace {

// One evaluation at dofs2: contraction of the first m rows into out (m x m).
int evaluate(pi_aligner_s* a, const double* dofs2, int m, double* out) {
  PI_CUDA(cudaMemcpyAsync(a->dofs.p, dofs2, ND * sizeof(double), cudaMemcpyHostToDevice, a->s));
  int rc = pi_batch_set_all_dofs(a->b2, static_cast<const double*>(a->dofs.p), reinterpret_cast<pi_stream>(a->s));
  if (rc) return rc;
  float2* X = static_cast<float2*>(a->X.p);
  if ((rc = pi_form_factors(a->kg, a->b2, 1, X + a->Q, reinterpret_cast<pi_stream>(a->s)))) return rc;
  if (m > 2 && (rc = pi::launch_jacobian(a->kg, a->b2, X + 2 * a->Q, a->s))) return rc;
  if ((rc = pi_contract(a->kg, X, m, PI_CONTRACT_FP32, static_cast<double*>(a->H.p), a->ws.p, a->ws_bytes,
                        reinterpret_cast<pi_stream>(a->s))))
    return rc;
  PI_CUDA(cudaMemcpyAsync(out, a->H.p, (size_t)m * m * sizeof(double), cudaMemcpyDeviceToHost, a->s));
  PI_CUDA(cudaStreamSynchronize(a->s));
  return PI_OK;
}

pi_object affine_object(const pi_object& g, const double* dofs) {
  pi_object o = g;
  o.dof_type = PI_DOF_AFFINE;
  o.dofs = dofs;
  o.n_dofs = ND;
  return o;
}

}  // namespace

extern "C" {

int pi_aligner_create(const pi_object* geom1, const pi_object* geom2, const double* dirs, const double* kmag,
                      const double* w, int64_t Q, pi_aligner* out) {
  if (!geom1 || !geom2 || !dirs || !kmag || !w || Q <= 0 || !out)
    return fail(PI_ERR_INVALID_ARGUMENT, "pi_aligner_create: bad arguments");
  *out = nullptr;
  pi_aligner_s* a = new pi_aligner_s();
  std::unique_ptr<pi_aligner_s> guard(a);
  a->Q = Q;
  PI_CUDA(cudaStreamCreateWithFlags(&a->s, cudaStreamNonBlocking));
  int rc = pi_kgrid_create(dirs, kmag, w, Q, &a->kg);
  if (rc) return rc;
  const pi_object o1 = affine_object(*geom1, IDENTITY_DOFS), o2 = affine_object(*geom2, IDENTITY_DOFS);
  if ((rc = pi_batch_create(&o1, 1, 0, reinterpret_cast<pi_stream>(a->s), &a->b1)) ||
      (rc = pi_batch_create(&o2, 1, 0, reinterpret_cast<pi_stream>(a->s), &a->b2)))
    return rc;
  if ((rc = pi_contract_workspace_size(a->kg, ROWS, PI_CONTRACT_FP32, &a->ws_bytes))) return rc;
  PI_CUDA(cudaMalloc(&a->X.p, (size_t)ROWS * Q * sizeof(float2)));
  PI_CUDA(cudaMalloc(&a->ws.p, std::max<size_t>(a->ws_bytes, 16)));
  PI_CUDA(cudaMalloc(&a->H.p, (size_t)ROWS * ROWS * sizeof(double)));
  PI_CUDA(cudaMalloc(&a->dofs.p, ND * sizeof(double)));
  if ((rc = pi_form_factors(a->kg, a->b1, 1, a->X.p, reinterpret_cast<pi_stream>(a->s)))) return rc;
  if ((rc = pi_contract(a->kg, a->X.p, 1, PI_CONTRACT_FP32, static_cast<double*>(a->H.p), a->ws.p, a->ws_bytes,
                        reinterpret_cast<pi_stream>(a->s))))
    return rc;
  PI_CUDA(cudaMemcpyAsync(&a->V11, a->H.p, sizeof(double), cudaMemcpyDeviceToHost, a->s));
  PI_CUDA(cudaStreamSynchronize(a->s));
  *out = guard.release();
  return PI_OK;
}

int pi_aligner_destroy(pi_aligner a) {
  delete a;
  return PI_OK;
}

int pi_aligner_fixed_volume(pi_aligner a, double* V1) {
  if (!a || !V1) return fail(PI_ERR_INVALID_ARGUMENT, "pi_aligner_fixed_volume: bad arguments");
  *V1 = a->V11;
  return PI_OK;
}

int pi_similarity(pi_aligner a, const double* dofs2, int measure, double V1, int flags, double* value,
                  double* similarity, double* grad, double* hess) {
  if (!a || !dofs2 || measure < PI_SIM_OCHIAI || measure > PI_SIM_DICE)
    return fail(PI_ERR_INVALID_ARGUMENT, "pi_similarity: bad arguments");
  const bool need_g = (flags & PI_SIM_GRADIENT) != 0, need_h = (flags & PI_SIM_HESSIAN) != 0;
  if ((need_g && !grad) || (need_h && !hess)) return fail(PI_ERR_INVALID_ARGUMENT, "pi_similarity: missing output");
  const int m = (need_g || need_h) ? ROWS : 2;
  double X[ROWS * ROWS];
  int rc = evaluate(a, dofs2, m, X);
  if (rc) return rc;
  const double Vint = X[0 * m + 1], V2 = X[1 * m + 1];
  double gI[ND] = {0}, g2[ND] = {0}, H2[ND * ND] = {0};  // grad V_int, grad V2, H_V2 (H_V_int = 0)
  if (m == ROWS) {
    for (int i = 0; i < ND; ++i) {
      gI[i] = X[(2 + i) * m + 0];
      g2[i] = 2.0 * X[(2 + i) * m + 1];
      for (int j = 0; j < ND; ++j) H2[i * ND + j] = 2.0 * X[(2 + i) * m + 2 + j];
    }
  }
  double s = 0.0, gs[ND] = {0}, Hs[ND * ND] = {0};
  auto outer = [&](double c, const double* u, const double* v) {
    for (int i = 0; i < ND; ++i)
      for (int j = 0; j < ND; ++j) Hs[i * ND + j] += c * u[i] * v[j];
  };
  if (measure == PI_SIM_OCHIAI) {  // V_int / sqrt(V1 V2)
    const double inv = 1.0 / std::sqrt(V1 * V2);
    s = inv * Vint;
    const double coeff = -0.5 * inv * inv * inv * Vint * V1;
    for (int i = 0; i < ND; ++i) gs[i] = inv * gI[i] + coeff * g2[i];
    for (int i = 0; i < ND * ND; ++i) Hs[i] = -0.5 * inv * Vint / V2 * H2[i];
    outer(0.75 * inv * Vint / (V2 * V2), g2, g2);
    outer(-0.5 * inv / V2, gI, g2);
    outer(-0.5 * inv / V2, g2, gI);
  } else if (measure == PI_SIM_JACCARD) {  // V_int / (V1 + V2 - V_int)
    const double den = V1 + V2 - Vint, inv = 1.0 / den, inv2 = inv * inv;
    s = Vint / den;
    double dD[ND];
    for (int i = 0; i < ND; ++i) {
      dD[i] = g2[i] - gI[i];
      gs[i] = inv * gI[i] - inv2 * Vint * dD[i];
    }
    for (int i = 0; i < ND * ND; ++i) Hs[i] = -inv2 * Vint * H2[i];  // H_V_int = 0
    outer(-inv2, gI, dD);
    outer(-inv2, dD, gI);
    outer(2.0 * inv2 * inv * Vint, dD, dD);
  } else {  // Dice: 2 V_int / (V1 + V2)
    const double den = V1 + V2, inv = 2.0 / den, coeff = -2.0 * Vint / (den * den);
    s = 2.0 * Vint / den;
    for (int i = 0; i < ND; ++i) gs[i] = inv * gI[i] + coeff * g2[i];
    for (int i = 0; i < ND * ND; ++i) Hs[i] = coeff * H2[i];
    outer(-inv / den, gI, g2);
    outer(-inv / den, g2, gI);
    outer(-2.0 * coeff / den, g2, g2);
  }
  // objective -log(s), s clamped to 1e-10
  const double ss = std::max(s, 1e-10);
  if (similarity) *similarity = s;
  if (value) *value = -std::log(ss);
  if (need_g)
    for (int i = 0; i < ND; ++i) grad[i] = -gs[i] / ss;
  if (need_h)
    for (int i = 0; i < ND; ++i)
      for (int j = 0; j < ND; ++j) hess[i * ND + j] = gs[i] * gs[j] / (ss * ss) - Hs[i * ND + j] / ss;
  return PI_OK;
}

int pi_optimize_alignment(pi_aligner a, const double* initial_dofs, int measure, double V1, double tolerance,
                          int max_iterations, double damping, pi_optimization_state* st) {
  if (!a || !initial_dofs || !st) return fail(PI_ERR_INVALID_ARGUMENT, "pi_optimize_alignment: bad arguments");
  std::memset(st, 0, sizeof(*st));
  std::memcpy(st->dofs, initial_dofs, sizeof(st->dofs));
  auto set_status = [&](const char* msg) { std::snprintf(st->status, sizeof(st->status), "%s", msg); };
  const double alpha_init = 1.0, alpha_min = 1e-10, c = 0.1, rho = 0.5;
  const int max_ls_iter = 20;
  double g[ND], H[ND * ND];
  for (int iter = 0; iter < max_iterations; ++iter) {
    st->iteration = iter;
    st->evaluations++;
    double f0 = 0.0, sim = 0.0;
    int rc = pi_similarity(a, st->dofs, measure, V1, PI_SIM_ALL, &f0, &sim, g, H);
    if (rc) return rc;
    st->similarity = sim;
    st->similarity_loss = f0;
    double gn = 0.0;
    for (double v : g) gn += v * v;
    if (std::sqrt(gn) < tolerance) {
      st->converged = 1;
      set_status("Converged (gradient norm < tolerance)");
      break;
    }
    // Project the Hessian to PSD (negative eigenvalues to zero), add damping I
    std::vector<double> lam, Qv;
    jacobi_eigen(std::vector<double>(H, H + ND * ND), ND, lam, Qv);
    std::vector<double> Hf((size_t)ND * ND, 0.0);
    for (int i = 0; i < ND; ++i)
      for (int j = 0; j < ND; ++j) {
        double v = 0.0;
        for (int k = 0; k < ND; ++k) v += Qv[(size_t)i * ND + k] * std::max(lam[k], 0.0) * Qv[(size_t)j * ND + k];
        Hf[(size_t)i * ND + j] = v + (i == j ? damping : 0.0);
      }
    double rhs[ND], delta[ND];
    for (int i = 0; i < ND; ++i) rhs[i] = -g[i];
    if (!ldlt_solve(Hf, ND, rhs, delta)) {
      set_status("Hessian solve failed");
      break;
    }
    double descent = 0.0;
    for (int i = 0; i < ND; ++i) descent -= delta[i] * g[i];
    // Armijo backtracking: f(x + alpha d) <= f(x) + c alpha d.g
    double alpha = alpha_init, trial[ND], f_new = 0.0;
    for (int i = 0; i < ND; ++i) trial[i] = st->dofs[i] + alpha * delta[i];
    st->evaluations++;
    if ((rc = pi_similarity(a, trial, measure, V1, PI_SIM_FUNC_ONLY, &f_new, nullptr, nullptr, nullptr))) return rc;
    int ls = 0;
    while (f_new > f0 - c * alpha * descent && alpha > alpha_min && ls < max_ls_iter) {
      alpha *= rho;
      for (int i = 0; i < ND; ++i) trial[i] = st->dofs[i] + alpha * delta[i];
      st->evaluations++;
      if ((rc = pi_similarity(a, trial, measure, V1, PI_SIM_FUNC_ONLY, &f_new, nullptr, nullptr, nullptr))) return rc;
      ++ls;
    }
    if (alpha <= alpha_min) {
      set_status("Line search failed (step size too small)");
      break;
    }
    std::memcpy(st->dofs, trial, sizeof(st->dofs));
    st->steps++;
  }
  // As in the reference, any exit without convergence reports the iteration cap.
  if (!st->converged) set_status("Reached max iterations");
  return PI_OK;
}

// Moments of a geometry under x = A x0 + t (warm_start.cpp:8-131): triangle
// meshes from signed tetrahedra (0, a, b, c) with the second moment taken at
// each tetrahedron's centroid; disks / Gaussians from the divergence-theorem
// volume and area- / weight-weighted element centres (Gaussians add sigma^2 I).
int pi_compute_moments(const pi_object* geom, const double* dofs, double* volume, double* centroid,
                       double* covariance) {
  if (!geom || !dofs || !volume || !centroid || !covariance || (geom->n_elems > 0 && !geom->elems))
    return fail(PI_ERR_INVALID_ARGUMENT, "pi_compute_moments: bad arguments");
  const double* t = dofs;
  const double* A = dofs + 3;
  auto xf = [&](const double* x, double* y) {
    for (int r = 0; r < 3; ++r) y[r] = A[3 * r] * x[0] + A[3 * r + 1] * x[1] + A[3 * r + 2] * x[2] + t[r];
  };
  std::fill(centroid, centroid + 3, 0.0);
  std::fill(covariance, covariance + 9, 0.0);
  *volume = 0.0;
  if (geom->geom_type == PI_GEOM_TRIANGLE) {
    const pi_tri_packed* T = static_cast<const pi_tri_packed*>(geom->elems);
    double V = 0.0, m1[3] = {0, 0, 0}, m2[9] = {0};
    for (int64_t f = 0; f < geom->n_elems; ++f) {
      double p0[3], p1[3], p2[3], a[3], b[3], c[3];
      for (int k = 0; k < 3; ++k) { p0[k] = T[f].a[k]; p1[k] = T[f].a[k] + T[f].e1[k]; p2[k] = T[f].a[k] + T[f].e2[k]; }
      xf(p0, a); xf(p1, b); xf(p2, c);
      const double u[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]}, v[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
      const double cr[3] = {u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2], u[0] * v[1] - u[1] * v[0]};
      const double vt = (a[0] * cr[0] + a[1] * cr[1] + a[2] * cr[2]) / 6.0;
      const double ct[3] = {(a[0] + b[0] + c[0]) / 4.0, (a[1] + b[1] + c[1]) / 4.0, (a[2] + b[2] + c[2]) / 4.0};
      V += vt;
      for (int r = 0; r < 3; ++r) {
        m1[r] += vt * ct[r];
        for (int q = 0; q < 3; ++q) m2[3 * r + q] += vt * ct[r] * ct[q];
      }
    }
    if (std::fabs(V) > 1e-10) {
      *volume = V;
      for (int r = 0; r < 3; ++r) centroid[r] = m1[r] / V;
      for (int r = 0; r < 3; ++r)
        for (int q = 0; q < 3; ++q) covariance[3 * r + q] = m2[3 * r + q] / V - centroid[r] * centroid[q];
    }
    return PI_OK;
  }
  if (geom->geom_type != PI_GEOM_DISK && geom->geom_type != PI_GEOM_GAUSSIAN)
    return fail(PI_ERR_INVALID_ARGUMENT, "pi_compute_moments: unknown geometry type");
  const pi_object o = affine_object(*geom, dofs);
  int rc = pi_self_volume(&o, volume);
  if (rc) return rc;
  const bool disk = geom->geom_type == PI_GEOM_DISK;
  const pi_disk_packed* Dk = static_cast<const pi_disk_packed*>(geom->elems);
  const pi_gaussian_packed* Gs = static_cast<const pi_gaussian_packed*>(geom->elems);
  double wsum = 0.0, s1[3] = {0, 0, 0};
  for (int64_t e = 0; e < geom->n_elems; ++e) {
    double c[3];
    xf(disk ? Dk[e].c : Gs[e].c, c);
    const double wt = disk ? Dk[e].area : Gs[e].w;
    for (int r = 0; r < 3; ++r) s1[r] += wt * c[r];
    wsum += wt;
  }
  if (wsum > 1e-10)
    for (int r = 0; r < 3; ++r) centroid[r] = s1[r] / wsum;
  for (int64_t e = 0; e < geom->n_elems; ++e) {
    double c[3];
    xf(disk ? Dk[e].c : Gs[e].c, c);
    const double wt = disk ? Dk[e].area : Gs[e].w;
    const double d[3] = {c[0] - centroid[0], c[1] - centroid[1], c[2] - centroid[2]};
    const double s2 = disk ? 0.0 : Gs[e].sigma * Gs[e].sigma;
    for (int r = 0; r < 3; ++r)
      for (int q = 0; q < 3; ++q) covariance[3 * r + q] += wt * (d[r] * d[q] + (r == q ? s2 : 0.0));
  }
  if (wsum > 1e-10)
    for (int i = 0; i < 9; ++i) covariance[i] /= wsum;
  return PI_OK;
}

// Similarity warm start (warm_start.cpp:133-243): A = s R, t = c1 - A c2 with
// R aligning the principal axes (P1 P2^T after making both right-handed, which
// is already the Procrustes rotation of two orthonormal frames) and
// s = cbrt(V1 / V2) clamped to [0.1, 10] (mean sqrt eigenvalue ratio when
// |V2| <= 1e-10).  Eigenvectors are taken with ascending eigenvalues and the
// largest-magnitude component of each made positive; the reference leaves
// their signs to its eigen-solver, so warm starts agree up to those flips.
int pi_compute_warm_start(const pi_object* geom1, const pi_object* geom2, double* dofs_out) {
  if (!geom1 || !geom2 || !dofs_out) return fail(PI_ERR_INVALID_ARGUMENT, "pi_compute_warm_start: bad arguments");
  double v1, v2, c1[3], c2[3], C1[9], C2[9];
  int rc = pi_compute_moments(geom1, IDENTITY_DOFS, &v1, c1, C1);
  if (rc) return rc;
  if ((rc = pi_compute_moments(geom2, IDENTITY_DOFS, &v2, c2, C2))) return rc;
  std::vector<double> l1, P1, l2, P2;
  jacobi_eigen(std::vector<double>(C1, C1 + 9), 3, l1, P1);
  jacobi_eigen(std::vector<double>(C2, C2 + 9), 3, l2, P2);
  for (std::vector<double>* P : {&P1, &P2})
    if (det3(P->data()) < 0)
      for (int r = 0; r < 3; ++r) (*P)[3 * r + 2] = -(*P)[3 * r + 2];
  double R[9];
  for (int r = 0; r < 3; ++r)
    for (int q = 0; q < 3; ++q) R[3 * r + q] = P1[3 * r] * P2[3 * q] + P1[3 * r + 1] * P2[3 * q + 1] + P1[3 * r + 2] * P2[3 * q + 2];
  double s = 1.0;
  if (std::fabs(v2) > 1e-10) {
    s = std::cbrt(v1 / v2);
  } else {
    double mr = 0.0;
    int cnt = 0;
    for (int i = 0; i < 3; ++i)
      if (l2[i] > 1e-6) { mr += std::sqrt(l1[i] / l2[i]); ++cnt; }
    s = cnt ? mr / cnt : 1.0;
  }
  s = std::max(0.1, std::min(10.0, s));
  for (int r = 0; r < 3; ++r) {
    double Ac2 = 0.0;
    for (int q = 0; q < 3; ++q) {
      dofs_out[3 + 3 * r + q] = s * R[3 * r + q];
      Ac2 += s * R[3 * r + q] * c2[q];
    }
    dofs_out[r] = c1[r] - Ac2;
  }
  return PI_OK;
}

}  // extern "C"
