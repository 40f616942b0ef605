// Host-side parts of the C ABI that need no GPU: error state, quadrature,
// Lebedev loading, packing, test-shape generators, analytic volumes and the
// divergence-theorem self-volume.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>
#include <atomic>
#include <map>
#include <mutex>
#include <utility>
#include "pi_internal.h"

namespace pi {

namespace {
thread_local std::string g_last_error;
thread_local int64_t g_launches = 0;
}  // namespace

void set_error(const std::string& msg) { g_last_error = msg; }
int fail(int status, const std::string& msg) {
  g_last_error = msg;
  return status;
}
int cuda_fail(cudaError_t e, const char* what) {
  g_last_error = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
  return e == cudaErrorMemoryAllocation ? PI_ERR_OUT_OF_MEMORY : PI_ERR_CUDA;
}
void count_launch(int n) { g_launches += n; }

int current_sm_count() {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      sms <= 0)
    return 148;
  return sms;
}

int ensure_smem_limit(const void* fn, int bytes, const char* what) {
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, cudaError_t> done;  // (function, device) -> result
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  std::lock_guard<std::mutex> lock(mu);
  auto it = done.find({fn, dev});
  if (it == done.end())
    it = done.emplace(std::make_pair(fn, dev), cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes))
             .first;
  return it->second == cudaSuccess ? PI_OK : cuda_fail(it->second, what);
}

}  // namespace pi

using pi::fail;

static const double PI_D = 3.14159265358979323846;

extern "C" {

const char* pi_status_string(int status) {
  switch (status) {
    case PI_OK: return "ok";
    case PI_ERR_INVALID_ARGUMENT: return "invalid argument";
    case PI_ERR_CUDA: return "CUDA error";
    case PI_ERR_UNSUPPORTED: return "unsupported";
    case PI_ERR_OUT_OF_MEMORY: return "out of memory";
    case PI_ERR_NOT_FOUND: return "not found";
    case PI_ERR_WORKSPACE_TOO_SMALL: return "workspace too small";
    case PI_ERR_IO: return "I/O error";
    case PI_ERR_TIMEOUT: return "timeout";
    default: return "unknown status";
  }
}

const char* pi_last_error(void) { return pi::g_last_error.c_str(); }
int pi_version(void) { return 1; }
int64_t pi_launch_count(void) { return pi::g_launches; }

// Gauss-Legendre nodes/weights on [a,b]: Newton iteration on P_n from the
// Chebyshev-like initial guess cos(pi (i + 3/4)/(n + 1/2)), stopping at 1e-14,
// weights 2/((1-x^2) P_n'(x)^2) -- the recipe of
// cpp/include/quadrature/gauss_legendre.hpp:16-62, so nodes match bitwise.
int pi_gauss_legendre(int n, double a, double b, double* x, double* w) {
  if (n <= 0 || !x || !w) return fail(PI_ERR_INVALID_ARGUMENT, "pi_gauss_legendre: n must be > 0");
  const int m = (n + 1) / 2;
  for (int i = 0; i < m; ++i) {
    double z = std::cos(PI_D * (i + 0.75) / (n + 0.5)), z1, pp;
    int it = 0;
    do {
      double p1 = 1.0, p2 = 0.0;
      for (int j = 1; j <= n; ++j) {
        double p3 = p2;
        p2 = p1;
        p1 = ((2.0 * j - 1.0) * z * p2 - (j - 1.0) * p3) / j;
      }
      pp = n * (z * p1 - p2) / (z * z - 1.0);
      z1 = z;
      z = z1 - p1 / pp;
    } while (std::abs(z - z1) > 1e-14 && ++it < 1000);
    double p1 = 1.0, p2 = 0.0;
    for (int j = 1; j <= n; ++j) {
      double p3 = p2;
      p2 = p1;
      p1 = ((2.0 * j - 1.0) * z * p2 - (j - 1.0) * p3) / j;
    }
    pp = n * (z * p1 - p2) / (z * z - 1.0);
    const double wi = 2.0 / ((1.0 - z * z) * pp * pp);
    const double xm = 0.5 * (b + a), xl = 0.5 * (b - a);
    x[i] = xm - xl * z;
    x[n - 1 - i] = xm + xl * z;
    w[i] = xl * wi;
    w[n - 1 - i] = xl * wi;
  }
  return PI_OK;
}

// Lebedev text rows "theta_deg phi_deg weight"; direction
// (cos th sin ph, sin th sin ph, cos ph); weights summing to ~1 are rescaled to
// 4 pi (cpp/include/quadrature/lebedev_io.hpp:24-59).
int pi_load_lebedev(const char* path, double* dirs, double* w, int64_t cap, int64_t* n_rows) {
  if (!path) return fail(PI_ERR_INVALID_ARGUMENT, "pi_load_lebedev: null path");
  std::ifstream in(path);
  if (!in) return fail(PI_ERR_IO, std::string("failed to open Lebedev file: ") + path);
  std::vector<double> d, ws;
  std::string line;
  double sum = 0.0;
  while (std::getline(in, line)) {
    if (line.empty() || line[0] == '#') continue;
    std::istringstream ss(line);
    double th, ph, wt;
    if (!(ss >> th >> ph >> wt)) continue;
    th *= PI_D / 180.0;
    ph *= PI_D / 180.0;
    d.push_back(std::cos(th) * std::sin(ph));
    d.push_back(std::sin(th) * std::sin(ph));
    d.push_back(std::cos(ph));
    ws.push_back(wt);
    sum += wt;
  }
  if (ws.empty()) return fail(PI_ERR_IO, "Lebedev file had no data");
  if (std::abs(sum - 1.0) < 0.1)
    for (double& v : ws) v *= 4.0 * PI_D;
  const int64_t n = (int64_t)ws.size();
  if (n_rows) *n_rows = n;
  for (int64_t i = 0; i < n && i < cap; ++i) {
    if (dirs) { dirs[3 * i] = d[3 * i]; dirs[3 * i + 1] = d[3 * i + 1]; dirs[3 * i + 2] = d[3 * i + 2]; }
    if (w) w[i] = ws[i];
  }
  return PI_OK;
}

// k = tan t over Gauss-Legendre t in [0, pi/2]; node q = ir*M + j; weight
// w_leb * w_GL * sec^2 t (cpp/include/quadrature/kgrid.hpp:17-47).
int pi_build_kgrid(const double* ld, const double* lw, int64_t M, int n_radial, double* dirs, double* kmag,
                   double* w) {
  if (M <= 0 || n_radial <= 0 || !ld || !lw || !dirs || !kmag || !w)
    return fail(PI_ERR_INVALID_ARGUMENT, "pi_build_kgrid: bad arguments");
  std::vector<double> t(n_radial), wt(n_radial);
  int rc = pi_gauss_legendre(n_radial, 0.0, 0.5 * PI_D, t.data(), wt.data());
  if (rc) return rc;
  for (int ir = 0; ir < n_radial; ++ir) {
    const double sec2 = 1.0 / std::cos(t[ir]) / std::cos(t[ir]);
    const double k = std::tan(t[ir]);
    for (int64_t j = 0; j < M; ++j) {
      const int64_t q = (int64_t)ir * M + j;
      dirs[3 * q] = ld[3 * j];
      dirs[3 * q + 1] = ld[3 * j + 1];
      dirs[3 * q + 2] = ld[3 * j + 2];
      kmag[q] = k;
      w[q] = lw[j] * (wt[ir] * sec2);
    }
  }
  return PI_OK;
}

int pi_pack_tris(const double* V, int64_t n_verts, const int32_t* F, int64_t n_faces, pi_tri_packed* out) {
  if ((n_faces > 0 && (!V || !F || !out)) || n_verts < 0 || n_faces < 0)
    return fail(PI_ERR_INVALID_ARGUMENT, "pi_pack_tris: bad arguments");
  for (int64_t i = 0; i < n_faces; ++i) {
    const int32_t ia = F[3 * i], ib = F[3 * i + 1], ic = F[3 * i + 2];
    if (ia < 0 || ib < 0 || ic < 0 || ia >= n_verts || ib >= n_verts || ic >= n_verts)
      return fail(PI_ERR_INVALID_ARGUMENT, "pi_pack_tris: face index out of range");
    const double* a = V + 3 * ia;
    const double* b = V + 3 * ib;
    const double* c = V + 3 * ic;
    pi_tri_packed& T = out[i];
    for (int k = 0; k < 3; ++k) {
      T.a[k] = a[k];
      T.e1[k] = b[k] - a[k];
      T.e2[k] = c[k] - a[k];
    }
    T.S[0] = 0.5 * (T.e1[1] * T.e2[2] - T.e1[2] * T.e2[1]);
    T.S[1] = 0.5 * (T.e1[2] * T.e2[0] - T.e1[0] * T.e2[2]);
    T.S[2] = 0.5 * (T.e1[0] * T.e2[1] - T.e1[1] * T.e2[0]);
    T.vid0 = ia; T.vid1 = ib; T.vid2 = ic; T.pad_ = 0;
  }
  return PI_OK;
}

int pi_pack_disks(const double* P, const double* N, const double* r, int64_t n, int is_radius, pi_disk_packed* out) {
  if (n < 0 || (n > 0 && (!P || !N || !r || !out))) return fail(PI_ERR_INVALID_ARGUMENT, "pi_pack_disks: bad arguments");
  for (int64_t i = 0; i < n; ++i) {
    const double* nn = N + 3 * i;
    const double len = std::sqrt(nn[0] * nn[0] + nn[1] * nn[1] + nn[2] * nn[2]);
    pi_disk_packed& D = out[i];
    for (int k = 0; k < 3; ++k) { D.c[k] = P[3 * i + k]; D.n[k] = nn[k] / len; }
    if (is_radius) { D.rho = r[i]; D.area = PI_D * r[i] * r[i]; }
    else { D.area = r[i]; D.rho = std::sqrt(r[i] / PI_D); }
  }
  return PI_OK;
}

int pi_pack_gaussians(const double* P, const double* N, const double* s, const double* wt, int64_t n,
                      pi_gaussian_packed* out) {
  if (n < 0 || (n > 0 && (!P || !N || !s || !wt || !out)))
    return fail(PI_ERR_INVALID_ARGUMENT, "pi_pack_gaussians: bad arguments");
  for (int64_t i = 0; i < n; ++i) {
    const double* nn = N + 3 * i;
    const double len = std::sqrt(nn[0] * nn[0] + nn[1] * nn[1] + nn[2] * nn[2]);
    pi_gaussian_packed& G = out[i];
    for (int k = 0; k < 3; ++k) { G.c[k] = P[3 * i + k]; G.n[k] = nn[k] / len; }
    G.sigma = s[i];
    G.w = wt[i];
  }
  return PI_OK;
}

// Unit cube [-1/2,1/2]^3, 12 outward-oriented triangles, vertex/face order of
// cpp/src/geometry/geometry_helpers.cpp:16-38.
int pi_create_unit_cube_mesh(double* V, int32_t* F) {
  if (!V || !F) return fail(PI_ERR_INVALID_ARGUMENT, "pi_create_unit_cube_mesh: null output");
  static const double v[24] = {-0.5, -0.5, -0.5, 0.5, -0.5, -0.5, 0.5, 0.5, -0.5, -0.5, 0.5, -0.5,
                               -0.5, -0.5, 0.5,  0.5, -0.5, 0.5,  0.5, 0.5, 0.5,  -0.5, 0.5, 0.5};
  static const int32_t f[36] = {0, 2, 1, 0, 3, 2, 4, 5, 6, 4, 6, 7, 0, 1, 5, 0, 5, 4,
                                2, 7, 6, 2, 3, 7, 0, 4, 7, 0, 7, 3, 1, 6, 5, 1, 2, 6};
  std::memcpy(V, v, sizeof v);
  std::memcpy(F, f, sizeof f);
  return PI_OK;
}

// Fibonacci (golden-angle) sphere samples, y from 1 to -1
// (cpp/src/geometry/geometry_helpers.cpp:40-131).
static void fibonacci(int n, double* P, double* N) {
  const double ga = PI_D * (3.0 - std::sqrt(5.0));
  for (int i = 0; i < n; ++i) {
    const double y = 1.0 - (2.0 * i) / (n - 1.0);
    const double ry = std::sqrt(1.0 - y * y);
    const double th = ga * i;
    const double x = ry * std::cos(th), z = ry * std::sin(th);
    P[3 * i] = x; P[3 * i + 1] = y; P[3 * i + 2] = z;
    N[3 * i] = x; N[3 * i + 1] = y; N[3 * i + 2] = z;
  }
}

int pi_create_sphere_pointcloud(int n, double* P, double* N, double* radii) {
  if (n < 2 || !P || !N || !radii) return fail(PI_ERR_INVALID_ARGUMENT, "pi_create_sphere_pointcloud: n >= 2");
  fibonacci(n, P, N);
  const double r = std::sqrt((4.0 * PI_D / n) / PI_D);
  for (int i = 0; i < n; ++i) radii[i] = r;
  return PI_OK;
}

int pi_create_sphere_gaussians(int n, double* P, double* N, double* sigmas, double* weights) {
  if (n < 2 || !P || !N || !sigmas || !weights)
    return fail(PI_ERR_INVALID_ARGUMENT, "pi_create_sphere_gaussians: n >= 2");
  fibonacci(n, P, N);
  const double wt = 4.0 * PI_D / n, s = std::sqrt(wt / (4.0 * PI_D));
  for (int i = 0; i < n; ++i) { weights[i] = wt; sigmas[i] = s; }
  return PI_OK;
}

double pi_box_box_intersection_volume(const double* c1, const double* h1, const double* c2, const double* h2) {
  double v = 1.0;
  for (int i = 0; i < 3; ++i) {
    const double lo = std::fmax(c1[i] - h1[i], c2[i] - h2[i]);
    const double hi = std::fmin(c1[i] + h1[i], c2[i] + h2[i]);
    v *= std::fmax(0.0, hi - lo);
  }
  return v;
}

double pi_sphere_sphere_intersection_volume(const double* c1, double r1, const double* c2, double r2) {
  const double dx = c2[0] - c1[0], dy = c2[1] - c1[1], dz = c2[2] - c1[2];
  const double d = std::sqrt(dx * dx + dy * dy + dz * dz);
  if (d >= r1 + r2) return 0.0;
  if (d <= std::fabs(r1 - r2)) {
    const double r = std::fmin(r1, r2);
    return 4.0 * PI_D / 3.0 * r * r * r;
  }
  const double t1 = (r1 + r2 - d) * (r1 + r2 - d);
  const double t2 = d * d + 2.0 * d * (r1 + r2) - 3.0 * (r1 * r1 + r2 * r2) + 6.0 * r1 * r2;
  return PI_D * t1 * t2 / (12.0 * d);
}

int pi_self_volume(const pi_object* o, double* volume) {
  if (!o || !volume || (o->n_elems > 0 && !o->elems) || !o->dofs)
    return fail(PI_ERR_INVALID_ARGUMENT, "pi_self_volume: bad arguments");
  if (o->dof_type == PI_DOF_TRIANGLE_MESH) {
    if (o->geom_type != PI_GEOM_TRIANGLE) return fail(PI_ERR_INVALID_ARGUMENT, "TriangleMeshDoF needs triangles");
    const pi_tri_packed* T = static_cast<const pi_tri_packed*>(o->elems);
    const int64_t nv = o->n_dofs / 3;
    double s = 0.0;
    for (int64_t f = 0; f < o->n_elems; ++f) {
      const int32_t i = T[f].vid0, j = T[f].vid1, k = T[f].vid2;
      if (i < 0 || j < 0 || k < 0 || i >= nv || j >= nv || k >= nv) continue;
      const double* a = o->dofs + 3 * i;
      const double* b = o->dofs + 3 * j;
      const double* c = o->dofs + 3 * k;
      s += a[0] * (b[1] * c[2] - b[2] * c[1]) + a[1] * (b[2] * c[0] - b[0] * c[2]) + a[2] * (b[0] * c[1] - b[1] * c[0]);
    }
    *volume = s / 6.0;
    return PI_OK;
  }
  if (o->dof_type != PI_DOF_AFFINE || o->n_dofs != 12) return fail(PI_ERR_INVALID_ARGUMENT, "AffineDoF needs 12 DoFs");
  const double* A = o->dofs + 3;
  const double det = A[0] * (A[4] * A[8] - A[5] * A[7]) - A[1] * (A[3] * A[8] - A[5] * A[6]) +
                     A[2] * (A[3] * A[7] - A[4] * A[6]);
  double vb = 0.0;
  if (o->geom_type == PI_GEOM_TRIANGLE) {
    const pi_tri_packed* T = static_cast<const pi_tri_packed*>(o->elems);
    for (int64_t i = 0; i < o->n_elems; ++i) vb += T[i].a[0] * T[i].S[0] + T[i].a[1] * T[i].S[1] + T[i].a[2] * T[i].S[2];
  } else if (o->geom_type == PI_GEOM_DISK) {
    const pi_disk_packed* D = static_cast<const pi_disk_packed*>(o->elems);
    for (int64_t i = 0; i < o->n_elems; ++i)
      vb += (D[i].c[0] * D[i].n[0] + D[i].c[1] * D[i].n[1] + D[i].c[2] * D[i].n[2]) * D[i].area;
  } else if (o->geom_type == PI_GEOM_GAUSSIAN) {
    const pi_gaussian_packed* G = static_cast<const pi_gaussian_packed*>(o->elems);
    for (int64_t i = 0; i < o->n_elems; ++i)
      vb += (G[i].c[0] * G[i].n[0] + G[i].c[1] * G[i].n[1] + G[i].c[2] * G[i].n[2]) * G[i].w;
  } else {
    return fail(PI_ERR_INVALID_ARGUMENT, "unknown geometry type");
  }
  *volume = vb / 3.0 * std::fabs(det);
  return PI_OK;
}

}  // extern "C"
