// ============================================================================
// FP64 CPU ORACLE for the Fourier intersection-volume path.
//
// TEST INFRASTRUCTURE ONLY.  This file restates, in plain C++17 + OpenMP, the
// reference's CPU algorithm (PoIntInt, cpp/src/*.cpp) so that the CUDA product
// can be checked against it.  Only tests/, __graft_entry__.smoke() and the
// cpu_baseline / reference legs of bench.py may load it.  It is never part of
// the shipped path and the product never falls back to it.
//
// Parity anchors (reference file:line, paths inside the PoIntInt project):
//   element functions   cpp/src/element_functions.cpp:17-120
//   element form factors cpp/src/form_factor_helpers.cpp:23-87
//   analytic transforms cpp/src/form_factor_helpers.cpp:145-179
//   AffineDoF            cpp/src/dof/affine_dof.cpp:17-462
//   TriangleMeshDoF      cpp/src/dof/triangle_mesh_dof.cpp:18-218
//   pair driver          cpp/src/compute_intersection_volume_cpu.cpp:21-208
//   matrix driver        cpp/src/compute_intersection_volume_multi_object.cpp:31-361
//   quadrature           cpp/include/quadrature/{gauss_legendre,lebedev_io,kgrid}.hpp
//   packing / shapes     cpp/src/geometry/packing.cpp:10-124,
//                        cpp/src/geometry/geometry_helpers.cpp:16-131
//   analytic volumes     cpp/src/analytical_intersection.cpp:15-60
//
// Recorded deviations from the reference (allowed, numerically benign):
//   * sums over k-nodes and over elements run in a fixed order (sequential per
//     k-node, fixed-order pairwise over k-nodes), not TBB's scheduling order;
//   * AffineDoF transforms each element once per call instead of once per
//     (element, k) pair -- the arithmetic per element is identical.
// Additions with no reference counterpart (pinned by finite differences and by
// the translation-sum identity in the tests):
//   * per-disk / per-Gaussian position and normal gradients (identity DoFs).
// ============================================================================
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#include <omp.h>

namespace {

using cd = std::complex<double>;
const cd I1(0.0, 1.0);
const double PI = 3.14159265358979323846;

// Packed element layouts: byte-compatible with the reference's TriPacked,
// DiskPacked, GaussianPacked (cpp/include/geometry/types.hpp:9-37).
struct Tri { double a[3], e1[3], e2[3], S[3]; int32_t vid0, vid1, vid2, pad; };
struct Disk { double c[3], n[3], rho, area; };
struct Gauss { double c[3], n[3], sigma, w; };
static_assert(sizeof(Tri) == 112, "TriPacked layout");
static_assert(sizeof(Disk) == 64, "DiskPacked layout");
static_assert(sizeof(Gauss) == 64, "GaussianPacked layout");

enum { GEOM_TRIANGLE = 0, GEOM_DISK = 1, GEOM_GAUSSIAN = 2 };
enum { DOF_AFFINE = 0, DOF_TRIANGLE_MESH = 1 };
enum { FLAG_VOLUME = 1, FLAG_GRADIENT = 2, FLAG_HESSIAN = 4 };

struct V3 { double x, y, z; };
inline V3 v3(const double* p) { return {p[0], p[1], p[2]}; }
inline double dot(const V3& a, const V3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(const V3& a, const V3& b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline V3 add(const V3& a, const V3& b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 sub(const V3& a, const V3& b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 scl(const V3& a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline double norm(const V3& a) { return std::sqrt(dot(a, a)); }

struct M3 { double m[3][3]; };
inline V3 mul(const M3& A, const V3& v) {
  return {A.m[0][0] * v.x + A.m[0][1] * v.y + A.m[0][2] * v.z,
          A.m[1][0] * v.x + A.m[1][1] * v.y + A.m[1][2] * v.z,
          A.m[2][0] * v.x + A.m[2][1] * v.y + A.m[2][2] * v.z};
}
inline V3 mulT(const M3& A, const V3& v) {
  return {A.m[0][0] * v.x + A.m[1][0] * v.y + A.m[2][0] * v.z,
          A.m[0][1] * v.x + A.m[1][1] * v.y + A.m[2][1] * v.z,
          A.m[0][2] * v.x + A.m[1][2] * v.y + A.m[2][2] * v.z};
}

// ---------------------------------------------------------------------------
// Element functions (cpp/src/element_functions.cpp:17-120)
// ---------------------------------------------------------------------------
cd E_func(double z) {
  if (std::abs(z) < 1e-4) {
    double z2 = z * z, z4 = z2 * z2;
    return cd(1.0 - z2 / 6.0 + z4 / 120.0, z * 0.5 - z * z2 / 24.0 + z4 * z / 720.0);
  }
  return cd(std::sin(z) / z, (1.0 - std::cos(z)) / z);
}

cd E_prime(double z) {
  if (std::abs(z) < 1e-4) {
    double z2 = z * z, z3 = z2 * z, z4 = z2 * z2;
    return cd(-z / 3.0 + z3 / 30.0, 0.5 - z2 / 8.0 + z4 / 144.0);
  }
  double s = std::sin(z), c = std::cos(z), z2 = z * z;
  return cd((z * c - s) / z2, (z * s - (1.0 - c)) / z2);
}

cd E_double_prime(double z) {
  double z2 = z * z;
  if (std::abs(z) < 1e-4) return cd(-1.0 / 3.0 + z2 / 10.0, -z / 4.0 + z2 * z / 36.0);
  double s = std::sin(z), c = std::cos(z), z3 = z2 * z;
  return cd((2.0 * s - 2.0 * z * c - z2 * s) / z3, (2.0 * (1.0 - c) - 2.0 * z * s + z2 * c) / z3);
}

cd Phi_ab(double a, double b) {
  double d = b - a;
  if (std::abs(d) < 1e-3) return -2.0 * I1 * E_prime(0.5 * (a + b));
  return -2.0 * I1 * (E_func(b) - E_func(a)) / d;
}

void Phi_ab_grad(double a, double b, cd* dPa, cd* dPb) {
  double d = b - a;
  if (std::abs(d) < 1e-3) {
    cd g = -I1 * E_double_prime(0.5 * (a + b));
    *dPa = g; *dPb = g;
    return;
  }
  cd t1 = (E_func(b) - E_func(a)) / (d * d);
  *dPa = -2.0 * I1 * (t1 - E_prime(a) / d);
  *dPb = 2.0 * I1 * (t1 - E_prime(b) / d);
}

double J1x(double x) {
  if (std::abs(x) < 1e-5) { double x2 = x * x; return 0.5 - x2 / 16.0 + x2 * x2 / 384.0; }
  return std::cyl_bessel_j(1.0, x) / x;
}

double J1x_prime(double x) {
  if (std::abs(x) < 1e-5) return -x / 8.0 + x * x * x / 96.0;
  return -std::cyl_bessel_j(2.0, x) / x;
}

// ---------------------------------------------------------------------------
// Objects and DoFs
// ---------------------------------------------------------------------------
struct Object {
  int32_t geom_type, dof_type;
  int64_t n_elems;
  const void* elems;
  int64_t n_dofs;
  const double* dofs;
};

// AffineDoF layout [tx,ty,tz, A00..A22 row-major] (cpp/src/dof/affine_dof.cpp:17-29)
void affine_of(const double* d, M3* A, V3* t) {
  *t = {d[0], d[1], d[2]};
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) A->m[r][c] = d[3 + 3 * r + c];
}

double det3(const M3& A) {
  const auto& m = A.m;
  return m[0][0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1]) -
         m[0][1] * (m[1][0] * m[2][2] - m[1][2] * m[2][0]) +
         m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]);
}

// Per-call element transform: triangle (a', e1', e2', S'), restating
// affine_dof.cpp:83-86 and triangle_mesh_dof.cpp:46-54.
struct TriT { V3 a, e1, e2, S; V3 a0, e10, e20, S0; int vid[3]; };

std::vector<TriT> transform_tris(const Object& o) {
  const Tri* T = static_cast<const Tri*>(o.elems);
  std::vector<TriT> out(o.n_elems);
  if (o.dof_type == DOF_AFFINE) {
    M3 A; V3 t; affine_of(o.dofs, &A, &t);
    for (int64_t i = 0; i < o.n_elems; ++i) {
      TriT& x = out[i];
      x.a0 = v3(T[i].a); x.e10 = v3(T[i].e1); x.e20 = v3(T[i].e2); x.S0 = v3(T[i].S);
      x.a = add(mul(A, x.a0), t);
      x.e1 = mul(A, x.e10);
      x.e2 = mul(A, x.e20);
      x.S = scl(cross(x.e1, x.e2), 0.5);
      x.vid[0] = T[i].vid0; x.vid[1] = T[i].vid1; x.vid[2] = T[i].vid2;
    }
  } else {
    for (int64_t i = 0; i < o.n_elems; ++i) {
      TriT& x = out[i];
      x.vid[0] = T[i].vid0; x.vid[1] = T[i].vid1; x.vid[2] = T[i].vid2;
      if (x.vid[0] < 0 || x.vid[1] < 0 || x.vid[2] < 0) { x.vid[0] = -1; continue; }
      V3 v0 = v3(o.dofs + 3 * x.vid[0]), v1 = v3(o.dofs + 3 * x.vid[1]), v2 = v3(o.dofs + 3 * x.vid[2]);
      x.a = v0; x.e1 = sub(v1, v0); x.e2 = sub(v2, v0);
      x.S = scl(cross(x.e1, x.e2), 0.5);
      x.a0 = x.a; x.e10 = x.e1; x.e20 = x.e2; x.S0 = x.S;
    }
  }
  return out;
}

// Disks / Gaussians under AffineDoF: c' = A c + t; k' = A^T k is used for k.n
// and |k_perp|; the normal itself is not transformed; divide by |k|
// (affine_dof.cpp:103-167).
struct SurfT { V3 c0, c, n; double p0, p1; };  // p0 = rho|sigma, p1 = area|w

std::vector<SurfT> transform_surfels(const Object& o) {
  M3 A; V3 t; affine_of(o.dofs, &A, &t);
  std::vector<SurfT> out(o.n_elems);
  if (o.geom_type == GEOM_DISK) {
    const Disk* D = static_cast<const Disk*>(o.elems);
    for (int64_t i = 0; i < o.n_elems; ++i) {
      out[i].c0 = v3(D[i].c); out[i].c = add(mul(A, out[i].c0), t); out[i].n = v3(D[i].n);
      out[i].p0 = D[i].rho; out[i].p1 = D[i].area;
    }
  } else {
    const Gauss* G = static_cast<const Gauss*>(o.elems);
    for (int64_t i = 0; i < o.n_elems; ++i) {
      out[i].c0 = v3(G[i].c); out[i].c = add(mul(A, out[i].c0), t); out[i].n = v3(G[i].n);
      out[i].p0 = G[i].sigma; out[i].p1 = G[i].w;
    }
  }
  return out;
}

struct Prepared {
  Object o;
  M3 A; V3 t;
  std::vector<TriT> tris;
  std::vector<SurfT> surf;
};

Prepared prepare(const Object& o) {
  Prepared p; p.o = o;
  if (o.dof_type == DOF_AFFINE) affine_of(o.dofs, &p.A, &p.t);
  if (o.geom_type == GEOM_TRIANGLE) p.tris = transform_tris(o);
  else p.surf = transform_surfels(o);
  return p;
}

// A(k) of one prepared object (affine_dof.cpp:55-170, triangle_mesh_dof.cpp:18-74,
// form_factor_helpers.cpp:23-87).
cd form_factor(const Prepared& p, const V3& k) {
  double km = norm(k);
  if (km < 1e-10) return cd(0, 0);
  V3 kh = scl(k, 1.0 / km);
  cd acc(0, 0);
  if (p.o.geom_type == GEOM_TRIANGLE) {
    for (const TriT& x : p.tris) {
      if (p.o.dof_type == DOF_TRIANGLE_MESH && x.vid[0] < 0) continue;
      double al = dot(k, x.e1), be = dot(k, x.e2), ga = dot(kh, x.S);
      acc += std::exp(I1 * dot(k, x.a)) * Phi_ab(al, be) * ga;
    }
  } else if (p.o.geom_type == GEOM_DISK) {
    V3 kp = mulT(p.A, k);
    double kp2 = dot(kp, kp);
    for (const SurfT& x : p.surf) {
      double kn = dot(kp, x.n);
      double r = std::sqrt(std::max(0.0, kp2 - kn * kn));
      double rr = x.p0 * r;
      double Sm = (rr < 1e-10) ? x.p1 : 2.0 * x.p1 * J1x(rr);
      acc += std::exp(dot(k, x.c) * I1) * (Sm * kn / km);
    }
  } else {
    V3 kp = mulT(p.A, k);
    double kp2 = dot(kp, kp);
    for (const SurfT& x : p.surf) {
      double kn = dot(kp, x.n);
      double r2 = kp2 - kn * kn;  // the reference CPU path does not clamp here
      double Sm = x.p1 * std::exp(-0.5 * x.p0 * x.p0 * r2);
      acc += std::exp(dot(k, x.c) * I1) * (Sm * kn / km);
    }
  }
  return acc;
}

inline M3 crossmat(const V3& v) {
  M3 c = {{{0, -v.z, v.y}, {v.z, 0, -v.x}, {-v.y, v.x, 0}}};
  return c;
}

// dA(k)/d(dofs) of one prepared object.  Affine: 12 complex values laid out
// [t0,t1,t2, A00..A22 row-major] (affine_dof.cpp:172-322).  Mesh: 3V values
// (triangle_mesh_dof.cpp:76-143).  `g` must hold n_dofs entries.
void form_factor_grad(const Prepared& p, const V3& k, cd* g) {
  int64_t nd = p.o.n_dofs;
  for (int64_t i = 0; i < nd; ++i) g[i] = 0;
  double km = norm(k);
  if (km < 1e-10) return;
  V3 kh = scl(k, 1.0 / km);
  double kv[3] = {k.x, k.y, k.z};
  if (p.o.dof_type == DOF_TRIANGLE_MESH) {
    for (const TriT& x : p.tris) {
      if (x.vid[0] < 0) continue;
      double kap = dot(kh, x.S);
      V3 dk[3] = {scl(cross(kh, sub(x.e2, x.e1)), 0.5), scl(cross(kh, x.e2), -0.5),
                  scl(cross(kh, x.e1), 0.5)};
      cd T = std::exp(I1 * dot(k, x.a));
      double al = dot(k, x.e1), be = dot(k, x.e2);
      cd psi = Phi_ab(al, be), dPa, dPb;
      Phi_ab_grad(al, be, &dPa, &dPb);
      cd fk[3] = {psi * I1 - dPa - dPb, dPa, dPb};
      for (int v = 0; v < 3; ++v) {
        double dkv[3] = {dk[v].x, dk[v].y, dk[v].z};
        for (int c = 0; c < 3; ++c) g[3 * x.vid[v] + c] += T * (psi * dkv[c] + kap * kv[c] * fk[v]);
      }
    }
    return;
  }
  // AffineDoF
  cd gt[3] = {0, 0, 0};
  cd gA[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  if (p.o.geom_type == GEOM_TRIANGLE) {
    M3 ck = crossmat(kh);
    for (const TriT& x : p.tris) {
      double al = dot(k, x.e1), be = dot(k, x.e2), ga = dot(kh, x.S);
      cd phi = Phi_ab(al, be), ph = std::exp(I1 * dot(k, x.a));
      cd At = ph * phi * ga, dPa, dPb;
      Phi_ab_grad(al, be, &dPa, &dPb);
      for (int r = 0; r < 3; ++r) gt[r] += I1 * At * kv[r];
      double a0[3] = {x.a0.x, x.a0.y, x.a0.z}, e10[3] = {x.e10.x, x.e10.y, x.e10.z},
             e20[3] = {x.e20.x, x.e20.y, x.e20.z};
      // -[khat]x A [S]x * phase * phi   (affine_dof.cpp:224)
      M3 cS = crossmat(x.S0);
      double KA[3][3], KAS[3][3];
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
          KA[r][c] = 0;
          for (int m = 0; m < 3; ++m) KA[r][c] += ck.m[r][m] * p.A.m[m][c];
        }
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
          KAS[r][c] = 0;
          for (int m = 0; m < 3; ++m) KAS[r][c] += KA[r][m] * cS.m[m][c];
        }
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c)
          gA[r][c] += At * I1 * kv[r] * a0[c] + ga * ph * kv[r] * (dPa * e10[c] + dPb * e20[c]) -
                      KAS[r][c] * ph * phi;
    }
  } else {
    V3 kp = mulT(p.A, k);
    double kp2 = dot(kp, kp);
    double khv[3] = {kh.x, kh.y, kh.z};
    for (const SurfT& x : p.surf) {
      double kn = dot(kp, x.n);
      cd ph = std::exp(dot(k, x.c) * I1);
      double Sm, dS;
      if (p.o.geom_type == GEOM_DISK) {
        double r = std::sqrt(std::max(0.0, kp2 - kn * kn));
        double rr = x.p0 * r;
        Sm = (rr < 1e-10) ? x.p1 : 2.0 * x.p1 * J1x(rr);
        dS = (rr < 1e-10) ? -0.25 * x.p0 : 2.0 * J1x_prime(rr) / r;
        dS *= x.p0 * x.p1;
      } else {
        double r2 = kp2 - kn * kn;
        Sm = x.p1 * std::exp(-0.5 * x.p0 * x.p0 * r2);
        dS = -x.p0 * x.p0 * Sm;
      }
      cd Ae = ph * (Sm * kn / km);
      for (int r = 0; r < 3; ++r) gt[r] += I1 * Ae * kv[r];
      double c0[3] = {x.c0.x, x.c0.y, x.c0.z}, nn[3] = {x.n.x, x.n.y, x.n.z};
      double kperp[3] = {kp.x - kn * x.n.x, kp.y - kn * x.n.y, kp.z - kn * x.n.z};
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c)
          gA[r][c] += Ae * I1 * kv[r] * c0[c] + khv[r] * nn[c] * ph * Sm +
                      ph * (kn / km) * dS * kv[r] * kperp[c];
    }
  }
  for (int r = 0; r < 3; ++r) g[r] = gt[r];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) g[3 + 3 * r + c] = gA[r][c];
}

// Fixed-order pairwise sum (deterministic; replaces TBB's reduction order).
double pairwise_sum(const double* x, int64_t n) {
  if (n <= 64) {
    double s = 0;
    for (int64_t i = 0; i < n; ++i) s += x[i];
    return s;
  }
  int64_t h = n / 2;
  return pairwise_sum(x, h) + pairwise_sum(x + h, n - h);
}

const double INV8PI3 = 1.0 / (8.0 * PI * PI * PI);

}  // namespace

// ===========================================================================
// extern "C" API used by tests/ (via oracle/oracle.py)
// ===========================================================================
extern "C" {

typedef Object or_object;

int or_max_threads(void) { return omp_get_max_threads(); }
void or_set_threads(int n) { if (n > 0) omp_set_num_threads(n); }

void or_E(double z, double* o) { cd v = E_func(z); o[0] = v.real(); o[1] = v.imag(); }
void or_E_prime(double z, double* o) { cd v = E_prime(z); o[0] = v.real(); o[1] = v.imag(); }
void or_E_double_prime(double z, double* o) { cd v = E_double_prime(z); o[0] = v.real(); o[1] = v.imag(); }
void or_Phi(double a, double b, double* o) { cd v = Phi_ab(a, b); o[0] = v.real(); o[1] = v.imag(); }
void or_Phi_grad(double a, double b, double* o) {
  cd x, y; Phi_ab_grad(a, b, &x, &y);
  o[0] = x.real(); o[1] = x.imag(); o[2] = y.real(); o[3] = y.imag();
}
double or_J1_over_x(double x) { return J1x(x); }
double or_J1_over_x_prime(double x) { return J1x_prime(x); }

// Gauss-Legendre on [a,b] by Newton on P_n (cpp/include/quadrature/gauss_legendre.hpp:16-62)
int or_gauss_legendre(int n, double a, double b, double* x, double* w) {
  if (n <= 0) return 1;
  int m = (n + 1) / 2;
  for (int i = 0; i < m; ++i) {
    double z = std::cos(PI * (i + 0.75) / (n + 0.5)), z1, pp = 0;
    do {
      double p1 = 1.0, p2 = 0.0;
      for (int j = 1; j <= n; ++j) {
        double p3 = p2; p2 = p1;
        p1 = ((2.0 * j - 1.0) * z * p2 - (j - 1.0) * p3) / j;
      }
      pp = n * (z * p1 - p2) / (z * z - 1.0);
      z1 = z;
      z = z1 - p1 / pp;
    } while (std::abs(z - z1) > 1e-14);
    double p1 = 1.0, p2 = 0.0;
    for (int j = 1; j <= n; ++j) {
      double p3 = p2; p2 = p1;
      p1 = ((2.0 * j - 1.0) * z * p2 - (j - 1.0) * p3) / j;
    }
    pp = n * (z * p1 - p2) / (z * z - 1.0);
    double wi = 2.0 / ((1.0 - z * z) * pp * pp);
    double xm = 0.5 * (b + a), xl = 0.5 * (b - a);
    x[i] = xm - xl * z; x[n - 1 - i] = xm + xl * z;
    w[i] = xl * wi; w[n - 1 - i] = xl * wi;
  }
  return 0;
}

// Tensor k-grid, q = ir*M + j, k = tan t, w = w_leb * w_GL * sec^2 t
// (cpp/include/quadrature/kgrid.hpp:17-47)
int or_build_kgrid(const double* ld, const double* lw, int M, int nrad, double* dirs, double* kmag,
                   double* w) {
  std::vector<double> t(nrad), wt(nrad);
  if (or_gauss_legendre(nrad, 0.0, 0.5 * PI, t.data(), wt.data())) return 1;
  for (int ir = 0; ir < nrad; ++ir) {
    double sec2 = 1.0 / std::cos(t[ir]) / std::cos(t[ir]), k = std::tan(t[ir]);
    for (int j = 0; j < M; ++j) {
      int64_t q = (int64_t)ir * M + j;
      dirs[3 * q] = ld[3 * j]; dirs[3 * q + 1] = ld[3 * j + 1]; dirs[3 * q + 2] = ld[3 * j + 2];
      kmag[q] = k;
      w[q] = lw[j] * (wt[ir] * sec2);
    }
  }
  return 0;
}

// Lebedev row (theta_deg, phi_deg) -> direction (cpp/include/quadrature/lebedev_io.hpp:37-43)
void or_lebedev_dir(double theta_deg, double phi_deg, double* d) {
  // theta *= M_PI / 180.0 (lebedev_io.hpp:37-38): the factor is rounded first
  double th = theta_deg * (PI / 180.0), ph = phi_deg * (PI / 180.0);
  d[0] = std::cos(th) * std::sin(ph); d[1] = std::sin(th) * std::sin(ph); d[2] = std::cos(ph);
}

double or_exact_cube_form_factor(double kx, double ky, double kz) {
  auto sinc = [](double x) {
    if (std::abs(x) < 1e-4) return 1.0 - x * x / 6.0 + x * x * x * x / 120.0;
    return std::sin(x) / x;
  };
  return sinc(0.5 * kx) * sinc(0.5 * ky) * sinc(0.5 * kz);
}

double or_exact_sphere_form_factor(double k, double R) {
  if (std::abs(k) < 1e-4) {
    double R3 = R * R * R;
    return 4.0 * PI * R3 / 3.0 * (1.0 - k * k * R * R / 10.0 + k * k * k * k * R * R * R * R / 280.0);
  }
  double kR = k * R;
  return 4.0 * PI * (std::sin(kR) - kR * std::cos(kR)) / (k * k * k);
}

double or_box_box_intersection_volume(const double* c1, const double* h1, const double* c2,
                                      const double* h2) {
  double v = 1.0;
  for (int i = 0; i < 3; ++i) {
    double lo = std::max(c1[i] - h1[i], c2[i] - h2[i]), hi = std::min(c1[i] + h1[i], c2[i] + h2[i]);
    v *= std::max(0.0, hi - lo);
  }
  return v;
}

double or_sphere_sphere_intersection_volume(const double* c1, double r1, const double* c2, double r2) {
  double dx = c2[0] - c1[0], dy = c2[1] - c1[1], dz = c2[2] - c1[2];
  double d = std::sqrt(dx * dx + dy * dy + dz * dz);
  if (d >= r1 + r2) return 0.0;
  if (d <= std::abs(r1 - r2)) { double r = std::min(r1, r2); return 4.0 * PI / 3.0 * r * r * r; }
  double t1 = (r1 + r2 - d) * (r1 + r2 - d);
  double t2 = d * d + 2.0 * d * (r1 + r2) - 3.0 * (r1 * r1 + r2 * r2) + 6.0 * r1 * r2;
  return PI * t1 * t2 / (12.0 * d);
}

// Packing (cpp/src/geometry/packing.cpp:10-112)
void or_pack_tris(const double* V, const int32_t* F, int64_t nf, void* out) {
  Tri* T = static_cast<Tri*>(out);
  for (int64_t i = 0; i < nf; ++i) {
    int ia = F[3 * i], ib = F[3 * i + 1], ic = F[3 * i + 2];
    V3 a = v3(V + 3 * ia), b = v3(V + 3 * ib), c = v3(V + 3 * ic);
    V3 e1 = sub(b, a), e2 = sub(c, a), S = scl(cross(e1, e2), 0.5);
    double* dst[4] = {T[i].a, T[i].e1, T[i].e2, T[i].S};
    V3 src[4] = {a, e1, e2, S};
    for (int j = 0; j < 4; ++j) { dst[j][0] = src[j].x; dst[j][1] = src[j].y; dst[j][2] = src[j].z; }
    T[i].vid0 = ia; T[i].vid1 = ib; T[i].vid2 = ic; T[i].pad = 0;
  }
}

void or_pack_disks(const double* P, const double* N, const double* r, int64_t n, int is_radius, void* out) {
  Disk* D = static_cast<Disk*>(out);
  for (int64_t i = 0; i < n; ++i) {
    V3 nn = v3(N + 3 * i); nn = scl(nn, 1.0 / norm(nn));
    double rho, area;
    if (is_radius) { rho = r[i]; area = PI * rho * rho; } else { area = r[i]; rho = std::sqrt(area / PI); }
    D[i].c[0] = P[3 * i]; D[i].c[1] = P[3 * i + 1]; D[i].c[2] = P[3 * i + 2];
    D[i].n[0] = nn.x; D[i].n[1] = nn.y; D[i].n[2] = nn.z;
    D[i].rho = rho; D[i].area = area;
  }
}

void or_pack_gaussians(const double* P, const double* N, const double* s, const double* w, int64_t n, void* out) {
  Gauss* G = static_cast<Gauss*>(out);
  for (int64_t i = 0; i < n; ++i) {
    V3 nn = v3(N + 3 * i); nn = scl(nn, 1.0 / norm(nn));
    G[i].c[0] = P[3 * i]; G[i].c[1] = P[3 * i + 1]; G[i].c[2] = P[3 * i + 2];
    G[i].n[0] = nn.x; G[i].n[1] = nn.y; G[i].n[2] = nn.z;
    G[i].sigma = s[i]; G[i].w = w[i];
  }
}

// A(k) for an object at nk arbitrary k-vectors; out is nk complex (re,im).
int or_form_factor(const or_object* o, const double* kvecs, int64_t nk, double* out) {
  Prepared p = prepare(*o);
#pragma omp parallel for schedule(static)
  for (int64_t q = 0; q < nk; ++q) {
    cd a = form_factor(p, v3(kvecs + 3 * q));
    out[2 * q] = a.real(); out[2 * q + 1] = a.imag();
  }
  return 0;
}

// dA/d(dofs) at nk k-vectors; out is nk x n_dofs complex, row-major.
int or_form_factor_grad(const or_object* o, const double* kvecs, int64_t nk, double* out) {
  Prepared p = prepare(*o);
  int64_t nd = o->n_dofs;
#pragma omp parallel
  {
    std::vector<cd> g(nd);
#pragma omp for schedule(static)
    for (int64_t q = 0; q < nk; ++q) {
      form_factor_grad(p, v3(kvecs + 3 * q), g.data());
      for (int64_t d = 0; d < nd; ++d) { out[2 * (q * nd + d)] = g[d].real(); out[2 * (q * nd + d) + 1] = g[d].imag(); }
    }
  }
  return 0;
}

// Form-factor matrix J (Q x N complex, row-major q*N+obj) for N objects over a
// k-grid (multi_object.cpp:70-93).  `stride` > 1 evaluates only k-nodes with
// q % stride == 0 (bounded CPU timing samples); other rows are left untouched.
int or_form_factor_matrix(const or_object* objs, int n, const double* dirs, const double* kmag,
                          int64_t Q, int64_t stride, double* J) {
  std::vector<Prepared> P;
  for (int i = 0; i < n; ++i) P.push_back(prepare(objs[i]));
  if (stride < 1) stride = 1;
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t q = 0; q < Q; q += stride) {
    V3 k = {dirs[3 * q] * kmag[q], dirs[3 * q + 1] * kmag[q], dirs[3 * q + 2] * kmag[q]};
    for (int i = 0; i < n; ++i) {
      cd a = form_factor(P[i], k);
      J[2 * (q * n + i)] = a.real(); J[2 * (q * n + i) + 1] = a.imag();
    }
  }
  return 0;
}

// V = Re(J^H diag(w) J) / (8 pi^3) from a precomputed J (multi_object.cpp:100-149),
// fixed-order pairwise sums over q.
int or_contract(const double* J, const double* w, int64_t Q, int n, double* V) {
  int npairs = n * (n + 1) / 2;
#pragma omp parallel
  {
    std::vector<double> term(Q);
#pragma omp for schedule(dynamic, 1)
    for (int idx = 0; idx < npairs; ++idx) {
      int i = 0, rem = idx;
      while (rem >= n - i) { rem -= n - i; ++i; }
      int j = i + rem;
      for (int64_t q = 0; q < Q; ++q) {
        const double* a = J + 2 * (q * n + i);
        const double* b = J + 2 * (q * n + j);
        term[q] = w[q] * (a[0] * b[0] + a[1] * b[1]);
      }
      double v = pairwise_sum(term.data(), Q) * INV8PI3;
      V[i * n + j] = v; V[j * n + i] = v;
    }
  }
  return 0;
}

// Volume matrix with optional gradients and Gauss-Newton cross-Hessians
// (multi_object.cpp:31-292).  grad: packed per (i,j) row-major, block (i,j)
// holds dV_ij/d(theta_i) with n_dofs[i] entries at offset goff[i]*n + j*n_dofs[i]
// -- callers pass a buffer of sum_i n*n_dofs[i] doubles.  hess_ij: for each
// (i,j) a n_dofs[i] x n_dofs[j] block, packed in (i,j) row-major order.
int or_volume_matrix(const or_object* objs, int n, const double* dirs, const double* kmag,
                     const double* w, int64_t Q, int flags, double* V, double* grad, double* hess) {
  std::vector<double> J((size_t)2 * Q * n);
  or_form_factor_matrix(objs, n, dirs, kmag, Q, 1, J.data());
  or_contract(J.data(), w, Q, n, V);
  if (!(flags & (FLAG_GRADIENT | FLAG_HESSIAN))) return 0;
  std::vector<Prepared> P;
  std::vector<int64_t> nd(n), goff(n + 1, 0);
  for (int i = 0; i < n; ++i) { P.push_back(prepare(objs[i])); nd[i] = objs[i].n_dofs; goff[i + 1] = goff[i] + nd[i]; }
  int64_t D = goff[n];
  std::vector<cd> G((size_t)Q * D);  // dA_i/dtheta_i at every q
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t q = 0; q < Q; ++q) {
    V3 k = {dirs[3 * q] * kmag[q], dirs[3 * q + 1] * kmag[q], dirs[3 * q + 2] * kmag[q]};
    for (int i = 0; i < n; ++i) form_factor_grad(P[i], k, &G[(size_t)q * D + goff[i]]);
  }
  if (flags & FLAG_GRADIENT) {
    // grad block (i,j) at offset n*goff[i] + j*nd[i]
#pragma omp parallel
    {
      std::vector<double> term(Q);
#pragma omp for collapse(2) schedule(dynamic, 1)
      for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j)
          for (int64_t d = 0; d < nd[i]; ++d) {
            for (int64_t q = 0; q < Q; ++q) {
              cd g = G[(size_t)q * D + goff[i] + d];
              const double* aj = &J[2 * (q * n + j)];
              term[q] = w[q] * (g.real() * aj[0] + g.imag() * aj[1]);
            }
            grad[n * goff[i] + j * nd[i] + d] = pairwise_sum(term.data(), Q) * INV8PI3;
          }
    }
  }
  if (flags & FLAG_HESSIAN) {
    std::vector<int64_t> hoff((size_t)n * n + 1, 0);
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) hoff[i * n + j + 1] = hoff[i * n + j] + nd[i] * nd[j];
#pragma omp parallel
    {
      std::vector<double> term(Q);
#pragma omp for collapse(2) schedule(dynamic, 1)
      for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j)
          for (int64_t a = 0; a < nd[i]; ++a)
            for (int64_t b = 0; b < nd[j]; ++b) {
              for (int64_t q = 0; q < Q; ++q) {
                cd gi = G[(size_t)q * D + goff[i] + a], gj = G[(size_t)q * D + goff[j] + b];
                term[q] = w[q] * (gi.real() * gj.real() + gi.imag() * gj.imag());
              }
              hess[hoff[i * n + j] + a * nd[j] + b] = pairwise_sum(term.data(), Q) * INV8PI3;
            }
    }
  }
  return 0;
}

// Pair volume with gradients and Gauss-Newton Hessian blocks
// (compute_intersection_volume_cpu.cpp:21-186).  H11 is d1 x d1, H22 d2 x d2, H12 d1 x d2.
int or_pair_volume(const or_object* o1, const or_object* o2, const double* dirs, const double* kmag,
                   const double* w, int64_t Q, int flags, double* vol, double* g1, double* g2,
                   double* H11, double* H22, double* H12) {
  Prepared p1 = prepare(*o1), p2 = prepare(*o2);
  int64_t d1 = o1->n_dofs, d2 = o2->n_dofs;
  bool need_g = flags & (FLAG_GRADIENT | FLAG_HESSIAN);
  std::vector<cd> A1(Q), A2(Q), G1, G2;
  if (need_g) { G1.resize((size_t)Q * d1); G2.resize((size_t)Q * d2); }
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t q = 0; q < Q; ++q) {
    V3 k = {dirs[3 * q] * kmag[q], dirs[3 * q + 1] * kmag[q], dirs[3 * q + 2] * kmag[q]};
    A1[q] = form_factor(p1, k);
    A2[q] = form_factor(p2, k);
    if (need_g) { form_factor_grad(p1, k, &G1[(size_t)q * d1]); form_factor_grad(p2, k, &G2[(size_t)q * d2]); }
  }
  std::vector<double> term(Q);
  for (int64_t q = 0; q < Q; ++q) term[q] = w[q] * (A1[q].real() * A2[q].real() + A1[q].imag() * A2[q].imag());
  *vol = pairwise_sum(term.data(), Q) * INV8PI3;
  if (flags & FLAG_GRADIENT) {
    for (int64_t d = 0; d < d1; ++d) {
      for (int64_t q = 0; q < Q; ++q) { cd g = G1[q * d1 + d]; term[q] = w[q] * (g.real() * A2[q].real() + g.imag() * A2[q].imag()); }
      g1[d] = pairwise_sum(term.data(), Q) * INV8PI3;
    }
    for (int64_t d = 0; d < d2; ++d) {
      for (int64_t q = 0; q < Q; ++q) { cd g = G2[q * d2 + d]; term[q] = w[q] * (A1[q].real() * g.real() + A1[q].imag() * g.imag()); }
      g2[d] = pairwise_sum(term.data(), Q) * INV8PI3;
    }
  }
  if (flags & FLAG_HESSIAN) {
    auto gn = [&](const std::vector<cd>& Ga, int64_t da, const std::vector<cd>& Gb, int64_t db, double* H) {
#pragma omp parallel
      {
        std::vector<double> t(Q);
#pragma omp for collapse(2)
        for (int64_t a = 0; a < da; ++a)
          for (int64_t b = 0; b < db; ++b) {
            for (int64_t q = 0; q < Q; ++q) {
              cd x = Ga[q * da + a], y = Gb[q * db + b];
              t[q] = w[q] * (x.real() * y.real() + x.imag() * y.imag());
            }
            H[a * db + b] = pairwise_sum(t.data(), Q) * INV8PI3;
          }
      }
    };
    gn(G1, d1, G1, d1, H11);
    gn(G2, d2, G2, d2, H22);
    gn(G1, d1, G2, d2, H12);
  }
  return 0;
}

// Divergence-theorem self-volume through the DoF (affine_dof.cpp:324-384,
// triangle_mesh_dof.cpp:145-179).
double or_self_volume(const or_object* o) {
  if (o->dof_type == DOF_TRIANGLE_MESH) {
    const Tri* T = static_cast<const Tri*>(o->elems);
    double s = 0;
    for (int64_t f = 0; f < o->n_elems; ++f) {
      if (T[f].vid0 < 0 || T[f].vid1 < 0 || T[f].vid2 < 0) continue;
      V3 a = v3(o->dofs + 3 * T[f].vid0), b = v3(o->dofs + 3 * T[f].vid1), c = v3(o->dofs + 3 * T[f].vid2);
      s += dot(a, cross(b, c));
    }
    return s / 6.0;
  }
  M3 A; V3 t; affine_of(o->dofs, &A, &t);
  double vb = 0;
  if (o->geom_type == GEOM_TRIANGLE) {
    const Tri* T = static_cast<const Tri*>(o->elems);
    for (int64_t i = 0; i < o->n_elems; ++i) vb += dot(v3(T[i].a), v3(T[i].S));
  } else if (o->geom_type == GEOM_DISK) {
    const Disk* D = static_cast<const Disk*>(o->elems);
    for (int64_t i = 0; i < o->n_elems; ++i) vb += dot(v3(D[i].c), v3(D[i].n)) * D[i].area;
  } else {
    const Gauss* G = static_cast<const Gauss*>(o->elems);
    for (int64_t i = 0; i < o->n_elems; ++i) vb += dot(v3(G[i].c), v3(G[i].n)) * G[i].w;
  }
  return vb / 3.0 * std::abs(det3(A));
}

// Per-element adjoint for disks / Gaussians at identity DoFs (no reference
// counterpart): for L = sum_ij C_ij V_ij, returns dL/dc (3), dL/dn (3) per
// element of every object, packed object after object.  Disk/Gaussian
// element formulas restate form_factor_helpers.cpp:45-87.
int or_surfel_param_grad(const or_object* objs, int n, const double* dirs, const double* kmag,
                         const double* w, int64_t Q, const double* C, double* gpos, double* gnrm) {
  std::vector<double> J((size_t)2 * Q * n);
  or_form_factor_matrix(objs, n, dirs, kmag, Q, 1, J.data());
  int64_t off = 0;
  for (int m = 0; m < n; ++m) {
    const or_object& o = objs[m];
    if (o.geom_type == GEOM_TRIANGLE) return 2;
    // cotangent B_m(q) = sum_j (C_mj + C_jm) A_j(q)
    std::vector<cd> B(Q);
    for (int64_t q = 0; q < Q; ++q) {
      cd s(0, 0);
      for (int j = 0; j < n; ++j) s += (C[m * n + j] + C[j * n + m]) * cd(J[2 * (q * n + j)], J[2 * (q * n + j) + 1]);
      B[q] = s;
    }
#pragma omp parallel
    {
      std::vector<double> t[6];
      for (auto& v : t) v.resize(Q);
#pragma omp for schedule(dynamic, 8)
      for (int64_t e = 0; e < o.n_elems; ++e) {
        V3 c, nn; double p0, p1;
        if (o.geom_type == GEOM_DISK) {
          const Disk& d = static_cast<const Disk*>(o.elems)[e];
          c = v3(d.c); nn = v3(d.n); p0 = d.rho; p1 = d.area;
        } else {
          const Gauss& g = static_cast<const Gauss*>(o.elems)[e];
          c = v3(g.c); nn = v3(g.n); p0 = g.sigma; p1 = g.w;
        }
        for (int64_t q = 0; q < Q; ++q) {
          V3 k = {dirs[3 * q] * kmag[q], dirs[3 * q + 1] * kmag[q], dirs[3 * q + 2] * kmag[q]};
          double km = norm(k);
          if (km < 1e-10) { for (auto& v : t) v[q] = 0; continue; }
          double kn = dot(k, nn), kk = dot(k, k);
          cd ph = std::exp(dot(k, c) * I1);
          double Sm, dSdn_coef;  // dS/d(kn) through r
          if (o.geom_type == GEOM_DISK) {
            double r = std::sqrt(std::max(0.0, kk - kn * kn)), rr = p0 * r;
            Sm = (rr < 1e-10) ? p1 : 2.0 * p1 * J1x(rr);
            // dS/dn = (dS/dr) dr/dn with dr/dn = -kn k / r; (dS/dr)/r -> -rho^2 area/4 as r -> 0
            double dSr_over_r = (rr < 1e-10) ? -0.25 * p0 * p0 * p1 : 2.0 * p1 * p0 * J1x_prime(rr) / r;
            dSdn_coef = -dSr_over_r * kn;
          } else {
            double r2 = std::max(0.0, kk - kn * kn);
            Sm = p1 * std::exp(-0.5 * p0 * p0 * r2);
            dSdn_coef = p0 * p0 * Sm * kn;  // d/dn of exp(-s^2 (kk-kn^2)/2) = s^2 kn k * S
          }
          cd Ae = ph * (Sm * kn / km);
          double wr = w[q] * INV8PI3;
          cd cb = std::conj(B[q]);
          // dA/dc = i k A
          double gc = wr * (I1 * Ae * cb).real();
          // dA/dn = ph/|k| * (S k + kn * dSdn_coef k)
          double gn = wr * (ph * cb).real() * (Sm + kn * dSdn_coef) / km;
          double kv[3] = {k.x, k.y, k.z};
          for (int a = 0; a < 3; ++a) { t[a][q] = gc * kv[a]; t[3 + a][q] = gn * kv[a]; }
        }
        for (int a = 0; a < 3; ++a) {
          gpos[3 * (off + e) + a] = pairwise_sum(t[a].data(), Q);
          gnrm[3 * (off + e) + a] = pairwise_sum(t[3 + a].data(), Q);
        }
      }
    }
    off += o.n_elems;
  }
  return 0;
}

}  // extern "C"
