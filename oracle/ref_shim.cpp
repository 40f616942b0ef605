// TEST INFRASTRUCTURE ONLY: a C-ABI shim over the parts of the reference that
// compile standalone -- cpp/src/element_functions.cpp (needs only <complex>)
// and the header-only quadrature (cpp/include/quadrature/*.hpp).  It is built
// by oracle/build_ref.sh against the reference sources where they lie and is
// used only to pin the oracle restatement (tests/golden/make_golden.py and the
// oracle tests).  Nothing from here ships.
#include <complex>
#include <cstdint>
#include <cstring>
#include <string>
#include "element_functions.hpp"
#include "quadrature/gauss_legendre.hpp"
#include "quadrature/kgrid.hpp"
#include "quadrature/lebedev_io.hpp"

using namespace PoIntInt;

extern "C" {

static void put(const std::complex<double>& v, double* o) { o[0] = v.real(); o[1] = v.imag(); }

void ref_E(double z, double* o) { put(Triangle_E_func(z), o); }
void ref_E_prime(double z, double* o) { put(Triangle_E_prime(z), o); }
void ref_E_double_prime(double z, double* o) { put(Triangle_E_double_prime(z), o); }
void ref_Phi(double a, double b, double* o) { put(Triangle_Phi_ab(a, b), o); }
void ref_Phi_grad(double a, double b, double* o) {
  auto g = Triangle_Phi_ab_gradient(a, b);
  put(g.first, o);
  put(g.second, o + 2);
}
double ref_J1_over_x(double x) { return Disk_J1_over_x(x); }
double ref_J1_over_x_prime(double x) { return Disk_J1_over_x_prime(x); }

int ref_gauss_legendre(int n, double a, double b, double* x, double* w) {
  auto r = gauss_legendre_interval(n, a, b);
  std::memcpy(x, r.first.data(), sizeof(double) * n);
  std::memcpy(w, r.second.data(), sizeof(double) * n);
  return 0;
}

// Loads a Lebedev file and returns the number of rows; fills up to cap rows.
int64_t ref_load_lebedev(const char* path, double* dirs, double* w, int64_t cap) {
  LebedevGrid L = load_lebedev_txt(std::string(path));
  int64_t n = (int64_t)L.dirs.size();
  for (int64_t i = 0; i < n && i < cap; ++i) {
    dirs[3 * i] = L.dirs[i][0]; dirs[3 * i + 1] = L.dirs[i][1]; dirs[3 * i + 2] = L.dirs[i][2];
    w[i] = L.weights[i];
  }
  return n;
}

// build_kgrid from Lebedev arrays; outputs Q = M * nrad nodes.
int ref_build_kgrid(const double* ld, const double* lw, int64_t M, int nrad, double* dirs, double* kmag,
                    double* w) {
  std::vector<std::array<double, 3>> d(M);
  std::vector<double> wl(lw, lw + M);
  for (int64_t j = 0; j < M; ++j) d[j] = {ld[3 * j], ld[3 * j + 1], ld[3 * j + 2]};
  KGrid K = build_kgrid(d, wl, nrad);
  for (size_t q = 0; q < K.kmag.size(); ++q) {
    dirs[3 * q] = K.dirs[q][0]; dirs[3 * q + 1] = K.dirs[q][1]; dirs[3 * q + 2] = K.dirs[q][2];
    kmag[q] = K.kmag[q];
    w[q] = K.w[q];
  }
  return 0;
}

}  // extern "C"
