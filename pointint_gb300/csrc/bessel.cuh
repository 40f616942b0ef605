// FP32 Bessel ratios for the oriented-disk form factor:
//   j1x(x)  = J1(x)/x      (the disk's 2 area J1(rho r)/(rho r), reference
//                           Disk_J1_over_x, cpp/src/element_functions.cpp:100-109)
//   j2x2(x) = J2(x)/x^2    (-(J1(x)/x)'/x, for the disk's gradient,
//                           reference Disk_J1_over_x_prime, :111-120)
//
// Coefficients are this project's own least-squares fits (numpy Chebyshev /
// polynomial fits against scipy's J1, J2, Y1, Y2, 4e5 samples), except below 1:
//  * 0 <= x < 1: the power series in y = x^2/4 (J1(x)/x = 1/2 sum_m (-y)^m /
//    (m! (m+1)!), J2(x)/x^2 = 1/4 sum_m (-y)^m / (m! (m+2)!)) cut after m = 5,
//    relative truncation below 8e-11 (scipy, 2e5 points): five FMAs where the
//    Chebyshev sum takes 22 instructions.  Most disk x k evaluations of a
//    surfel cloud have x = k rho |k'_perp| / |k| < 1;
//  * 1 <= x < 8: Chebyshev series in u = 2 (x/8)^2 - 1 (the ratios are even,
//    entire functions), degree 11, summed by Clenshaw's recurrence, which is
//    stable in FP32 (max abs error 1.5e-7 for J1/x, 3e-8 for J2/x^2);
//  * x >= 8: the Hankel modulus/phase form
//      J_nu(x) = sqrt(2/(pi x)) (P_nu cos chi - Q_nu sin chi),
//      chi = x - (nu/2 + 1/4) pi,
//    with P_nu and (x/8) Q_nu fitted as degree-6 polynomials in s = (8/x)^2
//    (fit error < 2e-10); chi is reduced in double-float.
// CUDA's j1f carries up to 2.2e-6 absolute error for x >= 8, correlated across
// a cloud of similar disks, which is why it is not used here.
#pragma once
#include "dfmath.cuh"

namespace pi {

__device__ __forceinline__ float clenshaw12(const float* c, float u) {
  float b1 = 0.f, b2 = 0.f;
  const float u2 = u + u;
#pragma unroll
  for (int k = 11; k >= 1; --k) {
    const float b0 = fmaf(u2, b1, c[k] - b2);
    b2 = b1;
    b1 = b0;
  }
  return fmaf(u, b1, c[0] - b2);
}

__device__ __forceinline__ float horner7(const float* c, float s) {
  return fmaf(s, fmaf(s, fmaf(s, fmaf(s, fmaf(s, fmaf(s, c[6], c[5]), c[4]), c[3]), c[2]), c[1]), c[0]);
}

// J_nu(x) sqrt(x) for x >= 8 (nu = 1 or 2): sqrt(2/pi) (P cos chi - Q sin chi).
__device__ __forceinline__ float hankel_scaled(float x, const float* P, const float* Q, float phase_hi,
                                               float phase_lo) {
  const float ix = rcp_fast(x);
  const float s = 64.0f * ix * ix;
  const float p = horner7(P, s);
  const float q = horner7(Q, s) * 8.0f * ix;
  const df chi = df_add(df{x, 0.f}, df{-phase_hi, -phase_lo});
  const cf e = cis(chi);
  return 0.79788456080286536f * (p * e.re - q * e.im);  // sqrt(2/pi)
}

__device__ __forceinline__ float j1x(float x) {
  const float c[12] = {8.104484528e-02f, -1.489751488e-01f, 1.609992683e-01f, -8.268049359e-02f,
                       2.221363969e-02f, -3.646940691e-03f, 4.050337593e-04f, -3.255554839e-05f,
                       1.985876452e-06f, -9.522089073e-08f, 3.685906469e-09f, -1.194069843e-10f};
  const float P[7] = {1.000000000e+00f, 1.831054571e-03f, -3.520296377e-05f, 2.574856353e-06f,
                      -3.913895057e-07f, 7.990912110e-08f, -1.163217167e-08f};
  const float Q[7] = {4.687500000e-02f, -2.002715482e-04f, 8.470226021e-06f, -9.461746231e-07f,
                      1.892280608e-07f, -4.536089548e-08f, 7.152803683e-09f};
  if (x < 1.0f) {
    const float y = 0.25f * x * x;
    return fmaf(y, fmaf(y, fmaf(y, fmaf(y, fmaf(y, -1.0f / 172800.0f, 1.0f / 5760.0f), -1.0f / 288.0f),
                                1.0f / 24.0f), -0.25f), 0.5f);
  }
  if (x < 8.0f) return clenshaw12(c, fmaf(x * x, 2.0f / 64.0f, -1.0f));
  // 3 pi / 4 = 2.35619449019234492885 -> FP32 hi + lo
  return hankel_scaled(x, P, Q, 2.356194496154785f, -5.962440319e-09f) * rsqrtf(x) * rcp_fast(x);
}

__device__ __forceinline__ float j2x2(float x) {
  const float c[12] = {2.596750483e-02f, -5.166240036e-02f, 3.331311420e-02f, -1.141258609e-02f,
                       2.307931194e-03f, -3.057658323e-04f, 2.859338929e-05f, -1.990491000e-06f,
                       1.072843929e-07f, -4.613698756e-09f, 1.620504286e-10f, -4.802348189e-12f};
  const float P[7] = {1.000000000e+00f, -1.281738281e-02f, 7.744745380e-05f, -4.293725397e-06f,
                      5.753120718e-07f, -1.105211496e-07f, 1.565981123e-08f};
  const float Q[7] = {2.343750000e-01f, 6.008147611e-04f, -1.573086774e-05f, 1.463545800e-06f,
                      -2.668556647e-07f, 6.115627116e-08f, -9.458235084e-09f};
  if (x < 1.0f) {
    const float y = 0.25f * x * x;
    return fmaf(y, fmaf(y, fmaf(y, fmaf(y, fmaf(y, -1.0f / 2419200.0f, 1.0f / 69120.0f), -1.0f / 2880.0f),
                                1.0f / 192.0f), -1.0f / 24.0f), 0.125f);
  }
  if (x < 8.0f) return clenshaw12(c, fmaf(x * x, 2.0f / 64.0f, -1.0f));
  // 5 pi / 4 = 3.92699081698724154808 -> FP32 hi + lo
  const float ix = rcp_fast(x);
  return hankel_scaled(x, P, Q, 3.9269907474517822f, 6.953546006e-08f) * rsqrtf(x) * ix * ix;
}

}  // namespace pi
