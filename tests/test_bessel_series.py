"""The disk kernels' J1(x)/x and J2(x)/x^2 ratios below x = 1 (bessel.cuh: j1x,
j2x2), emulated in FP32 on the host and held against scipy in FP64.

Below 1 both are the power series in y = x^2/4 cut after m = 5:
  J1(x)/x   = 1/2 sum_m (-y)^m / (m! (m+1)!),
  J2(x)/x^2 = 1/4 sum_m (-y)^m / (m! (m+2)!),
evaluated by Horner's rule with FMAs (emulated exactly: the product of two
FP32 values is exact in FP64).  The bound, 2e-7 relative, is FP32 rounding of
a Horner sum of six terms; the series' truncation is below 8e-11.  At x = 1
the series meets the Chebyshev fit used from 1 to 8 within that fit's
1.5e-7 absolute error.
"""
from math import factorial

import numpy as np
import pytest

sp = pytest.importorskip("scipy.special")
f32 = np.float32


def fma(a, b, c):
    return f32(np.float64(a) * np.float64(b) + np.float64(c))


# the constants as written in bessel.cuh (1.0f / n rounded to FP32)
J1X = [f32(0.5), f32(-0.25), f32(1.0 / 24.0), f32(-1.0 / 288.0), f32(1.0 / 5760.0), f32(-1.0 / 172800.0)]
J2X2 = [f32(0.125), f32(-1.0 / 24.0), f32(1.0 / 192.0), f32(-1.0 / 2880.0), f32(1.0 / 69120.0), f32(-1.0 / 2419200.0)]


def horner(c, x):
    x = f32(x)
    y = f32(f32(f32(0.25) * x) * x)
    r = c[-1]
    for a in reversed(c[:-1]):
        r = fma(y, r, a)
    return r


def test_coefficients_are_the_series():
    for m in range(6):
        assert J1X[m] == f32(0.5 * (-1) ** m / (factorial(m) * factorial(m + 1)))
        assert J2X2[m] == f32(0.25 * (-1) ** m / (factorial(m) * factorial(m + 2)))


@pytest.mark.parametrize("name", ["j1x", "j2x2"])
def test_series_below_one_against_scipy(name):
    xs = np.concatenate([np.linspace(0.0, 1.0, 20001)[1:], 10 ** np.linspace(-8, 0, 2001)[:-1]])
    c, ref = (J1X, sp.j1(xs) / xs) if name == "j1x" else (J2X2, sp.jv(2, xs) / xs ** 2)
    got = np.array([horner(c, x) for x in xs], dtype=np.float64)
    err = np.max(np.abs(got - ref) / np.abs(ref))
    print(f"\n{name}: FP32 series below 1, worst relative error {err:.2e}")
    assert err < 2e-7
    # at the switch to the Chebyshev fit (absolute error 1.5e-7 for J1/x, 3e-8 for J2/x^2)
    assert abs(horner(c, 1.0) - (sp.j1(1.0) if name == "j1x" else sp.jv(2, 1.0))) < 1e-7
