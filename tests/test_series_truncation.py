"""The small-spread series the CUDA kernels evaluate, against exact divided
differences of e^{iz} (mpmath, 40 digits), on random triangles.

For centred vertex phases x = k (d_a, d_b, d_c) (d_a + d_b + d_c = 0) the
triangle's e[x_a, x_b, x_c] = sum_m i^{m+2} h_m(x) / (m+2)!, and the vertex
derivative pieces e[x_a, x_b, x_b, x_c] = sum_m i^{m+3} h_m(x, x_b) / (m+3)!,
with h_m the complete homogeneous symmetric polynomials.  The kernels take
  * the form factor series to h_13 for k sp < 3 (sp = the largest |k.e|),
    and to h_7 (a[0..3], b[0..2]) where k |e|max < 1 (|e|max = longest edge);
  * the derivative series to h_12 for k sp < 2, and to h_8 where k |e|max < 1.
Each cut must stay well below FP32 rounding of the leading term (6e-8)."""
import math

import numpy as np
import pytest

mp = pytest.importorskip("mpmath")
mp.mp.dps = 40


def random_cases(n, seed):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        e1 = rng.normal(size=3) * rng.uniform(0.05, 2.0)
        e2 = e1 * rng.uniform(-1.0, 1.0) + rng.normal(size=3) * rng.uniform(0.02, 2.0)  # thin and fat shapes
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        out.append((e1, e2, d))
    return out


def centred(e1, e2, d):
    s1, s2 = float(d @ e1), float(d @ e2)
    da = -(s1 + s2) / 3.0
    return (da, da + s1, da + s2), max(abs(s1), abs(s2), abs(s2 - s1)), \
        max(np.linalg.norm(e1), np.linalg.norm(e2), np.linalg.norm(e2 - e1))


def hseries(dv):
    """h_0..h_13 of the centred dots: the recurrence the kernels use."""
    da, db, dc = dv
    mu = 0.5 * (da * da + db * db + dc * dc)
    nu = da * db * dc
    h = [1.0, 0.0, mu, nu]
    for m in range(4, 14):
        h.append(mu * h[m - 2] + nu * h[m - 3])
    return h


def series_F(dv, k, top):
    h = hseries(dv)
    return sum((1j) ** (m + 2) * k ** m * h[m] / math.factorial(m + 2) for m in range(top + 1))


def series_Db(dv, k, top):
    h = hseries(dv)
    hb, s = 1.0, 0.0
    for m in range(top + 1):
        if m > 0:
            hb = dv[1] * hb + h[m]
        s += (1j) ** (m + 3) * k ** m * hb / math.factorial(m + 3)
    return s


def exact_F(dv, k):
    f = lambda z: mp.expj(z)
    xa, xb, xc = (mp.mpf(k) * mp.mpf(v) for v in dv)
    fab = (f(xb) - f(xa)) / (xb - xa)
    fbc = (f(xc) - f(xb)) / (xc - xb)
    return complex((fbc - fab) / (xc - xa))


def exact_Db(dv, k):
    f = lambda z: mp.expj(z)
    xa, xb, xc = (mp.mpf(k) * mp.mpf(v) for v in dv)
    fbb = 1j * f(xb)
    fab = (f(xb) - f(xa)) / (xb - xa)
    fbc = (f(xc) - f(xb)) / (xc - xb)
    fabb = (fbb - fab) / (xb - xa)
    fbbc = (fbc - fbb) / (xc - xb)
    return complex((fbbc - fabb) / (xc - xa))


@pytest.mark.parametrize("seed", [0, 1])
def test_series_cuts_against_exact_divided_differences(seed):
    worst = {"F13": 0.0, "F7": 0.0, "Db12": 0.0, "Db8": 0.0}
    rng = np.random.default_rng(100 + seed)
    for e1, e2, d in random_cases(150, seed):
        dv, sp, lmax = centred(e1, e2, d)
        if min(abs(dv[0] - dv[1]), abs(dv[1] - dv[2]), abs(dv[0] - dv[2])) < 1e-6 * sp:
            continue  # near-coincident nodes: the exact quotient form loses digits
        u = rng.uniform(0.3, 1.0)
        k_f = 3.0 / sp * u  # k sp up to the form factor series' threshold 3
        k_d = 2.0 / sp * u  # k sp up to the derivative series' threshold 2
        k_short = 1.0 / lmax * rng.uniform(0.3, 1.0)  # k |e|max up to the short-series bound 1
        # leading terms: i^2 / 2! for F, i^3 / 3! for D_b
        worst["F13"] = max(worst["F13"], abs(series_F(dv, k_f, 13) - exact_F(dv, k_f)) / 0.5)
        worst["Db12"] = max(worst["Db12"], abs(series_Db(dv, k_d, 12) - exact_Db(dv, k_d)) * 6.0)
        worst["F7"] = max(worst["F7"], abs(series_F(dv, k_short, 7) - exact_F(dv, k_short)) / 0.5)
        worst["Db8"] = max(worst["Db8"], abs(series_Db(dv, k_short, 8) - exact_Db(dv, k_short)) * 6.0)
    print("\nseries truncation, worst relative to the leading term:",
          {k: f"{v:.2e}" for k, v in worst.items()})
    for key, v in worst.items():
        assert v < 2e-8, (key, v)
