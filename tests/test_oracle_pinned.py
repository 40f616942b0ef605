"""Pins the FP64 oracle (and the native host quadrature) to the reference's own
arithmetic: golden vectors produced by the reference's element_functions.cpp and
quadrature headers (tests/golden/make_golden.py), and, where the reference
sources are present, the live reference build in oracle/_ref."""
import os

import numpy as np
import pytest

import pointint_gb300 as pg
from pointint_gb300 import kgrid as pkg

RTOL = 1e-13


def _cplx(fn, z):
    return np.array([[v.real, v.imag] for v in (fn(x) for x in z)])


def test_element_functions_match_golden(orc, golden):
    z = golden["z"]
    np.testing.assert_allclose(_cplx(orc.E_func, z), golden["E"], rtol=RTOL, atol=1e-15)
    np.testing.assert_allclose(_cplx(orc.E_prime, z), golden["Ep"], rtol=RTOL, atol=1e-15)
    np.testing.assert_allclose(_cplx(orc.E_double_prime, z), golden["Epp"], rtol=RTOL, atol=1e-15)


def test_phi_and_gradient_match_golden(orc, golden):
    ab = golden["ab"]
    phi = np.array([[v.real, v.imag] for v in (orc.Phi(a, b) for a, b in ab)])
    np.testing.assert_allclose(phi, golden["Phi"], rtol=RTOL, atol=1e-14)
    dphi = []
    for a, b in ab:
        x, y = orc.Phi_grad(a, b)
        dphi.append([x.real, x.imag, y.real, y.imag])
    np.testing.assert_allclose(np.array(dphi), golden["dPhi"], rtol=1e-12, atol=1e-13)


def test_bessel_match_golden(orc, golden):
    x = golden["x"]
    np.testing.assert_allclose([orc.J1_over_x(v) for v in x], golden["J1x"], rtol=RTOL, atol=1e-16)
    np.testing.assert_allclose([orc.J1_over_x_prime(v) for v in x], golden["J1xp"], rtol=RTOL, atol=1e-16)


@pytest.mark.parametrize("n", [1, 2, 3, 16, 32, 64, 128])
def test_gauss_legendre_oracle_and_native_match_golden(orc, golden, n):
    xo, wo = orc.gauss_legendre(n, 0.0, 0.5 * np.pi)
    xn, wn = pkg.gauss_legendre(n, 0.0, 0.5 * np.pi)
    for x, w in ((xo, wo), (xn, wn)):
        np.testing.assert_allclose(x, golden[f"gl{n}_x"], rtol=1e-14, atol=1e-15)
        np.testing.assert_allclose(w, golden[f"gl{n}_w"], rtol=1e-13, atol=1e-15)


@pytest.mark.parametrize("order", [3, 9, 29])
def test_lebedev_loading_matches_golden(orc, golden, order):
    path = pkg.lebedev_path(order)
    d, w = pkg.load_lebedev(path)
    np.testing.assert_allclose(d, golden[f"leb{order}_dirs"], rtol=0, atol=1e-15)
    np.testing.assert_allclose(w, golden[f"leb{order}_w"], rtol=1e-15)
    d2, w2 = orc.load_lebedev(path)
    np.testing.assert_allclose(d2, golden[f"leb{order}_dirs"], rtol=0, atol=1e-15)
    np.testing.assert_allclose(w2, golden[f"leb{order}_w"], rtol=1e-15)
    assert abs(w.sum() - 4 * np.pi) < 1e-9


def test_kgrid_matches_golden(orc, golden):
    d, w = golden["leb9_dirs"], golden["leb9_w"]
    kg = pkg.build_kgrid(d, w, 16)
    np.testing.assert_allclose(kg.dirs, golden["kg9_16_dirs"], rtol=0, atol=0)
    np.testing.assert_allclose(kg.kmag, golden["kg9_16_kmag"], rtol=1e-14)
    np.testing.assert_allclose(kg.w, golden["kg9_16_w"], rtol=1e-13)
    od, ok, ow = orc.build_kgrid(d, w, 16)
    np.testing.assert_allclose(ok, golden["kg9_16_kmag"], rtol=1e-14)
    np.testing.assert_allclose(ow, golden["kg9_16_w"], rtol=1e-13)


def test_oracle_matches_live_reference_build(orc):
    """Denser sweep against the reference compiled from its sources (oracle/_ref)."""
    R = orc.ref_lib()
    if R is None:
        pytest.skip("oracle/_ref not built (reference sources absent)")
    rng = np.random.default_rng(3)
    for a, b in rng.uniform(-50, 50, size=(300, 2)).tolist() + [(x, x + d) for x in (0.2, 9.0) for d in
                                                                 np.geomspace(1e-9, 1e-2, 25)]:
        buf = np.zeros(2)
        R.ref_Phi(a, b, buf.ctypes.data)
        v = orc.Phi(a, b)
        assert abs(v.real - buf[0]) <= 1e-13 * (1 + abs(buf[0])) and abs(v.imag - buf[1]) <= 1e-13 * (1 + abs(buf[1]))
    for x in np.geomspace(1e-8, 80, 200):
        assert abs(orc.J1_over_x(x) - R.ref_J1_over_x(x)) <= 1e-14
        assert abs(orc.J1_over_x_prime(x) - R.ref_J1_over_x_prime(x)) <= 1e-14
