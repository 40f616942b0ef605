"""Generates tests/golden/ref_golden.npz from the reference's own sources.

Run in a checkout where the reference is present (it builds oracle/_ref from
the reference's cpp/src/element_functions.cpp and header-only quadrature via
oracle/build_ref.sh):

    python tests/golden/make_golden.py

The fixtures pin the FP64 oracle restatement (oracle/oracle.cpp) and the
native library's host quadrature to the reference's arithmetic: element
functions E, E', E'', Phi, dPhi, J1(x)/x, (J1(x)/x)' at points chosen around
each branch threshold, Gauss-Legendre rules, Lebedev loading, and a small
k-grid.  The reference has no golden-vector files of its own.
"""
from __future__ import annotations

import ctypes
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle  # noqa: E402  (test infrastructure)

REF_DATA = os.environ.get("POINTINT_REF_DIR", "/root/reference") + "/data/lebedev"
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "ref_golden.npz")


def z_points() -> np.ndarray:
    base = [0.0, 1e-9, 3e-6, 5e-5, 9.99e-5, 1.0e-4, 1.01e-4, 3e-4, 1e-3, 0.01, 0.1, 0.5, 1.0, 2.0, 3.14159,
            5.0, 10.0, 33.3, 100.0, 1234.5, 5e4]
    return np.array(sorted(set(base + [-x for x in base])))


def ab_points() -> np.ndarray:
    rng = np.random.default_rng(7)
    pts = []
    for a in [0.0, 1e-5, 0.3, -2.0, 7.5, 150.0]:
        for d in [0.0, 1e-7, 5e-4, 9.99e-4, 1.0e-3, 1.01e-3, 2e-3, 0.1, 1.0, 10.0, -0.5]:
            pts.append((a, a + d))
    pts += [tuple(x) for x in rng.uniform(-20, 20, size=(40, 2))]
    return np.array(pts)


def x_points() -> np.ndarray:
    return np.array([0.0, 1e-12, 1e-6, 9.99e-6, 1.0e-5, 1.01e-5, 1e-3, 0.1, 0.5, 1.0, 2.5, 5.0, 7.99, 8.0, 12.0,
                     12.01, 20.0, 47.3, 100.0])


def main() -> None:
    ref_path = oracle.build_ref()
    if ref_path is None:
        raise SystemExit("reference sources not present; cannot regenerate golden vectors")
    R = oracle.ref_lib()
    out = {}
    z = z_points()
    for name, fn in (("E", R.ref_E), ("Ep", R.ref_E_prime), ("Epp", R.ref_E_double_prime)):
        vals = np.zeros((len(z), 2))
        for i, zz in enumerate(z):
            buf = np.zeros(2)
            fn(float(zz), buf.ctypes.data)
            vals[i] = buf
        out[name] = vals
    out["z"] = z
    ab = ab_points()
    phi, dphi = np.zeros((len(ab), 2)), np.zeros((len(ab), 4))
    for i, (a, b) in enumerate(ab):
        b1, b2 = np.zeros(2), np.zeros(4)
        R.ref_Phi(float(a), float(b), b1.ctypes.data)
        R.ref_Phi_grad(float(a), float(b), b2.ctypes.data)
        phi[i], dphi[i] = b1, b2
    out["ab"], out["Phi"], out["dPhi"] = ab, phi, dphi
    x = x_points()
    out["x"] = x
    out["J1x"] = np.array([R.ref_J1_over_x(float(v)) for v in x])
    out["J1xp"] = np.array([R.ref_J1_over_x_prime(float(v)) for v in x])
    for n in (1, 2, 3, 16, 32, 64, 128):
        xs, ws = np.zeros(n), np.zeros(n)
        R.ref_gauss_legendre(n, 0.0, 0.5 * np.pi, xs.ctypes.data, ws.ctypes.data)
        out[f"gl{n}_x"], out[f"gl{n}_w"] = xs, ws
    for order in (3, 9, 29):
        path = f"{REF_DATA}/lebedev_{order:03d}.txt".encode()
        n = R.ref_load_lebedev(path, None, None, 0)
        d, w = np.zeros((n, 3)), np.zeros(n)
        R.ref_load_lebedev(path, d.ctypes.data, w.ctypes.data, n)
        out[f"leb{order}_dirs"], out[f"leb{order}_w"] = d, w
    d9, w9 = out["leb9_dirs"], out["leb9_w"]
    Q = len(w9) * 16
    kd, km, kw = np.zeros((Q, 3)), np.zeros(Q), np.zeros(Q)
    R.ref_build_kgrid(d9.ctypes.data, w9.ctypes.data, len(w9), 16, kd.ctypes.data, km.ctypes.data, kw.ctypes.data)
    out["kg9_16_dirs"], out["kg9_16_kmag"], out["kg9_16_w"] = kd, km, kw
    np.savez_compressed(OUT, **out)
    print(f"wrote {OUT}: {sorted(out)}")


if __name__ == "__main__":
    main()
