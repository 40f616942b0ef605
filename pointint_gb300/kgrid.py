"""Quadrature: Lebedev directions x Gauss-Legendre radii (host side, native).

``KGrid`` mirrors the reference's KGrid (cpp/include/quadrature/kgrid.hpp:9-13):
``dirs`` (Q x 3), ``kmag`` (Q), ``w`` (Q), node q = ir*M + j, k = tan t on
Gauss-Legendre t in [0, pi/2], w = w_leb * w_GL * sec^2 t.  The arithmetic runs
in the native library (pi_gauss_legendre / pi_load_lebedev / pi_build_kgrid).
The device copy is created lazily, once per grid, and reused by every call.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import _lib

DATA_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "lebedev")


def lebedev_path(order: int) -> str:
    """Path of the bundled Lebedev rule of the given algebraic order (3, 9, 29, 59, 131)."""
    p = os.path.join(DATA_DIR, f"lebedev_{order:03d}.txt")
    if not os.path.exists(p):
        raise FileNotFoundError(p)
    return p


def gauss_legendre(n: int, a: float, b: float):
    x, w = np.zeros(n), np.zeros(n)
    _lib.check(_lib.lib().pi_gauss_legendre(int(n), float(a), float(b), x.ctypes.data, w.ctypes.data))
    return x, w


def load_lebedev(path: str):
    """(dirs[M,3], weights[M] summing to 4 pi) -- reference load_lebedev_txt."""
    n = ctypes.c_int64(0)
    _lib.check(_lib.lib().pi_load_lebedev(path.encode(), None, None, 0, ctypes.byref(n)))
    dirs, w = np.zeros((n.value, 3)), np.zeros(n.value)
    _lib.check(_lib.lib().pi_load_lebedev(path.encode(), dirs.ctypes.data, w.ctypes.data, n.value, ctypes.byref(n)))
    return dirs, w


class KGrid:
    """Host k-grid (reference KGrid) with a lazily created device copy."""

    def __init__(self, dirs=None, kmag=None, w=None):
        self.dirs = np.ascontiguousarray(dirs if dirs is not None else np.zeros((0, 3)), dtype=np.float64).reshape(-1, 3)
        self.kmag = np.ascontiguousarray(kmag if kmag is not None else np.zeros(0), dtype=np.float64).reshape(-1)
        self.w = np.ascontiguousarray(w if w is not None else np.zeros(0), dtype=np.float64).reshape(-1)
        if not (len(self.dirs) == len(self.kmag) == len(self.w)):
            raise ValueError("dirs, kmag and w must have the same length")
        self._handle = None

    @property
    def num_nodes(self) -> int:
        return int(len(self.kmag))

    def __len__(self) -> int:
        return self.num_nodes

    def handle(self):
        """Device k-grid handle (created on first use, freed with the object)."""
        if self._handle is None:
            h = ctypes.c_void_p()
            _lib.check(_lib.lib().pi_kgrid_create(self.dirs.ctypes.data, self.kmag.ctypes.data, self.w.ctypes.data,
                                                  self.num_nodes, ctypes.byref(h)))
            self._handle = h
        return self._handle

    def info(self):
        Q, M, L = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        _lib.check(_lib.lib().pi_kgrid_info(self.handle(), ctypes.byref(Q), ctypes.byref(M), ctypes.byref(L)))
        return Q.value, M.value, L.value

    def direction_pairs(self) -> np.ndarray:
        """(n_eval, 2) int32: the directions the kernels evaluate, each with
        its antipode (or -1), in evaluation order (host only; the pairing the
        device k-grid stores)."""
        Q = self.num_nodes
        out = np.zeros((Q, 2), dtype=np.int32)
        n = ctypes.c_int64()
        _lib.check(_lib.lib().pi_kgrid_direction_pairs(self.dirs.ctypes.data, self.kmag.ctypes.data, Q,
                                                       out.ctypes.data, Q, ctypes.byref(n)))
        return out[:n.value].copy()

    def __del__(self):
        h = getattr(self, "_handle", None)
        if h is not None and _lib._lib is not None:
            try:
                _lib._lib.pi_kgrid_destroy(h)
            except Exception:
                pass


def build_kgrid(leb_dirs, leb_weights, n_radial: int) -> KGrid:
    ld = np.ascontiguousarray(leb_dirs, dtype=np.float64).reshape(-1, 3)
    lw = np.ascontiguousarray(leb_weights, dtype=np.float64).reshape(-1)
    M = len(lw)
    Q = M * int(n_radial)
    dirs, kmag, w = np.zeros((Q, 3)), np.zeros(Q), np.zeros(Q)
    _lib.check(_lib.lib().pi_build_kgrid(ld.ctypes.data, lw.ctypes.data, M, int(n_radial), dirs.ctypes.data,
                                         kmag.ctypes.data, w.ctypes.data))
    return KGrid(dirs, kmag, w)


def standard_kgrid(lebedev_order: int, n_radial: int) -> KGrid:
    """k-grid from a bundled Lebedev rule: e.g. (29, 32) -> N_k = 9,664,
    (59, 64) -> 76,928, (131, 128) -> 743,680."""
    d, w = load_lebedev(lebedev_path(lebedev_order))
    return build_kgrid(d, w, n_radial)
