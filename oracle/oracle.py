"""FP64 CPU oracle for the Fourier intersection-volume path (ctypes wrapper).

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` may import this
module.  The product (``pointint_gb300``) never imports it and never falls back
to it.

The C++ side (``oracle/oracle.cpp``) restates the reference's CPU path
(PoIntInt ``cpp/src/element_functions.cpp``, ``form_factor_helpers.cpp``,
``dof/affine_dof.cpp``, ``dof/triangle_mesh_dof.cpp``,
``compute_intersection_volume_cpu.cpp``,
``compute_intersection_volume_multi_object.cpp``).  Its element functions and
quadrature are pinned against the reference's own sources compiled into
``oracle/_ref`` (``oracle/build_ref.sh``) and against golden vectors produced
from that build (``tests/golden/``).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_LIB_PATH = os.path.join(HERE, "_ref", "libpointint_ref.so")

GEOM_TRIANGLE, GEOM_DISK, GEOM_GAUSSIAN = 0, 1, 2
DOF_AFFINE, DOF_TRIANGLE_MESH = 0, 1
VOLUME_ONLY, GRADIENT, HESSIAN = 1, 2, 4

# Byte layouts of the reference's TriPacked / DiskPacked / GaussianPacked
# (cpp/include/geometry/types.hpp:9-37).
TRI_DTYPE = np.dtype([("a", "<f8", 3), ("e1", "<f8", 3), ("e2", "<f8", 3), ("S", "<f8", 3),
                      ("vid", "<i4", 3), ("pad", "<i4")])
DISK_DTYPE = np.dtype([("c", "<f8", 3), ("n", "<f8", 3), ("rho", "<f8"), ("area", "<f8")])
GAUSS_DTYPE = np.dtype([("c", "<f8", 3), ("n", "<f8", 3), ("sigma", "<f8"), ("w", "<f8")])
assert TRI_DTYPE.itemsize == 112 and DISK_DTYPE.itemsize == 64 and GAUSS_DTYPE.itemsize == 64

IDENTITY_AFFINE = np.array([0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0, 1], dtype=np.float64)


class _CObj(ctypes.Structure):
    _fields_ = [("geom_type", ctypes.c_int32), ("dof_type", ctypes.c_int32),
                ("n_elems", ctypes.c_int64), ("elems", ctypes.c_void_p),
                ("n_dofs", ctypes.c_int64), ("dofs", ctypes.c_void_p)]


@dataclass
class Obj:
    """One object: packed elements + DoF parameterization + DoF vector."""
    geom_type: int
    elems: np.ndarray
    dof_type: int = DOF_AFFINE
    dofs: np.ndarray | None = None

    def __post_init__(self):
        if self.dofs is None:
            self.dofs = IDENTITY_AFFINE.copy()
        self.dofs = np.ascontiguousarray(self.dofs, dtype=np.float64)
        self.elems = np.ascontiguousarray(self.elems)

    def c(self) -> _CObj:
        return _CObj(self.geom_type, self.dof_type, len(self.elems), self.elems.ctypes.data,
                     len(self.dofs), self.dofs.ctypes.data)


_lock = threading.Lock()
_lib = None
_ref = None


def build(force: bool = False) -> str:
    """Compile oracle.cpp into oracle/liboracle.so (plain g++, OpenMP)."""
    src = os.path.join(HERE, "oracle.cpp")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        tmp = LIB_PATH + f".tmp{os.getpid()}"
        subprocess.check_call(["g++", "-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared", src, "-o", tmp])
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


def build_ref() -> str | None:
    """Build oracle/_ref from the reference sources when they are present."""
    subprocess.check_call(["bash", os.path.join(HERE, "build_ref.sh")])
    return REF_LIB_PATH if os.path.exists(REF_LIB_PATH) else None


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(LIB_PATH)
            P, I64, I32, D = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_double
            OP = ctypes.POINTER(_CObj)
            sig = {
                "or_max_threads": (I32, []), "or_set_threads": (None, [I32]),
                "or_E": (None, [D, P]), "or_E_prime": (None, [D, P]), "or_E_double_prime": (None, [D, P]),
                "or_Phi": (None, [D, D, P]), "or_Phi_grad": (None, [D, D, P]),
                "or_J1_over_x": (D, [D]), "or_J1_over_x_prime": (D, [D]),
                "or_gauss_legendre": (I32, [I32, D, D, P, P]),
                "or_build_kgrid": (I32, [P, P, I32, I32, P, P, P]),
                "or_lebedev_dir": (None, [D, D, P]),
                "or_exact_cube_form_factor": (D, [D, D, D]),
                "or_exact_sphere_form_factor": (D, [D, D]),
                "or_box_box_intersection_volume": (D, [P, P, P, P]),
                "or_sphere_sphere_intersection_volume": (D, [P, D, P, D]),
                "or_pack_tris": (None, [P, P, I64, P]),
                "or_pack_disks": (None, [P, P, P, I64, I32, P]),
                "or_pack_gaussians": (None, [P, P, P, P, I64, P]),
                "or_form_factor": (I32, [OP, P, I64, P]),
                "or_form_factor_grad": (I32, [OP, P, I64, P]),
                "or_form_factor_matrix": (I32, [OP, I32, P, P, I64, I64, P]),
                "or_contract": (I32, [P, P, I64, I32, P]),
                "or_volume_matrix": (I32, [OP, I32, P, P, P, I64, I32, P, P, P]),
                "or_pair_volume": (I32, [OP, OP, P, P, P, I64, I32, P, P, P, P, P, P]),
                "or_self_volume": (D, [OP]),
                "or_surfel_param_grad": (I32, [OP, I32, P, P, P, I64, P, P, P]),
            }
            for name, (res, args) in sig.items():
                f = getattr(L, name)
                f.restype = res
                f.argtypes = args
            _lib = L
        return _lib


def ref_lib():
    """The reference's own element functions / quadrature (None if not built)."""
    global _ref
    with _lock:
        if _ref is None and os.path.exists(REF_LIB_PATH):
            R = ctypes.CDLL(REF_LIB_PATH)
            P, D = ctypes.c_void_p, ctypes.c_double
            for n in ("ref_E", "ref_E_prime", "ref_E_double_prime"):
                getattr(R, n).argtypes = [D, P]; getattr(R, n).restype = None
            R.ref_Phi.argtypes = [D, D, P]; R.ref_Phi.restype = None
            R.ref_Phi_grad.argtypes = [D, D, P]; R.ref_Phi_grad.restype = None
            R.ref_J1_over_x.argtypes = [D]; R.ref_J1_over_x.restype = D
            R.ref_J1_over_x_prime.argtypes = [D]; R.ref_J1_over_x_prime.restype = D
            R.ref_gauss_legendre.argtypes = [ctypes.c_int, D, D, P, P]; R.ref_gauss_legendre.restype = ctypes.c_int
            R.ref_load_lebedev.argtypes = [ctypes.c_char_p, P, P, ctypes.c_int64]
            R.ref_load_lebedev.restype = ctypes.c_int64
            R.ref_build_kgrid.argtypes = [P, P, ctypes.c_int64, ctypes.c_int, P, P, P]
            R.ref_build_kgrid.restype = ctypes.c_int
            _ref = R
        return _ref


def _p(a: np.ndarray):
    return a.ctypes.data


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


# ----------------------------------------------------------------------------- scalar functions
def _cplx_fn(name):
    def f(z: float) -> complex:
        o = np.zeros(2)
        getattr(lib(), name)(float(z), _p(o))
        return complex(o[0], o[1])
    return f


E_func = _cplx_fn("or_E")
E_prime = _cplx_fn("or_E_prime")
E_double_prime = _cplx_fn("or_E_double_prime")


def Phi(a: float, b: float) -> complex:
    o = np.zeros(2)
    lib().or_Phi(float(a), float(b), _p(o))
    return complex(o[0], o[1])


def Phi_grad(a: float, b: float) -> tuple[complex, complex]:
    o = np.zeros(4)
    lib().or_Phi_grad(float(a), float(b), _p(o))
    return complex(o[0], o[1]), complex(o[2], o[3])


def J1_over_x(x: float) -> float:
    return lib().or_J1_over_x(float(x))


def J1_over_x_prime(x: float) -> float:
    return lib().or_J1_over_x_prime(float(x))


def exact_cube_form_factor(kx, ky, kz) -> float:
    return lib().or_exact_cube_form_factor(float(kx), float(ky), float(kz))


def exact_sphere_form_factor(k, R) -> float:
    return lib().or_exact_sphere_form_factor(float(k), float(R))


def box_box_intersection_volume(c1, h1, c2, h2) -> float:
    a = [_f64(x) for x in (c1, h1, c2, h2)]
    return lib().or_box_box_intersection_volume(*[_p(x) for x in a])


def sphere_sphere_intersection_volume(c1, r1, c2, r2) -> float:
    a, b = _f64(c1), _f64(c2)
    return lib().or_sphere_sphere_intersection_volume(_p(a), float(r1), _p(b), float(r2))


# ----------------------------------------------------------------------------- quadrature
def gauss_legendre(n: int, a: float, b: float):
    x, w = np.zeros(n), np.zeros(n)
    lib().or_gauss_legendre(n, float(a), float(b), _p(x), _p(w))
    return x, w


def load_lebedev(path: str):
    """(dirs[M,3], weights[M] summing to 4 pi) -- lebedev_io.hpp:24-59."""
    rows = []
    with open(path) as fh:
        for line in fh:
            if not line.strip() or line.startswith("#"):
                continue
            p = line.split()
            if len(p) < 3:
                continue
            rows.append((float(p[0]), float(p[1]), float(p[2])))
    dirs = np.zeros((len(rows), 3))
    w = np.array([r[2] for r in rows])
    for i, (th, ph, _) in enumerate(rows):
        lib().or_lebedev_dir(th, ph, _p(dirs[i]))
    s = w.sum()
    if abs(s - 1.0) < 0.1:
        w = w * (4.0 * np.pi)
    return dirs, w


def build_kgrid(leb_dirs, leb_w, n_radial: int):
    ld, lw = _f64(leb_dirs), _f64(leb_w)
    M = len(lw)
    Q = M * n_radial
    dirs, kmag, w = np.zeros((Q, 3)), np.zeros(Q), np.zeros(Q)
    lib().or_build_kgrid(_p(ld), _p(lw), M, n_radial, _p(dirs), _p(kmag), _p(w))
    return dirs, kmag, w


# ----------------------------------------------------------------------------- packing
def pack_tris(V, F) -> np.ndarray:
    V, F = _f64(V), np.ascontiguousarray(F, dtype=np.int32)
    out = np.zeros(len(F), dtype=TRI_DTYPE)
    lib().or_pack_tris(_p(V), _p(F), len(F), _p(out))
    return out


def pack_disks(P, N, radii_or_areas, is_radius=True) -> np.ndarray:
    P, N, r = _f64(P), _f64(N), _f64(radii_or_areas)
    out = np.zeros(len(P), dtype=DISK_DTYPE)
    lib().or_pack_disks(_p(P), _p(N), _p(r), len(P), int(bool(is_radius)), _p(out))
    return out


def pack_gaussians(P, N, sigmas, weights) -> np.ndarray:
    P, N, s, w = _f64(P), _f64(N), _f64(sigmas), _f64(weights)
    out = np.zeros(len(P), dtype=GAUSS_DTYPE)
    lib().or_pack_gaussians(_p(P), _p(N), _p(s), _p(w), len(P), _p(out))
    return out


# ----------------------------------------------------------------------------- form factors / drivers
def form_factor(obj: Obj, kvecs) -> np.ndarray:
    k = _f64(kvecs).reshape(-1, 3)
    out = np.zeros(2 * len(k))
    co = obj.c()
    lib().or_form_factor(ctypes.byref(co), _p(k), len(k), _p(out))
    return out.view(np.complex128)


def form_factor_grad(obj: Obj, kvecs) -> np.ndarray:
    k = _f64(kvecs).reshape(-1, 3)
    nd = len(obj.dofs)
    out = np.zeros(2 * len(k) * nd)
    co = obj.c()
    lib().or_form_factor_grad(ctypes.byref(co), _p(k), len(k), _p(out))
    return out.view(np.complex128).reshape(len(k), nd)


def _objarr(objs):
    arr = (_CObj * len(objs))(*[o.c() for o in objs])
    return arr


def form_factor_matrix(objs, dirs, kmag, stride: int = 1) -> np.ndarray:
    """J[q, obj] (Q x N complex); with stride > 1 only rows q % stride == 0 are filled."""
    d, km = _f64(dirs), _f64(kmag)
    Q = len(km)
    J = np.zeros(2 * Q * len(objs))
    arr = _objarr(objs)
    lib().or_form_factor_matrix(arr, len(objs), _p(d), _p(km), Q, int(stride), _p(J))
    return J.view(np.complex128).reshape(Q, len(objs))


def contract(J: np.ndarray, w) -> np.ndarray:
    J = np.ascontiguousarray(J, dtype=np.complex128)
    Q, n = J.shape
    wv = _f64(w)
    V = np.zeros((n, n))
    lib().or_contract(_p(J.view(np.float64)), _p(wv), Q, n, _p(V))
    return V


def volume_matrix(objs, kgrid, flags: int = VOLUME_ONLY):
    """Returns (V, grad, hess_ij).  grad[i][j] = dV_ij/dtheta_i; hess_ij[i][j] is
    the Gauss-Newton cross block (multi_object.cpp:186-292)."""
    dirs, kmag, w = (_f64(x) for x in kgrid)
    n = len(objs)
    nd = [len(o.dofs) for o in objs]
    V = np.zeros((n, n))
    g = np.zeros(max(1, n * sum(nd)))
    h = np.zeros(max(1, sum(nd[i] * nd[j] for i in range(n) for j in range(n))))
    arr = _objarr(objs)
    lib().or_volume_matrix(arr, n, _p(dirs), _p(kmag), _p(w), len(kmag), int(flags), _p(V), _p(g), _p(h))
    grad = hess = None
    if flags & GRADIENT:
        grad, off = [], 0
        for i in range(n):
            grad.append([g[off + j * nd[i]: off + (j + 1) * nd[i]].copy() for j in range(n)])
            off += n * nd[i]
    if flags & HESSIAN:
        hess, off = [[None] * n for _ in range(n)], 0
        for i in range(n):
            for j in range(n):
                hess[i][j] = h[off: off + nd[i] * nd[j]].reshape(nd[i], nd[j]).copy()
                off += nd[i] * nd[j]
    return V, grad, hess


def pair_volume(o1: Obj, o2: Obj, kgrid, flags: int = VOLUME_ONLY) -> dict:
    dirs, kmag, w = (_f64(x) for x in kgrid)
    d1, d2 = len(o1.dofs), len(o2.dofs)
    vol = np.zeros(1)
    g1, g2 = np.zeros(d1), np.zeros(d2)
    H11, H22, H12 = np.zeros((d1, d1)), np.zeros((d2, d2)), np.zeros((d1, d2))
    c1, c2 = o1.c(), o2.c()
    lib().or_pair_volume(ctypes.byref(c1), ctypes.byref(c2), _p(dirs), _p(kmag), _p(w), len(kmag),
                         int(flags), _p(vol), _p(g1), _p(g2), _p(H11), _p(H22), _p(H12))
    out = {"volume": float(vol[0])}
    if flags & GRADIENT:
        out["grad_geom1"], out["grad_geom2"] = g1, g2
    if flags & HESSIAN:
        out["hessian_geom1"], out["hessian_geom2"], out["hessian_cross"] = H11, H22, H12
    return out


def self_volume(obj: Obj) -> float:
    co = obj.c()
    return lib().or_self_volume(ctypes.byref(co))


def surfel_param_grad(objs, kgrid, C):
    """dL/dc, dL/dn per disk/Gaussian (identity DoFs) for L = sum_ij C_ij V_ij."""
    dirs, kmag, w = (_f64(x) for x in kgrid)
    C = _f64(C)
    ne = sum(len(o.elems) for o in objs)
    gp, gn = np.zeros((ne, 3)), np.zeros((ne, 3))
    arr = _objarr(objs)
    rc = lib().or_surfel_param_grad(arr, len(objs), _p(dirs), _p(kmag), _p(w), len(kmag), _p(C), _p(gp), _p(gn))
    if rc != 0:
        raise ValueError("surfel_param_grad supports disks and Gaussians only")
    return gp, gn


def set_threads(n: int) -> None:
    lib().or_set_threads(int(n))


def max_threads() -> int:
    return lib().or_max_threads()
