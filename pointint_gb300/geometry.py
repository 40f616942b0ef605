"""Geometry containers, packing and shape generators (host side).

``Geometry`` mirrors the reference's ``Geometry`` (cpp/include/geometry/geometry.hpp:8-38):
a type tag plus one packed element array whose byte layout is the reference's
TriPacked / DiskPacked / GaussianPacked (cpp/include/geometry/types.hpp:9-37).
Packing runs in the native library (pi_pack_*), restating
cpp/src/geometry/packing.cpp:10-112.

The generators at the bottom build the seeded synthetic inputs of the
benchmark configurations (icospheres, boxes, affine-deformed and rotated
copies, spherical-harmonic star-shaped solids, area-uniform surfel sampling).
They have no reference counterpart; they stand in for the reference's missing
asset files.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from ._lib import GEOM_TRIANGLE, GEOM_DISK, GEOM_GAUSSIAN, DOF_AFFINE, DOF_TRIANGLE_MESH

TRI_DTYPE = np.dtype([("a", "<f8", 3), ("e1", "<f8", 3), ("e2", "<f8", 3), ("S", "<f8", 3),
                      ("vid", "<i4", 3), ("pad", "<i4")])
DISK_DTYPE = np.dtype([("c", "<f8", 3), ("n", "<f8", 3), ("rho", "<f8"), ("area", "<f8")])
GAUSS_DTYPE = np.dtype([("c", "<f8", 3), ("n", "<f8", 3), ("sigma", "<f8"), ("w", "<f8")])
assert TRI_DTYPE.itemsize == 112 and DISK_DTYPE.itemsize == 64 and GAUSS_DTYPE.itemsize == 64

IDENTITY_AFFINE = np.array([0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0, 1], dtype=np.float64)
_DTYPES = {GEOM_TRIANGLE: TRI_DTYPE, GEOM_DISK: DISK_DTYPE, GEOM_GAUSSIAN: GAUSS_DTYPE}
_NAMES = {GEOM_TRIANGLE: "Triangle mesh", GEOM_DISK: "Point cloud", GEOM_GAUSSIAN: "Gaussian splat"}


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def _ptr(a: np.ndarray):
    return a.ctypes.data


@dataclass
class Geometry:
    """Packed geometry of one object (reference Geometry)."""
    type: int = GEOM_TRIANGLE
    elems: np.ndarray = field(default_factory=lambda: np.zeros(0, dtype=TRI_DTYPE))

    def __post_init__(self):
        want = _DTYPES[self.type]
        if self.elems.dtype != want:
            raise TypeError(f"{_NAMES[self.type]} needs elements of dtype {want}")
        self.elems = np.ascontiguousarray(self.elems)

    def num_elements(self) -> int:
        return int(len(self.elems))

    def is_empty(self) -> bool:
        return self.num_elements() == 0

    @property
    def tris(self):
        return self.elems if self.type == GEOM_TRIANGLE else np.zeros(0, TRI_DTYPE)

    @property
    def disks(self):
        return self.elems if self.type == GEOM_DISK else np.zeros(0, DISK_DTYPE)

    @property
    def gaussians(self):
        return self.elems if self.type == GEOM_GAUSSIAN else np.zeros(0, GAUSS_DTYPE)

    def num_vertices(self) -> int:
        """Vertex count implied by the triangles' vertex ids (TriangleMeshDoF size / 3)."""
        if self.type != GEOM_TRIANGLE or len(self.elems) == 0:
            return 0
        return int(self.elems["vid"].max()) + 1


@dataclass
class SceneObject:
    """A geometry with its DoF parameterization and DoF vector (reference
    DoFParameterization + VectorXd pair)."""
    geom: Geometry
    dof_type: int = DOF_AFFINE
    dofs: np.ndarray | None = None

    def __post_init__(self):
        if self.dofs is None:
            if self.dof_type != DOF_AFFINE:
                raise ValueError("TriangleMeshDoF needs an explicit vertex DoF vector")
            self.dofs = IDENTITY_AFFINE.copy()
        self.dofs = _f64(self.dofs).reshape(-1)

    def as_c(self) -> _lib.PiObject:
        e = self.geom.elems
        return _lib.PiObject(self.geom.type, self.dof_type, len(e), e.ctypes.data if len(e) else None,
                             len(self.dofs), self.dofs.ctypes.data)


# ----------------------------------------------------------------------------- packing (native)
def pack_tris(V, F) -> np.ndarray:
    V = _f64(V).reshape(-1, 3)
    F = np.ascontiguousarray(F, dtype=np.int32).reshape(-1, 3)
    out = np.zeros(len(F), dtype=TRI_DTYPE)
    _lib.check(_lib.lib().pi_pack_tris(_ptr(V), len(V), _ptr(F), len(F), _ptr(out)))
    return out


def pack_disks(P, N, radii_or_areas, is_radius: bool = True) -> np.ndarray:
    P, N, r = _f64(P).reshape(-1, 3), _f64(N).reshape(-1, 3), _f64(radii_or_areas).reshape(-1)
    if not (len(P) == len(N) == len(r)):
        raise ValueError("P, N and radii must have the same length")
    out = np.zeros(len(P), dtype=DISK_DTYPE)
    _lib.check(_lib.lib().pi_pack_disks(_ptr(P), _ptr(N), _ptr(r), len(P), int(bool(is_radius)), _ptr(out)))
    return out


def pack_gaussians(P, N, sigmas, weights) -> np.ndarray:
    P, N = _f64(P).reshape(-1, 3), _f64(N).reshape(-1, 3)
    s, w = _f64(sigmas).reshape(-1), _f64(weights).reshape(-1)
    if not (len(P) == len(N) == len(s) == len(w)):
        raise ValueError("P, N, sigmas and weights must have the same length")
    out = np.zeros(len(P), dtype=GAUSS_DTYPE)
    _lib.check(_lib.lib().pi_pack_gaussians(_ptr(P), _ptr(N), _ptr(s), _ptr(w), len(P), _ptr(out)))
    return out


def make_triangle_mesh(V, F) -> Geometry:
    return Geometry(GEOM_TRIANGLE, pack_tris(V, F))


def make_point_cloud(P, N, radii, is_radius: bool = True) -> Geometry:
    return Geometry(GEOM_DISK, pack_disks(P, N, radii, is_radius))


def make_gaussian_splat(P, N, sigmas, weights) -> Geometry:
    return Geometry(GEOM_GAUSSIAN, pack_gaussians(P, N, sigmas, weights))


def create_unit_cube_mesh():
    V = np.zeros((8, 3))
    F = np.zeros((12, 3), dtype=np.int32)
    _lib.check(_lib.lib().pi_create_unit_cube_mesh(_ptr(V), _ptr(F)))
    return V, F


def create_sphere_pointcloud(n: int = 1000):
    P, N, r = np.zeros((n, 3)), np.zeros((n, 3)), np.zeros(n)
    _lib.check(_lib.lib().pi_create_sphere_pointcloud(int(n), _ptr(P), _ptr(N), _ptr(r)))
    return P, N, r


def create_sphere_gaussians(n: int = 1000):
    P, N, s, w = np.zeros((n, 3)), np.zeros((n, 3)), np.zeros(n), np.zeros(n)
    _lib.check(_lib.lib().pi_create_sphere_gaussians(int(n), _ptr(P), _ptr(N), _ptr(s), _ptr(w)))
    return P, N, s, w


def translate_points(points, translation) -> np.ndarray:
    return _f64(points).reshape(-1, 3) + _f64(translation).reshape(1, 3)


def self_volume(obj: SceneObject) -> float:
    v = ctypes.c_double(0.0)
    c = obj.as_c()
    _lib.check(_lib.lib().pi_self_volume(ctypes.byref(c), ctypes.byref(v)))
    return float(v.value)


def box_box_intersection_volume(c1, h1, c2, h2) -> float:
    a = [_f64(x).reshape(3) for x in (c1, h1, c2, h2)]
    return float(_lib.lib().pi_box_box_intersection_volume(*[_ptr(x) for x in a]))


def sphere_sphere_intersection_volume(c1, r1, c2, r2) -> float:
    a, b = _f64(c1).reshape(3), _f64(c2).reshape(3)
    return float(_lib.lib().pi_sphere_sphere_intersection_volume(_ptr(a), float(r1), _ptr(b), float(r2)))


# ----------------------------------------------------------------------------- synthetic shapes
def icosphere(subdivisions: int, radius: float = 1.0):
    """Unit icosphere: icosahedron with each face split in 4 per level, vertices
    projected to the sphere.  subdivisions=3 -> 1,280 faces, 4 -> 5,120."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    V = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    F = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
         (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
         (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    V = [np.array(v, dtype=np.float64) / np.linalg.norm(v) for v in V]
    for _ in range(subdivisions):
        cache = {}
        newF = []

        def mid(a, b):
            key = (min(a, b), max(a, b))
            if key not in cache:
                m = V[a] + V[b]
                V.append(m / np.linalg.norm(m))
                cache[key] = len(V) - 1
            return cache[key]

        for a, b, c in F:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            newF += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        F = newF
    return np.array(V) * radius, np.array(F, dtype=np.int32)


def geodesic_sphere(frequency: int):
    """Geodesic icosahedron of the given frequency (Class I): each icosahedron
    face split into frequency^2 triangles, vertices projected to the unit
    sphere; 20 * frequency^2 faces (frequency 100 -> 200,000)."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    base = np.array([(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t),
                     (0, 1, -t), (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)], dtype=np.float64)
    base /= np.linalg.norm(base, axis=1, keepdims=True)
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
             (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
             (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    n = frequency
    verts, vid, Fout = [], {}, []

    def key_of(p):
        return tuple(np.round(p * 1e9).astype(np.int64))

    for (ia, ib, ic) in faces:
        A, B, C = base[ia], base[ib], base[ic]
        local = {}
        for i in range(n + 1):
            for j in range(n + 1 - i):
                p = A + (B - A) * (i / n) + (C - A) * (j / n)
                p = p / np.linalg.norm(p)
                k = key_of(p)
                if k not in vid:
                    vid[k] = len(verts)
                    verts.append(p)
                local[(i, j)] = vid[k]
        for i in range(n):
            for j in range(n - i):
                Fout.append((local[(i, j)], local[(i + 1, j)], local[(i, j + 1)]))
                if i + j + 1 < n:
                    Fout.append((local[(i + 1, j)], local[(i + 1, j + 1)], local[(i, j + 1)]))
    return np.array(verts), np.array(Fout, dtype=np.int32)


def box_mesh(side) -> tuple[np.ndarray, np.ndarray]:
    """Axis-aligned box of the given side lengths centred at the origin (12 triangles)."""
    V, F = create_unit_cube_mesh()
    return V * np.asarray(side, dtype=np.float64).reshape(1, 3) * np.ones((1, 3)), F


def random_rotation(rng: np.random.Generator) -> np.ndarray:
    """Uniform random rotation (QR of a Gaussian matrix with sign fix)."""
    q, r = np.linalg.qr(rng.standard_normal((3, 3)))
    q = q * np.sign(np.diag(r))[None, :]
    if np.linalg.det(q) < 0:
        q[:, 0] = -q[:, 0]
    return q


def affine_dofs(A: np.ndarray, t) -> np.ndarray:
    """AffineDoF vector [t, A row-major] (cpp/src/dof/affine_dof.cpp:17-29)."""
    return np.concatenate([_f64(t).reshape(3), _f64(A).reshape(9)])


def _real_sph_harm_basis(lmax: int, theta: np.ndarray, phi: np.ndarray) -> np.ndarray:
    """Real spherical harmonics Y_lm (l <= lmax) at polar angle theta, azimuth phi,
    via the associated Legendre recurrence (orthonormal on the sphere)."""
    from math import factorial
    x = np.cos(theta)
    s = np.sqrt(np.maximum(0.0, 1.0 - x * x))
    P = {}
    P[(0, 0)] = np.ones_like(x)
    for m in range(1, lmax + 1):
        P[(m, m)] = -(2 * m - 1) * s * P[(m - 1, m - 1)]
    for m in range(0, lmax):
        P[(m + 1, m)] = (2 * m + 1) * x * P[(m, m)]
    for m in range(0, lmax + 1):
        for l in range(m + 2, lmax + 1):
            P[(l, m)] = ((2 * l - 1) * x * P[(l - 1, m)] - (l + m - 1) * P[(l - 2, m)]) / (l - m)
    cols = []
    for l in range(lmax + 1):
        for m in range(-l, l + 1):
            am = abs(m)
            norm = np.sqrt((2 * l + 1) / (4 * np.pi) * factorial(l - am) / factorial(l + am))
            if m == 0:
                cols.append(norm * P[(l, 0)])
            elif m > 0:
                cols.append(np.sqrt(2.0) * norm * P[(l, am)] * np.cos(am * phi))
            else:
                cols.append(np.sqrt(2.0) * norm * P[(l, am)] * np.sin(am * phi))
    return np.stack(cols, axis=1)


def star_shape(rng: np.random.Generator, frequency: int = 100, lmax: int = 8, sigma: float = 0.05,
               r_min: float = 0.5):
    """Unit sphere with a seeded real spherical-harmonic radial perturbation,
    r = 1 + sum_{l<=lmax} c_lm Y_lm with c ~ N(0, sigma^2), clamped to r > r_min,
    on a geodesic mesh of 20 frequency^2 faces."""
    V, F = geodesic_sphere(frequency)
    theta = np.arccos(np.clip(V[:, 2], -1.0, 1.0))
    phi = np.arctan2(V[:, 1], V[:, 0])
    Y = _real_sph_harm_basis(lmax, theta, phi)
    c = rng.normal(0.0, sigma, size=Y.shape[1])
    r = np.maximum(1.0 + Y @ c, r_min)
    return V * r[:, None], F


def sample_surface(V, F, n: int, rng: np.random.Generator):
    """Area-uniform samples on a triangle mesh: positions, face normals, and the
    per-sample area share (total area / n)."""
    V = _f64(V)
    F = np.asarray(F)
    a, b, c = V[F[:, 0]], V[F[:, 1]], V[F[:, 2]]
    cr = np.cross(b - a, c - a)
    area = 0.5 * np.linalg.norm(cr, axis=1)
    total = area.sum()
    idx = rng.choice(len(F), size=n, p=area / total)
    u, v = rng.random(n), rng.random(n)
    flip = u + v > 1.0
    u[flip], v[flip] = 1.0 - u[flip], 1.0 - v[flip]
    P = a[idx] + (b[idx] - a[idx]) * u[:, None] + (c[idx] - a[idx]) * v[:, None]
    N = cr[idx] / np.linalg.norm(cr[idx], axis=1, keepdims=True)
    return P, N, total / n
