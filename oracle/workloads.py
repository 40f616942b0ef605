"""Seeded benchmark workloads built from the oracle alone.

TEST INFRASTRUCTURE ONLY, like the rest of ``oracle/``: ``bench.py``'s
``--impl reference`` leg times the FP64 oracle on these inputs, so it must not
import the product package or load its native library.  The builders draw the
same random numbers in the same order as the product's workload builders, and
pack elements and build the k-grid with the oracle's restatements of
``cpp/src/geometry/packing.cpp:10-112`` and ``cpp/include/quadrature/kgrid.hpp:17-47``;
``tests/test_oracle_workloads.py`` checks that both give byte-identical inputs.

  matrix256   256 objects: icosphere-4 (5,120 triangles) under
              R1 diag(U[0.5,1.5]^3) R2^T for the first half, boxes of side
              U[0.5,2] (12 triangles) under R1 for the rest; centres U[0,8]^3;
              k-grid L=64 x Lebedev-1202 (N_k = 76,928)
"""
from __future__ import annotations

import os

import numpy as np

from . import oracle as orc

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LEBEDEV_DIR = os.path.join(ROOT, "pointint_gb300", "data", "lebedev")


def icosphere(subdivisions: int):
    """Unit icosphere: the icosahedron with every face split in four per level
    and new vertices projected to the sphere (vertex order: the 12 corners,
    then edge midpoints in face order)."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    V = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    F = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
         (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
         (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    V = [np.array(v, dtype=np.float64) / np.linalg.norm(v) for v in V]
    for _ in range(subdivisions):
        edge_mid = {}
        split = []
        for a, b, c in F:
            m = []
            for u, v in ((a, b), (b, c), (c, a)):
                key = (min(u, v), max(u, v))
                if key not in edge_mid:
                    s = V[u] + V[v]
                    V.append(s / np.linalg.norm(s))
                    edge_mid[key] = len(V) - 1
                m.append(edge_mid[key])
            ab, bc, ca = m
            split += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        F = split
    return np.array(V), np.array(F, dtype=np.int32)


def unit_cube():
    """The reference's 12-triangle unit cube [-1/2, 1/2]^3, outward-facing
    (cpp/src/geometry/geometry_helpers.cpp:16-38 layout)."""
    V = np.array([[-0.5, -0.5, -0.5], [0.5, -0.5, -0.5], [0.5, 0.5, -0.5], [-0.5, 0.5, -0.5],
                  [-0.5, -0.5, 0.5], [0.5, -0.5, 0.5], [0.5, 0.5, 0.5], [-0.5, 0.5, 0.5]])
    F = np.array([[0, 2, 1], [0, 3, 2], [4, 5, 6], [4, 6, 7], [0, 1, 5], [0, 5, 4],
                  [2, 7, 6], [2, 3, 7], [0, 4, 7], [0, 7, 3], [1, 6, 5], [1, 2, 6]], dtype=np.int32)
    return V, F


def random_rotation(rng: np.random.Generator) -> np.ndarray:
    """Uniform random rotation: QR of a 3 x 3 Gaussian matrix, columns signed by
    diag(R), first column flipped if the determinant is negative."""
    q, r = np.linalg.qr(rng.standard_normal((3, 3)))
    q = q * np.sign(np.diag(r))[None, :]
    if np.linalg.det(q) < 0:
        q[:, 0] = -q[:, 0]
    return q


def affine_dofs(A, t) -> np.ndarray:
    """AffineDoF vector [t, A row-major] (cpp/src/dof/affine_dof.cpp:17-29)."""
    return np.concatenate([np.asarray(t, dtype=np.float64).reshape(3), np.asarray(A, dtype=np.float64).reshape(9)])


def kgrid(lebedev_order: int, n_radial: int):
    """(dirs, kmag, w) of the bundled Lebedev rule x n_radial Gauss-Legendre radii."""
    d, w = orc.load_lebedev(os.path.join(LEBEDEV_DIR, f"lebedev_{lebedev_order:03d}.txt"))
    return orc.build_kgrid(d, w, n_radial)


def matrix256(seed: int = 0, n_objects: int = 256, with_kgrid: bool = True):
    """(kgrid, objects, meta): the 256-object volume-matrix workload as oracle objects."""
    rng = np.random.default_rng(seed)
    n_sph = n_objects // 2
    Vs, Fs = icosphere(4)
    sph = orc.pack_tris(Vs, Fs)
    Vc, Fc = unit_cube()
    box = orc.pack_tris(Vc, Fc)
    objs = []
    for i in range(n_objects):
        R1 = random_rotation(rng)
        c = rng.uniform(0.0, 8.0, size=3)
        if i < n_sph:
            R2 = random_rotation(rng)
            A = R1 @ np.diag(rng.uniform(0.5, 1.5, size=3)) @ R2.T
            objs.append(orc.Obj(orc.GEOM_TRIANGLE, sph, orc.DOF_AFFINE, affine_dofs(A, c)))
        else:
            A = R1 * rng.uniform(0.5, 2.0)
            objs.append(orc.Obj(orc.GEOM_TRIANGLE, box, orc.DOF_AFFINE, affine_dofs(A, c)))
    kg = kgrid(59, 64) if with_kgrid else None
    n_tri = sum(len(o.elems) for o in objs)
    meta = {"workload": f"{n_objects}-object volume matrix: {n_sph} icosphere-4 (5120 tris, affine sv U[0.5,1.5]) + "
                        f"{n_objects - n_sph} boxes (side U[0.5,2]), rotations random, centres U[0,8]^3",
            "seed": seed, "n_objects": n_objects, "mix": f"{n_sph}/{n_objects - n_sph}", "n_triangles": n_tri,
            "n_k": 76928, "L": 64, "M": 1202}
    return kg, objs, meta
