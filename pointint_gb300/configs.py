"""Seeded synthetic workloads of the benchmark configurations.

Each builder returns (kgrid, objects, meta) where objects are SceneObjects in
the reference's packed layout with their DoFs.  Sizes follow the workload
definitions exactly; seeds and mix ratios are recorded in ``meta``.

  pair_sweep      unit cube (12 tris) vs unit icosphere-3 (1,280 tris) at 64
                  offsets U[-1.2,1.2]^3, L=32 x Lebedev-302 (N_k = 9,664)
  matrix256       256 objects: 128 icosphere-4 (5,120 tris) under
                  R diag(U[0.5,1.5]^3) R' + 128 boxes of side U[0.5,2] with
                  random rotations; centres U[0,8]^3; L=64 x Lebedev-1202
                  (N_k = 76,928)
  large_mesh      32 star-shaped solids, 200,000 tris each, L=128 x
                  Lebedev-5810 (N_k = 743,680)
  surfels64       64 objects x 50,000 disks (and the same as Gaussians),
                  area-uniform samples of matrix256 shapes, L=64 x Lebedev-1202
  serving_stream  library of spheres / ellipsoids meshed with 1k-50k tris
                  (log-uniform); scenes of N ~ logU[2, 512] library objects,
                  each translated by N(0, 0.5^2) and rotated with probability
                  0.2; Poisson arrival times; L=64 x Lebedev-1202
"""
from __future__ import annotations

import numpy as np

from . import geometry as G
from ._lib import DOF_AFFINE
from .kgrid import standard_kgrid


def pair_sweep(seed: int = 0, n_offsets: int = 64):
    rng = np.random.default_rng(seed)
    kg = standard_kgrid(29, 32)
    Vc, Fc = G.create_unit_cube_mesh()
    Vs, Fs = G.icosphere(3)
    cube = G.SceneObject(G.make_triangle_mesh(Vc, Fc))
    sphere_geom = G.make_triangle_mesh(Vs, Fs)
    offsets = rng.uniform(-1.2, 1.2, size=(n_offsets, 3))
    spheres = [G.SceneObject(sphere_geom, DOF_AFFINE, G.affine_dofs(np.eye(3), t)) for t in offsets]
    meta = {"workload": "cube(12 tris) x icosphere-3(1280 tris), 64 offsets U[-1.2,1.2]^3",
            "seed": seed, "n_k": kg.num_nodes, "L": 32, "M": 302}
    return kg, cube, spheres, offsets, meta


def matrix256(seed: int = 0, n_objects: int = 256, n_spheres: int | None = None, kgrid=True):
    """The 256-object volume matrix workload (first half icospheres, second half boxes)."""
    rng = np.random.default_rng(seed)
    n_sph = n_objects // 2 if n_spheres is None else n_spheres
    Vs, Fs = G.icosphere(4)
    sph = G.make_triangle_mesh(Vs, Fs)
    Vc, Fc = G.create_unit_cube_mesh()
    box = G.make_triangle_mesh(Vc, Fc)
    objs = []
    for i in range(n_objects):
        R1 = G.random_rotation(rng)
        c = rng.uniform(0.0, 8.0, size=3)
        if i < n_sph:
            R2 = G.random_rotation(rng)
            A = R1 @ np.diag(rng.uniform(0.5, 1.5, size=3)) @ R2.T
            objs.append(G.SceneObject(sph, DOF_AFFINE, G.affine_dofs(A, c)))
        else:
            A = R1 * rng.uniform(0.5, 2.0)
            objs.append(G.SceneObject(box, DOF_AFFINE, G.affine_dofs(A, c)))
    kg = standard_kgrid(59, 64) if kgrid else None
    n_tri = sum(o.geom.num_elements() for o in objs)
    meta = {"workload": f"{n_objects}-object volume matrix: {n_sph} icosphere-4 (5120 tris, affine sv U[0.5,1.5]) + "
                        f"{n_objects - n_sph} boxes (side U[0.5,2]), rotations random, centres U[0,8]^3",
            "seed": seed, "n_objects": n_objects, "mix": f"{n_sph}/{n_objects - n_sph}", "n_triangles": n_tri,
            "n_k": 76928, "L": 64, "M": 1202}
    return kg, objs, meta


def surfels64(seed: int = 0, n_objects: int = 64, n_surfels: int = 50000, gaussian: bool = False, kgrid=True):
    """Disk (or isotropic Gaussian) clouds sampled area-uniformly from matrix256
    shapes; radius sqrt(area/(pi N)), Gaussian sigma equal to that radius."""
    rng = np.random.default_rng(seed)
    _, shapes, _ = matrix256(seed, n_objects=n_objects, kgrid=False)
    Vs, Fs = G.icosphere(4)
    Vc, Fc = G.create_unit_cube_mesh()
    objs = []
    for o in shapes:
        A = o.dofs[3:].reshape(3, 3)
        t = o.dofs[:3]
        V, F = (Vs, Fs) if o.geom.num_elements() > 12 else (Vc, Fc)
        Vw = V @ A.T + t
        P, N, a_share = G.sample_surface(Vw, F, n_surfels, rng)
        total_area = a_share * n_surfels
        rho = np.sqrt(total_area / (np.pi * n_surfels))
        if gaussian:
            geom = G.make_gaussian_splat(P, N, np.full(n_surfels, rho), np.full(n_surfels, a_share))
        else:
            geom = G.make_point_cloud(P, N, np.full(n_surfels, rho), True)
        objs.append(G.SceneObject(geom))
    kg = standard_kgrid(59, 64) if kgrid else None
    meta = {"workload": f"{n_objects} objects x {n_surfels} {'Gaussians' if gaussian else 'disks'}",
            "seed": seed, "n_k": 76928}
    return kg, objs, meta


def large_mesh(seed: int = 0, n_objects: int = 32, frequency: int = 100, kgrid=True):
    rng = np.random.default_rng(seed)
    V0, F = G.geodesic_sphere(frequency)
    theta = np.arccos(np.clip(V0[:, 2], -1.0, 1.0))
    phi = np.arctan2(V0[:, 1], V0[:, 0])
    Y = G._real_sph_harm_basis(8, theta, phi)
    objs = []
    for _ in range(n_objects):
        c = rng.normal(0.0, 0.05, size=Y.shape[1])
        r = np.maximum(1.0 + Y @ c, 0.5)
        objs.append(G.SceneObject(G.make_triangle_mesh(V0 * r[:, None], F)))
    kg = standard_kgrid(131, 128) if kgrid else None
    meta = {"workload": f"{n_objects} star-shaped solids x {len(F)} tris (SH degree<=8, N(0,0.05^2))",
            "seed": seed, "n_triangles_each": int(len(F)), "n_k": 743680}
    return kg, objs, meta


def serving_stream(seed: int = 0, n_library: int = 64, n_queries: int = 10000, p_rot: float = 0.2,
                   n_min: int = 2, n_max: int = 512, rate_hz: float = 100.0, kgrid=True):
    """Scene-query stream: (kgrid, library, queries, arrival_s, meta).

    Library meshes are geodesic spheres of frequency f (20 f^2 triangles, f in
    7..50 for 1k-50k triangles, log-uniform), half of them stretched into
    ellipsoids by R diag(U[0.5,1.5]^3) R'.  A query is (objects, rotations,
    translations) with N log-uniform in [n_min, n_max] objects drawn with
    replacement.  Arrivals are a Poisson process of rate rate_hz."""
    rng = np.random.default_rng(seed)
    cache = {}
    lib, tris = [], []
    for i in range(n_library):
        t = float(np.exp(rng.uniform(np.log(1000.0), np.log(50000.0))))
        f = int(min(50, max(7, round(np.sqrt(t / 20.0)))))
        if f not in cache:
            cache[f] = G.geodesic_sphere(f)
        V, F = cache[f]
        if i % 2:
            R = G.random_rotation(rng)
            V = V @ (R @ np.diag(rng.uniform(0.5, 1.5, size=3)) @ R.T).T
        lib.append(G.SceneObject(G.make_triangle_mesh(V, F)))
        tris.append(len(F))
    queries = []
    for _ in range(n_queries):
        n = int(min(n_max, max(n_min, round(np.exp(rng.uniform(np.log(n_min), np.log(n_max)))))))
        objects = rng.integers(0, n_library, size=n).astype(np.int32)
        rot = np.zeros((n, 3, 3))
        for k in range(n):
            rot[k] = G.random_rotation(rng) if rng.random() < p_rot else np.eye(3)
        trans = rng.normal(0.0, 0.5, size=(n, 3))
        queries.append((objects, rot, trans))
    arrival = np.cumsum(rng.exponential(1.0 / rate_hz, size=n_queries))
    kg = standard_kgrid(59, 64) if kgrid else None
    meta = {"workload": f"scene stream: N ~ logU[{n_min},{n_max}] of {n_library} library meshes "
                        f"(geodesic spheres/ellipsoids, {min(tris)}-{max(tris)} tris), translations N(0,0.5^2), "
                        f"rotation p={p_rot}, Poisson arrivals",
            "seed": seed, "n_library": n_library, "library_tris": tris, "n_queries": n_queries,
            "mean_objects": float(np.mean([len(q[0]) for q in queries])), "p_rot": p_rot}
    return kg, lib, queries, arrival, meta
