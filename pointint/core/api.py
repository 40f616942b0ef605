"""Pair-volume entry points of pointint.core, computed by the Fourier path.

``get_mesh_intersection_volume`` and ``get_ptcld_intersection_volume`` keep
the signatures of the reference's pointint/core/api.py:6-71.  The reference
computed them by a regularised direct sum over surface samples (its Warp
kernel module is absent); here they are the Fourier volume
(1/8 pi^3) sum_q w_q Re(A_1(k_q) conj A_2(k_q)) on a Gauss-Legendre x Lebedev
k-grid, with meshes as exact triangle form factors and point clouds as
oriented disks.  ``eps`` (the direct sum's regulariser) has no counterpart:
the k-grid's finite radial range plays that role, so it is accepted and
unused.
"""
from __future__ import annotations

import ctypes

import numpy as np

from pointint_gb300 import _lib
from pointint_gb300.geometry import SceneObject, make_point_cloud, make_triangle_mesh
from pointint_gb300.kgrid import KGrid, standard_kgrid

_default = {}


def default_kgrid() -> KGrid:
    """L = 32 Gauss-Legendre radii x Lebedev-302 directions (N_k = 9,664), the
    grid of the reference's pair-volume experiments (demo/exp.py:73-76)."""
    if "kg" not in _default:
        _default["kg"] = standard_kgrid(29, 32)
    return _default["kg"]


def _select_device(device) -> None:
    if device is None:
        return
    import torch
    d = torch.device(device)
    if d.type != "cuda":
        raise ValueError(f"pointint.core runs on CUDA devices only, not {device!r}")
    torch.cuda.set_device(d)


def _pair(o1: SceneObject, o2: SceneObject, kgrid: KGrid) -> float:
    c1, c2 = o1.as_c(), o2.as_c()
    v = ctypes.c_double(0.0)
    _lib.check(_lib.lib().pi_pair_volume_host(ctypes.byref(c1), ctypes.byref(c2), kgrid.dirs.ctypes.data,
                                              kgrid.kmag.ctypes.data, kgrid.w.ctypes.data, kgrid.num_nodes,
                                              ctypes.byref(v)))
    return float(v.value)


def knn_area_weights(P: np.ndarray, k_neighbors: int = 30) -> np.ndarray:
    """Per-point surface area of an oriented point cloud: pi r_k^2 / k with r_k
    the distance to the k-th nearest neighbour (a disk of radius r_k on a
    locally flat, evenly sampled surface holds k points).  Stands in for the
    reference's Voronoi cross-section weights (pointint/core/area.py), which
    are preprocessing outside the Fourier path."""
    from scipy.spatial import cKDTree
    P = np.ascontiguousarray(P, dtype=np.float64).reshape(-1, 3)
    k = int(min(max(1, k_neighbors), len(P) - 1))
    if k < 1:
        raise ValueError("area weights need at least two points")
    d, _ = cKDTree(P).query(P, k=k + 1)  # the first neighbour is the point itself
    return np.pi * d[:, k] ** 2 / k


def mesh_intersection_volume(vertices1, faces1, vertices2, faces2, kgrid: KGrid | None = None) -> float:
    """Fourier intersection volume of two closed, outward-oriented triangle meshes."""
    g1 = make_triangle_mesh(vertices1, faces1)
    g2 = make_triangle_mesh(vertices2, faces2)
    return _pair(SceneObject(g1), SceneObject(g2), kgrid or default_kgrid())


def ptcld_intersection_volume(P1, N1, W1, P2, N2, W2, kgrid: KGrid | None = None) -> float:
    """Fourier intersection volume of two oriented point clouds with per-point
    area weights W (each point a disk of area W, radius sqrt(W/pi))."""
    g1 = make_point_cloud(P1, N1, W1, False)
    g2 = make_point_cloud(P2, N2, W2, False)
    return _pair(SceneObject(g1), SceneObject(g2), kgrid or default_kgrid())


def get_ptcld_intersection_volume(P1, N1, P2, N2, eps: float = 1e-3, k_neighbors: int = 30, device: str = None,
                                  kgrid: KGrid | None = None, W1=None, W2=None) -> float:
    """Intersection volume of two oriented point clouds (reference
    pointint/core/api.py:6-37).  Area weights come from ``knn_area_weights``
    unless W1 / W2 are given; ``eps`` is unused (no regulariser in the Fourier
    method)."""
    _select_device(device)
    W1 = knn_area_weights(P1, k_neighbors) if W1 is None else W1
    W2 = knn_area_weights(P2, k_neighbors) if W2 is None else W2
    return ptcld_intersection_volume(P1, N1, W1, P2, N2, W2, kgrid)


def get_mesh_intersection_volume(vertices1, faces1, vertices2, faces2, eps: float = 1e-3, device: str = None,
                                 kgrid: KGrid | None = None) -> float:
    """Intersection volume of two triangle meshes (reference
    pointint/core/api.py:40-71); ``eps`` is unused (no regulariser in the
    Fourier method)."""
    _select_device(device)
    return mesh_intersection_volume(vertices1, faces1, vertices2, faces2, kgrid)
