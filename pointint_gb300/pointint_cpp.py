"""Drop-in for the reference's pybind11 module ``pointint_cpp`` (demo/bindings.cpp:16-103).

Same function names, argument names and defaults, over the GB300 C ABI.  The
reference module exposed only identity-DoF pair volumes; the matrix, DoF and
Gaussian entry points it lacked are added at the end.

    import pointint_cpp as pi            # top-level alias of this module
    P, N, R = pi.create_sphere_pointcloud(1000)
    g1 = pi.make_point_cloud(P, N, R, True)
    dirs, w = pi.load_lebedev(path)
    kg = pi.build_kgrid(dirs, w, 32)
    v = pi.compute_intersection_volume_cuda(g1, g2, kg)
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .geometry import (Geometry, SceneObject, make_triangle_mesh, make_point_cloud, make_gaussian_splat,
                       create_unit_cube_mesh, create_sphere_pointcloud, create_sphere_gaussians,
                       box_box_intersection_volume, sphere_sphere_intersection_volume, translate_points,
                       self_volume, IDENTITY_AFFINE)
from .kgrid import KGrid, load_lebedev as _load_lebedev, build_kgrid as _build_kgrid
from ._lib import DOF_AFFINE, DOF_TRIANGLE_MESH, GEOM_TRIANGLE, GEOM_DISK, GEOM_GAUSSIAN

__all__ = ["Geometry", "KGrid", "make_triangle_mesh", "make_point_cloud", "make_gaussian_splat",
           "create_unit_cube_mesh", "create_sphere_pointcloud", "create_sphere_gaussians", "load_lebedev",
           "build_kgrid", "compute_intersection_volume_cpu", "compute_intersection_volume_cuda",
           "compute_volume_cpu", "box_box_intersection_volume", "sphere_sphere_intersection_volume",
           "translate_points", "compute_intersection_volume_matrix_cuda", "compute_Ak_cuda",
           "compute_Ak_gradient_cuda"]


def load_lebedev(path: str):
    """(dirs, weights) -- reference returned (list of 3-arrays, list of floats)."""
    return _load_lebedev(path)


def build_kgrid(leb_dirs, leb_weights, n_radial: int) -> KGrid:
    return _build_kgrid(leb_dirs, leb_weights, n_radial)


def _identity(g: Geometry) -> SceneObject:
    return SceneObject(g, DOF_AFFINE, IDENTITY_AFFINE.copy())


def compute_intersection_volume_cuda(geom1: Geometry, geom2: Geometry, kgrid: KGrid, block_size: int = 256) -> float:
    """Intersection volume of two geometries on the GPU (identity AffineDoF),
    reference compute_intersection_volume.hpp:81-96 via bindings.cpp:72-77."""
    o1, o2 = _identity(geom1).as_c(), _identity(geom2).as_c()
    v = ctypes.c_double(0.0)
    _lib.check(_lib.lib().pi_pair_volume_host(ctypes.byref(o1), ctypes.byref(o2), kgrid.dirs.ctypes.data,
                                              kgrid.kmag.ctypes.data, kgrid.w.ctypes.data, kgrid.num_nodes,
                                              ctypes.byref(v)))
    return float(v.value)


def compute_intersection_volume_cpu(geom1: Geometry, geom2: Geometry, kgrid: KGrid) -> float:
    """Intersection volume of two geometries (identity AffineDoF), under the
    name of the reference's CPU binding (bindings.cpp:63-69).

    This build has no CPU compute path: the value comes from the same CUDA
    kernels as compute_intersection_volume_cuda, with the same arguments and
    result (FP32 form factors and contraction, 1e-5 relative to the FP64
    algorithm).  Callers that used it to cross-check the GPU get the GPU
    value twice; the FP64 cross-check lives in the test oracle."""
    return compute_intersection_volume_cuda(geom1, geom2, kgrid)


def compute_volume_cpu(geom: Geometry) -> float:
    """Divergence-theorem volume of one geometry (reference compute_volume.cpp:61-73)."""
    return self_volume(_identity(geom))


# ---------------------------------------------------------------------- additions
def compute_intersection_volume_matrix_cuda(geometries, kgrid: KGrid, block_size: int = 256,
                                            precision: str = "fp32", dofs=None, dof_types=None) -> np.ndarray:
    """n x n intersection-volume matrix (reference
    compute_intersection_volume_multi_object.hpp:51-59 / :78-98)."""
    from .core import volume_matrix_host
    objs = []
    for i, g in enumerate(geometries):
        dt = DOF_AFFINE if dof_types is None else dof_types[i]
        d = IDENTITY_AFFINE.copy() if dofs is None else dofs[i]
        objs.append(SceneObject(g, dt, d))
    return volume_matrix_host(kgrid, objs, precision)


def compute_Ak_gradient_cuda(geom: Geometry, k, dof_type: int = DOF_AFFINE, dofs=None) -> np.ndarray:
    """dA(k)/dtheta at one k-vector, complex128 of length n_dofs (reference
    compute_intersection_volume.hpp:129-135): 12 AffineDoF entries [t, A
    row-major] or 3V vertex coordinates; zeros at |k| < 1e-10."""
    obj = SceneObject(geom, dof_type, IDENTITY_AFFINE.copy() if dofs is None else dofs)
    c = obj.as_c()
    kv = np.ascontiguousarray(k, dtype=np.float64).reshape(3)
    out = np.zeros(2 * len(obj.dofs))
    _lib.check(_lib.lib().pi_compute_Ak_gradient_single(ctypes.byref(c), kv.ctypes.data, out.ctypes.data))
    return out.view(np.complex128).copy()


def compute_Ak_cuda(geom: Geometry, k, dof_type: int = DOF_AFFINE, dofs=None) -> complex:
    """A(k) at one k-vector (reference compute_intersection_volume.hpp:120-126)."""
    obj = SceneObject(geom, dof_type, IDENTITY_AFFINE.copy() if dofs is None else dofs).as_c()
    kv = np.ascontiguousarray(k, dtype=np.float64).reshape(3)
    out = np.zeros(2)
    _lib.check(_lib.lib().pi_compute_Ak_single(ctypes.byref(obj), kv.ctypes.data, out.ctypes.data))
    return complex(out[0], out[1])
