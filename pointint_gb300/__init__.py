"""pointint_gb300: GB300-native (sm_103a) Fourier intersection-volume path.

A drop-in for PoIntInt's Fourier path: per-object form factors over a
Gauss-Legendre x Lebedev k-grid, the pairwise contraction V = Re(J^H D J), and
the adjoint for gradients, behind the C ABI in include/pointint_gb300.h.
"""
from ._lib import (PointIntError, GEOM_TRIANGLE, GEOM_DISK, GEOM_GAUSSIAN, DOF_AFFINE, DOF_TRIANGLE_MESH,
                   VOLUME_ONLY, GRADIENT, HESSIAN, ALL, CONTRACT_FP32, CONTRACT_BF16X3, CONTRACT_TF32X3, CONTRACT_FP16X3, lib, lib_exists,
                   launch_count)
from .geometry import (Geometry, SceneObject, make_triangle_mesh, make_point_cloud, make_gaussian_splat,
                       create_unit_cube_mesh, create_sphere_pointcloud, create_sphere_gaussians, pack_tris,
                       pack_disks, pack_gaussians, IDENTITY_AFFINE, TRI_DTYPE, DISK_DTYPE, GAUSS_DTYPE)
from .kgrid import KGrid, build_kgrid, load_lebedev, standard_kgrid, lebedev_path, gauss_legendre

__version__ = "0.1.0"
