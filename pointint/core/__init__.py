"""pointint.core: the Fourier intersection-volume path, as a torch layer.

The reference package of this name (pointint/core/api.py) held a Warp
direct-sum method whose kernel module is absent from the reference, so it does
not import as shipped.  Here the same entry points (``get_mesh_intersection_volume``,
``get_ptcld_intersection_volume``) compute the Fourier volume on the GPU, and
the device-resident layer of the GB300 library is re-exported beside them:

    import pointint.core as pc
    kg = pc.standard_kgrid(59, 64)                  # N_k = 76,928
    V = pc.volume_matrix(kg, objects, "fp16x3")    # float64 [n, n] CUDA tensor
    scene = pc.Scene(kg, objects)                  # autograd through the adjoint kernels

Everything runs on the current torch CUDA stream; there is no CPU path.
"""
from pointint_gb300.core import (ObjectBatch, Scene, Workspace, contract, contract_workspace_size, dof_gradients,
                                 dof_jacobian, element_gradients, form_factors, pair_volume_grad_host,
                                 pair_volume_hessian_host, volume_matrix, volume_matrix_grad_host,
                                 volume_matrix_hessian_host, volume_matrix_host, PRECISIONS)
from pointint_gb300.geometry import (Geometry, SceneObject, affine_dofs, make_gaussian_splat, make_point_cloud,
                                     make_triangle_mesh)
from pointint_gb300.kgrid import KGrid, build_kgrid, lebedev_path, load_lebedev, standard_kgrid
from pointint_gb300.serving import Server

from .api import (default_kgrid, get_mesh_intersection_volume, get_ptcld_intersection_volume, knn_area_weights,
                  mesh_intersection_volume, ptcld_intersection_volume)

__all__ = ["ObjectBatch", "Scene", "Workspace", "contract", "contract_workspace_size", "dof_gradients",
           "dof_jacobian", "element_gradients", "form_factors", "pair_volume_grad_host", "pair_volume_hessian_host",
           "volume_matrix", "volume_matrix_grad_host", "volume_matrix_hessian_host", "volume_matrix_host",
           "PRECISIONS", "Geometry", "SceneObject", "affine_dofs", "make_gaussian_splat", "make_point_cloud",
           "make_triangle_mesh", "KGrid", "build_kgrid", "lebedev_path", "load_lebedev", "standard_kgrid", "Server",
           "default_kgrid", "get_mesh_intersection_volume", "get_ptcld_intersection_volume", "knn_area_weights",
           "mesh_intersection_volume", "ptcld_intersection_volume"]
