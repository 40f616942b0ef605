"""ctypes binding to libpointint_gb300.so (the C ABI in include/pointint_gb300.h).

There is no fallback: if the library is missing, importing the compute entry
points raises.  Build it with ``python -m pointint_gb300.build`` or
``__graft_entry__.build()``.
"""
from __future__ import annotations

import ctypes
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libpointint_gb300.so")

PI_OK = 0
STATUS_NAMES = {0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "unsupported", 4: "out of memory",
                5: "not found", 6: "workspace too small", 7: "I/O error", 8: "timeout"}

GEOM_TRIANGLE, GEOM_DISK, GEOM_GAUSSIAN = 0, 1, 2
DOF_AFFINE, DOF_TRIANGLE_MESH = 0, 1
VOLUME_ONLY, GRADIENT, HESSIAN, ALL = 1, 2, 4, 7
CONTRACT_FP32, CONTRACT_BF16X3, CONTRACT_TF32X3, CONTRACT_FP16X3 = 0, 1, 2, 3


class PointIntError(RuntimeError):
    """A non-zero status from the C ABI."""

    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class PiObject(ctypes.Structure):
    """pi_object: packed elements + DoF type + DoF vector (host or device pointers)."""
    _fields_ = [("geom_type", ctypes.c_int32), ("dof_type", ctypes.c_int32),
                ("n_elems", ctypes.c_int64), ("elems", ctypes.c_void_p),
                ("n_dofs", ctypes.c_int64), ("dofs", ctypes.c_void_p)]


class ServerConfig(ctypes.Structure):
    """pi_server_config (zero fields take the library's defaults)."""
    _fields_ = [("hbm_budget_bytes", ctypes.c_int64), ("max_batch_queries", ctypes.c_int32),
                ("max_batch_rows", ctypes.c_int32), ("max_batch_evals", ctypes.c_int32),
                ("inflight_batches", ctypes.c_int32), ("precision", ctypes.c_int32),
                ("use_graphs", ctypes.c_int32), ("autotune", ctypes.c_int32), ("items_per_sm_x4", ctypes.c_int32)]


class Query(ctypes.Structure):
    """pi_query: library indices + optional per-object rotations (n x 9) and translations (n x 3)."""
    _fields_ = [("n_objects", ctypes.c_int32), ("reserved_", ctypes.c_int32), ("objects", ctypes.c_void_p),
                ("rotations", ctypes.c_void_p), ("translations", ctypes.c_void_p)]


class ServerStats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int64) for n in ("submitted", "completed", "failed", "cancelled", "batches",
                                             "evaluations", "resident_hits", "resident_misses", "evictions",
                                             "pool_rows", "resident_rows", "graph_launches")] + \
               [("tuned_items_per_sm", ctypes.c_int32 * 4), ("tuned_k_splits", ctypes.c_int32 * 4)]


class OptimizationState(ctypes.Structure):
    """pi_optimization_state (the reference's OptimizationState plus two counters)."""
    _fields_ = [("dofs", ctypes.c_double * 12), ("similarity", ctypes.c_double), ("similarity_loss", ctypes.c_double),
                ("iteration", ctypes.c_int32), ("converged", ctypes.c_int32), ("steps", ctypes.c_int32),
                ("evaluations", ctypes.c_int32), ("status", ctypes.c_char * 64)]


SIM_OCHIAI, SIM_JACCARD, SIM_DICE = 0, 1, 2
SIM_FUNC_ONLY, SIM_GRADIENT, SIM_HESSIAN, SIM_FUNC_GRAD, SIM_ALL = 1, 2, 4, 3, 7

QUERY_PENDING, QUERY_RUNNING, QUERY_DONE, QUERY_FAILED, QUERY_CANCELLED = 0, 1, 2, 3, 4

_lock = threading.Lock()
_lib = None

P, I32, I64, D, SZ = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_double, ctypes.c_size_t
PP = ctypes.POINTER(ctypes.c_void_p)
OBJP = ctypes.POINTER(PiObject)

# name -> (restype, argtypes); every symbol declared in include/pointint_gb300.h
SIGNATURES = {
    "pi_status_string": (ctypes.c_char_p, [I32]),
    "pi_last_error": (ctypes.c_char_p, []),
    "pi_version": (I32, []),
    "pi_launch_count": (I64, []),
    "pi_gauss_legendre": (I32, [I32, D, D, P, P]),
    "pi_load_lebedev": (I32, [ctypes.c_char_p, P, P, I64, ctypes.POINTER(I64)]),
    "pi_build_kgrid": (I32, [P, P, I64, I32, P, P, P]),
    "pi_pack_tris": (I32, [P, I64, P, I64, P]),
    "pi_pack_disks": (I32, [P, P, P, I64, I32, P]),
    "pi_pack_gaussians": (I32, [P, P, P, P, I64, P]),
    "pi_create_unit_cube_mesh": (I32, [P, P]),
    "pi_create_sphere_pointcloud": (I32, [I32, P, P, P]),
    "pi_create_sphere_gaussians": (I32, [I32, P, P, P, P]),
    "pi_box_box_intersection_volume": (D, [P, P, P, P]),
    "pi_sphere_sphere_intersection_volume": (D, [P, D, P, D]),
    "pi_self_volume": (I32, [OBJP, ctypes.POINTER(D)]),
    "pi_kgrid_create": (I32, [P, P, P, I64, PP]),
    "pi_kgrid_destroy": (I32, [P]),
    "pi_kgrid_info": (I32, [P, ctypes.POINTER(I64), ctypes.POINTER(I64), ctypes.POINTER(I64)]),
    "pi_kgrid_direction_pairs": (I32, [P, P, I64, P, I64, ctypes.POINTER(I64)]),
    "pi_batch_create": (I32, [OBJP, I32, I32, P, PP]),
    "pi_batch_set_dofs": (I32, [P, I32, P, P]),
    "pi_batch_prepare": (I32, [P, P]),
    "pi_batch_set_all_dofs": (I32, [P, P, P]),
    "pi_batch_destroy": (I32, [P]),
    "pi_batch_count": (I32, [P, ctypes.POINTER(I32)]),
    "pi_form_factors": (I32, [P, P, I32, P, P]),
    "pi_form_factors_rowmax": (I32, [P, P, I32, P, P, P]),
    "pi_contract_rowmax": (I32, [P, P, P, I32, I32, P, P, SZ, P]),
    "pi_contract_error": (I32, [I32, P, P]),
    "pi_test_set_contract_faults": (I32, [I64, I64]),
    "pi_contract_workspace_size": (I32, [P, I32, I32, ctypes.POINTER(SZ)]),
    "pi_contract": (I32, [P, P, I32, I32, P, P, SZ, P]),
    "pi_contract_fp32_static": (I32, [P, I64, I32, P, P, P]),
    "pi_batch_set_elements": (I32, [P, I32, P, P]),
    "pi_batch_layout": (I32, [P, I32, ctypes.POINTER(I64), ctypes.POINTER(I64), ctypes.POINTER(I64)]),
    "pi_adjoint_workspace_size": (I32, [P, P, ctypes.POINTER(SZ)]),
    "pi_element_gradients": (I32, [P, P, P, P, P, P, P, SZ, P]),
    "pi_dof_gradients": (I32, [P, P, P, P, P, P, SZ, P]),
    "pi_pair_volume_grad_host": (I32, [OBJP, OBJP, P, P, P, I64, ctypes.POINTER(D), P, P]),
    "pi_volume_matrix_grad_host": (I32, [OBJP, I32, P, P, P, I64, P, P]),
    "pi_dof_jacobian": (I32, [P, P, P, P]),
    "pi_volume_matrix_hessian_host": (I32, [OBJP, I32, P, P, P, I64, P, P, P]),
    "pi_pair_volume_hessian_host": (I32, [OBJP, OBJP, P, P, P, I64, ctypes.POINTER(D), P, P, P, P, P]),
    "pi_volume_matrix_host": (I32, [OBJP, I32, P, P, P, I64, I32, I32, P]),
    "pi_pair_volume_host": (I32, [OBJP, OBJP, P, P, P, I64, ctypes.POINTER(D)]),
    "pi_compute_Ak": (I32, [OBJP, P, P, I64, P, I32]),
    "pi_compute_Ak_single": (I32, [OBJP, P, P]),
    "pi_compute_Ak_gradient": (I32, [OBJP, P, P, I64, P, I32]),
    "pi_compute_Ak_gradient_single": (I32, [OBJP, P, P]),
    "pi_server_create": (I32, [P, OBJP, I32, ctypes.POINTER(ServerConfig), PP]),
    "pi_server_submit": (I32, [P, ctypes.POINTER(Query), P, ctypes.POINTER(ctypes.c_uint64)]),
    "pi_server_poll": (I32, [P, ctypes.c_uint64, ctypes.POINTER(ctypes.c_int32)]),
    "pi_server_wait": (I32, [P, ctypes.c_uint64, D]),
    "pi_server_cancel": (I32, [P, ctypes.c_uint64]),
    "pi_server_times": (I32, [P, ctypes.c_uint64, ctypes.POINTER(I64), ctypes.POINTER(I64), ctypes.POINTER(I64)]),
    "pi_server_release": (I32, [P, ctypes.c_uint64]),
    "pi_server_stats_get": (I32, [P, ctypes.POINTER(ServerStats)]),
    "pi_server_destroy": (I32, [P]),
    "pi_aligner_create": (I32, [OBJP, OBJP, P, P, P, I64, PP]),
    "pi_aligner_destroy": (I32, [P]),
    "pi_aligner_fixed_volume": (I32, [P, ctypes.POINTER(D)]),
    "pi_similarity": (I32, [P, P, I32, D, I32, ctypes.POINTER(D), ctypes.POINTER(D), P, P]),
    "pi_optimize_alignment": (I32, [P, P, I32, D, D, I32, D, ctypes.POINTER(OptimizationState)]),
    "pi_compute_moments": (I32, [OBJP, P, ctypes.POINTER(D), P, P]),
    "pi_compute_warm_start": (I32, [OBJP, OBJP, P]),
}


def lib_exists() -> bool:
    return os.path.exists(LIB_PATH)


def lib() -> ctypes.CDLL:
    """Load the library (no implicit build, no fallback)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise ImportError(
                    f"{LIB_PATH} is missing: build it with `python -m pointint_gb300.build` "
                    "(the GB300 path has no CPU fallback)")
            L = ctypes.CDLL(LIB_PATH)
            for name, (res, args) in SIGNATURES.items():
                f = getattr(L, name)
                f.restype = res
                f.argtypes = args
            _lib = L
        return _lib


def check(rc: int) -> None:
    if rc != PI_OK:
        msg = lib().pi_last_error()
        raise PointIntError(rc, msg.decode() if msg else "")


def launch_count() -> int:
    return int(lib().pi_launch_count())
