"""Device-resident layer over the C ABI, with PyTorch providing device memory
and streams.

    kg = standard_kgrid(59, 64)                     # N_k = 76,928
    batch = ObjectBatch([SceneObject(geom, DOF_AFFINE, dofs), ...])
    Jw = form_factors(kg, batch)                    # complex64 [n, Q], sqrt|w|-scaled
    V = contract(kg, Jw, "bf16x3")                  # float64 [n, n], 1/(8 pi^3) applied

Everything runs on the current torch CUDA stream; nothing synchronizes
implicitly.  There is no CPU path: the native library must be present.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from ._lib import CONTRACT_FP32, CONTRACT_BF16X3, CONTRACT_TF32X3
from .geometry import SceneObject
from .kgrid import KGrid

PRECISIONS = {"fp32": CONTRACT_FP32, "bf16x3": CONTRACT_BF16X3, "tf32x3": CONTRACT_TF32X3}


def _stream(stream=None) -> ctypes.c_void_p:
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def _precision(p) -> int:
    if isinstance(p, int):
        return p
    if p not in PRECISIONS:
        raise ValueError(f"precision must be one of {list(PRECISIONS)}")
    return PRECISIONS[p]


class ObjectBatch:
    """Objects transformed by their DoFs into the kernels' device layout
    (pi_batch).  Host objects are uploaded once; DoFs can be replaced in place."""

    def __init__(self, objects: list[SceneObject], stream=None):
        self.objects = list(objects)
        arr = (_lib.PiObject * max(1, len(self.objects)))(*[o.as_c() for o in self.objects])
        h = ctypes.c_void_p()
        _lib.check(_lib.lib().pi_batch_create(arr, len(self.objects), 0, _stream(stream), ctypes.byref(h)))
        self._handle = h

    def __len__(self) -> int:
        return len(self.objects)

    @property
    def handle(self):
        return self._handle

    def set_dofs(self, index: int, dofs: torch.Tensor, stream=None) -> None:
        """Replace object `index`'s DoF vector (float64 CUDA tensor) and re-transform it."""
        if not (dofs.is_cuda and dofs.dtype == torch.float64 and dofs.is_contiguous()):
            raise TypeError("dofs must be a contiguous float64 CUDA tensor")
        if dofs.numel() != len(self.objects[index].dofs):
            raise ValueError("DoF vector length must not change")
        _lib.check(_lib.lib().pi_batch_set_dofs(self._handle, int(index), ctypes.c_void_p(dofs.data_ptr()),
                                                _stream(stream)))

    def prepare(self, stream=None) -> None:
        """Re-run the DoF transform of every object (stream-ordered)."""
        _lib.check(_lib.lib().pi_batch_prepare(self._handle, _stream(stream)))

    def __del__(self):
        h = getattr(self, "_handle", None)
        if h is not None and _lib._lib is not None:
            try:
                _lib._lib.pi_batch_destroy(h)
            except Exception:
                pass


def form_factors(kgrid: KGrid, batch: ObjectBatch, scale_sqrt_w: bool = True, out: torch.Tensor | None = None,
                 stream=None) -> torch.Tensor:
    """J[n, q] = A_n(k_q) (times sqrt|w_q| when scale_sqrt_w), complex64 on the device."""
    Q = kgrid.num_nodes
    n = len(batch)
    if out is None:
        out = torch.empty((n, Q), dtype=torch.complex64, device="cuda")
    if out.shape != (n, Q) or out.dtype != torch.complex64 or not out.is_contiguous():
        raise ValueError("out must be a contiguous complex64 tensor of shape (n_objects, Q)")
    _lib.check(_lib.lib().pi_form_factors(kgrid.handle(), batch.handle, int(bool(scale_sqrt_w)),
                                          ctypes.c_void_p(out.data_ptr()), _stream(stream)))
    return out


class Workspace:
    """Grow-only device scratch for the contraction."""

    def __init__(self):
        self.buf = None

    def get(self, nbytes: int) -> torch.Tensor:
        if self.buf is None or self.buf.numel() < nbytes:
            self.buf = torch.empty(max(nbytes, 16), dtype=torch.uint8, device="cuda")
        return self.buf


_default_ws = Workspace()


def contract_workspace_size(kgrid: KGrid, n: int, precision="fp32") -> int:
    sz = ctypes.c_size_t(0)
    _lib.check(_lib.lib().pi_contract_workspace_size(kgrid.handle(), int(n), _precision(precision), ctypes.byref(sz)))
    return int(sz.value)


def contract(kgrid: KGrid, Jw: torch.Tensor, precision="fp32", out: torch.Tensor | None = None,
             workspace: Workspace | None = None, stream=None) -> torch.Tensor:
    """V = Re(J^H diag(w) J) / (8 pi^3) from the sqrt|w|-scaled J; float64 [n, n]."""
    if Jw.dtype != torch.complex64 or not Jw.is_contiguous() or Jw.dim() != 2 or Jw.shape[1] != kgrid.num_nodes:
        raise ValueError("Jw must be a contiguous complex64 tensor of shape (n_objects, Q)")
    n = Jw.shape[0]
    p = _precision(precision)
    if out is None:
        out = torch.empty((n, n), dtype=torch.float64, device="cuda")
    ws = (workspace or _default_ws).get(contract_workspace_size(kgrid, n, p))
    _lib.check(_lib.lib().pi_contract(kgrid.handle(), ctypes.c_void_p(Jw.data_ptr()), int(n), p,
                                      ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(ws.data_ptr()),
                                      ctypes.c_size_t(ws.numel()), _stream(stream)))
    return out


def volume_matrix(kgrid: KGrid, objects, precision="fp32") -> torch.Tensor:
    """Cold volume matrix: form factors + contraction (device tensors)."""
    batch = objects if isinstance(objects, ObjectBatch) else ObjectBatch(objects)
    Jw = form_factors(kgrid, batch, True)
    return contract(kgrid, Jw, precision)


def volume_matrix_host(kgrid: KGrid, objects: list[SceneObject], precision="fp32") -> np.ndarray:
    """The one-shot host-buffer entry point (pi_volume_matrix_host): host in, host out."""
    n = len(objects)
    V = np.zeros((n, n))
    arr = (_lib.PiObject * max(1, n))(*[o.as_c() for o in objects])
    _lib.check(_lib.lib().pi_volume_matrix_host(arr, n, kgrid.dirs.ctypes.data, kgrid.kmag.ctypes.data,
                                                kgrid.w.ctypes.data, kgrid.num_nodes, _lib.VOLUME_ONLY,
                                                _precision(precision), V.ctypes.data))
    return V
