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
from ._lib import CONTRACT_FP32, CONTRACT_BF16X3, CONTRACT_TF32X3, CONTRACT_FP16X3
from .geometry import SceneObject
from .kgrid import KGrid

PRECISIONS = {"fp32": CONTRACT_FP32, "bf16x3": CONTRACT_BF16X3, "tf32x3": CONTRACT_TF32X3, "fp16x3": CONTRACT_FP16X3}


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

    def set_all_dofs(self, dofs: torch.Tensor, stream=None) -> None:
        """Replace every DoF vector (float64 CUDA tensor, concatenated in object order)."""
        if not (dofs.is_cuda and dofs.dtype == torch.float64):
            raise TypeError("dofs must be a float64 CUDA tensor")
        d = dofs.detach().contiguous()
        if d.numel() != sum(len(o.dofs) for o in self.objects):
            raise ValueError("wrong DoF count")
        _lib.check(_lib.lib().pi_batch_set_all_dofs(self._handle, ctypes.c_void_p(d.data_ptr()), _stream(stream)))

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
                 stream=None, row_amax: torch.Tensor | None = None) -> torch.Tensor:
    """J[n, q] = A_n(k_q) (times sqrt|w_q| when scale_sqrt_w), complex64 on the device.
    With row_amax (float32 [n] CUDA tensor) each row's largest |Re|, |Im| is
    written there too, for contract(..., row_amax=...)."""
    Q = kgrid.num_nodes
    n = len(batch)
    if out is None:
        out = torch.empty((n, Q), dtype=torch.complex64, device="cuda")
    if out.shape != (n, Q) or out.dtype != torch.complex64 or not out.is_contiguous():
        raise ValueError("out must be a contiguous complex64 tensor of shape (n_objects, Q)")
    if row_amax is None:
        _lib.check(_lib.lib().pi_form_factors(kgrid.handle(), batch.handle, int(bool(scale_sqrt_w)),
                                              ctypes.c_void_p(out.data_ptr()), _stream(stream)))
    else:
        _check_amax(row_amax, n)
        _lib.check(_lib.lib().pi_form_factors_rowmax(kgrid.handle(), batch.handle, int(bool(scale_sqrt_w)),
                                                     ctypes.c_void_p(out.data_ptr()),
                                                     ctypes.c_void_p(row_amax.data_ptr()), _stream(stream)))
    return out


def _check_amax(row_amax: torch.Tensor, n: int) -> None:
    if not (row_amax.is_cuda and row_amax.dtype == torch.float32 and row_amax.is_contiguous()
            and row_amax.numel() == n):
        raise ValueError("row_amax must be a contiguous float32 CUDA tensor of n_objects entries")


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
             workspace: Workspace | None = None, stream=None, row_amax: torch.Tensor | None = None) -> torch.Tensor:
    """V = Re(J^H diag(w) J) / (8 pi^3) from the sqrt|w|-scaled J; float64 [n, n].
    row_amax: the rows' maxima from form_factors(..., row_amax=...), which spares
    the FP16-split contraction a pass over J."""
    if Jw.dtype != torch.complex64 or not Jw.is_contiguous() or Jw.dim() != 2 or Jw.shape[1] != kgrid.num_nodes:
        raise ValueError("Jw must be a contiguous complex64 tensor of shape (n_objects, Q)")
    n = Jw.shape[0]
    p = _precision(precision)
    if out is None:
        out = torch.empty((n, n), dtype=torch.float64, device="cuda")
    ws = (workspace or _default_ws).get(contract_workspace_size(kgrid, n, p))
    if row_amax is not None:
        _check_amax(row_amax, n)
    _lib.check(_lib.lib().pi_contract_rowmax(kgrid.handle(), ctypes.c_void_p(Jw.data_ptr()),
                                             ctypes.c_void_p(row_amax.data_ptr()) if row_amax is not None else None,
                                             int(n), p, ctypes.c_void_p(out.data_ptr()),
                                             ctypes.c_void_p(ws.data_ptr()), ctypes.c_size_t(ws.numel()),
                                             _stream(stream)))
    return out


def volume_matrix(kgrid: KGrid, objects, precision="fp32") -> torch.Tensor:
    """Cold volume matrix: form factors + contraction (device tensors)."""
    batch = objects if isinstance(objects, ObjectBatch) else ObjectBatch(objects)
    amax = torch.empty(len(batch), dtype=torch.float32, device="cuda")
    Jw = form_factors(kgrid, batch, True, row_amax=amax)
    return contract(kgrid, Jw, precision, row_amax=amax)


def volume_matrix_host(kgrid: KGrid, objects: list[SceneObject], precision="fp32") -> np.ndarray:
    """The one-shot host-buffer entry point (pi_volume_matrix_host): host in, host out."""
    n = len(objects)
    V = np.zeros((n, n))
    arr = (_lib.PiObject * max(1, n))(*[o.as_c() for o in objects])
    _lib.check(_lib.lib().pi_volume_matrix_host(arr, n, kgrid.dirs.ctypes.data, kgrid.kmag.ctypes.data,
                                                kgrid.w.ctypes.data, kgrid.num_nodes, _lib.VOLUME_ONLY,
                                                _precision(precision), V.ctypes.data))
    return V


# ----------------------------------------------------------------------------- gradients
def adjoint_workspace_size(kgrid: KGrid, batch: ObjectBatch) -> int:
    sz = ctypes.c_size_t(0)
    _lib.check(_lib.lib().pi_adjoint_workspace_size(kgrid.handle(), batch.handle, ctypes.byref(sz)))
    return int(sz.value)


def _w64(W, n) -> np.ndarray:
    W = np.ascontiguousarray(np.asarray(W, dtype=np.float64))
    if W.shape != (n, n):
        raise ValueError(f"cotangent weights must be {n} x {n}")
    return W


def element_gradients(kgrid: KGrid, batch: ObjectBatch, Jw: torch.Tensor, W, workspace: Workspace | None = None,
                      stream=None):
    """Per-element gradients for cotangents B_i = sum_j W_ij A_j (W = C + C^T for
    L = sum C_ij V_ij).  Returns (tri [n_tri, 9], surf [n_surf, 12]) float32
    tensors in pool (object) order: triangles dL/dv0,dv1,dv2; surfels dL/dc,
    dL/dn', dL/dM(6)."""
    n = len(batch)
    W = _w64(W, n)
    n_tri = sum(o.geom.num_elements() for o in batch.objects if o.geom.type == _lib.GEOM_TRIANGLE)
    n_surf = sum(o.geom.num_elements() for o in batch.objects if o.geom.type != _lib.GEOM_TRIANGLE)
    tri = torch.empty((max(n_tri, 1), 9), dtype=torch.float32, device="cuda")
    surf = torch.empty((max(n_surf, 1), 12), dtype=torch.float32, device="cuda")
    ws = (workspace or _default_ws).get(adjoint_workspace_size(kgrid, batch))
    _lib.check(_lib.lib().pi_element_gradients(kgrid.handle(), batch.handle, ctypes.c_void_p(Jw.data_ptr()),
                                               W.ctypes.data, ctypes.c_void_p(tri.data_ptr()),
                                               ctypes.c_void_p(surf.data_ptr()), ctypes.c_void_p(ws.data_ptr()),
                                               ctypes.c_size_t(ws.numel()), _stream(stream)))
    return tri[:n_tri], surf[:n_surf]


def dof_gradients(kgrid: KGrid, batch: ObjectBatch, Jw: torch.Tensor, W, workspace: Workspace | None = None,
                  stream=None) -> torch.Tensor:
    """DoF gradients of every object, concatenated in object order (float64)."""
    n = len(batch)
    W = _w64(W, n)
    nd = sum(len(o.dofs) for o in batch.objects)
    g = torch.empty(max(nd, 1), dtype=torch.float64, device="cuda")
    ws = (workspace or _default_ws).get(adjoint_workspace_size(kgrid, batch))
    _lib.check(_lib.lib().pi_dof_gradients(kgrid.handle(), batch.handle, ctypes.c_void_p(Jw.data_ptr()), W.ctypes.data,
                                           ctypes.c_void_p(g.data_ptr()), ctypes.c_void_p(ws.data_ptr()),
                                           ctypes.c_size_t(ws.numel()), _stream(stream)))
    return g[:nd]


def pair_volume_grad_host(kgrid: KGrid, o1: SceneObject, o2: SceneObject):
    """Reference compute_intersection_volume_cuda(..., GRADIENT): (volume, grad1, grad2)."""
    c1, c2 = o1.as_c(), o2.as_c()
    v = ctypes.c_double(0.0)
    g1, g2 = np.zeros(len(o1.dofs)), np.zeros(len(o2.dofs))
    _lib.check(_lib.lib().pi_pair_volume_grad_host(ctypes.byref(c1), ctypes.byref(c2), kgrid.dirs.ctypes.data,
                                                   kgrid.kmag.ctypes.data, kgrid.w.ctypes.data, kgrid.num_nodes,
                                                   ctypes.byref(v), g1.ctypes.data, g2.ctypes.data))
    return float(v.value), g1, g2


def volume_matrix_grad_host(kgrid: KGrid, objects: list[SceneObject]):
    """Reference compute_intersection_volume_matrix_cuda(..., GRADIENT): (V, grad)
    with grad[i][j] = dV_ij/dtheta_i."""
    n = len(objects)
    nd = [len(o.dofs) for o in objects]
    V = np.zeros((n, n))
    g = np.zeros(max(1, n * sum(nd)))
    arr = (_lib.PiObject * n)(*[o.as_c() for o in objects])
    _lib.check(_lib.lib().pi_volume_matrix_grad_host(arr, n, kgrid.dirs.ctypes.data, kgrid.kmag.ctypes.data,
                                                     kgrid.w.ctypes.data, kgrid.num_nodes, V.ctypes.data,
                                                     g.ctypes.data))
    grad, off = [], 0
    for i in range(n):
        grad.append([g[off + j * nd[i]: off + (j + 1) * nd[i]].copy() for j in range(n)])
        off += n * nd[i]
    return V, grad


# ----------------------------------------------------------------------------- Gauss-Newton Hessian
def dof_jacobian(kgrid: KGrid, batch: ObjectBatch, out: torch.Tensor | None = None, stream=None) -> torch.Tensor:
    """G[d, q] = sqrt|w_q| dA(k_q)/dtheta_d over the concatenated DoF vector
    (complex64 [D, Q] on the device).  contract(kgrid, G) is the full
    Gauss-Newton Hessian; contract of the stack [J; G] adds V and dV/dtheta."""
    D = sum(len(o.dofs) for o in batch.objects)
    Q = kgrid.num_nodes
    if out is None:
        out = torch.empty((D, Q), dtype=torch.complex64, device="cuda")
    if out.shape != (D, Q) or out.dtype != torch.complex64 or not out.is_contiguous():
        raise ValueError("out must be a contiguous complex64 tensor of shape (n_dofs_total, Q)")
    _lib.check(_lib.lib().pi_dof_jacobian(kgrid.handle(), batch.handle, ctypes.c_void_p(out.data_ptr()),
                                          _stream(stream)))
    return out


def volume_matrix_hessian_host(kgrid: KGrid, objects: list[SceneObject]):
    """Reference compute_intersection_volume_matrix_cuda(..., GRADIENT | HESSIAN):
    (V, grad, hess) with grad[i][j] = dV_ij/dtheta_i and hess[i][j] the
    Gauss-Newton block hessian_ij (n_dofs[i] x n_dofs[j])."""
    n = len(objects)
    nd = [len(o.dofs) for o in objects]
    V = np.zeros((n, n))
    g = np.zeros(max(1, n * sum(nd)))
    h = np.zeros(max(1, sum(a * b for a in nd for b in nd)))
    arr = (_lib.PiObject * n)(*[o.as_c() for o in objects])
    _lib.check(_lib.lib().pi_volume_matrix_hessian_host(arr, n, kgrid.dirs.ctypes.data, kgrid.kmag.ctypes.data,
                                                        kgrid.w.ctypes.data, kgrid.num_nodes, V.ctypes.data,
                                                        g.ctypes.data, h.ctypes.data))
    grad, off = [], 0
    for i in range(n):
        grad.append([g[off + j * nd[i]: off + (j + 1) * nd[i]].copy() for j in range(n)])
        off += n * nd[i]
    hess, off = [[None] * n for _ in range(n)], 0
    for i in range(n):
        for j in range(n):
            hess[i][j] = h[off: off + nd[i] * nd[j]].reshape(nd[i], nd[j]).copy()
            off += nd[i] * nd[j]
    return V, grad, hess


def pair_volume_hessian_host(kgrid: KGrid, o1: SceneObject, o2: SceneObject) -> dict:
    """Reference compute_intersection_volume_cuda(..., GRADIENT | HESSIAN) as a
    dict with the reference's result field names."""
    c1, c2 = o1.as_c(), o2.as_c()
    d1, d2 = len(o1.dofs), len(o2.dofs)
    v = ctypes.c_double(0.0)
    g1, g2 = np.zeros(d1), np.zeros(d2)
    H11, H22, H12 = np.zeros((d1, d1)), np.zeros((d2, d2)), np.zeros((d1, d2))
    _lib.check(_lib.lib().pi_pair_volume_hessian_host(ctypes.byref(c1), ctypes.byref(c2), kgrid.dirs.ctypes.data,
                                                      kgrid.kmag.ctypes.data, kgrid.w.ctypes.data, kgrid.num_nodes,
                                                      ctypes.byref(v), g1.ctypes.data, g2.ctypes.data,
                                                      H11.ctypes.data, H22.ctypes.data, H12.ctypes.data))
    return {"volume": float(v.value), "grad_geom1": g1, "grad_geom2": g2, "hessian_geom1": H11,
            "hessian_geom2": H22, "hessian_cross": H12}


class _DofVolumeFn(torch.autograd.Function):
    """V(theta) for all DoFs theta (concatenated), backward through the adjoint."""

    @staticmethod
    def forward(ctx, scene, dofs):
        scene.batch.set_all_dofs(dofs)
        Jw = form_factors(scene.kgrid, scene.batch, True)
        V = contract(scene.kgrid, Jw, scene.precision)
        ctx.scene, ctx.Jw = scene, Jw
        return V

    @staticmethod
    def backward(ctx, gV):
        G = gV.detach().double().cpu().numpy()
        g = dof_gradients(ctx.scene.kgrid, ctx.scene.batch, ctx.Jw, G + G.T)
        return None, g


class _SurfelVolumeFn(torch.autograd.Function):
    """V(c, n) for surfel-only scenes; gradients w.r.t. every disk / Gaussian
    centre and (unnormalised) normal through the adjoint."""

    @staticmethod
    def forward(ctx, scene, c, n):
        scene.set_surfels(c, n)
        Jw = form_factors(scene.kgrid, scene.batch, True)
        V = contract(scene.kgrid, Jw, scene.precision)
        ctx.scene, ctx.Jw = scene, Jw
        return V

    @staticmethod
    def backward(ctx, gV):
        G = gV.detach().double().cpu().numpy()
        _, surf = element_gradients(ctx.scene.kgrid, ctx.scene.batch, ctx.Jw, G + G.T)
        return None, surf[:, 0:3].double(), surf[:, 3:6].double()


class Scene:
    """Device-resident objects + k-grid with differentiable volume matrices.

        scene = Scene(kgrid, objects)
        V = scene.volume_matrix_of_dofs(theta)        # theta: concatenated DoFs, requires_grad
        V = scene.volume_matrix_of_surfels(c, n)       # surfel scenes: centres / normals
        V.sum().backward()
    """

    def __init__(self, kgrid: KGrid, objects: list[SceneObject], precision="fp32"):
        self.kgrid = kgrid
        self.objects = list(objects)
        self.batch = ObjectBatch(self.objects)
        self.precision = precision
        self.counts = [o.geom.num_elements() for o in self.objects]
        self._packed = None

    def dofs(self) -> torch.Tensor:
        return torch.tensor(np.concatenate([o.dofs for o in self.objects]), dtype=torch.float64, device="cuda")

    def volume_matrix_of_dofs(self, dofs: torch.Tensor) -> torch.Tensor:
        return _DofVolumeFn.apply(self, dofs)

    def _surfel_rows(self) -> np.ndarray:
        """Every surfel's 64-byte record as 8 doubles (c, n, rho|sigma, area|w),
        in object order; disks and Gaussians share the layout."""
        return np.concatenate([o.geom.elems.view(np.float64).reshape(-1, 8) for o in self.objects])

    def surfel_params(self):
        """Current (c, n) of every surfel, concatenated in object order (float64 CUDA)."""
        e = self._surfel_rows()
        c = torch.tensor(np.ascontiguousarray(e[:, 0:3]), device="cuda")
        n = torch.tensor(np.ascontiguousarray(e[:, 3:6]), device="cuda")
        return c, n

    def set_surfels(self, c: torch.Tensor, n: torch.Tensor) -> None:
        if any(o.geom.type == _lib.GEOM_TRIANGLE for o in self.objects):
            raise TypeError("surfel parameters apply to disk / Gaussian scenes only")
        if self._packed is None:
            self._packed = torch.tensor(self._surfel_rows(), device="cuda")
        self._packed[:, 0:3] = c.detach()
        self._packed[:, 3:6] = n.detach()
        off = 0
        s = _stream(None)
        for i, cnt in enumerate(self.counts):
            _lib.check(_lib.lib().pi_batch_set_elements(self.batch.handle, i,
                                                        ctypes.c_void_p(self._packed[off].data_ptr()) if cnt else None,
                                                        s))
            off += cnt

    def volume_matrix_of_surfels(self, c: torch.Tensor, n: torch.Tensor) -> torch.Tensor:
        return _SurfelVolumeFn.apply(self, c, n)
