"""The allocation-free contraction entry point, pi_contract_fp32_static.

It exists for callers that cannot call cudaMalloc: an application whose device
memory belongs to a host framework's pre-reserved pool, or a latency-critical
loop in which an allocation would synchronise the device.  It keeps its split-K
scratch in a fixed 8 MiB device array inside the library.  This file is
collected last, so a run that stops at the first failure has already run every
other test; it also passes on its own in a fresh process.
"""
import ctypes

import numpy as np
import pytest
import torch

import pointint_gb300 as pg
from pointint_gb300 import _lib, core, geometry as G
from pointint_gb300.kgrid import KGrid, standard_kgrid

pytestmark = pytest.mark.gpu


def _objects(rng, n):
    V, F = G.icosphere(2)
    out = []
    for _ in range(n):
        A = G.random_rotation(rng) @ np.diag(rng.uniform(0.5, 1.5, 3))
        out.append(G.SceneObject(G.make_triangle_mesh(V, F), pg.DOF_AFFINE, G.affine_dofs(A, rng.uniform(0, 3, 3))))
    return out


def _static(Jw, Q, n, sign, V):
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    return _lib.lib().pi_contract_fp32_static(ctypes.c_void_p(Jw.data_ptr()), Q, n,
                                              ctypes.c_void_p(sign.data_ptr()) if sign is not None else None,
                                              ctypes.c_void_p(V.data_ptr()), stream)


@pytest.mark.parametrize("negative_weights", [False, True])
def test_static_contraction_matches_workspace_entry_point(cuda, negative_weights):
    rng = np.random.default_rng(17)
    kg = standard_kgrid(29, 32)
    if negative_weights:  # flip some quadrature weights to exercise the sign path
        w = kg.w.copy()
        w[::5] *= -1.0
        kg = KGrid(kg.dirs, kg.kmag, w)
    n = 70  # not a multiple of the 64-object tile
    Jw = core.form_factors(kg, core.ObjectBatch(_objects(rng, n)), True)
    ref = core.contract(kg, Jw, "fp32")  # the entry point with a caller workspace
    sign = torch.tensor(np.sign(kg.w), dtype=torch.float32, device="cuda") if negative_weights else None
    for call in range(2):  # two calls in a row share the array
        V = torch.full((n, n), float("nan"), dtype=torch.float64, device="cuda")
        _lib.check(_static(Jw, kg.num_nodes, n, sign, V))
        torch.cuda.synchronize()
        err = (V - ref).abs().max().item() / ref.abs().max().item()
        assert torch.isfinite(V).all(), call
        assert err <= 1e-12, (call, err)  # same kernels, same split plan: identical sums


def _cond_err(V, R):
    d = torch.sqrt(torch.outer(torch.diagonal(R), torch.diagonal(R)).abs())
    return ((V - R).abs() / torch.maximum(R.abs(), 1e-3 * d)).max().item()


@pytest.mark.parametrize("n", [1500, 1920])
def test_static_contraction_near_its_size_limit(cuda, n):
    """1,920 objects (15 tiles of 128) is the largest count the 8 MiB array
    holds: the plan lowers the K split to fit, so the counts below it (1,500
    among them) all run."""
    Q = 2000
    g = torch.Generator(device="cuda").manual_seed(n)
    Jw = torch.randn((n, Q), dtype=torch.complex64, device="cuda", generator=g)
    kg = KGrid(np.tile([[0.0, 0.0, 1.0]], (Q, 1)), np.linspace(0.1, 5.0, Q), np.ones(Q))
    ref = core.contract(kg, Jw, "fp32")
    for call in range(2):
        V = torch.full((n, n), float("nan"), dtype=torch.float64, device="cuda")
        _lib.check(_static(Jw, Q, n, None, V))
        torch.cuda.synchronize()
        assert torch.isfinite(V).all(), call
        err = _cond_err(V, ref)
        assert err <= 1e-5, (n, call, err)  # the FP32 contraction tolerance


def test_static_contraction_reads_8_byte_aligned_rows(cuda):
    """A complex64 view offset by one node is only 8-byte aligned: the rows are
    read element-wise, with the same sums as an aligned copy."""
    n, Q = 70, 1202
    g = torch.Generator(device="cuda").manual_seed(5)
    flat = torch.randn(n * Q + 1, dtype=torch.complex64, device="cuda", generator=g)
    Jw = flat[1:].view(n, Q)
    assert Jw.data_ptr() % 16 == 8
    V = torch.full((n, n), float("nan"), dtype=torch.float64, device="cuda")
    _lib.check(_static(Jw, Q, n, None, V))
    kg = KGrid(np.tile([[0.0, 0.0, 1.0]], (Q, 1)), np.linspace(0.1, 5.0, Q), np.ones(Q))
    ref = core.contract(kg, Jw.contiguous().clone(), "fp32")
    torch.cuda.synchronize()
    assert _cond_err(V, ref) <= 1e-12


def test_static_contraction_rejects_oversized_problems(cuda):
    kg = standard_kgrid(3, 4)
    Jw = torch.zeros((4, kg.num_nodes), dtype=torch.complex64, device="cuda")
    V = torch.zeros((4, 4), dtype=torch.float64, device="cuda")
    for n in (1921, 4000):  # rejected before any launch: 16 tiles of 128 need 136 partial tiles > 128
        rc = _static(Jw, kg.num_nodes, n, None, V)
        assert rc == 6  # PI_ERR_WORKSPACE_TOO_SMALL
        assert b"8388608-byte" in _lib.lib().pi_last_error()
