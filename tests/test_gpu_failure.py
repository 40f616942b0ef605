"""Failure paths, exercised without any GPU fault.

The tensor-core contractions wait on shared-memory barriers, each wait bounded
(~2 s of SM clock); when one runs out the kernel records a code, every role
leaves its loop, drains its copies and tensor-core operations, frees its
tensor memory, and the reduction writes NaN.  A testing hook shortens the
limit to ~0.1 ms and makes the loader of the first CTA skip one chunk, so one
barrier is never completed: the call must report PI_ERR_TIMEOUT with NaN
output, and the next call on the same GPU must give the normal result.
Host-side waits are bounded too: pi_server_wait with a short timeout on a query
that is still running returns PI_ERR_TIMEOUT, and a later wait gets the result.
"""
import ctypes
import time

import numpy as np
import pytest
import torch

from pointint_gb300 import _lib, core, geometry as G
from pointint_gb300.kgrid import KGrid, standard_kgrid
from pointint_gb300.serving import Server

pytestmark = pytest.mark.gpu

PI_ERR_TIMEOUT = 8


@pytest.mark.parametrize("precision", ["fp16x3", "bf16x3"])
def test_contraction_wait_expiry_reports_error_and_recovers(cuda, precision):
    n, Q = 256, 76928
    g = torch.Generator(device="cuda").manual_seed(3)
    J = torch.randn((n, Q), dtype=torch.complex64, device="cuda", generator=g)
    kg = KGrid(np.tile([[0.0, 0.0, 1.0]], (Q, 1)), np.linspace(0.1, 5.0, Q), np.ones(Q))
    ws = core.Workspace()
    L = _lib.lib()
    p = core.PRECISIONS[precision]
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    ref = core.contract(kg, J, precision, workspace=ws).clone()
    assert L.pi_contract_error(p, ctypes.c_void_p(ws.buf.data_ptr()), stream) == 0
    assert torch.isfinite(ref).all()
    L.pi_test_set_contract_faults(200_000, 3)  # ~0.1 ms waits; CTA 0 never loads its fourth chunk
    try:
        t0 = time.perf_counter()
        V = core.contract(kg, J, precision, workspace=ws)
        rc = L.pi_contract_error(p, ctypes.c_void_p(ws.buf.data_ptr()), stream)
        elapsed = time.perf_counter() - t0
        msg = L.pi_last_error().decode()
    finally:
        L.pi_test_set_contract_faults(0, -1)
    print(f"\n[{precision}] starved barrier: status {rc}, {msg!r}, {elapsed * 1e3:.2f} ms")
    assert rc == PI_ERR_TIMEOUT, (rc, msg)
    assert "bounded wait" in msg
    assert torch.isnan(V).all()
    assert elapsed < 1.0  # every wait, drains included, gave up under the short limit
    V2 = core.contract(kg, J, precision, workspace=ws)  # the same GPU context, normal limits
    assert L.pi_contract_error(p, ctypes.c_void_p(ws.buf.data_ptr()), stream) == 0
    assert torch.equal(V2, ref)


def test_fp32_contraction_has_no_device_waits(cuda):
    L = _lib.lib()
    assert L.pi_contract_error(core.PRECISIONS["fp32"], None, None) == 0


def test_server_wait_times_out_then_completes(cuda):
    """A cold 48-object scene of icosphere-4 meshes (2.5e8 triangle x k
    evaluations per object) is still running a millisecond after submission."""
    kg = standard_kgrid(59, 64)
    V, F = G.icosphere(4)
    lib = [G.SceneObject(G.make_triangle_mesh(V * (0.5 + 0.02 * i), F)) for i in range(48)]
    ids = np.arange(48, dtype=np.int32)
    trans = np.random.default_rng(1).uniform(0.0, 3.0, size=(48, 3))
    with Server(kg, lib, autotune=False) as srv:
        t = srv.submit(ids, None, trans)
        t0 = time.perf_counter()
        rc = _lib.lib().pi_server_wait(srv._h, t.id, 1e-3)
        waited = time.perf_counter() - t0
        assert rc == PI_ERR_TIMEOUT, rc
        assert b"timed out" in _lib.lib().pi_last_error()
        assert waited < 0.5
        Vs = srv.wait(t)  # the query itself is unaffected
        assert srv.poll(t) == "done"
        assert np.isfinite(Vs).all() and np.all(np.diag(Vs) > 0)
        srv.release(t)
