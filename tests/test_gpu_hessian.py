"""Gauss-Newton Hessian (pi_dof_jacobian, pi_*_hessian_host) vs the FP64 oracle.

Reference pin (cpp/test/test_volume_unified.cpp:1176-1208): GPU and CPU
hessian_ij agree to a block Frobenius error below 1e-5.  Here each block's
error is measured against its conditioning scale sqrt(|H_ii|_F |H_jj|_F)
(Cauchy-Schwarz bounds every entry of H_ij by the diagonal blocks) and held
to 1e-5, the FP32 contract; every entry is also held to 1e-4 of
sqrt(H_aa H_bb), so that DoFs with small derivatives (a mesh vertex, an
entry of A) are checked too.
"""
import numpy as np
import pytest
import torch

import pointint_gb300 as pg
from pointint_gb300 import core
from pointint_gb300.kgrid import standard_kgrid
from test_gpu_gradients import assert_grad_close, scene_objects, to_or

pytestmark = pytest.mark.gpu

HESS_TOL = 1e-5
ENTRY_TOL = 1e-4


@pytest.fixture(scope="module")
def kg():
    return standard_kgrid(9, 16)


def block_errors(H, R, Hii, Hjj):
    """(block Frobenius error / sqrt(|H_ii| |H_jj|), max entry error / sqrt(H_aa H_bb))."""
    scale = np.sqrt(np.linalg.norm(Hii) * np.linalg.norm(Hjj))
    fro = np.linalg.norm(H - R) / max(scale, 1e-300)
    da, db = np.sqrt(np.abs(np.diag(Hii))), np.sqrt(np.abs(np.diag(Hjj)))
    den = np.maximum(np.outer(da, db), 1e-12 * scale)
    return fro, (np.abs(H - R) / den).max()


@pytest.mark.parametrize("pair", [(0, 1), (0, 2), (1, 2), (3, 0), (3, 2)])
def test_pair_hessian_matches_oracle(cuda, orc, kg, pair):
    """hessian_geom1/2/cross and the gradients (compute_intersection_volume_cpu.cpp:94-186)."""
    objs = scene_objects(np.random.default_rng(1))
    o1, o2 = objs[pair[0]], objs[pair[1]]
    got = core.pair_volume_hessian_host(kg, o1, o2)
    ref = orc.pair_volume(to_or(orc, o1), to_or(orc, o2), (kg.dirs, kg.kmag, kg.w), orc.VOLUME_ONLY | orc.GRADIENT | orc.HESSIAN)
    assert abs(got["volume"] - ref["volume"]) <= 1e-5 * abs(ref["volume"]) + 1e-9
    assert_grad_close(got["grad_geom1"], ref["grad_geom1"], what=f"pair {pair} grad1")
    assert_grad_close(got["grad_geom2"], ref["grad_geom2"], what=f"pair {pair} grad2")
    H11, H22 = ref["hessian_geom1"], ref["hessian_geom2"]
    for key, Hi, Hj in (("hessian_geom1", H11, H11), ("hessian_geom2", H22, H22), ("hessian_cross", H11, H22)):
        fro, ent = block_errors(got[key], ref[key], Hi, Hj)
        print(f"\npair {pair} {key}: block {fro:.3e}, entry {ent:.3e}")
        assert fro <= HESS_TOL and ent <= ENTRY_TOL, (key, fro, ent)
    assert np.allclose(got["hessian_geom1"], got["hessian_geom1"].T, rtol=0, atol=1e-12 * np.abs(H11).max())


def test_matrix_hessian_matches_oracle(cuda, orc, kg):
    """hessian_ij[i][j] for every pair of a 4-object scene (multi_object.cpp:236-292)."""
    objs = scene_objects(np.random.default_rng(2))
    V, grad, hess = core.volume_matrix_hessian_host(kg, objs)
    Vr, gr, hr = orc.volume_matrix([to_or(orc, o) for o in objs], (kg.dirs, kg.kmag, kg.w), orc.VOLUME_ONLY | orc.GRADIENT | orc.HESSIAN)
    n = len(objs)
    assert np.abs(V - Vr).max() <= 1e-5 * np.abs(Vr).max()
    worst = (0.0, 0.0)
    for i in range(n):
        for j in range(n):
            assert_grad_close(grad[i][j], gr[i][j], what=f"grad_matrix[{i}][{j}]")
            fro, ent = block_errors(hess[i][j], hr[i][j], hr[i][i], hr[j][j])
            worst = (max(worst[0], fro), max(worst[1], ent))
            assert fro <= HESS_TOL and ent <= ENTRY_TOL, (i, j, fro, ent)
            assert np.array_equal(hess[i][j], hess[j][i].T)
    print(f"\nmatrix hessian: worst block {worst[0]:.3e}, worst entry {worst[1]:.3e}")


def test_jacobian_agrees_with_adjoint(cuda, kg):
    """Forward mode against reverse mode on the device: Re(G J^H)/(8 pi^3) from
    pi_dof_jacobian equals the adjoint's dV_ij/dtheta_i (pi_dof_gradients)."""
    objs = scene_objects(np.random.default_rng(6))
    batch = core.ObjectBatch(objs)
    J = core.form_factors(kg, batch, True)
    Gm = core.dof_jacobian(kg, batch)
    fwd = (torch.view_as_real(Gm).reshape(Gm.shape[0], -1).double() @
           torch.view_as_real(J).reshape(J.shape[0], -1).double().T) / (8 * np.pi ** 3)
    n = len(objs)
    for j in range(n):
        W = np.zeros((n, n))
        W[:, j] = 1.0
        rev = core.dof_gradients(kg, batch, J, W)
        assert_grad_close(fwd[:, j].cpu().numpy(), rev.cpu().numpy(), what=f"column {j}")


def test_hessian_of_256_object_matrix(cuda):
    """The 256-object AffineDoF scene (3,072 DoFs, N_k = 76,928): G's rows
    against J reproduce the adjoint's gradients, the Hessian is symmetric with
    a non-negative diagonal, and its translation blocks are k-weighted copies
    of V's integrand (H_tt for object i equals Re sum w k k^T |A_i|^2 / 8 pi^3,
    checked on a few objects in FP64 on the device)."""
    from pointint_gb300 import configs
    kg, objs, _ = configs.matrix256()
    batch = core.ObjectBatch(objs)
    J = core.form_factors(kg, batch, True)
    Gm = core.dof_jacobian(kg, batch)
    assert Gm.shape == (12 * len(objs), kg.num_nodes)
    H = core.contract(kg, Gm, "fp32").cpu().numpy()
    assert np.array_equal(H, H.T)
    assert (np.diag(H) >= 0).all()
    kvec = torch.tensor(kg.dirs * kg.kmag[:, None], device="cuda")
    for i in (0, 77, 255):
        a2 = (J[i].abs().double() ** 2)  # sqrt|w| already folded into J
        ref = (kvec.T * a2) @ kvec / (8 * np.pi ** 3)
        got = H[12 * i: 12 * i + 3, 12 * i: 12 * i + 3]
        r = ref.cpu().numpy()
        assert np.abs(got - r).max() <= 1e-5 * np.abs(r).max(), i
    W = np.zeros((len(objs), len(objs)))
    W[:, 5] = 1.0
    rev = core.dof_gradients(kg, batch, J, W).cpu().numpy()
    fwd = ((torch.view_as_real(Gm).reshape(Gm.shape[0], -1).double() @
            torch.view_as_real(J[5]).reshape(-1).double()) / (8 * np.pi ** 3)).cpu().numpy()
    assert_grad_close(fwd, rev, tol=5e-5, what="256-object gradients through G")
