"""Antipodal direction pairs of the k-grid (host only, no GPU).

The form factor of a real solid obeys A(-k) = -conj A(k), so the kernels
evaluate one direction of each antipodal pair and write the other from it.
These tests check the pairing the device k-grid stores
(``pi_kgrid_direction_pairs``): every direction written exactly once, the
mirror antipodal, one warp's 32 directions a compact cluster, and grids
without antipodes left in index order.  The identity itself is checked on
the FP64 oracle."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

from pointint_gb300 import kgrid  # noqa: E402


def _coverage(p, M):
    seen = np.zeros(M, dtype=np.int64)
    np.add.at(seen, p[:, 0], 1)
    np.add.at(seen, p[p[:, 1] >= 0, 1], 1)
    return seen


@pytest.mark.parametrize("order,n_radial", [(29, 32), (59, 64), (131, 8)])
def test_lebedev_grids_pair_every_direction(order, n_radial):
    kg = kgrid.standard_kgrid(order, n_radial)
    Q, M, L = len(kg), None, n_radial
    M = Q // L
    p = kg.direction_pairs()
    d = kg.dirs[:M]
    assert len(p) == M // 2
    assert (p[:, 1] >= 0).all()
    assert (_coverage(p, M) == 1).all()
    assert np.abs(d[p[:, 0]] + d[p[:, 1]]).max() < 1e-12
    # evaluated member in the upper half-space
    assert (d[p[:, 0], 2] >= 0).all()
    # a warp's 32 directions: a cap well inside a hemisphere (32 consecutive
    # directions in file order are spread over the whole sphere)
    def radius(idx):
        u = d[idx]
        c = u.mean(0)
        c /= np.linalg.norm(c)
        return np.degrees(np.arccos(np.clip(u @ c, -1.0, 1.0))).max()
    rad = [radius(p[w:w + 32, 0]) for w in range(0, len(p) - 31, 32)]
    file_order = [radius(np.arange(w, w + 32)) for w in range(0, M - 31, 32)]
    assert max(rad) < 60.0
    assert np.mean(rad) < 0.5 * np.mean(file_order)


def test_pairs_are_deterministic():
    kg = kgrid.standard_kgrid(59, 4)
    assert np.array_equal(kg.direction_pairs(), kg.direction_pairs())


def test_grid_without_antipodes_keeps_index_order():
    rng = np.random.default_rng(3)
    d = rng.normal(size=(50, 3))
    d[:, 2] = np.abs(d[:, 2]) + 0.1  # upper half-space only: no antipodes
    d /= np.linalg.norm(d, axis=1)[:, None]
    L = 3
    dirs = np.tile(d, (L, 1))
    kmag = np.repeat([0.5, 1.0, 2.0], len(d))
    p = kgrid.KGrid(dirs, kmag, np.ones(len(kmag))).direction_pairs()
    assert np.array_equal(p[:, 0], np.arange(len(d)))
    assert (p[:, 1] == -1).all()


def test_partial_symmetry_on_a_node_list():
    # a non-tensor node list: k vectors pair when k' = -k (here 4 of 6 do)
    k = np.array([[1.0, 0, 0], [-1.0, 0, 0], [0, 2.0, 0.5], [0, -2.0, -0.5], [0.3, 0.1, 0.2], [0.3, 0.1, -0.2]])
    kmag = np.linalg.norm(k, axis=1)
    p = kgrid.KGrid(k / kmag[:, None], kmag, np.ones(6)).direction_pairs()
    assert len(p) == 4
    assert (_coverage(p, 6) == 1).all()
    pairs = {tuple(sorted(r)) for r in p.tolist() if r[1] >= 0}
    assert pairs == {(0, 1), (2, 3)}
    assert sorted(int(r[0]) for r in p if r[1] < 0) == [4, 5]


def test_oracle_form_factor_is_antisymmetric_hermitian():
    """A(-k) = -conj A(k) for triangles, disks and Gaussian surfels (FP64 oracle)."""
    from oracle import oracle as orc
    from oracle import workloads as w
    rng = np.random.default_rng(1)
    V, F = w.icosphere(1)
    tri = orc.Obj(orc.GEOM_TRIANGLE, orc.pack_tris(V, F), orc.DOF_AFFINE,
                  w.affine_dofs(np.diag([1.2, 0.7, 1.0]), [0.3, -0.2, 1.1]))
    P = rng.normal(size=(20, 3))
    N = rng.normal(size=(20, 3))
    N /= np.linalg.norm(N, axis=1)[:, None]
    disk = orc.Obj(orc.GEOM_DISK, orc.pack_disks(P, N, rng.uniform(0.05, 0.2, 20)), orc.DOF_AFFINE,
                   w.affine_dofs(np.eye(3) * 1.1, [0.1, 0.2, 0.3]))
    gau = orc.Obj(orc.GEOM_GAUSSIAN, orc.pack_gaussians(P, N, rng.uniform(0.05, 0.2, 20), rng.uniform(0.5, 1.5, 20)),
                  orc.DOF_AFFINE, w.affine_dofs(np.eye(3), [0.0, 0.5, 0.0]))
    k = rng.normal(size=(30, 3)) * 3.0
    for o in (tri, disk, gau):
        a, b = orc.form_factor(o, k), orc.form_factor(o, -k)
        assert np.abs(b + np.conj(a)).max() <= 1e-12 * np.abs(a).max()


def test_planar_node_list_pairs_quickly():
    # every k vector in the x = 0 plane: candidates are searched along the
    # widest coordinate, so this stays fast and pairs every point
    import time
    rng = np.random.default_rng(5)
    n = 20000
    ang = rng.uniform(0.0, np.pi, n)
    r = rng.uniform(0.5, 2.0, n)
    k = np.stack([np.zeros(n), np.cos(ang) * r, np.sin(ang) * r], axis=1)
    k = np.concatenate([k, -k])
    kmag = np.linalg.norm(k, axis=1)
    t0 = time.perf_counter()
    p = kgrid.KGrid(k / kmag[:, None], kmag, np.ones(len(kmag))).direction_pairs()
    assert time.perf_counter() - t0 < 5.0
    assert len(p) == n and (p[:, 1] >= 0).all()
    assert (_coverage(p, 2 * n) == 1).all()
    assert np.abs(k[p[:, 0]] + k[p[:, 1]]).max() < 1e-12


def test_adjoint_folding_identity_on_oracle_derivatives():
    """The adjoint kernels evaluate dA/dtheta at the evaluated direction only
    and contract it with B_j - conj(B_j') (each with its weight and origin
    phase): with dA(-k) = -conj dA(k) this equals the sum over both nodes
    for any cotangent.  Checked here with the FP64 oracle's DoF derivatives
    at k and -k, random cotangents and unequal weights."""
    from oracle import oracle as orc
    from oracle import workloads as w
    rng = np.random.default_rng(7)
    V, F = w.icosphere(1)
    obj = orc.Obj(orc.GEOM_TRIANGLE, orc.pack_tris(V, F), orc.DOF_AFFINE,
                  w.affine_dofs(np.diag([1.1, 0.8, 1.3]) @ w.random_rotation(rng), [0.4, -0.3, 0.9]))
    k = rng.normal(size=(16, 3)) * 2.5
    dp, dm = orc.form_factor_grad(obj, k), orc.form_factor_grad(obj, -k)  # (16, 12)
    assert np.abs(dm + np.conj(dp)).max() <= 1e-12 * np.abs(dp).max()
    B = rng.normal(size=16) + 1j * rng.normal(size=16)
    Bm = rng.normal(size=16) + 1j * rng.normal(size=16)
    s, sm = rng.uniform(0.5, 2.0, 16), rng.uniform(0.5, 2.0, 16)
    both = (np.real(np.conj(s * B)[:, None] * dp) + np.real(np.conj(sm * Bm)[:, None] * dm)).sum(0)
    folded = np.real(np.conj(s * B - np.conj(sm * Bm))[:, None] * dp).sum(0)
    assert np.allclose(folded, both, rtol=1e-12, atol=1e-12 * np.abs(both).max())
