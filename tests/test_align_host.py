"""Alignment caller, host parts (no GPU): moments and warm start against the
oracle restatement of cpp/app/align/warm_start.cpp, the warm start's moment
matching as a property, and the oracle's similarity derivatives against
finite differences of its own value (pins the restated formulas of
similarity_measure.cpp before they judge the device path)."""
import numpy as np
import pytest

from pointint_gb300 import align, geometry as G
from pointint_gb300.kgrid import standard_kgrid


def ellipsoid(rng, sub=2, axes=(1.4, 0.9, 0.6), offset=True):
    V, F = G.icosphere(sub)
    R = G.random_rotation(rng)
    c = rng.normal(size=3) if offset else np.zeros(3)
    return G.make_triangle_mesh((V * np.array(axes)) @ R.T + c, F)


def clouds(rng):
    P, N, Rr = G.create_sphere_pointcloud(300)
    S = np.diag([1.3, 0.8, 0.6])
    Rot = G.random_rotation(rng)
    disks = G.make_point_cloud(P @ S @ Rot.T + 0.3, N @ Rot.T, Rr)
    P, N, Sg, W = G.create_sphere_gaussians(300)
    gauss = G.make_gaussian_splat(P @ S @ Rot.T - 0.2, N @ Rot.T, Sg, W)
    return disks, gauss


def as_or(geom):
    return (geom.type, geom.elems)


def test_moments_match_oracle():
    from oracle import align as ora
    rng = np.random.default_rng(0)
    geoms = [ellipsoid(rng), *clouds(rng)]
    dofs = G.affine_dofs(G.random_rotation(rng) @ np.diag([1.2, 0.9, 1.1]), [0.5, -0.3, 0.2])
    for g in geoms:
        for d in (align.IDENTITY, dofs):
            v, c, C = align.compute_moments(g, d)
            vr, cr, Cr = ora.compute_moments(g.type, g.elems, d)
            assert abs(v - vr) <= 1e-12 * abs(vr)
            np.testing.assert_allclose(c, cr, rtol=0, atol=1e-12)
            np.testing.assert_allclose(C, Cr, rtol=0, atol=1e-12)


def test_warm_start_matches_oracle_and_matches_moments():
    """The warm start equals the restatement, and for a rotated, scaled copy
    of an origin-centred geometry 1 with distinct axes it maps geometry 2's
    moments exactly onto geometry 1's.  (The reference's second moment takes
    each origin-fan tetrahedron at its centroid, which is covariant under
    linear maps but not under translations, so the check uses no offset.)"""
    from oracle import align as ora
    rng = np.random.default_rng(1)
    g1 = ellipsoid(rng, offset=False)
    s, R, t = 0.8, G.random_rotation(rng), np.zeros(3)
    V = (g1.elems["a"], g1.elems["e1"], g1.elems["e2"])
    # geometry 2: geometry 1 under x -> s R x + t (same triangle order)
    e = g1.elems.copy()
    e["a"] = s * V[0] @ R.T + t
    e["e1"] = s * V[1] @ R.T
    e["e2"] = s * V[2] @ R.T
    e["S"] = s * s * g1.elems["S"] @ R.T
    g2 = G.Geometry(G.GEOM_TRIANGLE, e)
    d = align.compute_warm_start(g1, g2)
    dr = ora.compute_warm_start(as_or(g1), as_or(g2))
    np.testing.assert_allclose(d, dr, rtol=0, atol=1e-9)
    v1, c1, C1 = align.compute_moments(g1)
    v2, c2, C2 = align.compute_moments(g2, d)
    np.testing.assert_allclose(c2, c1, atol=1e-9)
    np.testing.assert_allclose(C2, C1, atol=1e-9 * np.abs(C1).max())
    assert abs(v2 - v1) <= 1e-9 * abs(v1)
    A = d[3:].reshape(3, 3)
    assert abs(np.linalg.det(A) - 1 / s ** 3) <= 1e-9


@pytest.mark.parametrize("measure", [0, 1, 2])
def test_oracle_similarity_gradient_matches_fd(measure):
    from oracle import align as ora
    rng = np.random.default_rng(2 + measure)
    kg = standard_kgrid(9, 12)
    g1 = ellipsoid(rng, 1, offset=False)
    g2 = ellipsoid(rng, 1, axes=(1.1, 1.0, 0.7), offset=False)
    kgrid = (kg.dirs, kg.kmag, kg.w)
    d0 = G.affine_dofs(np.eye(3) + 0.05 * rng.normal(size=(3, 3)), 0.2 * rng.normal(size=3))
    from oracle import oracle as orc
    V1 = orc.volume_matrix([orc.Obj(g1.type, g1.elems)], kgrid)[0][0, 0]
    r = ora.similarity(as_or(g1), as_or(g2), d0, kgrid, measure, V1, ora.ALL)
    assert 0.2 < r["similarity"] < 1.0
    h = 1e-6
    fd = np.zeros(12)
    for i in range(12):
        dp, dm = d0.copy(), d0.copy()
        dp[i] += h
        dm[i] -= h
        fd[i] = (ora.similarity(as_or(g1), as_or(g2), dp, kgrid, measure, V1, ora.FUNC_ONLY)["value"] -
                 ora.similarity(as_or(g1), as_or(g2), dm, kgrid, measure, V1, ora.FUNC_ONLY)["value"]) / (2 * h)
    assert np.abs(r["gradient"] - fd).max() <= 1e-6 * max(np.abs(fd).max(), 1.0)
    H = r["hessian"]
    assert np.allclose(H, H.T, atol=1e-12 * np.abs(H).max())
