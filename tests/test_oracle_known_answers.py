"""Known-answer checks of the FP64 oracle, restating the reference's own tests
(cpp/test/test_unit_cube.cpp, test_multi_object.cpp, test_volume_unified.cpp,
test_intersection_volume_gradient.cpp, test_dof_parameterization.cpp) with the
analytic cube / ball transforms as second oracle, plus finite-difference checks
of every gradient the oracle provides."""
import numpy as np
import pytest

import pointint_gb300 as pg
from pointint_gb300 import geometry as G
from pointint_gb300.kgrid import standard_kgrid


def cube_obj(orc, dofs=None, dof_type=0):
    V, F = G.create_unit_cube_mesh()
    return orc.Obj(orc.GEOM_TRIANGLE, orc.pack_tris(V, F), dof_type, dofs if dofs is not None else None), V, F


def kg_tuple(kg):
    return kg.dirs, kg.kmag, kg.w


@pytest.fixture(scope="module")
def kg9():
    return standard_kgrid(9, 16)


@pytest.fixture(scope="module")
def kg29():
    return standard_kgrid(29, 32)


def test_cube_form_factor_is_exact(orc):
    """A_mesh(k) = i |k| F_cube(k) for the exact polyhedron (test_unit_cube.cpp:22-85)."""
    obj, _, _ = cube_obj(orc)
    rng = np.random.default_rng(0)
    ks = np.concatenate([rng.normal(size=(200, 3)) * 4.0,
                         np.array([[1e-3, 0, 0], [0.1, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1], [0, 2, 0]])])
    A = orc.form_factor(obj, ks)
    for k, a in zip(ks, A):
        exact = 1j * np.linalg.norm(k) * orc.exact_cube_form_factor(*k)
        assert abs(a - exact) <= 1e-7 * max(1.0, np.linalg.norm(k)), (k, a, exact)


def test_affine_cube_follows_transform_rule(orc):
    """F_{A Omega + t}(k) = |det A| e^{ik.t} F(A^T k)
    (docs/form_factor_intersection_theory.md:34; affine_dof.cpp:55-101)."""
    rng = np.random.default_rng(1)
    A = G.random_rotation(rng) @ np.diag([0.7, 1.2, 0.9])
    t = np.array([0.3, -0.2, 0.5])
    obj, _, _ = cube_obj(orc, G.affine_dofs(A, t))
    ks = rng.normal(size=(100, 3)) * 3.0
    got = orc.form_factor(obj, ks)
    for k, a in zip(ks, got):
        exact = 1j * np.linalg.norm(k) * abs(np.linalg.det(A)) * np.exp(1j * k @ t) * orc.exact_cube_form_factor(*(A.T @ k))
        assert abs(a - exact) <= 1e-7 * max(1.0, np.linalg.norm(k))


def test_quadrature_integrates_ball_volume(orc, kg29):
    """(1/8 pi^3) sum_q w |F|^2 k^2 ~= V for the unit ball (the quadrature check of
    test_unit_cube.cpp:90-145 applied to exact_sphere_form_factor,
    form_factor_helpers.cpp:162-173; the cube's axis-aligned Lebedev nodes see
    an undamped sinc^2 k^2 tail, so the ball is the well-posed instance).  The
    tan-mapped radial rule cannot resolve the oscillating tail, so the
    discretisation error at L = 32 is a few percent: 5%."""
    F = np.array([orc.exact_sphere_form_factor(k, 1.0) for k in kg29.kmag])
    vol = np.sum(kg29.w * F * F * kg29.kmag ** 2) / (8 * np.pi ** 3)
    assert abs(vol - 4.0 / 3.0 * np.pi) < 0.05 * 4.0 / 3.0 * np.pi


def test_cube_self_volume(orc, kg29):
    """Self-intersection volume of the unit cube ~= 1 (test_unit_cube.cpp:150-178, 5%)."""
    obj, _, _ = cube_obj(orc)
    v = orc.pair_volume(obj, obj, kg_tuple(kg29))["volume"]
    assert abs(v - 1.0) < 0.05


def test_three_translated_cubes_match_box_box(orc, kg29):
    """test_multi_object.cpp:17-131: symmetric, diagonal ~1, pairs within 15%."""
    V, F = G.create_unit_cube_mesh()
    shifts = [np.zeros(3), np.array([0.5, 0, 0]), np.array([0.25, 0.25, 0.0])]
    objs = [orc.Obj(orc.GEOM_TRIANGLE, orc.pack_tris(V + s, F)) for s in shifts]
    M, _, _ = orc.volume_matrix(objs, kg_tuple(kg29))
    assert np.allclose(M, M.T, atol=1e-12)
    for i in range(3):
        for j in range(3):
            exact = orc.box_box_intersection_volume(shifts[i], [0.5] * 3, shifts[j], [0.5] * 3)
            assert abs(M[i, j] - exact) <= 0.15 * max(exact, 1e-3) + 0.02


def test_sphere_pointcloud_volume(orc, kg29):
    """Fibonacci disk sphere volume vs 4/3 pi (test_sphere_pointcloud.cpp:140-171, 15%)."""
    P, N, R = G.create_sphere_pointcloud(500)
    obj = orc.Obj(orc.GEOM_DISK, orc.pack_disks(P, N, R, True))
    v = orc.pair_volume(obj, obj, kg_tuple(kg29))["volume"]
    assert abs(v - 4.0 / 3.0 * np.pi) < 0.15 * 4.0 / 3.0 * np.pi


def test_mesh_dof_equals_identity_affine(orc, kg9):
    V, F = G.icosphere(1)
    tris = orc.pack_tris(V, F)
    a = orc.Obj(orc.GEOM_TRIANGLE, tris)
    m = orc.Obj(orc.GEOM_TRIANGLE, tris, orc.DOF_TRIANGLE_MESH, V.reshape(-1))
    kv = kg9.dirs * kg9.kmag[:, None]
    np.testing.assert_allclose(orc.form_factor(m, kv), orc.form_factor(a, kv), rtol=0, atol=1e-12)
    assert abs(orc.self_volume(m) - orc.self_volume(a)) < 1e-12


def _fd_grad_A(orc, obj, ks, h=1e-6):
    base = obj.dofs.copy()
    out = np.zeros((len(ks), len(base)), dtype=complex)
    for d in range(len(base)):
        p, m = base.copy(), base.copy()
        p[d] += h
        m[d] -= h
        Ap = orc.form_factor(orc.Obj(obj.geom_type, obj.elems, obj.dof_type, p), ks)
        Am = orc.form_factor(orc.Obj(obj.geom_type, obj.elems, obj.dof_type, m), ks)
        out[:, d] = (Ap - Am) / (2 * h)
    return out


@pytest.mark.parametrize("kind", ["tri", "disk", "gauss"])
def test_affine_form_factor_gradient_vs_fd(orc, kind):
    """dA/dtheta for AffineDoF (affine_dof.cpp:172-322) vs central differences
    (test_dof_parameterization.cpp:57-340)."""
    rng = np.random.default_rng(5)
    if kind == "tri":
        V, F = G.icosphere(1)
        elems, gt = orc.pack_tris(V, F), orc.GEOM_TRIANGLE
    elif kind == "disk":
        P, N, R = G.create_sphere_pointcloud(60)
        elems, gt = orc.pack_disks(P, N, R), orc.GEOM_DISK
    else:
        P, N, S, W = G.create_sphere_gaussians(60)
        elems, gt = orc.pack_gaussians(P, N, S, W), orc.GEOM_GAUSSIAN
    A = np.eye(3) + 0.1 * rng.normal(size=(3, 3))
    obj = orc.Obj(gt, elems, orc.DOF_AFFINE, G.affine_dofs(A, [0.1, -0.2, 0.05]))
    ks = rng.normal(size=(12, 3)) * 2.5
    g = orc.form_factor_grad(obj, ks)
    fd = _fd_grad_A(orc, obj, ks)
    np.testing.assert_allclose(g, fd, rtol=0, atol=2e-6 * max(1.0, np.abs(fd).max()))


def test_mesh_vertex_gradient_vs_fd(orc):
    """Per-vertex dA/dv (triangle_mesh_dof.cpp:76-143, formula :131-133)."""
    V, F = G.icosphere(1)
    rng = np.random.default_rng(2)
    V = V * (1 + 0.05 * rng.normal(size=(len(V), 1)))
    obj = orc.Obj(orc.GEOM_TRIANGLE, orc.pack_tris(V, F), orc.DOF_TRIANGLE_MESH, V.reshape(-1))
    ks = rng.normal(size=(6, 3)) * 2.0
    g = orc.form_factor_grad(obj, ks)
    fd = _fd_grad_A(orc, obj, ks)
    np.testing.assert_allclose(g, fd, rtol=0, atol=2e-6 * max(1.0, np.abs(fd).max()))


def test_pair_volume_gradient_vs_fd(orc, kg9):
    """dV/dtheta of the pair driver vs 5-point FD (test_volume_unified.cpp:123-171, 0.01 max-abs)."""
    V, F = G.create_unit_cube_mesh()
    o1 = orc.Obj(orc.GEOM_TRIANGLE, orc.pack_tris(V, F))
    P, N, R = G.create_sphere_pointcloud(80)
    o2 = orc.Obj(orc.GEOM_DISK, orc.pack_disks(P * 0.6, N, R * 0.6), orc.DOF_AFFINE,
                 G.affine_dofs(np.eye(3), [0.3, 0.1, 0.0]))
    kg = kg_tuple(kg9)
    r = orc.pair_volume(o1, o2, kg, orc.VOLUME_ONLY | orc.GRADIENT | orc.HESSIAN)
    eps = 1e-4
    for which, obj, key in ((0, o1, "grad_geom1"), (1, o2, "grad_geom2")):
        for d in range(12):
            vals = []
            for s in (2, 1, -1, -2):
                dd = obj.dofs.copy()
                dd[d] += s * eps
                o = orc.Obj(obj.geom_type, obj.elems, obj.dof_type, dd)
                pair = (o, o2) if which == 0 else (o1, o)
                vals.append(orc.pair_volume(*pair, kg)["volume"])
            fd = (-vals[0] + 8 * vals[1] - 8 * vals[2] + vals[3]) / (12 * eps)
            assert abs(r[key][d] - fd) < 1e-6 + 1e-5 * abs(fd)
    H = r["hessian_cross"]
    assert H.shape == (12, 12) and np.isfinite(H).all()


def test_matrix_gradients_consistent_with_pair(orc, kg9):
    """grad_matrix[i][j] = dV_ij/dtheta_i equals the pair driver's gradient."""
    V, F = G.create_unit_cube_mesh()
    o1 = orc.Obj(orc.GEOM_TRIANGLE, orc.pack_tris(V, F))
    o2 = orc.Obj(orc.GEOM_TRIANGLE, orc.pack_tris(V, F), orc.DOF_AFFINE, G.affine_dofs(np.eye(3), [0.4, 0, 0]))
    kg = kg_tuple(kg9)
    M, grad, hess = orc.volume_matrix([o1, o2], kg, orc.VOLUME_ONLY | orc.GRADIENT | orc.HESSIAN)
    r = orc.pair_volume(o1, o2, kg, orc.VOLUME_ONLY | orc.GRADIENT | orc.HESSIAN)
    assert abs(M[0, 1] - r["volume"]) < 1e-13
    np.testing.assert_allclose(grad[0][1], r["grad_geom1"], atol=1e-12)
    np.testing.assert_allclose(grad[1][0], r["grad_geom2"], atol=1e-12)
    np.testing.assert_allclose(hess[0][1], r["hessian_cross"], atol=1e-12)


@pytest.mark.parametrize("gt", [1, 2])
def test_surfel_param_grad_vs_fd_and_translation_sum(orc, kg9, gt):
    """Per-disk / per-Gaussian dL/dc, dL/dn (no reference counterpart): central
    FD on the packed arrays, and sum_e dL/dc_e == dL/dt from the AffineDoF
    translation gradient (affine_dof.cpp:262, :305)."""
    P, N, R = G.create_sphere_pointcloud(40)
    # rotate so that no normal lies on a Lebedev direction: at k || n the
    # reference's clamp r = sqrt(max(0, |k|^2 - (k.n)^2)) has a kink in n
    Rot = G.random_rotation(np.random.default_rng(11))
    P, N = P @ Rot.T, N @ Rot.T
    objs = []
    for s, sc in ((np.zeros(3), 0.8), (np.array([0.5, 0.2, 0.0]), 0.6)):
        if gt == 1:
            e = orc.pack_disks(P * sc + s, N, R * sc)
        else:
            e = orc.pack_gaussians(P * sc + s, N, R * sc * 0.5, np.full(len(P), 4 * np.pi * sc * sc / len(P)))
        objs.append(orc.Obj(gt, e))
    kg = kg_tuple(kg9)
    C = np.ones((2, 2))
    gp, gn = orc.surfel_param_grad(objs, kg, C)

    def loss(os_):
        M, _, _ = orc.volume_matrix(os_, kg)
        return float(np.sum(C * M))

    h = 1e-6
    for e_idx in (0, 7, 23):
        for comp in range(3):
            for field, gref in (("c", gp), ("n", gn)):
                vals = []
                for sgn in (1, -1):
                    el = objs[0].elems.copy()
                    el[field][e_idx, comp] += sgn * h
                    vals.append(loss([orc.Obj(gt, el), objs[1]]))
                fd = (vals[0] - vals[1]) / (2 * h)
                assert abs(gref[e_idx, comp] - fd) < 1e-7 + 1e-5 * abs(fd), (field, e_idx, comp)
    # translation-sum identity against the AffineDoF gradient
    M, grad, _ = orc.volume_matrix(objs, kg, orc.VOLUME_ONLY | orc.GRADIENT)
    n0 = len(objs[0].elems)
    for m in range(2):
        dLdt = 2 * sum(grad[m][j][:3] for j in range(2))
        np.testing.assert_allclose(gp[m * n0:(m + 1) * n0].sum(axis=0), dLdt, rtol=1e-9, atol=1e-12)
