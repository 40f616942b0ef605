"""GPU adjoint vs the FP64 oracle and finite differences.

Reference pins (cpp/test/test_volume_unified.cpp:390-396, 890-896): CPU and GPU
gradients agree to 1e-6 in FP64 and match 5-point FD to 0.01 max-abs.  The FP32
adjoint here is held to 1e-5 of the gradient's max-abs entry against the
oracle (the FP32 tolerance; the worst case measured is 5.0e-6, a normal
gradient on the 64-radius grid), and the autograd path to central FD with
h = 1e-3 at 1e-2 (FD of an FP32 loss resolves ~1e-3 of the slope at that
step).
"""
import numpy as np
import pytest
import torch

import pointint_gb300 as pg
from pointint_gb300 import geometry as G, core
from pointint_gb300.kgrid import standard_kgrid

pytestmark = pytest.mark.gpu

GRAD_TOL = 1e-5


def tangent_part(u, n):
    """u minus its component along each unit normal n: normals moved along it
    keep |n| = 1 to first order.  A normal that grows past unit length makes
    |k'_perp|^2 = |k'|^2 - (k'.n)^2 negative for directions near it, where the
    kernels clamp it at zero, a kink that a difference quotient across it
    does not resolve at large k."""
    nh = n / n.norm(dim=1, keepdim=True)
    return u - (u * nh).sum(dim=1, keepdim=True) * nh


def to_or(orc, o):
    return orc.Obj(o.geom.type, o.geom.elems, o.dof_type, o.dofs)


def assert_grad_close(g, ref, tol=GRAD_TOL, what=""):
    g, ref = np.asarray(g), np.asarray(ref)
    scale = max(np.abs(ref).max(), 1e-12)
    err = np.abs(g - ref).max() / scale
    print(f"\n{what}: max |dg| / max |g| = {err:.3e}")
    assert err <= tol, (what, err)


@pytest.fixture(scope="module", params=[(9, 16), (9, 64)], ids=["16radii", "64radii"])
def kg(request):
    """38 directions x 16 radii (k up to ~400), and x 64 radii (k up to
    ~1,800), where the adjoint's large-spread branches and FP32 phases carry
    most of the weight."""
    return standard_kgrid(*request.param)


def scene_objects(rng):
    Vc, Fc = G.create_unit_cube_mesh()
    cube = G.SceneObject(G.make_triangle_mesh(Vc, Fc), pg.DOF_AFFINE,
                         G.affine_dofs(np.eye(3) + 0.05 * rng.normal(size=(3, 3)), [0.1, -0.05, 0.0]))
    P, N, R = G.create_sphere_pointcloud(300)
    Rot = G.random_rotation(rng)
    disks = G.SceneObject(G.make_point_cloud(P @ Rot.T * 0.7, N @ Rot.T, R * 0.7), pg.DOF_AFFINE,
                          G.affine_dofs(np.eye(3) + 0.1 * rng.normal(size=(3, 3)), [0.4, 0.1, 0.0]))
    P, N, S, W = G.create_sphere_gaussians(300)
    gauss = G.SceneObject(G.make_gaussian_splat(P @ Rot.T * 0.6, N @ Rot.T, S * 0.6, W * 0.36), pg.DOF_AFFINE,
                          G.affine_dofs(np.eye(3) + 0.1 * rng.normal(size=(3, 3)), [-0.2, 0.3, 0.1]))
    Vs, Fs = G.icosphere(1)
    Vs = Vs * (1 + 0.05 * rng.normal(size=(len(Vs), 1))) * 0.8 + np.array([0.0, 0.0, 0.35])
    mesh = G.SceneObject(G.make_triangle_mesh(Vs, Fs), pg.DOF_TRIANGLE_MESH, Vs.reshape(-1))
    return [cube, disks, gauss, mesh]


@pytest.mark.parametrize("pair", [(0, 1), (0, 2), (1, 2), (3, 0), (3, 1)])
def test_pair_gradient_matches_oracle(cuda, orc, kg, pair):
    """pi_pair_volume_grad_host vs the oracle's pair driver with GRADIENT
    (compute_intersection_volume_cpu.cpp:94-151)."""
    objs = scene_objects(np.random.default_rng(1))
    o1, o2 = objs[pair[0]], objs[pair[1]]
    v, g1, g2 = core.pair_volume_grad_host(kg, o1, o2)
    r = orc.pair_volume(to_or(orc, o1), to_or(orc, o2), (kg.dirs, kg.kmag, kg.w), orc.VOLUME_ONLY | orc.GRADIENT)
    assert abs(v - r["volume"]) <= 1e-5 * abs(r["volume"]) + 1e-9
    assert_grad_close(g1, r["grad_geom1"], what=f"pair {pair} grad1")
    assert_grad_close(g2, r["grad_geom2"], what=f"pair {pair} grad2")


def test_matrix_gradients_match_oracle(cuda, orc, kg):
    """grad_matrix[i][j] = dV_ij/dtheta_i for every pair (multi_object.cpp:186-234)."""
    objs = scene_objects(np.random.default_rng(2))
    V, grad = core.volume_matrix_grad_host(kg, objs)
    Vr, gr, _ = orc.volume_matrix([to_or(orc, o) for o in objs], (kg.dirs, kg.kmag, kg.w), orc.VOLUME_ONLY | orc.GRADIENT)
    for i in range(len(objs)):
        for j in range(len(objs)):
            assert_grad_close(grad[i][j], gr[i][j], what=f"grad_matrix[{i}][{j}]")


def test_dof_autograd_matches_oracle(cuda, orc, kg):
    """torch.autograd through the adjoint: d(sum_ij C_ij V_ij)/dtheta."""
    objs = scene_objects(np.random.default_rng(3))
    scene = core.Scene(kg, objs)
    theta = scene.dofs().requires_grad_(True)
    C = torch.tensor(np.random.default_rng(4).uniform(0.5, 1.5, size=(4, 4)), device="cuda")
    V = scene.volume_matrix_of_dofs(theta)
    (C * V).sum().backward()
    Vr, gr, _ = orc.volume_matrix([to_or(orc, o) for o in objs], (kg.dirs, kg.kmag, kg.w), orc.VOLUME_ONLY | orc.GRADIENT)
    Cn = C.cpu().numpy()
    ref = np.concatenate([sum(Cn[m, j] * gr[m][j] + Cn[j, m] * gr[m][j] for j in range(4)) for m in range(4)])
    assert_grad_close(theta.grad.cpu().numpy(), ref, what="autograd dofs")


@pytest.mark.parametrize("gt", [1, 2])
def test_surfel_autograd_matches_oracle_and_fd(cuda, orc, kg, gt):
    """Per-disk / per-Gaussian position and normal gradients of L = sum_ij V_ij
    (no reference counterpart): the oracle's formula gradient, and central FD
    of the GPU loss.  On the 16-radius grid (k up to ~120) FD runs per surfel
    with h = 1e-3 (a phase turn k h <= 0.12 rad).  On the 64-radius grid (k up
    to ~1,830) h = 1e-3 would turn a phase by 1.8 rad, and a step small enough
    for the difference quotient leaves one surfel's change in an FP32 loss
    below its rounding, so FD runs along whole-field directions (every surfel
    moved by h u_e) with h = 1e-5."""
    rng = np.random.default_rng(10 + gt)
    objs = []
    for s, sc in ((np.zeros(3), 0.8), (np.array([0.5, 0.2, 0.0]), 0.6), (np.array([-0.3, 0.4, 0.2]), 0.5)):
        P, N, R = G.create_sphere_pointcloud(200)
        Rot = G.random_rotation(rng)
        P, N = P @ Rot.T, N @ Rot.T
        geom = (G.make_point_cloud(P * sc + s, N, R * sc) if gt == 1 else
                G.make_gaussian_splat(P * sc + s, N, R * sc * 0.5, np.full(len(P), 4 * np.pi * sc * sc / len(P))))
        objs.append(G.SceneObject(geom))
    scene = core.Scene(kg, objs)
    c, n = scene.surfel_params()
    c.requires_grad_(True)
    n.requires_grad_(True)
    L = scene.volume_matrix_of_surfels(c, n).sum()
    L.backward()
    gp, gn = orc.surfel_param_grad([to_or(orc, o) for o in objs], (kg.dirs, kg.kmag, kg.w), np.ones((3, 3)))
    assert_grad_close(c.grad.cpu().numpy(), gp, what="dL/dc")
    assert_grad_close(n.grad.cpu().numpy(), gn, what="dL/dn")
    kmax = float(kg.kmag.max())
    with torch.no_grad():
        if kmax * 1e-3 <= 0.15:
            h = 1e-3
            for e in (3, 250, 555):
                for comp in range(3):
                    for which, t, g in (("c", c, c.grad), ("n", n, n.grad)):
                        vals = []
                        for sgn in (1, -1):
                            cc, nn = c.detach().clone(), n.detach().clone()
                            (cc if which == "c" else nn)[e, comp] += sgn * h
                            vals.append(scene.volume_matrix_of_surfels(cc, nn).sum().item())
                        fd = (vals[0] - vals[1]) / (2 * h)
                        # h = 1e-3 differences of an FP32 loss resolve ~1e-3 of the slope
                        assert abs(g[e, comp].item() - fd) <= 1e-2 * max(abs(fd), 0.1 * g.abs().max().item()), \
                            (which, e, comp)
        else:
            h = 1e-5
            for which, g in (("c", c.grad), ("n", n.grad)):
                u = torch.sign(g)
                if which == "n":  # along the tangent plane: |n| = 1 keeps |k'_perp|^2 >= 0 (see tangent_part)
                    u = tangent_part(u, n.detach())
                vals = []
                for sgn in (1, -1):
                    cc, nn = c.detach().clone(), n.detach().clone()
                    (cc if which == "c" else nn).add_(sgn * h * u)
                    vals.append(scene.volume_matrix_of_surfels(cc, nn).sum().item())
                fd = (vals[0] - vals[1]) / (2 * h)
                an = float((g * u).sum())
                assert abs(an - fd) <= 1e-2 * abs(an), (which, an, fd)
