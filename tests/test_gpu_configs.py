"""GPU parity on the two largest workload configurations, against the FP64 oracle.

  large mesh   star-shaped solids of 200,000 triangles on L = 128 radii x
               Lebedev-5810 (N_k = 743,680; k up to ~7.3e3, where the FP32
               phases of the form factors are hardest)
  surfels      50,000-disk and 50,000-Gaussian clouds sampled from the
               256-object shapes, on L = 64 x Lebedev-1202 (N_k = 76,928),
               forward and backward

The oracle cannot evaluate all 743,680 nodes of 200,000-triangle objects in
test time, so each case also runs on a sub-grid: every radius of the grid (the
kernel's radial blocking is that of the full grid) at a strided subset of its
directions, kept in the reference's tensor order q = r M + j.  The volumes
compared are the contractions over that sub-grid's nodes, which are real nodes
of the configuration with their real weights.  A launch on the full grid is
checked against the oracle at the same nodes.

Tolerances (the FP32 contract): ||dJ|| / ||J|| <= 2e-6 and max |dJ| <= 1e-5
max |J| on form factors; volumes 1e-5 conditioned,
  err_ij = |dV_ij| / max(|V_ij|, 1e-3 sqrt(V_ii V_jj)).
Gradients: 1e-5 of the largest entry against the oracle's formula gradient,
and central differences along whole-field directions at 1e-2 (h = 1e-5, see below).
"""
import numpy as np
import pytest
import torch

from pointint_gb300 import configs, core
from pointint_gb300.kgrid import KGrid

pytestmark = pytest.mark.gpu

J_NORM_TOL, J_MAX_TOL, VOL_TOL, GRAD_TOL = 2e-6, 1e-5, 1e-5, 1e-5


def to_oracle(orc, objs):
    return [orc.Obj(o.geom.type, o.geom.elems, o.dof_type, o.dofs) for o in objs]


def sub_grid(kg: KGrid, n_dirs: int, dir_stride: int):
    """Every radius of a tensor-order grid at every dir_stride-th direction."""
    L = kg.num_nodes // n_dirs
    js = np.arange(0, n_dirs, dir_stride)
    sel = (np.arange(L)[:, None] * n_dirs + js[None, :]).reshape(-1)
    return KGrid(kg.dirs[sel], kg.kmag[sel], kg.w[sel]), sel


def cond_rel_err(V, R):
    d = np.sqrt(np.abs(np.outer(np.diag(R), np.diag(R))))
    return np.abs(V - R) / np.maximum(np.abs(R), 1e-3 * d)


def check_J(Jg, Jo, kmag, what):
    """Jg [n, Q] GPU, Jo [Q, n] oracle; prints the error by radial band."""
    Jo = Jo.T
    err = np.abs(Jg - Jo)
    nrm = np.linalg.norm(err) / np.linalg.norm(Jo)
    mx = err.max() / np.abs(Jo).max()
    bands = [(0, 10), (10, 100), (100, 1000), (1000, np.inf)]
    txt = []
    for lo, hi in bands:
        m = (kmag >= lo) & (kmag < hi)
        if m.any():
            txt.append(f"k in [{lo},{hi}): {np.linalg.norm(err[:, m]) / np.linalg.norm(Jo[:, m]):.2e}")
    print(f"\n{what}: ||dJ||/||J|| {nrm:.2e}, max {mx:.2e}; by band " + ", ".join(txt))
    assert nrm <= J_NORM_TOL, (what, nrm)
    assert mx <= J_MAX_TOL, (what, mx)


@pytest.fixture(scope="module")
def large_mesh():
    return configs.large_mesh(n_objects=2)


def test_large_mesh_config_matches_oracle(cuda, orc, large_mesh):
    """Two 200,000-triangle solids: J and V on 59 directions x 128 radii
    (7,552 nodes, k from 0.012 to 7.3e3), and the full-grid launch at those
    nodes."""
    kg, objs, meta = large_mesh
    assert kg.num_nodes == 743680 and meta["n_triangles_each"] == 200000
    sub, sel = sub_grid(kg, 5810, 100)
    assert sub.info() == (7552, 59, 128)
    assert sub.kmag.max() > 7.0e3
    batch = core.ObjectBatch(objs)
    Jg = core.form_factors(sub, batch, False).cpu().numpy()
    Vg = core.contract(sub, core.form_factors(sub, batch, True), "fp32").cpu().numpy()
    Jo = orc.form_factor_matrix(to_oracle(orc, objs), sub.dirs, sub.kmag)
    check_J(Jg, Jo, sub.kmag, "large mesh, sub-grid")
    Vo = orc.contract(Jo, sub.w)
    err = cond_rel_err(Vg, Vo)
    print(f"large mesh volumes on the sub-grid: max cond rel err {err.max():.3e}")
    assert err.max() <= VOL_TOL, err
    # the production launch: all 743,680 nodes, read back at the sub-grid's nodes
    Jfull = core.form_factors(kg, batch, False)
    check_J(Jfull[:, torch.as_tensor(sel, device="cuda")].cpu().numpy(), Jo, sub.kmag, "large mesh, full grid")


@pytest.fixture(scope="module")
def surfel_pair():
    """A 50,000-disk cloud (sampled from an icosphere-4 shape) and a
    50,000-Gaussian cloud (sampled from a box) of the 64-object sets."""
    kg, disks, _ = configs.surfels64()
    _, gauss, _ = configs.surfels64(gaussian=True, kgrid=False)
    assert disks[0].geom.num_elements() == 50000 and gauss[40].geom.num_elements() == 50000
    return kg, [disks[0], gauss[40]]


def test_surfel_config_forward_matches_oracle(cuda, orc, surfel_pair):
    kg, objs = surfel_pair
    sub, sel = sub_grid(kg, 1202, 8)
    assert sub.info() == (9664, 151, 64)
    batch = core.ObjectBatch(objs)
    Jg = core.form_factors(sub, batch, False).cpu().numpy()
    Vg = core.contract(sub, core.form_factors(sub, batch, True), "fp32").cpu().numpy()
    Jo = orc.form_factor_matrix(to_oracle(orc, objs), sub.dirs, sub.kmag)
    check_J(Jg, Jo, sub.kmag, "surfels, sub-grid")
    Vo = orc.contract(Jo, sub.w)
    err = cond_rel_err(Vg, Vo)
    print(f"surfel volumes on the sub-grid: max cond rel err {err.max():.3e}")
    assert err.max() <= VOL_TOL, err
    Jfull = core.form_factors(kg, batch, False)
    check_J(Jfull[:, torch.as_tensor(sel, device="cuda")].cpu().numpy(), Jo, sub.kmag, "surfels, full grid")


def test_surfel_config_backward_matches_oracle_and_fd(cuda, orc, surfel_pair):
    """dL/dc and dL/dn of every one of the 100,000 surfels for L = sum_ij V_ij
    on the sub-grid (all 64 radii, k up to 1.8e3), against the oracle's
    formula gradient, and central differences of the GPU loss."""
    kg, objs = surfel_pair
    sub, _ = sub_grid(kg, 1202, 8)
    scene = core.Scene(sub, objs)
    c, n = scene.surfel_params()
    c.requires_grad_(True)
    n.requires_grad_(True)
    scene.volume_matrix_of_surfels(c, n).sum().backward()
    gp, gn = orc.surfel_param_grad(to_oracle(orc, objs), (sub.dirs, sub.kmag, sub.w), np.ones((2, 2)))
    for name, g, ref in (("dL/dc", c.grad.cpu().numpy(), gp), ("dL/dn", n.grad.cpu().numpy(), gn)):
        err = np.abs(g - ref).max() / np.abs(ref).max()
        print(f"\nsurfels, 100,000 elements, {name}: max |dg| / max |g| = {err:.3e}")
        assert err <= GRAD_TOL, (name, err)
    # Central differences along whole-field directions u (every surfel moved
    # by h u_e): one surfel alone changes an FP32 loss by less than its
    # rounding, the whole field by sum_e g_e . u_e.  The step is 1e-5: at
    # h = 1e-3 the phase k.c of a surfel moves by ~1.8 rad at this grid's
    # largest radius (k ~ 1,832), where a difference quotient no longer
    # approximates the derivative (the 16-radius FD test keeps h = 1e-3).
    h = 1e-5
    with torch.no_grad():
        for which, g in (("c", c.grad), ("n", n.grad)):
            for kind in ("sign", "scaled sign"):
                # directions that move the loss by sum |g| (well above its FP32 rounding)
                u = torch.sign(g)
                if kind == "scaled sign":
                    u = u * torch.as_tensor(np.random.default_rng(9).uniform(0.5, 1.5, size=g.shape), device="cuda")
                if which == "n":  # along the tangent plane: |n| = 1 keeps |k'_perp|^2 >= 0
                    nh = n.detach() / n.detach().norm(dim=1, keepdim=True)
                    u = u - (u * nh).sum(dim=1, keepdim=True) * nh
                vals = []
                for sgn in (1, -1):
                    cc, nn = c.detach().clone(), n.detach().clone()
                    if which == "c":
                        cc += sgn * h * u
                    else:
                        nn += sgn * h * u
                    vals.append(scene.volume_matrix_of_surfels(cc, nn).sum().item())
                fd = (vals[0] - vals[1]) / (2 * h)
                an = float((g * u).sum())
                print(f"surfels, d/de L({which} + e u), u {kind}: adjoint {an:.6e}, central difference {fd:.6e}")
                assert abs(an - fd) <= 1e-2 * abs(an), (which, kind, an, fd)
