"""GPU parity: the CUDA path (through the C ABI) against the FP64 oracle.

Tolerances (the FP32 contract): FP32 paths 1e-5 relative on volumes, using
the conditioned relative error for off-diagonal entries
  err_ij = |dV_ij| / max(|V_ij|, 1e-3 sqrt(V_ii V_jj))
(nearly disjoint pairs are a cancellation of O(sqrt(V_ii V_jj)) terms).  Form
factors: ||dJ|| / ||J|| <= 2e-6 and max |dJ| <= 1e-5 max |J|.
"""
import ctypes

import numpy as np
import pytest
import torch

import pointint_gb300 as pg
from pointint_gb300 import geometry as G, core, configs, _lib
from pointint_gb300.kgrid import standard_kgrid, KGrid

pytestmark = pytest.mark.gpu

VOL_TOL = 1e-5


def to_oracle(orc, objs):
    return [orc.Obj(o.geom.type, o.geom.elems, o.dof_type, o.dofs) for o in objs]


def cond_rel_err(V, R):
    d = np.sqrt(np.abs(np.outer(np.diag(R), np.diag(R))))
    return np.abs(V - R) / np.maximum(np.abs(R), 1e-3 * d + 1e-300)


def gpu_J(kg, objs, scale=False):
    b = core.ObjectBatch(objs)
    J = core.form_factors(kg, b, scale)
    torch.cuda.synchronize()
    return J.cpu().numpy()


def check_J(Jg, Jo):
    """Jg: [n, Q] GPU, Jo: [Q, n] oracle."""
    Jo = Jo.T
    err = np.abs(Jg - Jo)
    assert np.linalg.norm(err) <= 2e-6 * np.linalg.norm(Jo), np.linalg.norm(err) / np.linalg.norm(Jo)
    assert err.max() <= 1e-5 * np.abs(Jo).max(), err.max() / np.abs(Jo).max()


def shapes(kind, rng):
    if kind == "cube":
        V, F = G.create_unit_cube_mesh()
        return G.SceneObject(G.make_triangle_mesh(V, F))
    if kind == "ico3":
        V, F = G.icosphere(3)
        return G.SceneObject(G.make_triangle_mesh(V, F), pg.DOF_AFFINE, G.affine_dofs(np.eye(3), [0.4, -0.3, 0.2]))
    if kind == "ico2_affine":
        V, F = G.icosphere(2)
        A = G.random_rotation(rng) @ np.diag([0.5, 1.4, 1.0]) @ G.random_rotation(rng).T
        return G.SceneObject(G.make_triangle_mesh(V, F), pg.DOF_AFFINE, G.affine_dofs(A, [3.0, 5.0, 7.5]))
    if kind == "mesh_dof":
        V, F = G.icosphere(2)
        V = V * (1 + 0.1 * rng.normal(size=(len(V), 1))) + np.array([1.0, 2.0, 0.5])
        return G.SceneObject(G.make_triangle_mesh(V, F), pg.DOF_TRIANGLE_MESH, V.reshape(-1))
    if kind == "box_far":
        V, F = G.create_unit_cube_mesh()
        return G.SceneObject(G.make_triangle_mesh(V, F), pg.DOF_AFFINE,
                             G.affine_dofs(G.random_rotation(rng) * 1.7, [7.9, 0.2, 6.5]))
    if kind == "disks":
        P, N, R = G.create_sphere_pointcloud(700)
        return G.SceneObject(G.make_point_cloud(P, N, R), pg.DOF_AFFINE, G.affine_dofs(np.eye(3), [0.3, 0, 0]))
    if kind == "disks_affine":
        P, N, R = G.create_sphere_pointcloud(500)
        A = np.eye(3) + 0.2 * rng.normal(size=(3, 3))
        return G.SceneObject(G.make_point_cloud(P, N, R), pg.DOF_AFFINE, G.affine_dofs(A, [0.1, 0.2, -0.1]))
    if kind == "gauss":
        P, N, S, W = G.create_sphere_gaussians(600)
        return G.SceneObject(G.make_gaussian_splat(P, N, S, W), pg.DOF_AFFINE, G.affine_dofs(np.eye(3), [0, 0.4, 0]))
    if kind == "gauss_affine":
        P, N, S, W = G.create_sphere_gaussians(400)
        A = np.eye(3) + 0.2 * rng.normal(size=(3, 3))
        return G.SceneObject(G.make_gaussian_splat(P, N, S, W), pg.DOF_AFFINE, G.affine_dofs(A, [-0.2, 0.1, 0.3]))
    raise KeyError(kind)


KINDS = ["cube", "ico3", "ico2_affine", "mesh_dof", "box_far", "disks", "disks_affine", "gauss", "gauss_affine"]


@pytest.fixture(scope="module")
def kg29():
    return standard_kgrid(29, 32)


@pytest.mark.parametrize("kind", KINDS)
def test_form_factors_match_oracle(cuda, orc, kg29, kind):
    obj = shapes(kind, np.random.default_rng(KINDS.index(kind)))
    Jg = gpu_J(kg29, [obj])
    Jo = orc.form_factor_matrix(to_oracle(orc, [obj]), kg29.dirs, kg29.kmag)
    check_J(Jg, Jo)


@pytest.mark.parametrize("L", [2, 3, 6, 33])
def test_partial_radial_blocks_match_oracle(cuda, orc, L):
    """Radius counts that leave the last radial block partly empty: the
    form-factor kernel takes 2 radii per thread below 4 radii, 4 below 32,
    8 from 32 on, in pairs for its packed FP32 loops (L = 3: blocks of 2 + 1;
    L = 6: 4 + 2; L = 33: four blocks of 8 + 1)."""
    kg = standard_kgrid(9, L)
    rng = np.random.default_rng(L)
    objs = [shapes(k, rng) for k in ("ico3", "ico2_affine", "disks_affine", "gauss")]
    Jg = gpu_J(kg, objs)
    Jo = orc.form_factor_matrix(to_oracle(orc, objs), kg.dirs, kg.kmag)
    check_J(Jg, Jo)


def test_volume_matrix_matches_oracle(cuda, orc, kg29):
    rng = np.random.default_rng(42)
    objs = [shapes(k, rng) for k in KINDS]
    V = core.volume_matrix(kg29, objs).cpu().numpy()
    R, _, _ = orc.volume_matrix(to_oracle(orc, objs), (kg29.dirs, kg29.kmag, kg29.w))
    assert np.array_equal(V, V.T)
    err = cond_rel_err(V, R)
    print(f"\nvolume matrix, 32 radii: max cond rel err {err.max():.3e}")
    assert err.max() <= VOL_TOL, (err.max(), np.unravel_index(err.argmax(), err.shape))


@pytest.mark.parametrize("seed", [3, 11])
def test_volume_matrix_64_radii_matches_oracle(cuda, orc, seed):
    """The same object kinds on a 64-radius grid (k up to 1,832, where the
    quadrature weights are largest): a mesh against a disk cloud measured
    2.3e-5 and 1.5e-5 here while a disk's |k'_perp|^2 was formed as the
    difference qd - (k'.n)^2, and FP32 element centroids alone leave phase
    errors of k |m| 6e-8 rad."""
    kg = standard_kgrid(29, 64)
    rng = np.random.default_rng(seed)
    objs = [shapes(k, rng) for k in KINDS]
    V = core.volume_matrix(kg, objs).cpu().numpy()
    R, _, _ = orc.volume_matrix(to_oracle(orc, objs), (kg.dirs, kg.kmag, kg.w))
    err = cond_rel_err(V, R)
    print(f"\n64 radii, seed {seed}: max cond rel err {err.max():.3e}")
    assert err.max() <= VOL_TOL, (err.max(), [KINDS[i] for i in np.unravel_index(err.argmax(), err.shape)])


def test_far_translation_leaves_volumes_unchanged(cuda, orc):
    """Every object moved by the same far offset (|t| ~ 4,600, so origin
    phases k.o reach ~9e6 rad at the largest of 64 radii) gives the same volume
    matrix: element phases stay in each object's local frame and the origin
    phase is formed and reduced in FP64.  The unmoved matrix is checked
    against the oracle on this 64-radius grid (k up to 1,832), where FP32
    element centroids alone would leave phase errors of k |m| 6e-8 rad
    (3.3e-5 conditioned on the cube row)."""
    kg = standard_kgrid(29, 64)
    rng = np.random.default_rng(7)
    objs = [shapes(k, rng) for k in KINDS]
    shift = np.array([3000.0, -2500.0, 2000.0])

    def moved(o):
        d = o.dofs.copy()
        if o.dof_type == pg.DOF_AFFINE:
            d[:3] += shift
        else:  # vertex DoFs
            d = (d.reshape(-1, 3) + shift).reshape(-1)
        return G.SceneObject(o.geom, o.dof_type, d)

    V = core.volume_matrix(kg, objs).cpu().numpy()
    R, _, _ = orc.volume_matrix(to_oracle(orc, objs), (kg.dirs, kg.kmag, kg.w))
    assert cond_rel_err(V, R).max() <= VOL_TOL
    assert float(np.max(kg.kmag)) * np.linalg.norm(shift) > 6.6e6  # past 2^22 quarter turns
    V2 = core.volume_matrix(kg, [moved(o) for o in objs]).cpu().numpy()
    err = cond_rel_err(V2, V)
    print(f"\nfar translation: max cond rel change {err.max():.3e}")
    assert err.max() <= VOL_TOL


def test_pair_sweep_config_matches_oracle(cuda, orc):
    """Cube x icosphere-3 at the 64 seeded offsets, N_k = 9,664, through the
    reference-facing pair entry point (host buffers)."""
    kg, cube, spheres, offsets, _ = configs.pair_sweep()
    from pointint_gb300 import pointint_cpp as pc
    J = orc.form_factor_matrix(to_oracle(orc, [cube] + spheres), kg.dirs, kg.kmag)
    ref = np.array([np.sum(kg.w * (J[:, 0] * np.conj(J[:, 1 + i])).real) / (8 * np.pi ** 3) for i in range(64)])
    diag = np.array([np.sum(kg.w * np.abs(J[:, i]) ** 2) / (8 * np.pi ** 3) for i in range(65)])
    got = []
    for s in spheres:
        o1, o2 = cube.as_c(), s.as_c()
        v = ctypes.c_double()
        _lib.check(_lib.lib().pi_pair_volume_host(ctypes.byref(o1), ctypes.byref(o2), kg.dirs.ctypes.data,
                                                  kg.kmag.ctypes.data, kg.w.ctypes.data, kg.num_nodes,
                                                  ctypes.byref(v)))
        got.append(v.value)
    got = np.array(got)
    scale = 1e-3 * np.sqrt(diag[0] * diag[1:])
    err = np.abs(got - ref) / np.maximum(np.abs(ref), scale)
    print(f"\npair sweep: max cond rel err {err.max():.3e}")
    assert err.max() <= VOL_TOL, err.max()
    # identical through the drop-in Python binding (identity DoFs, offsets baked into geometry)
    Vs, Fs = G.icosphere(3)
    g2 = pc.make_triangle_mesh(Vs + offsets[5], Fs)
    v5 = pc.compute_intersection_volume_cuda(cube.geom, g2, kg)
    assert abs(v5 - ref[5]) <= VOL_TOL * max(abs(ref[5]), scale[5])


def test_registry_plugin_compute_Ak(cuda, orc, kg29):
    """pi_compute_Ak writes Q complex doubles to caller-owned device memory
    (CudaComputeAkFunc, dof_cuda_interface.hpp:24-30)."""
    obj = shapes("ico2_affine", np.random.default_rng(3))
    out = torch.zeros(kg29.num_nodes * 2, dtype=torch.float64, device="cuda")
    c = obj.as_c()
    _lib.check(_lib.lib().pi_compute_Ak(ctypes.byref(c), kg29.dirs.ctypes.data, kg29.kmag.ctypes.data,
                                        kg29.num_nodes, ctypes.c_void_p(out.data_ptr()), 256))
    got = out.cpu().numpy().view(np.complex128)
    ref = orc.form_factor_matrix(to_oracle(orc, [obj]), kg29.dirs, kg29.kmag)[:, 0]
    check_J(got[None, :], ref[:, None])


def test_single_k_compute_Ak(cuda, orc):
    from pointint_gb300 import pointint_cpp as pc
    V, F = G.create_unit_cube_mesh()
    g = pc.make_triangle_mesh(V, F)
    for k in ([1.0, 0, 0], [0.3, -2.0, 1.1], [0, 0, 0], [40.0, 3.0, -7.0]):
        a = pc.compute_Ak_cuda(g, k)
        exact = 1j * np.linalg.norm(k) * orc.exact_cube_form_factor(*k)
        assert abs(a - exact) <= 2e-6 * max(1.0, np.linalg.norm(k))


@pytest.mark.parametrize("kind", ["ico2_affine", "mesh_dof", "disks_affine", "gauss_affine"])
def test_registry_gradient_plugin_and_single_k_gradient(cuda, orc, kg29, kind):
    """pi_compute_Ak_gradient (the registry's gradient function: Q x D
    complex doubles on the device, dof_cuda_interface.hpp:32-40) and
    compute_Ak_gradient_cuda (one k-vector, compute_intersection_volume.hpp:129-135)
    against the oracle's dA(k)/dtheta (affine_dof.cpp:172-322,
    triangle_mesh_dof.cpp:76-143), within 2e-5 of the largest entry."""
    from pointint_gb300 import pointint_cpp as pc
    obj = shapes(kind, np.random.default_rng(KINDS.index(kind)))
    D = len(obj.dofs)
    sel = np.arange(0, kg29.num_nodes, 37)
    dirs, kmag = np.ascontiguousarray(kg29.dirs[sel]), np.ascontiguousarray(kg29.kmag[sel])
    out = torch.zeros(len(sel) * D * 2, dtype=torch.float64, device="cuda")
    c = obj.as_c()
    _lib.check(_lib.lib().pi_compute_Ak_gradient(ctypes.byref(c), dirs.ctypes.data, kmag.ctypes.data, len(sel),
                                                 ctypes.c_void_p(out.data_ptr()), 256))
    got = out.cpu().numpy().view(np.complex128).reshape(len(sel), D)
    ref = orc.form_factor_grad(to_oracle(orc, [obj])[0], dirs * kmag[:, None])
    err = np.abs(got - ref).max() / np.abs(ref).max()
    print(f"\n{kind}: registry gradient plugin, {len(sel)} nodes x {D} DoFs: max err {err:.2e}")
    assert err <= 2e-5, err
    for q in (0, len(sel) // 2, len(sel) - 1):
        k = dirs[q] * kmag[q]
        g1 = pc.compute_Ak_gradient_cuda(obj.geom, k, obj.dof_type, obj.dofs)
        assert np.abs(g1 - ref[q]).max() <= 2e-5 * np.abs(ref).max()
    assert not pc.compute_Ak_gradient_cuda(obj.geom, [0.0, 0.0, 0.0], obj.dof_type, obj.dofs).any()


def test_cpu_binding_name_returns_the_volume(cuda, orc, kg29):
    """compute_intersection_volume_cpu (bindings.cpp:63-69) returns the
    intersection volume (computed by the GPU kernels) rather than raising."""
    from pointint_gb300 import pointint_cpp as pc
    Vc, Fc = G.create_unit_cube_mesh()
    Vs, Fs = G.icosphere(3)
    g1, g2 = pc.make_triangle_mesh(Vc, Fc), pc.make_triangle_mesh(Vs * 0.7 + 0.2, Fs)
    v_cpu = pc.compute_intersection_volume_cpu(g1, g2, kg29)
    v_gpu = pc.compute_intersection_volume_cuda(g1, g2, kg29)
    ref = orc.pair_volume(orc.Obj(0, g1.elems), orc.Obj(0, g2.elems), (kg29.dirs, kg29.kmag, kg29.w))["volume"]
    assert v_cpu == v_gpu
    assert abs(v_cpu - ref) <= VOL_TOL * abs(ref)


def test_ball_transform(cuda, orc):
    """Second analytic oracle: icospheres rescaled to the unit ball's volume
    against the exact ball transform A(k) = i|k| F_ball(k)
    (form_factor_helpers.cpp:162-173), |k| < 8.  The polyhedron differs from
    the ball by O(h^2): the error falls ~4x per subdivision level and is
    within 3e-5 of the ball's volume at level 5."""
    kg = standard_kgrid(9, 16)
    sel = kg.kmag < 8.0
    sub = KGrid(kg.dirs[sel], kg.kmag[sel], kg.w[sel])
    ex = np.array([1j * k * orc.exact_sphere_form_factor(k, 1.0) for k in sub.kmag])
    vball = 4.0 / 3.0 * np.pi
    errs = []
    for level in (4, 5):
        V, F = G.icosphere(level)
        g = G.make_triangle_mesh(V, F)
        s = (vball / G.self_volume(G.SceneObject(g))) ** (1.0 / 3.0)
        obj = G.SceneObject(G.make_triangle_mesh(V * s, F))
        A = core.form_factors(sub, core.ObjectBatch([obj]), False).cpu().numpy()[0]
        errs.append(np.abs(A - ex).max() / vball)
    print(f"\nball transform: max |A - exact| / V = {errs[0]:.2e} (level 4), {errs[1]:.2e} (level 5)")
    assert errs[1] <= 3e-5 and errs[0] / errs[1] > 3.0


def test_edge_cases(cuda, orc):
    """Empty object, degenerate triangle, k = 0 node, non-tensor grid with an
    odd node count, negative weights, object count not a multiple of 64."""
    rng = np.random.default_rng(9)
    empty = G.SceneObject(G.Geometry(pg.GEOM_TRIANGLE, np.zeros(0, dtype=G.TRI_DTYPE)))
    V = np.array([[0, 0, 0], [1, 0, 0], [2, 0, 0.0]])
    degen = G.SceneObject(G.make_triangle_mesh(V, np.array([[0, 1, 2]])))
    objs = [shapes("cube", rng), empty, degen] + [shapes("ico2_affine", rng) for _ in range(66)]
    # generic grid: random k-vectors (one exactly zero), odd count, some negative weights
    Q = 1001
    dirs = rng.normal(size=(Q, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    kmag = rng.uniform(0, 6, size=Q)
    kmag[17] = 0.0
    w = rng.uniform(0.5, 1.5, size=Q) * 0.05
    w[::7] *= -1.0
    kg = KGrid(dirs, kmag, w)
    assert kg.info() == (Q, Q, 1)
    Jg = gpu_J(kg, objs)
    Jo = orc.form_factor_matrix(to_oracle(orc, objs), dirs, kmag)
    assert np.all(Jg[1] == 0) and np.all(Jg[2] == 0) and np.all(Jg[:, 17] == 0)
    check_J(Jg, Jo)
    Vg = core.volume_matrix(kg, objs).cpu().numpy()
    R = orc.contract(Jo, w)
    err = np.abs(Vg - R) / (np.abs(R) + 1e-3 * np.sqrt(np.abs(np.outer(np.diag(R), np.diag(R)))) + 1e-12)
    assert err.max() <= VOL_TOL
    assert np.all(Vg[1] == 0) and np.all(Vg[:, 2] == 0)
    # the tensor-core contraction refuses negative weights with a status
    with pytest.raises(_lib.PointIntError):
        Jw = core.form_factors(kg, core.ObjectBatch(objs[:3]), True)
        core.contract(kg, Jw, "bf16x3")


def test_batch_set_dofs_matches_rebuild(cuda, orc, kg29):
    rng = np.random.default_rng(5)
    objs = [shapes("ico2_affine", rng), shapes("disks_affine", rng)]
    b = core.ObjectBatch(objs)
    new = G.affine_dofs(G.random_rotation(rng) * 0.9, [1.0, 1.0, 1.0])
    b.set_dofs(0, torch.tensor(new, dtype=torch.float64, device="cuda"))
    J1 = core.form_factors(kg29, b, False).cpu().numpy()
    objs[0] = G.SceneObject(objs[0].geom, pg.DOF_AFFINE, new)
    J2 = gpu_J(kg29, objs)
    assert np.array_equal(J1, J2)


def test_deterministic_reruns(cuda, kg29):
    rng = np.random.default_rng(8)
    objs = [shapes(k, rng) for k in KINDS]
    V1 = core.volume_matrix(kg29, objs).cpu().numpy()
    V2 = core.volume_matrix(kg29, objs).cpu().numpy()
    assert np.array_equal(V1, V2)


def test_host_entry_point_matches_device_path(cuda, kg29):
    rng = np.random.default_rng(12)
    objs = [shapes(k, rng) for k in KINDS]
    Vh = core.volume_matrix_host(kg29, objs)
    Vd = core.volume_matrix(kg29, objs).cpu().numpy()
    assert np.array_equal(Vh, Vd)
    assert _lib.launch_count() > 0


def test_host_entry_point_large_batch_matches_device_path(cuda, kg29):
    """The host entry on a batch of 13.8 MB of elements (24 instances of one
    icosphere-4 mesh, whose element array the host entry uploads once, 4
    copies of a second mesh, and objects of every kind), its buffers carved
    from one device block: bit for bit the device path's result."""
    rng = np.random.default_rng(21)
    V4, F4 = G.icosphere(4)
    shared = G.make_triangle_mesh(V4, F4)
    objs = [G.SceneObject(shared, pg.DOF_AFFINE,
                          G.affine_dofs(G.random_rotation(rng) * rng.uniform(0.6, 1.4), rng.uniform(0, 4, 3)))
            for _ in range(24)]
    other = G.make_triangle_mesh(*G.icosphere(3))
    objs += [G.SceneObject(other, pg.DOF_AFFINE, G.affine_dofs(np.eye(3) * (1 + 0.1 * i), [0.2 * i, 0, 0]))
             for i in range(4)]
    objs += [shapes(k, rng) for k in KINDS[:8]]
    assert sum(o.geom.elems.nbytes for o in objs) > 8 * (1 << 20)
    assert objs[0].geom.elems is objs[23].geom.elems
    Vh = core.volume_matrix_host(kg29, objs, "fp16x3")
    Vd = core.volume_matrix(kg29, objs, "fp16x3").cpu().numpy()
    assert np.array_equal(Vh, Vd)


@pytest.mark.slow
def test_matrix256_subsampled_parity_and_properties(cuda, orc):
    """Full-size 256-object workload: J parity at every 61st k-node (oracle
    cost bounded), the volumes of 10 of its objects on the full grid against
    the oracle, symmetry, and translation invariance of V."""
    kg, objs, _ = configs.matrix256()
    b = core.ObjectBatch(objs)
    J = core.form_factors(kg, b, False).cpu().numpy()
    stride = 61
    Jo = orc.form_factor_matrix(to_oracle(orc, objs), kg.dirs, kg.kmag, stride=stride)
    sel = np.arange(0, kg.num_nodes, stride)
    check_J(J[:, sel], Jo[sel])
    # volumes on the full grid for 10 of the objects (5 icospheres, 5 boxes,
    # 45 pairs), the GPU's form factors against the oracle's, both contracted
    # in FP64.  (Volumes over a subset of the nodes are not a test of the
    # configuration: with every 61st node the few nodes at the largest radius,
    # where a box's FP32 edge phases k |e| 6e-8 rad leave ~3e-5 of its form
    # factor, carry 61x the weight they have in the full quadrature.)
    rows = [3, 7, 50, 99, 127, 128, 200, 244, 250, 255]
    Jr = orc.form_factor_matrix(to_oracle(orc, [objs[r] for r in rows]), kg.dirs, kg.kmag).T
    Jg = J[rows].astype(np.complex128)
    Vg = ((Jg * kg.w) @ Jg.conj().T).real / (8 * np.pi ** 3)
    Vo = ((Jr * kg.w) @ Jr.conj().T).real / (8 * np.pi ** 3)
    err = cond_rel_err(Vg, Vo)
    print(f"\nmatrix256, 10 objects on the full grid: volumes vs the oracle, max cond rel err {err.max():.3e}")
    assert err.max() <= VOL_TOL
    V = core.volume_matrix(kg, b).cpu().numpy()
    assert np.array_equal(V, V.T)
    # global translation leaves every V_ij unchanged
    shift = np.array([0.37, -1.1, 2.3])
    moved = [G.SceneObject(o.geom, o.dof_type, np.concatenate([o.dofs[:3] + shift, o.dofs[3:]])) for o in objs]
    V2 = core.volume_matrix(kg, moved).cpu().numpy()
    assert cond_rel_err(V2, V).max() <= VOL_TOL
    # self volumes are close to the divergence-theorem volumes; the gap is the
    # reference quadrature's discretisation error (largest for the small boxes)
    sv = np.array([G.self_volume(o) for o in objs])
    gap = np.abs(np.diag(V) - sv) / sv
    print(f"\nmatrix256: max |V_ii - V_div| / V_div = {gap.max():.3e} (median {np.median(gap):.3e})")
    assert np.median(gap) <= 0.05 and gap.max() <= 0.5
