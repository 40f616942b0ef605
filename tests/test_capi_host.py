"""The C ABI library loads, exports every declared symbol, and its host-side
functions (no GPU) agree with the oracle and the reference's conventions."""
import ctypes
import os
import re

import numpy as np
import pytest

import pointint_gb300 as pg
from pointint_gb300 import _lib, geometry as G, kgrid as K

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "pointint_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(pi_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    L = _lib.lib()
    names = declared_symbols()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    assert set(names) <= set(_lib.SIGNATURES), set(names) - set(_lib.SIGNATURES)


def test_status_strings_and_version():
    L = _lib.lib()
    assert L.pi_version() >= 1
    assert L.pi_status_string(0) == b"ok"
    assert L.pi_status_string(3) == b"unsupported"


def test_struct_layouts_match_reference():
    # TriPacked 112 B, DiskPacked / GaussianPacked 64 B (types.hpp:9-37)
    assert G.TRI_DTYPE.itemsize == 112 and G.DISK_DTYPE.itemsize == 64 and G.GAUSS_DTYPE.itemsize == 64
    assert ctypes.sizeof(_lib.PiObject) == 40


def test_packing_matches_oracle(orc):
    V, F = G.icosphere(2)
    a, b = G.pack_tris(V, F), orc.pack_tris(V, F)
    assert a.tobytes() == b.tobytes()
    P, N, R = G.create_sphere_pointcloud(100)
    N2 = N * 3.0  # unnormalised input normals get normalised (packing.cpp:47)
    for is_r in (True, False):
        assert np.allclose(G.pack_disks(P, N2, R, is_r).view(np.float64), orc.pack_disks(P, N2, R, is_r).view(np.float64),
                           rtol=1e-15, atol=1e-16)
    P, N, S, W = G.create_sphere_gaussians(64)
    assert np.allclose(G.pack_gaussians(P, N, S, W).view(np.float64), orc.pack_gaussians(P, N, S, W).view(np.float64))


def test_shape_helpers_follow_reference_formulas():
    V, F = G.create_unit_cube_mesh()
    assert V.shape == (8, 3) and F.shape == (12, 3) and np.all(np.abs(V) == 0.5)
    assert abs(G.self_volume(G.SceneObject(G.make_triangle_mesh(V, F))) - 1.0) < 1e-14
    n = 500
    P, N, R = G.create_sphere_pointcloud(n)
    assert np.allclose(np.linalg.norm(P, axis=1), 1.0) and np.allclose(P, N)
    assert np.allclose(R, np.sqrt(4.0 / n))  # area 4 pi/n, rho = sqrt(area/pi)
    P, N, S, W = G.create_sphere_gaussians(n)
    assert np.allclose(W, 4 * np.pi / n) and np.allclose(S, np.sqrt(1.0 / n))
    assert P[0, 1] == 1.0 and P[-1, 1] == -1.0


def test_self_volume_matches_oracle(orc):
    rng = np.random.default_rng(0)
    V, F = G.icosphere(2)
    A = G.random_rotation(rng) @ np.diag([0.6, 1.3, 0.9])
    d = G.affine_dofs(A, [1, 2, 3])
    ob = G.SceneObject(G.make_triangle_mesh(V, F), pg.DOF_AFFINE, d)
    assert abs(G.self_volume(ob) - orc.self_volume(orc.Obj(0, G.pack_tris(V, F), 0, d))) < 1e-12
    om = G.SceneObject(G.make_triangle_mesh(V, F), pg.DOF_TRIANGLE_MESH, V.reshape(-1))
    assert abs(G.self_volume(om) - orc.self_volume(orc.Obj(0, G.pack_tris(V, F), 1, V.reshape(-1)))) < 1e-12
    P, N, R = G.create_sphere_pointcloud(300)
    od = G.SceneObject(G.make_point_cloud(P, N, R), pg.DOF_AFFINE, d)
    assert abs(G.self_volume(od) - orc.self_volume(orc.Obj(1, G.pack_disks(P, N, R), 0, d))) < 1e-12


def test_analytic_volumes_match_oracle(orc):
    rng = np.random.default_rng(4)
    for _ in range(50):
        c1, c2 = rng.normal(size=3), rng.normal(size=3)
        h1, h2 = rng.uniform(0.1, 1, 3), rng.uniform(0.1, 1, 3)
        r1, r2 = rng.uniform(0.2, 1.5, 2)
        assert G.box_box_intersection_volume(c1, h1, c2, h2) == pytest.approx(orc.box_box_intersection_volume(c1, h1, c2, h2), abs=1e-15)
        assert G.sphere_sphere_intersection_volume(c1, r1, c2, r2) == pytest.approx(
            orc.sphere_sphere_intersection_volume(c1, r1, c2, r2), rel=1e-14, abs=1e-15)


def test_kgrid_sizes_of_the_configs():
    for order, L, Q in ((29, 32, 9664), (59, 64, 76928)):
        kg = K.standard_kgrid(order, L)
        assert kg.num_nodes == Q
        assert np.all(kg.w > 0)


def test_invalid_arguments_return_status_not_crash():
    L = _lib.lib()
    assert L.pi_gauss_legendre(0, 0.0, 1.0, None, None) == 1
    assert b"n must be" in L.pi_last_error()
    assert L.pi_load_lebedev(b"/nonexistent/file.txt", None, None, 0, None) == 7
    V = np.zeros((3, 3)); F = np.array([[0, 1, 5]], dtype=np.int32)
    out = np.zeros(1, dtype=G.TRI_DTYPE)
    assert L.pi_pack_tris(V.ctypes.data, 3, F.ctypes.data, 1, out.ctypes.data) == 1
    with pytest.raises(_lib.PointIntError):
        G.pack_tris(V, F)
    obj = _lib.PiObject(0, 0, 0, None, 5, None)  # AffineDoF with 5 DoFs
    v = ctypes.c_double()
    assert L.pi_self_volume(ctypes.byref(obj), ctypes.byref(v)) == 1


def test_device_entry_points_fail_loudly_without_gpu():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    kg = K.standard_kgrid(3, 4)
    with pytest.raises(_lib.PointIntError) as ei:
        kg.handle()
    assert ei.value.status == 2
    from pointint_gb300 import pointint_cpp as pc
    V, F = pc.create_unit_cube_mesh()
    g = pc.make_triangle_mesh(V, F)
    with pytest.raises(_lib.PointIntError):
        pc.compute_intersection_volume_cuda(g, g, kg)
    with pytest.raises(_lib.PointIntError):  # the CPU binding name runs the GPU kernels too
        pc.compute_intersection_volume_cpu(g, g, kg)


def test_server_fails_loudly_without_gpu():
    """The serving entry points go through the C ABI and report the missing
    device as a status (no host fallback)."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from pointint_gb300 import geometry as G
    from pointint_gb300.serving import Server
    V, F = G.create_unit_cube_mesh()
    with pytest.raises(_lib.PointIntError):
        Server(K.standard_kgrid(3, 16), [G.SceneObject(G.make_triangle_mesh(V, F))], autotune=False)
    srv = Server.__new__(Server)
    srv._h = None
    with pytest.raises(_lib.PointIntError) as ei:
        _lib.check(_lib.lib().pi_server_submit(None, None, None, None))
    assert ei.value.status == 1
