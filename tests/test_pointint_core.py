"""pointint.core: the reference's Python package name, computing the Fourier
volume through the GB300 library (no CPU path)."""
import numpy as np
import pytest


def test_pointint_core_imports_with_the_reference_entry_points():
    import inspect

    import pointint.core as pc
    for name in ("get_mesh_intersection_volume", "get_ptcld_intersection_volume", "volume_matrix", "Scene",
                 "form_factors", "contract", "ObjectBatch", "standard_kgrid", "Server"):
        assert hasattr(pc, name), name
    # same leading parameters as pointint/core/api.py:6-14 and :40-47
    assert list(inspect.signature(pc.get_ptcld_intersection_volume).parameters)[:7] == \
        ["P1", "N1", "P2", "N2", "eps", "k_neighbors", "device"]
    assert list(inspect.signature(pc.get_mesh_intersection_volume).parameters)[:6] == \
        ["vertices1", "faces1", "vertices2", "faces2", "eps", "device"]


def test_knn_area_weights_of_an_even_sphere_sample():
    from pointint.core import knn_area_weights
    from pointint_gb300 import geometry as G
    P, _, _ = G.create_sphere_pointcloud(4000)
    W = knn_area_weights(P, 30)
    assert abs(W.sum() / (4 * np.pi) - 1.0) < 0.05  # total area of the unit sphere


@pytest.mark.gpu
def test_pointint_core_pair_volumes_match_oracle(cuda, orc):
    import pointint.core as pc
    from pointint_gb300 import geometry as G
    kg = pc.default_kgrid()
    Vc, Fc = G.create_unit_cube_mesh()
    Vs, Fs = G.icosphere(3)
    Vs = Vs * 0.7 + np.array([0.2, -0.1, 0.3])
    v = pc.get_mesh_intersection_volume(Vc, Fc, Vs, Fs, device="cuda:0")
    ref = orc.pair_volume(orc.Obj(0, orc.pack_tris(Vc, Fc)), orc.Obj(0, orc.pack_tris(Vs, Fs)),
                          (kg.dirs, kg.kmag, kg.w))["volume"]
    assert abs(v - ref) <= 1e-5 * abs(ref)
    P1, N1, _ = G.create_sphere_pointcloud(1500)
    P2 = P1 * 0.8 + np.array([0.5, 0.0, 0.0])
    W1, W2 = pc.knn_area_weights(P1), pc.knn_area_weights(P2)
    v = pc.get_ptcld_intersection_volume(P1, N1, P2, N1)
    ref = orc.pair_volume(orc.Obj(1, orc.pack_disks(P1, N1, W1, False)), orc.Obj(1, orc.pack_disks(P2, N1, W2, False)),
                          (kg.dirs, kg.kmag, kg.w))["volume"]
    assert abs(v - ref) <= 1e-5 * abs(ref)
