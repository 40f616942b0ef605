"""k-range sharding (pointint_gb300.sharding): the partition of the k-grid and
the cross-rank sum, on CPU ranks over gloo (world sizes 2 and 3).  Each rank's
partial volume matrix comes from the FP64 oracle on its shard of the grid; the
all-reduced matrix must equal the oracle on the whole grid."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from pointint_gb300 import geometry as G
from pointint_gb300.kgrid import KGrid, standard_kgrid
from pointint_gb300.sharding import radial_structure, shard_nodes, kgrid_shard


@pytest.mark.parametrize("world", [1, 2, 3, 5, 40])
def test_shards_partition_the_grid(world):
    for kg in (standard_kgrid(9, 16), standard_kgrid(3, 4)):
        M, L = radial_structure(kg)
        assert M * L == kg.num_nodes and L > 1
        parts = [shard_nodes(kg, r, world) for r in range(world)]
        allidx = np.sort(np.concatenate(parts))
        assert np.array_equal(allidx, np.arange(kg.num_nodes))
        for r, p in enumerate(parts):
            assert len(p) % M == 0  # whole Lebedev spheres
            sub = kgrid_shard(kg, r, world)
            if len(p):
                assert radial_structure(sub) == (M, len(p) // M)
    # a grid without tensor structure is cut node by node
    rng = np.random.default_rng(0)
    kg = KGrid(rng.normal(size=(37, 3)), rng.uniform(0.1, 3.0, 37), rng.uniform(0.1, 1.0, 37))
    assert radial_structure(kg) == (37, 1)
    parts = [shard_nodes(kg, r, 4) for r in range(4)]
    assert np.array_equal(np.sort(np.concatenate(parts)), np.arange(37))


def _objects():
    V, F = G.create_unit_cube_mesh()
    cube = G.SceneObject(G.make_triangle_mesh(V, F))
    Vs, Fs = G.icosphere(1)
    sph = G.SceneObject(G.make_triangle_mesh(Vs * 0.7, Fs), 0, G.affine_dofs(np.eye(3), [0.3, 0.1, -0.2]))
    P, N, R = G.create_sphere_pointcloud(60)
    disks = G.SceneObject(G.make_point_cloud(P * 0.5 + 0.2, N, R * 0.5))
    return [cube, sph, disks]


def _oracle_compute(sub, objects):
    from oracle import oracle as orc
    objs = [orc.Obj(o.geom.type, o.geom.elems, o.dof_type, o.dofs) for o in objects]
    V, _, _ = orc.volume_matrix(objs, (sub.dirs, sub.kmag, sub.w))
    return V


def _rank_main(rank, world, port, out_path):
    import torch.distributed as dist
    from pointint_gb300.sharding import volume_matrix_sharded
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        kg = standard_kgrid(9, 16)
        V = volume_matrix_sharded(kg, _objects(), group=None, compute=_oracle_compute)
        np.save(f"{out_path}.{rank}.npy", V.numpy())
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.mark.parametrize("world", [2, 3])
def test_sharded_volume_matrix_equals_whole_grid(orc, tmp_path, world):
    out = str(tmp_path / "V")
    mp.start_processes(_rank_main, args=(world, _free_port(), out), nprocs=world, join=True, start_method="spawn")
    full = _oracle_compute(standard_kgrid(9, 16), _objects())
    for r in range(world):
        V = np.load(f"{out}.{r}.npy")
        np.testing.assert_allclose(V, full, rtol=1e-12, atol=1e-15 * np.abs(full).max())
