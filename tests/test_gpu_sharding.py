"""k-range shards through the device path: the per-shard volume matrices of
three shards sum to the whole grid's matrix (FP32 path, 1e-5 conditioned), and
a single-rank process group through volume_matrix_sharded returns the whole
matrix.  Ranks that exchange partial sums are covered on CPU ranks
(tests/test_sharding.py)."""
import os
import socket

import numpy as np
import pytest
import torch

from pointint_gb300 import core
from pointint_gb300.kgrid import standard_kgrid
from pointint_gb300.sharding import kgrid_shard, volume_matrix_sharded
from test_gpu_parity import cond_rel_err
from test_sharding import _objects

pytestmark = pytest.mark.gpu


def test_shard_volumes_sum_to_whole_grid(cuda):
    kg = standard_kgrid(29, 32)
    objs = _objects()
    full = core.volume_matrix(kg, objs, "fp32").cpu().numpy()
    parts = sum(core.volume_matrix(kgrid_shard(kg, r, 3), objs, "fp32").cpu().numpy() for r in range(3))
    assert cond_rel_err(parts, full).max() <= 1e-5


def test_single_rank_group_returns_whole_matrix(cuda):
    import torch.distributed as dist
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("nccl", rank=0, world_size=1, device_id=torch.device("cuda", 0))
    try:
        kg = standard_kgrid(9, 16)
        objs = _objects()
        V = volume_matrix_sharded(kg, objs).cpu().numpy()
        ref = core.volume_matrix(kg, objs, "fp32").cpu().numpy()
        assert np.array_equal(V, ref)
    finally:
        dist.destroy_process_group()
