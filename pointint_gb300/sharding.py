"""k-range sharding of the volume matrix across ranks.

V = Re(J^H diag(w) J) / (8 pi^3) is a sum over k-nodes, so a k-grid can be cut
into shards, each rank computing the partial sum over its own nodes, and the
partials summed with one all-reduce of n x n values (the only exchange; form
factors never move).  Gradients are sums over the same nodes and reduce the
same way.

Shards take every `world`-th radial node of a Gauss-Legendre x Lebedev grid
(q = r M + j), so each shard keeps whole Lebedev spheres and sees small and
large |k| alike; a grid without that structure is cut node by node, also
strided.  On one GPU per process the default compute is the device path of
pointint_gb300.core; `compute` can replace it (the CPU tests pass the FP64
oracle).
"""
from __future__ import annotations

import numpy as np

from .kgrid import KGrid


def radial_structure(kg: KGrid) -> tuple[int, int]:
    """(M, L) when the grid is in the reference's tensor order q = r M + j with
    kmag constant over each block of M nodes and the same directions in every
    block; (Q, 1) otherwise."""
    Q = kg.num_nodes
    if Q == 0:
        return 0, 0
    M = 1
    while M < Q and kg.kmag[M] == kg.kmag[0]:
        M += 1
    if Q % M:
        return Q, 1
    L = Q // M
    d = kg.dirs.reshape(L, M, 3)
    k = kg.kmag.reshape(L, M)
    if not (np.all(d == d[0:1]) and np.all(k == k[:, :1])):
        return Q, 1
    return M, L


def shard_nodes(kg: KGrid, rank: int, world: int) -> np.ndarray:
    """Indices of the k-nodes owned by `rank` (ascending)."""
    if world < 1 or not (0 <= rank < world):
        raise ValueError("need 0 <= rank < world")
    M, L = radial_structure(kg)
    if L > 1:
        radii = np.arange(rank, L, world)
        return (radii[:, None] * M + np.arange(M)[None, :]).reshape(-1)
    return np.arange(rank, kg.num_nodes, world)


def kgrid_shard(kg: KGrid, rank: int, world: int) -> KGrid:
    """The k-grid of one shard (a KGrid of its own, tensor order preserved)."""
    idx = shard_nodes(kg, rank, world)
    return KGrid(kg.dirs[idx], kg.kmag[idx], kg.w[idx])


def volume_matrix_sharded(kg: KGrid, objects, precision: str = "fp32", group=None, compute=None):
    """Volume matrix of `objects` with the k-grid split over the ranks of
    `group` (torch.distributed, already initialised).  Every rank returns the
    full n x n matrix (float64 torch tensor on the rank's compute device)."""
    import torch
    import torch.distributed as dist
    rank = dist.get_rank(group)
    world = dist.get_world_size(group)
    sub = kgrid_shard(kg, rank, world)
    n = len(objects)
    if sub.num_nodes == 0:  # more ranks than radial nodes: this rank adds nothing
        device = "cpu" if compute is not None or dist.get_backend(group) == "gloo" else "cuda"
        V = torch.zeros((n, n), dtype=torch.float64, device=device)
    elif compute is None:
        from . import core
        V = core.volume_matrix(sub, objects, precision)
    else:
        V = torch.as_tensor(compute(sub, objects), dtype=torch.float64)
    dist.all_reduce(V, op=dist.ReduceOp.SUM, group=group)
    return V
