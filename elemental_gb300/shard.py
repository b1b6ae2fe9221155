"""Sharding of independent systems across ranks (one process per GPU).

The single large factorization does not shard in this tier (replicas only);
the batched and learned-selector forms are independent systems, split across
ranks by estimated cost with no device collective -- each rank solves its
share in its own persistent launch and only host-side results are gathered.

    partition_by_cost(ns, kinds, world) -> list of index arrays, one per rank
    max_over_ranks(t)                   -> the slowest rank's time (bench)
"""
from __future__ import annotations

import heapq

import numpy as np


def system_cost(n, kind="lu"):
    """Relative cost of one system: the factorization's flops (2/3 n^3 for
    LU, 1/3 n^3 for Cholesky)."""
    return (2.0 / 3.0 if kind == "lu" else 1.0 / 3.0) * float(n) ** 3


def partition_by_cost(ns, world, kinds=None):
    """Greedy longest-processing-time split of the systems over `world`
    ranks: largest first, each to the currently lightest rank.  Returns one
    sorted int64 index array per rank (disjoint, covering every system)."""
    ns = np.asarray(ns)
    cost = np.array([system_cost(n, kinds[i] if kinds is not None else "lu")
                     for i, n in enumerate(ns)])
    order = np.argsort(-cost, kind="stable")
    heap = [(0.0, r) for r in range(world)]
    parts = [[] for _ in range(world)]
    for i in order:
        load, r = heapq.heappop(heap)
        parts[r].append(int(i))
        heapq.heappush(heap, (load + cost[i], r))
    return [np.array(sorted(p), dtype=np.int64) for p in parts]


def max_over_ranks(t, device=None):
    """The largest of a per-rank time over the default process group (the
    bench's whole-job time); the value itself without a group."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(t)
    tt = torch.tensor([float(t)], dtype=torch.float64,
                      device=device if device is not None else "cpu")
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return float(tt.item())
