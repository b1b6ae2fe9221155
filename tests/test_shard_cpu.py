"""Host logic of the multi-rank forms on CPU: cost-balanced sharding of
independent systems, and the max-over-ranks timing over a world-size-2
gloo process group (the bench's N > 1 path without GPUs)."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from elemental_gb300 import shard


def test_partition_covers_disjoint_and_balanced():
    rng = np.random.default_rng(0)
    ns = rng.integers(16, 513, 4096)
    kinds = ["lu" if i % 2 == 0 else "chol" for i in range(len(ns))]
    for world in (1, 2, 3, 8):
        parts = shard.partition_by_cost(ns, world, kinds)
        allidx = np.concatenate(parts)
        assert len(allidx) == len(ns) and len(np.unique(allidx)) == len(ns)
        loads = [sum(shard.system_cost(ns[i], kinds[i]) for i in p) for p in parts]
        biggest = max(shard.system_cost(n) for n in ns)
        assert max(loads) - min(loads) <= biggest + 1e-6


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        rng = np.random.default_rng(7)
        ns = rng.integers(64, 2049, 500)
        parts = shard.partition_by_cost(ns, world)
        mine = parts[rank]
        # each rank "times" its share; the job time is the slowest rank's
        t = float(sum(shard.system_cost(n) for n in ns[mine])) * 1e-12
        tmax = shard.max_over_ranks(t)
        counts = torch.tensor([len(mine)], dtype=torch.int64)
        dist.all_reduce(counts)
        # a host gather of per-system results (here: their indices)
        got = [None] * world
        dist.all_gather_object(got, mine.tolist())
        q.put((rank, t, tmax, int(counts.item()), sorted(sum(got, []))))
    finally:
        dist.destroy_process_group()


def test_two_rank_gloo_max_over_ranks_and_gather():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    ts = {r: t for r, t, _, _, _ in out}
    for r, t, tmax, count, gathered in out:
        assert tmax == pytest.approx(max(ts.values()))
        assert count == 500
        assert gathered == list(range(500))
