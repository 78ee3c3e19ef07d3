"""Multi-process (world size 2, gloo on CPU) host logic of replica runs:
member sharding, max-over-ranks timing, and the barystatic volume sum of
domains coupled through one sea level."""
import os
import socket

import pytest

from fastisostasy_gb300 import replicas


def test_shard_is_a_balanced_partition():
    costs = [float((7 * i) % 11 + 1) for i in range(37)]
    parts = [replicas.shard(costs, r, 3) for r in range(3)]
    flat = sorted(i for p in parts for i in p)
    assert flat == list(range(len(costs)))
    loads = [sum(costs[i] for i in p) for p in parts]
    assert max(loads) - min(loads) <= max(costs)
    assert replicas.shard(costs, 0, 1) == list(range(len(costs)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, size, port, q):
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=size)
    try:
        r, w = replicas.world()
        mine = replicas.shard([1.0, 5.0, 2.0, 2.0, 3.0, 1.0], r, w)
        t = replicas.max_over_ranks(0.5 + rank)                 # per-rank timed region
        dv = replicas.sum_over_ranks(sum(mine) * 1e9)           # coupled barystatic volume
        q.put((rank, w, mine, t, dv))
    finally:
        dist.destroy_process_group()


def test_two_rank_gloo_group():
    pytest.importorskip("torch.distributed")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, w0, m0, t0, d0), (r1, w1, m1, t1, d1) = out
    assert (w0, w1) == (2, 2)
    assert sorted(m0 + m1) == list(range(6)) and not set(m0) & set(m1)
    assert t0 == t1 == 1.5
    assert d0 == d1 == sum(range(6)) * 1e9
