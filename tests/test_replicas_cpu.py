"""Multi-rank host logic of the view sharding (deepdrr_gb300.replicas) with world_size-2 gloo ranks
on the CPU: every view is rendered exactly once, timings reduce to their maximum, and a sharded
gradient sums to the single-process one."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist
import torch.multiprocessing as mp

from deepdrr_gb300.replicas import max_over_ranks, shard, shard_bounds, sum_gradient_


@pytest.mark.parametrize("n,world", [(0, 2), (1, 2), (32, 2), (33, 4), (7, 8), (256, 8)])
def test_shards_cover_every_view_once(n, world):
    seen = []
    sizes = []
    for r in range(world):
        part = shard(list(range(n)), r, world)
        seen += part
        sizes.append(len(part))
    assert seen == list(range(n))
    assert max(sizes) - min(sizes) <= 1


def test_shard_rejects_bad_ranks():
    with pytest.raises(ValueError):
        shard_bounds(4, 2, 2)
    with pytest.raises(ValueError):
        shard_bounds(4, 0, 0)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # a linear "back-projection": view v adds v * basis(v mod 5) to a 5-element gradient
        views = list(range(11))
        mine = shard(views, rank, world)
        g = torch.zeros(5, dtype=torch.float64)
        for v in mine:
            g[v % 5] += v
        sum_gradient_(g)
        t = max_over_ranks(10.0 + rank)
        q.put((rank, mine, g.tolist(), t))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_shard_views_and_reduce():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    results = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    results.sort()
    views = [v for _, mine, _, _ in results for v in mine]
    assert views == list(range(11))
    want = np.zeros(5)
    for v in range(11):
        want[v % 5] += v
    for _, _, g, t in results:
        np.testing.assert_array_equal(g, want)
        assert t == 11.0
