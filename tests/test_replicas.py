"""Replicas over ranks (no exchange step): the measurement's reduction and the
view sharding, as two gloo ranks on the CPU."""

import os

import numpy as np
import pytest

from fluidmarch.replicas import shard_views, throughput

torch = pytest.importorskip("torch")


def test_shard_views_balanced_and_complete():
    rng = np.random.default_rng(3)
    costs = rng.choice([307200, 921600, 2073600], size=146)
    for world in (1, 2, 3, 8):
        parts = shard_views(costs, world)
        assert sorted(i for p in parts for i in p) == list(range(len(costs)))
        loads = [costs[p].sum() for p in parts]
        assert max(loads) - min(loads) <= costs.max()  # greedy longest-first bound
        assert parts == shard_views(costs, world)  # deterministic


def _rank(rank, world, port, q):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    # every rank rendered 1000 * (rank + 1) rays in (rank + 1) / 10 s
    v, total, tmax = throughput(1000.0 * (rank + 1), (rank + 1) / 10.0, dist, "cpu")
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, v, total, tmax))


def test_throughput_two_gloo_ranks():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29000 + (os.getpid() % 1000)
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for _, v, total, tmax in out:
        assert total == pytest.approx(3000.0)
        assert tmax == pytest.approx(0.2)
        assert v == pytest.approx(15000.0)


def test_throughput_single_process():
    assert throughput(500.0, 0.25) == (2000.0, 500.0, 0.25)
