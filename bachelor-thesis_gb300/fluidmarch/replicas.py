"""Replicas over GPUs: the march has no exchange step.

Rays, views and scenes are independent (the reference marches every pixel on
its own, RayMarcher.cpp:256-344), so several GPUs split the work and never
talk during a frame: one process per GPU renders its share; only the
measurement combines the ranks (total units over the slowest rank's time).

* ``shard_views``   splits a list of views (with costs, e.g. pixel counts)
                    over ranks, longest first onto the least-loaded rank, so
                    every rank gets a fixed, deterministic subset;
* ``throughput``    units of all ranks over the slowest rank's seconds (a
                    SUM and a MAX all-reduce on the given process group).
"""

from __future__ import annotations

import heapq


def shard_views(costs, world: int) -> list:
    """Indices of the views each of `world` ranks renders (greedy longest-first)."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(costs)), key=lambda i: (-float(costs[i]), i))
    heap = [(0.0, r) for r in range(world)]
    out = [[] for _ in range(world)]
    for i in order:
        load, r = heapq.heappop(heap)
        out[r].append(i)
        heapq.heappush(heap, (load + float(costs[i]), r))
    return [sorted(v) for v in out]


def throughput(units: float, seconds: float, dist=None, device=None) -> tuple:
    """(total units / max seconds, total units, max seconds) over the ranks of `dist`'s default group."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return units / seconds, units, seconds
    import torch

    t = torch.tensor([float(units), float(seconds)], dtype=torch.float64, device=device)
    u = t[:1].clone()
    s = t[1:].clone()
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    dist.all_reduce(s, op=dist.ReduceOp.MAX)
    total, tmax = float(u.item()), float(s.item())
    return total / tmax, total, tmax
