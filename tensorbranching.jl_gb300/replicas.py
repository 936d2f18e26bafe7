"""Several GPUs, one process each: the independent units of a solve (index
slices, branches) sharded over ranks.

The items of a batch do not depend on each other, so each rank contracts its
share on its own GPU and the only exchange is one scalar: the max over ranks
(an all-reduce MAX), the multi-GPU form of ``maximum(res)`` in
``dynamic_ob_mis`` (src/dynamic_ob.jl:27).  Shares are balanced by greedy
longest-first bin packing of each item's cost 2^tc.  No data moves between
GPUs.
"""
from __future__ import annotations

import heapq

import numpy as np


def shard(costs, world_size: int) -> list[list[int]]:
    """Item indices of each rank: longest first onto the least-loaded rank
    (ties to the lower rank), each share in ascending index order."""
    if world_size < 1:
        raise ValueError("world_size must be >= 1")
    heap = [(0.0, r) for r in range(world_size)]
    out: list[list[int]] = [[] for _ in range(world_size)]
    for i in sorted(range(len(costs)), key=lambda k: (-float(costs[k]), k)):
        load, r = heapq.heappop(heap)
        out[r].append(i)
        heapq.heappush(heap, (load + float(costs[i]), r))
    return [sorted(x) for x in out]


def item_costs(plans) -> list[float]:
    return [2.0 ** float(p.stats()["tc"]) for p in plans]


def solve_sharded(engine, plans, slice_vals=None, r=None, mode: str = "auto", group=None):
    """Solve a batch across the ranks of ``group`` (torch.distributed must be
    initialised; every rank passes the same batch).  Returns (max over all
    items, this rank's item indices, their results)."""
    import torch
    import torch.distributed as dist

    rank = dist.get_rank(group)
    ws = dist.get_world_size(group)
    mine = shard(item_costs(plans), ws)[rank]
    local = float("-inf")
    vals = np.zeros(0, np.float32)
    if mine:
        sub = [plans[i] for i in mine]
        sv = None if slice_vals is None else [slice_vals[i] for i in mine]
        rr = None if r is None else np.asarray(r, np.float32)[mine]
        vals, local = engine.solve_batch(sub, slice_vals=sv, r=rr, mode=mode)
    dev = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
    t = torch.tensor([local], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item()), mine, vals
