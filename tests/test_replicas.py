"""The multi-GPU path on CPU: two gloo ranks shard a batch of independent
items, each solves its share (oracle-backed stand-in for the engine) and one
all-reduce MAX gives every rank the batch's max."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from cases import rr_case


def test_shard_balances_and_covers(tb):
    rp = tb.replicas

    costs = [2.0 ** x for x in (10, 3, 7, 10, 9, 1, 12, 4)]
    for ws in (1, 2, 3, 8, 11):
        parts = rp.shard(costs, ws)
        assert len(parts) == ws
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(costs)))
        loads = [sum(costs[i] for i in p) for p in parts]
        assert max(loads) <= max(costs) + sum(costs) / ws


class _Plan:
    def __init__(self, code, w, tc):
        self.code, self.w, self.tc = code, w, tc

    def stats(self):
        return {"tc": self.tc}


class _OracleEngine:
    """Stands in for the GPU engine in this CPU test: solves with the oracle."""

    def __init__(self, orc):
        self.orc = orc

    def solve_batch(self, plans, slice_vals=None, r=None, mode="auto"):
        r = np.zeros(len(plans), np.float32) if r is None else np.asarray(r, np.float32)
        vals = np.array([self.orc.solve(p.code, p.w) for p in plans], np.float32) + r
        return vals, float(vals.max())


def _items(tb):
    items = []
    for seed in range(7):
        g, w, code = rr_case(tb, 16 + 2 * seed, seed)
        items.append(_Plan(code, w, code.complexity()[0]))
    return items, np.arange(7, dtype=np.float32)


def _rank(rank, ws, port, q):
    import sys

    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, os.path.dirname(here))
    sys.path.insert(0, here)
    import torch.distributed as dist

    import __graft_entry__ as ge

    tb = ge.load_package()
    orc = ge.load_oracle()
    from tensorbranching_gb300 import replicas

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=ws)
    try:
        plans, r = _items(tb)
        mx, mine, vals = replicas.solve_sharded(_OracleEngine(orc), plans, r=r, mode="batched")
        q.put((rank, mx, mine, [float(v) for v in vals]))
    finally:
        dist.destroy_process_group()


def test_two_rank_gloo_solve(tb, orc):
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(k, 2, port, q)) for k in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    plans, r = _items(tb)
    want = [orc.solve(p.code, p.w) + float(x) for p, x in zip(plans, r)]
    got = {}
    for rank, mx, mine, vals in res:
        assert mx == max(want)
        got.update(dict(zip(mine, vals)))
    assert sorted(got) == list(range(len(plans)))
    assert all(got[i] == np.float32(want[i]) for i in got)
