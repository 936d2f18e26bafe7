"""Serving MIS requests with continuous batching (tb_serve_* in include/tb.h).

A request is one graph: the host side prepares it (kernelization, contraction
order, index slicing when its space complexity exceeds a cap) into one or more
items (plan, slice values, r); the engine's owner thread admits requests as
device memory, item slots and stream slots free up, and runs the requests
admitted together as one cohort on its own stream without waiting for it, so
new requests overlap with running ones.

The workload generator restates the serving mix: 3-regular graphs and
King's subgraphs at filling 0.8, unit or U{1..10} weights, arriving as a
Poisson process.  King's subgraphs span L in [10, 36] (the reductions leave
kernels of sc <= ~18 even at L = 36).  3-regular graphs stop at n = 200: the
work of a contraction order of a random 3-regular graph grows about as
2^(0.16 n) (this host's annealer: ~2^31 at n = 180, ~2^42 at n = 220 after two
seconds of annealing), so n = 400 (~2^64) is out of reach of any order and of
any serving latency.
"""
from __future__ import annotations

import ctypes
import threading
import time
from ctypes import c_double, c_float, c_int32, c_int64, c_void_p
from dataclasses import dataclass, field

import numpy as np

from . import _native
from . import mis as _mis
from . import order as _order
from .engine import Engine, Plan
from .graphs import Graph, random_ksg, random_regular_graph, random_weights
from .network import CompressedEinsum


@dataclass
class Prepared:
    """A request ready for submission: its items and the known offset r."""

    name: str
    graph: Graph
    weights: np.ndarray
    plans: list = field(default_factory=list)
    slice_vals: list = field(default_factory=list)
    r: list = field(default_factory=list)
    constant: float | None = None  # kernel emptied the graph: the answer is r

    @property
    def n_items(self) -> int:
        return len(self.plans)


def prepare(engine: Engine, g: Graph, w, sc_cap: float = 24.0, name: str = "", seed: int = 0) -> Prepared:
    """Kernelize, order (min-fill + a short anneal) and index-slice a graph
    until every item has sc <= sc_cap; returns the request's items."""
    w = np.asarray(w, np.float32)
    kr = _mis.kernelize(g, w)
    p = Prepared(name, g, w)
    if kr.g.n == 0:
        p.constant = float(kr.r)
        return p
    code = _order.initialize_code(kr.g, _order.GreedyMethod(seed))
    # larger kernels get a longer anneal: their work grows as 2^tc
    big = kr.g.n > 150
    code = _order.treesa(code, _order.TreeSA(sc_target=sc_cap if not big else 20.0,
                                             betas=np.arange(0.5 if big else 1.0, 20.0 if big else 15.0,
                                                             0.1 if big else 1.0),
                                             ntrials=8 if big else 2, niters=100 if big else 20, seed=seed,
                                             nthreads=0 if big else 1))
    sliced, cc = _order.greedy_slice(code, sc_cap, 24)
    if cc[1] > sc_cap:
        raise ValueError(f"{name}: space complexity {cc[1]:.0f} after slicing 24 labels exceeds {sc_cap}")
    plan = engine.plan(code, kr.weights, sliced=sliced)
    k = len(sliced)
    rows = ((np.arange(1 << k)[:, None] >> np.arange(k)[None, :]) & 1).astype(np.int8) if k else [np.zeros(0, np.int8)]
    for row in rows:
        p.plans.append(plan)
        p.slice_vals.append(np.asarray(row, np.int8))
        p.r.append(float(kr.r))
    return p


def serving_mix(n_requests: int, seed: int, n_max: int = 200, l_max: int = 36):
    """(name, graph, weights) of the serving mix: 3-regular graphs with even n
    in [60, n_max] and King's subgraphs with L in [10, l_max] (see the module
    note on the 3-regular range)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n_requests):
        s = int(rng.integers(1 << 30))
        if rng.random() < 0.5:
            n = int(rng.integers(30, n_max // 2 + 1)) * 2
            g = random_regular_graph(n, 3, s)
            name = f"rr{n}"
        else:
            L = int(rng.integers(10, l_max + 1))
            g = random_ksg(L, 0.8, s)
            name = f"ksg{L}"
        w = np.ones(g.n, np.float32) if rng.random() < 0.5 else random_weights(g.n, s)
        out.append((name, g, w))
    return out


class Request:
    def __init__(self, server: "Server", handle, prepared: Prepared, t_submit: float):
        self.server = server
        self.handle = handle
        self.prepared = prepared
        self.t_submit = t_submit

    def done(self) -> bool:
        if self.handle is None:
            return True
        d = c_int32()
        _native.check(self.server.lib.tb_poll(self.handle, ctypes.byref(d)))
        return bool(d.value)

    def wait(self, timeout_ms: int = -1) -> tuple[float, float]:
        """(MIS value, submit-to-done latency in ms)."""
        if self.handle is None:
            return self.prepared.constant, 0.0
        v = c_float()
        lat = c_double()
        _native.check(self.server.lib.tb_wait(self.handle, timeout_ms, ctypes.byref(v), ctypes.byref(lat)))
        return float(v.value), float(lat.value)

    def free(self):
        if self.handle is not None:
            self.server.lib.tb_request_free(self.handle)
            self.handle = None


class Server:
    """tb_serve_* on an Engine (its context then serves only requests)."""

    def __init__(self, engine: Engine, pool_bytes: int = 0, max_items: int = 0):
        self.engine = engine
        self.lib = engine.lib
        _native.check(self.lib.tb_serve_start(engine.ctx, int(pool_bytes), int(max_items)), engine.ctx)
        self._open = True

    def submit(self, p: Prepared) -> Request:
        if p.constant is not None:
            return Request(self, None, p, time.perf_counter())
        n = p.n_items
        arr = (c_void_p * n)(*[pl.handle for pl in p.plans])
        sv = np.ascontiguousarray(np.concatenate([np.asarray(x, np.int8).ravel() for x in p.slice_vals])
                                  if p.slice_vals else np.zeros(0, np.int8), dtype=np.int8)
        r = np.ascontiguousarray(p.r, dtype=np.float32)
        h = c_void_p()
        st = self.lib.tb_submit(self.engine.ctx, n, ctypes.cast(arr, c_void_p), sv.ctypes.data if sv.size else None,
                                r.ctypes.data, ctypes.byref(h))
        _native.check(st, self.engine.ctx)
        return Request(self, h, p, time.perf_counter())

    def stats(self) -> dict:
        v = [c_int64() for _ in range(4)]
        _native.check(self.lib.tb_serve_stats(self.engine.ctx, *[ctypes.byref(x) for x in v]), self.engine.ctx)
        return dict(zip(("steps", "launches", "completed", "active"), (x.value for x in v)))

    def close(self):
        if self._open:
            _native.check(self.lib.tb_serve_stop(self.engine.ctx), self.engine.ctx)
            self._open = False

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def run_poisson(server: Server, prepared: list[Prepared], rate: float, seed: int = 0) -> dict:
    """Submit requests at Poisson arrival times (rate per second) from this
    thread while a waiter thread collects them; returns latencies (ms),
    results and the wall time from the first submission to the last
    completion."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, size=len(prepared)) if rate > 0 else np.zeros(len(prepared))
    reqs: list[Request] = []
    lock = threading.Lock()
    t0 = time.perf_counter()
    t_next = t0
    for p, gap in zip(prepared, gaps):
        t_next += gap
        dt = t_next - time.perf_counter()
        if dt > 0:
            time.sleep(dt)
        with lock:
            reqs.append(server.submit(p))
    lat, vals = [], []
    for q in reqs:
        v, l_ms = q.wait()
        lat.append(l_ms)
        vals.append(v)
        q.free()
    wall = time.perf_counter() - t0
    return {"latency_ms": lat, "values": vals, "wall_s": wall}
