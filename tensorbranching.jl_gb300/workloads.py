"""The benchmark workloads (synthetic, seeded), built reproducibly.

Each workload follows one configuration of the benchmark plan:

  rr100_b10   random 3-regular n=100, unit weights, kernelize + branch until
              sc <= 10 (dynamic_ob_mis with ContractionTreeSlicer(sc_target=10),
              test/dynamic_ob.jl:10-26); 32 graphs (seeds 1..32), every branch
              of every graph in one batch
  rr220       random 3-regular n=220, unit weights, one contraction, no slicing
  rr300_s22   random 3-regular n=300, integer weights U{1..10}; index slicing
              until every slice has sc <= 22; 2^k slices
  ksg32_b20   King's subgraph L=32, filling 0.8, unit weights; kernelize +
              branch until sc <= 20

Contraction trees come from simulated annealing, whose floating-point
acceptance tests can differ between machines, so each workload's trees are
stored once in ``data/<name>.json`` (written by ``python bench.py --make NAME``)
and loaded from there; the graphs themselves are regenerated from their seeds
and checked against the stored edge lists.
"""
from __future__ import annotations

import json
import os
import sys
import time

import numpy as np

from . import mis as _mis
from . import order as _order
from .graphs import Graph, random_ksg, random_regular_graph, random_weights
from .network import CompressedEinsum, MISProblem, SlicedBranch, rawcode

DATA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data")

WORKLOADS = {
    "rr100_b10": "32 random 3-regular graphs n=100 (seeds 1..32), unit weights, branched to sc<=10",
    "rr220": "random 3-regular n=220 (seed 1), unit weights, one contraction, no slicing",
    "rr300_s22": "random 3-regular n=300 (seed 3), weights U{1..10}, index-sliced to sc<=22",
    "ksg32_b20": "King's subgraph L=32 filling 0.8 (seed 1), unit weights, branched to sc<=20",
}


def _code_json(code: CompressedEinsum) -> dict:
    return {"children": code.children.tolist(), "n_labels": code.n_labels}


def _branch_json(b: SlicedBranch, vmap=None) -> dict:
    return {"n": b.p.g.n, "edges": [list(e) for e in b.p.g.edges], "weights": b.p.weight_array().tolist(),
            "r": float(b.r), "code": None if b.code is None else _code_json(b.code)}


def _branch_from(d: dict) -> SlicedBranch:
    g = Graph(d["n"], [tuple(e) for e in d["edges"]])
    w = np.array(d["weights"], np.float32)
    code = None
    if d["code"] is not None:
        ixs, iy = rawcode(g)
        code = CompressedEinsum(ixs, iy, np.array(d["code"]["children"], np.int32).reshape(-1, 2),
                                n_labels=g.n)
    return SlicedBranch(MISProblem(g, w), code, float(d["r"]))


# -- builders ------------------------------------------------------------------
def _anneal(code, sc_target, rounds=3, niters=1000, seed=0):
    best = code
    bc = code.complexity()
    for rnd in range(rounds):
        lo = 0.3 if rnd == 0 else 3.0
        opt = _order.TreeSA(sc_target=sc_target, betas=np.arange(lo, 30.0, 0.1), ntrials=8, niters=niters,
                            seed=seed * 100 + rnd)
        code = _order.treesa(code, opt)
        c = code.complexity()
        if (c[1], c[0]) < (bc[1], bc[0]):
            best, bc = code, c
    return best


def build_rr220() -> dict:
    g = random_regular_graph(220, 3, 1)
    code = _order.initialize_code(g, _order.GreedyMethod(1))
    code = _anneal(code, 24, rounds=3, niters=1000, seed=1)
    return {"name": "rr220", "graph": {"n": g.n, "edges": [list(e) for e in g.edges]}, "seed": 1,
            "weights": "unit", "code": _code_json(code), "cc": list(code.complexity())}


def build_rr300_s22() -> dict:
    g = random_regular_graph(300, 3, 3)
    w = random_weights(300, 3)
    code = _order.initialize_code(g, _order.GreedyMethod(3))
    code = _anneal(code, 30, rounds=2, niters=400, seed=3)
    sliced, cc = _order.greedy_slice(code, 22, 40)
    return {"name": "rr300_s22", "graph": {"n": g.n, "edges": [list(e) for e in g.edges]}, "seed": 3,
            "weights": w.tolist(), "code": _code_json(code), "cc": list(code.complexity()),
            "sliced": sliced, "sliced_cc": list(cc)}


def _branched(g: Graph, w, sc_target: int, seed: int) -> list[SlicedBranch]:
    kr = _mis.kernelize(g, w)
    if kr.g.n == 0:
        return [SlicedBranch(MISProblem(kr.g, kr.weights), None, kr.r)]
    code = _order.initialize_code(kr.g, _order.GreedyMethod(seed))
    code = _order.treesa(code, _order.TreeSA(sc_target=sc_target, betas=np.arange(0.5, 20, 0.25), ntrials=4,
                                             niters=60, seed=seed))
    slicer = _mis.ContractionTreeSlicer(sc_target=sc_target)
    return _mis.slice(MISProblem(kr.g, kr.weights), code, kr.r, slicer)


def build_rr100_b10() -> dict:
    graphs = []
    for s in range(1, 33):
        g = random_regular_graph(100, 3, s)
        brs = _branched(g, np.ones(100, np.float32), 10, s)
        graphs.append({"seed": s, "edges": [list(e) for e in g.edges], "branches": [_branch_json(b) for b in brs]})
    return {"name": "rr100_b10", "graphs": graphs}


def build_ksg32_b20() -> dict:
    g = random_ksg(32, 0.8, 1)
    brs = _branched(g, np.ones(g.n, np.float32), 20, 1)
    return {"name": "ksg32_b20", "graph": {"n": g.n, "edges": [list(e) for e in g.edges]}, "seed": 1,
            "branches": [_branch_json(b) for b in brs]}


BUILDERS = {"rr220": build_rr220, "rr300_s22": build_rr300_s22, "rr100_b10": build_rr100_b10,
            "ksg32_b20": build_ksg32_b20}


def path(name: str) -> str:
    return os.path.join(DATA, name + ".json")


def make(name: str) -> dict:
    t = time.time()
    d = BUILDERS[name]()
    os.makedirs(DATA, exist_ok=True)
    with open(path(name), "w") as f:
        json.dump(d, f, separators=(",", ":"))
    print(f"{name}: built in {time.time() - t:.0f}s", file=sys.stderr)
    return d


def load_raw(name: str) -> dict:
    p = path(name)
    if not os.path.exists(p):
        raise FileNotFoundError(f"workload {name} not built; run: python bench.py --make {name}")
    with open(p) as f:
        return json.load(f)


# -- loaders -------------------------------------------------------------------
def load(name: str) -> dict:
    """Workload as host objects:
      branches     list of SlicedBranch (one per network to contract)
      sliced       labels fixed per item (index slicing), or []
      slice_values item rows for the sliced labels, or None
      mis          the known answer when the builder stored one
    """
    d = load_raw(name)
    if name == "rr220":
        g = random_regular_graph(220, 3, d["seed"])
        assert [list(e) for e in g.edges] == d["graph"]["edges"], "graph generator changed"
        ixs, iy = rawcode(g)
        code = CompressedEinsum(ixs, iy, np.array(d["code"]["children"], np.int32).reshape(-1, 2), n_labels=g.n)
        b = SlicedBranch(MISProblem(g, np.ones(g.n, np.float32)), code, 0.0)
        return {"name": name, "graph": g, "branches": [b], "sliced": [], "slice_values": None}
    if name == "rr300_s22":
        g = random_regular_graph(300, 3, d["seed"])
        assert [list(e) for e in g.edges] == d["graph"]["edges"], "graph generator changed"
        w = np.array(d["weights"], np.float32)
        ixs, iy = rawcode(g)
        code = CompressedEinsum(ixs, iy, np.array(d["code"]["children"], np.int32).reshape(-1, 2), n_labels=g.n)
        b = SlicedBranch(MISProblem(g, w), code, 0.0)
        return {"name": name, "graph": g, "branches": [b], "sliced": list(d["sliced"]), "slice_values": None}
    if name == "rr100_b10":
        brs, gs = [], []
        for gd in d["graphs"]:
            g = random_regular_graph(100, 3, gd["seed"])
            assert [list(e) for e in g.edges] == gd["edges"], "graph generator changed"
            gs.append(g)
            brs.append([_branch_from(x) for x in gd["branches"]])
        return {"name": name, "graphs": gs, "branch_sets": brs, "branches": [b for bs in brs for b in bs],
                "sliced": [], "slice_values": None}
    if name == "ksg32_b20":
        g = random_ksg(32, 0.8, d["seed"])
        assert [list(e) for e in g.edges] == d["graph"]["edges"], "graph generator changed"
        brs = [_branch_from(x) for x in d["branches"]]
        return {"name": name, "graph": g, "branches": brs, "sliced": [], "slice_values": None}
    raise KeyError(name)
