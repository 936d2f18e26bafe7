"""The benchmark workloads (synthetic, seeded), built reproducibly.

Each workload follows one configuration of the benchmark plan:

  rr100_b10   random 3-regular n=100, unit weights, kernelize + branch until
              sc <= 10 (dynamic_ob_mis with ContractionTreeSlicer(sc_target=10),
              test/dynamic_ob.jl:10-26) by the two-way vertex rule; 32 graphs
              (seeds 1..32), every branch of every graph in one batch
  rr100_ob10  the same 32 graphs branched by the reference's default rule
              (ScoreRS + GreedyBrancher, src/types.jl:43-49): fewer, larger
              branches
  rr220       random 3-regular n=220, unit weights, one contraction, no slicing
  rr220w_s22  the rr220 graph and tree with integer weights U{1..10}; index
              slicing until every slice has sc <= 22: 2^6 slices, all of them
              in one step
  rr300w_s22  the sliced batch configuration at its stated size: random
              3-regular n=300, weights U{1..10}, index-sliced to sc <= 22
              (2^22 slices of tc ~28); a step contracts evenly spaced slices
              and the rate is extrapolated by the share of slices covered
  ksg32_b20   King's subgraph L=32, filling 0.8, unit weights; kernelize +
              branch until sc <= 20 by the two-way vertex rule
  ksg32_ob20  the same King's subgraph branched by the reference's default
              rule (ScoreRS + GreedyBrancher) to sc <= 20: 186 branches
  ksg32_dom20 the same with the domination reduction as well: it leaves a
              416-vertex kernel of sc 16, so no branching (one network)

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
    "rr100_ob10": "32 random 3-regular graphs n=100 (seeds 1..32), unit weights, branched to sc<=10 by the "
                  "optimal branching rule (ScoreRS sc_score regions, GreedyBrancher)",
    "rr220": "random 3-regular n=220 (seed 1), unit weights, one contraction, no slicing",
    "rr220w_s22": "random 3-regular n=220 (seed 1), weights U{1..10} (seed 1), rr220's tree index-sliced to sc<=22",
    "rr300w_s22": "random 3-regular n=300 (seed 1), weights U{1..10} (seed 1), index-sliced to sc<=22 "
                  "(2^k slices; a step contracts evenly spaced slices of them)",
    "ksg32_b20": "King's subgraph L=32 filling 0.8 (seed 1), unit weights, isolated/pendant reductions, "
                 "branched to sc<=20 by the two-way vertex rule",
    "ksg32_ob20": "King's subgraph L=32 filling 0.8 (seed 1), unit weights, isolated/pendant reductions, "
                  "branched to sc<=20 by the optimal branching rule (ScoreRS sc_score regions, GreedyBrancher)",
    "ksg32_dom20": "King's subgraph L=32 filling 0.8 (seed 1), unit weights, every exact reduction (domination "
                   "included: 416 vertices left, sc 16), so the optimal branching rule at sc<=20 makes no branches",
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


def build_rr220w_s22() -> dict:
    base = load_raw("rr220")
    g = random_regular_graph(220, 3, base["seed"])
    ixs, iy = rawcode(g)
    code = CompressedEinsum(ixs, iy, np.array(base["code"]["children"], np.int32).reshape(-1, 2), n_labels=g.n)
    w = random_weights(220, 1)
    sliced, cc = _order.greedy_slice(code, 22, 40)
    return {"name": "rr220w_s22", "graph": {"n": g.n, "edges": [list(e) for e in g.edges]}, "seed": base["seed"],
            "weights": w.tolist(), "code": base["code"], "cc": list(code.complexity()), "sliced": sliced,
            "sliced_cc": list(cc)}


def build_rr300w_s22() -> dict:
    """3-regular n=300 (seed 1), weights U{1..10} (seed 1), index-sliced to
    sc <= 22.  The tree: min-fill, annealed at falling space targets, then
    the sliced labels chosen greedily and the tree annealed again with them
    removed (each slice's network is what runs), twice."""
    g = random_regular_graph(300, 3, 1)
    w = random_weights(300, 1)
    ixs, iy = rawcode(g)
    code = _order.initialize_code(g, _order.GreedyMethod(2))
    for rnd, (tgt, lo, hi, nit) in enumerate([(40, 0.1, 15.0, 100), (36, 0.5, 20.0, 200), (34, 1.0, 25.0, 300),
                                             (34, 1.0, 30.0, 600)]):
        c2 = _order.treesa(code, _order.TreeSA(sc_target=tgt, betas=np.arange(lo, hi, 0.05), ntrials=8, niters=nit,
                                               seed=rnd, rw_weight=0.2))
        if (c2.complexity()[1], c2.complexity()[0]) < (code.complexity()[1], code.complexity()[0]):
            code = c2
    sliced, cc = _order.greedy_slice(code, 22, 40)
    for rnd in range(3):
        cs = _order.treesa(code.remove_labels(sliced),
                           _order.TreeSA(sc_target=22, betas=np.arange(1.0, 30.0, 0.05), ntrials=8, niters=200,
                                         seed=10 + rnd, rw_weight=0.2))
        code = CompressedEinsum(ixs, iy, cs.children, n_labels=g.n)
        s2, c2 = _order.greedy_slice(code, 22, 40)
        if len(s2) + c2[0] < len(sliced) + cs.complexity()[0]:
            sliced = s2
    cc = code.remove_labels(sliced).complexity()
    return {"name": "rr300w_s22", "graph": {"n": g.n, "edges": [list(e) for e in g.edges]}, "seed": 1,
            "weights": w.tolist(), "code": _code_json(code), "cc": list(code.complexity()), "sliced": sliced,
            "sliced_cc": list(cc)}


def _pack_branches(brs: list[SlicedBranch]) -> dict:
    """Branches of one graph as flat int arrays: the kept vertices of the
    kernel graph (vmap), the elimination order each tree was built from, and
    r.  Trees are rebuilt by order2eincode (integer-deterministic)."""
    vm, vo, eo, eoo, rs, has = [], [0], [], [0], [], []
    for b in brs:
        vm.extend(b.vmap if b.vmap is not None else [])
        vo.append(len(vm))
        if b.code is not None and b.order is None:
            raise ValueError("branch tree was re-annealed: its elimination order is not stored")
        eo.extend(b.order if b.order is not None else [])
        eoo.append(len(eo))
        rs.append(b.r)
        has.append(b.code is not None)
    return {"vmap": np.array(vm, np.int32), "vmap_off": np.array(vo, np.int64), "order": np.array(eo, np.int32),
            "order_off": np.array(eoo, np.int64), "r": np.array(rs, np.float64), "has_code": np.array(has, bool)}


def _unpack_branches(kernel_g: Graph, kernel_w: np.ndarray, d) -> list[SlicedBranch]:
    out = []
    for i in range(len(d["r"])):
        vm = d["vmap"][d["vmap_off"][i]:d["vmap_off"][i + 1]].tolist()
        g, _ = kernel_g.induced_subgraph(vm)
        w = kernel_w[vm] if vm else np.zeros(0, np.float32)
        code = None
        if d["has_code"][i]:
            eo = d["order"][d["order_off"][i]:d["order_off"][i + 1]].tolist()
            code = _order.order2eincode(g, eo)
        out.append(SlicedBranch(MISProblem(g, w.astype(np.float32)), code, float(d["r"][i]), order=None, vmap=vm))
    return out


def _branch_set(g: Graph, w, sc_target: int, seed: int, init_niters: int, reductions, brancher=None):
    """Kernelize, anneal briefly, branch without re-annealing (so every tree
    is determined by its elimination order); the vertex rule unless
    ``brancher`` is given."""
    kr = _mis.kernelize(g, w, rules=reductions)
    if kr.g.n == 0:
        return kr, [SlicedBranch(MISProblem(kr.g, kr.weights), None, kr.r, vmap=[])]
    code = _order.initialize_code(kr.g, _order.GreedyMethod(seed))
    code = _order.treesa(code, _order.TreeSA(sc_target=sc_target, betas=np.arange(1.0, 15.0, 1.0), ntrials=2,
                                             niters=init_niters, seed=seed))
    slicer = _mis.ContractionTreeSlicer(sc_target=sc_target, refine=False, reductions=reductions,
                                        brancher=brancher or _mis.VertexBrancher())
    brs = _mis.slice(MISProblem(kr.g, kr.weights), code, kr.r, slicer)
    if len(brs) == 1 and brs[0].vmap is None:
        # no branching needed: the root tree is the annealed one; store its order
        b = brs[0]
        eo = _mis.eincode2order(code)
        b.order, b.vmap = eo, list(range(kr.g.n))
        b.code = _order.order2eincode(kr.g, eo)
    return kr, brs


def build_rr100_b10(brancher=None) -> dict:
    graphs = {}
    for s in range(1, 33):
        g = random_regular_graph(100, 3, s)
        kr, brs = _branch_set(g, np.ones(100, np.float32), 10, s, 20, _mis.REDUCTIONS_ALL, brancher)
        for k, v in _pack_branches(brs).items():
            graphs[f"g{s}_{k}"] = v
    return graphs


def build_rr100_ob10() -> dict:
    from .branching import GreedyBrancher

    return build_rr100_b10(GreedyBrancher())


def build_ksg32_b20() -> dict:
    # the reductions without domination (which alone empties King's subgraphs
    # with unit weights), a short annealing of the initial tree, and branching
    # without re-annealing each branch: an uneven batch of subnetworks
    g = random_ksg(32, 0.8, 1)
    kr, brs = _branch_set(g, np.ones(g.n, np.float32), 20, 1, 20, _mis.REDUCTIONS_BASIC)
    return _pack_branches(brs)


def build_ksg32_ob20() -> dict:
    # the reference's default branching rule (ScoreRS regions, GreedyBrancher
    # set cover) with the isolated / pendant reductions: 186 uneven branches
    from .branching import GreedyBrancher

    g = random_ksg(32, 0.8, 1)
    kr, brs = _branch_set(g, np.ones(g.n, np.float32), 20, 1, 20, _mis.REDUCTIONS_BASIC, GreedyBrancher())
    return _pack_branches(brs)


def build_ksg32_dom20() -> dict:
    # every exact reduction, domination included: it leaves 416 of the 804
    # vertices, whose network already has sc <= 20, so the rule makes no
    # branches (one network)
    from .branching import GreedyBrancher

    g = random_ksg(32, 0.8, 1)
    kr, brs = _branch_set(g, np.ones(g.n, np.float32), 20, 1, 20, _mis.REDUCTIONS_ALL, GreedyBrancher())
    return _pack_branches(brs)


BUILDERS = {"rr220": build_rr220, "rr220w_s22": build_rr220w_s22, "rr300w_s22": build_rr300w_s22,
            "rr100_b10": build_rr100_b10,
            "rr100_ob10": build_rr100_ob10, "ksg32_b20": build_ksg32_b20, "ksg32_ob20": build_ksg32_ob20,
            "ksg32_dom20": build_ksg32_dom20}


NPZ = {"rr100_b10", "rr100_ob10", "ksg32_b20", "ksg32_ob20", "ksg32_dom20"}
MULTI = {"rr100_b10", "rr100_ob10"}  # 32 graphs per step


def path(name: str) -> str:
    return os.path.join(DATA, name + (".npz" if name in NPZ else ".json"))


def make(name: str):
    t = time.time()
    d = BUILDERS[name]()
    os.makedirs(DATA, exist_ok=True)
    if name in NPZ:
        np.savez_compressed(path(name), **d)
    else:
        with open(path(name), "w") as f:
            json.dump(d, f, separators=(",", ":"))
    print(f"{name}: built in {time.time() - t:.0f}s", file=sys.stderr)
    return d


def load_raw(name: str):
    p = path(name)
    if not os.path.exists(p):
        raise FileNotFoundError(f"workload {name} not built; run: python bench.py --make {name}")
    if name in NPZ:
        return dict(np.load(p))
    with open(p) as f:
        return json.load(f)


# -- loaders -------------------------------------------------------------------
def gemm_node_network(m: int, n: int, k: int, bt: int, seed: int = 0):
    """An MIS network whose middle contraction is a GEMM node with m, n, k
    and bt labels in its M, N, K and batch groups: vertex groups M, N, K, Bt
    with complete M-K and N-K bipartite edges, batch vertices joined to one M
    and one N vertex, and pendant vertices keeping M, N and Bt open above the
    node.  Returns (graph, weights U{1..9}, contraction plan)."""
    rng = np.random.default_rng(seed)
    M = list(range(0, m))
    N = list(range(m, m + n))
    K = list(range(m + n, m + n + k))
    B = list(range(m + n + k, m + n + k + bt))
    base = m + n + k + bt
    OM = list(range(base, base + m))
    ON = list(range(base + m, base + m + n))
    OB = list(range(base + m + n, base + m + n + bt))
    nv = base + m + n + bt
    left_edges = [(x, y) for x in M for y in K] + [(x, y) for x in B for y in M[:1]]
    right_edges = [(x, y) for x in N for y in K] + [(x, y) for x in B for y in N[:1]]
    up_edges = list(zip(M, OM)) + list(zip(N, ON)) + list(zip(B, OB))
    g = Graph(nv, left_edges + right_edges + up_edges)
    ixs, iy = rawcode(g)
    eid = {e: nv + i for i, e in enumerate(g.edges)}
    key = lambda e: (min(e), max(e))  # noqa: E731
    ch = []
    nxt = [len(ixs)]

    def chain(ids):
        cur = ids[0]
        for x in ids[1:]:
            ch.append((cur, x))
            cur = nxt[0]
            nxt[0] += 1
        return cur

    a = chain(M + K + B + [eid[key(e)] for e in left_edges])
    b = chain(N + [eid[key(e)] for e in right_edges])
    ch.append((a, b))
    cur = nxt[0]
    nxt[0] += 1
    for (x, o) in up_edges:
        for y in (eid[key((x, o))], o):
            ch.append((cur, y))
            cur = nxt[0]
            nxt[0] += 1
    code = CompressedEinsum(ixs, iy, np.array(ch, np.int32), n_labels=nv)
    w = rng.integers(1, 10, nv).astype(np.float32)
    return g, w, code


def _gemm_workload(name: str) -> dict:
    # gemm_m<M>n<N>k<K>b<B>: one network around a GEMM node of that shape
    import re

    mt = re.fullmatch(r"gemm_m(\d+)n(\d+)k(\d+)b(\d+)", name)
    if not mt:
        raise KeyError(name)
    m, n, k, bt = (int(x) for x in mt.groups())
    g, w, code = gemm_node_network(m, n, k, bt)
    b = SlicedBranch(MISProblem(g, w), code, 0.0)
    return {"name": name, "graph": g, "branches": [b], "sliced": [], "slice_values": None}


SLICED_ITEMS_PER_STEP = 64  # slices of an index-sliced workload one benchmark step contracts


def step_items(wl: dict, max_items: int = 0) -> list[dict]:
    """The contraction items of one benchmark step, in order.

    A branch with a network is one item; a branch of an index-sliced workload
    gives evenly spaced slices (``SLICED_ITEMS_PER_STEP``, or ``max_items``),
    each fixing the sliced labels to the bits of its slice index (the first
    ``open_bits`` sliced labels stay open in the root instead).  Branches
    without a network (empty graph, value r) are not items.  Each item is a
    dict: ``branch`` (index into wl["branches"]), ``code`` (the network, open
    labels included), ``weights``, ``fixed`` (labels fixed per item),
    ``values`` (int8 row for them), ``index`` (slice index, -1 when not
    sliced) and ``r``.  Sets wl["step_fraction"], the share of all slices a
    step covers (1 when not sliced).
    """
    items = []
    sliced = wl["sliced"]
    frac = 1.0
    for bi, b in enumerate(wl["branches"]):
        if b.code is None:
            continue
        if sliced:
            ob = wl.get("open_bits", 0)
            opened, fixed = list(sliced[:ob]), list(sliced[ob:])
            code = CompressedEinsum(b.code.ixs, opened, b.code.children, n_labels=b.code.n_labels)
            k = len(fixed)
            total = 1 << k
            take = min(total, max_items or wl.get("items_per_step", SLICED_ITEMS_PER_STEP))
            frac = take / total
            idx = np.linspace(0, total - 1, take).astype(np.int64)
            vals = ((idx[:, None] >> np.arange(k)[None, :]) & 1).astype(np.int8)
            for i, row in zip(idx.tolist(), vals):
                items.append({"branch": bi, "code": code, "weights": b.p.weight_array(), "fixed": fixed,
                              "values": row, "index": int(i), "r": float(b.r)})
        else:
            items.append({"branch": bi, "code": b.code, "weights": b.p.weight_array(), "fixed": [],
                          "values": np.zeros(0, np.int8), "index": -1, "r": float(b.r)})
            if max_items and len(items) >= max_items:
                break
    wl["step_fraction"] = frac
    return items


def plans_for(engine, items: list[dict]):
    """Plans and per-item inputs of ``step_items``' items on an Engine: one
    plan per branch, shared by its slices.  Returns (plans, slice values per
    item or None when nothing is sliced, r as float32)."""
    by_branch = {}
    plans, svs, rs = [], [], []
    for it in items:
        p = by_branch.get(it["branch"])
        if p is None:
            p = by_branch[it["branch"]] = engine.plan(it["code"], it["weights"], sliced=it["fixed"])
        plans.append(p)
        svs.append(it["values"])
        rs.append(it["r"])
    if all(len(x) == 0 for x in svs):
        svs = None
    return plans, svs, np.array(rs, np.float32)


def load(name: str) -> dict:
    """Workload as host objects:
      branches     list of SlicedBranch (one per network to contract)
      sliced       labels fixed per item (index slicing), or []
      slice_values item rows for the sliced labels, or None
      mis          the known answer when the builder stored one
    """
    if name.startswith("gemm_"):
        return _gemm_workload(name)
    d = load_raw(name)
    if name == "rr220":
        g = random_regular_graph(220, 3, d["seed"])
        assert [list(e) for e in g.edges] == d["graph"]["edges"], "graph generator changed"
        ixs, iy = rawcode(g)
        code = CompressedEinsum(ixs, iy, np.array(d["code"]["children"], np.int32).reshape(-1, 2), n_labels=g.n)
        b = SlicedBranch(MISProblem(g, np.ones(g.n, np.float32)), code, 0.0)
        return {"name": name, "graph": g, "branches": [b], "sliced": [], "slice_values": None}
    if name in ("rr220w_s22", "rr300w_s22"):
        g = random_regular_graph(d["graph"]["n"], 3, d["seed"])
        assert [list(e) for e in g.edges] == d["graph"]["edges"], "graph generator changed"
        w = np.array(d["weights"], np.float32)
        ixs, iy = rawcode(g)
        code = CompressedEinsum(ixs, iy, np.array(d["code"]["children"], np.int32).reshape(-1, 2), n_labels=g.n)
        b = SlicedBranch(MISProblem(g, w), code, 0.0)
        # rr300w_s22's slices are small (tc ~28): a step takes more of them
        return {"name": name, "graph": g, "branches": [b], "sliced": list(d["sliced"]), "slice_values": None,
                "open_bits": 0, "items_per_step": 1024 if name == "rr300w_s22" else SLICED_ITEMS_PER_STEP}
    if name in MULTI:
        brs, gs = [], []
        for s in range(1, 33):
            g = random_regular_graph(100, 3, s)
            kr = _mis.kernelize(g, np.ones(100, np.float32), rules=_mis.REDUCTIONS_ALL)
            sub = {k[len(f"g{s}_"):]: v for k, v in d.items() if k.startswith(f"g{s}_")}
            gs.append(g)
            brs.append(_unpack_branches(kr.g, kr.weights, sub))
        return {"name": name, "graphs": gs, "branch_sets": brs, "branches": [b for bs in brs for b in bs],
                "sliced": [], "slice_values": None}
    if name in ("ksg32_b20", "ksg32_ob20", "ksg32_dom20"):
        g = random_ksg(32, 0.8, 1)
        rules = _mis.REDUCTIONS_ALL if name == "ksg32_dom20" else _mis.REDUCTIONS_BASIC
        kr = _mis.kernelize(g, np.ones(g.n, np.float32), rules=rules)
        brs = _unpack_branches(kr.g, kr.weights, d)
        return {"name": name, "graph": g, "branches": brs, "sliced": [], "slice_values": None}
    raise KeyError(name)
