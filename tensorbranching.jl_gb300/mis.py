"""Host pipeline around the GPU contraction, mirroring the reference API.

  dynamic_ob_mis       src/dynamic_ob.jl:6-28   kernelize -> order -> slice
                                                 -> contract_slices -> max
  solve_slice          src/dynamic_ob.jl:30-34  one branch, plain GPU path
  contract_slices      src/dynamic_ob.jl:36-48  all branches, one batched call
  kernelize            src/kernelize.jl:4-17    exact reductions to a fixed point
  slice                src/slice.jl:4-11        branch until sc <= sc_target
  ContractionTreeSlicer src/types.jl:43-49

The contraction itself always runs on the GPU through include/tb.h.  The
reductions are our own simplification of the reference's (which live in
OptimalBranchingMIS); the branching rule is the reference's optimal branching
(``branching``) or a plain vertex rule.  Every rule used is exact, so the MIS
value of a branch set equals the MIS of the input graph.
"""
from __future__ import annotations

import os
from dataclasses import dataclass, field

import numpy as np

from . import branching as _br
from . import order as _order
from .engine import Engine, Plan
from .graphs import Graph
from .network import CompressedEinsum, MISProblem, SlicedBranch, UnitWeight, derive_node_labels, weights_array


# ---------------------------------------------------------------------------
# kernelization
# ---------------------------------------------------------------------------
@dataclass
class KernelResult:
    g: Graph
    weights: np.ndarray
    r: float
    vmap: list[int]  # kernel vertex -> input vertex


REDUCTIONS_ALL = ("isolated", "pendant", "domination")
REDUCTIONS_BASIC = ("isolated", "pendant")


def kernelize(g: Graph, weights=None, verbose: int = 0, rules=REDUCTIONS_ALL) -> KernelResult:
    """Apply exact MIS reductions until none applies:
    isolated vertex (take it if its weight is positive), pendant vertex v with
    neighbour u and w(v) >= w(u) (take v), and neighbourhood domination
    N[u] within N[v] with w(u) >= w(v) (drop v).  ``rules`` selects a subset
    (domination alone empties most King's subgraphs with unit weights)."""
    use_dom = "domination" in rules
    use_pend = "pendant" in rules
    w = weights_array(weights, g.n).astype(np.float64)
    adj = g.adjacency()
    for u, v in g.edges:
        if u == v:  # a self-loop forbids its vertex
            adj[u].add(u)
    alive = set(range(g.n))
    r = 0.0

    def remove(x):
        alive.discard(x)
        for y in list(adj[x]):
            adj[y].discard(x)
        adj[x] = set()

    changed = True
    while changed:
        changed = False
        for v in sorted(alive):
            if v not in alive:
                continue
            if v in adj[v]:
                remove(v)
                changed = True
                continue
            nb = adj[v]
            if not nb:
                if w[v] > 0:
                    r += w[v]
                remove(v)
                changed = True
            elif len(nb) == 1 and use_pend:
                u = next(iter(nb))
                if w[v] >= w[u]:
                    r += w[v]
                    remove(u)
                    remove(v)
                    changed = True
            elif use_dom and len(nb) > 1:
                closed_v = nb | {v}
                for u in sorted(nb):
                    if w[u] >= w[v] and (adj[u] | {u}) <= closed_v:
                        remove(v)
                        changed = True
                        break
    keep = sorted(alive)
    sub, vmap = g.induced_subgraph(keep)
    return KernelResult(sub, w[vmap].astype(np.float32) if keep else np.zeros(0, np.float32), r, vmap)


# ---------------------------------------------------------------------------
# slicing by branching (ContractionTreeSlicer)
# ---------------------------------------------------------------------------
@dataclass
class VertexBrancher:
    """Two-way branching on the vertex that appears in the most large
    tensors (weighted by 2^(size - sc_target)): v out, or v in with its
    neighbours out."""


@dataclass
class ContractionTreeSlicer:
    """Branch until every branch has sc <= sc_target (ContractionTreeSlicer,
    src/types.jl:43-49).  The default rule is the reference's: a region
    chosen by ``region_selector`` and the clause set chosen by ``brancher``
    (``branching.GreedyBrancher`` / ``branching.FixedPointBrancher``);
    ``VertexBrancher()`` selects the plain two-way vertex rule."""

    sc_target: int = 30
    refine: bool = True
    refiner: _order.TreeSA = field(default_factory=lambda: _order.TreeSA(
        betas=np.arange(1.0, 16.0, 1.0), ntrials=2, niters=30, nthreads=1))
    max_branches: int = 1 << 16
    reductions: tuple = REDUCTIONS_ALL
    region_selector: _br.ScoreRS = field(default_factory=_br.ScoreRS)
    brancher: object = field(default_factory=_br.GreedyBrancher)


def eincode2order(code: CompressedEinsum) -> list[int]:
    """Elimination order of a tree: labels in the order nodes drop them,
    nodes in post-order (eincode2order, src/decompose.jl:2-12)."""
    lab = [list(dict.fromkeys(ix)) for ix in code.ixs] + code.labels_of_nodes()
    T = code.n_tensors
    eo = []
    for j, (a, b) in enumerate(code.children):
        uni = list(dict.fromkeys(lab[int(a)] + lab[int(b)]))
        keep = set(lab[T + j])
        eo.extend(x for x in uni if x not in keep)
    if code.n_nodes == 0 and code.ixs:
        eo.extend(code.ixs[0])
    return list(dict.fromkeys(eo))


def update_order(code_old: CompressedEinsum, vmap: list[int]) -> list[int]:
    """The old tree's elimination order mapped onto an induced subgraph
    (update_order, src/decompose.jl:49-56)."""
    inv = {old: new for new, old in enumerate(vmap)}
    return [inv[v] for v in eincode2order(code_old) if v in inv]


def update_code(g_new: Graph, code_old: CompressedEinsum, vmap: list[int]) -> CompressedEinsum:
    """Map the old tree's elimination order onto an induced subgraph and
    rebuild the tree (update_code, src/decompose.jl:96-100)."""
    return _order.order2eincode(g_new, update_order(code_old, vmap))


def _branch_vertex(code: CompressedEinsum, sc_target: float) -> int:
    labs = code.labels_of_nodes()
    score: dict[int, float] = {}
    for ls in labs:
        if len(ls) > sc_target:
            wgt = 2.0 ** (len(ls) - sc_target)
            for x in ls:
                score[x] = score.get(x, 0.0) + wgt
    if not score:
        # fall back to the most frequent label
        for ix in code.ixs:
            for x in ix:
                score[x] = score.get(x, 0.0) + 1.0
    return max(sorted(score), key=lambda x: score[x])


def _make_branch(g: Graph, w: np.ndarray, code: CompressedEinsum, r: float, removed: set[int],
                 slicer: ContractionTreeSlicer) -> SlicedBranch:
    keep = [v for v in range(g.n) if v not in removed]
    sub, vmap = g.induced_subgraph(keep)
    kr = kernelize(sub, w[vmap] if keep else np.zeros(0, np.float32), rules=slicer.reductions)
    vmap2 = [vmap[i] for i in kr.vmap]
    r2 = r + kr.r
    if kr.g.n == 0:
        return SlicedBranch(MISProblem(kr.g, kr.weights), None, r2, vmap=vmap2)
    eo = update_order(code, vmap2)
    new_code = _order.order2eincode(kr.g, eo)
    if slicer.refine and new_code.complexity()[1] > slicer.sc_target:
        ref = slicer.refiner
        new_code = _order.treesa(new_code, _order.TreeSA(sc_target=slicer.sc_target, betas=ref.betas,
                                                         ntrials=ref.ntrials, niters=ref.niters,
                                                         seed=ref.seed, nthreads=ref.nthreads))
        eo = None
    return SlicedBranch(MISProblem(kr.g, kr.weights), new_code, r2, order=eo, vmap=vmap2)


def slice(p: MISProblem, code: CompressedEinsum, r: float, slicer: ContractionTreeSlicer,
          verbose: int = 0) -> list[SlicedBranch]:
    """Branch until every branch has sc <= sc_target (slice / slice_bfs,
    src/slice.jl:4-11,68-90), each step by the slicer's rule (``_branch_once``);
    every child is kernelized and re-ordered."""
    root = SlicedBranch(p, code, r)
    if code is None or code.complexity()[1] <= slicer.sc_target:
        return [root]
    done, todo = [], [root]
    while todo:
        b = todo.pop()
        if b.code is None or b.code.complexity()[1] <= slicer.sc_target:
            done.append(b)
            continue
        if len(done) + len(todo) > slicer.max_branches:
            raise RuntimeError("branching exceeded max_branches")
        todo.extend(_branch_once(b, slicer))
    if verbose:
        scs = [x.sc() for x in done]
        print(f"branches: {len(done)}, max sc: {max(scs) if scs else 0}")
    return done


def _branch_once(b: SlicedBranch, slicer: ContractionTreeSlicer) -> list[SlicedBranch]:
    """The children of one branching step on b under the slicer's rule, with
    ``vmap`` relative to the graph the branching started from."""
    g = b.p.g
    if isinstance(slicer.brancher, VertexBrancher):
        w = b.p.weight_array()
        v = _branch_vertex(b.code, slicer.sc_target)
        nbv = set(g.neighbors(v))
        kids = [_make_branch(g, w, b.code, b.r, {v}, slicer),
                _make_branch(g, w, b.code, b.r + float(w[v]), nbv | {v}, slicer)]
    else:
        kids = _br.branch_step(b, slicer)
    base = b.vmap if b.vmap is not None else list(range(g.n))
    for child in kids:
        child.vmap = [base[x] for x in child.vmap]
    return kids


# ---------------------------------------------------------------------------
# LP bound and the depth-first slicing loop with pruning
# ---------------------------------------------------------------------------
def LP_MWIS(g: Graph, weights) -> float:
    """Upper bound on the weighted MIS: the LP relaxation with one
    constraint x_u + x_v <= 1 per edge and x_a + x_b + x_c <= 1 per triangle,
    0 <= x <= 1 (LP_MWIS, src/utils.jl:274-293), solved with scipy's HiGHS."""
    from scipy.optimize import linprog
    from scipy.sparse import coo_matrix

    n = g.n
    if n == 0:
        return 0.0
    w = weights_array(weights, n).astype(np.float64)
    adj = g.adjacency()
    rows, cols = [], []
    k = 0
    for u, v in g.edges:
        if u == v:
            rows.append(k); cols.append(u)
        else:
            rows += [k, k]; cols += [u, v]
        k += 1
    for u in range(n):
        for v in adj[u]:
            if v <= u:
                continue
            for x in adj[u] & adj[v]:
                if x > v:
                    rows += [k, k, k]; cols += [u, v, x]
                    k += 1
    if k == 0:
        return float(np.sum(np.maximum(w, 0.0)))
    A = coo_matrix((np.ones(len(rows)), (rows, cols)), shape=(k, n)).tocsr()
    res = linprog(-w, A_ub=A, b_ub=np.ones(k), bounds=[(0.0, 1.0)] * n, method="highs")
    if not res.success:
        raise RuntimeError(f"LP_MWIS: {res.message}")
    return float(-res.fun)


def slice_dfs_lp(branch: SlicedBranch, slicer: ContractionTreeSlicer, dirname: str, element_type=np.float32,
                 usecuda: bool = True, engine: Engine | None = None, solve=None, verbose: int = 0) -> dict:
    """Branch until sc <= sc_target, solving each finished slice at once on
    the GPU (plain single-slice path, solve_slice) to raise a primal bound;
    children whose LP bound + r cannot beat the primal bound by 0.99 are
    pruned, the rest are visited best LP bound first, and finished slices are
    written to ``dirname`` in the reference's slice format with their
    solutions (slice_dfs_lp / _slice_single, src/slice.jl:13-66,118-146).
    The loop stops once a solution reaches the LP bound of the root.
    ``solve(branch)`` replaces the GPU solve (the MIS of the branch without
    r).  Returns the primal bound, the LP bound and the slice count."""
    from . import slice_io

    os.makedirs(dirname, exist_ok=True)
    solve = solve or (lambda b: solve_slice(b, element_type, usecuda, engine, mode="plain"))
    rows = []
    lp_bound = LP_MWIS(branch.p.g, branch.p.weight_array()) + branch.r
    primal = 0.0
    unfinished = [branch]
    next_id = 1
    converged = False
    while unfinished:
        b = unfinished.pop()
        sc = b.sc()
        if b.code is None or sc <= slicer.sc_target:
            value = b.r if b.code is None or b.p.g.n == 0 else solve(b) + b.r
            rows.append((next_id, sc, b.tc(), b.r, value))
            if b.code is not None:
                slice_io.save_finished(dirname, b, next_id)
            next_id += 1
            primal = max(primal, float(value))
            if verbose:
                print(f"feasible solution {value}, primal bound {primal}")
            if abs(value - lp_bound) < 1e-6:
                converged = True
                break
            continue
        kids = []
        for c in _branch_once(b, slicer):
            lp = LP_MWIS(c.p.g, c.p.weight_array()) + c.r if c.p.g.n else c.r
            if lp >= primal + 0.99:
                kids.append((lp, c))
        kids.sort(key=lambda t: (-t[0], t[1].p.g.n))
        # children go to the front of the list, which is consumed from its
        # end (the visiting order of src/slice.jl:28-57)
        unfinished[:0] = [c for _, c in kids]
    slice_io.save_slices_csv(dirname, rows)
    return {"primal": primal, "lp_bound": lp_bound, "slices": len(rows), "converged": converged}


# ---------------------------------------------------------------------------
# index slicing (SlicedEinsum): 2^k restrictions of one tree
# ---------------------------------------------------------------------------
def index_slices(code: CompressedEinsum, sc_target: float, open_bits: int = 0, max_slices: int = 40):
    """Choose labels to slice so that every slice has sc <= sc_target.
    Returns (sliced labels per item, open labels, item slice values): the
    first ``open_bits`` chosen labels stay open (2^open_bits slices per item),
    the rest are fixed per item."""
    labels, _ = _order.greedy_slice(code, sc_target, max_slices)
    open_bits = min(open_bits, len(labels))
    opened = labels[:open_bits]
    fixed = labels[open_bits:]
    k = len(fixed)
    vals = ((np.arange(1 << k)[:, None] >> np.arange(k)[None, :]) & 1).astype(np.int8)
    return fixed, opened, vals


# ---------------------------------------------------------------------------
# the contraction calls (GPU)
# ---------------------------------------------------------------------------
_engines: dict[str, Engine] = {}


def _engine_for(element_type) -> Engine:
    dt = np.dtype(element_type)
    key = {np.dtype(np.float32): "f32", np.dtype(np.int32): "i32"}.get(dt)
    if key is None:
        raise ValueError("element_type must be float32 or int32")
    if key not in _engines:
        _engines[key] = Engine(dtype=key)
    return _engines[key]


def _plan_for(engine: Engine, branch: SlicedBranch) -> Plan:
    cache = getattr(branch, "_plans", None)
    if cache is None:
        cache = {}
        branch._plans = cache
    key = id(engine)
    if key not in cache:
        cache[key] = engine.plan(branch.code, branch.p.weight_array(), sliced=branch.sliced)
    return cache[key]


def contract_slices(branches, element_type=np.float32, usecuda: bool = True, engine: Engine | None = None,
                    mode: str = "batched") -> np.ndarray:
    """Contract every branch, one batched GPU call; returns per-branch
    values (contract_slices, src/dynamic_ob.jl:36-48).  A branch carrying
    slice_values contributes one item per row and reports their max."""
    if not usecuda:
        raise ValueError("this engine contracts on the GPU only (usecuda=True)")
    engine = engine or _engine_for(element_type)
    res = np.full(len(branches), -np.inf, np.float32)
    plans, svs, rs, owner = [], [], [], []
    for i, b in enumerate(branches):
        if b.code is None or b.p.g.n == 0:
            res[i] = np.float32(b.r)
            continue
        p = _plan_for(engine, b)
        if b.slice_values is not None and len(b.sliced):
            for row in np.asarray(b.slice_values, np.int8):
                plans.append(p)
                svs.append(row)
                rs.append(b.r)
                owner.append(i)
        else:
            plans.append(p)
            svs.append(np.zeros(0, np.int8))
            rs.append(b.r)
            owner.append(i)
    if plans:
        out, _ = engine.solve_batch(plans, slice_vals=svs, r=np.array(rs, np.float32), mode=mode)
        for v, i in zip(out, owner):
            res[i] = max(res[i], v)
    return res


def solve_slice(branch: SlicedBranch, element_type=np.float32, usecuda: bool = True,
                engine: Engine | None = None, mode: str = "plain") -> float:
    """MIS value of one branch without r (solve_slice, src/dynamic_ob.jl:30-34)."""
    v = contract_slices([branch], element_type, usecuda, engine, mode)[0]
    return float(v - np.float32(branch.r))


def dynamic_ob_mis(g: Graph, weights=None, slicer: ContractionTreeSlicer | None = None, optimizer=None,
                   usecuda: bool = True, element_type=np.float32, verbose: int = 0, engine: Engine | None = None,
                   mode: str = "batched") -> float:
    """Maximum (weighted) independent set size: kernelize, order, branch
    until sc <= sc_target, contract every branch on the GPU, take the max
    (dynamic_ob_mis, src/dynamic_ob.jl:6-28)."""
    slicer = slicer or ContractionTreeSlicer()
    w = weights_array(weights, g.n)
    kr = kernelize(g, w, verbose)
    if verbose:
        print(f"kernelized graph: {{{kr.g.n}, {kr.g.ne()}}}")
    if kr.g.n == 0:
        return float(kr.r)
    code = _order.initialize_code(kr.g, optimizer or _order.TreeSA(sc_target=slicer.sc_target))
    branches = slice(MISProblem(kr.g, kr.weights), code, kr.r, slicer, verbose)
    res = contract_slices(branches, element_type, usecuda, engine, mode)
    return float(np.max(res))
