"""The reference's optimal branching rule for ``ContractionTreeSlicer``.

One branching step on a branch whose contraction tree is too large:

  list_subtree          src/utils.jl:27-36     nodes whose output has >= sc_target labels
  ob_region             src/branch.jl:4-39     grow one region per large-tensor label, keep the best
  optimal_branches      src/branch.jl:73-110   branching table -> reduction or set cover
  generate_subsets      src/branch.jl:44-71    candidate clauses grouped by removed vertices
  slicer_loss           src/branch.jl:112-128
  sc_score              src/branch.jl:131-147  1 + sum over large tensors of 2^t - 1
  bag_score             src/branch.jl:150-174  the same over separators of the tree decomposition
  sc_measure            src/branch.jl:177-191  removed labels counted over large tensors
  set_cover             src/branch.jl:193-199  weighted minimum set cover (GreedyBrancher)
  fixed_point_set_cover src/branch.jl:201-211  FixedPointBrancher
  generate_branch       src/branch.jl:212-231  remove, kernelize, map the order, refine
  ScoreRS, GreedyBrancher, FixedPointBrancher  src/types.jl:9-25

The branching-table machinery the reference imports from OptimalBranching 0.2
(OptimalBranchingCore / OptimalBranchingMIS, pinned in Project.toml and not
vendored) is restated from the published method (Gao, Ye, Liu, Wang, Zhang,
"Automated discovery of branching rules with optimal complexity for the
maximum independent set problem", 2024):

* ``select_region`` grows a region around one vertex by whole neighbour
  shells while it stays within ``n_max`` vertices;
* ``branching_table``: for every configuration sigma of the region's boundary
  (its vertices with neighbours outside), alpha(sigma) is the best weight of
  an independent set of the region with that boundary; sigma is dropped when
  a strict subset sigma' of it has alpha(sigma') >= alpha(sigma) (sigma' leaves
  the outside less constrained at no loss).  Each kept sigma is one row: the
  region configurations that reach alpha(sigma).  Some optimal independent
  set of the whole graph agrees on the region with a configuration of some
  row, so any set of clauses covering every row is an exact branching;
* a clause fixes some region vertices (``mask``) to values (``val``);
  ``candidate_clauses`` are the clauses on which a set of table
  configurations agree (closure of pairwise agreement), ``covered_items``
  the rows holding a configuration that satisfies a clause;
* ``intersect_clauses`` looks for one clause satisfied by a configuration of
  every row: that single branch is a reduction;
* ``removed_vertices``: a vertex fixed to 0 leaves the graph, one fixed to 1
  leaves with its neighbours; ``clause_size`` is the weight of the vertices
  fixed to 1;
* ``weighted_minimum_set_cover`` is the integer program min sum w_i x_i over
  candidates subject to every row being covered (solved with HiGHS through
  scipy, as the reference's IPSolver uses an IP solver);
  ``complexity_bv`` solves sum_i gamma^(-d_i) = 1 for the branching factor.

Every branch set produced here is exact: the max over branches of the
branch's MIS plus its ``r`` equals the MIS of the branched graph.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .graphs import Graph
from .network import CompressedEinsum, SlicedBranch


# ---------------------------------------------------------------------------
# options (src/types.jl:9-25)
# ---------------------------------------------------------------------------
@dataclass
class ScoreRS:
    """Region selector: regions of at most ``n_max`` vertices grown by
    ``strategy`` around every label of a large tensor, ranked by ``loss``
    ("sc_score", "bag_score" or "num_uniques") (ScoreRS, src/types.jl:9-13)."""

    n_max: int = 20
    strategy: str = "neighbor"
    loss: str = "sc_score"


@dataclass
class IPSolver:
    """Set-cover solver: an integer program (HiGHS).  ``gamma0`` and
    ``max_itr`` drive the fixed-point iteration of FixedPointBrancher."""

    max_itr: int = 20
    gamma0: float = 2.0
    max_candidates: int = 1 << 14


@dataclass
class GreedyBrancher:
    """Pick the cheapest clause set covering the table, a clause costing its
    ``loss`` (GreedyBrancher, src/types.jl:17-20)."""

    loss: str = "sc_score"
    setcover_solver: IPSolver = field(default_factory=IPSolver)


@dataclass
class FixedPointBrancher:
    """Pick the clause set of least branching factor gamma, with each clause's
    progress measured by ``measure`` (FixedPointBrancher, src/types.jl:22-25)."""

    measure: str = "sc_measure"
    setcover_solver: IPSolver = field(default_factory=IPSolver)


@dataclass(frozen=True)
class Clause:
    """Region vertices i with bit i of ``mask`` set are fixed to bit i of ``val``."""

    mask: int
    val: int


@dataclass
class BranchingTable:
    """``rows[j]``: int64 array of region configurations (bit i = region
    vertex i in the set) that are optimal for the j-th kept boundary
    configuration."""

    bit_length: int
    rows: list


# ---------------------------------------------------------------------------
# large tensors, regions and their scores
# ---------------------------------------------------------------------------
def list_subtree(code: CompressedEinsum, threshold: float) -> list[list[int]]:
    """Output labels of the tree's nodes holding at least 2^threshold entries,
    in post-order (list_subtree, src/utils.jl:27-36)."""
    return [ls for ls in code.labels_of_nodes() if len(ls) >= threshold]


def select_region(adj: list[set[int]], v: int, n_max: int, strategy: str = "neighbor") -> list[int]:
    """Region around vertex ``v``: add the open neighbourhood of the region
    shell by shell while the region stays within ``n_max`` vertices."""
    if strategy != "neighbor":
        raise ValueError(f"region strategy {strategy!r} is not implemented")
    region, inside = [v], {v}
    while len(region) < n_max:
        shell = sorted({u for x in region for u in adj[x]} - inside)
        if not shell or len(region) + len(shell) > n_max:
            break
        region += shell
        inside.update(shell)
    return region


def _as_bits(rvs) -> tuple[list[int], np.ndarray]:
    """Vertex sets as (labels, bool matrix [set, label])."""
    if isinstance(rvs, tuple) and len(rvs) == 2 and isinstance(rvs[1], np.ndarray):
        return rvs
    ext = sorted({int(x) for rv in rvs for x in rv})
    pos = {v: i for i, v in enumerate(ext)}
    bits = np.zeros((len(rvs), len(ext)), bool)
    for i, rv in enumerate(rvs):
        bits[i, [pos[int(x)] for x in rv]] = True
    return ext, bits


def _removed_counts(sets: list, rvs) -> np.ndarray:
    """counts[i, j] = |rvs[i] & sets[j]|; ``rvs`` a list of vertex sets or
    (labels, bool matrix)."""
    ext, bits = _as_bits(rvs)
    mem = np.array([[v in st for v in ext] for st in sets], np.int32).reshape(len(sets), len(ext))
    return bits.astype(np.int32) @ mem.T


def _pow_score(sets: list, rvs, sc_target: float) -> np.ndarray:
    n = _as_bits(rvs)[1].shape[0]
    if not sets:
        return np.ones(n)
    sizes = np.array([len(st) for st in sets], np.float64)
    t = np.maximum(0.0, sizes[None, :] - _removed_counts(sets, rvs) - sc_target)
    return 1.0 + (np.exp2(t) - 1.0).sum(axis=1)


def sc_score(sc_target: float, code: CompressedEinsum, rvs) -> np.ndarray:
    """1 + sum over the large tensors of 2^max(0, |iy| - |rv & iy| - sc_target) - 1
    for each vertex set ``rv`` (sc_score, src/branch.jl:131-147)."""
    return _pow_score([set(x) for x in list_subtree(code, sc_target)], rvs, sc_target)


def tree_separators(code: CompressedEinsum) -> list[set[int]]:
    """Separators of the tree decomposition given by the tree's elimination
    order on the labels' interaction graph (labels adjacent when they share
    a tensor): eliminating v makes its remaining neighbours a clique, the bag
    of v is v with them, and the bag of v meets its parent bag (that of its
    first-eliminated neighbour) in exactly those neighbours
    (decompose, src/decompose.jl:30-34, as bag_score uses it)."""
    from .mis import eincode2order

    adj: dict[int, set[int]] = {}
    for ix in list(code.ixs) + [list(code.iy)]:
        for a in ix:
            adj.setdefault(a, set())
            for b in ix:
                if a != b:
                    adj[a].add(b)
    eo = eincode2order(code)
    eo += [x for x in sorted(adj) if x not in set(eo)]
    seps = []
    for v in eo:
        nb = adj.pop(v, set())
        for a in nb:
            adj[a].discard(v)
            adj[a].update(nb - {a})
        if nb:
            seps.append(set(nb))
    return seps


def bag_score(sc_target: float, code: CompressedEinsum, rvs) -> np.ndarray:
    """sc_score over the separators of the tree decomposition instead of the
    large tensors (bag_score, src/branch.jl:150-174)."""
    return _pow_score(tree_separators(code), rvs, sc_target)


def sc_measure(sc_target: float, code: CompressedEinsum, rvs) -> np.ndarray:
    """Labels of the large tensors each vertex set removes, summed over the
    tensors (sc_measure, src/branch.jl:177-191)."""
    sets = [set(x) for x in list_subtree(code, sc_target)]
    if not sets:
        return np.zeros(_as_bits(rvs)[1].shape[0])
    return _removed_counts(sets, rvs).sum(axis=1).astype(np.float64)


def ob_region(g: Graph, code: CompressedEinsum, sc_target: float, selector: ScoreRS,
              adj: list[set[int]] | None = None) -> tuple[list[int], float]:
    """One region per label of the large tensors (labels in post-order of
    their nodes, first occurrence), the best by the selector's loss
    (ob_region, src/branch.jl:4-39).  With "num_uniques" the reference
    intersects each region with its own seed label, so every region scores 1
    and the first one is kept; that is reproduced."""
    adj = g.adjacency() if adj is None else adj
    seeds = list(dict.fromkeys(x for ls in list_subtree(code, sc_target) for x in ls))
    regions = [select_region(adj, v, selector.n_max, selector.strategy) for v in seeds]
    if selector.loss == "sc_score":
        losses = sc_score(sc_target, code, regions)
        i = int(np.argmin(losses))
    elif selector.loss == "bag_score":
        losses = bag_score(sc_target, code, regions)
        i = int(np.argmin(losses))
    elif selector.loss == "num_uniques":
        losses = np.array([float(v in r) for v, r in zip(seeds, regions)])
        i = int(np.argmax(losses))
    else:
        raise ValueError(f"region loss {selector.loss!r} is not implemented")
    return regions[i], float(losses[i])


# ---------------------------------------------------------------------------
# branching table and clauses
# ---------------------------------------------------------------------------
def branching_table(adj: list[set[int]], weights: np.ndarray, region: list[int], blocked=()) -> BranchingTable:
    """The reduced table of the region (see the module docstring).
    ``blocked`` vertices (self-loops) are never in the set."""
    k = len(region)
    pos = {v: i for i, v in enumerate(region)}
    lower = [0] * k  # region neighbours with a smaller bit index
    bnd = []
    for i, v in enumerate(region):
        for u in adj[v]:
            j = pos.get(u)
            if j is None:
                if not bnd or bnd[-1] != i:
                    bnd.append(i)
            elif j < i:
                lower[i] |= 1 << j
    # independent sets of the region, grown one vertex at a time
    cfg = np.zeros(1, np.int64)
    wt = np.zeros(1, np.float64)
    for i, v in enumerate(region):
        if v in blocked:
            continue
        ok = (cfg & lower[i]) == 0
        cfg = np.concatenate([cfg, cfg[ok] | (1 << i)])
        wt = np.concatenate([wt, wt[ok] + float(weights[v])])
    nb = len(bnd)
    sig = np.zeros(cfg.shape, np.int64)
    for j, i in enumerate(bnd):
        sig |= ((cfg >> i) & 1) << j
    alpha = np.full(1 << nb, -np.inf)
    np.maximum.at(alpha, sig, wt)
    # best over subsets (inclusive), then over strict subsets
    sub = alpha.copy()
    idx = np.arange(1 << nb)
    for j in range(nb):
        has = (idx >> j) & 1 == 1
        sub[has] = np.maximum(sub[has], sub[idx[has] ^ (1 << j)])
    strict = np.full(1 << nb, -np.inf)
    for j in range(nb):
        has = (idx >> j) & 1 == 1
        strict[has] = np.maximum(strict[has], sub[idx[has] ^ (1 << j)])
    keep = np.flatnonzero((alpha > -np.inf) & ~(strict >= alpha))
    best = alpha[sig]
    opt = wt == best
    rows = []
    for s in keep:
        rows.append(np.sort(cfg[opt & (sig == s)]))
    return BranchingTable(k, rows)


def _flat(tbl: BranchingTable) -> tuple[np.ndarray, np.ndarray]:
    cfgs = np.concatenate(tbl.rows) if tbl.rows else np.zeros(0, np.int64)
    row_of = np.concatenate([np.full(len(r), j, np.int64) for j, r in enumerate(tbl.rows)]) \
        if tbl.rows else np.zeros(0, np.int64)
    return cfgs, row_of


def covered_items(tbl: BranchingTable, clause: Clause, flat=None) -> list[int]:
    """Rows with a configuration that satisfies ``clause``."""
    cfgs, row_of = flat if flat is not None else _flat(tbl)
    return np.unique(row_of[(cfgs & clause.mask) == clause.val]).tolist()


def _candidate_arrays(tbl: BranchingTable, limit: int) -> tuple[np.ndarray, np.ndarray]:
    """(masks, vals) of the candidate clauses, level by level: level 0 is the
    table's configurations, level j+1 the new clauses that agree with a
    configuration on part of a level-j clause."""
    k = tbl.bit_length
    if k > 31:
        raise ValueError("regions of more than 31 vertices are not supported")
    full = np.int64((1 << k) - 1)
    base = np.unique(np.concatenate(tbl.rows)) if tbl.rows else np.zeros(0, np.int64)
    keys = (full << k) | base
    levels = [keys]
    known = keys
    frontier = keys
    total = keys.size
    step = max(1, (1 << 20) // max(base.size, 1))
    while frontier.size and total < limit:
        parts = []
        for a in range(0, frontier.size, step):
            ch = frontier[a:a + step]
            fm, fv = ch >> k, ch & full
            m = fm[:, None] & ~(fv[:, None] ^ base[None, :]) & full
            nk = (m << k) | (fv[:, None] & m)
            parts.append(np.unique(nk[m != 0]))
        cand = np.unique(np.concatenate(parts))
        cand = cand[~np.isin(cand, known, assume_unique=True)]
        cand = cand[:max(0, limit - total)]
        if not cand.size:
            break
        levels.append(cand)
        known = np.union1d(known, cand)
        total += cand.size
        frontier = cand
    keys = np.concatenate(levels)
    return keys >> k, keys & full


def candidate_clauses(tbl: BranchingTable, limit: int = 1 << 14) -> list[Clause]:
    """The table's configurations as full clauses, closed under agreement
    (c1, c2 -> the bits where both are fixed to the same value).  Stops
    adding at ``limit`` clauses; any subset of the closure that holds every
    configuration still gives an exact branching."""
    masks, vals = _candidate_arrays(tbl, limit)
    return [Clause(int(m), int(v)) for m, v in zip(masks, vals)]


def intersect_clauses(tbl: BranchingTable, max_nodes: int = 1 << 16) -> list[Clause]:
    """A clause satisfied by some configuration of every row, found by a
    depth-first choice of one configuration per row; empty if none (within
    ``max_nodes`` search steps)."""
    if not tbl.rows:
        return []
    rows = sorted(tbl.rows, key=len)
    full = (1 << tbl.bit_length) - 1
    budget = [max_nodes]

    def dfs(j: int, mask: int, val: int):
        if j == len(rows):
            return Clause(mask, val & mask)
        for c in rows[j]:
            budget[0] -= 1
            if budget[0] < 0:
                return None
            m = mask & ~(val ^ int(c))
            if m:
                got = dfs(j + 1, m, val)
                if got is not None:
                    return got
        return None

    got = None
    for c in rows[0]:
        got = dfs(1, full, int(c))
        if got is not None or budget[0] < 0:
            break
    return [got] if got is not None else []


def removed_vertices(region: list[int], adj: list[set[int]], clause: Clause) -> list[int]:
    """Vertices a clause removes: every fixed vertex, and the neighbours of
    those fixed to 1."""
    rv = set()
    for i, v in enumerate(region):
        if clause.mask >> i & 1:
            rv.add(v)
            if clause.val >> i & 1:
                rv.update(adj[v])
    return sorted(rv)


def clause_size(weights: np.ndarray, bits: int, region: list[int]) -> float:
    """Weight of the region vertices whose bit is set."""
    return float(sum(float(weights[v]) for i, v in enumerate(region) if bits >> i & 1))


def _subset_arrays(adj: list[set[int]], weights: np.ndarray, tbl: BranchingTable, region: list[int],
                   limit: int):
    """Grouped candidates as arrays: (cover [group, row] bool, removed
    vertices as (labels, [group, label] bool), largest fixed weight [group])."""
    masks, vals = _candidate_arrays(tbl, limit)
    k = tbl.bit_length
    # coverage: clause c covers row j when a configuration of row j satisfies it
    cfgs, row_of = _flat(tbl)
    starts = np.flatnonzero(np.r_[True, row_of[1:] != row_of[:-1]]) if row_of.size else np.zeros(0, np.int64)
    sat = (cfgs[None, :] & masks[:, None]) == vals[:, None]
    cov = np.logical_or.reduceat(sat, starts, axis=1) if starts.size else np.zeros((masks.size, 0), bool)
    # removed vertices over the region and its neighbours, packed 63 to a word
    ext = list(region) + sorted({u for v in region for u in adj[v]} - set(region))
    epos = {v: i for i, v in enumerate(ext)}
    words = (len(ext) + 62) // 63
    self_bits = np.zeros((k, words), np.int64)
    nb_bits = np.zeros((k, words), np.int64)
    for i, v in enumerate(region):
        self_bits[i, i // 63] |= np.int64(1) << (i % 63)
        for u in adj[v]:
            j = epos[u]
            nb_bits[i, j // 63] |= np.int64(1) << (j % 63)
    rk = np.zeros((masks.size, words), np.int64)
    size = np.zeros(masks.size, np.float64)
    wr = np.array([float(weights[v]) for v in region], np.float64)
    for i in range(k):
        fixed = ((masks >> i) & 1).astype(bool)
        one = fixed & ((vals >> i) & 1).astype(bool)
        rk[fixed] |= self_bits[i]
        rk[one] |= nb_bits[i]
        size[one] += wr[i]
    # group equal removed sets (lexicographic sort of the packed words)
    order = np.lexsort(rk.T[::-1]) if words else np.arange(masks.size)
    rs = rk[order]
    new = np.r_[True, np.any(rs[1:] != rs[:-1], axis=1)] if masks.size else np.zeros(0, bool)
    gstart = np.flatnonzero(new)
    gcov = np.logical_or.reduceat(cov[order], gstart, axis=0)
    gsize = np.maximum.reduceat(size[order], gstart)
    keys = rs[gstart]
    e = np.arange(len(ext))
    bits = ((keys[:, e // 63] >> (e % 63)) & 1).astype(bool)
    return gcov, (ext, bits), gsize


def generate_subsets(adj: list[set[int]], weights: np.ndarray, tbl: BranchingTable, region: list[int],
                     limit: int = 1 << 14):
    """Candidate clauses grouped by the vertices they remove: for each
    distinct removed set, the rows its clauses cover and the largest weight
    they fix to 1 (generate_subsets, src/branch.jl:44-71).  Returns
    (subsets, rvs, residuals) with subsets[i] the sorted covered rows."""
    gcov, (ext, bits), gsize = _subset_arrays(adj, weights, tbl, region, limit)
    subsets = [np.flatnonzero(c).tolist() for c in gcov]
    rvs = [sorted(ext[j] for j in np.flatnonzero(r)) for r in bits]
    return subsets, rvs, [float(x) for x in gsize]


# ---------------------------------------------------------------------------
# set cover
# ---------------------------------------------------------------------------
def _cover_solve(weights, cover: np.ndarray) -> list[int]:
    """min sum w_i x_i, x binary, every column of ``cover`` [subset, item]
    (or row of its sparse transpose) hit at least once (HiGHS through scipy)."""
    from scipy.optimize import Bounds, LinearConstraint, milp
    from scipy.sparse import csr_matrix

    if isinstance(cover, np.ndarray):
        if cover.shape[1] and not np.all(cover.any(axis=0)):
            raise ValueError("set cover: an item is covered by no subset")
        cover = csr_matrix(cover.T.astype(np.float64))
    a = cover  # [item, subset]
    n_items, n = a.shape
    res = milp(c=np.asarray(weights, np.float64), integrality=np.ones(n), bounds=Bounds(0, 1),
               constraints=LinearConstraint(a, lb=np.ones(n_items), ub=np.full(n_items, np.inf)))
    if res.x is None:
        raise RuntimeError(f"set cover: {res.message}")
    return [int(i) for i in np.flatnonzero(res.x > 0.5)]


def _cover_matrix(subsets: list, n_items: int) -> np.ndarray:
    cover = np.zeros((len(subsets), n_items), bool)
    for i, st in enumerate(subsets):
        cover[i, list(st)] = True
    return cover


def weighted_minimum_set_cover(weights, subsets, n_items: int) -> list[int]:
    """Indices of the subsets of least total weight covering 0..n_items-1
    (an integer program).  ``subsets`` is a list of item lists or a bool
    matrix [subset, item]."""
    cover = subsets if isinstance(subsets, np.ndarray) else _cover_matrix(subsets, n_items)
    return _cover_solve(weights, cover)


def complexity_bv(deltas) -> float:
    """Branching factor gamma >= 1 with sum_i gamma^(-d_i) = 1 (inf when a
    branch makes no progress and there is more than one branch)."""
    d = np.asarray(deltas, np.float64)
    if d.size <= 1:
        return 1.0
    if np.any(d <= 0):
        return float("inf")

    def f(x):  # x = log gamma
        return float(np.exp(-d * x).sum()) - 1.0

    lo, hi = 0.0, 1.0
    while f(hi) > 0:
        hi *= 2.0
    for _ in range(100):
        mid = 0.5 * (lo + hi)
        if f(mid) > 0:
            lo = mid
        else:
            hi = mid
    return float(np.exp(0.5 * (lo + hi)))


def fixed_point_set_cover(solver: IPSolver, deltas, subsets, n_items: int) -> list[int]:
    """Iterate: cover with weights gamma^(-d_i), then gamma := branching
    factor of the pick, until gamma settles (fixed_point_set_cover,
    src/branch.jl:201-211).  The weights are scaled by gamma^min(d), which
    leaves the minimiser unchanged and keeps them away from underflow."""
    d = np.asarray(deltas, np.float64)
    from scipy.sparse import csr_matrix

    cover = subsets if isinstance(subsets, np.ndarray) else _cover_matrix(subsets, n_items)
    if cover.shape[1] and not np.all(cover.any(axis=0)):
        raise ValueError("set cover: an item is covered by no subset")
    cover = csr_matrix(cover.T.astype(np.float64))
    gamma = solver.gamma0
    picked = None
    for _ in range(solver.max_itr):
        picked = _cover_solve(gamma ** (-(d - d.min())), cover)
        nxt = complexity_bv(d[picked])
        if not np.isfinite(nxt) or abs(nxt - gamma) <= 1e-9 * max(1.0, gamma):
            break
        gamma = nxt
    return picked


# ---------------------------------------------------------------------------
# one branching step
# ---------------------------------------------------------------------------
def optimal_branches(b: SlicedBranch, slicer, region: list[int], adj: list[set[int]] | None = None,
                     make_branch=None) -> list[SlicedBranch]:
    """Branches of ``b`` on ``region``: a single branch when one clause
    covers the whole table, otherwise the set cover of the candidates under
    the brancher's loss (optimal_branches, src/branch.jl:73-110).  Each
    branch removes its vertices, adds the weight it fixes to 1 to ``r`` and
    is kernelized and re-ordered (generate_branch, src/branch.jl:212-231).
    ``vmap`` of the result is relative to ``b``'s graph."""
    from .mis import _make_branch

    make_branch = make_branch or _make_branch
    g, w, code = b.p.g, b.p.weight_array(), b.code
    adj = g.adjacency() if adj is None else adj
    tbl = branching_table(adj, w, region, {u for u, v in g.edges if u == v})
    red = intersect_clauses(tbl)
    if red:
        c = red[0]
        rv = removed_vertices(region, adj, c)
        return [make_branch(g, w, code, b.r + clause_size(w, c.val & c.mask, region), set(rv), slicer)]
    brancher = slicer.brancher
    solver = brancher.setcover_solver
    cover, rvb, residuals = _subset_arrays(adj, w, tbl, region, solver.max_candidates)
    if isinstance(brancher, GreedyBrancher):
        if brancher.loss == "sc_score":
            losses = sc_score(slicer.sc_target, code, rvb)
        elif brancher.loss == "bag_score":
            losses = bag_score(slicer.sc_target, code, rvb)
        else:
            raise ValueError(f"brancher loss {brancher.loss!r} is not implemented")
        picked = _cover_solve(losses, cover)
    elif isinstance(brancher, FixedPointBrancher):
        if brancher.measure != "sc_measure":
            raise ValueError(f"brancher measure {brancher.measure!r} is not implemented")
        picked = fixed_point_set_cover(solver, sc_measure(slicer.sc_target, code, rvb), cover, len(tbl.rows))
    else:
        raise TypeError(f"unknown brancher {type(brancher).__name__}")
    ext, bits = rvb
    return [make_branch(g, w, code, b.r + float(residuals[i]), {ext[j] for j in np.flatnonzero(bits[i])}, slicer)
            for i in picked]


def branch_step(b: SlicedBranch, slicer) -> list[SlicedBranch]:
    """ob_region + optimal_branches on one branch (_slice_bfs body,
    src/slice.jl:100-107); ``vmap`` of the results is relative to ``b``'s
    graph."""
    adj = b.p.g.adjacency()
    region, _ = ob_region(b.p.g, b.code, slicer.sc_target, slicer.region_selector, adj)
    return optimal_branches(b, slicer, region, adj)
