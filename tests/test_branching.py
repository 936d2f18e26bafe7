"""The reference's optimal branching rule (src/branch.jl, with the
OptimalBranching table / clause / set-cover machinery restated) on the CPU:
tables and clauses against brute-force restatements, the branching factor,
and the relation test/dynamic_ob.jl:10-26 checks for every brancher and
region loss: the max over branches of MIS(branch) + r is the MIS of the
graph (branch values by the oracle)."""
import itertools

import numpy as np
import pytest

from cases import rr_case


@pytest.fixture(scope="module")
def br(tb):
    import sys

    return sys.modules["tensorbranching_gb300.branching"]


def _brute_table(adj, w, region):
    """Rows by enumeration of all 2^k region configurations."""
    k = len(region)
    inside = set(region)
    bnd = [i for i, v in enumerate(region) if adj[v] - inside]
    alpha, best = {}, {}
    for c in range(1 << k):
        sel = [region[i] for i in range(k) if c >> i & 1]
        if any(u in adj[v] for v in sel for u in sel):
            continue
        s = tuple(c >> i & 1 for i in bnd)
        wt = sum(float(w[v]) for v in sel)
        if s not in alpha or wt > alpha[s]:
            alpha[s], best[s] = wt, [c]
        elif wt == alpha[s]:
            best[s].append(c)
    rows = []
    for s, a in alpha.items():
        dominated = any(t != s and all(x <= y for x, y in zip(t, s)) and alpha[t] >= a for t in alpha)
        if not dominated:
            rows.append(sorted(best[s]))
    return sorted(rows)


@pytest.mark.parametrize("seed", range(6))
def test_table_matches_enumeration(tb, br, seed):
    g = tb.random_regular_graph(24, 3, seed) if seed % 2 else tb.random_ksg(6, 0.8, seed)
    w = tb.random_weights(g.n, seed) if seed % 3 else np.ones(g.n, np.float32)
    adj = g.adjacency()
    for v in (0, g.n // 2):
        region = br.select_region(adj, v, 10 + seed)
        assert len(region) <= 10 + seed and region[0] == v
        got = sorted(r.tolist() for r in br.branching_table(adj, w, region).rows)
        assert got == _brute_table(adj, w, region)


def test_single_vertex_region_is_the_vertex_rule(tb, br):
    g = tb.random_regular_graph(12, 3, 0)
    adj = g.adjacency()
    tbl = br.branching_table(adj, np.ones(g.n), [0])
    assert [r.tolist() for r in tbl.rows] == [[0], [1]]
    assert br.intersect_clauses(tbl) == []
    subsets, rvs, res = br.generate_subsets(adj, np.ones(g.n), tbl, [0])
    got = sorted(zip(map(tuple, rvs), map(tuple, subsets), res))
    assert got == sorted([((0,), (0,), 0.0), (tuple(sorted({0} | adj[0])), (1,), 1.0)])


def test_candidate_clauses_are_the_agreement_closure(tb, br):
    g = tb.random_regular_graph(20, 3, 3)
    adj = g.adjacency()
    region = br.select_region(adj, 5, 10)
    tbl = br.branching_table(adj, np.ones(g.n), region)
    full = (1 << tbl.bit_length) - 1
    base = {int(c) for r in tbl.rows for c in r}
    want = {(full, c) for c in base}
    todo = list(want)
    while todo:  # plain closure
        m, v = todo.pop()
        for c in base:
            nm = m & ~(v ^ c)
            if nm and (nm, v & nm) not in want:
                want.add((nm, v & nm))
                todo.append((nm, v & nm))
    got = {(c.mask, c.val) for c in br.candidate_clauses(tbl)}
    assert got == want
    for m, v in got:  # every candidate holds some configuration
        assert any((c & m) == v for c in base)


def test_intersect_clauses_finds_a_reduction(br):
    tbl = br.BranchingTable(4, [np.array([0b0101, 0b0110]), np.array([0b1001]), np.array([0b0001, 0b1000])])
    red = br.intersect_clauses(tbl)
    assert len(red) == 1
    c = red[0]
    assert c.mask & 1 and c.val & 1  # bit 0 set in one configuration of every row
    assert br.covered_items(tbl, c) == [0, 1, 2]
    tbl2 = br.BranchingTable(2, [np.array([0b01]), np.array([0b10])])
    assert br.intersect_clauses(tbl2) == []


def test_removed_vertices_and_clause_size(tb, br):
    g = tb.Graph(5, [(0, 1), (1, 2), (2, 3), (3, 4)])
    adj = g.adjacency()
    region = [1, 2, 3]
    c = br.Clause(mask=0b101, val=0b001)  # vertex 1 in, vertex 3 out
    assert br.removed_vertices(region, adj, c) == [0, 1, 2, 3]
    w = np.array([1, 2, 3, 4, 5], np.float32)
    assert br.clause_size(w, c.val & c.mask, region) == 2.0


def test_set_cover_and_branching_factor(br):
    subsets = [[0, 1], [1, 2], [2, 3], [0, 3], [0, 1, 2, 3]]
    assert br.weighted_minimum_set_cover([1, 1, 1, 1, 3], subsets, 4) in ([0, 2], [1, 3])
    assert br.weighted_minimum_set_cover([1, 1, 1, 1, 1.5], subsets, 4) == [4]
    with pytest.raises(ValueError):
        br.weighted_minimum_set_cover([1.0], [[0]], 2)
    assert br.complexity_bv([1, 1]) == pytest.approx(2.0)
    assert br.complexity_bv([1, 2]) == pytest.approx((1 + 5 ** 0.5) / 2)
    assert br.complexity_bv([3]) == 1.0
    assert br.complexity_bv([0, 2]) == float("inf")
    # fixed point: d = (1, 1, 2, 2, 2): two branches of d=2 covering all
    picked = br.fixed_point_set_cover(br.IPSolver(), [1, 1, 2, 2, 2], [[0], [1], [0, 1], [0], [1]], 2)
    assert picked == [2]


def test_scores(tb, br):
    g, w, code = rr_case(tb, 40, 1)
    large = br.list_subtree(code, 5)
    assert large and all(len(x) >= 5 for x in large)
    rvs = [[], list(range(g.n))]
    s = br.sc_score(5, code, rvs)
    want = 1.0 + sum(2.0 ** max(0, len(x) - 5) - 1.0 for x in large)
    assert s[0] == pytest.approx(want) and s[1] == 1.0
    m = br.sc_measure(5, code, rvs)
    assert m[0] == 0 and m[1] == sum(len(x) for x in large)
    seps = br.tree_separators(code)
    assert seps and br.bag_score(5, code, [list(range(g.n))])[0] == 1.0


@pytest.mark.parametrize("brancher", ["greedy", "fixed_point"])
@pytest.mark.parametrize("loss", ["num_uniques", "sc_score", "bag_score"])
@pytest.mark.parametrize("weighted", [False, True])
def test_optimal_branching_keeps_the_mis(tb, br, orc, exact, brancher, loss, weighted):
    """test/dynamic_ob.jl:10-26 in small: every brancher and region loss."""
    seed = 7 if weighted else 2
    g = tb.random_regular_graph(50, 3, seed)
    w = tb.random_weights(g.n, seed) if weighted else np.ones(g.n, np.float32)
    kr = tb.kernelize(g, w)
    code = tb.initialize_code(kr.g, tb.GreedyMethod(seed))
    b = br.GreedyBrancher() if brancher == "greedy" else br.FixedPointBrancher()
    # regions of at most 12 vertices keep the CPU run short (the default is 20)
    slicer = tb.ContractionTreeSlicer(sc_target=5, refine=False, brancher=b,
                                      region_selector=br.ScoreRS(n_max=12, loss=loss))
    branches = tb.slice(tb.MISProblem(kr.g, kr.weights), code, kr.r, slicer)
    vals = []
    for x in branches:
        if x.code is None or x.p.g.n == 0:
            vals.append(x.r)
            continue
        assert x.code.complexity()[1] <= 5
        # vmap maps the branch's vertices back into the kernel
        assert len(x.vmap) == x.p.g.n and len(set(x.vmap)) == x.p.g.n
        vals.append(orc.solve(x.code, x.p.weight_array()) + x.r)
    assert max(vals) == pytest.approx(exact.branch_and_bound(g.n, g.edges, w))


def test_each_step_is_exact(tb, br, exact):
    """One step from several branch states: max over children of
    MIS(child) + r == MIS(parent) + r."""
    for seed in range(3):
        g = tb.random_ksg(7, 0.8, seed)
        w = tb.random_weights(g.n, seed)
        code = tb.initialize_code(g, tb.GreedyMethod(seed))
        b = tb.SlicedBranch(tb.MISProblem(g, w), code, 0.0)
        slicer = tb.ContractionTreeSlicer(sc_target=3, refine=False)
        kids = br.branch_step(b, slicer)
        assert kids
        got = max(k.r + (exact.branch_and_bound(k.p.g.n, k.p.g.edges, k.p.weight_array()) if k.p.g.n else 0.0)
                  for k in kids)
        assert got == pytest.approx(exact.branch_and_bound(g.n, g.edges, w))


def test_self_loops_are_never_selected(tb, br):
    g = tb.Graph(4, [(0, 0), (0, 1), (1, 2), (2, 3)])
    tbl = br.branching_table(g.adjacency(), np.ones(4), [0, 1, 2, 3], blocked={0})
    assert all(int(c) & 1 == 0 for r in tbl.rows for c in r)
