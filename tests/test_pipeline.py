"""The host pipeline around the contraction (CPU; contractions by the
oracle): kernelization is exact (MIS(kernel) + r == MIS(g), as
test/kernelize.jl:11-25), and branching to sc <= sc_target keeps the MIS
(max over branches of MIS(branch) + r == MIS(g), as test/slice.jl:22-35)."""
import numpy as np
import pytest

from cases import rr_case


@pytest.mark.parametrize("seed", range(4))
@pytest.mark.parametrize("weighted", [False, True])
def test_kernelize_is_exact(tb, exact, seed, weighted):
    g = tb.random_regular_graph(30 + 6 * seed, 3, seed)
    w = tb.random_weights(g.n, seed) if weighted else np.ones(g.n, np.float32)
    kr = tb.kernelize(g, w)
    full = exact.branch_and_bound(g.n, g.edges, w)
    kern = exact.branch_and_bound(kr.g.n, kr.g.edges, kr.weights) if kr.g.n else 0.0
    assert kern + kr.r == pytest.approx(full)


@pytest.mark.parametrize("seed", range(3))
def test_branching_keeps_the_mis(tb, orc, exact, seed):
    g = tb.random_regular_graph(60, 3, seed)
    w = tb.random_weights(g.n, seed) if seed % 2 else np.ones(g.n, np.float32)
    kr = tb.kernelize(g, w)
    code = tb.initialize_code(kr.g, tb.GreedyMethod(seed))
    slicer = tb.ContractionTreeSlicer(sc_target=6, refine=False)
    branches = tb.slice(tb.MISProblem(kr.g, kr.weights), code, kr.r, slicer)
    assert len(branches) > 1
    vals = []
    for b in branches:
        if b.code is None or b.p.g.n == 0:
            vals.append(b.r)
            continue
        assert b.code.complexity()[1] <= 6
        vals.append(orc.solve(b.code, b.p.weight_array()) + b.r)
    assert max(vals) == pytest.approx(exact.branch_and_bound(g.n, g.edges, w))


def test_index_slices_cover_the_full_solve(tb, orc):
    g, w, code = rr_case(tb, 50, 4)
    full = orc.solve(code, w)
    fixed, opened, vals = tb.index_slices(code, code.complexity()[1] - 3, open_bits=1)
    assert len(fixed) >= 1 and len(opened) == 1
    c2 = tb.CompressedEinsum(code.ixs, opened, code.children, n_labels=code.n_labels)
    best = max(orc.solve(c2, w, sliced=fixed, slice_vals=tuple(int(x) for x in row)) for row in vals)
    assert best == full


def test_tree_variants_agree(tb, orc):
    """order2eincode of a tree's elimination order and an annealed tree give
    the same value (test/decompose.jl:13-32)."""
    for seed in range(3):
        g = tb.random_regular_graph(40, 3, seed)
        w = tb.random_weights(g.n, seed)
        code = tb.initialize_code(g, tb.GreedyMethod(seed))
        ref = orc.solve(code, w)
        c2 = tb.order2eincode(g, tb.eincode2order(code))
        c3 = tb.initialize_code(g, tb.TreeSA(ntrials=1, niters=5, betas=np.arange(1.0, 6.0), nthreads=1))
        assert orc.solve(c2, w) == ref and orc.solve(c3, w) == ref


def test_lp_bound_is_an_upper_bound(tb, exact):
    for seed in range(4):
        g = tb.random_regular_graph(30, 3, seed)
        w = tb.random_weights(g.n, seed)
        lp = tb.LP_MWIS(g, w)
        assert lp >= exact.branch_and_bound(g.n, g.edges, w) - 1e-6
    g = tb.Graph(3, [(0, 1), (1, 2), (0, 2)])  # a triangle: the clique cut makes the LP exact
    assert tb.LP_MWIS(g, np.ones(3, np.float32)) == pytest.approx(1.0)


@pytest.mark.parametrize("seed", range(2))
def test_slice_dfs_lp(tb, orc, exact, tmp_path, seed):
    """Depth-first slicing with LP pruning (test/slice.jl:37-48): the best
    solution written to slices.csv is the MIS."""
    import csv

    g = tb.random_regular_graph(50, 3, seed)
    w = tb.random_weights(g.n, seed)
    kr = tb.kernelize(g, w)
    code = tb.initialize_code(kr.g, tb.GreedyMethod(seed))
    b = tb.SlicedBranch(tb.MISProblem(kr.g, kr.weights), code, kr.r)
    res = tb.slice_dfs_lp(b, tb.ContractionTreeSlicer(sc_target=6, refine=False), str(tmp_path),
                          solve=lambda x: orc.solve(x.code, x.p.weight_array()))
    want = exact.branch_and_bound(g.n, g.edges, w)
    assert res["primal"] == pytest.approx(want)
    with open(tmp_path / "slices.csv") as f:
        sols = [float(r["solution"]) for r in csv.DictReader(f)]
    assert max(sols) == pytest.approx(want) and len(sols) == res["slices"]
