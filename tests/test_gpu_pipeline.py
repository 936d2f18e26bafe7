"""The reference's entry point end to end on the GPU: dynamic_ob_mis with
ContractionTreeSlicer(sc_target=10) on 3-regular graphs equals the exact MIS
(test/dynamic_ob.jl:10-52), and every known-answer case of
tests/golden/mis_known.json solves to its stored value in one batch."""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.mark.parametrize("seed", range(3))
@pytest.mark.parametrize("mode", ["batched", "plain"])
def test_dynamic_ob_mis(tb, exact, engine, seed, mode):
    g = tb.random_regular_graph(80, 3, seed)
    w = tb.random_weights(g.n, seed) if seed % 2 else np.ones(g.n, np.float32)
    slicer = tb.ContractionTreeSlicer(sc_target=10)
    got = tb.dynamic_ob_mis(g, w, slicer=slicer, engine=engine, mode=mode)
    assert got == pytest.approx(exact.branch_and_bound(g.n, g.edges, w))


@pytest.mark.parametrize("brancher", ["greedy", "fixed_point", "vertex"])
@pytest.mark.parametrize("weighted", [False, True])
def test_dynamic_ob_mis_branchers(tb, orc, engine, brancher, weighted):
    """The brancher grid of test/dynamic_ob.jl:10-26 (sc_target=10): the
    reference's optimal branching with either brancher, and the vertex rule;
    every branch set is contracted in one batch on the GPU and the answer is
    the full network's (the oracle's contraction of the unbranched graph, as
    the reference test compares with the full solve)."""
    seed = 11 if weighted else 12
    g = tb.random_regular_graph(80, 3, seed)
    w = tb.random_weights(g.n, seed) if weighted else np.ones(g.n, np.float32)
    b = {"greedy": tb.GreedyBrancher(), "fixed_point": tb.FixedPointBrancher(), "vertex": tb.VertexBrancher()}[brancher]
    slicer = tb.ContractionTreeSlicer(sc_target=10, refine=False, brancher=b)
    got = tb.dynamic_ob_mis(g, w, slicer=slicer, engine=engine, mode="auto")
    assert got == orc.solve(tb.initialize_code(g, tb.GreedyMethod(seed)), w)


def test_golden_cases_in_one_batch(tb, engine):
    cases = json.load(open(os.path.join(HERE, "golden", "mis_known.json")))["cases"]
    plans, want = [], []
    for c in cases:
        g = tb.Graph(c["n"], [tuple(e) for e in c["edges"]])
        w = np.ones(c["n"], np.float32) if c["weights"] is None else np.array(c["weights"], np.float32)
        plans.append(engine.plan(tb.initialize_code(g, tb.GreedyMethod(1)), w))
        want.append(c["mis"])
    for mode in ("batched", "layered"):
        out, mx = engine.solve_batch(plans, mode=mode)
        assert np.array_equal(out, np.array(want, np.float32)), mode


def test_slices_from_disk_on_the_gpu(tb, exact, engine, tmp_path):
    """A directory in the reference's slice format (src/io.jl) contracted by
    contract_slices on the GPU: max + r is the MIS."""
    sio = tb.slice_io
    g = tb.random_regular_graph(70, 3, 4)
    w = tb.random_weights(g.n, 4)
    kr = tb.kernelize(g, w)
    code = tb.initialize_code(kr.g, tb.GreedyMethod(4))
    branches = tb.slice(tb.MISProblem(kr.g, kr.weights), code, kr.r,
                        tb.ContractionTreeSlicer(sc_target=8, refine=False))
    for i, b in enumerate(branches):
        sio.save_finished(str(tmp_path), b, 7 + i)
    sio.save_slices_csv(str(tmp_path), [(7 + i, b.sc(), b.tc(), b.r) for i, b in enumerate(branches)])
    back = sio.load_all_finished(str(tmp_path))
    res = tb.contract_slices(back, engine=engine, mode="batched")
    assert float(np.max(res)) == pytest.approx(exact.branch_and_bound(g.n, g.edges, w))


def test_slice_dfs_lp_on_the_gpu(tb, exact, engine, tmp_path):
    g = tb.random_regular_graph(80, 3, 6)
    w = tb.random_weights(g.n, 6)
    kr = tb.kernelize(g, w)
    code = tb.initialize_code(kr.g, tb.GreedyMethod(6))
    b = tb.SlicedBranch(tb.MISProblem(kr.g, kr.weights), code, kr.r)
    res = tb.slice_dfs_lp(b, tb.ContractionTreeSlicer(sc_target=8, refine=False), str(tmp_path), engine=engine)
    assert res["primal"] == pytest.approx(exact.branch_and_bound(g.n, g.edges, w))
    back = tb.slice_io.load_all_finished(str(tmp_path))
    assert len(back) == sum(1 for x in back)  # the directory reads back
