"""TB_MODE_FUSED (one block per network, every tensor in shared memory) on
the GPU: bit-exact against the oracle for uneven branch batches, sliced
items, open labels, r offsets, f32 and int32; plans past its limits are
refused; TB_MODE_AUTO falls back to the tuned tile schedule for them."""
import numpy as np
import pytest

from cases import corner_cases, ksg_case, rr_case

pytestmark = pytest.mark.gpu


def _uneven(tb, orc, engine, n=13):
    plans, refs, rs = [], [], []
    for seed in range(n):
        if seed % 3 == 0:
            g, w, code = ksg_case(tb, 4 + seed % 4, seed, weighted=bool(seed % 2))
        else:
            g, w, code = rr_case(tb, 12 + 4 * seed, seed, weighted=bool(seed % 2))
        plans.append(engine.plan(code, w))
        refs.append(orc.solve(code, w))
        rs.append(0.5 * seed)
    return plans, np.array(refs, np.float32) + np.array(rs, np.float32), np.array(rs, np.float32)


def test_fused_uneven_batch(tb, orc, engine):
    plans, expect, rs = _uneven(tb, orc, engine)
    assert all(p.stats()["small_words"] > 0 for p in plans)
    for _ in range(2):  # capture, then graph replay
        out, mx = engine.solve_batch(plans, r=rs, mode="fused")
        assert np.array_equal(out, expect)
        assert mx == expect.max()


def test_fused_int32(tb, orc, engine_i32):
    plans, refs = [], []
    for seed in range(6):
        g, w, code = rr_case(tb, 30 + 4 * seed, seed)
        plans.append(engine_i32.plan(code, w))
        refs.append(orc.solve(code, w, dtype=np.int32))
    out, mx = engine_i32.solve_batch(plans, mode="fused")
    assert np.array_equal(out, np.array(refs, np.float32))


def test_fused_sliced_and_open(tb, orc, engine):
    g, w, code = rr_case(tb, 40, 5)
    full = orc.solve(code, w)
    sliced = [0, 7, 13]
    plan = engine.plan(code, w, sliced=sliced)
    vals = ((np.arange(8)[:, None] >> np.arange(3)[None, :]) & 1).astype(np.int8)
    refs = np.array([orc.solve(code, w, sliced=sliced, slice_vals=v) for v in vals], np.float32)
    out, mx = engine.solve_batch([plan] * 8, slice_vals=list(vals), mode="fused")
    assert np.array_equal(out, refs) and mx == full
    opened = tb.CompressedEinsum(code.ixs, [3, 11], code.children, n_labels=code.n_labels)
    plan = engine.plan(opened, w, sliced=[20])
    _, mx = engine.solve_batch([plan, plan], slice_vals=[np.array([0], np.int8), np.array([1], np.int8)],
                               mode="fused")
    assert mx == full


def test_fused_corner_cases(tb, orc, engine):
    for name, g, w, code in corner_cases(tb):
        plan = engine.plan(code, w)
        _, mx = engine.solve_batch([plan], mode="fused")
        assert mx == orc.solve(code, w), name


def test_fused_refuses_large_plans_and_auto_falls_back(tb, orc):
    eng = tb.Engine()
    try:
        plans, expect, rs = _uneven(tb, orc, eng, n=9)
        res = eng.autotune(plans, r=rs)
        out, _ = eng.solve_batch(plans, r=rs, mode="auto")
        assert np.array_equal(out, expect), res
        g, w, code = rr_case(tb, 120, 3)
        big = eng.plan(code, w)
        assert big.stats()["small_words"] == 0
        with pytest.raises(tb._native.TbError) as ei:
            eng.solve_batch([big], mode="fused")
        assert ei.value.status == tb._native.TB_ERR_UNSUPPORTED
        _, mx = eng.solve_batch([big], mode="auto")
        assert mx == orc.solve(code, w)
    finally:
        eng.close()


def test_fused_branch_batch(tb, orc, engine):
    """Every branch of the reference's branching rule on two graphs, one
    fused launch; max per graph equals the full contraction."""
    plans, graphs, owner, rs = [], [], [], []
    for seed in (21, 22):
        g = tb.random_regular_graph(70, 3, seed)
        w = tb.random_weights(g.n, seed)
        kr = tb.kernelize(g, w)
        code = tb.initialize_code(kr.g, tb.GreedyMethod(seed))
        brs = tb.slice(tb.MISProblem(kr.g, kr.weights), code, kr.r,
                       tb.ContractionTreeSlicer(sc_target=9, refine=False))
        graphs.append((g, w))
        for b in brs:
            if b.code is None or b.p.g.n == 0:
                continue
            plans.append(engine.plan(b.code, b.p.weight_array()))
            owner.append(len(graphs) - 1)
            rs.append(b.r)
    out, _ = engine.solve_batch(plans, r=np.array(rs, np.float32), mode="fused")
    lay, _ = engine.solve_batch(plans, r=np.array(rs, np.float32), mode="layered")
    assert np.array_equal(out, lay)
    for k, (g, w) in enumerate(graphs):
        got = max(float(v) for v, o in zip(out, owner) if o == k)
        assert got == orc.solve(tb.initialize_code(g, tb.GreedyMethod(1)), w)
