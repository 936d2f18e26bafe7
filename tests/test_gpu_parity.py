"""GPU parity: every execution mode, through the C ABI, equals the CPU oracle
bit for bit -- per item, per intermediate tensor, for f32 and int32."""
import numpy as np
import pytest

from cases import corner_cases, ksg_case, random_generic_network, random_tensor, rr_case

pytestmark = pytest.mark.gpu
MODES = ["plain", "layered", "batched"]


@pytest.mark.parametrize("seed", range(4))
def test_rr_all_modes(tb, orc, exact, engine, seed):
    g, w, code = rr_case(tb, 30 + 10 * seed, seed)
    ref = orc.solve(code, w)
    plan = engine.plan(code, w)
    for mode in MODES:
        out, mx = engine.solve_batch([plan], mode=mode)
        assert np.float32(mx) == np.float32(ref) == out[0], (mode, mx, ref)
    if g.n <= 60:
        assert ref == exact.branch_and_bound(g.n, g.edges, w)


@pytest.mark.parametrize("mode", ["plain", "layered"])
def test_intermediates_bit_exact(tb, orc, engine, mode):
    g, w, code = rr_case(tb, 40, 3)
    plan = engine.plan(code, w)
    labs = plan.all_node_labels()
    ref_root, dumps = orc.execute(code, w, node_iy=labs, dump=True)
    got = engine.dump(plan, mode=mode)
    assert len(got) == len(dumps)
    for a, b in zip(got, dumps):
        assert np.array_equal(a, b)


def test_int32_engine(tb, orc, engine_i32):
    for seed in range(3):
        g, w, code = rr_case(tb, 40, seed)
        ref = orc.solve(code, w, dtype=np.int32)
        plan = engine_i32.plan(code, w)
        for mode in MODES:
            _, mx = engine_i32.solve_batch([plan], mode=mode)
            assert mx == ref, (mode, mx, ref)


def test_corner_cases(tb, orc, engine):
    for name, g, w, code in corner_cases(tb):
        plan = engine.plan(code, w)
        ref = orc.solve(code, w)
        for mode in MODES:
            _, mx = engine.solve_batch([plan], mode=mode)
            assert mx == ref, (name, mode)


def test_uneven_batch_of_branches(tb, orc, engine):
    """Many different plans in one batched launch (branch batch)."""
    plans, refs, rs = [], [], []
    for seed in range(12):
        if seed % 3 == 0:
            g, w, code = ksg_case(tb, 4 + seed % 4, seed)
        else:
            g, w, code = rr_case(tb, 12 + 4 * seed, seed)
        plans.append(engine.plan(code, w))
        refs.append(orc.solve(code, w))
        rs.append(float(seed))
    expect = np.array(refs, np.float32) + np.array(rs, np.float32)
    for mode in MODES:
        out, mx = engine.solve_batch(plans, r=np.array(rs, np.float32), mode=mode)
        assert np.array_equal(out, expect), mode
        assert mx == expect.max()
    # graph replay of the same batch gives the same numbers
    out2, _ = engine.solve_batch(plans, r=np.array(rs, np.float32), mode="batched")
    assert np.array_equal(out2, expect)


def test_sliced_items(tb, orc, engine):
    g, w, code = rr_case(tb, 40, 5)
    full = orc.solve(code, w)
    sliced = [0, 7, 13]
    plan = engine.plan(code, w, sliced=sliced)
    vals = ((np.arange(8)[:, None] >> np.arange(3)[None, :]) & 1).astype(np.int8)
    refs = np.array([orc.solve(code, w, sliced=sliced, slice_vals=v) for v in vals], np.float32)
    for mode in MODES:
        out, mx = engine.solve_batch([plan] * 8, slice_vals=list(vals), mode=mode)
        assert np.array_equal(out, refs), mode
        assert mx == full


def test_open_labels_with_slices(tb, orc, engine):
    g, w, code = rr_case(tb, 36, 8)
    full = orc.solve(code, w)
    opened = tb.CompressedEinsum(code.ixs, [3, 11], code.children, n_labels=code.n_labels)
    plan = engine.plan(opened, w, sliced=[20])
    out, mx = engine.solve_batch([plan, plan], slice_vals=[np.array([0], np.int8), np.array([1], np.int8)],
                                 mode="batched")
    assert mx == full


def test_contract_generic_tensors(tb, orc, engine):
    """code(tensors...) with arbitrary tropical tensors (test/utils.jl:34)."""
    rng = np.random.default_rng(9)
    for it in range(30):
        ixs, iy, ch = random_generic_network(rng, n_labels=12, n_tensors=7, max_rank=5,
                                             n_open=int(rng.integers(0, 3)))
        code = tb.CompressedEinsum(ixs, iy, ch)
        data = [random_tensor(rng, len(ix)) for ix in ixs]
        ref = orc.execute(code, None, leaf_data=data)
        plan = engine.plan(code)
        for mode in ("plain", "layered"):
            got = engine.contract(plan, data, mode=mode)
            assert np.array_equal(got, ref), (it, mode)


@pytest.mark.parametrize("shape", [(4, 4, 5, 1), (5, 4, 6, 2), (6, 6, 5, 0), (7, 5, 5, 1), (7, 7, 6, 2),
                                   (8, 7, 5, 1), (4, 4, 8, 0), (6, 6, 9, 1), (5, 5, 7, 2), (7, 7, 8, 1),
                                   (6, 6, 4, 1), (7, 7, 4, 2), (7, 6, 4, 0),
                                   (8, 4, 4, 1), (4, 9, 4, 0), (9, 5, 5, 1), (5, 8, 6, 1)])
def test_fused_gemm_nodes(tb, orc, engine, shape):
    from cases import gemm_case

    g, w, code = gemm_case(tb, *shape)
    plan = engine.plan(code, w)
    labs = plan.all_node_labels()
    ref, dumps = orc.execute(code, w, node_iy=labs, dump=True)
    for mode in MODES:
        _, mx = engine.solve_batch([plan], mode=mode)
        assert mx == np.max(ref), mode
    for mode in ("layered", "plain"):
        got = engine.dump(plan, mode=mode)
        for a, b in zip(got, dumps):
            assert np.array_equal(a, b), mode


def test_rebinding_weights_between_solves(tb, orc, engine):
    """Weights travel with each solve: re-binding between two solves of the
    same batch (CUDA graph replayed) gives the new weights' results in every
    mode, and the dump path (LeafDesc weights) follows too."""
    g, w, code = rr_case(tb, 36, 9)
    plan = engine.plan(code, w)
    plan2 = engine.plan(code, w)
    rng = np.random.default_rng(3)
    for rep in range(3):
        w2 = rng.integers(1, 10, g.n).astype(np.float32)
        plan.bind_mis(w2)
        plan2.bind_mis(w2[::-1].copy())
        ref = orc.solve(code, w2)
        ref2 = orc.solve(code, w2[::-1].copy())
        for mode in MODES:
            out, mx = engine.solve_batch([plan, plan2, plan], r=[0.0, 0.0, 1.0], mode=mode)
            assert list(out) == [np.float32(ref), np.float32(ref2), np.float32(ref + 1)], (rep, mode)
        dumps = engine.dump(plan, mode="layered")
        assert np.max(dumps[-1]) == np.float32(ref)
    w3 = rng.integers(1, 10, g.n).astype(np.float32)
    engine.bind_batch([plan, plan2], [w3, w3[::-1].copy()])
    out, _ = engine.solve_batch([plan, plan2], mode="batched")
    assert list(out) == [np.float32(orc.solve(code, w3)), np.float32(orc.solve(code, w3[::-1].copy()))]


@pytest.mark.parametrize("arith", ["f32", "i16x2"])
@pytest.mark.parametrize("kind", ["small_int", "large_int", "fractional", "negative"])
def test_gemm_arithmetic_forms(tb, orc, engine, engine_i16, kind, arith):
    """By default GEMM tiles compute in f32; a context opened with
    gemm_arith="i16x2" runs exact packed-int16 GEMM tiles when the weights
    are integers >= 0 summing below 8192, f32 otherwise; split-K parts
    combine by atomic max when the weights are >= 0, through partials
    otherwise; all equal the oracle."""
    from cases import gemm_case

    eng = engine if arith == "f32" else engine_i16
    for shape, atomic in (((7, 7, 6, 1), False), ((8, 7, 5, 1), False), ((7, 6, 8, 0), False),
                          ((7, 6, 8, 0), True), ((7, 7, 4, 1), False)):
        eng.set_kpart_atomic(atomic)
        g, w, code = gemm_case(tb, *shape)
        if kind == "large_int":
            w = (w * 300).astype(np.float32)           # sum > 8192
        elif kind == "fractional":
            w = (w + 0.5).astype(np.float32)
        elif kind == "negative":
            # negative values: split-K parts go through partials, not atomics
            w = (w - 5.0).astype(np.float32)
        plan = eng.plan(code, w)
        ref, dumps = orc.execute(code, w, node_iy=plan.all_node_labels(), dump=True)
        for mode in ("batched", "layered"):
            out, mx = eng.solve_batch([plan, plan], r=[0.0, 2.0], mode=mode)
            assert mx == np.max(ref) + 2 and out[0] == np.max(ref), (kind, shape, mode, arith, atomic)
    eng.set_kpart_atomic(False)


@pytest.mark.parametrize("wide", [False, True])
@pytest.mark.parametrize("bits", [8, 10, 11])
def test_stream_tile_configurations(tb, orc, engine, bits, wide):
    """Every stream tile size and stream kernel form the autotuner may choose
    gives the oracle's intermediates in the fused modes."""
    engine.set_stream_wide(wide)
    import ctypes

    lib = engine.lib
    lib.tbi_plan_retile.restype = ctypes.c_int32
    lib.tbi_plan_retile.argtypes = [ctypes.c_void_p, ctypes.c_int32]
    for g, w, code in (rr_case(tb, 60, 3), ksg_case(tb, 7, 2)):
        plan = engine.plan(code, w)
        assert lib.tbi_plan_retile(plan.handle, bits) == 0
        labs = plan.all_node_labels()
        ref, dumps = orc.execute(code, w, node_iy=labs, dump=True)
        for mode in ("batched", "layered"):
            out, mx = engine.solve_batch([plan, plan], r=[0.0, 1.0], mode=mode)
            assert mx == np.max(ref) + 1 and out[0] == np.max(ref), (mode, bits)
        got = engine.dump(plan, mode="layered")
        for a, b in zip(got, dumps):
            assert np.array_equal(a, b)
    engine.set_stream_wide(True)  # the default
