"""CPU replay of the device programs the engine compiles (index arithmetic
of csrc/kernels.cuh): every access in bounds, every output written once, and
every intermediate equal to the oracle's, for the fused and the plain path."""
import numpy as np
import pytest

import emulate
from cases import corner_cases, ksg_case, rr_case


@pytest.fixture(scope="module")
def lib(native):
    return native.engine_lib()


def _check(lib, orc, code, w, sliced=(), sv=()):
    """The fused program with every stream step as a stream tile (the
    persistent executor) and with the small ones as tiny steps (the per-level
    launches), and the plain program, against the oracle."""
    d = emulate.describe(lib, code, sliced)
    root, nodes = emulate.run_fused(d, w, sv)
    roott, nodest = emulate.run_fused(d, w, sv, lib=lib)
    rootp, nodesp = emulate.run_plain(emulate.describe(lib, code, sliced), w, sv)
    ref, dumps = orc.execute(code, w, sliced=sliced, slice_vals=sv, dump=True)
    assert np.array_equal(root, ref) and np.array_equal(roott, ref) and np.array_equal(rootp, ref)
    for a, t, b, c in zip(nodes, nodest, nodesp, dumps or []):
        assert np.array_equal(a, c) and np.array_equal(t, c) and np.array_equal(b, c)
    return float(np.max(ref))


@pytest.mark.parametrize("case", ["ksg", (2, 2, 3, 0), (1, 1, 5, 0), (3, 2, 4, 1)])
def test_tiny_steps(tb, orc, lib, case):
    """Tiny steps (one warp each, straight from global memory): the small
    nodes of a King's subgraph network, and middle nodes reducing 2^3 to 2^5
    terms (lanes over outputs and terms, a shuffle max per output); their
    TinyDesc offsets give the oracle's intermediates."""
    from cases import gemm_case

    g, w, code = ksg_case(tb, 6, 3) if case == "ksg" else gemm_case(tb, *case)
    d = emulate.describe(lib, code)
    tiny = [emulate.tiny_desc(lib, d["tiles"][s.desc]) for s in d["steps"] if s.kind == emulate.STEP_TILE]
    tiny = [t for ok, t in tiny if ok]
    if case == "ksg":
        assert len(tiny) > 10
    else:
        assert max(t.n_tr for t in tiny) == case[2]
    _check(lib, orc, code, w)


@pytest.mark.parametrize("seed", range(4))
def test_rr_fused_and_plain(tb, orc, lib, seed):
    g, w, code = rr_case(tb, 20 + 4 * seed, seed)
    _check(lib, orc, code, w)


def test_slices_and_open_labels(tb, orc, lib):
    g, w, code = rr_case(tb, 24, 11)
    full = _check(lib, orc, code, w)
    vals = [_check(lib, orc, code, w, [0, 5], (a, b)) for a in (0, 1) for b in (0, 1)]
    assert max(vals) == full
    opened = tb.CompressedEinsum(code.ixs, [2, 9], code.children, n_labels=code.n_labels)
    _check(lib, orc, opened, w)
    for a in (0, 1):
        _check(lib, orc, opened, w, [4], (a,))


def test_ksg(tb, orc, lib):
    g, w, code = ksg_case(tb, 5, 1)
    _check(lib, orc, code, w)


def test_corner_cases(tb, orc, lib):
    for name, g, w, code in corner_cases(tb):
        _check(lib, orc, code, w)


def test_explicit_node_labels(tb, orc, lib):
    """Node outputs given explicitly (as a DynamicNestedEinsum carries them),
    including labels kept longer than needed."""
    g, w, code = rr_case(tb, 20, 4)
    labs = code.labels_of_nodes()
    # keep one extra label alive in a few nodes where it is available
    T = code.n_tensors
    full = [list(dict.fromkeys(ix)) for ix in code.ixs] + labs
    extra = []
    for j, (a, b) in enumerate(code.children):
        uni = list(dict.fromkeys(full[a] + full[b]))
        keep = list(labs[j])
        drop = [x for x in uni if x not in keep]
        if drop and j % 3 == 0 and j < code.n_nodes - 1:
            keep = keep + [drop[0]]
        extra.append(keep)
        full[T + j] = keep
    c2 = tb.CompressedEinsum(code.ixs, code.iy, code.children, node_iy=extra, n_labels=code.n_labels)
    d = emulate.describe(lib, c2, use_node_iy=True)
    root, nodes = emulate.run_fused(d, w)
    ref, dumps = orc.execute(c2, w, node_iy=extra, dump=True)
    assert np.array_equal(root, ref)
    for a, b in zip(nodes, dumps):
        assert np.array_equal(a, b)


def test_invalid_plans_rejected(tb, lib):
    g, w, code = rr_case(tb, 20, 1)
    bad = code.children.copy()
    bad[-1, 0] = bad[-1, 1]
    with pytest.raises(ValueError):
        emulate.describe(lib, tb.CompressedEinsum(code.ixs, [], bad, n_labels=code.n_labels))
    labs = code.labels_of_nodes()
    labs[0] = []  # drops labels needed later
    with pytest.raises(ValueError):
        emulate.describe(lib, tb.CompressedEinsum(code.ixs, [], code.children, node_iy=labs,
                                                  n_labels=code.n_labels), use_node_iy=True)


@pytest.mark.parametrize("shape", [(4, 4, 5, 1), (5, 4, 6, 2), (6, 6, 5, 0), (7, 5, 5, 1), (4, 4, 8, 0),
                                   (6, 6, 9, 1), (5, 5, 7, 2), (6, 6, 4, 1), (7, 7, 4, 2), (7, 6, 4, 0),
                                   (8, 4, 4, 1), (4, 9, 4, 0), (9, 5, 5, 1), (5, 8, 6, 1)])
def test_gemm_steps(tb, orc, lib, shape):
    """GEMM steps, including K split into parts plus a max over the parts
    when the output tiles are too few for the GPU."""
    from cases import gemm_case

    g, w, code = gemm_case(tb, *shape)
    d = emulate.describe(lib, code)
    gem = [s for s in d["steps"] if s.kind == emulate.STEP_GEMM]
    assert len(gem) == 1  # K = 16 (k = 4 labels) included: BK = 16 tiles
    ks = d["gemms"][gem[0].desc].ks_log2
    assert (ks > 0) == (shape[2] >= 7)
    if ks > 0:
        fills = [s for s in d["steps"] if s.kind == emulate.STEP_FILL]
        assert len(fills) == 1 and gem[0].dep0 == d["steps"].index(fills[0])
        assert fills[0].level < gem[0].level
    ref, dumps = orc.execute(code, w, dump=True)
    # the K parts through partials and a max step, and by atomic max of the
    # value bits into the filled output (the weights are >= 0), in list order
    # and in an order that follows only the dependencies
    for atomic in (False, True):
        for by_deps in (False, True):
            root, nodes = emulate.run_fused(d, w, kpart_atomic=atomic, by_deps=by_deps)
            assert np.array_equal(root, ref)
            for a, b in zip(nodes, dumps):
                assert np.array_equal(a, b)
    # the merged form (batches that fill the GPU): one pass over the whole K
    # into the output, the fill and max steps without tiles
    m = emulate.merged(d)
    g0, g1 = d["gemms"][gem[0].desc], m["gemms"][gem[0].desc]
    si = d["steps"].index(gem[0])
    assert g1.ks_log2 == 0 and g1.c_off == g0.c_fin and g1.n_tiles == g0.n_tiles >> ks
    assert m["steps"][si].n_tiles == g1.n_tiles
    for k, st in enumerate(d["steps"]):
        if st.kind in (emulate.STEP_FILL, emulate.STEP_KRED):
            assert m["steps"][k].n_tiles == 0
    for atomic in (False, True):
        root, nodes = emulate.run_fused(m, w, kpart_atomic=atomic, by_deps=True)
        assert np.array_equal(root, ref)
        for a, b in zip(nodes, dumps):
            assert np.array_equal(a, b)


@pytest.mark.parametrize("shape,tile", [((4, 4, 4, 1), None), ((5, 7, 4, 0), None), ((6, 6, 4, 1), (6, 6)),
                                         ((4, 4, 5, 1), (4, 4)), ((4, 8, 4, 0), (4, 8)), ((9, 5, 4, 1), (8, 4)),
                                         ((5, 7, 5, 0), (5, 5)), ((7, 6, 5, 0), (7, 6))])
def test_gemm_threshold(tb, lib, shape, tile):
    """A node with K = 16 becomes a GEMM only when M and N are >= 64, or one
    is >= 16 and the other >= 256 (256 x 16 tiles); with K >= 32, M and N >=
    16 suffice.  The CTA tile (log2 of its rows and columns) follows M and N."""
    from cases import gemm_case

    g, w, code = gemm_case(tb, *shape)
    d = emulate.describe(lib, code)
    gem = [s for s in d["steps"] if s.kind == emulate.STEP_GEMM]
    assert bool(gem) == (tile is not None)
    if gem:
        gd = d["gemms"][gem[0].desc]
        assert (gd.bm_log2, gd.bn_log2) == tile


@pytest.mark.parametrize("bits", [8, 10, 11])
def test_tile_sizes_of_the_autotuner(tb, orc, lib, bits):
    """Every stream tile size tb_autotune may pick (tile_bits 8..11) keeps
    every access in bounds and every intermediate equal to the oracle's."""
    for g, w, code in (rr_case(tb, 60, 3), ksg_case(tb, 8, 2)):
        D = emulate.describe(lib, code, tile_bits=bits)
        root, nodes = emulate.run_fused(D, w, ())
        ref, dumps = orc.execute(code, w, dump=True)
        assert np.array_equal(root, ref)
        for a, c in zip(nodes, dumps or []):
            assert np.array_equal(a, c)
    # the knob changes the tiling
    g, w, code = rr_case(tb, 60, 3)
    n8 = sum(s.n_tiles for s in emulate.describe(lib, code, tile_bits=8)["steps"])
    n10 = sum(s.n_tiles for s in emulate.describe(lib, code, tile_bits=10)["steps"])
    assert n8 > n10


# ---------------------------------------------------------------------------
# fused small form (TB_MODE_FUSED): one block per network, shared memory only
# ---------------------------------------------------------------------------
def _check_small(lib, orc, code, w, sliced=(), sv=(), r=0.0):
    sd = emulate.describe_small(lib, code, sliced)
    assert sd["ok"]
    desc = emulate.describe(lib, code, sliced)
    ch = code.children if code.n_nodes else np.zeros((0, 2), np.int32)
    got = emulate.run_small(sd, desc["leaves"], ch, w, sv, r)
    ref = orc.execute(code, w, sliced=sliced, slice_vals=sv)
    assert got == float(np.max(ref)) + r
    return sd


@pytest.mark.parametrize("seed", range(4))
def test_small_form_rr(tb, orc, lib, seed):
    g, w, code = rr_case(tb, 24 + 6 * seed, seed, weighted=bool(seed % 2))
    sd = _check_small(lib, orc, code, w, r=1.5 * seed)
    assert sd["words"] >= sum(1 << len(set(ix)) for ix in code.ixs)


def test_small_form_slices_open_labels_and_corners(tb, orc, lib):
    g, w, code = rr_case(tb, 24, 11)
    for a in (0, 1):
        for b in (0, 1):
            _check_small(lib, orc, code, w, [0, 5], (a, b))
    opened = tb.CompressedEinsum(code.ixs, [2, 9], code.children, n_labels=code.n_labels)
    _check_small(lib, orc, opened, w)
    _check_small(lib, orc, opened, w, [4], (1,))
    for name, g, w, code in corner_cases(tb):
        _check_small(lib, orc, code, w)
    g, w, code = ksg_case(tb, 5, 1, weighted=True)
    _check_small(lib, orc, code, w)


def test_small_form_limits(tb, lib):
    """Networks past the shared-memory budget or the rank limit have no
    small form (TB_MODE_FUSED refuses them)."""
    g, w, code = rr_case(tb, 120, 3)
    assert code.complexity()[1] > 13
    assert not emulate.describe_small(lib, code)["ok"]
    g, w, code = rr_case(tb, 40, 3)
    assert code.complexity()[1] <= 13 and emulate.describe_small(lib, code)["ok"]


def test_small_form_branch_batch(tb, orc, lib):
    """Branches of the reference's rule (sc <= 8) all have a small form and
    replay to the oracle's values."""
    g = tb.random_regular_graph(60, 3, 5)
    w = np.ones(g.n, np.float32)
    kr = tb.kernelize(g, w)
    code = tb.initialize_code(kr.g, tb.GreedyMethod(5))
    branches = tb.slice(tb.MISProblem(kr.g, kr.weights), code, kr.r,
                        tb.ContractionTreeSlicer(sc_target=8, refine=False,
                                                 region_selector=tb.ScoreRS(n_max=12)))
    for b in branches:
        if b.code is None or b.p.g.n == 0:
            continue
        _check_small(lib, orc, b.code, b.p.weight_array(), r=b.r)


def test_level_spans(lib):
    """Every ticket of a per-level launch goes to exactly one CTA, and the
    CTAs given to the tiny steps (listed first) take no other tile: k_level's
    split of its grid (LevelSpan) over random ranges."""
    import ctypes

    lib.tbi_level_span.restype = ctypes.c_int32
    lib.tbi_level_span.argtypes = [ctypes.c_int64] * 4 + [ctypes.c_void_p]
    rng = np.random.default_rng(0)
    cases = [(1, 0, 304), (1, 1, 304), (5, 5, 1), (13290, 11735, 304), (2000, 3, 304), (300, 297, 304)]
    cases += [(int(c), int(rng.integers(0, c + 1)), int(rng.integers(1, 700)))
              for c in rng.integers(1, 20000, 40)]
    for count, tiny, ctas in cases:
        out = np.zeros(7, np.int64)
        assert lib.tbi_level_span(100, count, tiny, ctas, out.ctypes.data) == 0
        grid, first, mid, last, chunk, chunk2, split = (int(x) for x in out)
        assert 1 <= grid <= ctas and first == 100 and last == 100 + count and 0 <= split <= grid
        if 0 < tiny < count and ctas >= 2:
            assert mid == 100 + tiny and 0 < split < grid  # the tiny CTAs end at the last tiny step
        hits = np.zeros(count, np.int64)
        for b in range(grid):
            if b < split:
                t0, t1 = first + b * chunk, min(first + (b + 1) * chunk, mid)
            else:
                t0 = mid + (b - split) * chunk2
                t1 = min(t0 + chunk2, last)
            if t0 < t1:
                hits[t0 - 100:t1 - 100] += 1
        assert np.all(hits == 1), (count, tiny, ctas)


@pytest.mark.parametrize("name", ["rr220", "rr220w_s22", "rr300w_s22"])
def test_merged_form_of_workload_plans(tb, lib, name):
    """The merged split-K form of the benchmark workloads' plans (the form a
    batch that fills the GPU runs): no step with tiles waits on a step
    without tiles (the persistent executor counts those as done at once, so
    such a wait would be no wait), each merged GEMM covers the whole K into
    its node's output and waits on the step that wrote its A operand."""
    from tensorbranching_gb300 import workloads

    wl = workloads.load(name)
    it = workloads.step_items(wl, 1)[0]
    d = emulate.describe(lib, it["code"], it["fixed"], tile_bits=10)
    steps, merged = d["steps"], d["steps_merged"]
    split = [k for k, s in enumerate(steps) if s.kind == emulate.STEP_GEMM and d["gemms"][s.desc].ks_log2 > 0]
    assert split  # each of these plans splits K at one GEMM node for one item alone
    for k, s in enumerate(merged):
        if s.n_tiles > 0:
            for dep in (s.dep0, s.dep1):
                assert dep < 0 or merged[dep].n_tiles > 0, (name, k, dep)
    for k in split:
        g0, g1 = d["gemms"][steps[k].desc], d["gemms_merged"][steps[k].desc]
        assert g1.ks_log2 == 0 and g1.c_off == g0.c_fin and merged[k].n_tiles == g0.n_tiles >> g0.ks_log2
        fill = steps[steps[k].dep0]
        assert fill.kind == emulate.STEP_FILL and merged[k].dep0 == fill.dep0
