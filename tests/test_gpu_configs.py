"""Parity at the benchmark workloads' own sizes (GPU, through the C ABI).

Each workload bench.py times is solved here item by item and compared with
the oracle's stored answers (tests/golden/workload_answers.json, made by
tests/golden/make_answers.py from the CPU oracle and the exact MIS integer
program) and, on a sample the oracle finishes in seconds, with the oracle
run now.  The relations are the reference's own: the network's MIS equals
the exact MIS (test/utils.jl:34,37), and the max over a graph's branches and
slices, each + r, equals the full solve (test/slice.jl:32-33,
test/dynamic_ob.jl:20,38,51).  Values are integers: every comparison is exact.
"""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def answers():
    with open(os.path.join(HERE, "golden", "workload_answers.json")) as f:
        return json.load(f)


@pytest.fixture(scope="module")
def workloads(tb):
    from tensorbranching_gb300 import workloads as w

    return w


def _graph_values(ans, out):
    """Per graph: max over its items and its empty branches' r."""
    vals = [-np.inf] * len(ans["graph_mis"])
    for g, v in zip(ans["graph_of_item"], out):
        vals[g] = max(vals[g], float(v))
    for g, r in enumerate(ans["graph_empty_r"]):
        if r is not None:
            vals[g] = max(vals[g], r)
    return vals


def _solve(eng, workloads, name, modes, max_items=0):
    wl = workloads.load(name)
    items = workloads.step_items(wl, max_items)
    plans, svs, rs = workloads.plans_for(eng, items)
    res = {m: eng.solve_batch(plans, slice_vals=svs, r=rs, mode=m) for m in modes}
    return wl, items, res


@pytest.mark.parametrize("arith,atomic", [("f32", False), ("f32", True), ("i16x2", False)])
def test_rr220_full_contraction(tb, orc, workloads, answers, engine, engine_i16, arith, atomic):
    """3-regular n=220: one contraction with tensors up to 2^28 entries, GEMM
    tiles in f32 and in the exact packed-int16 form, the split-K node's parts
    through partials and by atomic max; MIS 99 by the oracle (run now) and by
    the integer program (stored)."""
    eng = engine if arith == "f32" else engine_i16
    eng.set_kpart_atomic(atomic)
    wl, items, res = _solve(eng, workloads, "rr220", ("layered", "batched"))
    eng.set_kpart_atomic(False)
    ref = orc.solve(items[0]["code"], items[0]["weights"])
    ans = answers["rr220"]
    assert ans["graph_mis"] == [ref] == ans["items"]
    for mode, (out, mx) in res.items():
        assert mx == ref and list(out) == ans["items"], (mode, arith)


def test_rr100_ob10_whole_batch(tb, orc, workloads, answers, engine):
    """The 2604 branch networks of 32 graphs (n=100, the reference's
    branching rule, sc <= 10) in one batch, fused and per-level: every item
    equals the oracle's, and per graph the max + r equals the exact MIS."""
    wl, items, res = _solve(engine, workloads, "rr100_ob10", ("fused", "layered"))
    ans = answers["rr100_ob10"]
    for mode, (out, mx) in res.items():
        assert list(out) == ans["items"], mode
        assert _graph_values(ans, out) == ans["graph_mis"], mode
    # a sample against the oracle run now
    for k in np.linspace(0, len(items) - 1, 24).astype(int):
        it = items[k]
        assert ans["items"][k] == orc.solve(it["code"], it["weights"]) + it["r"]


def test_rr100_b10_whole_batch(tb, workloads, answers, engine):
    """The same 32 graphs branched by the two-way vertex rule (5062
    networks)."""
    wl, items, res = _solve(engine, workloads, "rr100_b10", ("fused",))
    ans = answers["rr100_b10"]
    out, mx = res["fused"]
    assert list(out) == ans["items"]
    assert _graph_values(ans, out) == ans["graph_mis"]


def test_ksg32_b20_whole_batch(tb, orc, workloads, answers, engine):
    """King's subgraph L=32: all 448 branches (sc <= 20) per level; every
    item equals the stored oracle value, the max + r equals the exact MIS,
    and six branches agree with the oracle run now."""
    wl, items, res = _solve(engine, workloads, "ksg32_b20", ("layered",))
    ans = answers["ksg32_b20"]
    out, mx = res["layered"]
    assert list(out) == ans["items"]
    assert _graph_values(ans, out) == ans["graph_mis"]
    for k in np.linspace(0, len(items) - 1, 6).astype(int):
        it = items[k]
        assert out[k] == orc.solve(it["code"], it["weights"]) + it["r"]


@pytest.mark.parametrize("name", ["ksg32_ob20", "ksg32_dom20"])
def test_ksg32_reference_rule(tb, orc, workloads, answers, engine, name):
    """The same King's subgraph branched by the reference's rule (186
    branches), and with the domination reduction too (one network): items
    equal the oracle's, max + r equals the exact MIS."""
    wl, items, res = _solve(engine, workloads, name, ("layered", "batched"))
    ans = answers[name]
    for mode, (out, mx) in res.items():
        assert list(out) == ans["items"], mode
        assert _graph_values(ans, out) == ans["graph_mis"], mode
    for k in sorted(set(np.linspace(0, len(items) - 1, 4).astype(int).tolist())):
        it = items[k]
        assert ans["items"][k] == orc.solve(it["code"], it["weights"]) + it["r"]


@pytest.mark.parametrize("name", ["rr220w_s22", "rr300w_s22"])
def test_sliced_batches(tb, orc, workloads, answers, engine, name):
    """3-regular n=220 (all 2^6 slices) and n=300 (1024 evenly spaced of its
    2^20 slices), weights U{1..10}, index-sliced to sc <= 22: every slice
    equals the oracle's value of the same slice; over all slices of n=220
    the max is the exact MWIS, over a sample of n=300 at most the MWIS."""
    wl, items, res = _solve(engine, workloads, name, ("layered", "batched"))
    ans = answers[name]
    assert [it["index"] for it in items] == ans["slice_index"]
    complete = wl["step_fraction"] == 1.0
    for mode, (out, mx) in res.items():
        assert list(out) == ans["items"], mode
        assert (mx == ans["graph_mis"][0]) if complete else (mx <= ans["graph_mis"][0])
    for k in sorted(set(np.linspace(0, len(items) - 1, 4).astype(int).tolist())):
        it = items[k]
        assert ans["items"][k] == orc.solve(it["code"], it["weights"], sliced=it["fixed"],
                                            slice_vals=it["values"])


@pytest.mark.parametrize("merge,atomic", [(False, False), (False, True), (True, True)])
def test_split_k_forms_in_a_batch(tb, workloads, answers, engine, merge, atomic):
    """The 64 slices of 3-regular n=220 share one plan whose GEMM splits K
    for one item alone: the batch fills the GPU, so by default the GEMM runs
    as one pass over the whole K.  The split form (partials and a max step,
    or atomic max into the filled output) and the merged one give the same
    values."""
    engine.set_kpart_merge(merge)
    engine.set_kpart_atomic(atomic)
    try:
        wl, items, res = _solve(engine, workloads, "rr220w_s22", ("layered", "batched"))
    finally:
        engine.set_kpart_merge(True)
        engine.set_kpart_atomic(False)
    ans = answers["rr220w_s22"]
    for mode, (out, mx) in res.items():
        assert list(out) == ans["items"], (mode, merge, atomic)
        assert mx == ans["graph_mis"][0]
