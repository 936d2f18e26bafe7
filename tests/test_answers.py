"""The stored oracle answers of the benchmark workloads
(tests/golden/workload_answers.json) against the exact MIS solvers, on the
CPU: per graph, the max over its items and its empty branches (each + r)
equals the exact MIS (test/dynamic_ob.jl:20,38,51, test/slice.jl:32-33); for
the sampled slices of an index-sliced workload it is at most the MIS.  The
item lists match the workloads' step items."""
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def answers():
    with open(os.path.join(HERE, "golden", "workload_answers.json")) as f:
        return json.load(f)


def _graph_values(ans):
    vals = [-np.inf] * len(ans["graph_mis"])
    for g, v in zip(ans["graph_of_item"], ans["items"]):
        vals[g] = max(vals[g], v)
    for g, r in enumerate(ans["graph_empty_r"]):
        if r is not None:
            vals[g] = max(vals[g], r)
    return vals


def test_every_workload_has_answers(tb, answers):
    from tensorbranching_gb300 import workloads

    for name in workloads.BUILDERS:
        assert name in answers, name


def test_complete_slice_sets_give_the_mis(answers):
    """rr220w_s22's step covers all 2^6 slices: their max is the MWIS."""
    ans = answers["rr220w_s22"]
    assert len(ans["items"]) == 64 and max(ans["items"]) == ans["graph_mis"][0]


def test_items_explain_the_exact_mis(answers):
    for name, ans in answers.items():
        vals = _graph_values(ans)
        if ans["sliced"] and len(ans["items"]) < (1 << 30):
            assert all(v <= m for v, m in zip(vals, ans["graph_mis"])), name
        else:
            assert vals == ans["graph_mis"], name


@pytest.mark.parametrize("name", ["rr220", "rr100_ob10", "rr220w_s22", "rr300w_s22", "ksg32_dom20"])
def test_items_are_the_step_items(tb, answers, name):
    from tensorbranching_gb300 import workloads

    wl = workloads.load(name)
    items = workloads.step_items(wl)
    ans = answers[name]
    assert len(items) == len(ans["items"])
    assert [it["index"] for it in items] == ans["slice_index"]


def test_exact_mis_recomputed(tb, exact, answers):
    """The stored MIS of rr220 and of four rr100 graphs, recomputed by the
    integer program and by branch and bound."""
    from tensorbranching_gb300 import workloads

    g = tb.random_regular_graph(220, 3, 1)
    assert exact.ip(g.n, g.edges) == answers["rr220"]["graph_mis"][0] == 99.0
    for s in (1, 7, 19, 32):
        g = tb.random_regular_graph(100, 3, s)
        m = answers["rr100_ob10"]["graph_mis"][s - 1]
        assert exact.branch_and_bound(g.n, g.edges) == m == answers["rr100_b10"]["graph_mis"][s - 1]
