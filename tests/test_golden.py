"""Known-answer MIS values (tests/golden/mis_known.json, written by
tests/golden/make_golden.py): structural answers for named graphs and
exhaustive-enumeration answers for small seeded graphs.  They pin the
oracle's tensor-network contraction, the exact solvers and the generators."""
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CASES = json.load(open(os.path.join(HERE, "golden", "mis_known.json")))["cases"]


def _graph(tb, c):
    g = tb.Graph(c["n"], [tuple(e) for e in c["edges"]])
    w = np.ones(c["n"], np.float32) if c["weights"] is None else np.array(c["weights"], np.float32)
    return g, w


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_oracle_contraction_matches_known_answer(tb, orc, exact, case):
    g, w = _graph(tb, case)
    code = tb.initialize_code(g, tb.GreedyMethod(0))
    assert orc.solve(code, w) == np.float32(case["mis"])
    assert exact.branch_and_bound(g.n, g.edges, w) == pytest.approx(case["mis"])


def test_generators_reproduce_the_stored_graphs(tb):
    for c in CASES:
        name = c["name"]
        if name.startswith("rr"):
            n, seed = name[2:].split("_s")
            g = tb.random_regular_graph(int(n), 3, int(seed))
        elif name.startswith("ksg5"):
            g = tb.random_ksg(5, 0.8, int(name.split("_s")[1]))
        else:
            continue
        assert g.n == c["n"] and [list(e) for e in g.edges] == c["edges"], name
