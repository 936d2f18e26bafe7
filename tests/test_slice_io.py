"""The reference's on-disk slice format (src/io.jl): round trips of graphs,
weights and plans (as test/io.jl:9-38), a plan file in OMEinsum's nested
layout written by hand, and a directory of finished slices whose contracted
max + r equals the MIS of the graph they came from."""
import json
import os

import numpy as np
import pytest

from cases import rr_case


def test_round_trips(tb, orc, tmp_path):
    sio = tb.slice_io
    g, w, code = rr_case(tb, 24, 5)
    sio.savegraph(str(tmp_path / "g.dot"), g)
    g2 = sio.loadgraph(str(tmp_path / "g.dot"))
    assert g2.n == g.n and sorted(g2.edges) == sorted(g.edges)
    for weights in (tb.UnitWeight(g.n), w.astype(np.float32), w.astype(np.float64), w.astype(np.int64)):
        sio.save_weights(str(tmp_path / "w.txt"), weights)
        back = sio.load_weights(str(tmp_path / "w.txt"))
        if isinstance(weights, tb.UnitWeight):
            assert back == weights
        else:
            assert back.dtype == weights.dtype and np.array_equal(back, weights)
    sio.save_code(str(tmp_path / "c.json"), code)
    c2 = sio.load_code(str(tmp_path / "c.json"))
    assert c2.ixs == code.ixs and np.array_equal(c2.children, code.children)
    assert orc.solve(c2, w) == orc.solve(code, w)
    sio.save_code(str(tmp_path / "n.json"), None)
    assert sio.load_code(str(tmp_path / "n.json")) is None


def test_hand_written_nested_einsum_and_dot(tb, orc, tmp_path):
    """A path graph 1-2-3 with the plan ((v1, e12), (v2, (e23, v3))) written
    in OMEinsum's nested layout, 1-based, with an n-ary root."""
    d = {"label-type": "Int64", "inputs": [[1], [2], [3], [1, 2], [2, 3]], "output": [],
         "tree": {"isleaf": False, "eins": {"ixs": [[2], [2], [2]], "iy": []},
                  "args": [{"isleaf": False, "eins": {"ixs": [[1], [1, 2]], "iy": [2]},
                            "args": [{"isleaf": True, "tensorindex": 1}, {"isleaf": True, "tensorindex": 4}]},
                           {"isleaf": True, "tensorindex": 2},
                           {"isleaf": False, "eins": {"ixs": [[2, 3], [3]], "iy": [2]},
                            "args": [{"isleaf": True, "tensorindex": 5}, {"isleaf": True, "tensorindex": 3}]}]}}
    (tmp_path / "c.json").write_text(json.dumps(d))
    code = tb.slice_io.load_code(str(tmp_path / "c.json"))
    assert code.n_tensors == 5 and code.n_nodes == 4
    w = np.array([2.0, 3.0, 2.0], np.float32)
    assert orc.solve(code, w) == 4.0
    (tmp_path / "g.dot").write_text('graph G {\n  node [shape=circle];\n  1 -- 2;\n  2 -- 3;\n}\n')
    g = tb.slice_io.loadgraph(str(tmp_path / "g.dot"))
    assert g.n == 3 and sorted(g.edges) == [(0, 1), (1, 2)]


@pytest.mark.parametrize("seed", [0, 1])
def test_finished_slices_directory(tb, orc, exact, tmp_path, seed):
    sio = tb.slice_io
    g = tb.random_regular_graph(50, 3, seed)
    w = tb.random_weights(g.n, seed)
    kr = tb.kernelize(g, w)
    code = tb.initialize_code(kr.g, tb.GreedyMethod(seed))
    branches = tb.slice(tb.MISProblem(kr.g, kr.weights), code, kr.r,
                        tb.ContractionTreeSlicer(sc_target=6, refine=False))
    rows = []
    for i, b in enumerate(branches):
        sio.save_finished(str(tmp_path), b, 1000 + i)
        rows.append((1000 + i, b.sc(), b.tc(), b.r))
    sio.save_slices_csv(str(tmp_path), rows)
    back = sio.load_all_finished(str(tmp_path))
    assert len(back) == len(branches)
    vals = [b.r if b.code is None or b.p.g.n == 0 else orc.solve(b.code, b.p.weight_array()) + b.r for b in back]
    assert max(vals) == pytest.approx(exact.branch_and_bound(g.n, g.edges, w))
