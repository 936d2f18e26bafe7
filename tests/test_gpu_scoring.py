"""tb_score_trees: complexities and peak memory of many candidate trees of
one network, one warp per tree, equal to the host cost model
(order.complexity / order.peak_memory) tree by tree."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _random_trees(tb, g, k, seed):
    rng = np.random.default_rng(seed)
    ixs, iy = tb.rawcode(g)
    codes = [tb.initialize_code(g, tb.GreedyMethod(s)) for s in range(3)]
    T = len(ixs)
    while len(codes) < k:
        live = list(range(T))
        ch = []
        nxt = T
        while len(live) > 1:
            i, j = rng.choice(len(live), 2, replace=False)
            a, b = live[i], live[j]
            live = [x for q, x in enumerate(live) if q not in (i, j)]
            ch.append((a, b))
            live.append(nxt)
            nxt += 1
        codes.append(tb.CompressedEinsum(ixs, iy, np.array(ch, np.int32), n_labels=g.n))
    return codes


@pytest.mark.parametrize("seed", range(3))
def test_scores_match_the_host_cost_model(tb, engine, seed):
    g = tb.random_regular_graph(40 + 20 * seed, 3, seed)
    codes = _random_trees(tb, g, 40, seed)
    out = engine.score_trees(codes)
    for c, row in zip(codes, out):
        tc, sc, rw = tb.complexity(c)
        assert row[1] == sc
        assert row[0] == pytest.approx(tc, abs=1e-9) and row[2] == pytest.approx(rw, abs=1e-9)
        assert row[3] == pytest.approx(tb.peak_memory(c), abs=1e-9)


def test_open_labels_and_single_tensor(tb, engine):
    g = tb.random_regular_graph(30, 3, 7)
    code = tb.initialize_code(g, tb.GreedyMethod(0))
    opened = tb.CompressedEinsum(code.ixs, [3, 11], code.children, n_labels=code.n_labels)
    row = engine.score_trees([opened])[0]
    tc, sc, rw = tb.complexity(opened)
    assert row[1] == sc and row[0] == pytest.approx(tc, abs=1e-9)
    one = tb.CompressedEinsum([[0, 1]], [], np.zeros((0, 2), np.int32), n_labels=2)
    r1 = engine.score_trees([one])[0]
    assert list(r1[:3]) == [2.0, 2.0, 2.0]
