"""Continuous-batching server: every request's result is the same served
alone (tb_solve_batch) and in the mix, and equals the exact MIS."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_results_same_alone_and_in_mix(tb, orc, exact):
    from tensorbranching_gb300 import serving

    eng = tb.Engine()
    mix = []
    rng = np.random.default_rng(3)
    for i in range(10):
        if i % 2 == 0:
            g = tb.random_regular_graph(int(rng.integers(30, 61)) * 2, 3, 100 + i)
        else:
            g = tb.random_ksg(int(rng.integers(8, 13)), 0.8, 100 + i)
        w = tb.random_weights(g.n, i) if i % 3 == 0 else np.ones(g.n, np.float32)
        mix.append((g, w))
    preps = [serving.prepare(eng, g, w, sc_cap=12.0, seed=i) for i, (g, w) in enumerate(mix)]
    assert any(p.n_items > 1 for p in preps), "some requests must be sliced into several items"
    alone = []
    for p in preps:
        if p.constant is not None:
            alone.append(p.constant)
            continue
        _, mx = eng.solve_batch(p.plans, slice_vals=p.slice_vals, r=np.array(p.r, np.float32), mode="batched")
        alone.append(mx)
    for (g, w), v in zip(mix, alone):
        assert v == exact.ip(g.n, g.edges, w)
    srv_eng = tb.Engine()
    # plans belong to the context they were made on: prepare again there
    preps2 = [serving.prepare(srv_eng, g, w, sc_cap=12.0, seed=i) for i, (g, w) in enumerate(mix)]
    with serving.Server(srv_eng, pool_bytes=1 << 30, max_items=64) as srv:
        out = serving.run_poisson(srv, preps2, rate=2000.0, seed=1)
        st = srv.stats()
    assert out["values"] == alone
    assert st["completed"] == sum(1 for p in preps2 if p.constant is None)
    assert all(l >= 0 for l in out["latency_ms"])
