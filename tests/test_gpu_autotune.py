"""tb_autotune: every configuration it times gives the oracle's results, and
TB_MODE_AUTO afterwards runs the chosen tiles and schedule bit-exactly."""
import numpy as np
import pytest

from cases import ksg_case, rr_case

pytestmark = pytest.mark.gpu


def _batch(tb, orc):
    plans, svs, rs, refs = [], [], [], []
    eng = tb.Engine()
    g, w, code = rr_case(tb, 70, 5)
    sliced = [3, 17]
    p = eng.plan(code, w, sliced=sliced)
    for a in (0, 1):
        for b in (0, 1):
            plans.append(p)
            svs.append(np.array([a, b], np.int8))
            rs.append(1.0 * a)
            refs.append(orc.solve(code, w, sliced=sliced, slice_vals=(a, b)) + 1.0 * a)
    for seed in range(6):
        g, w, code = ksg_case(tb, 5 + seed % 3, seed) if seed % 2 else rr_case(tb, 30 + 4 * seed, seed)
        plans.append(eng.plan(code, w))
        svs.append(np.zeros(0, np.int8))
        rs.append(float(seed))
        refs.append(orc.solve(code, w) + float(seed))
    return eng, plans, svs, np.array(rs, np.float32), np.array(refs, np.float32)


def test_autotune_then_auto_mode(tb, orc):
    eng, plans, svs, rs, refs = _batch(tb, orc)
    try:
        res = eng.autotune(plans, slice_vals=svs, r=rs)
        assert res["mode"] in ("batched", "layered", "fused")
        assert 8 <= res["tile_bits"] <= 11
        assert res["ctas_per_sm"] >= 1 and res["chunk_div"] in (1, 4, 16)
        assert res["n_tried"] >= 5 and 0 < res["ms"] <= res["ms_default"]
        for mode in ("auto", "batched", "layered", "plain"):
            out, mx = eng.solve_batch(plans, slice_vals=svs, r=rs, mode=mode)
            assert np.array_equal(out, refs), mode
            assert mx == refs.max()
    finally:
        eng.close()


def test_auto_mode_tunes_on_first_use(tb, orc):
    eng, plans, svs, rs, refs = _batch(tb, orc)
    try:
        out, mx = eng.solve_batch(plans, slice_vals=svs, r=rs, mode="auto")
        assert np.array_equal(out, refs)
        out2, _ = eng.solve_batch(plans, slice_vals=svs, r=rs, mode="auto")
        assert np.array_equal(out2, refs)
    finally:
        eng.close()
