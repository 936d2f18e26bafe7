"""Failure detection without a GPU fault: the persistent executor's waits
are bounded.  A chunk list that omits every producer of the final step makes
its wait run out; the kernel sets the error word and returns, the host
reports TB_ERR_TIMEOUT, and the same context then solves correctly."""
import ctypes

import numpy as np
import pytest

from cases import rr_case

pytestmark = pytest.mark.gpu


def test_bounded_wait_times_out_and_context_survives(tb, orc, native):
    g, w, code = rr_case(tb, 40, 2)
    ref = orc.solve(code, w)
    eng = tb.Engine()
    try:
        plan = eng.plan(code, w)
        lib = eng.lib
        lib.tbi_timeout_probe.restype = ctypes.c_int32
        lib.tbi_timeout_probe.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32]
        st = lib.tbi_timeout_probe(eng.ctx, plan.handle, 50)
        assert st == native.TB_ERR_TIMEOUT
        assert b"timed out" in lib.tb_last_error(eng.ctx)
        for mode in ("batched", "layered", "plain"):
            out, mx = eng.solve_batch([plan], mode=mode)
            assert mx == np.float32(ref), mode
    finally:
        eng.close()


def test_host_side_errors_are_status_codes(tb, native):
    """Malformed requests come back as status codes with a message."""
    g, w, code = rr_case(tb, 20, 1)
    eng = tb.Engine()
    try:
        bad = tb.CompressedEinsum(code.ixs, [], code.children[::-1].copy(), n_labels=code.n_labels)
        with pytest.raises(native.TbError) as e:
            eng.plan(bad, w)
        assert e.value.status == native.TB_ERR_INVALID
        plan = eng.plan(code)  # no weights bound
        with pytest.raises(native.TbError) as e:
            eng.solve_batch([plan])
        assert e.value.status == native.TB_ERR_INVALID and "weights" in str(e.value)
        sliced = eng.plan(code, w, sliced=[0])
        with pytest.raises(native.TbError) as e:
            eng.solve_batch([sliced], slice_vals=[np.array([2], np.int8)])
        assert e.value.status == native.TB_ERR_INVALID
    finally:
        eng.close()


def test_plans_outliving_their_context(tb):
    """Destroying a context before its plans leaves the plans destroyable
    (and refused by everything else), in any order the garbage collector
    picks."""
    import numpy as np

    eng = tb.Engine()
    g = tb.random_regular_graph(20, 3, 1)
    code = tb.initialize_code(g, tb.GreedyMethod(1))
    plans = [eng.plan(code, np.ones(g.n, np.float32)) for _ in range(3)]
    eng.solve_batch(plans, mode="fused")
    eng.close()
    with pytest.raises(tb._native.TbError):
        tb._native.check(eng.lib.tb_plan_bind_mis(plans[0].handle, np.ones(g.n, np.float32).ctypes.data), None)
    for p in plans:
        p.close()
