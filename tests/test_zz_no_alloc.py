"""tb_solve_static: the entry point for callers that cannot allocate device
memory (it keeps its scratch in a fixed __device__ array).  Its MIS values
must equal tb_solve_batch's exactly, on two calls in a row, and networks
larger than its fixed scratch must be refused with a clear error."""
import ctypes

import numpy as np
import pytest

from cases import rr_case

pytestmark = pytest.mark.gpu


def _solve_static(native, code, w):
    lib = native.engine_lib()
    off, lab = code.csr()
    ch = code.children if code.n_nodes else np.zeros((1, 2), np.int32)
    wv = np.ascontiguousarray(w, np.float32)
    out = ctypes.c_float(np.nan)
    st = lib.tb_solve_static(code.n_labels, code.n_tensors, off.ctypes.data, lab.ctypes.data, code.n_nodes,
                             ch.ctypes.data, wv.ctypes.data, ctypes.byref(out), None)
    return st, out.value, lib.tb_last_error(None).decode()


def test_static_matches_solve_batch_twice(tb, orc, native, engine):
    # rr100 seed 3 has stream tiles that need more than 48 KiB of shared memory
    cases = [rr_case(tb, 60, 1), rr_case(tb, 44, 2, weighted=False), rr_case(tb, 100, 3)]
    for g, w, code in cases:  # two calls in a row, different networks
        st, v, msg = _solve_static(native, code, w)
        assert st == 0, msg
        _, ref = engine.solve_batch([engine.plan(code, w)], mode="plain")
        assert v == ref == orc.solve(code, w)
    # and the first network again, after the second one left its data behind
    g, w, code = cases[0]
    st, v, msg = _solve_static(native, code, w)
    assert st == 0, msg
    _, ref = engine.solve_batch([engine.plan(code, w)], mode="batched")
    assert v == ref


def test_static_refuses_oversized_network(tb, native):
    g = tb.random_regular_graph(80, 3, 5)
    code = tb.initialize_code(g, tb.GreedyMethod(0))
    # a bad order: one tensor holding every label -> far beyond 64 MiB
    T = code.n_tensors
    ch = np.array([(0, 1)] + [(T + j, j + 2) for j in range(T - 2)], np.int32)
    big = tb.CompressedEinsum(code.ixs, [], ch, n_labels=code.n_labels)
    st, v, msg = _solve_static(native, big, np.ones(g.n, np.float32))
    assert st != 0
    assert "scratch" in msg or "rank" in msg
