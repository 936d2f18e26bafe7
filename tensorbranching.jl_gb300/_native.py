"""ctypes bindings to the native libraries (engine ``libtb.so`` and host
order tools ``libtborder.so``).  Loading fails loudly when a library is
missing: there is no Python fallback for the contraction."""
from __future__ import annotations

import ctypes
import os
from ctypes import POINTER, c_char_p, c_double, c_float, c_int8, c_int32, c_int64, c_uint64, c_void_p

from . import build as _build

TB_OK = 0
TB_ERR_INVALID = 1
TB_ERR_OOM = 2
TB_ERR_TIMEOUT = 3
TB_ERR_CUDA = 4
TB_ERR_UNSUPPORTED = 5
TB_ERR_BUSY = 6

TB_DTYPE_F32 = 0
TB_DTYPE_I32 = 1

TB_MODE_PLAIN = 0
TB_MODE_BATCHED = 1
TB_MODE_LAYERED = 2
TB_MODE_AUTO = 3
TB_MODE_FUSED = 4

MODES = {"plain": TB_MODE_PLAIN, "batched": TB_MODE_BATCHED, "layered": TB_MODE_LAYERED, "auto": TB_MODE_AUTO,
         "fused": TB_MODE_FUSED}


class TbOptions(ctypes.Structure):
    _fields_ = [
        ("dtype", c_int32),
        ("use_graphs", c_int32),
        ("max_device_bytes", c_int64),
        ("timeout_ms", c_int32),
        ("autotune", c_int32),
        ("persistent_ctas", c_int32),
        ("gemm_i16", c_int32),
        ("reserved", c_int32 * 8),
    ]


class TbPlanStats(ctypes.Structure):
    _fields_ = [
        ("tc", c_double),
        ("sc", c_double),
        ("rwc", c_double),
        ("ops", c_double),
        ("bytes", c_double),
        ("arena_bytes", c_int64),
        ("n_steps", c_int32),
        ("n_tensors", c_int32),
        ("n_open", c_int32),
        ("n_sliced", c_int32),
        ("n_tiles", c_int32),
        ("small_words", c_int32),
        ("reserved", c_int32 * 6),
    ]


class TbTuneResult(ctypes.Structure):
    _fields_ = [
        ("mode", c_int32),
        ("tile_bits", c_int32),
        ("ctas_per_sm", c_int32),
        ("chunk_div", c_int32),
        ("ms", c_double),
        ("ms_default", c_double),
        ("n_tried", c_int32),
        ("stream_ctas_per_sm", c_int32),
        ("kpart_atomic", c_int32),
        ("reserved", c_int32 * 5),
    ]


class TbError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"tb status {status}: {msg}")
        self.status = status


# every symbol include/tb.h declares, with its ctypes signature
ENGINE_SIGNATURES = {
    "tb_options_default": (None, [POINTER(TbOptions)]),
    "tb_ctx_create": (c_int32, [c_int32, POINTER(TbOptions), POINTER(c_void_p)]),
    "tb_ctx_destroy": (None, [c_void_p]),
    "tb_last_error": (c_char_p, [c_void_p]),
    "tb_version": (c_char_p, []),
    "tb_plan_create": (c_int32, [c_void_p, c_int32, c_int32, c_void_p, c_void_p, c_int32, c_void_p, c_int32,
                                 c_void_p, c_void_p, c_void_p, c_int32, c_void_p, POINTER(c_void_p)]),
    "tb_plan_destroy": (None, [c_void_p]),
    "tb_plan_stats_get": (c_int32, [c_void_p, POINTER(TbPlanStats)]),
    "tb_plan_node_labels": (c_int32, [c_void_p, c_int32, c_int32, c_void_p, POINTER(c_int32)]),
    "tb_plan_bind_mis": (c_int32, [c_void_p, c_void_p]),
    "tb_plan_bind_mis_batch": (c_int32, [c_int32, c_void_p, c_void_p, c_void_p]),
    "tb_solve_batch": (c_int32, [c_void_p, c_int32, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_int32]),
    "tb_contract": (c_int32, [c_void_p, c_void_p, c_void_p, c_void_p, c_int32]),
    "tb_dump_intermediates": (c_int32, [c_void_p, c_void_p, c_void_p, c_void_p, c_int32]),
    "tb_last_timing": (c_int32, [c_void_p, POINTER(c_double), POINTER(c_int64)]),
    "tb_gemm_device": (c_int32, [c_void_p, c_int64, c_int64, c_int64, c_int64, c_void_p, c_void_p, c_void_p,
                                 c_void_p]),
    "tb_solve_static": (c_int32, [c_int32, c_int32, c_void_p, c_void_p, c_int32, c_void_p, c_void_p, c_void_p,
                                  c_void_p]),
    "tb_autotune": (c_int32, [c_void_p, c_int32, c_void_p, c_void_p, c_void_p, POINTER(TbTuneResult)]),
    "tb_score_trees": (c_int32, [c_void_p, c_int32, c_int32, c_void_p, c_void_p, c_int32, c_void_p, c_int32,
                                 c_void_p, c_void_p]),
    "tb_serve_start": (c_int32, [c_void_p, c_int64, c_int32]),
    "tb_serve_stop": (c_int32, [c_void_p]),
    "tb_submit": (c_int32, [c_void_p, c_int32, c_void_p, c_void_p, c_void_p, POINTER(c_void_p)]),
    "tb_poll": (c_int32, [c_void_p, POINTER(c_int32)]),
    "tb_wait": (c_int32, [c_void_p, c_int32, POINTER(c_float), POINTER(c_double)]),
    "tb_request_free": (None, [c_void_p]),
    "tb_serve_stats": (c_int32, [c_void_p, POINTER(c_int64), POINTER(c_int64), POINTER(c_int64), POINTER(c_int64)]),
}

ORDER_SIGNATURES = {
    "tbo_complexity": (c_int32, [c_int32, c_void_p, c_void_p, c_int32, c_int32, c_void_p, c_void_p, c_void_p]),
    "tbo_node_labels": (c_int32, [c_int32, c_void_p, c_void_p, c_int32, c_int32, c_void_p, c_void_p, c_void_p]),
    "tbo_peak_memory": (c_int32, [c_int32, c_void_p, c_void_p, c_int32, c_int32, c_void_p, c_void_p, c_void_p]),
    "tbo_minfill_order": (c_int32, [c_int32, c_void_p, c_void_p, c_int32, c_uint64, c_void_p]),
    "tbo_tree_from_order": (c_int32, [c_int32, c_void_p, c_void_p, c_int32, c_int32, c_void_p, c_int32, c_void_p,
                                      c_void_p]),
    "tbo_treesa": (c_int32, [c_int32, c_void_p, c_void_p, c_int32, c_int32, c_void_p, c_void_p, c_double, c_double,
                             c_double, c_void_p, c_int32, c_int32, c_int32, c_int32, c_uint64, c_void_p]),
    "tbo_greedy_tree": (c_int32, [c_int32, c_void_p, c_void_p, c_int32, c_int32, c_void_p, c_uint64, c_void_p]),
    "tbo_greedy_slice": (c_int32, [c_int32, c_void_p, c_void_p, c_int32, c_int32, c_void_p, c_void_p, c_double,
                                   c_int32, c_void_p, c_void_p, c_void_p]),
}

_engine = None
_order = None


def _bind(lib, sigs):
    for name, (res, args) in sigs.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    return lib


def engine_lib(build: bool = True):
    """The CUDA engine.  Builds it when missing; raises if it cannot."""
    global _engine
    if _engine is None:
        path = _build.build_engine() if build else _build.engine_path()
        if not os.path.exists(path):
            raise RuntimeError(f"CUDA engine library missing: {path}")
        _engine = _bind(ctypes.CDLL(path), ENGINE_SIGNATURES)
    return _engine


def order_lib(build: bool = True):
    global _order
    if _order is None:
        path = _build.build_order() if build else _build.order_path()
        if not os.path.exists(path):
            raise RuntimeError(f"order library missing: {path}")
        _order = _bind(ctypes.CDLL(path), ORDER_SIGNATURES)
    return _order


def check(status: int, ctx=None) -> None:
    if status != TB_OK:
        lib = engine_lib(build=False)
        msg = lib.tb_last_error(ctx).decode(errors="replace")
        raise TbError(status, msg)
