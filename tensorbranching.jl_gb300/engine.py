"""Python handle on the C ABI of include/tb.h (ctypes).

``Engine`` owns a ``tb_ctx``; ``Plan`` owns a ``tb_plan``.  Every call goes
through the native library; there is no host fallback for the contraction.
"""
from __future__ import annotations

import ctypes
from ctypes import POINTER, c_double, c_int32, c_int64, c_void_p

import numpy as np

from . import _native
from .network import CompressedEinsum


class Plan:
    """A compiled contraction plan bound to an Engine."""

    def __init__(self, engine: "Engine", code: CompressedEinsum, sliced=(), use_node_iy: bool = True):
        self.engine = engine
        self.code = code
        self.sliced = [int(x) for x in sliced]
        lib = engine.lib
        off, lab = code.csr()
        iy = np.array(code.iy if code.iy else [0], np.int32)
        ch = code.children if code.n_nodes else np.zeros((1, 2), np.int32)
        niy_off, niy_lab = code.node_iy_csr() if use_node_iy else (None, None)
        sl = np.array(self.sliced if self.sliced else [0], np.int32)
        h = c_void_p()
        self._keep = (off, lab, iy, ch, niy_off, niy_lab, sl)
        st = lib.tb_plan_create(engine.ctx, code.n_labels, code.n_tensors, off.ctypes.data, lab.ctypes.data,
                                len(code.iy), iy.ctypes.data, code.n_nodes, ch.ctypes.data,
                                None if niy_off is None else niy_off.ctypes.data,
                                None if niy_lab is None else niy_lab.ctypes.data,
                                len(self.sliced), sl.ctypes.data, ctypes.byref(h))
        _native.check(st, engine.ctx)
        self.handle = h
        self._keep = None

    def bind_mis(self, weights) -> "Plan":
        w = np.ascontiguousarray(weights, dtype=np.float32)
        if w.shape[0] < self.code.n_labels:
            raise ValueError("one weight per label is required")
        _native.check(self.engine.lib.tb_plan_bind_mis(self.handle, w.ctypes.data), self.engine.ctx)
        return self

    def stats(self) -> dict:
        s = _native.TbPlanStats()
        _native.check(self.engine.lib.tb_plan_stats_get(self.handle, ctypes.byref(s)), self.engine.ctx)
        return {k: getattr(s, k) for k, _ in s._fields_ if k != "reserved"}

    def node_labels(self, j: int) -> list[int]:
        buf = np.zeros(64, np.int32)
        n = c_int32()
        _native.check(self.engine.lib.tb_plan_node_labels(self.handle, j, 64, buf.ctypes.data, ctypes.byref(n)),
                      self.engine.ctx)
        return buf[: n.value].tolist()

    def all_node_labels(self) -> list[list[int]]:
        return [self.node_labels(j) for j in range(self.code.n_nodes)]

    def close(self):
        if getattr(self, "handle", None):
            self.engine.lib.tb_plan_destroy(self.handle)
            self.handle = None
            self.engine._plans_closed = getattr(self.engine, "_plans_closed", 0) + 1

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Engine:
    """A tb_ctx on one CUDA device."""

    def __init__(self, device: int = 0, dtype: str = "f32", use_graphs: bool = True,
                 max_device_bytes: int = 0, timeout_ms: int = 20000, persistent_ctas: int = 0,
                 gemm_arith: str = "f32"):
        """gemm_arith "f32" (default): every contraction computes in f32 (or
        in int32 for dtype "i32"); "i16x2": GEMM tiles of plans whose weights
        are integers >= 0 summing below 8192 compute in exact packed int16
        pairs (tb_options.gemm_i16)."""
        self.lib = _native.engine_lib()
        opt = _native.TbOptions()
        self.lib.tb_options_default(ctypes.byref(opt))
        opt.dtype = {"f32": _native.TB_DTYPE_F32, "i32": _native.TB_DTYPE_I32}[dtype]
        opt.use_graphs = 1 if use_graphs else 0
        opt.max_device_bytes = int(max_device_bytes)
        opt.timeout_ms = int(timeout_ms)
        opt.persistent_ctas = int(persistent_ctas)
        opt.gemm_i16 = {"f32": 0, "i16x2": 1}[gemm_arith]
        self.dtype = dtype
        self.gemm_arith = gemm_arith
        h = c_void_p()
        _native.check(self.lib.tb_ctx_create(device, ctypes.byref(opt), ctypes.byref(h)), None)
        self.ctx = h

    def plan(self, code: CompressedEinsum, weights=None, sliced=(), use_node_iy: bool = True) -> Plan:
        p = Plan(self, code, sliced, use_node_iy)
        if weights is not None:
            p.bind_mis(weights)
        return p

    def bind_batch(self, plans, weights, offsets=None) -> None:
        """tb_plan_bind_mis for many plans in one call: weights[i] for
        plans[i], or one flat float32 array with plan i's weights at
        offsets[i]."""
        n = len(plans)
        if offsets is None:
            ws = [np.ascontiguousarray(w, dtype=np.float32) for w in weights]
            for p, w in zip(plans, ws):
                if w.shape[0] < p.code.n_labels:
                    raise ValueError("one weight per label is required")
            offs = np.zeros(n, np.int64)
            if n > 1:
                offs[1:] = np.cumsum([w.shape[0] for w in ws[:-1]])
            flat = np.concatenate(ws) if n else np.zeros(1, np.float32)
        else:
            flat = weights
            offs = offsets
            if flat.dtype != np.float32 or not flat.flags.c_contiguous or offs.dtype != np.int64 or len(offs) != n:
                raise ValueError("flat weights must be contiguous float32 with one int64 offset per plan")
        key = tuple(plans)
        cached = getattr(self, "_bind_cache", None)
        if cached is not None and cached[3] == getattr(self, "_plans_closed", 0) and cached[0] == key:
            arr, n_labels = cached[1], cached[2]
        else:
            if not all(p.handle for p in plans):
                raise ValueError("a plan of the batch is closed")
            arr = (c_void_p * max(n, 1))(*[p.handle for p in plans])
            n_labels = np.array([p.code.n_labels for p in plans], np.int64)
            self._bind_cache = (key, arr, n_labels, getattr(self, "_plans_closed", 0))
        if offsets is not None and n and (np.any(offs < 0) or np.any(offs + n_labels > flat.shape[0])):
            raise ValueError("weights out of range")
        _native.check(self.lib.tb_plan_bind_mis_batch(n, ctypes.cast(arr, c_void_p), flat.ctypes.data,
                                                      offs.ctypes.data), self.ctx)

    def _batch_args(self, plans, slice_vals, r):
        n = len(plans)
        # the handle array is kept with the plans it holds (so none of them
        # can be freed while cached) and reused when the same plans come again
        # (a closed plan invalidates every cached array)
        key = tuple(plans)
        cached = getattr(self, "_arr_cache", None)
        if cached is not None and cached[2] == getattr(self, "_plans_closed", 0) and cached[0] == key:
            arr = cached[1]
        else:
            if not all(p.handle for p in plans):
                raise ValueError("a plan of the batch is closed")
            arr = (c_void_p * n)(*[p.handle for p in plans])
            self._arr_cache = (key, arr, getattr(self, "_plans_closed", 0))
        sv = None
        if slice_vals is not None and isinstance(slice_vals, (list, tuple)) and all(len(x) == 0 for x in slice_vals):
            slice_vals = None
        if slice_vals is not None:
            sv = np.ascontiguousarray(np.concatenate([np.asarray(x, np.int8).ravel() for x in slice_vals])
                                      if isinstance(slice_vals, (list, tuple)) else
                                      np.asarray(slice_vals, np.int8).ravel(), dtype=np.int8)
            if sv.size == 0:
                sv = None
        rr = None if r is None else np.ascontiguousarray(r, dtype=np.float32)
        return n, arr, sv, rr

    def info(self) -> dict:
        """Resident CTAs of the stream-tile, GEMM-tile and persistent kernels
        on this device, and its SM count."""
        f = self.lib.tbi_ctx_info
        f.restype = c_int32
        f.argtypes = [c_void_p, c_void_p]
        out = np.zeros(4, np.int32)
        _native.check(f(self.ctx, out.ctypes.data), self.ctx)
        return {"stream_ctas": int(out[0]), "gemm_ctas": int(out[1]), "persistent_ctas": int(out[2]),
                "sms": int(out[3])}

    def set_stream_wide(self, wide: bool) -> None:
        """Per-level stream launches with 128 registers a thread and two CTAs
        per SM (True, the default) or 80 and three (False), as the autotuner
        may choose (tbi_ctx_set_stream_wide, an internal engine symbol)."""
        f = self.lib.tbi_ctx_set_stream_wide
        f.restype = c_int32
        f.argtypes = [c_void_p, c_int32]
        _native.check(f(self.ctx, 1 if wide else 0), self.ctx)

    def stream_wide(self) -> bool:
        """Whether the per-level launches run the 128-register stream form
        (k_level<T, 5>) rather than the 80-register one (k_level<T, 1>)
        (tbi_ctx_stream_wide, an internal engine symbol)."""
        f = self.lib.tbi_ctx_stream_wide
        f.restype = c_int32
        f.argtypes = [c_void_p]
        v = f(self.ctx)
        if v < 0:
            _native.check(v, self.ctx)
        return bool(v)

    def set_kpart_atomic(self, atomic: bool) -> None:
        """Split-K GEMM parts by atomic max into the output where every value
        is >= 0 or -inf (True) or through partials and a max step (False), as
        the autotuner may choose (tbi_ctx_set_kpart_atomic, an internal engine
        symbol)."""
        f = self.lib.tbi_ctx_set_kpart_atomic
        f.restype = c_int32
        f.argtypes = [c_void_p, c_int32]
        _native.check(f(self.ctx, 1 if atomic else 0), self.ctx)

    def set_kpart_merge(self, merge: bool) -> None:
        """Split-K GEMMs of batches whose items fill the GPU without the
        split run as one pass over the whole K (True, the default) or always
        as the plan split them (False) (tbi_ctx_set_kpart_merge, an internal
        engine symbol)."""
        f = self.lib.tbi_ctx_set_kpart_merge
        f.restype = c_int32
        f.argtypes = [c_void_p, c_int32]
        _native.check(f(self.ctx, 1 if merge else 0), self.ctx)

    def retile(self, plan: "Plan", bits: int) -> None:
        """Re-plan a plan's stream tiles for up to 2^bits outputs (8..11), as
        the autotuner does (tbi_plan_retile, an internal engine symbol)."""
        f = self.lib.tbi_plan_retile
        f.restype = c_int32
        f.argtypes = [c_void_p, c_int32]
        _native.check(f(plan.handle, int(bits)), self.ctx)

    def score_trees(self, codes) -> np.ndarray:
        """tb_score_trees: (tc, sc, rwc, log2 peak memory) of each tree; the
        codes share leaves and open labels and differ in their trees."""
        c0 = codes[0]
        off, lab = c0.csr()
        iy = np.array(c0.iy if c0.iy else [0], np.int32)
        nodes = c0.n_tensors - 1
        for c in codes:
            if c.ixs != c0.ixs or c.iy != c0.iy:
                raise ValueError("trees of one network only")
        ch = np.ascontiguousarray(np.stack([c.children for c in codes]).reshape(-1) if nodes else
                                  np.zeros(1, np.int32), dtype=np.int32)
        out = np.zeros((len(codes), 4), np.float64)
        st = self.lib.tb_score_trees(self.ctx, c0.n_labels, c0.n_tensors, off.ctypes.data, lab.ctypes.data,
                                     len(c0.iy), iy.ctypes.data, len(codes), ch.ctypes.data, out.ctypes.data)
        _native.check(st, self.ctx)
        return out

    def autotune(self, plans, slice_vals=None, r=None) -> dict:
        """tb_autotune on this batch: tile size and schedule by timing; the
        choice serves later mode="auto" solves."""
        n, arr, sv, rr = self._batch_args(plans, slice_vals, r)
        res = _native.TbTuneResult()
        st = self.lib.tb_autotune(self.ctx, n, ctypes.cast(arr, c_void_p), None if sv is None else sv.ctypes.data,
                                  None if rr is None else rr.ctypes.data, ctypes.byref(res))
        _native.check(st, self.ctx)
        names = {v: k for k, v in _native.MODES.items()}
        return {"mode": names[res.mode], "tile_bits": res.tile_bits, "ctas_per_sm": res.ctas_per_sm,
                "chunk_div": res.chunk_div, "stream_ctas_per_sm": res.stream_ctas_per_sm,
                "kpart_atomic": bool(res.kpart_atomic), "ms": res.ms,
                "ms_default": res.ms_default, "n_tried": res.n_tried}

    def solve_batch(self, plans, slice_vals=None, r=None, mode: str = "batched"):
        """Per-item results (max root + r) and their max."""
        n, arr, sv, rr = self._batch_args(plans, slice_vals, r)
        out = np.zeros(n, np.float32)
        mx = np.zeros(1, np.float32)
        st = self.lib.tb_solve_batch(self.ctx, n, ctypes.cast(arr, c_void_p),
                                     None if sv is None else sv.ctypes.data,
                                     None if rr is None else rr.ctypes.data, out.ctypes.data, mx.ctypes.data,
                                     _native.MODES[mode])
        _native.check(st, self.ctx)
        return out, float(mx[0])

    def contract(self, plan: Plan, tensors, mode: str = "layered") -> np.ndarray:
        """Contract with explicit leaf tensors (column-major, -inf = zero)."""
        bufs = [np.ascontiguousarray(np.asarray(t, np.float32).ravel(order="F")) for t in tensors]
        for ix, b in zip(plan.code.ixs, bufs):
            if b.size != 1 << len(ix):
                raise ValueError("leaf tensor size does not match its labels")
        ptrs = (c_void_p * len(bufs))(*[b.ctypes.data for b in bufs])
        out = np.zeros(1 << len(plan.code.iy), np.float32)
        st = self.lib.tb_contract(self.ctx, plan.handle, ctypes.cast(ptrs, c_void_p), out.ctypes.data,
                                  _native.MODES[mode])
        _native.check(st, self.ctx)
        return out

    def dump(self, plan: Plan, slice_vals=None, mode: str = "layered") -> list[np.ndarray]:
        labs = plan.all_node_labels()
        outs = [np.zeros(1 << len(l), np.float32) for l in labs]
        ptrs = (c_void_p * max(len(outs), 1))(*[o.ctypes.data for o in outs])
        sv = None if slice_vals is None else np.ascontiguousarray(slice_vals, dtype=np.int8)
        st = self.lib.tb_dump_intermediates(self.ctx, plan.handle, None if sv is None else sv.ctypes.data,
                                            ctypes.cast(ptrs, c_void_p), _native.MODES[mode])
        _native.check(st, self.ctx)
        return outs

    def profile_levels(self, plans, slice_vals=None, r=None) -> list[dict]:
        """Per launch of the per-level schedule of this batch (run without a
        graph, a CUDA event after each launch; tbi_profile_levels, an internal
        engine symbol): device ms, kind ("stream" tiles with leaves and final
        steps, or "gemm" tiles) and the algorithmic ops and bytes it runs."""
        f = self.lib.tbi_profile_levels
        f.restype = c_int32
        f.argtypes = [c_void_p, c_int32, c_void_p, c_void_p, c_void_p, c_int32, c_void_p, c_void_p, c_void_p,
                      c_void_p, POINTER(c_int32)]
        n, arr, sv, rr = self._batch_args(plans, slice_vals, r)
        cap = 4096
        ms = np.zeros(cap)
        kinds = np.zeros(cap, np.int32)
        ops = np.zeros(cap)
        byts = np.zeros(cap)
        nout = c_int32()
        st = f(self.ctx, n, ctypes.cast(arr, c_void_p), None if sv is None else sv.ctypes.data,
               None if rr is None else rr.ctypes.data, cap, ms.ctypes.data, kinds.ctypes.data, ops.ctypes.data,
               byts.ctypes.data, ctypes.byref(nout))
        _native.check(st, self.ctx)
        return [{"ms": float(ms[k]), "kind": "gemm" if kinds[k] == 2 else "stream", "ops": float(ops[k]),
                 "bytes": float(byts[k])} for k in range(nout.value)]

    def last_timing(self) -> tuple[float, int]:
        ms = c_double()
        n = c_int64()
        _native.check(self.lib.tb_last_timing(self.ctx, ctypes.byref(ms), ctypes.byref(n)), self.ctx)
        return ms.value, n.value

    def gemm(self, M, N, K, batch, A_ptr, B_ptr, C_ptr, stream_ptr=None):
        st = self.lib.tb_gemm_device(self.ctx, M, N, K, batch, A_ptr, B_ptr, C_ptr, stream_ptr)
        _native.check(st, self.ctx)

    def close(self):
        if getattr(self, "ctx", None):
            # cached handle arrays hold plans; drop them with the context
            self._arr_cache = None
            self._bind_cache = None
            self.lib.tb_ctx_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default: Engine | None = None


def measure_maxplus_peak(device: int = 0) -> float:
    """Measured f32 SIMT max-plus rate of this GPU in ops/s (max and add
    counted as two ops): a loop-carried add.f32x2 + 3-input max.f32 probe
    over every SM (tbi_measure_maxplus_peak, an internal engine symbol)."""
    lib = _native.engine_lib()
    f = lib.tbi_measure_maxplus_peak
    f.restype = c_int32
    f.argtypes = [c_int32, POINTER(c_double)]
    v = c_double()
    _native.check(f(int(device), ctypes.byref(v)))
    return float(v.value)


def measure_maxplus_peak_i16(device: int = 0) -> float:
    """Measured packed-int16 max-plus rate in ops/s (__viaddmax_s16x2, two
    tropical MACs per instruction), the ceiling of the int16 GEMM tiles."""
    lib = _native.engine_lib()
    f = lib.tbi_measure_maxplus_peak_i16
    f.restype = c_int32
    f.argtypes = [c_int32, POINTER(c_double)]
    v = c_double()
    _native.check(f(int(device), ctypes.byref(v)))
    return float(v.value)


def plan_node_kinds(plan: "Plan") -> np.ndarray:
    """Per node: 2 = stream tiles, 3 = GEMM tiles in the fused form."""
    lib = _native.engine_lib()
    f = lib.tbi_plan_node_kinds
    f.restype = c_int32
    f.argtypes = [c_void_p, c_void_p]
    out = np.zeros(max(plan.code.n_nodes, 1), np.int32)
    _native.check(f(plan.handle, out.ctypes.data))
    return out[: plan.code.n_nodes]


def default_engine() -> Engine:
    global _default
    if _default is None:
        _default = Engine()
    return _default
