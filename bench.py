"""Benchmark: MIS solves/s of the tropical contraction on GB300.

Default workload: ``rr220`` -- one random 3-regular graph, n=220, unit
weights, contracted in one piece with no slicing (a step = one full MIS solve
= one contraction of the whole network).  Other workloads: ``--config``.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--config rr220|rr100_b10|rr100_ob10|rr220w_s22|ksg32_b20|serve] [--mode batched|layered|plain]
    python bench.py --make rr220 ...     # (re)build workload fixtures

Under torchrun each rank runs its own replica of the workload on its own GPU
(independent units, no collective on the data path): scaling is weak and
``value`` is the units of all ranks over the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
import __graft_entry__ as _ge  # noqa: E402

METRIC = "MIS solves/s"


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


def _node_work(plan, cache={}):
    """Per-node (ops, bytes) of a plan as the engine runs it (sliced labels
    removed): ops = 2 * 2^|ix1 u ix2|, bytes = 4 (2^|ix1| + 2^|ix2| + 2^|iy|)."""
    key = id(plan)
    if key in cache:
        return cache[key]
    code = plan.code.remove_labels(plan.sliced) if plan.sliced else plan.code
    labs = [list(dict.fromkeys(ix)) for ix in code.ixs] + code.labels_of_nodes()
    T = code.n_tensors
    ops, byts = [], []
    for j, (a, b) in enumerate(code.children):
        la, lb, ly = labs[int(a)], labs[int(b)], labs[T + j]
        ops.append(2.0 * 2.0 ** len(set(la) | set(lb) | set(ly)))
        byts.append(4.0 * (2.0 ** len(la) + 2.0 ** len(lb) + 2.0 ** len(ly)))
    cache[key] = (np.array(ops), np.array(byts))
    return cache[key]


def roofline(plans, seconds, simt_ops_s, hbm_gbs, i16_ops_s=None):
    """Node-weighted roofline of one step: every node is bounded by
    max(ops / P, bytes / BW_hbm), P the f32 SIMT max-plus peak, or the
    packed-int16 one for GEMM-tile nodes running that form; the step's bound
    is the sum."""
    from tensorbranching_gb300.engine import plan_node_kinds

    ops = byts = t_simt = t_hbm = t_bound = 0.0
    kinds_of = {}
    for p in plans:
        o, b = _node_work(p)
        peak = np.full(o.shape, simt_ops_s)
        if i16_ops_s:
            k = kinds_of.get(id(p))
            if k is None:
                k = kinds_of[id(p)] = plan_node_kinds(p)
            peak = np.where(k == 3, i16_ops_s, simt_ops_s)
        ts, th = o / peak, b / (hbm_gbs * 1e9)
        ops += o.sum()
        byts += b.sum()
        t_simt += ts.sum()
        t_hbm += th.sum()
        t_bound += np.maximum(ts, th).sum()
    return ops, byts, t_simt, t_hbm, t_bound


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower() in ("active", "1"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def load_workload(tb, name):
    from tensorbranching_gb300 import workloads

    return workloads.load(name)


def make_items(engine, wl, tb, max_items=0):
    """Plans and per-item inputs of one step of the workload
    (``workloads.step_items``): one plan per branch, shared by its slices."""
    from tensorbranching_gb300 import workloads

    items = workloads.step_items(wl, max_items)
    plans, svs, rs = workloads.plans_for(engine, items)
    wmap = wl.setdefault("plan_weights", {})
    for it, p in zip(items, plans):
        wmap[id(p)] = it["weights"]
    return plans, svs, rs


def expected_answer(wl):
    """Solves (MIS values) one step completes: graphs per step, or the
    fraction of one solve a step of a sliced workload covers."""
    if "graphs" in wl:
        return len(wl["graphs"]) if not wl.get("truncated") else 0.0
    return wl.get("step_fraction", 1.0) if not wl.get("truncated") else 0.0


def _node_ops(code):
    labs = [list(dict.fromkeys(ix)) for ix in code.ixs] + code.labels_of_nodes()
    ops = np.array([2.0 * 2 ** len(set(labs[int(a)]) | set(labs[int(c)])) for a, c in code.children])
    return labs, ops


def _subtree(tb, code, labs, j):
    """The sub-network under internal node j, open on node j's labels."""
    T = code.n_tensors
    nodes, leaves = [], []
    stack = [T + j]
    while stack:
        x = stack.pop()
        if x < T:
            leaves.append(x)
        else:
            nodes.append(x - T)
            stack.extend(int(y) for y in code.children[x - T])
    nodes.sort()
    leaves.sort()
    idmap = {old: i for i, old in enumerate(leaves)}
    ch, niy = [], []
    for q in nodes:
        a, b = (int(x) for x in code.children[q])
        ch.append((idmap[a], idmap[b]))
        idmap[T + q] = len(leaves) + len(ch) - 1
        niy.append(labs[T + q])
    return tb.CompressedEinsum([code.ixs[x] for x in leaves], list(labs[T + j]), np.array(ch, np.int32),
                               node_iy=niy, n_labels=code.n_labels), nodes


def run_cpu_baseline(tb, orc, wl, budget_s: float, threads: int = 0):
    """The oracle port (GEMM lowering, OpenMP on `threads` host cores, 0:
    every core) on a bounded sample: the largest subtree of the first network
    whose contraction fits the time budget, extrapolated by algorithmic ops
    to whole steps."""
    threads = orc.set_threads(threads)
    sliced = wl["sliced"]
    total_ops = 0.0
    for br in wl["branches"]:
        if br.code is None:
            continue
        code = br.code.remove_labels(sliced) if sliced else br.code
        total_ops += _node_ops(code)[1].sum() * ((1 << len(sliced)) if sliced else 1)
    br = next(x for x in wl["branches"] if x.code is not None)
    code = br.code.remove_labels(sliced) if sliced else br.code
    w = br.p.weight_array()
    labs, ops = _node_ops(code)
    T = code.n_tensors
    # subtree ops
    sub = ops.copy()
    for j in range(code.n_nodes):
        for c in code.children[j]:
            if c >= T:
                sub[j] += sub[int(c) - T]
    order = np.argsort(sub)
    rate = None
    best = None
    last = 0.0
    for j in order:
        if sub[j] < 2 * last and j != order[-1]:
            continue  # geometric steps through subtree sizes
        last = sub[j]
        if rate is not None and sub[j] / rate > 4 * budget_s:
            break
        s_code, nodes = _subtree(tb, code, labs, int(j))
        t0 = time.perf_counter()
        orc.execute(s_code, w, mode="gemm")
        dt = time.perf_counter() - t0
        if dt > 0.05:
            rate = sub[j] / dt
            best = (int(j), len(nodes), sub[j], dt)
        if dt > budget_s:
            break
    if best is None:
        s_code, nodes = _subtree(tb, code, labs, code.n_nodes - 1)
        t0 = time.perf_counter()
        orc.execute(s_code, w, mode="gemm")
        dt = time.perf_counter() - t0
        best = (code.n_nodes - 1, len(nodes), sub[-1], dt)
        rate = sub[-1] / dt
    j, nn, sops, dt = best
    reps = 1
    if dt < budget_s / 3:
        # a short sample: repeat it to about a third of the budget
        s_code, _ = _subtree(tb, code, labs, j)
        reps = max(1, int(budget_s / 3 / max(dt, 1e-3)))
        t0 = time.perf_counter()
        for _ in range(reps):
            orc.execute(s_code, w, mode="gemm")
        dt = (time.perf_counter() - t0) / reps
    graphs = len(wl["graphs"]) if "graphs" in wl else 1
    solves_per_s = (sops / dt) / total_ops * graphs
    sample = (f"subtree of {nn} of {code.n_nodes} contraction nodes of the first network ({sops:.3g} of "
              f"{total_ops:.3g} tropical ops per step) in {dt:.2f}s (mean of {reps}); solves/s extrapolated by "
              f"algorithmic ops")
    return {"value": solves_per_s, "unit": "solves/s", "cores": threads, "kind": "port", "sample": sample,
            "ops_per_s": sops / dt}


ANSWERS = os.path.join(ROOT, "tests", "golden", "workload_answers.json")
EXTRA_CONFIGS = "rr100_ob10,ksg32_ob20,ksg32_b20,ksg32_dom20,rr300w_s22,rr220w_s22"
PLAIN_MAX_ITEMS = 256


def stored_answers(name):
    """The oracle's item values for this workload (tests/golden/
    workload_answers.json, made by tests/golden/make_answers.py), or None."""
    if not os.path.exists(ANSWERS):
        return None
    with open(ANSWERS) as f:
        return json.load(f).get(name)


def check_answer(name, out, max_items):
    """Every item value of a step against the stored oracle values."""
    ans = stored_answers(name)
    if ans is None:
        return False, "no stored oracle answer for this workload"
    ref = ans["items"]
    if max_items:
        ref = ref[: len(out)] if not ans["sliced"] else None
        if ref is None:
            return False, "a --max-items run of a sliced workload samples other slices"
    if len(ref) != len(out):
        return False, f"{len(out)} items, {len(ref)} stored"
    bad = int(np.sum(np.asarray(out, np.float64) != np.asarray(ref, np.float64)))
    if bad:
        raise AssertionError(f"{name}: {bad} of {len(out)} item values differ from the oracle's")
    return True, f"all {len(out)} item values equal the oracle's (tests/golden/workload_answers.json)"


def workload_config(wl, name):
    """The workload as both arms describe it (no engine settings)."""
    br = next(x for x in wl["branches"] if x.code is not None)
    code = br.code.remove_labels(wl["sliced"]) if wl["sliced"] else br.code
    tc, sc, rwc = code.complexity()
    from tensorbranching_gb300 import workloads

    items = workloads.step_items(wl)
    return {"workload": name, "detail": _desc(name), "items_per_step": len(items),
            "graphs_per_step": expected_answer(wl), "tc": tc, "sc": sc, "rwc": rwc,
            "sliced_labels": len(wl["sliced"]), "l2": "flushed between steps (256 MiB write)"}


def level_roofline(prof, simt, hbm, simt_i16=None, stream_wide=True):
    """Per-kernel roofline from a per-launch profile: the GEMM-tile launches
    (k_level<float, 2>) against the SIMT max-plus peak of their form, the
    stream-tile launches (k_level<float, 5>, the 128-register form, or
    k_level<float, 1>) against HBM; the dominant kernel is the one with the
    larger share of device time."""
    tot = sum(p["ms"] for p in prof) or 1e-9
    out = {}
    stream_name = ("k_level<float,5> (stream tiles, 128-register form)" if stream_wide else
                   "k_level<float,1> (stream tiles, 80-register form)")
    for kind, name in (("gemm", "k_level<float,2> (GEMM tiles)"), ("stream", stream_name)):
        ps = [p for p in prof if p["kind"] == kind]
        if not ps:
            continue
        t = sum(p["ms"] for p in ps) / 1000.0
        o = sum(p["ops"] for p in ps)
        b = sum(p["bytes"] for p in ps)
        if kind == "gemm":
            peak = simt_i16 if simt_i16 else simt
            out[kind] = {"kernel": name, "launches": len(ps), "share": t * 1000.0 / tot, "bound": "simt",
                         "achieved": o / t / 1e12, "peak": peak / 1e12, "unit": "TFLOP/s",
                         "frac": o / t / peak, "ms": t * 1000.0, "algorithmic_ops": o}
        else:
            out[kind] = {"kernel": name, "launches": len(ps), "share": t * 1000.0 / tot, "bound": "hbm",
                         "achieved": b / t / 1e9, "peak": hbm, "unit": "GB/s", "frac": b / t / (hbm * 1e9),
                         "ms": t * 1000.0, "algorithmic_bytes": b}
    return out


def measure(tb, eng, wl, name, args, steps, warmup, plain_steps, flush, dev, ws, simt, simt_i16, hbm, peak_kind,
            with_profile=True):
    """Time one workload on one engine: the device-timed step (inputs
    resident, L2 flushed between steps), the end-to-end step through the
    public API (host weights bound, results read back), the per-launch
    roofline and the plain drop-in path on the same items."""
    import torch

    plans, svs, rs = make_items(eng, wl, tb, args.max_items)
    units = expected_answer(wl)
    if args.tile_bits:
        for p in {id(p): p for p in plans}.values():
            eng.retile(p, args.tile_bits)
    uniq = {id(p): p for p in plans}
    ops = sum(p.stats()["ops"] for p in plans)
    tuned = eng.autotune(plans, slice_vals=svs, r=rs) if args.mode == "auto" else None
    mode = tuned["mode"] if tuned else args.mode
    out0, mx0 = eng.solve_batch(plans, slice_vals=svs, r=rs, mode=args.mode)
    checked, note = check_answer(name, out0, args.max_items)
    # the caller's host buffers of the per-item inputs: slice values of all
    # items concatenated (None when no item is sliced) and r as float32
    sv_host = (None if not svs or all(len(x) == 0 for x in svs) else
               np.ascontiguousarray(np.concatenate([np.asarray(x, np.int8).ravel() for x in svs]), np.int8))
    r_host = np.ascontiguousarray(rs, np.float32)

    def step():
        return eng.solve_batch(plans, slice_vals=sv_host, r=r_host, mode=args.mode)

    for _ in range(warmup):
        step()
    dev_ms, launches = [], 0
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(dev) as clk:
        for _ in range(steps):
            flush.zero_()
            torch.cuda.synchronize()
            o, m = step()
            ms, nl = eng.last_timing()
            dev_ms.append(ms)
            launches += nl
            if not np.array_equal(o, out0):
                raise AssertionError(f"{name}: a timed step's item values changed")
    torch.cuda.synchronize()
    t_dev = sum(dev_ms) / 1000.0
    # e2e: bind weights from host (H2D) + solve + result read-back (D2H), wall clock
    uplans = list(uniq.values())
    h2d = sum(4 * p.code.n_labels for p in uplans) + 4 * len(plans) + (sum(len(x) for x in svs) if svs else 0)
    d2h = 4 * (len(plans) + 1)
    host_w = [np.ascontiguousarray(_weights_of(wl, p), np.float32) for p in uplans]
    w_offs = np.zeros(len(uplans), np.int64)
    if len(uplans) > 1:
        w_offs[1:] = np.cumsum([len(w) for w in host_w[:-1]])
    w_flat = np.ascontiguousarray(np.concatenate(host_w), np.float32)  # the caller's host buffer
    # at least 0.2 s of end-to-end steps (short steps: a few steps would
    # weigh one host hiccup too much)
    e2e_steps = max(steps, min(1000, int(0.2 / max(t_dev / steps, 1e-6))))
    if ws > 1:
        t_es = torch.tensor([e2e_steps], dtype=torch.int64, device=f"cuda:{dev}")
        torch.distributed.all_reduce(t_es, op=torch.distributed.ReduceOp.MAX)
        e2e_steps = int(t_es[0])
        torch.distributed.barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        eng.bind_batch(uplans, w_flat, w_offs)
        o, m = step()
        if not np.array_equal(o, out0):
            raise AssertionError(f"{name}: an end-to-end step's item values changed")
    t_e2e = (time.perf_counter() - t0) * steps / e2e_steps  # per `steps` steps, as t_dev
    if ws > 1:
        tt = torch.tensor([t_dev, t_e2e], dtype=torch.float64, device=f"cuda:{dev}")
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        t_dev, t_e2e = float(tt[0]), float(tt[1])
    ms_per_step = 1000.0 * t_dev / steps
    t_step = ms_per_step / 1000.0
    i16 = eng.gemm_arith == "i16x2" and _gemm_arith(wl) != "f32"
    r_ops, r_bytes, t_simt, t_hbm, t_bound = roofline(plans, t_step, simt, hbm, simt_i16 if i16 else None)
    res = {"value": ws * steps * units / t_dev, "unit": "solves/s", "ms_per_step": ms_per_step,
           "dtype": "int16x2 (exact: integer weights >= 0 summing below 8192)" if i16 else "f32",
           "mode": mode, "autotune": tuned, "answer": mx0, "answer_checked": checked, "answer_note": note,
           "tropical_gops": ops / t_step / 1e9, "gpu_launches": launches,
           "items_per_s": ws * steps * len(plans) / t_dev,
           "e2e": {"value": ws * steps * units / t_e2e, "unit": "solves/s", "h2d_bytes_per_step": h2d,
                   "d2h_bytes_per_step": d2h, "steps": e2e_steps},
           "clocks": clk.summary()}
    # the step as a whole against the node-weighted roofline
    step_roof = {"attainable_frac": t_bound / t_step, "algorithmic_ops": r_ops, "algorithmic_bytes": r_bytes}
    if t_simt >= t_hbm:
        step_roof.update({"bound": "simt", "achieved": r_ops / t_step / 1e12, "peak": r_ops / t_simt / 1e12,
                          "unit": "TFLOP/s", "frac": t_simt / t_step})
    else:
        step_roof.update({"bound": "hbm", "achieved": r_bytes / t_step / 1e9, "peak": hbm, "unit": "GB/s",
                          "frac": r_bytes / t_step / (hbm * 1e9)})
    res["step_roofline"] = step_roof
    if with_profile and mode == "layered":
        # per-launch device times of the same schedule (CUDA events on the
        # engine's stream, L2 flushed before each of three runs)
        runs = []
        for _ in range(3):
            flush.zero_()
            torch.cuda.synchronize()
            runs.append(eng.profile_levels(plans, slice_vals=svs, r=rs))
        prof = [dict(p, ms=float(np.mean([r[k]["ms"] for r in runs]))) for k, p in enumerate(runs[0])]
        res["kernels"] = level_roofline(prof, simt, hbm, simt_i16 if i16 else None, eng.stream_wide())
    if plain_steps > 0:
        # the drop-in path on the same items: one item at a time, per-node
        # launches (permute + K1 GEMM + permute), a result read-back per item.
        # It runs the items one after another, so a strided sample of at most
        # PLAIN_MAX_ITEMS of them, scaled by the item count, times the step.
        n = len(plans)
        stride = -(-n // PLAIN_MAX_ITEMS)
        idx = list(range(0, n, stride))
        p_s = [plans[i] for i in idx]
        sv_s = [svs[i] for i in idx] if svs is not None else None
        pl_ms = 0.0
        for _ in range(plain_steps):
            flush.zero_()
            torch.cuda.synchronize()
            o, m = eng.solve_batch(p_s, slice_vals=sv_s, r=rs[idx], mode="plain")
            if not np.array_equal(o, out0[idx]):
                raise AssertionError(f"{name}: the plain path's item values differ")
            pl_ms += eng.last_timing()[0] * n / len(idx)
        pv = plain_steps * units / (pl_ms / 1000.0)
        res["plain"] = {"value": pv, "unit": "solves/s", "ms_per_step": pl_ms / plain_steps, "steps": plain_steps,
                        "items_timed": len(idx), "items": n, "speedup_vs_plain": res["value"] / pv,
                        "note": "items timed one after another, the per-item device time scaled to the step's "
                                "item count" if len(idx) < n else "every item of the step"}
    return res, plans


def gemm_square(tb, eng, simt, n=2048, batch=8, reps=5):
    """The plain path's batched max-plus GEMM (K1, tb_gemm_device) at a dense
    square shape, M = N = K = n, on device buffers: 2 n^3 batch tropical ops
    per launch over the mean of `reps` launches (CUDA events on the launching
    stream, after two warm-up launches)."""
    import torch

    g = torch.Generator(device="cuda").manual_seed(0)
    A = torch.randint(0, 64, (batch * n * n,), device="cuda", generator=g).float()
    B = torch.randint(0, 64, (batch * n * n,), device="cuda", generator=g).float()
    C = torch.empty(batch * n * n, device="cuda")
    s = torch.cuda.current_stream()
    for _ in range(2):
        eng.gemm(n, n, n, batch, A.data_ptr(), B.data_ptr(), C.data_ptr(), s.cuda_stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(s)
    for _ in range(reps):
        eng.gemm(n, n, n, batch, A.data_ptr(), B.data_ptr(), C.data_ptr(), s.cuda_stream)
    e1.record(s)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / reps
    # spot check one output column of one batch against a host max-plus product
    b, j = batch - 1, n // 3
    Ah = A[b * n * n:(b + 1) * n * n].view(n, n).T.cpu().numpy()       # [m, k] (column-major storage)
    Bh = B[b * n * n + j * n:b * n * n + (j + 1) * n].cpu().numpy()     # column j: [k]
    ref = (Ah + Bh[None, :]).max(axis=1)
    got = C[b * n * n + j * n:b * n * n + (j + 1) * n].cpu().numpy()
    ok = bool(np.array_equal(ref, got))
    ops = 2.0 * n ** 3 * batch
    return {"kernel": "gemm_k1 (tb_gemm_device)", "M": n, "N": n, "K": n, "batch": batch, "ms": ms,
            "achieved": ops / (ms / 1000.0) / 1e12, "peak": simt / 1e12, "unit": "TFLOP/s",
            "frac": ops / (ms / 1000.0) / simt, "dtype": "f32", "column_checked": ok}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="rr220")
    ap.add_argument("--mode", default="auto", choices=["auto", "batched", "layered", "plain", "fused"],
                    help="auto: tb_autotune picks tile size and schedule before the warm-up (untimed)")
    ap.add_argument("--gemm-arith", default="f32", choices=["f32", "i16x2"],
                    help="arithmetic of the headline's GEMM tiles (f32: the reference's Float32)")
    ap.add_argument("--configs", default=EXTRA_CONFIGS,
                    help="further workloads timed in the same run and reported under 'configs' ('' for none)")
    ap.add_argument("--config-steps", type=int, default=5)
    ap.add_argument("--no-i16", action="store_true", help="skip the packed-int16 GEMM form of the headline")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain drop-in comparison")
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--requests", type=int, default=48)
    ap.add_argument("--make", nargs="*")
    ap.add_argument("--max-items", type=int, default=0,
                    help="run only the first N branches / sliced items (small cases for ncu captures)")
    ap.add_argument("--no-graphs", action="store_true",
                    help="launch kernels directly instead of replaying a CUDA graph")
    ap.add_argument("--tile-bits", type=int, default=0,
                    help="stream tiles of up to 2^N outputs (8..11) instead of the default / autotuned size")
    args = ap.parse_args()

    tb = _ge.load_package()
    if args.make is not None:
        from tensorbranching_gb300 import workloads

        for nm in args.make or list(workloads.BUILDERS):
            workloads.make(nm)
        return

    ws, rank, local = dist_env()
    if args.config == "serve":
        if args.impl == "reference":
            if rank == 0:
                print(json.dumps({"impl": "reference", "metric": METRIC, "unavailable":
                                  "the reference has no serving loop (dynamic_ob_mis solves one request at a time)"}))
            return
        return run_serve(tb, args)
    wl = load_workload(tb, args.config)
    if args.max_items and not wl["sliced"]:
        wl["truncated"] = True  # a subset of the branches answers no whole solve
        wl["branches"] = [b for b in wl["branches"] if b.code is not None][: args.max_items]
    cfg = workload_config(wl, args.config)
    units = expected_answer(wl)

    if args.impl == "reference":
        if rank != 0:
            return
        orc = _ge.load_oracle()
        orc.build()
        vals = []
        for i in range(args.warmup + args.steps):
            r = run_cpu_baseline(tb, orc, wl, max(2.0, args.cpu_budget / 4))
            if i >= args.warmup:
                vals.append(r["value"])
        v = statistics.median(vals)
        out = {"metric": METRIC, "value": v, "unit": "solves/s", "impl": "reference", "n_gpus": args.gpus,
               "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * units / v,
               "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
               "data": "synthetic (seeded graphs, weights as described)", "config": cfg,
               "cpu_baseline": {"value": v, "unit": "solves/s", "cores": r["cores"], "kind": "port",
                                "sample": r["sample"], "cpu": _cpu_model()},
               "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(out))
        return

    import torch

    if ws > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    dev = local if ws > 1 else 0
    torch.cuda.set_device(dev)
    from tensorbranching_gb300.engine import measure_maxplus_peak, measure_maxplus_peak_i16

    simt = measure_maxplus_peak(dev)
    simt_i16 = measure_maxplus_peak_i16(dev)
    hbm, peak_kind = _peaks()
    # L2 flush buffer (larger than the 129 MB L2)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=f"cuda:{dev}")
    eng = tb.Engine(device=dev, use_graphs=not args.no_graphs, gemm_arith=args.gemm_arith)
    head, plans = measure(tb, eng, wl, args.config, args, args.steps, args.warmup,
                          0 if args.no_plain or args.mode == "plain" else min(args.steps, 3), flush, dev, ws, simt,
                          simt_i16, hbm, peak_kind)
    extra = {}
    if rank == 0 and not args.no_i16 and args.gemm_arith == "f32" and _gemm_arith(wl) != "f32":
        # the same workload with the exact packed-int16 GEMM tiles
        eng16 = tb.Engine(device=dev, use_graphs=not args.no_graphs, gemm_arith="i16x2")
        r16, _ = measure(tb, eng16, load_workload(tb, args.config) if not args.max_items else wl, args.config, args,
                         args.steps, args.warmup, 0, flush, dev, 1, simt, simt_i16, hbm, peak_kind)
        eng16.close()
        extra["i16x2"] = {k: r16[k] for k in ("value", "unit", "ms_per_step", "dtype", "answer_checked", "e2e",
                                               "step_roofline", "kernels", "mode") if k in r16}
    configs = {}
    if rank == 0 and ws == 1 and args.configs and not args.max_items:
        for nm in [x for x in args.configs.split(",") if x and x != args.config]:
            try:
                wl2 = load_workload(tb, nm)
            except FileNotFoundError as ex:
                configs[nm] = {"unavailable": str(ex)}
                continue
            e2 = tb.Engine(device=dev, use_graphs=not args.no_graphs, gemm_arith=args.gemm_arith)
            r2, _ = measure(tb, e2, wl2, nm, args, args.config_steps, 3, 0 if args.no_plain else 1, flush, dev, 1,
                            simt, simt_i16, hbm, peak_kind)
            e2.close()
            r2["config"] = workload_config(wl2, nm)
            r2.pop("clocks", None)
            configs[nm] = r2
    if rank != 0:
        torch.distributed.destroy_process_group()
        return
    gk = head.get("kernels", {})
    dom = max(gk.values(), key=lambda k: k["share"]) if gk else None
    if dom is not None:
        roof = {k: dom[k] for k in ("bound", "achieved", "peak", "unit", "frac")}
        roof.update({"kernel": dom["kernel"], "share_of_step": dom["share"]})
    else:
        sr = head["step_roofline"]
        roof = {k: sr[k] for k in ("bound", "achieved", "peak", "unit", "frac")}
        roof["kernel"] = {"fused": "k_small", "batched": "k_persistent"}.get(head["mode"], head["mode"])
        roof["share_of_step"] = 1.0
    roof["traffic"], roof["traffic_source"] = _profiled_traffic(args.config, head["mode"], head["dtype"])
    roof["peak_source"] = (f"simt: measured f32 max-plus probe on this GPU ({simt / 1e12:.2f} Tops; the packed-int16 "
                           f"probe {simt_i16 / 1e12:.2f} Tops is the ceiling of int16x2 GEMM tiles); hbm: "
                           f"{peak_kind} copy bandwidth ({hbm:.0f} GB/s)")
    roof["note"] = ("achieved = algorithmic tropical ops 2*2^|L| (max and add; SIMT, no tensor cores) or bytes "
                    "4(|A|+|B|+|C|) of the nodes the kernel's launches run / their device time (CUDA events per "
                    "launch on the engine's stream); kernels: every kernel of the step with its share")
    res = {
        "metric": METRIC, "value": head["value"], "unit": "solves/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": head["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": head["dtype"], "data": "synthetic (seeded graphs, weights as described)",
        "config": cfg,
        "engine": {"mode": head["mode"], "autotune": head["autotune"], "gemm_arithmetic": head["dtype"],
                   "resident_ctas": eng.info(), "parallelism": f"replicas x{ws}"},
        "answer": head["answer"], "answer_checked": head["answer_checked"], "answer_note": head["answer_note"],
        "tropical_gops": head["tropical_gops"],
        "roofline": roof, "kernels": gk, "step_roofline": head["step_roofline"],
        "e2e": head["e2e"], "gpu_launches": head["gpu_launches"], "clocks": head["clocks"],
    }
    if rank == 0:
        res["gemm_square"] = gemm_square(tb, eng, simt)
    if "plain" in head:
        res["plain"] = head["plain"]
        res["speedup_vs_plain"] = head["plain"]["speedup_vs_plain"]
    res.update(extra)
    if configs:
        res["configs"] = configs
    if not args.no_cpu_baseline:
        orc = _ge.load_oracle()
        orc.build()
        cb = run_cpu_baseline(tb, orc, wl, args.cpu_budget)
        cb1 = run_cpu_baseline(tb, orc, wl, args.cpu_budget / 2, threads=1)
        orc.set_threads(0)
        cb["cpu"] = _cpu_model()
        cb["single_thread"] = {"value": cb1["value"], "cores": 1, "sample": cb1["sample"]}
        res["cpu_baseline"] = cb
    print(json.dumps(res))
    eng.close()
    if ws > 1:
        torch.distributed.destroy_process_group()


def _cpu_model():
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip() + f" ({os.cpu_count()} cores)"
    except Exception:
        pass
    return f"{os.cpu_count()} cores"


def run_serve(tb, args):
    """Serving mix: capacity with every request queued at once, then Poisson
    arrivals at 0.8x that capacity; p50/p99 submit-to-result latency."""
    from tensorbranching_gb300 import serving

    mix = serving.serving_mix(args.requests, seed=11)
    eng = tb.Engine()
    t0 = time.perf_counter()
    preps = [serving.prepare(eng, g, w, sc_cap=24.0, seed=i, name=nm) for i, (nm, g, w) in enumerate(mix)]
    prep_s = time.perf_counter() - t0
    # results served alone (reference values for the mix)
    alone = []
    for p in preps:
        if p.constant is not None:
            alone.append(p.constant)
        else:
            alone.append(eng.solve_batch(p.plans, slice_vals=p.slice_vals, r=np.array(p.r, np.float32),
                                         mode="batched")[1])
    with serving.Server(eng, pool_bytes=64 << 30, max_items=1 << 16) as srv:
        warm = serving.run_poisson(srv, preps[: min(4, len(preps))], rate=0.0)
        cap = serving.run_poisson(srv, preps, rate=0.0)
        capacity = len(preps) / cap["wall_s"]
        rate = 0.8 * capacity
        with ClockSampler(0) as clk:
            run = serving.run_poisson(srv, preps, rate=rate, seed=5)
        st = srv.stats()
    assert run["values"] == alone and cap["values"] == alone, "served results differ from results alone"
    lat = np.array(run["latency_ms"])
    res = {"metric": METRIC, "value": len(preps) / run["wall_s"], "unit": "solves/s", "n_gpus": 1,
           "steps": len(preps), "warmup": len(warm["values"]), "ms_per_step": 1000.0 * run["wall_s"] / len(preps),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic serving mix (seeded)",
           "config": {"workload": "serve", "requests": len(preps),
                      "detail": "Poisson arrivals at 0.8x measured capacity; 3-regular n in [60,200] and KSG L in "
                                "[10,36] filling 0.8; unit or U{1..10} weights; sc capped at 24 by index slicing; "
                                "admitted requests run as cohorts on 4 streams",
                      "arrival_rate_per_s": rate, "capacity_solves_per_s": capacity,
                      "items": int(sum(p.n_items for p in preps)), "host_prep_s": prep_s},
           "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                          "mean": float(lat.mean()), "max": float(lat.max())},
           "server": st, "same_alone_and_in_mix": True, "clocks": clk.summary()}
    print(json.dumps(res))


def _gemm_arith(wl):
    """The GEMM tiles use exact packed-int16 DPX arithmetic when every bound
    weight vector is integral, >= 0 and sums below 8192; f32 otherwise."""
    ok = True
    for w in wl.get("plan_weights", {}).values():
        w = np.asarray(w, np.float64)
        ok = ok and bool(np.all(w >= 0) and np.all(w == np.floor(w)) and w.sum() < 8192)
    return "int16x2 DPX (exact: integer weights >= 0 summing below 8192)" if ok else "f32"


def _weights_of(wl, plan):
    return wl["plan_weights"][id(plan)]


def _profiled_traffic(config, mode, dtype):
    """DRAM bytes per launch of the dominant kernel from the committed ncu
    summary for this workload and form (profiles/traffic_<config>_<mode>
    [_i16].txt, line 'traffic_bytes_per_launch: X'), and the file's name;
    (None, reason) when no capture exists."""
    sfx = "_i16" if dtype.startswith("int16") else ""
    nm = f"traffic_{config}_{mode}{sfx}.txt"
    p = os.path.join(ROOT, "profiles", nm)
    if os.path.exists(p):
        for line in open(p):
            if line.startswith("traffic_bytes_per_launch:"):
                return float(line.split(":")[1]), f"profiles/{nm}"
    return None, f"no ncu capture committed as profiles/{nm}"


def _desc(name):
    from tensorbranching_gb300 import workloads

    return workloads.WORKLOADS.get(name, name)


if __name__ == "__main__":
    main()
