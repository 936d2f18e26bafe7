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


OPEN_BITS = 4          # sliced labels kept open per item (2^4 slices per item)
SLICED_ITEMS_PER_STEP = 64


def make_items(engine, wl, tb, max_items=0):
    """Plans and per-item inputs of one step of the workload.  Index-sliced
    workloads group 2^OPEN_BITS slices per item (those labels stay open in the
    root tensor) and a step runs SLICED_ITEMS_PER_STEP of the items."""
    plans, svs, rs = [], [], []
    sliced = wl["sliced"]
    frac = 1.0
    for b in wl["branches"]:
        if b.code is None:
            continue
        wmap = wl.setdefault("plan_weights", {})
        if sliced:
            ob = wl.get("open_bits", OPEN_BITS)
            opened = sliced[:ob]
            fixed = sliced[ob:]
            code = tb.CompressedEinsum(b.code.ixs, list(opened), b.code.children, n_labels=b.code.n_labels)
            p = engine.plan(code, b.p.weight_array(), sliced=fixed)
            wmap[id(p)] = b.p.weight_array()
            k = len(fixed)
            total = 1 << k
            take = min(total, max_items or SLICED_ITEMS_PER_STEP)
            frac = take / total
            idx = np.linspace(0, total - 1, take).astype(np.int64)
            vals = ((idx[:, None] >> np.arange(k)[None, :]) & 1).astype(np.int8)
            for row in vals:
                plans.append(p)
                svs.append(row)
                rs.append(b.r)
        else:
            p = engine.plan(b.code, b.p.weight_array())
            wmap[id(p)] = b.p.weight_array()
            plans.append(p)
            svs.append(np.zeros(0, np.int8))
            rs.append(b.r)
    wl["step_fraction"] = frac
    if all(len(x) == 0 for x in svs):
        svs = None  # no sliced plan: a caller passes no slice values
    return plans, svs, np.array(rs, np.float32)


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


def run_cpu_baseline(tb, orc, wl, budget_s: float):
    """The oracle port (GEMM lowering, OpenMP on every host core) on a bounded
    sample: the largest subtree of the first network whose contraction fits
    the time budget, extrapolated by algorithmic ops to whole steps."""
    threads = os.cpu_count() or 1
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


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="rr220")
    ap.add_argument("--mode", default="auto", choices=["auto", "batched", "layered", "plain", "fused"],
                    help="auto: tb_autotune picks tile size and schedule before the warm-up (untimed)")
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--compare-plain", action="store_true")
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
               "data": "synthetic (seeded graphs)",
               "config": {"workload": args.config, "detail": _desc(args.config)},
               "cpu_baseline": {"value": v, "unit": "solves/s", "cores": r["cores"], "kind": "port",
                                "sample": r["sample"]},
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
    eng = tb.Engine(device=dev, use_graphs=not args.no_graphs)
    if args.max_items:
        wl["branches"] = [b for b in wl["branches"] if b.code is not None][: args.max_items]
    plans, svs, rs = make_items(eng, wl, tb, args.max_items)
    units = expected_answer(wl)
    if args.tile_bits:
        for p in {id(p): p for p in plans}.values():
            eng.retile(p, args.tile_bits)
    st = plans[0].stats()
    uniq = {id(p): p for p in plans}
    ops = sum(uniq[k].stats()["ops"] for k in uniq) if not wl["sliced"] else st["ops"] * len(plans)
    byts = sum(uniq[k].stats()["bytes"] for k in uniq) if not wl["sliced"] else st["bytes"] * len(plans)
    tuned = None
    if args.mode == "auto":
        tuned = eng.autotune(plans, slice_vals=svs, r=rs)
    # check the answer once
    out0, mx0 = eng.solve_batch(plans, slice_vals=svs, r=rs, mode=args.mode)
    from tensorbranching_gb300.engine import measure_maxplus_peak

    simt = measure_maxplus_peak(dev)
    from tensorbranching_gb300.engine import measure_maxplus_peak_i16

    simt_i16 = measure_maxplus_peak_i16(dev)
    # L2 flush buffer (larger than the 129 MB L2)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=f"cuda:{dev}")

    def step():
        return eng.solve_batch(plans, slice_vals=svs, r=rs, mode=args.mode)

    for _ in range(args.warmup):
        step()
    # device-timed region: inputs resident, L2 flushed between steps
    dev_ms = []
    launches = 0
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(dev) as clk:
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            o, m = step()
            ms, nl = eng.last_timing()
            dev_ms.append(ms)
            launches += nl
            assert m == mx0
    torch.cuda.synchronize()
    t_dev = sum(dev_ms) / 1000.0
    # e2e: bind weights from host (H2D) + solve + result read-back (D2H), wall clock
    uplans = list(uniq.values())
    # per step: the bound weights of every distinct plan, r and slice values
    h2d = sum(4 * p.code.n_labels for p in uplans) + 4 * len(plans) + (sum(len(x) for x in svs) if svs else 0)
    d2h = 4 * (len(plans) + 1)
    host_w = [np.ascontiguousarray(_weights_of(wl, p), np.float32) for p in uplans]
    w_offs = np.zeros(len(uplans), np.int64)
    if len(uplans) > 1:
        w_offs[1:] = np.cumsum([len(w) for w in host_w[:-1]])
    w_flat = np.ascontiguousarray(np.concatenate(host_w), np.float32)  # the caller's host buffer
    if ws > 1:
        torch.distributed.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        eng.bind_batch(uplans, w_flat, w_offs)
        o, m = step()
        assert m == mx0
    t_e2e = time.perf_counter() - t0
    if ws > 1:
        tt = torch.tensor([t_dev, t_e2e], dtype=torch.float64, device=f"cuda:{dev}")
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        t_dev, t_e2e = float(tt[0]), float(tt[1])
    if rank != 0:
        torch.distributed.destroy_process_group()
        return
    value = ws * args.steps * units / t_dev
    ms_per_step = 1000.0 * t_dev / args.steps
    hbm, peak_kind = _peaks()
    t_step = ms_per_step / 1000.0
    gemm_arith = _gemm_arith(wl)
    r_ops, r_bytes, t_simt, t_hbm, t_bound = roofline(plans, t_step, simt, hbm,
                                                      simt_i16 if gemm_arith != "f32" else None)
    traffic = _profiled_traffic(args.config, args.mode)
    if t_simt >= t_hbm:
        # peak = the ops-weighted ceiling of the step's nodes: the measured f32
        # max-plus rate, or the packed-int16 one for GEMM nodes in that form
        roof = {"bound": "simt", "achieved": r_ops / t_step / 1e12, "peak": r_ops / t_simt / 1e12,
                "unit": "TFLOP/s", "frac": t_simt / t_step, "peak_f32": simt / 1e12}
    else:
        roof = {"bound": "hbm", "achieved": r_bytes / t_step / 1e9, "peak": hbm, "unit": "GB/s",
                "frac": r_bytes / t_step / (hbm * 1e9)}
    roof.update({
        "peak_i16x2": simt_i16 / 1e12,
        "traffic": traffic, "attainable_frac": t_bound / t_step,
        "peak_source": f"simt: measured f32 max-plus probe on this GPU ({simt / 1e12:.2f} Tops); packed-int16 "
                       f"max-plus probe {simt_i16 / 1e12:.2f} Tops (the GEMM tiles' ceiling when they run that "
                       f"form; used per node in attainable_frac); hbm: {peak_kind} copy bandwidth ({hbm:.0f} GB/s)",
        "note": "dominant kernel k_persistent (batched) / k_level (layered) / k_small (fused: tensors stay in "
                "shared memory, so the HBM fraction is nominal) runs the whole step; achieved = "
                "algorithmic tropical ops 2*2^|L| (max and add; SIMT, no tensor cores) or bytes "
                "4(|A|+|B|+|C|) summed over nodes / device time of the step; a node's compute ceiling is the "
                "measured f32 max-plus rate, or the packed-int16 rate for GEMM nodes run in that form; "
                "attainable_frac = sum over nodes of max(ops/P_node, bytes/BW) / device time"})
    res = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded graphs, weights as described)",
        "config": {"workload": args.config, "detail": _desc(args.config), "mode": args.mode,
                   "items_per_step": len(plans), "graphs_per_step": units, "tc": st["tc"], "sc": st["sc"],
                   "rwc": st["rwc"], "l2": "flushed between steps (256 MiB write)",
                   "answer": mx0, "parallelism": f"replicas x{ws}", "autotune": tuned,
                   "gemm_arithmetic": gemm_arith,
                   "resident_ctas": eng.info()},
        "tropical_gops": ops / (ms_per_step / 1000.0) / 1e9,
        "roofline": roof,
        "e2e": {"value": ws * args.steps * units / t_e2e, "unit": "solves/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "gpu_launches": launches,
        "clocks": clk.summary(),
    }
    if args.compare_plain and args.mode != "plain":
        # the drop-in path on the same items: one item at a time, per-node launches
        t0 = time.perf_counter()
        n_pl = max(1, min(args.steps, 3))
        pl_ms = 0.0
        for _ in range(n_pl):
            flush.zero_()
            torch.cuda.synchronize()
            o, m = eng.solve_batch(plans, slice_vals=svs, r=rs, mode="plain")
            assert m == mx0
            pl_ms += eng.last_timing()[0]
        plain_value = n_pl * units / (pl_ms / 1000.0)
        res["plain"] = {"value": plain_value, "unit": "solves/s", "ms_per_step": pl_ms / n_pl,
                        "speedup_vs_plain": value / plain_value}
    if not args.no_cpu_baseline:
        orc = _ge.load_oracle()
        orc.build()
        res["cpu_baseline"] = run_cpu_baseline(tb, orc, wl, args.cpu_budget)
    print(json.dumps(res))
    if ws > 1:
        torch.distributed.destroy_process_group()


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
                                "[10,24] filling 0.8; unit or U{1..10} weights; sc capped at 24 by index slicing",
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


def _profiled_traffic(config, mode):
    """DRAM bytes per launch of the dominant kernel from the committed ncu
    summary, if one exists for this workload (line 'traffic_bytes_per_step: X')."""
    p = os.path.join(ROOT, "profiles", f"traffic_{config}_{mode}.txt")
    if os.path.exists(p):
        for line in open(p):
            if line.startswith("traffic_bytes_per_step:"):
                return float(line.split(":")[1])
    return None


def _desc(name):
    from tensorbranching_gb300 import workloads

    return workloads.WORKLOADS.get(name, name)


if __name__ == "__main__":
    main()
