"""Writes tests/golden/workload_answers.json: the oracle's answers for the
benchmark workloads (test infrastructure).

For every item of one benchmark step (``workloads.step_items``): the item's
value, max over its root tensor + r, from the CPU oracle (oracle/tropical.c,
GEMM lowering).  For every graph of the workload: its exact maximum (weight)
independent set from the integer program of oracle/mis_exact.py (IP_MWIS,
src/utils.jl:295-310), and the largest r of its branches that have no
network left (contract_slices returns r for those, src/dynamic_ob.jl:39-40).

bench.py checks the item values of every timed step against this file;
tests/test_answers.py pins the stored values to the exact solver: over each
graph, the max of its items and empty branches equals its MIS, the relation
test/dynamic_ob.jl:20,38,51 checks (for sampled slices of an index-sliced
workload, the max is at most the MIS).

Run: python tests/golden/make_answers.py [workload ...]
"""
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

import __graft_entry__ as ge  # noqa: E402
from oracle import mis_exact  # noqa: E402

OUT = os.path.join(HERE, "workload_answers.json")
DEFAULT = ["rr220", "rr100_ob10", "rr100_b10", "ksg32_b20", "rr220w_s22"]


def graphs_of(wl):
    """(graph, weights, branch indices) per graph of the workload."""
    if "graphs" in wl:
        out, k = [], 0
        for g, bs in zip(wl["graphs"], wl["branch_sets"]):
            out.append((g, np.ones(g.n), list(range(k, k + len(bs)))))
            k += len(bs)
        return out
    g = wl["graph"]
    b0 = wl["branches"][0]
    # the weights of the original graph: a single branch on the graph itself
    # carries them; branches of a kernel come from unit-weight graphs here
    w = b0.p.weight_array() if len(wl["branches"]) == 1 and b0.p.g.n == g.n else np.ones(g.n)
    return [(g, np.asarray(w, np.float64), list(range(len(wl["branches"]))))]


def answers(name):
    tb = ge.load_package()
    orc = ge.load_oracle()
    orc.build()
    from tensorbranching_gb300 import workloads

    wl = workloads.load(name)
    items = workloads.step_items(wl)
    t0 = time.time()
    vals = []
    for it in items:
        v = orc.solve(it["code"], it["weights"], sliced=it["fixed"], slice_vals=it["values"])
        vals.append(float(np.float32(v) + np.float32(it["r"])))
    t_items = time.time() - t0
    gs = graphs_of(wl)
    branch_graph = {}
    for gi, (_, _, bis) in enumerate(gs):
        for b in bis:
            branch_graph[b] = gi
    graph_of_item = [branch_graph[it["branch"]] for it in items]
    extra = []
    for g, w, bis in gs:
        rs = [float(wl["branches"][b].r) for b in bis if wl["branches"][b].code is None]
        extra.append(max(rs) if rs else None)
    t0 = time.time()
    mis = [float(mis_exact.ip(g.n, g.edges, w)) for g, w, _ in gs]
    t_ip = time.time() - t0
    return {"workload": name, "items": vals, "graph_of_item": graph_of_item, "slice_index": [it["index"] for it in items],
            "graph_empty_r": extra, "graph_mis": mis, "sliced": bool(wl["sliced"]),
            "how": f"items: oracle.solve (C restatement, GEMM lowering) in {t_items:.1f}s; graph_mis: HiGHS IP "
                   f"(IP_MWIS) in {t_ip:.1f}s"}


def main():
    names = sys.argv[1:] or DEFAULT
    data = {}
    if os.path.exists(OUT):
        with open(OUT) as f:
            data = json.load(f)
    for nm in names:
        t = time.time()
        data[nm] = answers(nm)
        print(f"{nm}: {len(data[nm]['items'])} items, MIS {data[nm]['graph_mis'][:4]}... in {time.time() - t:.0f}s",
              flush=True)
        with open(OUT, "w") as f:
            json.dump(data, f, separators=(",", ":"))


if __name__ == "__main__":
    main()
