"""Writes tests/golden/mis_known.json: MIS values that pin the oracle and
the engine independently of any tensor network.

  named    graphs whose MIS follows from their structure (cycles, paths,
           complete graphs, the Petersen graph, King's graphs)
  random   seeded 3-regular graphs and King's subgraphs (this package's
           generators), unit and U{1..10} weights, solved by exhaustive
           enumeration (n <= 24)

Run: python tests/golden/make_golden.py
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

import __graft_entry__ as ge  # noqa: E402
from oracle import mis_exact  # noqa: E402


def named():
    out = []
    for n in (3, 4, 5, 8, 11):
        out.append({"name": f"cycle{n}", "n": n, "edges": [[i, (i + 1) % n] for i in range(n)], "mis": n // 2})
        out.append({"name": f"path{n}", "n": n, "edges": [[i, i + 1] for i in range(n - 1)], "mis": (n + 1) // 2})
        out.append({"name": f"complete{n}", "n": n, "edges": [[i, j] for i in range(n) for j in range(i + 1, n)],
                    "mis": 1})
    outer = [[i, (i + 1) % 5] for i in range(5)]
    spokes = [[i, i + 5] for i in range(5)]
    inner = [[5 + i, 5 + (i + 2) % 5] for i in range(5)]
    out.append({"name": "petersen", "n": 10, "edges": outer + spokes + inner, "mis": 4})
    for L in (2, 3, 4, 5):  # full King's graph: MIS = ceil(L/2)^2
        idx = lambda i, j: i * L + j  # noqa: E731
        e = []
        for i in range(L):
            for j in range(L):
                for di, dj in ((0, 1), (1, -1), (1, 0), (1, 1)):
                    a, b = i + di, j + dj
                    if 0 <= a < L and 0 <= b < L:
                        e.append([idx(i, j), idx(a, b)])
        out.append({"name": f"king{L}", "n": L * L, "edges": e, "mis": ((L + 1) // 2) ** 2})
    for x in out:
        x["weights"] = None
    return out


def random_cases(tb):
    out = []
    for seed in range(12):
        n = 12 + 2 * (seed % 7)
        g = tb.random_regular_graph(n, 3, seed)
        w = tb.random_weights(n, seed) if seed % 2 else None
        v = mis_exact.brute_force(g.n, g.edges, w)
        out.append({"name": f"rr{n}_s{seed}", "n": g.n, "edges": [list(e) for e in g.edges],
                    "weights": None if w is None else [float(x) for x in w], "mis": float(v)})
    for seed in range(6):
        g = tb.random_ksg(5, 0.8, seed)
        w = tb.random_weights(g.n, seed) if seed % 2 else None
        v = mis_exact.brute_force(g.n, g.edges, w)
        out.append({"name": f"ksg5_s{seed}", "n": g.n, "edges": [list(e) for e in g.edges],
                    "weights": None if w is None else [float(x) for x in w], "mis": float(v)})
    return out


def main():
    tb = ge.load_package()
    cases = named() + random_cases(tb)
    with open(os.path.join(HERE, "mis_known.json"), "w") as f:
        f.write('{"generator": "tests/golden/make_golden.py", "cases": [\n')
        f.write(",\n".join(json.dumps(c, separators=(",", ":")) for c in cases))
        f.write("\n]}\n")
    print(f"{len(cases)} cases")


if __name__ == "__main__":
    main()
