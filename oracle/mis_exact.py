"""ORACLE -- test infrastructure only.

Exact maximum-weight independent set solvers, independent of any tensor
network, standing in for the reference tests' ``mis2(EliminateGraph(g))``
(EliminateGraphs inside OptimalBranching 0.2, not in the reference tree;
test/utils.jl:30, test/dynamic_ob.jl:20) and for ``IP_MWIS``
(src/utils.jl:295-310, JuMP + SCIP there; scipy's HiGHS here):

* ``brute_force``      every subset, n <= 24
* ``branch_and_bound`` recursive branching on a max-degree vertex with
                       pendant/isolated-vertex folding and a weight bound
* ``ip``               the integer program max w.x, x_u + x_v <= 1, x binary
"""
from __future__ import annotations

import sys

import numpy as np


def _adj(n, edges):
    adj = [0] * n
    for u, v in edges:
        if u == v:
            adj[u] |= 1 << u
        else:
            adj[u] |= 1 << v
            adj[v] |= 1 << u
    return adj


def brute_force(n: int, edges, w=None) -> float:
    if n > 24:
        raise ValueError("brute force is for n <= 24")
    w = np.ones(n) if w is None else np.asarray(w, np.float64)
    adj = _adj(n, edges)
    best = 0.0
    for s in range(1 << n):
        ok = True
        tot = 0.0
        x = s
        while x:
            v = (x & -x).bit_length() - 1
            x &= x - 1
            if adj[v] & s:
                ok = False
                break
            tot += w[v]
        if ok and tot > best:
            best = tot
    return float(best)


def branch_and_bound(n: int, edges, w=None) -> float:
    """Exact MWIS by branching on bitsets (for n up to about 100 on sparse
    graphs)."""
    w = np.ones(n) if w is None else np.asarray(w, np.float64)
    adj = _adj(n, edges)
    wl = [float(x) for x in w]
    sys.setrecursionlimit(10000)
    best = [0.0]

    def weight(s):
        t = 0.0
        while s:
            v = (s & -s).bit_length() - 1
            s &= s - 1
            t += max(wl[v], 0.0)
        return t

    def rec(cand: int, acc: float):
        # fold isolated / pendant vertices
        changed = True
        while changed and cand:
            changed = False
            s = cand
            while s:
                v = (s & -s).bit_length() - 1
                s &= s - 1
                if not (cand >> v) & 1:
                    continue
                if adj[v] >> v & 1:
                    cand &= ~(1 << v)
                    changed = True
                    continue
                nb = adj[v] & cand
                if nb == 0:
                    if wl[v] > 0:
                        acc += wl[v]
                    cand &= ~(1 << v)
                    changed = True
                elif nb & (nb - 1) == 0:
                    u = nb.bit_length() - 1
                    if wl[v] >= wl[u]:
                        acc += wl[v]
                        cand &= ~((1 << v) | (1 << u))
                        changed = True
        if acc > best[0]:
            best[0] = acc
        if not cand or acc + weight(cand) <= best[0]:
            return
        # branch on the vertex of largest degree in the candidate set
        s = cand
        bv, bd = -1, -1
        while s:
            v = (s & -s).bit_length() - 1
            s &= s - 1
            d = bin(adj[v] & cand).count("1")
            if d > bd:
                bv, bd = v, d
        v = bv
        rec(cand & ~(1 << v) & ~adj[v], acc + wl[v])
        rec(cand & ~(1 << v), acc)

    rec((1 << n) - 1, 0.0)
    return float(best[0])


def ip(n: int, edges, w=None, time_limit: float = 600.0) -> float:
    """IP_MWIS restated with scipy.optimize.milp (HiGHS)."""
    from scipy.optimize import Bounds, LinearConstraint, milp

    w = np.ones(n) if w is None else np.asarray(w, np.float64)
    rows, cols, vals = [], [], []
    ub = np.ones(n)
    k = 0
    for u, v in edges:
        if u == v:
            ub[u] = 0.0
            continue
        rows += [k, k]
        cols += [u, v]
        vals += [1.0, 1.0]
        k += 1
    from scipy.sparse import csr_matrix

    cons = []
    if k:
        A = csr_matrix((vals, (rows, cols)), shape=(k, n))
        cons.append(LinearConstraint(A, -np.inf, 1.0))
    res = milp(-w, constraints=cons, integrality=np.ones(n), bounds=Bounds(np.zeros(n), ub),
               options={"time_limit": time_limit})
    if not res.success:
        raise RuntimeError(f"milp did not finish: {res.message}")
    return float(round(-res.fun, 6))
