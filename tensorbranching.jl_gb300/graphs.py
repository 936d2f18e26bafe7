"""Seeded graph generators and a small simple-graph type.

Generators restate the reference's graph sources with our own seeded RNG
(numpy PCG64), so the same seed gives the same graph on every machine:

* ``random_regular_graph(n, d, seed)`` -- the Graphs.jl ``random_regular_graph``
  used by every reference test (test/utils.jl:21, test/dynamic_ob.jl:21);
  here a pairing model with rejection.
* ``random_ksg(L, filling, seed)`` -- ``random_ksg`` / GenericTensorNetworks
  ``random_diagonal_coupled_graph`` (src/utils.jl:191-195): an L x L grid
  with each site kept with probability ``filling`` and edges between kept
  sites at Chebyshev distance 1 (a unit-disk graph of radius 1.5), sites
  numbered column-major as Julia iterates them.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class Graph:
    """Undirected simple graph on vertices 0..n-1 (edges stored u < v)."""

    n: int
    edges: list[tuple[int, int]] = field(default_factory=list)

    def __post_init__(self):
        es = set()
        for u, v in self.edges:
            u, v = int(u), int(v)
            if not (0 <= u < self.n and 0 <= v < self.n):
                raise ValueError("edge endpoint out of range")
            if u == v:
                es.add((u, u))
            else:
                es.add((min(u, v), max(u, v)))
        self.edges = sorted(es)

    def nv(self) -> int:
        return self.n

    def ne(self) -> int:
        return len(self.edges)

    def adjacency(self) -> list[set[int]]:
        adj = [set() for _ in range(self.n)]
        for u, v in self.edges:
            if u != v:
                adj[u].add(v)
                adj[v].add(u)
        return adj

    def neighbors(self, v: int) -> list[int]:
        return sorted(self.adjacency()[v])

    def induced_subgraph(self, vs) -> tuple["Graph", list[int]]:
        """Induced subgraph on ``vs`` and ``vmap`` (new vertex -> old vertex),
        the convention of Graphs.jl ``induced_subgraph`` used by
        generate_branch (src/branch.jl:212-231)."""
        vmap = sorted(set(int(v) for v in vs))
        inv = {v: i for i, v in enumerate(vmap)}
        es = [(inv[u], inv[v]) for u, v in self.edges if u in inv and v in inv]
        return Graph(len(vmap), es), vmap

    def connected_components(self) -> list[list[int]]:
        adj = self.adjacency()
        seen = [False] * self.n
        comps = []
        for s in range(self.n):
            if seen[s]:
                continue
            stack, comp = [s], []
            seen[s] = True
            while stack:
                x = stack.pop()
                comp.append(x)
                for y in adj[x]:
                    if not seen[y]:
                        seen[y] = True
                        stack.append(y)
            comps.append(sorted(comp))
        return comps


def random_regular_graph(n: int, d: int, seed: int, max_tries: int = 100000) -> Graph:
    """Uniform-pairing d-regular simple graph on n vertices (n*d even)."""
    if (n * d) % 2 or d >= n:
        raise ValueError("no d-regular graph with these parameters")
    rng = np.random.default_rng(seed)
    stubs = np.repeat(np.arange(n), d)
    for _ in range(max_tries):
        perm = rng.permutation(stubs)
        pairs = perm.reshape(-1, 2)
        u = np.minimum(pairs[:, 0], pairs[:, 1])
        v = np.maximum(pairs[:, 0], pairs[:, 1])
        if np.any(u == v):
            continue
        keys = u.astype(np.int64) * n + v
        if len(np.unique(keys)) != len(keys):
            continue
        return Graph(n, list(zip(u.tolist(), v.tolist())))
    raise RuntimeError("pairing model did not produce a simple graph")


def random_ksg(L: int, filling: float, seed: int, m: int | None = None) -> Graph:
    """King's subgraph: L x m grid (m = L), sites kept with probability
    ``filling``, 8-neighbour couplings among kept sites."""
    m = L if m is None else m
    rng = np.random.default_rng(seed)
    keep = rng.random((m, L)) < filling  # keep[j, i]: column j, row i
    locs = []
    for j in range(m):
        for i in range(L):
            if keep[j, i]:
                locs.append((i, j))
    idx = {p: k for k, p in enumerate(locs)}
    es = []
    for (i, j), k in idx.items():
        for di, dj in ((1, 0), (0, 1), (1, 1), (1, -1)):
            q = (i + di, j + dj)
            if q in idx:
                es.append((k, idx[q]))
    return Graph(len(locs), es)


def random_weights(n: int, seed: int, low: int = 1, high: int = 10) -> np.ndarray:
    """Integer weights uniform in [low, high] stored as float32."""
    rng = np.random.default_rng(seed)
    return rng.integers(low, high + 1, size=n).astype(np.float32)
