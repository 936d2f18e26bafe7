"""Independent-set tensor networks and the plan objects of the reference.

Mirrors (src/types.jl):
  MISProblem(g, weights)
  CompressedEinsum{ixs, iy, ct}      src/types.jl:51-58
  SlicedBranch{p, code, r}           src/types.jl:85-103
  complexity / sc / tc               src/types.jl:115-121
and GenericTensorNetworks' ``rawcode(IndependentSet(g))``: one vertex tensor
``[v]`` per vertex followed by one edge tensor ``[u, v]`` per edge
(src/decompose.jl:65 relies on this order: tensor id of vertex v is v).

Labels are 0-based vertex ids (a Julia caller subtracts 1).  The contraction
tree is stored as post-order pairs ``children[j] = (left, right)``: ids below
``n_tensors`` are leaves, id ``n_tensors + k`` is internal node ``k``.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .graphs import Graph


class UnitWeight:
    """All vertex weights 1 (GenericTensorNetworks UnitWeight)."""

    def __init__(self, n: int):
        self.n = int(n)

    def __len__(self):
        return self.n

    def array(self) -> np.ndarray:
        return np.ones(self.n, np.float32)

    def __eq__(self, other):
        return isinstance(other, UnitWeight) and other.n == self.n

    def __repr__(self):
        return f"UnitWeight({self.n})"


def weights_array(weights, n: int) -> np.ndarray:
    if weights is None:
        return np.ones(n, np.float32)
    if isinstance(weights, UnitWeight):
        if weights.n != n:
            raise ValueError("UnitWeight size differs from the graph")
        return weights.array()
    w = np.asarray(weights, dtype=np.float32)
    if w.shape != (n,):
        raise ValueError(f"expected {n} weights, got shape {w.shape}")
    return w


@dataclass
class MISProblem:
    g: Graph
    weights: object = None  # UnitWeight, array or None (unit)

    def weight_array(self) -> np.ndarray:
        return weights_array(self.weights, self.g.n)


def rawcode(g: Graph) -> tuple[list[list[int]], list[int]]:
    """Leaf label lists of IndependentSet(g): vertices, then edges."""
    ixs = [[v] for v in range(g.n)] + [[u, v] for u, v in g.edges]
    return ixs, []


@dataclass
class CompressedEinsum:
    """A contraction plan: leaf labels, open labels and a binary tree."""

    ixs: list[list[int]]
    iy: list[int]
    children: np.ndarray  # (n_tensors - 1, 2) int32, post-order pairs
    node_iy: list[list[int]] | None = None
    n_labels: int = 0

    def __post_init__(self):
        self.ixs = [list(map(int, ix)) for ix in self.ixs]
        self.iy = list(map(int, self.iy))
        self.children = np.ascontiguousarray(np.asarray(self.children, dtype=np.int32).reshape(-1, 2))
        if self.n_labels <= 0:
            m = -1
            for ix in self.ixs:
                if ix:
                    m = max(m, max(ix))
            if self.iy:
                m = max(m, max(self.iy))
            self.n_labels = m + 1
        if self.children.shape[0] != max(len(self.ixs) - 1, 0):
            raise ValueError("a binary tree over n tensors has n - 1 internal nodes")

    @property
    def n_tensors(self) -> int:
        return len(self.ixs)

    @property
    def n_nodes(self) -> int:
        return self.children.shape[0]

    def csr(self) -> tuple[np.ndarray, np.ndarray]:
        off = np.zeros(self.n_tensors + 1, np.int32)
        off[1:] = np.cumsum([len(ix) for ix in self.ixs])
        lab = np.array([x for ix in self.ixs for x in ix], dtype=np.int32)
        if lab.size == 0:
            lab = np.zeros(1, np.int32)
        return off, lab

    def node_iy_csr(self):
        if self.node_iy is None:
            return None, None
        off = np.zeros(self.n_nodes + 1, np.int32)
        off[1:] = np.cumsum([len(x) for x in self.node_iy])
        lab = np.array([x for ix in self.node_iy for x in ix], dtype=np.int32)
        if lab.size == 0:
            lab = np.zeros(1, np.int32)
        return off, lab

    # -- nested form (the ContractionTree of the reference) ------------------
    def nested(self):
        """The tree as nested 2-tuples of leaf ids (ContractionTree shape)."""
        T = self.n_tensors
        if T == 1:
            return 0
        built = {}
        for j, (a, b) in enumerate(self.children):
            ga = built.pop(int(a)) if a >= T else int(a)
            gb = built.pop(int(b)) if b >= T else int(b)
            built[T + j] = (ga, gb)
        return built[T + self.n_nodes - 1]

    @staticmethod
    def from_nested(ixs, iy, tree, n_labels: int = 0) -> "CompressedEinsum":
        T = len(ixs)
        ch = []

        def walk(t):
            if isinstance(t, (int, np.integer)):
                return int(t)
            a = walk(t[0])
            b = walk(t[1])
            ch.append((a, b))
            return T + len(ch) - 1

        walk(tree)
        return CompressedEinsum(ixs, iy, np.array(ch, np.int32).reshape(-1, 2), n_labels=n_labels)

    # -- complexity (src/types.jl:115-121) -------------------------------------
    def complexity(self) -> tuple[float, float, float]:
        """(tc, sc, rwc), log2, as contraction_complexity reports them."""
        from . import order

        return order.complexity(self)

    def labels_of_nodes(self) -> list[list[int]]:
        """Output labels of every internal node under the derivation rule
        (operand labels still needed outside the subtree, union order)."""
        if self.node_iy is not None:
            return [list(x) for x in self.node_iy]
        return derive_node_labels(self.ixs, self.iy, self.children)

    def remove_labels(self, labels) -> "CompressedEinsum":
        """The same tree with ``labels`` deleted from every tensor (index
        slicing; the SlicedEinsum contents)."""
        rm = set(int(x) for x in labels)
        ixs = [[x for x in ix if x not in rm] for ix in self.ixs]
        iy = [x for x in self.iy if x not in rm]
        niy = None if self.node_iy is None else [[x for x in ix if x not in rm] for ix in self.node_iy]
        return CompressedEinsum(ixs, iy, self.children.copy(), niy, self.n_labels)


def derive_node_labels(ixs, iy, children) -> list[list[int]]:
    """Node output labels: labels of (left u right), in that order, that are
    still needed outside the subtree or are open; the root keeps iy."""
    T = len(ixs)
    count: dict[int, int] = {}
    lab = [list(dict.fromkeys(ix)) for ix in ixs]
    for ix in lab:
        for x in ix:
            count[x] = count.get(x, 0) + 1
    open_ = set(iy)
    cnt = [dict((x, 1) for x in ix) for ix in lab]
    out = []
    for j, (a, b) in enumerate(np.asarray(children).reshape(-1, 2)):
        a, b = int(a), int(b)
        uni = list(lab[a]) + [x for x in lab[b] if x not in lab[a]]
        c = {x: cnt[a].get(x, 0) + cnt[b].get(x, 0) for x in uni}
        keep = [x for x in uni if count[x] - c[x] > 0 or x in open_]
        lab.append(keep)
        cnt.append(c)
        out.append(keep)
    if out:
        out[-1] = list(iy)
    return out


@dataclass
class SlicedBranch:
    """A branch (slice) to contract: problem, plan and fixed weight r."""

    p: MISProblem
    code: CompressedEinsum | None
    r: float = 0.0
    sliced: list[int] = field(default_factory=list)      # labels fixed per item
    slice_values: np.ndarray | None = None               # (n_items, len(sliced)) int8
    order: list[int] | None = None                       # elimination order the tree was built from
    vmap: list[int] | None = None                        # branch vertex -> vertex of the sliced graph

    def complexity(self) -> tuple[float, float, float]:
        if self.code is None:
            return 0.0, 0.0, 0.0
        return self.code.complexity()

    def sc(self) -> float:
        return self.complexity()[1]

    def tc(self) -> float:
        return self.complexity()[0]


def add_r(branch: SlicedBranch, r: float) -> SlicedBranch:
    """add_r (src/types.jl:113)."""
    return SlicedBranch(branch.p, branch.code, branch.r + r, branch.sliced, branch.slice_values, branch.order,
                        branch.vmap)
