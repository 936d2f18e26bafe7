"""Contraction-order tools (host side, C++ in csrc/order.cpp).

Restates what the reference obtains from OMEinsumContractionOrders:
``initialize_code`` (src/dynamic_ob.jl:50-54, a TreeSA order of
IndependentSet(g)), ``order2eincode`` (src/decompose.jl:64-94), the TreeSA
refinement behind ``rethermalize`` (src/utils.jl:142-144) and ``refine``
(src/refine.jl), ``contraction_complexity`` (src/types.jl:115-121) and
``contraction_peak_memory`` (src/utils.jl:197-219).
"""
from __future__ import annotations

import os
from dataclasses import dataclass, field

import numpy as np

from . import _native
from .graphs import Graph
from .network import CompressedEinsum, rawcode


@dataclass
class GreedyMethod:
    """Min-fill elimination order turned into a tree."""

    seed: int = 0


@dataclass
class TreeSA:
    """Simulated annealing over tree rotations (OMEinsumContractionOrders
    TreeSA), started from a min-fill tree."""

    sc_target: float = 20.0
    betas: np.ndarray = field(default_factory=lambda: np.arange(0.3, 20.0, 0.2))
    ntrials: int = 8
    niters: int = 200
    sc_weight: float = 1.0
    rw_weight: float = 0.0
    seed: int = 0
    nthreads: int = 0


def _args(code: CompressedEinsum):
    off, lab = code.csr()
    iy = np.array(code.iy if code.iy else [0], np.int32)
    return off, lab, iy


def complexity(code: CompressedEinsum) -> tuple[float, float, float]:
    lib = _native.order_lib()
    off, lab, iy = _args(code)
    out = np.zeros(3)
    ch = code.children if code.n_nodes else np.zeros((1, 2), np.int32)
    rc = lib.tbo_complexity(code.n_tensors, off.ctypes.data, lab.ctypes.data, code.n_labels, len(code.iy),
                            iy.ctypes.data, ch.ctypes.data, out.ctypes.data)
    if rc:
        raise ValueError("invalid contraction tree")
    return float(out[0]), float(out[1]), float(out[2])


def peak_memory(code: CompressedEinsum) -> float:
    """log2 of the peak live elements of a post-order evaluation."""
    lib = _native.order_lib()
    off, lab, iy = _args(code)
    out = np.zeros(1)
    ch = code.children if code.n_nodes else np.zeros((1, 2), np.int32)
    rc = lib.tbo_peak_memory(code.n_tensors, off.ctypes.data, lab.ctypes.data, code.n_labels, len(code.iy),
                             iy.ctypes.data, ch.ctypes.data, out.ctypes.data)
    if rc:
        raise ValueError("invalid contraction tree")
    return float(out[0])


def minfill_order(ixs, n_labels: int, seed: int = 0) -> np.ndarray:
    lib = _native.order_lib()
    code = CompressedEinsum(ixs, [], np.zeros((max(len(ixs) - 1, 0), 2), np.int32), n_labels=n_labels)
    off, lab = code.csr()
    order = np.zeros(max(n_labels, 1), np.int32)
    rc = lib.tbo_minfill_order(len(ixs), off.ctypes.data, lab.ctypes.data, n_labels, seed, order.ctypes.data)
    if rc:
        raise ValueError("invalid network")
    return order[:n_labels]


def tree_from_order(ixs, iy, n_labels: int, order) -> CompressedEinsum:
    lib = _native.order_lib()
    T = len(ixs)
    tmp = CompressedEinsum(ixs, iy, np.zeros((max(T - 1, 0), 2), np.int32), n_labels=n_labels)
    off, lab, iya = _args(tmp)
    order = np.ascontiguousarray(order, dtype=np.int32)
    ch = np.zeros((max(T - 1, 1), 2), np.int32)
    rc = lib.tbo_tree_from_order(T, off.ctypes.data, lab.ctypes.data, n_labels, len(iy), iya.ctypes.data,
                                 len(order), order.ctypes.data if len(order) else iya.ctypes.data, ch.ctypes.data)
    if rc:
        raise ValueError("tree_from_order failed")
    return CompressedEinsum(ixs, iy, ch[: max(T - 1, 0)], n_labels=n_labels)


def order2eincode(g: Graph, eo) -> CompressedEinsum:
    """Contraction tree of IndependentSet(g) from an elimination order
    (src/decompose.jl:64-94; isolated vertices and disconnected components
    are merged at the end)."""
    ixs, iy = rawcode(g)
    return tree_from_order(ixs, iy, g.n, [v for v in eo if 0 <= v < g.n])


def greedy_tree(ixs, iy, n_labels: int, seed: int = 0) -> CompressedEinsum:
    """Greedy pairwise contraction tree (contract the pair whose result grows
    the least first; OMEinsumContractionOrders GreedyMethod)."""
    lib = _native.order_lib()
    T = len(ixs)
    tmp = CompressedEinsum(ixs, iy, np.zeros((max(T - 1, 0), 2), np.int32), n_labels=n_labels)
    off, lab, iya = _args(tmp)
    ch = np.zeros((max(T - 1, 1), 2), np.int32)
    rc = lib.tbo_greedy_tree(T, off.ctypes.data, lab.ctypes.data, n_labels, len(iy), iya.ctypes.data, seed,
                             ch.ctypes.data)
    if rc:
        raise ValueError("greedy_tree failed")
    return CompressedEinsum(ixs, iy, ch[: max(T - 1, 0)], n_labels=n_labels)


def treesa(code: CompressedEinsum, opt: TreeSA) -> CompressedEinsum:
    """Refine a tree with simulated annealing; returns a new plan."""
    if code.n_tensors <= 2:
        return code
    lib = _native.order_lib()
    off, lab, iy = _args(code)
    ch = np.ascontiguousarray(code.children.copy())
    betas = np.ascontiguousarray(opt.betas, dtype=np.float64)
    out = np.zeros(3)
    nthreads = opt.nthreads or (os.cpu_count() or 1)
    rc = lib.tbo_treesa(code.n_tensors, off.ctypes.data, lab.ctypes.data, code.n_labels, len(code.iy),
                        iy.ctypes.data, ch.ctypes.data, float(opt.sc_target), float(opt.sc_weight),
                        float(opt.rw_weight), betas.ctypes.data, len(betas), int(opt.niters), int(opt.ntrials),
                        int(nthreads), int(opt.seed), out.ctypes.data)
    if rc:
        raise ValueError("treesa failed")
    return CompressedEinsum(code.ixs, code.iy, ch, None, code.n_labels)


def optimize_code(ixs, iy, n_labels: int, optimizer) -> CompressedEinsum:
    seed = getattr(optimizer, "seed", 0)
    order = minfill_order(ixs, n_labels, seed)
    code = tree_from_order(ixs, iy, n_labels, order)
    if isinstance(optimizer, TreeSA):
        code = treesa(code, optimizer)
    return code


def initialize_code(g: Graph, optimizer=None) -> CompressedEinsum:
    """Contraction plan of IndependentSet(g) (initialize_code,
    src/dynamic_ob.jl:50-54)."""
    optimizer = optimizer if optimizer is not None else TreeSA()
    ixs, iy = rawcode(g)
    if g.n == 0:
        raise ValueError("empty graph has no tensor network")
    return optimize_code(ixs, iy, g.n, optimizer)


def greedy_slice(code: CompressedEinsum, sc_target: float, max_slices: int = 64):
    """Labels to fix (index slicing) until sc <= sc_target."""
    lib = _native.order_lib()
    off, lab, iy = _args(code)
    sliced = np.zeros(max(max_slices, 1), np.int32)
    ns = np.zeros(1, np.int32)
    out = np.zeros(3)
    ch = code.children if code.n_nodes else np.zeros((1, 2), np.int32)
    rc = lib.tbo_greedy_slice(code.n_tensors, off.ctypes.data, lab.ctypes.data, code.n_labels, len(code.iy),
                              iy.ctypes.data, ch.ctypes.data, float(sc_target), int(max_slices),
                              sliced.ctypes.data, ns.ctypes.data, out.ctypes.data)
    if rc:
        raise ValueError("greedy_slice failed")
    return [int(x) for x in sliced[: int(ns[0])]], (float(out[0]), float(out[1]), float(out[2]))
