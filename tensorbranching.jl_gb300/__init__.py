"""GB300 tropical contraction engine for the hot path of TensorBranching.jl.

The contraction of every slice / branch of ``dynamic_ob_mis`` runs on the GPU
through the C ABI of ``include/tb.h`` (``_build/libtb.so``, built for
sm_103a).  This package is the host side: graphs, plans, orders, the
branching pipeline and the Python mirror of the reference API.
"""
from .engine import Engine, Plan, default_engine
from .graphs import Graph, random_ksg, random_regular_graph, random_weights
from .branching import FixedPointBrancher, GreedyBrancher, IPSolver, ScoreRS
from .mis import (LP_MWIS, ContractionTreeSlicer, KernelResult, VertexBrancher, contract_slices, dynamic_ob_mis,
                  eincode2order, index_slices, kernelize, slice, slice_dfs_lp, solve_slice, update_code, update_order)
from .network import (CompressedEinsum, MISProblem, SlicedBranch, UnitWeight, add_r, derive_node_labels,
                      rawcode)
from .order import GreedyMethod, TreeSA, complexity, greedy_slice, initialize_code, order2eincode, peak_memory
from . import branching, replicas, serving, slice_io

__all__ = [
    "Engine", "Plan", "default_engine", "Graph", "random_ksg", "random_regular_graph", "random_weights",
    "ContractionTreeSlicer", "KernelResult", "contract_slices", "dynamic_ob_mis", "eincode2order",
    "index_slices", "kernelize", "slice", "slice_dfs_lp", "LP_MWIS", "solve_slice", "update_code", "update_order", "CompressedEinsum", "MISProblem",
    "SlicedBranch", "UnitWeight", "add_r", "derive_node_labels", "rawcode", "GreedyMethod", "TreeSA",
    "complexity", "greedy_slice", "initialize_code", "order2eincode", "peak_memory",
    "ScoreRS", "GreedyBrancher", "FixedPointBrancher", "IPSolver", "VertexBrancher",
]
