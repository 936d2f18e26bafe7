"""The reference's on-disk slice format (src/io.jl:1-121, src/slice.jl:16,45),
read and written so slices produced by the Julia slicer run on the GPU
unchanged.

A directory of finished slices holds, per slice id:

  graph_<id>.dot      the slice's graph as Graphs.jl ``savegraph`` writes it
                      (LG format: header ``nv,ne,u,<name>,<Int type>,simplegraph``
                      then one ``src,dst`` line per edge, 1-based); a DOT
                      file (``graph { 1 -- 2; ... }``) is read as well
  weights_<id>.txt    ``UnitWeight`` and n, or an element type name
                      (Float64, Float32, Int64, Int32) and one weight per line
  eincode_<id>.json   the contraction plan as OMEinsum ``writejson`` writes a
                      nested einsum: ``inputs`` (leaf label lists), ``output``,
                      ``tree`` = nested nodes, a leaf ``{"isleaf": true,
                      "tensorindex": i}`` (1-based), an internal node
                      ``{"isleaf": false, "eins": {"ixs": ..., "iy": ...},
                      "args": [...]}``; or the text ``nothing``
  slices.csv          columns ``id,sc,tc,r[,solution]``

Labels are vertex ids (1-based on disk, 0-based here).
"""
from __future__ import annotations

import csv
import json
import os
import re

import numpy as np

from .graphs import Graph
from .network import CompressedEinsum, MISProblem, SlicedBranch, UnitWeight


# ---------------------------------------------------------------------------
# graphs
# ---------------------------------------------------------------------------
def savegraph(filename: str, g: Graph, name: str = "graph") -> None:
    """LG format, as Graphs.jl ``savegraph(filename, g)``."""
    with open(filename, "w") as f:
        f.write(f"{g.n},{len(g.edges)},u,{name},Int64,simplegraph\n")
        for u, v in g.edges:
            f.write(f"{u + 1},{v + 1}\n")


def loadgraph(filename: str) -> Graph:
    with open(filename) as f:
        text = f.read()
    body = text.strip()
    if re.match(r"^(strict\s+)?(di)?graph\b", body) or "--" in body:
        return _load_dot(body)
    lines = [ln.strip() for ln in body.splitlines() if ln.strip() and not ln.startswith("#")]
    head = lines[0].split(",")
    n, ne = int(head[0]), int(head[1])
    if len(head) > 2 and head[2].strip() == "d":
        raise ValueError("directed graphs are not independent-set problems")
    edges = []
    for ln in lines[1:1 + ne]:
        a, b = ln.split(",")[:2]
        edges.append((int(a) - 1, int(b) - 1))
    if len(edges) != ne:
        raise ValueError(f"{filename}: header says {ne} edges, found {len(edges)}")
    return Graph(n, edges)


def _load_dot(body: str) -> Graph:
    inner = body[body.index("{") + 1:body.rindex("}")]
    nodes, edges = set(), []
    for stmt in re.split(r"[;\n]", inner):
        stmt = re.sub(r"\[.*?\]", "", stmt).strip()
        if not stmt or ("--" not in stmt and "=" in stmt):
            continue
        if "--" in stmt:
            parts = [p.strip().strip('"') for p in stmt.split("--")]
            ids = [int(p) for p in parts]
            nodes.update(ids)
            edges.extend((a - 1, b - 1) for a, b in zip(ids, ids[1:]))
        elif re.fullmatch(r'"?\d+"?', stmt):
            nodes.add(int(stmt.strip('"')))
    n = max(nodes) if nodes else 0
    return Graph(n, edges)


# ---------------------------------------------------------------------------
# weights (src/io.jl:1-44)
# ---------------------------------------------------------------------------
_WTYPES = {"Float64": np.float64, "Float32": np.float32, "Int64": np.int64, "Int32": np.int32}


def save_weights(filename: str, weights) -> None:
    with open(filename, "w") as f:
        if isinstance(weights, UnitWeight):
            f.write(f"UnitWeight\n{weights.n}\n")
            return
        w = np.asarray(weights)
        name = {np.dtype(np.float64): "Float64", np.dtype(np.float32): "Float32", np.dtype(np.int64): "Int64",
                np.dtype(np.int32): "Int32"}.get(w.dtype)
        if name is None:
            raise ValueError(f"unsupported weight type {w.dtype}")
        f.write(name + "\n")
        for x in w:
            f.write(f"{repr(float(x))}\n" if name.startswith("Float") else f"{int(x)}\n")


def load_weights(filename: str):
    with open(filename) as f:
        first = f.readline().strip()
        if first == "UnitWeight":
            return UnitWeight(int(f.readline().strip()))
        if first not in _WTYPES:
            raise ValueError(f"Unknown weight type: {first}")
        # Julia's Float32 literals may carry an f exponent (1.5f0)
        return np.array([float(x.replace("f", "e")) for x in f.read().split()], dtype=_WTYPES[first])


# ---------------------------------------------------------------------------
# contraction plans (src/io.jl:58-79)
# ---------------------------------------------------------------------------
def _node_to_dict(code: CompressedEinsum, labs, x: int):
    T = code.n_tensors
    if x < T:
        return {"isleaf": True, "tensorindex": x + 1}
    j = x - T
    a, b = (int(y) for y in code.children[j])
    ixs = [[v + 1 for v in labs[a]], [v + 1 for v in labs[b]]]
    return {"isleaf": False, "eins": {"ixs": ixs, "iy": [v + 1 for v in labs[x]]},
            "args": [_node_to_dict(code, labs, a), _node_to_dict(code, labs, b)]}


def save_code(filename: str, code: CompressedEinsum | None) -> None:
    """A nested einsum in the layout OMEinsum ``writejson`` uses."""
    with open(filename, "w") as f:
        if code is None:
            f.write("nothing")
            return
        labs = [list(dict.fromkeys(ix)) for ix in code.ixs] + code.labels_of_nodes()
        root = code.n_tensors + code.n_nodes - 1 if code.n_nodes else 0
        d = {"label-type": "Int64", "inputs": [[v + 1 for v in ix] for ix in code.ixs],
             "output": [v + 1 for v in code.iy], "tree": _node_to_dict(code, labs, root)}
        json.dump(d, f)


def _binary(node, ch, node_iy, T):
    """Post-order pairs of a nested einsum node (n-ary nodes folded left to
    right); returns the node's tensor id."""
    if node.get("isleaf"):
        return int(node["tensorindex"]) - 1
    args = node["args"]
    iy = [int(v) - 1 for v in node.get("eins", {}).get("iy", [])]
    ids = [_binary(a, ch, node_iy, T) for a in args]
    if len(ids) == 1:
        raise ValueError("unary einsum nodes are not contraction steps")
    cur = ids[0]
    for k, y in enumerate(ids[1:]):
        ch.append((cur, y))
        node_iy.append(iy if k == len(ids) - 2 else None)
        cur = T + len(ch) - 1
    return cur


def load_code(filename: str, n_labels: int = 0) -> CompressedEinsum | None:
    with open(filename) as f:
        text = f.read()
    if text.strip() == "nothing":
        return None
    d = json.loads(text)
    ixs = [[int(v) - 1 for v in ix] for ix in d["inputs"]]
    iy = [int(v) - 1 for v in d.get("output", [])]
    tree = d.get("tree", d)
    ch, niy = [], []
    _binary(tree, ch, niy, len(ixs))
    if len(ch) != len(ixs) - 1:
        raise ValueError("the tree does not contract every input exactly once")
    node_iy = None
    if all(x is not None for x in niy):
        node_iy = niy
        node_iy[-1] = iy
    m = max([max(ix) for ix in ixs if ix] + [max(iy) if iy else -1]) + 1
    return CompressedEinsum(ixs, iy, np.array(ch, np.int32).reshape(-1, 2), node_iy, max(n_labels, m))


# ---------------------------------------------------------------------------
# finished slices (src/io.jl:81-121)
# ---------------------------------------------------------------------------
def save_finished(dirname: str, branch: SlicedBranch, id: int) -> None:
    savegraph(os.path.join(dirname, f"graph_{id}.dot"), branch.p.g)
    save_code(os.path.join(dirname, f"eincode_{id}.json"), branch.code)
    save_weights(os.path.join(dirname, f"weights_{id}.txt"), branch.p.weights
                 if branch.p.weights is not None else UnitWeight(branch.p.g.n))


def load_finished(dirname: str, id: int):
    g = loadgraph(os.path.join(dirname, f"graph_{id}.dot"))
    code = load_code(os.path.join(dirname, f"eincode_{id}.json"), g.n)
    weights = load_weights(os.path.join(dirname, f"weights_{id}.txt"))
    return g, code, weights


def save_slices_csv(dirname: str, rows) -> None:
    """rows: (id, sc, tc, r[, solution])."""
    with open(os.path.join(dirname, "slices.csv"), "w", newline="") as f:
        w = csv.writer(f)
        n = len(rows[0]) if rows else 4
        w.writerow(["id", "sc", "tc", "r", "solution"][:n])
        for row in rows:
            w.writerow(row)


def load_all_finished(dirname: str) -> list[SlicedBranch]:
    """Every finished slice of a directory as SlicedBranch (r from slices.csv)."""
    out = []
    with open(os.path.join(dirname, "slices.csv"), newline="") as f:
        for row in csv.DictReader(f):
            id = int(row["id"])
            g, code, weights = load_finished(dirname, id)
            w = weights if isinstance(weights, UnitWeight) else np.asarray(weights, np.float32)
            out.append(SlicedBranch(MISProblem(g, w), code, float(row["r"])))
    return out
