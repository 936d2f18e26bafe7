"""ORACLE -- test infrastructure only.

Python face of the CPU restatement in ``tropical.c`` (see its header for
what it restates and why parity with the Julia implementation itself is
unpinned), plus a third, pure-numpy restatement of the binary tropical
einsum for small cases.  Only tests/, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` leg of bench.py import this module; the product never does.

Reference call sites these functions stand for:
  code(tensors...) on a binary DynamicNestedEinsum      test/utils.jl:34
  solve(GenericTensorNetwork(IndependentSet(g, w), code), SizeMax(), T)
                                                        src/dynamic_ob.jl:31-32
  generate_tensors(TropicalF32(1.0), IndependentSet(g)) test/utils.jl:24
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from ctypes import c_int, c_void_p

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")

_lib = None


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "tropical.c")
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
        r = subprocess.run(["make", "-C", HERE, "-B" if force else "all"], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(LIB)
        for sfx in ("f32", "i32"):
            f = getattr(_lib, f"or_einsum_naive_{sfx}")
            f.restype = c_int
            f.argtypes = [c_int, c_void_p, c_void_p, c_int, c_void_p, c_void_p, c_int, c_void_p, c_void_p]
            f = getattr(_lib, f"or_einsum_gemm_{sfx}")
            f.restype = c_int
            f.argtypes = [c_int, c_void_p, c_void_p, c_int, c_void_p, c_void_p, c_int, c_void_p, c_void_p]
            _lib.or_set_threads.restype = None
            _lib.or_set_threads.argtypes = [c_int]
            _lib.or_get_threads.restype = c_int
            _lib.or_get_threads.argtypes = []
            f = getattr(_lib, f"or_execute_{sfx}")
            f.restype = c_int
            f.argtypes = [c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_void_p, c_void_p, c_int,
                          c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_int]
    return _lib


I32_NEG = -536870912


def set_threads(n: int = 0) -> int:
    """OpenMP threads of later oracle calls (0: every host core); returns the
    count now in effect."""
    lib().or_set_threads(int(n))
    return int(lib().or_get_threads())


def _i(a):
    a = np.ascontiguousarray(a, dtype=np.int32)
    return a if a.size else np.zeros(1, np.int32)


def einsum(ia, A, ib, B, ic, mode: str = "naive", dtype=np.float32) -> np.ndarray:
    """C[ic] = max over the other labels of A[ia] (+ B[ib]); column-major."""
    L = lib()
    sfx = "i32" if np.dtype(dtype) == np.int32 else "f32"
    f = getattr(L, f"or_einsum_{mode}_{sfx}")
    A = np.ascontiguousarray(A, dtype=dtype)
    Bc = None if B is None else np.ascontiguousarray(B, dtype=dtype)
    C = np.zeros(1 << len(ic), dtype)
    ia_, ib_, ic_ = _i(ia), _i(ib if ib is not None else []), _i(ic)
    rc = f(len(ia), ia_.ctypes.data, A.ctypes.data, 0 if B is None else len(ib), ib_.ctypes.data,
           None if Bc is None else Bc.ctypes.data, len(ic), ic_.ctypes.data, C.ctypes.data)
    if rc:
        raise ValueError(f"oracle einsum failed ({rc})")
    return C


def einsum_numpy(ia, A, ib, B, ic) -> np.ndarray:
    """Pure-numpy tropical einsum (small cases): broadcast, add, max."""
    labels = list(dict.fromkeys(list(ia) + list(ib or [])))
    pos = {x: i for i, x in enumerate(labels)}

    def expand(ix, X):
        X = np.asarray(X, np.float64).reshape((2,) * len(ix), order="F") if ix else np.asarray(X, np.float64).reshape(())
        # diagonal for repeated labels
        uniq = list(dict.fromkeys(ix))
        if len(uniq) != len(ix):
            idx = np.indices((2,) * len(uniq))
            sel = tuple(idx[uniq.index(x)] for x in ix)
            X = X[sel]
        shape = [1] * len(labels)
        order = sorted(range(len(uniq)), key=lambda k: pos[uniq[k]])
        X = np.transpose(X, order) if uniq else X
        for k in order:
            shape[pos[uniq[k]]] = 2
        return X.reshape(shape)

    S = expand(ia, A)
    if B is not None:
        S = S + expand(ib, B)
    S = np.broadcast_to(S, (2,) * len(labels))
    red = tuple(i for i, x in enumerate(labels) if x not in ic)
    R = S.max(axis=red) if red else S
    keep = [x for x in labels if x in ic]
    R = np.transpose(R, [keep.index(x) for x in ic]) if ic else R
    return np.asarray(R, np.float32).ravel(order="F")


def mis_leaf(ix, w):
    """GenericTensorNetworks IndependentSet tensor of one leaf."""
    if len(ix) == 1:
        return np.array([0.0, w[ix[0]]], np.float32)
    return np.array([0.0, 0.0, 0.0, -np.inf], np.float32)


def execute(code, weights=None, node_iy=None, sliced=(), slice_vals=(), mode: str = "gemm",
            dtype=np.float32, leaf_data=None, dump: bool = False):
    """Contract a CompressedEinsum on the CPU.  Returns the root tensor and,
    with dump=True, every internal node's tensor (node_iy order)."""
    L = lib()
    sfx = "i32" if np.dtype(dtype) == np.int32 else "f32"
    f = getattr(L, f"or_execute_{sfx}")
    T = code.n_tensors
    off, lab = code.csr()
    if node_iy is None:
        node_iy = code.labels_of_nodes()
    if T == 1:
        node_iy = [list(code.iy)]
    noff = np.zeros(len(node_iy) + 1, np.int32)
    noff[1:] = np.cumsum([len(x) for x in node_iy])
    nlab = _i([x for ix in node_iy for x in ix])
    w = np.zeros(max(code.n_labels, 1), dtype)
    if weights is not None:
        w[: len(weights)] = np.asarray(weights, dtype)
    fix = _i(list(sliced))
    fv = np.ascontiguousarray(np.asarray(list(slice_vals) if len(sliced) else [0], np.int8))
    ch = code.children if code.n_nodes else np.zeros((1, 2), np.int32)
    keepalive = []
    leaf_ptrs = None
    if leaf_data is not None:
        arrs = []
        for x in leaf_data:
            a = np.ascontiguousarray(np.asarray(x, np.float32).ravel(order="F"))
            if np.dtype(dtype) == np.int32:
                a = np.where(np.isinf(a), I32_NEG, a).astype(np.int32)
            arrs.append(a)
        keepalive.append(arrs)
        leaf_ptrs = (c_void_p * T)(*[a.ctypes.data for a in arrs])
    root_rank = len([x for x in (code.iy if T > 1 else node_iy[0]) if x not in set(sliced)])
    out = np.zeros(1 << root_rank, dtype)
    dumps = None
    dump_ptrs = None
    if dump and code.n_nodes:
        sl = set(sliced)
        dumps = [np.zeros(1 << len([x for x in ix if x not in sl]), dtype) for ix in node_iy]
        dump_ptrs = (c_void_p * len(dumps))(*[d.ctypes.data for d in dumps])
    rc = f(T, off.ctypes.data, lab.ctypes.data, None if leaf_ptrs is None else ctypes.cast(leaf_ptrs, c_void_p),
           w.ctypes.data, len(sliced), fix.ctypes.data, fv.ctypes.data, code.n_nodes, ch.ctypes.data,
           noff.ctypes.data, nlab.ctypes.data, out.ctypes.data,
           None if dump_ptrs is None else ctypes.cast(dump_ptrs, c_void_p), 0 if mode == "naive" else 1)
    if rc:
        raise ValueError(f"oracle execute failed ({rc})")
    if np.dtype(dtype) == np.int32:
        out = np.where(out <= I32_NEG // 2, -np.inf, out).astype(np.float32)
        if dumps is not None:
            dumps = [np.where(d <= I32_NEG // 2, -np.inf, d).astype(np.float32) for d in dumps]
    return (out, dumps) if dump else out


def solve(code, weights, sliced=(), slice_vals=(), mode: str = "gemm", dtype=np.float32) -> float:
    """max over the root tensor: the MIS value of the (sliced) network."""
    return float(np.max(execute(code, weights, None, sliced, slice_vals, mode, dtype)))
