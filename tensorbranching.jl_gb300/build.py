"""Build the native libraries in-tree.

* ``_build/libtb.so``      -- the CUDA engine behind ``include/tb.h`` (sm_103a)
* ``_build/libtborder.so`` -- host contraction-order tools (C++, no CUDA)

Both are compiled for the machine that runs this (the CUDA engine always for
``sm_103a``).  Builds are skipped when the outputs are newer than every source.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
INCLUDE = os.path.join(ROOT, "include")

ENGINE_SOURCES = ["engine.cu", "static_solve.cu", "plan.cpp", "kern_level_f32.cu", "kern_level_i32.cu",
                  "kern_persist_f32.cu", "kern_persist_i32.cu", "kern_misc_f32.cu", "kern_misc_i32.cu",
                  "score.cu"]
ENGINE_HEADERS = ["kernels.cuh", "device_kernels.cuh", "launch.h", "plan.h", "tb_internal.h"]
ORDER_SOURCES = ["order.cpp"]

ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA engine cannot be built")


def _stale(out: str, deps: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def engine_path() -> str:
    return os.path.join(OUT, "libtb.so")


def order_path() -> str:
    return os.path.join(OUT, "libtborder.so")


def build_engine(force: bool = False, extra: list[str] | None = None) -> str:
    out = engine_path()
    srcs = [os.path.join(CSRC, s) for s in ENGINE_SOURCES]
    deps = srcs + [os.path.join(CSRC, h) for h in ENGINE_HEADERS] + [os.path.join(INCLUDE, "tb.h")]
    if not force and not _stale(out, deps):
        return out
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    objs = []
    jobs = []
    for s in srcs:
        o = os.path.join(OUT, os.path.basename(s) + ".o")
        objs.append(o)
        if s.endswith(".cu"):
            jobs.append([nvcc, ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                         "-I", INCLUDE, "-c", s, "-o", o] + (extra or []))
        else:
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-I", INCLUDE, "-c", s, "-o", o])
    with ThreadPoolExecutor(len(jobs)) as ex:
        list(ex.map(_run, jobs))
    tmp = out + ".tmp"
    _run([nvcc, ARCH, "-shared", "-o", tmp] + objs + ["-lpthread"])
    os.replace(tmp, out)
    return out


def build_order(force: bool = False) -> str:
    out = order_path()
    srcs = [os.path.join(CSRC, s) for s in ORDER_SOURCES]
    if not force and not _stale(out, srcs):
        return out
    os.makedirs(OUT, exist_ok=True)
    tmp = out + ".tmp"
    _run(["g++", "-O3", "-std=c++17", "-shared", "-fPIC", "-o", tmp] + srcs + ["-lpthread"])
    os.replace(tmp, out)
    return out


def build_all(force: bool = False) -> list[str]:
    with ThreadPoolExecutor(2) as ex:
        f1 = ex.submit(build_engine, force)
        f2 = ex.submit(build_order, force)
        return [f1.result(), f2.result()]


if __name__ == "__main__":
    print("\n".join(build_all(force="--force" in sys.argv)))
