"""Builds libg5bfs.so (the CUDA hot path) in-tree for sm_103a.

One nvcc per translation unit, compiled in parallel, then one link.  The
library lands next to this file; the Python layer loads it from there.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libg5bfs.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["g5_graph.cu", "g5_bfs.cu", "g5_codec.cu", "g5_bitmap.cu", "g5_batch.cu"]
CPP_SOURCES = ["g5_host.cpp", "g5_server.cpp"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout)


def build(verbose: bool = False) -> str:
    """Compiles every source that exists and links libg5bfs.so; returns its path."""
    nvcc = _nvcc()
    os.makedirs(OBJ, exist_ok=True)
    common = ["-O3", "-std=c++17", "-I" + INCLUDE, "-I" + CSRC, "-Xcompiler", "-fPIC"]
    jobs = []
    for src in CU_SOURCES:
        path = os.path.join(CSRC, src)
        if not os.path.exists(path):
            continue
        obj = os.path.join(OBJ, src + ".o")
        jobs.append([nvcc, *ARCH, "-lineinfo", *common, "-c", path, "-o", obj])
    for src in CPP_SOURCES:
        path = os.path.join(CSRC, src)
        if not os.path.exists(path):
            continue
        obj = os.path.join(OBJ, src + ".o")
        jobs.append([nvcc, *common, "-x", "c++", "-c", path, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        for f in [ex.submit(_run, j) for j in jobs]:
            f.result()
    objs = [j[-1] for j in jobs]
    tmp = LIB + ".tmp"
    _run([nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart_static", "-lpthread", "-ldl", "-lrt"])
    os.replace(tmp, LIB)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
