"""ctypes wrapper of the CPU oracle (libg5oracle.so).

TEST INFRASTRUCTURE ONLY: imported by the test suite, the smoke check and the
CPU-baseline leg of bench.py.  The product (gpugraph500_gb300) never imports
it.  See g5_oracle.h for what each function restates.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "libg5oracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libg5ref.so")
D4, DM = 0, 1

_lib = None


def build() -> None:
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        h = C.CDLL(LIB)
        P, I64, SZ = C.c_void_p, C.c_int64, C.c_size_t
        h.g5o_generate_kronecker.argtypes = [C.c_int, C.c_uint64, C.c_uint64, I64, I64, P]
        h.g5o_generate_kronecker_mt.argtypes = [C.c_int, C.c_uint64, C.c_uint64, I64, I64, P, C.c_int]
        h.g5o_build_csr.argtypes = [I64, P, I64, P, P]
        h.g5o_build_csr.restype = I64
        h.g5o_build_csr_mt.argtypes = [I64, P, I64, P, P, C.c_int]
        h.g5o_build_csr_mt.restype = I64
        h.g5o_endpoint_counts.argtypes = [I64, P, I64, P, C.c_int]
        h.g5o_teps_edges.argtypes = [I64, P, P]
        h.g5o_teps_edges.restype = I64
        h.g5o_bfs.argtypes = [I64, P, P, I64, P, P]
        h.g5o_validate.argtypes = [I64, P, I64, I64, P, C.POINTER(I64), P]
        h.g5o_codec_bound.argtypes = [SZ]
        h.g5o_codec_bound.restype = SZ
        h.g5o_codec_encode.argtypes = [P, SZ, P, C.c_int]
        h.g5o_codec_encode.restype = SZ
        h.g5o_codec_decode.argtypes = [P, SZ, P, SZ, C.c_int]
        h.g5o_codec_decode.restype = SZ
        h.g5o_plugin_compress.argtypes = [P, SZ, P, SZ, C.c_int]
        h.g5o_plugin_compress.restype = SZ
        h.g5o_plugin_decompress.argtypes = [P, SZ, SZ, P, SZ, C.c_int]
        h.g5o_plugin_decompress.restype = SZ
        h.g5o_bitmap_or.argtypes = [P, P, C.c_int, SZ]
        h.g5o_select_roots.argtypes = [I64, P, C.c_int, I64, P]
        h.g5o_mrg_skip_matrix.argtypes = [C.c_int, C.c_int, P]
        _lib = h
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data


def host_threads() -> int:
    """Host threads the oracle may use (all the cores this process may run on)."""
    try:
        return max(1, len(os.sched_getaffinity(0)))
    except (AttributeError, OSError):
        return max(1, os.cpu_count() or 1)


def kronecker(scale: int, seed1: int = 1, seed2: int = 2, edgefactor: int = 16,
              start: int = 0, end: int | None = None, threads: int = 0) -> np.ndarray:
    """Edges [start, end); threads = 0 uses every host thread, 1 the serial path."""
    m = edgefactor << scale
    end = m if end is None else end
    out = np.empty((end - start, 2), np.int64)
    t = threads or host_threads()
    if t == 1:
        lib().g5o_generate_kronecker(scale, seed1, seed2, start, end, _p(out))
    else:
        lib().g5o_generate_kronecker_mt(scale, seed1, seed2, start, end, _p(out), t)
    return out


def build_csr(n: int, edges: np.ndarray, threads: int = 1) -> tuple[np.ndarray, np.ndarray]:
    """threads = 1: one global sort (the reference's order of work); more (0 =
    every host thread): the counting build, identical arrays."""
    edges = np.ascontiguousarray(edges, dtype=np.int64)
    ro = np.empty(n + 1, np.int64)
    col = np.empty(max(2 * len(edges), 1), np.uint32)
    t = threads or host_threads()
    if t == 1:
        nnz = lib().g5o_build_csr(n, _p(edges), len(edges), _p(ro), _p(col))
    else:
        nnz = lib().g5o_build_csr_mt(n, _p(edges), len(edges), _p(ro), _p(col), t)
        if nnz < 0:
            raise MemoryError("g5o_build_csr_mt: host memory")
    return ro, col[:nnz].copy()


def endpoint_counts(n: int, edges: np.ndarray, threads: int = 0) -> np.ndarray:
    """Generated endpoints per vertex (duplicates included, self loops twice)."""
    edges = np.ascontiguousarray(edges, dtype=np.int64)
    out = np.empty(max(n, 1), np.uint32)
    lib().g5o_endpoint_counts(n, _p(edges), len(edges), _p(out), threads or host_threads())
    return out[:n]


def teps_edges(end_deg: np.ndarray, pred: np.ndarray) -> int:
    """TEPS edge count of a search from the endpoint counts (validate.h:440-443,485)."""
    end_deg = np.ascontiguousarray(end_deg, dtype=np.uint32)
    pred = np.ascontiguousarray(pred, dtype=np.int64)
    return int(lib().g5o_teps_edges(len(pred), _p(end_deg), _p(pred)))


def bfs(row_off: np.ndarray, col: np.ndarray, root: int) -> tuple[np.ndarray, np.ndarray]:
    n = len(row_off) - 1
    pred = np.empty(n, np.int64)
    level = np.empty(n, np.int32)
    lib().g5o_bfs(n, _p(row_off), _p(col) if len(col) else None, root, _p(pred), _p(level))
    return pred, level


def validate(n: int, edges: np.ndarray, root: int, pred: np.ndarray) -> tuple[bool, int, np.ndarray]:
    edges = np.ascontiguousarray(edges, dtype=np.int64)
    pred = np.ascontiguousarray(pred, dtype=np.int64)
    ne = C.c_int64()
    depth = np.empty(n, np.int32)
    ok = lib().g5o_validate(n, _p(edges), len(edges), root, _p(pred), C.byref(ne), _p(depth))
    return bool(ok), ne.value, depth


def encode(values: np.ndarray, mode: int = D4) -> np.ndarray:
    v = np.ascontiguousarray(values, dtype=np.uint32)
    out = np.zeros(lib().g5o_codec_bound(len(v)) + 8, np.uint32)
    w = lib().g5o_codec_encode(_p(v) if len(v) else None, len(v), _p(out), mode)
    return out[:w].copy()


def decode(stream: np.ndarray, cap: int, mode: int = D4) -> np.ndarray | None:
    s = np.ascontiguousarray(stream, dtype=np.uint32)
    out = np.zeros(max(cap, 1), np.uint32)
    n = lib().g5o_codec_decode(_p(s), len(s), _p(out), cap, mode)
    if n == C.c_size_t(-1).value:
        return None
    return out[:n].copy()


def plugin_compress(fq: np.ndarray, thr: int = 64, mode: int = DM) -> np.ndarray:
    fq = np.ascontiguousarray(fq, dtype=np.int64)
    out = np.zeros(lib().g5o_codec_bound(len(fq)) + 8, np.uint32)
    w = lib().g5o_plugin_compress(_p(fq) if len(fq) else None, len(fq), _p(out), thr, mode)
    return out[:w].copy()


def select_roots(row_off: np.ndarray, nroots: int = 64, maxgen: int = 32) -> np.ndarray:
    out = np.empty(max(nroots, 1), np.int64)
    k = lib().g5o_select_roots(len(row_off) - 1, _p(row_off), nroots, maxgen, _p(out))
    return out[:k].copy()


def bitmap_or(dst: np.ndarray, srcs: list[np.ndarray]) -> np.ndarray:
    d = np.ascontiguousarray(dst, dtype=np.uint64).copy()
    arr = (C.c_void_p * len(srcs))(*[s.ctypes.data for s in srcs])
    lib().g5o_bitmap_or(_p(d), arr, len(srcs), len(d))
    return d


def skip_matrix(byte_index: int, val: int) -> np.ndarray:
    out = np.empty(25, np.uint32)
    lib().g5o_mrg_skip_matrix(byte_index, val, _p(out))
    return out
