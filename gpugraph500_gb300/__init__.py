"""GB300-native BFS hot path of gpugraph500.

Python mirror of the reference's host interfaces over the C ABI of
libg5bfs.so (include/g5bfs.h):

* ``CudaBFS``      -- ``runBFS(start)`` / ``getPredecessor()`` of the
  reference's GlobalBFS + CUDA_BFS pair (cpu_2d/globalbfs.hh:548,
  cpu_2d/cuda/cuda_bfs.h:39-84) on a 1x1 grid.
* ``GpuSimd``      -- the ``Compression<int64_t, uint32_t>`` plugin of
  cpu_2d/compression/compression.hh:11-28 (CpuSimd, cpusimd.hh), encoding
  on the GPU.
* ``Graph``, ``Codec``, ``Batch``, ``bitmap_or``, ``select_roots`` -- the
  remaining entry points.

The CUDA library is required: importing works without it, but every call
raises ``G5Error`` if libg5bfs.so is missing or no GPU is visible.  There is
no CPU implementation behind these classes.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional, Sequence

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libg5bfs.so")

STATUS = {
    0: "ok", 1: "out of memory", 2: "capacity exceeded", 3: "invalid argument",
    4: "timeout", 5: "corrupt codec stream", 6: "CUDA error", 7: "no CUDA device",
    8: "round-trip mismatch",
}
G5_OK, G5_ERR_OOM, G5_ERR_CAPACITY, G5_ERR_INVALID_ARG = 0, 1, 2, 3
G5_ERR_TIMEOUT, G5_ERR_CORRUPT_STREAM, G5_ERR_CUDA, G5_ERR_NO_DEVICE, G5_ERR_MISMATCH = 4, 5, 6, 7, 8
G5_ERR_IO = 9

CODEC_NONE, CODEC_D4, CODEC_DM = 0, 1, 2
CODEC_NAMES = {"s4-bp128-d4": CODEC_D4, "s4-bp128-dm": CODEC_DM}


class G5Error(RuntimeError):
    def __init__(self, code: int, what: str = ""):
        self.code = code
        super().__init__(f"{what}: {STATUS.get(code, code)}" if what else STATUS.get(code, str(code)))


class BfsConfig(C.Structure):
    _fields_ = [("alpha", C.c_double), ("beta", C.c_double), ("codec", C.c_int),
                ("codec_threshold", C.c_uint32), ("use_graph", C.c_int),
                ("max_levels", C.c_int), ("want_levels", C.c_int), ("profile", C.c_int),
                ("parent_mode", C.c_int), ("tile_edges", C.c_uint32), ("bu_serial", C.c_int)]


class BfsStats(C.Structure):
    _fields_ = [("levels", C.c_int32), ("bottom_up_levels", C.c_int32), ("visited", C.c_int64),
                ("edges_td", C.c_int64), ("edges_bu", C.c_int64), ("queue_total", C.c_int64),
                ("codec_words", C.c_int64), ("codec_values", C.c_int64), ("alg_bytes", C.c_int64),
                ("device_ms", C.c_double), ("kernel_ms", C.c_double * 8)]

    KERNELS = ("prologue", "expand", "fixup", "count", "scan", "write", "codec", "host")

    def as_dict(self) -> dict:
        d = {k: getattr(self, k) for k, _ in self._fields_ if k != "kernel_ms"}
        d["kernel_ms"] = dict(zip(self.KERNELS, list(self.kernel_ms)))
        return d


_lib_handle = None

# name -> (restype, argtypes); every symbol of include/g5bfs.h
_P, _I64, _U64, _SZ, _I, _U32 = C.c_void_p, C.c_int64, C.c_uint64, C.c_size_t, C.c_int, C.c_uint32
SIGNATURES = {
    "g5_status_str": (C.c_char_p, [_I]),
    "g5_version": (_U32, []),
    "g5_graph_create": (_I, [_P, _P, _I64, _I64, C.POINTER(_P)]),
    "g5_graph_generate_kronecker": (_I, [_I, _I, _U64, _U64, C.POINTER(_P)]),
    "g5_kronecker_edges": (_I, [_I, _U64, _U64, _I64, _I64, _P]),
    "g5_graph_info": (_I, [_P, C.POINTER(_I64), C.POINTER(_I64)]),
    "g5_graph_copy_csr": (_I, [_P, _P, _P]),
    "g5_graph_device_csr": (_I, [_P, C.POINTER(_P), C.POINTER(_P)]),
    "g5_graph_destroy": (_I, [_P]),
    "g5_graph_save": (_I, [_P, C.c_char_p]),
    "g5_graph_load": (_I, [C.c_char_p, C.POINTER(_P)]),
    "g5_graph_kronecker_info": (_I, [_P, C.POINTER(C.c_int), C.POINTER(_I64)]),
    "g5_select_roots": (_I, [_P, _I, _I64, _P, C.POINTER(_I)]),
    "g5_bfs_config_default": (None, [C.POINTER(BfsConfig)]),
    "g5_bfs_create": (_I, [_P, C.POINTER(BfsConfig), C.POINTER(_P)]),
    "g5_bfs_destroy": (_I, [_P]),
    "g5_bfs_run": (_I, [_P, _I64, _P, _P, C.POINTER(BfsStats)]),
    "g5_bfs_level_log": (_I, [_P, _P, _I, C.POINTER(_I)]),
    "g5_bfs_profile_log": (_I, [_P, _P, _P, _I, C.POINTER(_I)]),
    "g5_bfs_device_pred": (_I, [_P, C.POINTER(_P)]),
    "g5_bfs_run_many": (_I, [_P, _P, _I, _P, _P]),
    "g5_bfs_codec_capture": (_I, [_P, _P, _U64, _P, _I]),
    "g5_bfs_codec_captured": (_I, [_P, C.POINTER(_I), C.POINTER(_I)]),
    "g5_bfs_teps_edges": (_I, [_P, C.POINTER(_I64)]),
    "g5_bfs_validate": (_I, [_P, _I64, C.POINTER(_I), C.POINTER(_I)]),
    "g5_batch_create": (_I, [_P, _I, C.POINTER(_P)]),
    "g5_batch_destroy": (_I, [_P]),
    "g5_batch_set_direction": (_I, [_P, C.c_double, C.c_double]),
    "g5_batch_profile": (_I, [_P, _P, _P, _P, _P, _P, _P, _P, _P, _I, C.POINTER(_I)]),
    "g5_batch_run": (_I, [_P, _P, _P, _P, C.POINTER(C.c_double)]),
    "g5_batch_root_parents": (_I, [_P, C.c_int64, _I, _I, _P, _P]),
    "g5_batch_launch": (_I, [_P, _P, _P, _P]),
    "g5_batch_poll": (_I, [_P, _I, C.POINTER(_I), C.POINTER(C.c_double)]),
    "g5_batch_serve_begin": (_I, [_P, _P, _P]),
    "g5_batch_serve_step": (_I, [_P, _P, _P, _P, _I, _P, _P, C.POINTER(C.c_double)]),
    "g5_bfs_launch": (_I, [_P, _I64]),
    "g5_bfs_poll": (_I, [_P, C.POINTER(_I), C.POINTER(C.c_double)]),
    "g5_server_create": (_I, [_P, _I, _SZ, _I, _I, C.POINTER(_P)]),
    "g5_server_create_modes": (_I, [_P, _I, _SZ, _I, _P, C.POINTER(_P)]),
    "g5_server_slots": (_I, [_P, _P]),
    "g5_server_cohort_policy": (_I, [_P, _I, C.c_double]),
    "g5_server_submit": (_I, [_P, _I, _I64, C.POINTER(_U64)]),
    "g5_server_wait": (_I, [_P, _U64, C.c_double, C.POINTER(_I)]),
    "g5_server_result": (_I, [_P, _U64, _P, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "g5_server_stats": (_I, [_P, C.POINTER(_U64), C.POINTER(_U64), C.POINTER(C.c_double)]),
    "g5_server_destroy": (_I, [_P]),
    "g5_codec_bound": (_SZ, [_SZ]),
    "g5_codec_create": (_I, [_SZ, C.POINTER(_P)]),
    "g5_codec_destroy": (_I, [_P]),
    "g5_codec_batch_bound": (_SZ, [_P, _I]),
    "g5_codec_encode_batch": (_I, [_P, _P, _P, _I, _P, _P, _P, _U32, _I, _P]),
    "g5_codec_decode_batch": (_I, [_P, _P, _P, _P, _P, _I, _P, _P, _P, _U32, _I, _P]),
    "g5_codec_encode": (_I, [_P, _P, _SZ, _P, C.POINTER(_SZ), _I, _P]),
    "g5_codec_encode_async": (_I, [_P, _P, _P, _P, _P, _I, _P]),
    "g5_codec_decode_async": (_I, [_P, _P, _P, _P, _SZ, _P, _I, _P]),
    "g5_codec_status": (_I, [_P]),
    "g5_codec_decode": (_I, [_P, _P, _SZ, _P, _SZ, C.POINTER(_SZ), _I, _P]),
    "g5_codec_encode_noalloc": (_I, [_P, _SZ, _P, C.POINTER(_SZ), _I, _P]),
    "g5_plugin_compress": (_I, [_P, _SZ, C.POINTER(_P), C.POINTER(_SZ), _U32, _I]),
    "g5_plugin_decompress": (_I, [_P, _SZ, C.POINTER(_P), C.POINTER(_SZ), _U32, _I]),
    "g5_bitmap_or": (_I, [_P, _P, _I, _SZ, _P]),
}


def lib():
    """Loads libg5bfs.so (raises if it was not built)."""
    global _lib_handle
    if _lib_handle is None:
        if not os.path.exists(LIB_PATH):
            raise G5Error(G5_ERR_NO_DEVICE, f"{LIB_PATH} is missing; run __graft_entry__.build()")
        h = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            if hasattr(h, name):
                f = getattr(h, name)
                f.restype = res
                f.argtypes = args
        _lib_handle = h
    return _lib_handle


def _check(code: int, what: str) -> None:
    if code != G5_OK:
        raise G5Error(code, what)


def _ptr(a) -> int:
    """Address of a numpy array, a torch tensor or an int."""
    if a is None:
        return None
    if isinstance(a, int):
        return a
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return a.data_ptr()  # torch tensor (device buffers)


class Graph:
    """A symmetric CSR resident in HBM (g5_graph)."""

    def __init__(self, handle: int, scale: Optional[int] = None):
        self._h = C.c_void_p(handle)
        n, nnz = C.c_int64(), C.c_int64()
        _check(lib().g5_graph_info(self._h, C.byref(n), C.byref(nnz)), "g5_graph_info")
        self.n, self.nnz, self.scale = n.value, nnz.value, scale

    @classmethod
    def from_csr(cls, row_off: np.ndarray, col: np.ndarray) -> "Graph":
        row_off = np.ascontiguousarray(row_off, dtype=np.int64)
        col = np.ascontiguousarray(col, dtype=np.uint32)
        h = C.c_void_p()
        n = len(row_off) - 1
        _check(lib().g5_graph_create(_ptr(row_off), _ptr(col) if len(col) else None, n, len(col),
                                     C.byref(h)), "g5_graph_create")
        return cls(h.value)

    @classmethod
    def kronecker(cls, scale: int, edgefactor: int = 16, seed1: int = 1, seed2: int = 2) -> "Graph":
        """Graph500 Kronecker graph generated and built on the GPU (seeds of cpu_2d/main.cpp:221)."""
        h = C.c_void_p()
        _check(lib().g5_graph_generate_kronecker(scale, edgefactor, seed1, seed2, C.byref(h)),
               "g5_graph_generate_kronecker")
        return cls(h.value, scale)

    @classmethod
    def load(cls, path: str) -> "Graph":
        """A graph saved with save(), uploaded to the current device."""
        h = C.c_void_p()
        _check(lib().g5_graph_load(os.fsencode(path), C.byref(h)), "g5_graph_load")
        sc = C.c_int()
        _check(lib().g5_graph_kronecker_info(h, C.byref(sc), None), "g5_graph_kronecker_info")
        return cls(h.value, sc.value if sc.value >= 0 else None)

    def save(self, path: str) -> None:
        """Binary CSR cache on disk (header, offsets, columns, generated endpoint counts)."""
        _check(lib().g5_graph_save(self._h, os.fsencode(path)), "g5_graph_save")

    def csr(self) -> tuple[np.ndarray, np.ndarray]:
        ro = np.empty(self.n + 1, np.int64)
        col = np.empty(self.nnz, np.uint32)
        _check(lib().g5_graph_copy_csr(self._h, _ptr(ro), _ptr(col) if self.nnz else None), "g5_graph_copy_csr")
        return ro, col

    def row_offsets(self) -> np.ndarray:
        ro = np.empty(self.n + 1, np.int64)
        _check(lib().g5_graph_copy_csr(self._h, _ptr(ro), None), "g5_graph_copy_csr")
        return ro

    def close(self) -> None:
        if self._h:
            lib().g5_graph_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def kronecker_edges(scale: int, seed1: int = 1, seed2: int = 2, start: int = 0,
                    end: Optional[int] = None, edgefactor: int = 16) -> np.ndarray:
    """Raw generated edge list [start, end) as an (m, 2) int64 array (GPU generator)."""
    if end is None:
        end = edgefactor << scale
    out = np.empty((end - start, 2), np.int64)
    _check(lib().g5_kronecker_edges(scale, seed1, seed2, start, end, _ptr(out)), "g5_kronecker_edges")
    return out


def select_roots(g: Graph, nroots: int = 64, maxgen: int = 32) -> np.ndarray:
    """Roots as the reference driver draws them (cpu_2d/main.cpp:351-392)."""
    out = np.empty(max(nroots, 1), np.int64)
    found = C.c_int()
    _check(lib().g5_select_roots(g._h, nroots, maxgen, _ptr(out), C.byref(found)), "g5_select_roots")
    return out[: found.value].copy()


def default_config() -> BfsConfig:
    cfg = BfsConfig()
    lib().g5_bfs_config_default(C.byref(cfg))
    return cfg


class CudaBFS:
    """One-root-per-search BFS with the reference's runBFS/getPredecessor shape.

    ``runBFS(start)`` runs GlobalBFS::runBFS at 1x1 (cpu_2d/globalbfs.hh:548);
    ``getPredecessor()`` returns the int64 parent array (-1 unvisited, root ->
    root), valid until the next ``runBFS`` like the reference's
    (cpu_2d/cuda/cuda_bfs.cu:43,328-378).
    """

    def __init__(self, graph: Graph, codec: int = CODEC_NONE, codec_threshold: int = 64,
                 alpha: float = 14.0, beta: float = 24.0, use_graph: bool = True,
                 want_levels: bool = False, max_levels: int = 4096, profile: bool = False,
                 parent_mode: Optional[int] = None, tile_edges: Optional[int] = None,
                 bu_serial: Optional[int] = None):
        self.graph = graph
        cfg = default_config()
        cfg.alpha, cfg.beta, cfg.codec, cfg.codec_threshold = alpha, beta, codec, codec_threshold
        cfg.use_graph, cfg.want_levels, cfg.max_levels = int(use_graph), int(want_levels), max_levels
        cfg.profile = int(profile)
        if parent_mode is not None:
            cfg.parent_mode = parent_mode
        if tile_edges is not None:
            cfg.tile_edges = tile_edges
        if bu_serial is not None:
            cfg.bu_serial = bu_serial
        self.cfg = cfg
        h = C.c_void_p()
        _check(lib().g5_bfs_create(graph._h, C.byref(cfg), C.byref(h)), "g5_bfs_create")
        self._h = h
        self._pred = np.empty(graph.n, np.int64)
        self._level = np.empty(graph.n, np.int32) if want_levels else None
        self.stats = BfsStats()
        self.last_root = None

    def run(self, root: int, pred_out=None, level_out=None, stats: bool = True) -> int:
        """Raw run: pred_out/level_out are numpy arrays, torch tensors, addresses or None."""
        code = lib().g5_bfs_run(self._h, int(root), _ptr(pred_out), _ptr(level_out),
                                C.byref(self.stats) if stats else None)
        self.last_root = int(root)
        return code

    def run_many(self, roots, pred_outs=None, device_ms: bool = False):
        """Searches every root, each search's parents copied to pred_outs[i]
        (host or device buffers of n int64, None entries skip the copy) while
        the next search runs.  Returns the per-search device ms if asked."""
        roots = np.ascontiguousarray(roots, dtype=np.int64)
        k = len(roots)
        outs = None
        if pred_outs is not None:
            outs = (C.c_void_p * k)(*[_ptr(p) for p in pred_outs])
        ms = np.zeros(max(k, 1), np.float64) if device_ms else None
        _check(lib().g5_bfs_run_many(self._h, _ptr(roots), k, outs, _ptr(ms)), "g5_bfs_run_many")
        if k:
            self.last_root = int(roots[-1])
        return ms[:k] if device_ms else None

    def runBFS(self, start: int) -> None:
        _check(self.run(start, self._pred, self._level), "g5_bfs_run")

    def getPredecessor(self) -> np.ndarray:
        return self._pred

    def getLevels(self) -> np.ndarray:
        return self._level

    def level_log(self) -> np.ndarray:
        """(levels, 4) int64: direction, frontier vertices, their edges, entries read."""
        out = np.zeros((4096, 4), np.int64)
        rows = C.c_int()
        _check(lib().g5_bfs_level_log(self._h, _ptr(out), 4096, C.byref(rows)), "g5_bfs_level_log")
        return out[: rows.value].copy()

    def profile_log(self) -> list:
        """Profile mode: [(kernel kind, ms)] for every launch of the last search."""
        kinds = np.zeros(65536, np.int32)
        ms = np.zeros(65536, np.float64)
        rows = C.c_int()
        _check(lib().g5_bfs_profile_log(self._h, _ptr(kinds), _ptr(ms), 65536, C.byref(rows)),
               "g5_bfs_profile_log")
        return [(BfsStats.KERNELS[k], float(t)) for k, t in zip(kinds[: rows.value], ms[: rows.value])]

    def codec_capture(self, buf_dev, cap_words: int, rec_dev, max_levels: int) -> None:
        """Copy every level's in-loop codec stream of the following searches to
        buf_dev (device, cap_words uint32) with (level, values, words, offset)
        per level in rec_dev (device, 4 x max_levels uint64); buf_dev None
        turns the copy off."""
        _check(lib().g5_bfs_codec_capture(self._h, _ptr(buf_dev), int(cap_words), _ptr(rec_dev), int(max_levels)),
               "g5_bfs_codec_capture")

    def codec_captured(self) -> tuple[int, bool]:
        """(levels recorded by the last search, whether any did not fit)."""
        lv, ov = C.c_int(), C.c_int()
        _check(lib().g5_bfs_codec_captured(self._h, C.byref(lv), C.byref(ov)), "g5_bfs_codec_captured")
        return lv.value, bool(ov.value)

    def device_pred_ptr(self) -> int:
        p = C.c_void_p()
        _check(lib().g5_bfs_device_pred(self._h, C.byref(p)), "g5_bfs_device_pred")
        return p.value

    def teps_edges(self) -> int:
        ne = C.c_int64()
        _check(lib().g5_bfs_teps_edges(self._h, C.byref(ne)), "g5_bfs_teps_edges")
        return ne.value

    def validate(self, root: Optional[int] = None) -> tuple[bool, bool]:
        """(valid, min_parent) of the last search on the device."""
        v, mp = C.c_int(), C.c_int()
        r = self.last_root if root is None else root
        _check(lib().g5_bfs_validate(self._h, int(r), C.byref(v), C.byref(mp)), "g5_bfs_validate")
        return bool(v.value), bool(mp.value)

    def close(self) -> None:
        if self._h:
            lib().g5_bfs_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Codec:
    """Device codec workspace (g5_codec); buffers are device pointers (torch tensors)."""

    def __init__(self, max_n: int):
        h = C.c_void_p()
        _check(lib().g5_codec_create(max_n, C.byref(h)), "g5_codec_create")
        self._h = h
        self.max_n = max_n

    @staticmethod
    def bound(n: int) -> int:
        return lib().g5_codec_bound(n)

    def encode(self, in_dev, n: int, out_dev, mode: int = CODEC_D4, stream=None) -> int:
        w = C.c_size_t()
        _check(lib().g5_codec_encode(self._h, _ptr(in_dev), n, _ptr(out_dev), C.byref(w), mode, stream),
               "g5_codec_encode")
        return w.value

    def decode(self, in_dev, words: int, out_dev, out_cap: int, mode: int = CODEC_D4, stream=None) -> int:
        n = C.c_size_t()
        _check(lib().g5_codec_decode(self._h, _ptr(in_dev), words, _ptr(out_dev), out_cap, C.byref(n),
                                     mode, stream), "g5_codec_decode")
        return n.value

    def encode_async(self, in_dev, n_dev, out_dev, out_words_dev, mode: int = CODEC_D4, stream=None) -> None:
        """Enqueues an encode whose length is in device memory (n_dev); the
        stream's words go to out_words_dev (device uint64).  Capturable."""
        _check(lib().g5_codec_encode_async(self._h, _ptr(in_dev), _ptr(n_dev), _ptr(out_dev), _ptr(out_words_dev),
                                           mode, stream), "g5_codec_encode_async")

    def decode_async(self, in_dev, words_dev, out_dev, out_cap: int, out_n_dev, mode: int = CODEC_D4,
                     stream=None) -> None:
        """Enqueues a decode of a stream whose length is in device memory."""
        _check(lib().g5_codec_decode_async(self._h, _ptr(in_dev), _ptr(words_dev), _ptr(out_dev), out_cap,
                                           _ptr(out_n_dev), mode, stream), "g5_codec_decode_async")

    def status(self) -> int:
        """Status code of the last call on this workspace (synchronous)."""
        return lib().g5_codec_status(self._h)

    @staticmethod
    def batch_bound(in_off: np.ndarray) -> int:
        """Output words encode_batch needs for queues with these offsets (k+1 entries)."""
        in_off = np.ascontiguousarray(in_off, dtype=np.uint64)
        return lib().g5_codec_batch_bound(_ptr(in_off), len(in_off) - 1)

    def encode_batch(self, in_dev, in_off: np.ndarray, out_dev, raw_threshold: int = 0, mode: int = CODEC_D4,
                     stream=None) -> tuple[np.ndarray, np.ndarray]:
        """Encodes k concatenated queues in one launch set; returns (out_off, out_words)."""
        in_off = np.ascontiguousarray(in_off, dtype=np.uint64)
        k = len(in_off) - 1
        out_off = np.zeros(k + 1, np.uint64)
        words = np.zeros(max(k, 1), np.uint64)
        _check(lib().g5_codec_encode_batch(self._h, _ptr(in_dev), _ptr(in_off), k, _ptr(out_dev), _ptr(out_off),
                                           _ptr(words), raw_threshold, mode, stream), "g5_codec_encode_batch")
        return out_off, words[:k]

    def decode_batch(self, in_dev, in_off: np.ndarray, words: np.ndarray, n: np.ndarray, out_dev,
                     raw_threshold: int = 0, mode: int = CODEC_D4, stream=None) -> tuple[np.ndarray, np.ndarray]:
        """Decodes k streams in one launch set; returns (out_off, per-stream ok flags).
        Raises G5Error if a stream is malformed (the flags say which)."""
        in_off = np.ascontiguousarray(in_off, dtype=np.uint64)
        words = np.ascontiguousarray(words, dtype=np.uint64)
        n = np.ascontiguousarray(n, dtype=np.uint64)
        k = len(n)
        out_off = np.zeros(k + 1, np.uint64)
        ok = np.zeros(max(k, 1), np.int32)
        code = lib().g5_codec_decode_batch(self._h, _ptr(in_dev), _ptr(in_off), _ptr(words), _ptr(n), k,
                                           _ptr(out_dev), _ptr(out_off), _ptr(ok), raw_threshold, mode, stream)
        if code != 0:
            err = G5Error(code, "g5_codec_decode_batch")
            err.stream_ok = ok[:k].copy()
            raise err
        return out_off, ok[:k]

    def close(self) -> None:
        if self._h:
            lib().g5_codec_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class GpuSimd:
    """Compression<int64_t, uint32_t> plugin (cpu_2d/compression/compression.hh:11-28).

    Same method names and argument meaning as CpuSimd (cpusimd.hh):
    ``compress(fq) -> (compressed, compressedsize)``, ``decompress(compressed,
    size, uncompressedsize) -> uncompressed``, raw below the threshold,
    ``isCompressed`` as cpusimd.hh:169-173.  The stream is s4-bp128-dm by
    default: what the reference plugin emits whatever name it is given.
    """

    def __init__(self):
        self.threshold = 64
        self.codec_name = "s4-bp128-dm"
        self.mode = CODEC_DM

    def reconfigure(self, compressionThreshold: int, compressionCodec: str) -> None:
        if compressionThreshold <= 0 or compressionCodec not in CODEC_NAMES:
            raise G5Error(G5_ERR_INVALID_ARG, "reconfigure")
        self.threshold = int(compressionThreshold)
        self.codec_name = compressionCodec
        self.mode = CODEC_NAMES[compressionCodec]

    def name(self) -> str:
        return "gpusimd"

    def init(self) -> None:
        pass

    def isCompressible(self, size: int) -> bool:
        return size > self.threshold

    def isCompressed(self, originalsize: int, compressedsize: int) -> bool:
        return self.isCompressible(originalsize) and originalsize != compressedsize

    def compress(self, fq_64: np.ndarray) -> tuple[np.ndarray, int]:
        fq = np.ascontiguousarray(fq_64, dtype=np.int64)
        out = C.c_void_p()
        cs = C.c_size_t()
        _check(lib().g5_plugin_compress(_ptr(fq) if len(fq) else None, len(fq), C.byref(out), C.byref(cs),
                                        self.threshold, self.mode), "g5_plugin_compress")
        arr = np.ctypeslib.as_array(C.cast(out, C.POINTER(C.c_uint32)), shape=(max(cs.value, 1),))
        res = arr[: cs.value].copy()
        C.CDLL(None).free(out)
        return res, cs.value

    def decompress(self, compressed: np.ndarray, size: int, uncompressedsize: int) -> np.ndarray:
        comp = np.ascontiguousarray(compressed, dtype=np.uint32)
        out = C.c_void_p()
        us = C.c_size_t(uncompressedsize)
        _check(lib().g5_plugin_decompress(_ptr(comp) if len(comp) else None, size, C.byref(out), C.byref(us),
                                          self.threshold, self.mode), "g5_plugin_decompress")
        arr = np.ctypeslib.as_array(C.cast(out, C.POINTER(C.c_int64)), shape=(max(us.value, 1),))
        res = arr[: us.value].copy()
        C.CDLL(None).free(out)
        return res


def batch_root_parents(pred_dev, n: int, nroots: int, r: int, dst_dev) -> None:
    """dst[v] = pred[v * nroots + r]: one root's parents out of a vertex-major
    batch array (device buffers with a data_ptr(), or raw device pointers)."""
    _check(lib().g5_batch_root_parents(_ptr(pred_dev), n, nroots, r, _ptr(dst_dev), None),
           "g5_batch_root_parents")


class Batch:
    """Batched BFS over up to 64 roots per graph in one level loop (g5_batch).

    Parents come out vertex-major per graph: graph g's block holds
    n_g x nroots[g] uint32 entries, vertex v's parent for root j at
    [v * nroots[g] + j]."""

    def __init__(self, graphs: Sequence[Graph]):
        self.graphs = list(graphs)
        arr = (C.c_void_p * len(self.graphs))(*[g._h.value for g in self.graphs])
        h = C.c_void_p()
        _check(lib().g5_batch_create(arr, len(self.graphs), C.byref(h)), "g5_batch_create")
        self._h = h

    def profile(self, roots: np.ndarray, nroots: Sequence[int], pred_out_dev) -> dict:
        """Host-driven run with per-kernel CUDA-event totals and active vertices per level."""
        roots = np.ascontiguousarray(roots, dtype=np.int64)
        nr = np.ascontiguousarray(nroots, dtype=np.int32)
        ms = np.zeros(5, np.float64)
        act = np.zeros(1024, np.int64)
        lms = np.zeros(1024, np.float64)
        lex = np.zeros(1024, np.int64)
        ldir = np.zeros(1024, np.int32)
        lv = C.c_int()
        _check(lib().g5_batch_profile(self._h, _ptr(roots), _ptr(nr), _ptr(pred_out_dev), _ptr(ms), _ptr(act),
                                      _ptr(lms), _ptr(lex), _ptr(ldir), 1024, C.byref(lv)), "g5_batch_profile")
        ex = lex[: lv.value]
        return {"kernel_ms": dict(zip(("count", "scan", "write", "expand", "fixup"), ms.tolist())),
                "active": act[: lv.value].tolist(), "expand_ms": lms[: lv.value].tolist(),
                "examined": np.diff(ex, prepend=0).tolist(),
                "dirs": ["".join(c for c, bit in (("T", 1), ("B", 2)) if d & bit) for d in ldir[: lv.value]]}

    def set_direction(self, alpha: float, beta: float) -> None:
        _check(lib().g5_batch_set_direction(self._h, alpha, beta), "g5_batch_set_direction")

    def run(self, roots: np.ndarray, nroots: Sequence[int], pred_out_dev) -> float:
        roots = np.ascontiguousarray(roots, dtype=np.int64)
        nr = np.ascontiguousarray(nroots, dtype=np.int32)
        ms = C.c_double()
        _check(lib().g5_batch_run(self._h, _ptr(roots), _ptr(nr), _ptr(pred_out_dev), C.byref(ms)),
               "g5_batch_run")
        return ms.value

    def launch(self, roots: np.ndarray, nroots: Sequence[int], pred_out_dev) -> None:
        """Asynchronous run: returns at once; poll() reports completion."""
        roots = np.ascontiguousarray(roots, dtype=np.int64)
        nr = np.ascontiguousarray(nroots, dtype=np.int32)
        _check(lib().g5_batch_launch(self._h, _ptr(roots), _ptr(nr), _ptr(pred_out_dev)), "g5_batch_launch")

    def poll(self, wait: bool = False):
        """(done, device ms) of the last launch."""
        done, ms = C.c_int(), C.c_double()
        _check(lib().g5_batch_poll(self._h, int(wait), C.byref(done), C.byref(ms)), "g5_batch_poll")
        return bool(done.value), ms.value

    def close(self) -> None:
        if self._h:
            lib().g5_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Resident graphs answering single-root queries with continuous batching (g5_server)."""

    STREAMS, LEVELS, AUTO, COHORTS = 0, 1, 2, 3

    def __init__(self, graphs: Sequence[Graph], mem_budget: int, keep_results: bool = True, mode: int = 0,
                 modes: Optional[Sequence[int]] = None):
        """mode: one slot kind for all graphs (or AUTO); modes: a kind per graph."""
        self.graphs = list(graphs)
        arr = (C.c_void_p * len(self.graphs))(*[g._h.value for g in self.graphs])
        h = C.c_void_p()
        if modes is not None:
            m = np.ascontiguousarray(modes, dtype=np.int32)
            _check(lib().g5_server_create_modes(arr, len(self.graphs), int(mem_budget), int(keep_results), _ptr(m),
                                                C.byref(h)), "g5_server_create_modes")
        else:
            _check(lib().g5_server_create(arr, len(self.graphs), int(mem_budget), int(keep_results), int(mode),
                                          C.byref(h)), "g5_server_create")
        self._h = h

    def cohort_policy(self, min_roots: int, max_wait_ms: float) -> None:
        """Cohort graphs: start a cohort at min_roots waiting queries or after max_wait_ms."""
        _check(lib().g5_server_cohort_policy(self._h, int(min_roots), float(max_wait_ms)), "g5_server_cohort_policy")

    def slots(self) -> list:
        out = np.zeros(len(self.graphs), np.int32)
        _check(lib().g5_server_slots(self._h, _ptr(out)), "g5_server_slots")
        return out.tolist()

    def submit(self, graph: int, root: int) -> int:
        t = C.c_uint64()
        _check(lib().g5_server_submit(self._h, graph, int(root), C.byref(t)), "g5_server_submit")
        return t.value

    def wait(self, ticket: int, timeout_s: float = 60.0) -> bool:
        done = C.c_int()
        _check(lib().g5_server_wait(self._h, ticket, timeout_s, C.byref(done)), "g5_server_wait")
        return bool(done.value)

    def result(self, ticket: int, with_pred: bool = True):
        """(parents or None, latency ms, queueing ms); frees the query's slot."""
        n = None
        pred = None
        lat, q = C.c_double(), C.c_double()
        if with_pred:
            # the graph of the ticket is not known here; size for the largest
            n = max(g.n for g in self.graphs)
            pred = np.empty(n, np.int64)
        _check(lib().g5_server_result(self._h, ticket, _ptr(pred), C.byref(lat), C.byref(q)),
               "g5_server_result")
        return pred, lat.value, q.value

    def stats(self) -> dict:
        st, cp, ms = C.c_uint64(), C.c_uint64(), C.c_double()
        _check(lib().g5_server_stats(self._h, C.byref(st), C.byref(cp), C.byref(ms)), "g5_server_stats")
        return {"steps": st.value, "completed": cp.value, "device_ms": ms.value}

    def close(self) -> None:
        if self._h:
            lib().g5_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def bitmap_or(dst_dev, srcs_dev: Sequence, words: int, stream=None) -> None:
    """dst |= OR(srcs) over uint64 words (device pointers)."""
    arr = (C.c_void_p * len(srcs_dev))(*[_ptr(s) for s in srcs_dev])
    _check(lib().g5_bitmap_or(_ptr(dst_dev), arr, len(srcs_dev), words, stream), "g5_bitmap_or")
