"""The C-ABI library builds, loads without a GPU and exports every symbol
include/g5bfs.h declares (no compute calls here)."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            src = open(os.path.join(ROOT, "include", fn)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            for m in re.finditer(r"^[\w\s\*]*?\b(g5_\w+)\s*\(", src, flags=re.M):
                names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def libg5():
    import gpugraph500_gb300 as g5
    if not os.path.exists(g5.LIB_PATH):
        from gpugraph500_gb300 import build
        build.build()
    return C.CDLL(g5.LIB_PATH)


def test_header_declares_api():
    names = declared_symbols()
    for must in ("g5_bfs_run", "g5_graph_create", "g5_codec_encode", "g5_codec_decode", "g5_bitmap_or",
                 "g5_batch_run", "g5_plugin_compress", "g5_select_roots"):
        assert must in names


def test_library_exports_every_declared_symbol(libg5):
    missing = [n for n in declared_symbols() if not hasattr(libg5, n)]
    assert not missing, missing


def test_python_signatures_cover_header():
    import gpugraph500_gb300 as g5
    assert set(declared_symbols()) <= set(g5.SIGNATURES)


def test_status_strings(libg5):
    libg5.g5_status_str.restype = C.c_char_p
    assert libg5.g5_status_str(0) == b"ok"
    assert libg5.g5_status_str(5) == b"corrupt codec stream"


def test_codec_bound_matches_oracle(libg5):
    import oracle as orc
    libg5.g5_codec_bound.restype = C.c_size_t
    libg5.g5_codec_bound.argtypes = [C.c_size_t]
    for n in [0, 1, 127, 128, 129, 2048, 2049, 10**6]:
        assert libg5.g5_codec_bound(n) >= orc.lib().g5o_codec_bound(n) - 8


def test_product_does_not_reference_oracle():
    """The product package never imports or loads the oracle."""
    pkg = os.path.join(ROOT, "gpugraph500_gb300")
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cu", ".cpp", ".h", ".cuh")):
                src = open(os.path.join(dirpath, f)).read()
                assert "g5_oracle" not in src and "libg5oracle" not in src and "import oracle" not in src, f


def test_config_defaults(libg5):
    """The defaults the tuner starts from: Beamer's thresholds, tile 256, serial 8."""
    import gpugraph500_gb300 as g5
    from gpugraph500_gb300 import tune
    cfg = g5.BfsConfig()
    g5.lib().g5_bfs_config_default(C.byref(cfg))
    assert (cfg.alpha, cfg.beta) == tune.DEFAULT_THRESHOLDS
    assert (cfg.tile_edges, cfg.bu_serial) == tune.DEFAULT_SIZES
    assert (cfg.parent_mode, cfg.codec_threshold, cfg.max_levels, cfg.use_graph) == (0, 64, 4096, 1)


def test_codec_batch_bound(libg5):
    """The batched bound: every stream's single-call bound rounded up to 4
    words (16-byte aligned stream starts), summed."""
    import numpy as np
    import gpugraph500_gb300 as g5
    sizes = [0, 1, 63, 64, 65, 127, 128, 2049, 100000]
    in_off = np.zeros(len(sizes) + 1, np.uint64)
    in_off[1:] = np.cumsum(sizes)
    libg5.g5_codec_bound.restype = C.c_size_t
    libg5.g5_codec_bound.argtypes = [C.c_size_t]
    want = sum((libg5.g5_codec_bound(n) + 3) // 4 * 4 for n in sizes)
    assert g5.Codec.batch_bound(in_off) == want
    assert g5.Codec.batch_bound(np.zeros(1, np.uint64)) == 0


def _header_fields(src, name):
    body = re.search(r"typedef struct " + name + r"\s*\{(.*?)\}\s*" + name + ";", src, flags=re.S).group(1)
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    return re.findall(r"\b(\w+)(?:\[(\d+)\])?\s*;", body)


@pytest.mark.parametrize("cname,pyname", [("g5_bfs_config", "BfsConfig"), ("g5_bfs_stats", "BfsStats")])
def test_structs_mirror_header(cname, pyname):
    """The Python ctypes mirrors have the header's fields in the header's order
    (a mismatch would shift every later field across the C ABI)."""
    import gpugraph500_gb300 as g5
    src = open(os.path.join(ROOT, "include", "g5bfs.h")).read()
    assert [f for f, _ in _header_fields(src, cname)] == [f for f, _ in getattr(g5, pyname)._fields_]


def test_stats_profile_buckets():
    """One profile bucket name per kernel_ms slot; the eighth is the host
    loop's gap after each level."""
    import gpugraph500_gb300 as g5
    src = open(os.path.join(ROOT, "include", "g5bfs.h")).read()
    slots = dict(_header_fields(src, "g5_bfs_stats"))["kernel_ms"]
    assert int(slots) == len(g5.BfsStats.KERNELS) == 8
    assert g5.BfsStats.KERNELS[-1] == "host"
