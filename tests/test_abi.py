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
