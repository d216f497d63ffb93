"""Binary CSR cache: a saved graph loads back identical, searches give the
same parents and TEPS edge counts, and damaged files are rejected."""
import os

import numpy as np
import pytest

import oracle as orc

pytestmark = pytest.mark.gpu

g5 = pytest.importorskip("gpugraph500_gb300")


def test_kronecker_round_trip(tmp_path):
    g = g5.Graph.kronecker(12)
    path = str(tmp_path / "k12.g5csr")
    g.save(path)
    h = g5.Graph.load(path)
    assert (h.n, h.nnz, h.scale) == (g.n, g.nnz, 12)
    ro, col = g.csr()
    ro2, col2 = h.csr()
    assert np.array_equal(ro, ro2) and np.array_equal(col, col2)
    roots = g5.select_roots(h, 8)
    assert np.array_equal(roots, g5.select_roots(g, 8))
    bg, bh = g5.CudaBFS(g), g5.CudaBFS(h)
    for r in roots:
        bg.runBFS(int(r))
        bh.runBFS(int(r))
        assert np.array_equal(bh.getPredecessor(), orc.bfs(ro, col, int(r))[0])
        assert bh.teps_edges() == bg.teps_edges()  # generated endpoint counts travel with the file
    bg.close(); bh.close(); g.close(); h.close()


def test_csr_graph_round_trip(tmp_path):
    edges = np.array([(0, 1), (1, 2), (2, 0), (5, 6), (7, 7)], np.int64)
    ro, col = orc.build_csr(9, edges)
    g = g5.Graph.from_csr(ro, col)
    path = str(tmp_path / "small.g5csr")
    g.save(path)
    h = g5.Graph.load(path)
    assert h.scale is None
    ro2, col2 = h.csr()
    assert np.array_equal(ro, ro2) and np.array_equal(col, col2)
    g.close(); h.close()


def test_damaged_files_rejected(tmp_path):
    g = g5.Graph.kronecker(10)
    path = str(tmp_path / "k10.g5csr")
    g.save(path)
    data = open(path, "rb").read()
    g.close()
    # missing file, truncated file, extra bytes, foreign magic
    with pytest.raises(g5.G5Error) as e:
        g5.Graph.load(str(tmp_path / "absent"))
    assert e.value.code == g5.G5_ERR_IO
    for bad in (data[:-4], data + b"\0" * 8, b"NOTG5CSR" + data[8:], data[:40]):
        p = str(tmp_path / "bad.g5csr")
        open(p, "wb").write(bad)
        with pytest.raises(g5.G5Error) as e:
            g5.Graph.load(p)
        assert e.value.code == g5.G5_ERR_IO
    # a well-sized file whose CSR is malformed: a column id out of range
    n = np.frombuffer(data[8:16], np.int64)[0]
    body = bytearray(data)
    col0 = 64 + 8 * (n + 1)
    body[col0:col0 + 4] = np.uint32(n + 5).tobytes()
    p = str(tmp_path / "badcol.g5csr")
    open(p, "wb").write(bytes(body))
    with pytest.raises(g5.G5Error) as e:
        g5.Graph.load(p)
    assert e.value.code == g5.G5_ERR_INVALID_ARG
    os.remove(p)
