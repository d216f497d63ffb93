"""Batched BFS (64 bit-sliced roots per graph, several graphs per launch)
against the oracle: every root's parents bit-exact."""
import numpy as np
import pytest

import oracle as orc

pytestmark = pytest.mark.gpu

g5 = pytest.importorskip("gpugraph500_gb300")
torch = pytest.importorskip("torch")


def oracle_u32(ro, col, r):
    p, _ = orc.bfs(ro, col, int(r))
    return p.astype(np.uint64).astype(np.uint32)  # -1 -> 0xFFFFFFFF


def check_batch(graphs, csrs, roots_per_graph):
    bt = g5.Batch(graphs)
    total = sum(len(r) * g.n for g, r in zip(graphs, roots_per_graph))
    out = torch.empty(max(total, 1), dtype=torch.int32, device="cuda")
    roots = np.concatenate([np.asarray(r, np.int64) for r in roots_per_graph])
    ms = bt.run(roots, [len(r) for r in roots_per_graph], out)
    assert ms > 0
    got = out.cpu().numpy().view(np.uint32)
    off = 0
    for g, (ro, col), rs in zip(graphs, csrs, roots_per_graph):
        block = got[off:off + g.n * len(rs)].reshape(g.n, len(rs))  # vertex-major
        for j, r in enumerate(rs):
            assert np.array_equal(block[:, j], oracle_u32(ro, col, r)), r
        off += g.n * len(rs)
    return bt


@pytest.mark.parametrize("scale,nroots", [(10, 64), (13, 64), (12, 17)])
def test_single_graph(scale, nroots):
    g = g5.Graph.kronecker(scale)
    ro, col = g.csr()
    roots = g5.select_roots(g, nroots)
    bt = check_batch([g], [(ro, col)], [roots])
    # a second run on the same workspace gives the same answer
    bt2 = check_batch([g], [(ro, col)], [roots[::-1]])
    bt.close(); bt2.close(); g.close()


def test_mixed_scales_one_launch():
    scales = [8, 9, 10, 11, 12, 12, 13, 14]
    graphs = [g5.Graph.kronecker(s) for s in scales]
    csrs = [g.csr() for g in graphs]
    roots = [g5.select_roots(g, 16) for g in graphs]
    bt = check_batch(graphs, csrs, roots)
    bt.close()
    for g in graphs:
        g.close()


def test_hand_graph_and_duplicate_roots():
    edges = np.array([(i, i + 1) for i in range(40)] + [(50, 51), (51, 52), (60, 60)], np.int64)
    ro, col = orc.build_csr(70, edges)
    g = g5.Graph.from_csr(ro, col)
    roots = [0, 20, 40, 50, 60, 65, 0]
    check_batch([g], [(ro, col)], [roots]).close()
    g.close()


def test_root_parents_extraction():
    g = g5.Graph.kronecker(11)
    ro, col = g.csr()
    roots = g5.select_roots(g, 9)
    bt = check_batch([g], [(ro, col)], [roots])
    out = torch.empty(9 * g.n, dtype=torch.int32, device="cuda")
    bt.run(np.asarray(roots, np.int64), [9], out)
    dst = torch.empty(g.n, dtype=torch.int32, device="cuda")
    for j, r in enumerate(roots):
        g5.batch_root_parents(out, g.n, 9, j, dst)
        assert np.array_equal(dst.cpu().numpy().view(np.uint32), oracle_u32(ro, col, r))
    with pytest.raises(g5.G5Error):
        g5.batch_root_parents(out, g.n, 9, 9, dst)
    bt.close(); g.close()


def test_degenerate_graphs_in_one_batch():
    """A graph without edges, a single-vertex graph and a graph whose size
    ends exactly on a chunk boundary, all in one launch with isolated roots."""
    ro0, col0 = orc.build_csr(37, np.zeros((0, 2), np.int64))
    ro1, col1 = orc.build_csr(1, np.zeros((0, 2), np.int64))
    n2 = 4096
    e2 = np.array([(i, (i * 5 + 1) % n2) for i in range(0, n2, 2)], np.int64)
    ro2, col2 = orc.build_csr(n2, e2)
    gs = [g5.Graph.from_csr(ro, col) for ro, col in ((ro0, col0), (ro1, col1), (ro2, col2))]
    bt = check_batch(gs, [(ro0, col0), (ro1, col1), (ro2, col2)], [[0, 36, 5], [0], [0, 1, 3, 4095, 2048]])
    bt.close()
    for g in gs:
        g.close()


def test_invalid_roots_rejected():
    g = g5.Graph.kronecker(8)
    bt = g5.Batch([g])
    out = torch.empty(4 * g.n, dtype=torch.int32, device="cuda")
    with pytest.raises(g5.G5Error):
        bt.run(np.array([0, g.n], np.int64), [2], out)
    with pytest.raises(g5.G5Error):
        bt.run(np.zeros(65, np.int64), [65], out)
    bt.close(); g.close()
