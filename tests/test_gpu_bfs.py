"""Plain BFS on the GPU against the oracle (parents bit-exact, levels exact)."""
import numpy as np
import pytest

import oracle as orc

pytestmark = pytest.mark.gpu

g5 = pytest.importorskip("gpugraph500_gb300")


def csr_from_edges(n, edges):
    return orc.build_csr(n, np.asarray(edges, np.int64).reshape(-1, 2))


def run_all_roots(ro, col, roots, **kw):
    g = g5.Graph.from_csr(ro, col)
    for use_graph in (True, False):
        b = g5.CudaBFS(g, want_levels=True, use_graph=use_graph, **kw)
        for r in roots:
            b.runBFS(int(r))
            want_pred, want_level = orc.bfs(ro, col, int(r))
            assert np.array_equal(b.getPredecessor(), want_pred), (r, use_graph)
            assert np.array_equal(b.getLevels(), want_level), (r, use_graph)
            valid, minpar = b.validate()
            assert valid and minpar
        b.close()
    g.close()


def test_hand_graphs():
    # path 0-1-2-...-9, star around 10, two components, self loops, duplicates
    edges = [(i, i + 1) for i in range(9)]
    edges += [(10, 11 + i) for i in range(12)]
    edges += [(30, 31), (31, 32), (32, 30), (33, 33), (30, 31), (31, 30)]
    edges += [(40, 41), (40, 41), (41, 41)]
    n = 64
    ro, col = csr_from_edges(n, edges)
    run_all_roots(ro, col, [0, 5, 9, 10, 11, 30, 33, 40])


def test_degenerate_graphs():
    """One vertex, no edges at all, an isolated root, and sizes at word and
    chunk boundaries: parents equal the oracle's (the root maps to itself,
    everything else stays -1 when nothing is reachable)."""
    ro, col = csr_from_edges(1, np.zeros((0, 2), np.int64))
    run_all_roots(ro, col, [0])
    ro, col = csr_from_edges(37, np.zeros((0, 2), np.int64))
    run_all_roots(ro, col, [0, 36])
    for n in (32, 64, 65536, 65537):
        edges = [(i, (i * 7 + 3) % n) for i in range(0, n, 3)]
        ro, col = csr_from_edges(n, edges)
        run_all_roots(ro, col, [1, n - 1, n // 3])  # n // 3 ... may be isolated


def test_long_path_many_levels():
    n = 3000
    edges = [(i, i + 1) for i in range(n - 1)]
    ro, col = csr_from_edges(n, edges)
    run_all_roots(ro, col, [0, 1500])


def test_odd_sizes():
    rng = np.random.default_rng(3)
    for n in (33, 95, 1000, 4097):
        e = rng.integers(0, n, size=(4 * n, 2))
        ro, col = csr_from_edges(n, e)
        run_all_roots(ro, col, [0, n - 1, n // 2])


@pytest.mark.parametrize("scale", [8, 11, 14])
def test_kronecker_parents_match_oracle(scale):
    e = orc.kronecker(scale)
    ro, col = orc.build_csr(1 << scale, e)
    roots = orc.select_roots(ro, 16)
    run_all_roots(ro, col, roots)


def test_direction_extremes():
    """Bottom-up from the first level on (alpha and beta huge), pure top-down
    (both tiny) and a mix agree."""
    e = orc.kronecker(12)
    ro, col = orc.build_csr(1 << 12, e)
    roots = orc.select_roots(ro, 4)
    for alpha, beta in ((1e12, 1e12), (1e-6, 1e-6), (1.0, 2.0)):
        run_all_roots(ro, col, roots, alpha=alpha, beta=beta)


@pytest.mark.parametrize("alpha,beta", [(1e12, 1e12), (14.0, 2000.0), (1e-6, 1e-6)])
def test_level_log_matches_oracle(alpha, beta):
    """Every level's frontier size and adjacency entries (the degree sum the
    direction switch reads) equal the oracle's.  With alpha and beta huge the
    search stays bottom-up from level 1 on, so the unvisited-list sweep, whose
    per-word degree sums the count pass adds up, runs at consecutive levels."""
    e = orc.kronecker(13)
    ro, col = orc.build_csr(1 << 13, e)
    deg = np.diff(ro)
    roots = orc.select_roots(ro, 6)
    g = g5.Graph.from_csr(ro, col)
    for use_graph in (True, False):
        b = g5.CudaBFS(g, alpha=alpha, beta=beta, use_graph=use_graph)
        for r in roots:
            b.runBFS(int(r))
            _, lev = orc.bfs(ro, col, int(r))
            log = b.level_log()
            nlev = int(lev.max()) + 1
            assert len(log) >= nlev
            for L in range(nlev):
                m = lev == L
                assert (int(log[L, 1]), int(log[L, 2])) == (int(m.sum()), int(deg[m].sum())), (r, L, use_graph)
            assert all(int(x) == 0 for x in log[nlev:, 1])
            if alpha > 1e6 and nlev > 3:
                assert int(log[2, 0]) == 1 and int(log[3, 0]) == 1  # consecutive bottom-up levels
        b.close()
    g.close()


@pytest.mark.parametrize("tile,serial", [(32, 1), (128, 4), (1024, 16), (4096, 64)])
def test_tile_and_serial_sizes(tile, serial):
    """Every top-down tile size and bottom-up serial length gives the same parents."""
    e = orc.kronecker(12)
    ro, col = orc.build_csr(1 << 12, e)
    roots = orc.select_roots(ro, 4)
    for alpha, beta in ((14.0, 24.0), (1e-6, 1e-6)):
        run_all_roots(ro, col, roots, alpha=alpha, beta=beta, tile_edges=tile, bu_serial=serial)


def test_bad_sizes_rejected():
    e = orc.kronecker(8)
    ro, col = orc.build_csr(1 << 8, e)
    g = g5.Graph.from_csr(ro, col)
    for kw in ({"tile_edges": 48}, {"tile_edges": 96}, {"tile_edges": 8192}, {"bu_serial": 0}, {"bu_serial": 65}):
        with pytest.raises(g5.G5Error):
            g5.CudaBFS(g, **kw)
    g.close()


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_parent_modes_agree(mode):
    """The three top-down parent strategies give the same (reference) parents."""
    e = orc.kronecker(13)
    ro, col = orc.build_csr(1 << 13, e)
    roots = orc.select_roots(ro, 6)
    for alpha in (14.0, 1e9):
        run_all_roots(ro, col, roots, parent_mode=mode, alpha=alpha)


def test_gpu_generator_and_csr_match_oracle():
    for scale in (6, 10, 13):
        g = g5.Graph.kronecker(scale)
        e = orc.kronecker(scale)
        assert np.array_equal(g5.kronecker_edges(scale), e)
        ro, col = orc.build_csr(1 << scale, e)
        gro, gcol = g.csr()
        assert np.array_equal(gro, ro) and np.array_equal(gcol, col)
        assert np.array_equal(g5.select_roots(g, 64), orc.select_roots(ro, 64))
        g.close()


def test_generator_slices():
    e = orc.kronecker(12, start=1000, end=5000)
    assert np.array_equal(g5.kronecker_edges(12, start=1000, end=5000), e)


def test_teps_edges_and_validation_match_oracle():
    scale = 12
    g = g5.Graph.kronecker(scale)
    e = orc.kronecker(scale)
    ro, col = orc.build_csr(1 << scale, e)
    b = g5.CudaBFS(g)
    for r in orc.select_roots(ro, 8):
        b.runBFS(int(r))
        ok, ne, _ = orc.validate(1 << scale, e, int(r), b.getPredecessor())
        assert ok
        assert b.teps_edges() == ne
        assert b.validate() == (True, True)
    b.close()
    g.close()


class _Dev:
    """A device array handed to torch through __cuda_array_interface__."""

    def __init__(self, ptr, n):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": "<i8", "data": (ptr, False), "version": 3}


def test_device_validator_rejects_corrupt_trees():
    torch = pytest.importorskip("torch")
    e = orc.kronecker(10)
    n = 1 << 10
    ro, col = orc.build_csr(n, e)
    g = g5.Graph.from_csr(ro, col)
    b = g5.CudaBFS(g, want_levels=True)
    root = int(orc.select_roots(ro, 1)[0])
    b.runBFS(root)
    good = b.getPredecessor().copy()
    lev = b.getLevels().copy()
    pred = torch.as_tensor(_Dev(b.device_pred_ptr(), n), device="cuda")
    adj = [set(col[ro[v]:ro[v + 1]].tolist()) for v in range(n)]
    # a vertex at level >= 2 with two neighbours one level up
    v2 = next(v for v in range(n) if lev[v] >= 2 and sum(lev[u] == lev[v] - 1 for u in adj[v]) >= 2)
    ups = sorted(u for u in adj[v2] if lev[u] == lev[v2] - 1)
    far = next(u for u in range(n) if u not in adj[v2] and u != v2 and lev[u] >= 0)
    leaf = next(v for v in range(n) if v != root and lev[v] > 0 and good[v] >= 0)

    def check(mutate, want_valid, want_min):
        p = good.copy()
        mutate(p)
        pred.copy_(torch.from_numpy(p))
        torch.cuda.synchronize()
        valid, minpar = b.validate(root)
        assert valid == want_valid, mutate
        if want_valid:  # the min-parent verdict is only meaningful for a valid tree
            assert minpar == want_min, mutate

    check(lambda p: None, True, True)
    check(lambda p: p.__setitem__(v2, ups[-1]), True, False)   # valid parent, not the smallest
    check(lambda p: p.__setitem__(v2, far), False, False)      # not an edge of the graph
    check(lambda p: p.__setitem__(root, ups[0]), False, False)  # the root does not map to itself
    check(lambda p: p.__setitem__(leaf, leaf), False, False)   # self parent
    check(lambda p: p.__setitem__(leaf, -1), False, False)     # a reachable vertex left out

    def cycle(p):
        p[v2] = ups[0]
        p[ups[0]] = v2
    check(cycle, False, False)
    b.close()
    g.close()


def test_codec_in_loop_round_trips():
    e = orc.kronecker(13)
    ro, col = orc.build_csr(1 << 13, e)
    roots = orc.select_roots(ro, 6)
    for codec in (g5.CODEC_D4, g5.CODEC_DM):
        run_all_roots(ro, col, roots, codec=codec)
    g = g5.Graph.from_csr(ro, col)
    b = g5.CudaBFS(g, codec=g5.CODEC_D4)
    b.runBFS(int(roots[0]))
    s = b.stats
    assert s.codec_values == s.queue_total - 1  # every level's queue except the root
    assert 0 < s.codec_words < s.codec_values


def test_invalid_root_and_config():
    ro, col = csr_from_edges(8, [(0, 1)])
    g = g5.Graph.from_csr(ro, col)
    b = g5.CudaBFS(g)
    assert b.run(-1) == g5.G5_ERR_INVALID_ARG
    assert b.run(8) == g5.G5_ERR_INVALID_ARG
    with pytest.raises(g5.G5Error):
        g5.CudaBFS(g, codec=7)
    b.runBFS(5)  # isolated root: only itself
    p = b.getPredecessor()
    assert p[5] == 5 and (np.delete(p, 5) == -1).all()


def test_level_cap_reports_timeout():
    n = 200
    ro, col = csr_from_edges(n, [(i, i + 1) for i in range(n - 1)])
    g = g5.Graph.from_csr(ro, col)
    for use_graph in (True, False):
        b = g5.CudaBFS(g, max_levels=50, use_graph=use_graph)
        assert b.run(0) == g5.G5_ERR_TIMEOUT
        b.close()


def test_bad_csr_rejected():
    ro = np.array([0, 1, 2], np.int64)
    col = np.array([1, 5], np.uint32)  # id out of range
    with pytest.raises(g5.G5Error):
        g5.Graph.from_csr(ro, col)


def test_run_many_pipelined_copies_match_oracle():
    """g5_bfs_run_many: every root's parents land in its own buffer (pageable
    host, pinned host, device or skipped), equal to the oracle's, and the
    workspace then refers to the last root."""
    torch = pytest.importorskip("torch")
    e = orc.kronecker(12)
    ro, col = orc.build_csr(1 << 12, e)
    n = 1 << 12
    roots = orc.select_roots(ro, 7)
    g = g5.Graph.from_csr(ro, col)
    b = g5.CudaBFS(g)
    outs = [np.full(n, 7, np.int64), torch.empty(n, dtype=torch.int64, pin_memory=True),
            torch.empty(n, dtype=torch.int64, device="cuda"), None,
            np.empty(n, np.int64), torch.empty(n, dtype=torch.int64, pin_memory=True), np.empty(n, np.int64)]
    for rep in range(2):
        ms = b.run_many(roots, outs, device_ms=True)
        assert len(ms) == len(roots) and (ms > 0).all()
        for r, o in zip(roots, outs):
            if o is None:
                continue
            got = o.cpu().numpy() if hasattr(o, "cpu") else o
            assert np.array_equal(got, orc.bfs(ro, col, int(r))[0]), (rep, int(r))
    # the workspace's parent array, TEPS count and validation are the last root's
    last = torch.as_tensor(_DevI64(b.device_pred_ptr(), n), device="cuda").cpu().numpy()
    assert np.array_equal(last, orc.bfs(ro, col, int(roots[-1]))[0])
    assert b.validate() == (True, True)
    b.runBFS(int(roots[0]))  # single runs still work after run_many
    assert np.array_equal(b.getPredecessor(), orc.bfs(ro, col, int(roots[0]))[0])
    with pytest.raises(g5.G5Error):
        b.run_many(np.array([0, n], np.int64), None)
    b.close()


def test_parents_stay_exact_across_roots_without_edges():
    """The parent array is not refilled per search: a root without edges
    (the only vertex without edges a search writes) is reset by the next
    search into the same array, in single runs and in both buffers of the
    pipelined call, and vertices of other components get -1."""
    rng = np.random.default_rng(11)
    n = 2000
    e = rng.integers(0, 1500, size=(3000, 2))  # vertices 1500.. have no edges
    e = np.concatenate([e, [[1600, 1601], [1601, 1602]]])  # a small second component
    ro, col = orc.build_csr(n, e)
    deg = np.diff(ro)
    iso = [int(v) for v in np.nonzero(deg == 0)[0][:4]]
    big = int(np.argmax(deg))
    roots = [iso[0], big, iso[1], iso[2], 1600, iso[3], big, 1601, iso[0]]
    g = g5.Graph.from_csr(ro, col)
    for use_graph in (True, False):
        b = g5.CudaBFS(g, use_graph=use_graph)
        for r in roots:
            b.runBFS(r)
            assert np.array_equal(b.getPredecessor(), orc.bfs(ro, col, r)[0]), (r, use_graph)
        if use_graph:
            outs = [np.empty(n, np.int64) for _ in roots]
            for rep in range(2):
                b.run_many(np.array(roots, np.int64), outs)
                for r, o in zip(roots, outs):
                    assert np.array_equal(o, orc.bfs(ro, col, r)[0]), (rep, r)
        b.close()
    g.close()
    g.close()


class _DevI64:
    """A device int64 array handed to torch through __cuda_array_interface__."""

    def __init__(self, ptr, n):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": "<i8", "data": (ptr, False), "version": 3}
