"""Serving with continuous batching: every query's parents are the same
alone and in a mix of concurrent queries on several graphs, and equal the
oracle's; memory-based admission queues what does not fit."""
import numpy as np
import pytest

import oracle as orc

pytestmark = pytest.mark.gpu

g5 = pytest.importorskip("gpugraph500_gb300")


@pytest.fixture(scope="module")
def graphs():
    gs = [g5.Graph.kronecker(s) for s in (10, 11, 12)]
    yield gs
    for g in gs:
        g.close()


def run_queries(sv, queries, concurrent):
    out = {}
    if concurrent:
        tickets = [(sv.submit(gi, r), gi, r) for gi, r in queries]
        for t, gi, r in tickets:
            assert sv.wait(t, 60.0)
            pred, lat, q = sv.result(t)
            out[(gi, r)] = pred
    else:
        for gi, r in queries:
            t = sv.submit(gi, r)
            assert sv.wait(t, 60.0)
            pred, lat, q = sv.result(t)
            out[(gi, r)] = pred
    return out


@pytest.mark.parametrize("mode", [0, 1, (1, 0, 1), 2, (3, 3, 3), (3, 0, 3)])
def test_alone_and_mixed_agree_with_oracle(graphs, mode):
    csrs = [g.csr() for g in graphs]
    roots = [g5.select_roots(g, 20) for g in graphs]
    rng = np.random.default_rng(0)
    queries = [(gi, int(r)) for gi in range(3) for r in roots[gi]]
    order = rng.permutation(len(queries))
    queries = [queries[i] for i in order]
    if isinstance(mode, tuple):  # a slot kind per graph (levels or cohorts beside stream workspaces)
        sv = g5.Server(graphs, mem_budget=1 << 30, modes=list(mode))
    else:
        sv = g5.Server(graphs, mem_budget=1 << 30, mode=mode)
    assert min(sv.slots()) >= 2
    alone = run_queries(sv, queries, concurrent=False)
    mixed = run_queries(sv, queries, concurrent=True)
    for (gi, r), p in alone.items():
        n = graphs[gi].n
        want, _ = orc.bfs(csrs[gi][0], csrs[gi][1], r)
        assert np.array_equal(p[:n], want), (gi, r)
        assert np.array_equal(mixed[(gi, r)][:n], p[:n]), (gi, r)
    st = sv.stats()
    assert st["completed"] == 2 * len(queries)
    sv.close()


@pytest.mark.parametrize("mode,per_slot", [(0, 48), (1, 4)])
def test_memory_admission_queues(graphs, mode, per_slot):
    # budget for about 3 slots of the largest graph: queries beyond the slots wait
    g = graphs[2]
    extra = 3 * (g.nnz // 64 + (1 << 20)) if mode == 0 else 0
    sv = g5.Server([g], mem_budget=3 * per_slot * g.n + extra, mode=mode)
    assert 1 <= sv.slots()[0] <= 3
    ro, col = g.csr()
    roots = g5.select_roots(g, 12)
    tickets = [sv.submit(0, int(r)) for r in roots]
    queued = 0
    for t, r in zip(tickets, roots):
        assert sv.wait(t, 60.0)
        pred, lat, q = sv.result(t)
        queued += q > 0
        want, _ = orc.bfs(ro, col, int(r))
        assert np.array_equal(pred[:g.n], want)
    sv.close()


@pytest.mark.parametrize("mode", [0, 1])
def test_repeated_slot_reuse(graphs, mode):
    g = graphs[0]
    ro, col = g.csr()
    sv = g5.Server([g], mem_budget=2 * (48 * g.n + g.nnz // 64 + (1 << 20)), mode=mode)
    roots = g5.select_roots(g, 10)
    for rep in range(3):
        for r in roots:
            t = sv.submit(0, int(r))
            assert sv.wait(t, 60.0)
            pred, _, _ = sv.result(t)
            want, _ = orc.bfs(ro, col, int(r))
            assert np.array_equal(pred[:g.n], want)
    sv.close()


def test_bad_queries(graphs):
    sv = g5.Server(graphs[:1], mem_budget=1 << 26)
    with pytest.raises(g5.G5Error):
        sv.submit(0, graphs[0].n)
    with pytest.raises(g5.G5Error):
        sv.submit(5, 0)
    sv.close()


def _cohort_bytes(g, slots, workspaces):
    """Device bytes of a cohort graph: the shared degree-ordered copy, two
    one-root workspaces, the batch workspaces and 4 bytes per vertex and root
    slot."""
    copy = 28 * g.n + 4 * g.nnz + (1 << 20)
    plain = 2 * (48 * g.n + g.nnz // 64 + (1 << 20))
    ws = 48 * g.n + g.nnz // 64 + (1 << 20)
    return copy + plain + workspaces * ws + workspaces * slots * 4 * g.n


def test_cohort_admission_and_reuse(graphs):
    """A budget for one batch workspace of 3 root slots: queries beyond the
    slots wait for the next cohort; results match the oracle; the workspace
    is reused once its cohort's results are released."""
    g = graphs[2]
    sv = g5.Server([g], mem_budget=_cohort_bytes(g, 3, 1), modes=[g5.Server.COHORTS])
    assert sv.slots() == [3]
    ro, col = g.csr()
    roots = g5.select_roots(g, 12)
    for rep in range(2):
        tickets = [sv.submit(0, int(r)) for r in roots]
        queued = 0
        for t, r in zip(tickets, roots):
            assert sv.wait(t, 60.0)
            pred, lat, q = sv.result(t)
            queued += q > 0.0
            want, _ = orc.bfs(ro, col, int(r))
            assert np.array_equal(pred[:g.n], want), (rep, int(r))
        assert queued >= 1
    st = sv.stats()
    assert st["completed"] == 24 and st["steps"] >= 8  # at most 3 queries per search
    sv.close()


def test_cohorts_mixed_with_lone_queries(graphs):
    """Queries trickling in one at a time run on the one-root workspaces, a
    burst forms cohorts; all parents equal the oracle's."""
    g = graphs[2]
    sv = g5.Server([g], mem_budget=_cohort_bytes(g, 16, 2), modes=[g5.Server.COHORTS])
    ro, col = g.csr()
    roots = g5.select_roots(g, 40)
    got = {}
    for r in roots[:5]:  # one at a time
        t = sv.submit(0, int(r))
        assert sv.wait(t, 60.0)
        got[int(r)] = sv.result(t)[0]
    tickets = [(sv.submit(0, int(r)), int(r)) for r in roots[5:]]  # a burst
    for t, r in tickets:
        assert sv.wait(t, 60.0)
        got[r] = sv.result(t)[0]
    for r, p in got.items():
        assert np.array_equal(p[:g.n], orc.bfs(ro, col, r)[0]), r
    st = sv.stats()
    assert st["completed"] == 40 and st["steps"] < 40  # the burst shared searches
    sv.close()


def test_cohorts_without_kept_results(graphs):
    """keep_results = False frees a cohort's workspace as soon as it ends."""
    g = graphs[1]
    sv = g5.Server([g], mem_budget=_cohort_bytes(g, 8, 2), keep_results=False, modes=[g5.Server.COHORTS])
    assert sv.slots() == [16]
    roots = g5.select_roots(g, 40)
    tickets = [sv.submit(0, int(r)) for r in roots]
    for t in tickets:
        assert sv.wait(t, 60.0)
        pred, lat, q = sv.result(t, with_pred=False)
        assert lat >= q >= 0.0
    assert sv.stats()["completed"] == 40
    sv.close()
