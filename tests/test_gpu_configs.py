"""Parity at the benchmark's configuration scales, on the GPU.

* scale 16 (the reference's CPU configuration): the GPU generator's edge
  list, the CSR, the 64 roots and the parents of all 64 searches, plain and
  batched, against the sha256 digests of the reference's own outputs
  (tests/golden/kron_s16.json, written by the reference compiled from its
  sources); TEPS edge counts and validator verdicts against the same file.
* scale 22 (plain GPU search with every level's queue through the
  s4-bp128-d4 codec): the CSR against the oracle's, parents and levels of 8
  roots bit-exact against the oracle's CPUBFS_bin restatement, and every
  level's in-loop stream word for word against the oracle encoder on that
  level's queue (the reference encodes each level's queue at
  cpu_2d/globalbfs.hh:853,873-877 through cpu_2d/compression/cpusimd.hh:
  70-118).
* scale 20 (batched form): 16 roots in one bit-sliced launch against the
  oracle.

The oracle searches of one graph run on host threads (its C calls release
the interpreter lock).
"""
import concurrent.futures as cf
import hashlib
import json
import os

import numpy as np
import pytest

import oracle as orc

pytestmark = pytest.mark.gpu

g5 = pytest.importorskip("gpugraph500_gb300")
torch = pytest.importorskip("torch")


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def oracle_searches(ro, col, roots):
    with cf.ThreadPoolExecutor(max_workers=min(len(roots), orc.host_threads())) as ex:
        return list(ex.map(lambda r: orc.bfs(ro, col, int(r)), roots))


def test_scale16_against_reference_digests(golden_dir):
    info = json.load(open(os.path.join(golden_dir, "kron_s16.json")))
    scale, n = info["scale"], info["n"]
    assert sha(g5.kronecker_edges(scale)) == info["edges_sha256"]
    g = g5.Graph.kronecker(scale)
    ro, col = g.csr()
    assert sha(ro) == info["row_off_sha256"] and sha(col) == info["col_u32_sha256"]
    roots = g5.select_roots(g, 64)
    assert [int(r) for r in roots] == info["roots"]
    bfs = g5.CudaBFS(g, want_levels=True)
    for i, r in enumerate(roots):
        bfs.runBFS(int(r))
        assert sha(bfs.getPredecessor()) == info["pred_sha256"][i], (i, int(r))
        assert int(bfs.getLevels().max()) + 1 == info["depth"][i]
        assert bfs.teps_edges() == info["nedge"][i]
        assert bfs.validate() == (bool(info["valid"][i]), True)
    bfs.close()
    # the batched form: all 64 roots in one launch, each root's parents widened
    # to the reference's int64 convention (-1 unvisited)
    bt = g5.Batch([g])
    out = torch.empty(64 * n, dtype=torch.int32, device="cuda")
    bt.run(roots, [64], out)
    block = out.cpu().numpy().view(np.uint32).reshape(n, 64)
    for j in range(64):
        p = block[:, j].astype(np.int64)
        p[p == 0xFFFFFFFF] = -1
        assert sha(p) == info["pred_sha256"][j], j
    bt.close()
    g.close()


def test_scale22_codec_in_loop_streams_and_parents():
    scale, n = 22, 1 << 22
    e = orc.kronecker(scale)
    ro, col = orc.build_csr(n, e, threads=0)
    del e
    g = g5.Graph.kronecker(scale)
    gro, gcol = g.csr()
    assert np.array_equal(gro, ro) and np.array_equal(gcol, col)
    del gro, gcol
    roots = g5.select_roots(g, 8)
    want = oracle_searches(ro, col, roots)
    bfs = g5.CudaBFS(g, codec=g5.CODEC_D4, codec_threshold=64, want_levels=True)
    max_levels = 64
    buf = torch.zeros(g5.Codec.bound(n) + 4 * max_levels + 1024, dtype=torch.int32, device="cuda")
    rec = torch.zeros(4 * max_levels, dtype=torch.int64, device="cuda")
    bfs.codec_capture(buf, buf.numel(), rec, max_levels)
    for r, (want_pred, want_level) in zip(roots, want):
        bfs.runBFS(int(r))  # the in-loop decode check would return G5_ERR_MISMATCH
        assert np.array_equal(bfs.getPredecessor(), want_pred), int(r)
        assert np.array_equal(bfs.getLevels(), want_level), int(r)
        assert bfs.stats.codec_values == int((want_level > 0).sum())
        levels, overflow = bfs.codec_captured()
        assert not overflow
        recs = rec[: 4 * levels].cpu().numpy().reshape(levels, 4)
        words = buf.cpu().numpy().view(np.uint32)
        depth = int(want_level.max())
        seen = set()
        for L, nv, w, off in (tuple(int(x) for x in row) for row in recs):
            q = np.nonzero(want_level == L)[0]  # the level's sorted queue
            assert nv == len(q), (int(r), L)
            if nv == 0:
                assert L == depth + 1 and w == 0
                continue
            ref = orc.plugin_compress(q, 64, orc.D4)
            assert np.array_equal(words[off:off + w], ref), (int(r), L, nv)
            seen.add(L)
        assert seen == set(range(1, depth + 1)), int(r)
    bfs.codec_capture(None, 0, None, 0)
    bfs.close()
    g.close()


def test_scale20_batched_16_roots():
    scale, n = 20, 1 << 20
    g = g5.Graph.kronecker(scale)
    ro, col = g.csr()
    roots = g5.select_roots(g, 16)
    want = oracle_searches(ro, col, roots)
    bt = g5.Batch([g])
    out = torch.empty(16 * n, dtype=torch.int32, device="cuda")
    bt.run(roots, [16], out)
    block = out.cpu().numpy().view(np.uint32).reshape(n, 16)
    for j, (p, _) in enumerate(want):
        assert np.array_equal(block[:, j], p.astype(np.uint64).astype(np.uint32)), j
    bt.close()
    g.close()
