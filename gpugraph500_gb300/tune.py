"""Autotuner for the direction-switch thresholds and the load-balancing sizes.

Beamer's alpha/beta (SC'12) were tuned for CPUs; on a GPU the cost of a
top-down edge and of a bottom-up probe differ, so the thresholds are picked by
measurement: every (alpha, beta) pair of a small grid runs a sample of roots,
and the pair with the best harmonic-mean TEPS wins.  A second stage then picks,
with those thresholds, the top-down tile size (frontier edges per warp tile)
and the bottom-up serial length (entries a lane scans alone before its warp
takes over the row: the cut-off between the lane and warp degree bins).
Searches are timed with the library's CUDA events.  Candidates within
TIE_TOL of the best harmonic-mean TEPS are not told apart by the measurement
(run-to-run noise is about that size), so among them the one closest to the
starting point wins: Beamer's published alpha = 14, beta = 24 for the
thresholds, the library's default tile of 256 edges and serial length of 8
for the sizes (closest in log distance).  Results are cached per (graph size,
edge count) in memory for the process.
"""
from __future__ import annotations

import itertools
import math
from typing import Sequence

ALPHAS = (4.0, 14.0, 25.0, 40.0, 70.0, 120.0, 400.0)
BETAS = (64.0, 200.0, 600.0, 1000.0, 2000.0, 3000.0, 6000.0)
TILES = (64, 128, 256, 512)
SERIALS = (4, 8, 16, 32)
# the batched search steps 64 roots at once and its bottom-up levels are
# cheap per root, so it leaves bottom-up at larger frontiers (smaller beta)
BATCH_BETAS = (12.0, 24.0, 64.0, 200.0)

TIE_TOL = 0.005
DEFAULT_THRESHOLDS = (14.0, 24.0)
DEFAULT_SIZES = (256, 8)

_cache: dict = {}


def _pick(results, default):
    """results: [(gteps, x, y)] sorted best first; the candidate within
    TIE_TOL of the best that is closest to `default` in log distance."""
    best = results[0][0]
    near = [r for r in results if r[0] >= best * (1.0 - TIE_TOL)]
    return min(near, key=lambda r: (abs(math.log(r[1] / default[0])) + abs(math.log(r[2] / default[1])), -r[0]))


def _hmean_teps(times_ms, nedges):
    inv = sum((t * 1e-3) / e for t, e in zip(times_ms, nedges))
    return len(times_ms) / inv / 1e9 if inv > 0 else 0.0


def tune_plain(g5, graph, roots: Sequence[int], nedges: Sequence[int], alphas=ALPHAS, betas=BETAS,
               reps: int = 2) -> dict:
    """Best (alpha, beta) for the one-root search on this graph."""
    key = ("plain", graph.n, graph.nnz, tuple(alphas), tuple(betas))
    if key in _cache:
        return _cache[key]
    results = []
    for a, b in itertools.product(alphas, betas):
        bfs = g5.CudaBFS(graph, alpha=a, beta=b)
        best = None
        for _ in range(reps):
            ts = []
            for r in roots:
                code = bfs.run(int(r), None, None, stats=True)
                if code != 0:
                    raise g5.G5Error(code, "tune")
                ts.append(bfs.stats.device_ms)
            v = _hmean_teps(ts, nedges)
            best = v if best is None else max(best, v)
        bfs.close()
        results.append((best, a, b))
    results.sort(reverse=True)
    pick = _pick(results, DEFAULT_THRESHOLDS)
    out = {"alpha": pick[1], "beta": pick[2], "gteps": pick[0],
           "grid": [{"alpha": a, "beta": b, "gteps": round(v, 2)} for v, a, b in results]}
    _cache[key] = out
    return out


def tune_batch(g5, torch, graphs, roots_per_graph, alphas=ALPHAS, betas=BATCH_BETAS) -> dict:
    """Best (alpha, beta) for a batched search over the given graphs and roots."""
    import numpy as np

    bt = g5.Batch(graphs)
    total = sum(len(r) * g.n for g, r in zip(graphs, roots_per_graph))
    out = torch.empty(max(total, 1), dtype=torch.int32, device="cuda")
    roots = np.concatenate([np.asarray(r, np.int64) for r in roots_per_graph])
    counts = [len(r) for r in roots_per_graph]
    results = []
    for a, b in itertools.product(alphas, betas):
        bt.set_direction(a, b)
        bt.run(roots, counts, out)  # builds the graph for these arguments
        ms = min(bt.run(roots, counts, out) for _ in range(2))
        results.append((ms, a, b))
    bt.close()
    results.sort()
    return {"alpha": results[0][1], "beta": results[0][2], "ms": results[0][0],
            "grid": [{"alpha": a, "beta": b, "ms": round(m, 3)} for m, a, b in results]}


def tune_sizes(g5, graph, roots: Sequence[int], nedges: Sequence[int], alpha: float, beta: float,
               tiles=TILES, serials=SERIALS, reps: int = 2) -> dict:
    """Best (tile_edges, bu_serial) for the one-root search with fixed thresholds."""
    key = ("sizes", graph.n, graph.nnz, alpha, beta, tuple(tiles), tuple(serials))
    if key in _cache:
        return _cache[key]
    results = []
    for t, sr in itertools.product(tiles, serials):
        bfs = g5.CudaBFS(graph, alpha=alpha, beta=beta, tile_edges=t, bu_serial=sr)
        best = None
        for _ in range(reps):
            ts = []
            for r in roots:
                code = bfs.run(int(r), None, None, stats=True)
                if code != 0:
                    raise g5.G5Error(code, "tune")
                ts.append(bfs.stats.device_ms)
            v = _hmean_teps(ts, nedges)
            best = v if best is None else max(best, v)
        bfs.close()
        results.append((best, t, sr))
    results.sort(reverse=True)
    pick = _pick(results, DEFAULT_SIZES)
    out = {"tile_edges": pick[1], "bu_serial": pick[2], "gteps": pick[0],
           "grid": [{"tile_edges": t, "bu_serial": sr, "gteps": round(v, 2)} for v, t, sr in results]}
    _cache[key] = out
    return out
