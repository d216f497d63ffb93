"""The autotuner on a GPU: the thresholds it picks run the same roots at
least as fast as Beamer's fixed alpha = 14, beta = 24 (within the timing
noise the tuner itself allows), and its pick is among the grid's best."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

g5 = pytest.importorskip("gpugraph500_gb300")
from gpugraph500_gb300 import tune  # noqa: E402


def hmean_gteps(g, roots, nedges, **kw):
    b = g5.CudaBFS(g, **kw)
    for r in roots:  # warm-up
        b.run(int(r), None, None, stats=True)
    best = 0.0
    for _ in range(3):
        ms = []
        for r in roots:
            assert b.run(int(r), None, None, stats=True) == 0
            ms.append(b.stats.device_ms)
        best = max(best, tune._hmean_teps(ms, nedges))
    b.close()
    return best


def test_tuned_thresholds_not_slower_than_defaults():
    g = g5.Graph.kronecker(22)
    roots = g5.select_roots(g, 16)
    probe = g5.CudaBFS(g)
    nedges = []
    for r in roots:
        probe.runBFS(int(r))
        nedges.append(probe.teps_edges())
    probe.close()
    tuned = tune.tune_plain(g5, g, roots, nedges)
    assert tuned["alpha"] in tune.ALPHAS and tuned["beta"] in tune.BETAS
    t = hmean_gteps(g, roots, nedges, alpha=tuned["alpha"], beta=tuned["beta"])
    d = hmean_gteps(g, roots, nedges, alpha=tune.DEFAULT_THRESHOLDS[0], beta=tune.DEFAULT_THRESHOLDS[1])
    assert t >= d * (1.0 - 3 * tune.TIE_TOL), (tuned, t, d)
    # the pick is within the tuner's tolerance of the best grid point it measured
    best = max(r["gteps"] for r in tuned["grid"])
    pick = [r["gteps"] for r in tuned["grid"] if (r["alpha"], r["beta"]) == (tuned["alpha"], tuned["beta"])][0]
    assert pick >= best * (1.0 - tune.TIE_TOL) - 0.01  # grid values are rounded to 0.01
    g.close()
