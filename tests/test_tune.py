"""The autotuner's choice among measured candidates (host logic, CPU)."""
import pytest

from gpugraph500_gb300 import tune


def test_clear_winner_wins():
    r = [(700.0, 400.0, 6000.0), (650.0, 14.0, 24.0)]
    assert tune._pick(r, tune.DEFAULT_THRESHOLDS)[1:] == (400.0, 6000.0)


def test_near_ties_prefer_the_default():
    # within TIE_TOL of the best: the measurement does not separate them
    r = [(641.5, 40.0, 6000.0), (639.4, 40.0, 2000.0), (639.3, 14.0, 2000.0), (600.0, 14.0, 24.0)]
    assert tune._pick(r, tune.DEFAULT_THRESHOLDS)[1:] == (14.0, 2000.0)
    r = [(649.2, 64, 8), (647.8, 128, 8), (642.1, 256, 8)]
    assert tune._pick(r, tune.DEFAULT_SIZES)[1:] == (128, 8)


def test_tolerance_edge():
    best = 1000.0
    inside = best * (1 - tune.TIE_TOL) + 1e-9
    outside = best * (1 - tune.TIE_TOL) - 1e-6
    assert tune._pick([(best, 400.0, 6000.0), (inside, 14.0, 24.0)], tune.DEFAULT_THRESHOLDS)[1:] == (14.0, 24.0)
    assert tune._pick([(best, 400.0, 6000.0), (outside, 14.0, 24.0)], tune.DEFAULT_THRESHOLDS)[1:] == (400.0, 6000.0)


@pytest.mark.parametrize("grid", [tune.ALPHAS, tune.BETAS, tune.BATCH_BETAS, tune.TILES, tune.SERIALS])
def test_grids_positive_and_sorted(grid):
    assert all(x > 0 for x in grid) and list(grid) == sorted(grid)
