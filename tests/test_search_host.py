"""Host logic of the batched search drivers (no GPU): the BSGL combination,
F*0 of semi-coherent searches, per-point grids."""

import math

import numpy as np
import pytest
import scipy.special

from pyfstat_gb300 import search
from pyfstat_gb300.window import transientWindowRange_t


def test_bsgl_matches_the_published_combination():
    rng = np.random.default_rng(0)
    twoFX = rng.uniform(0, 60, (20, 3))
    twoF = twoFX.sum(axis=1) * rng.uniform(0.5, 1.5, 20)
    oLGX = np.array([0.2, 0.3, 0.5])
    got = search.compute_log10BSGL(twoF, twoFX, Fstar0=12.0, oLGX=oLGX)
    want = [(0.5 * a + math.log(1 + oLGX.sum())
             - math.log(math.exp(12.0) + sum(o * math.exp(0.5 * x) for o, x in zip(oLGX, bx))))
            / math.log(10) for a, bx in zip(twoF, twoFX)]
    np.testing.assert_allclose(got, want, rtol=1e-12)


def test_bsgl_symmetry_and_max_approximation():
    twoFX = np.array([[30.0, 10.0], [10.0, 30.0]])
    twoF = np.array([40.0, 40.0])
    a = search.compute_log10BSGL(twoF, twoFX)
    assert a[0] == pytest.approx(a[1])
    exact = search.compute_log10BSGL(twoF, twoFX, use_log_correction=False)
    # dropping all but the largest denominator term can only raise the value,
    # by at most log10 of the number of terms
    assert np.all(exact >= a) and np.all(exact - a <= math.log10(3) + 1e-12)
    # a line (all of F from one detector) saturates at log10((1 + oLG) / oLGX)
    # = log10(4); a signal seen coherently by both detectors grows with F
    line = search.compute_log10BSGL(200.0, np.array([200.0, 0.0]))
    assert line <= math.log10(4.0) + 1e-12
    assert search.compute_log10BSGL(400.0, np.array([200.0, 200.0])) > 20.0


def test_fstar0_semicoherent():
    assert search.fstar0_semicoherent(1) == 15.0
    for nsegs in (2, 10, 50):
        f = search.fstar0_semicoherent(nsegs)
        grid = np.linspace(0, 1000, 10000)
        step = grid[1] - grid[0]
        p = scipy.special.gammaincc(2 * nsegs, [f - step, f, f + step])
        assert abs(p[1] - 1e-6) <= max(abs(p[0] - 1e-6), abs(p[2] - 1e-6))


def test_grid_of_window_type_none_is_one_cell_over_all_data():
    wr = transientWindowRange_t(type=0)
    w, t0s, taus, r = search._grid_for(wr, 1800, 700000000, 480)
    assert w == 1 and t0s.tolist() == [700000000] and taus.tolist() == [480 * 1800]
    wr = transientWindowRange_t(type=2, t0=700000000, t0Band=3600 * 10, dt0=3600, tau=1800,
                                tauBand=1800 * 7, dtau=1800)
    w, t0s, taus, r = search._grid_for(wr, 1800, 700000000, 480)
    assert w == 2 and t0s.size == 11 and taus.size == 8 and taus[-1] == 1800 * 8
    with pytest.raises(ValueError):
        search._grid_for(transientWindowRange_t(type=3), 1800, 0, 10)


def test_chunks_by_cells_covers_in_order_within_budget():
    cells = [5, 3, 9, 1, 1, 12, 4]
    ch = search.chunks_by_cells(cells, 10)
    assert ch[0][0] == 0 and ch[-1][1] == len(cells)
    assert all(b0 == a1 for (_, b0), (a1, _) in zip(ch[:-1], ch[1:]))
    for a, b in ch:
        assert b > a and (sum(cells[a:b]) <= 10 or b - a == 1)
    assert search.chunks_by_cells(cells, float("inf")) == [(0, len(cells))]
    assert search.chunks_by_cells([], 10) == []
