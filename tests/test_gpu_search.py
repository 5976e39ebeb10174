"""Batched search drivers on the GPU against the per-point drop-in path
(what the reference's per-point loop computes with version 'b200') and the
FP64 oracle."""

import numpy as np
import pytest

from _helpers import REL_TOL
from pyfstat_gb300 import search, synth
from pyfstat_gb300.atoms import MultiFstatAtomVector, merge_multi_atoms_binned
from pyfstat_gb300.tcw_fstat_map_funcs import b200_compute_transient_fstat_map
from pyfstat_gb300.window import transientWindowRange_t

pytestmark = pytest.mark.gpu


def points(n=5, nsft=150):
    return [synth.multi_detector_atoms(300 + k, nsft, ndet=2, gap_frac=0.1) for k in range(n)]


def window(wtype, t0=700000000):
    return transientWindowRange_t(type=wtype, t0=t0, t0Band=1800 * 100, dt0=3600, tau=1800,
                                  tauBand=1800 * 60, dtau=1800 * 2)


@pytest.mark.parametrize("wtype", [1, 2])
def test_grid_batch_equals_the_per_point_drop_in_path(wtype):
    pts = points()
    wr = window(wtype)
    out = search.TransientGridBatch(pts, wr, BtSG=True, BSGL=True,
                                    detector_names=["H1", "L1"]).run()
    for k, multi in enumerate(pts):
        m = b200_compute_transient_fstat_map(multi, window(wtype), BtSG=True)
        assert out["maxTwoF"][k] == pytest.approx(2 * float(m.maxF), rel=2e-6)
        assert (out["t0_ML"][k], out["tau_ML"][k]) == (m.t0_ML, m.tau_ML)
        assert out["lnBtSG"][k] == pytest.approx(m.lnBtSG, rel=2e-6)
        assert (out["t0_MP"][k], out["tau_MP"][k]) == (m.t0_MP, m.tau_MP)
        idx = m.get_maxF_idx()
        twoFX = []
        for x, ifo in enumerate(["H1", "L1"]):
            mx = b200_compute_transient_fstat_map(MultiFstatAtomVector([multi.data[x]]),
                                                  window(wtype), BtSG=False)
            twoFX.append(2.0 * float(mx.F_mn[idx]))
            assert out[f"twoF{ifo}atMaxTwoF"][k] == pytest.approx(twoFX[-1], rel=2e-6)
        assert out["log10BSGL"][k] == pytest.approx(
            float(search.compute_log10BSGL(2 * float(m.maxF), np.array(twoFX))), rel=1e-5,
            abs=1e-6)
        full = b200_compute_transient_fstat_map(multi, transientWindowRange_t(type=0))
        assert out["twoF"][k] == pytest.approx(2 * float(full.maxF), rel=2e-6)


def test_semicoherent_per_segment_twoF_matches_fp64_oracle(oracle):
    pts = points(n=3, nsft=240)
    t0 = 700000000
    nsegs = 6
    tb = t0 + np.arange(nsegs + 1) * (240 * 1800 // nsegs)
    out = search.semicoherent_twoF(pts, tb, BSGL=True, record_segments=True)
    Tcoh = int((tb[-1] - tb[0]) // nsegs)
    t0s = (tb[0] + Tcoh * np.arange(nsegs)).astype(np.uint32)
    for k, multi in enumerate(pts):
        t0d, A = merge_multi_atoms_binned(multi, 1800)
        F64 = oracle.map_f64(A, 1800, t0d, 1, t0s, np.array([Tcoh], np.uint32))[:, 0]
        np.testing.assert_allclose(out["twoF_per_segment"][k], 2 * F64, rtol=REL_TOL)
        assert out["twoF"][k] == pytest.approx(2 * F64.sum(), rel=REL_TOL)
        for x in range(2):
            t0x, Ax = merge_multi_atoms_binned(MultiFstatAtomVector([multi.data[x]]), 1800)
            FX = oracle.map_f64(Ax, 1800, t0x, 1, t0s, np.array([Tcoh], np.uint32))[:, 0]
            np.testing.assert_allclose(out["twoFX_per_segment"][k, x], 2 * FX, rtol=REL_TOL)
    np.testing.assert_allclose(
        out["log10BSGL"],
        search.compute_log10BSGL(out["twoF"], out["twoFX"],
                                 Fstar0=search.fstar0_semicoherent(nsegs)), rtol=1e-12)


def test_grid_batch_window_none_is_the_full_data_cell():
    """Window type 'none': every point's map is one rectangular cell over its
    own data (tcw:742-749), so maxTwoF equals the all-data twoF."""
    pts = points(n=4, nsft=90)
    out = search.TransientGridBatch(pts, transientWindowRange_t(type=0), BtSG=True).run()
    for k, multi in enumerate(pts):
        m = b200_compute_transient_fstat_map(multi, transientWindowRange_t(type=0), BtSG=True)
        assert out["maxTwoF"][k] == pytest.approx(2 * float(m.maxF), rel=2e-6)
        assert out["maxTwoF"][k] == out["twoF"][k]
        assert (out["t0_ML"][k], out["tau_ML"][k]) == (m.t0_ML, m.tau_ML)
        assert out["lnBtSG"][k] == pytest.approx(m.lnBtSG, rel=2e-6)


def test_grid_batch_in_memory_chunks_equals_one_launch():
    pts = points(n=6)
    wr = window(2)
    one = search.TransientGridBatch(pts, wr, BtSG=True, BSGL=True).run()
    # a budget of ~2 points' maps forces several launches
    small = search.TransientGridBatch(pts, window(2), BtSG=True, BSGL=True,
                                      map_budget_bytes=2 * 4 * 101 * 31).run()
    for key in one.dtype.names:
        np.testing.assert_allclose(small[key], one[key], rtol=2e-6, err_msg=key)
