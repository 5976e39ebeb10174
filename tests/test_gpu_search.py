"""Batched search drivers on the GPU against the per-point drop-in path
(what the reference's per-point loop computes with version 'b200') and the
FP64 oracle."""

import numpy as np
import pytest

from _helpers import REL_TOL, argmax_ok, index_ok
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


@pytest.mark.parametrize("wtype", [0, 1, 2])
def test_grid_batch_matches_the_fp64_oracle(oracle, wtype):
    """Every output column of the batched grid driver
    (grid_based_searches.py:1103-1134) against the FP64 oracle's map of each
    point plus the reference's post-processing restated in the oracle:
    maxTwoF, (t0_ML, tau_ML) at the oracle's argmax, lnBtSG, (t0_MP, tau_MP)
    at the oracle's max-posterior bins (centres t0 + (k + 1/2) t0Band / N,
    tcw:248-251, :283-286), the all-data twoF, the per-detector 2F at the
    argmax cell (core.py:1531-1541) and log10BSGL from those values."""
    from pyfstat_gb300.window import grid_sizes, uniform_grid

    pts = points(n=4, nsft=160)
    wr = window(wtype) if wtype else transientWindowRange_t(type=0)
    gb = search.TransientGridBatch(pts, wr, BtSG=True, BSGL=True, detector_names=["H1", "L1"])
    out = gb.run()
    assert gb.metadata["bsgl_parity"] == "unpinned"
    for k, multi in enumerate(pts):
        t0d, A = merge_multi_atoms_binned(multi, 1800)
        if wtype == 0:
            w, t0, dt0, t0Band, tau, dtau, tauBand = 1, t0d, 1800, 0, A.shape[0] * 1800, 1800, 0
            t0s, taus = np.array([t0d], np.uint32), np.array([tau], np.uint32)
        else:
            w, t0, dt0, t0Band, tau, dtau, tauBand = (wr.type, wr.t0, wr.dt0, wr.t0Band, wr.tau,
                                                      wr.dtau, wr.tauBand)
            N_t0, N_tau = grid_sizes(wr)
            t0s, taus = uniform_grid(t0, dt0, N_t0), uniform_grid(tau, dtau, N_tau)
        F64 = oracle.map_f64(A, 1800, t0d, w, t0s, taus)
        label = f"grid w{wtype} point {k}"
        assert out["maxTwoF"][k] == pytest.approx(2 * F64.max(), rel=REL_TOL)
        m = (int(out["t0_ML"][k]) - t0) // dt0
        n = (int(out["tau_ML"][k]) - tau) // dtau
        assert argmax_ok(m * taus.size + n, F64, label=label), label
        assert out["lnBtSG"][k] == pytest.approx(oracle.lnBtSG(F64), rel=REL_TOL)
        e = np.exp(F64 - F64.max())
        kt = round((out["t0_MP"][k] - t0) / (t0Band / t0s.size) - 0.5) if t0Band else 0
        kn = round((out["tau_MP"][k] - tau) / (tauBand / taus.size) - 0.5) if tauBand else 0
        assert index_ok(kt, e.sum(axis=1), label=label + " t0_MP"), label
        assert index_ok(kn, e.sum(axis=0), label=label + " tau_MP"), label
        Fall = oracle.map_f64(A, 1800, t0d, 1, np.array([t0d], np.uint32),
                              np.array([A.shape[0] * 1800], np.uint32))
        assert out["twoF"][k] == pytest.approx(2 * float(Fall[0, 0]), rel=REL_TOL)
        twoFX = []
        for x, ifo in enumerate(["H1", "L1"]):
            tx, Ax = merge_multi_atoms_binned(MultiFstatAtomVector([multi.data[x]]), 1800)
            FX = oracle.map_f64(Ax, 1800, tx, w, t0s, taus)
            twoFX.append(2.0 * float(FX[m, n]))
            assert out[f"twoF{ifo}atMaxTwoF"][k] == pytest.approx(twoFX[-1], rel=REL_TOL), label
        want = float(search.compute_log10BSGL(2 * F64.max(), np.array(twoFX)))
        assert out["log10BSGL"][k] == pytest.approx(want, rel=1e-5, abs=1e-5), label
