"""Host-side logic of the drop-in module: containers, binned merge, window
ranges, the result type, the dispatcher's error behaviour (no GPU needed)."""

import numpy as np
import pytest

from pyfstat_gb300 import atoms as A
from pyfstat_gb300 import synth
from pyfstat_gb300 import tcw_fstat_map_funcs as tcw
from pyfstat_gb300.window import (TRANSIENT_EXPONENTIAL, TRANSIENT_RECTANGULAR,
                                  expand_window_range, grid_sizes, transientWindowRange_t,
                                  uniform_grid)


def test_atom_vector_duck_types_lalpulsar_fields():
    v = synth.multi_detector_atoms(0, 10, 1).data[0]
    assert v.length == 10 and v.TAtom == 1800
    a = v.data[3]
    assert a.timestamp == 700000000 + 3 * 1800
    assert isinstance(a.Fa_alpha, complex)
    assert a.a2_alpha == pytest.approx(float(v.a2[3]))
    d = tcw.reshape_FstatAtomsVector(v)
    assert set(d) == {"timestamp", "a2_alpha", "b2_alpha", "ab_alpha", "Fa_alpha_re",
                      "Fa_alpha_im", "Fb_alpha_re", "Fb_alpha_im"}
    assert d["Fb_alpha_im"].dtype == np.float32 and d["timestamp"].dtype == np.uint32


class _ForeignAtom:
    def __init__(self, t, x):
        self.timestamp = t
        self.a2_alpha, self.b2_alpha, self.ab_alpha = x[0], x[1], x[2]
        self.Fa_alpha = complex(x[3], x[4])
        self.Fb_alpha = complex(x[5], x[6])


class _ForeignVector:
    def __init__(self, vec):
        self.length = vec.length
        self.TAtom = vec.TAtom
        m = vec.as_matrix()
        self.data = [_ForeignAtom(int(vec.timestamps[k]), m[k]) for k in range(vec.length)]


def test_foreign_atom_structs_are_read_attribute_by_attribute():
    v = synth.multi_detector_atoms(2, 12, 1).data[0]
    ts, mat, TAtom = A.vector_arrays(_ForeignVector(v))
    assert np.array_equal(ts, v.timestamps) and np.array_equal(mat, v.as_matrix())


def test_merge_binned_two_detectors():
    multi = synth.multi_detector_atoms(3, 20, 2, gap_frac=0.2)
    t0, M = A.merge_multi_atoms_binned(multi, 1800)
    assert t0 == 700000000
    assert M.shape == (20, 7)
    # every detector atom lands in bin floor((t - tMin)/1800), summed in FP32
    expect = np.zeros((20, 7), np.float32)
    for X in range(2):
        v = multi.data[X]
        idx = (v.timestamps.astype(np.int64) - t0) // 1800
        for k, i in enumerate(idx):
            expect[i] += v.as_matrix()[k]
    assert np.array_equal(M, expect)
    # the offsets (0 and Tsft/3) make floor and nearest-bin merging agree
    _, M2 = A.merge_multi_atoms_binned(multi, 1800, rule="round")
    assert np.array_equal(M, M2)


def test_merge_gap_bins_are_zero():
    v = synth.detector_atoms(np.random.default_rng(0), 30)
    keep = np.ones(30, bool)
    keep[[5, 6, 7, 20]] = False
    vg = A.FstatAtomVector(v.timestamps[keep], v.a2[keep], v.b2[keep], v.ab[keep], v.Fa[keep],
                           v.Fb[keep], 1800)
    t0, M = A.merge_multi_atoms_binned(A.MultiFstatAtomVector([vg]), 1800)
    assert M.shape == (30, 7)
    assert np.all(M[[5, 6, 7, 20]] == 0) and np.all(M[~np.isin(np.arange(30), [5, 6, 7, 20]), 0] > 0)


def test_window_range_expansion_matches_reference_sizes():
    wr = transientWindowRange_t(type=TRANSIENT_RECTANGULAR, t0=700000000, t0Band=86400 - 3600,
                                dt0=1800, tau=3600, tauBand=86400 - 3600, dtau=1800)
    assert grid_sizes(wr) == (47, 47)  # floor(Band/d) + 1 (tcw:775-780)
    t0s, taus = expand_window_range(wr)
    assert t0s[0] == 700000000 and t0s[-1] == 700000000 + 46 * 1800
    assert taus[0] == 3600 and taus[-1] == 3600 + 46 * 1800
    assert uniform_grid(2 ** 32 - 10, 5, 4).tolist() == [2 ** 32 - 10, 2 ** 32 - 5, 0, 5]


def test_result_type_methods(tmp_path):
    rng = np.random.default_rng(0)
    fm = tcw.pyTransientFstatMap(6, 5)
    assert fm.maxF == -1.0 and np.isnan(fm.lnBtSG)
    fm.F_mn = rng.uniform(0, 10, (6, 5)).astype(np.float32)
    fm.maxF = fm.F_mn.max()
    m, n = fm.get_maxF_idx()
    assert fm.F_mn[m, n] == fm.maxF
    lnB = fm.get_lnBtSG()
    expect = np.log(70.0 / 30) + np.log(np.sum(np.exp(fm.F_mn.astype(np.float64))))
    assert lnB == pytest.approx(expect, rel=1e-6)
    wr = transientWindowRange_t(type=TRANSIENT_EXPONENTIAL, t0=1000, t0Band=500, dt0=100,
                                tau=50, tauBand=400, dtau=100)
    t0_MP = fm.get_t0_max_posterior(wr)
    k = np.argmax(np.exp(fm.F_mn.astype(np.float64) - fm.maxF).sum(axis=1))
    assert t0_MP == 1000 + (k + 0.5) * 500 / 6
    tau_MP = fm.get_tau_max_posterior(wr)
    k = np.argmax(np.exp(fm.F_mn.astype(np.float64) - fm.maxF).sum(axis=0))
    assert tau_MP == 50 + (k + 0.5) * 400 / 5
    # text round trip (t0 tau 2F), as in tests/test_core.py:566-600 of the reference
    path = tmp_path / "Fmn.txt"
    wr2 = transientWindowRange_t(type=1, t0=1000, t0Band=500, dt0=100, tau=50, tauBand=400,
                                 dtau=100)
    fm.write_F_mn_to_file(str(path), wr2, ["a header line"])
    back = tcw.pyTransientFstatMap(from_file=str(path))
    assert back.F_mn.shape == (6, 5)
    np.testing.assert_allclose(back.F_mn, fm.F_mn, rtol=1e-7)
    assert back.maxF == pytest.approx(float(fm.maxF), rel=1e-7)
    assert (back.t0_ML, back.tau_ML) == (1000 + m * 100, 50 + n * 100)
    with pytest.raises(ValueError, match="Need either"):
        tcw.pyTransientFstatMap()


def test_dispatcher_errors_match_reference_messages():
    features = {"lal": False, "pycuda": False, "b200": False}
    with pytest.raises(Exception, match='method "nope" not implemented'):
        tcw.call_compute_transient_fstat_map("nope", features)
    with pytest.raises(Exception, match='method "lal" not available'):
        tcw.call_compute_transient_fstat_map("lal", features)
    with pytest.raises(ValueError, match="Unknown transient F-stat map computation feature"):
        tcw.init_transient_fstat_map_features("nope")
    assert set(tcw.fstatmap_versions) == {"lal", "pycuda", "b200"}


def test_unknown_window_type_raises_before_any_gpu_work():
    multi = synth.multi_detector_atoms(0, 10, 1)
    wr = transientWindowRange_t(type=3)
    with pytest.raises(ValueError, match="Unknown window-type"):
        tcw.b200_compute_transient_fstat_map(multi, wr)


@pytest.mark.parametrize("cc,expect", [((10, 3), True), ((10, 0), False), ((12, 0), False),
                                       ((9, 0), False)])
def test_b200_feature_requires_compute_capability_10_3(monkeypatch, cc, expect):
    # the library holds sm_103a code only: a cc 10.0 (B200) or 12.x device
    # cannot run it, so the 'b200' feature must be False there
    from pyfstat_gb300 import _lib

    monkeypatch.setattr(_lib, "device_count", lambda: 1)
    monkeypatch.setattr(_lib, "device_info",
                        lambda d: dict(name="fake", cc=cc, total_mem=1 << 30))
    assert tcw._b200_available() is expect
    assert tcw._get_transient_fstat_map_features()["b200"] is expect
    if not expect:
        with pytest.raises(RuntimeError, match="compute capability 10.3"):
            tcw.init_transient_fstat_map_features("b200")


def test_gpu_memory_debug_log_never_fails_the_call(caplog):
    # the reference logs free / total device memory at debug level around each
    # map (_print_GPU_memory_MB, tcw:648-653); without a device the line says
    # so instead of raising
    import logging

    with caplog.at_level(logging.DEBUG, logger=tcw.logger.name):
        tcw._print_GPU_memory_MB("Initial", 0)
    assert any("Initial GPU memory" in r.getMessage() for r in caplog.records)
