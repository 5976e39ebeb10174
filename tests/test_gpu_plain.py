"""Plain per-template maps on the GPU through the C ABI, against the FP64 oracle.

Bar: F within 1e-5 relative of the FP64 oracle on every cell outside the
threshold band around cond = 1e4; argmax and the posterior indices equal the
oracle's; lnBtSG within 1e-5 relative.
"""

import numpy as np
import pytest

from _helpers import REL_TOL, argmax_ok, golden_case, golden_cases, index_ok, rel_err
from pyfstat_gb300 import synth

pytestmark = pytest.mark.gpu

FLAGS_ALL = 0x1 | 0x2


@pytest.fixture(scope="module")
def lib():
    from pyfstat_gb300 import _lib

    _lib.load()
    return _lib


@pytest.fixture(scope="module")
def handle(lib):
    h = lib.Handle(0)
    yield h
    h.close()


def _check_case(handle, oracle, c, flags=FLAGS_ALL, tol=REL_TOL):
    F, res = handle.map_plain_host(c["atoms"], c["TAtom"], c["t0_data"], c["window"], c["t0s"],
                                   c["taus"], want_map=True, flags=flags)
    F64, cond = oracle.map_f64(c["atoms"], c["TAtom"], c["t0_data"], c["window"], c["t0s"],
                               c["taus"], with_cond=True)
    rel, nband = rel_err(F, F64, cond)
    assert rel.max() < tol, (c.get("name"), rel.max())
    # the device reduction agrees with the map it wrote
    assert float(res["maxF"]) == float(F.max())
    assert int(res["argmax"]) == int(np.argmax(F))
    if nband == 0:
        name = c.get("name")
        assert argmax_ok(res["argmax"], F64, label=f"{name} argmax"), name
        lnB64 = oracle.lnBtSG(F64)
        assert float(res["lnBtSG"]) == pytest.approx(lnB64, rel=tol, abs=1e-6)
        if flags & 0x2:
            e = np.exp(F64 - F64.max())
            assert index_ok(res["t0_mp_idx"], e.sum(axis=1), label=f"{name} t0_MP"), name
            assert index_ok(res["tau_mp_idx"], e.sum(axis=0), label=f"{name} tau_MP"), name
    return F, res


def test_rect_workload_480(handle, oracle):
    _check_case(handle, oracle, dict(synth.plain_rect_case(), name="rect480"))


def test_exp_workload_480x512_log_tau(handle, oracle):
    _check_case(handle, oracle, dict(synth.plain_exp_case(), name="exp480x512log"))


def test_golden_edge_cases(handle, oracle, golden):
    for name in golden_cases(golden):
        _check_case(handle, oracle, golden_case(golden, name))


def test_random_gappy_grids(handle, oracle):
    for seed in range(12):
        rng = np.random.default_rng(100 + seed)
        t0_data, A = synth.merged_atoms(seed, int(rng.integers(20, 400)), int(rng.integers(1, 3)),
                                        gap_frac=float(rng.uniform(0, 0.5)))
        A = A.copy()
        for _ in range(int(rng.integers(0, 4))):
            s = int(rng.integers(0, A.shape[0]))
            A[s:s + int(rng.integers(1, 40))] = 0
        for window in (1, 2):
            nt0, ntau = int(rng.integers(1, 300)), int(rng.integers(1, 300))
            t0 = int(t0_data + rng.integers(-5000, 3000))
            c = dict(name=f"rand{seed}w{window}", window=window, atoms=A, TAtom=1800,
                     t0_data=t0_data,
                     t0s=(t0 + np.arange(nt0) * int(rng.integers(1, 4000))).astype(np.uint32),
                     taus=(int(rng.integers(1, 5000)) + np.arange(ntau) *
                           int(rng.integers(0, 8000))).astype(np.uint32))
            _check_case(handle, oracle, c)


def test_fp64_determinant_flag(handle, oracle):
    for c in (synth.plain_rect_case(), synth.plain_exp_case()):
        _check_case(handle, oracle, c, flags=FLAGS_ALL | 0x4)


def test_uncompensated_flag_runs_and_is_less_accurate(handle, oracle):
    c = synth.plain_exp_case()
    F, _ = handle.map_plain_host(c["atoms"], 1800, c["t0_data"], 2, c["t0s"], c["taus"],
                                 flags=0x1 | 0x8)
    F64, cond = oracle.map_f64(c["atoms"], 1800, c["t0_data"], 2, c["t0s"], c["taus"],
                               with_cond=True)
    rel, _ = rel_err(F, F64, cond)
    good = cond < 100
    assert rel[good].max() < 1e-3
    assert rel.max() > REL_TOL


def test_window_none_is_one_rect_cell(handle, oracle):
    t0_data, A = synth.merged_atoms(6, 200, 1)
    F, res = handle.map_plain_host(A, 1800, t0_data, 0, [], [], flags=FLAGS_ALL)
    F64 = oracle.map_f64(A, 1800, t0_data, 1, [t0_data], [A.shape[0] * 1800])
    assert F.shape == (1, 1)
    assert abs(F[0, 0] - F64[0, 0]) / F64[0, 0] < REL_TOL


def test_device_pointer_entry_on_torch_stream(lib, handle, oracle):
    torch = pytest.importorskip("torch")
    c = synth.plain_rect_case()
    dev = torch.device("cuda:0")
    A = torch.from_numpy(c["atoms"]).to(dev)
    t0s = torch.from_numpy(c["t0s"].astype(np.int32)).to(dev)
    taus = torch.from_numpy(c["taus"].astype(np.int32)).to(dev)
    Fmn = torch.empty((len(c["t0s"]), len(c["taus"])), dtype=torch.float32, device=dev)
    res = torch.zeros(5, dtype=torch.float64, device=dev)  # 40-byte tcw_result
    # torch's default stream is handle 0; 0x1 (cudaStreamLegacy) names it for the library
    handle.set_stream(torch.cuda.current_stream().cuda_stream or 0x1)
    try:
        handle.map_plain(A, A.shape[0], 1800, c["t0_data"], 1, t0s, len(c["t0s"]), taus,
                         len(c["taus"]), Fmn, res, flags=FLAGS_ALL)
        torch.cuda.synchronize()
    finally:
        handle.set_stream(None)
    F = Fmn.cpu().numpy()
    rec = res.cpu().numpy().view(lib.RESULT_DTYPE)[0]
    F64, cond = oracle.map_f64(c["atoms"], 1800, c["t0_data"], 1, c["t0s"], c["taus"],
                               with_cond=True)
    rel, _ = rel_err(F, F64, cond)
    assert rel.max() < REL_TOL
    assert argmax_ok(rec["argmax"], F64)


def test_errors_are_status_codes_and_handle_survives(lib, handle):
    c = synth.plain_rect_case()
    with pytest.raises(lib.TcwError) as e:
        handle.map_plain_host(c["atoms"][:0], 1800, c["t0_data"], 1, c["t0s"], c["taus"])
    assert e.value.code == lib.TCW_ERR_INVALID_ARG
    with pytest.raises(lib.TcwError) as e:
        handle.map_plain_host(c["atoms"], 1800, c["t0_data"], 7, c["t0s"], c["taus"])
    assert e.value.code == lib.TCW_ERR_INVALID_ARG
    with pytest.raises(lib.TcwError) as e:  # rect needs non-decreasing taus
        handle.map_plain_host(c["atoms"], 1800, c["t0_data"], 1, c["t0s"], c["taus"][::-1])
    assert e.value.code == lib.TCW_ERR_INVALID_ARG
    with pytest.raises(lib.TcwError) as e:  # timestamps beyond u32
        handle.map_plain_host(c["atoms"], 1800, 0xFFFF0000, 1, c["t0s"], c["taus"])
    assert e.value.code == lib.TCW_ERR_OVERFLOW
    # allocation failure injected on the host: clean error, handle still usable
    h2 = lib.Handle(0)
    try:
        h2.fail_alloc(1)
        with pytest.raises(lib.TcwError) as e:
            h2.map_plain_host(c["atoms"], 1800, c["t0_data"], 1, c["t0s"], c["taus"])
        assert e.value.code == lib.TCW_ERR_ALLOC
        F, res = h2.map_plain_host(c["atoms"], 1800, c["t0_data"], 1, c["t0s"], c["taus"])
        assert np.isfinite(res["maxF"])
        h2.sync(1000)
    finally:
        h2.close()


def test_drop_in_dispatcher(oracle):
    """call_compute_transient_fstat_map with version 'b200' (tcw:495-544)."""
    from pyfstat_gb300 import tcw_fstat_map_funcs as tcw
    from pyfstat_gb300.window import transientWindowRange_t

    features, ctx = tcw.init_transient_fstat_map_features("b200")
    try:
        assert features["b200"]
        multi = synth.multi_detector_atoms(1, 48, 1, inject=(12, 24))
        for wtype in (1, 2):
            wr = transientWindowRange_t(type=wtype, t0=700000000, t0Band=86400 - 3600, dt0=1800,
                                        tau=3600, tauBand=86400 - 3600, dtau=1800)
            FstatMap, timing = tcw.call_compute_transient_fstat_map("b200", features, multi, wr,
                                                                    BtSG=True)
            assert timing >= 0
            t0_data, A = synth.merged_atoms(1, 48, 1, inject=(12, 24))
            t0s = 700000000 + 1800 * np.arange(47)
            taus = 3600 + 1800 * np.arange(47)
            F64 = oracle.map_f64(A, 1800, t0_data, wtype, t0s, taus)
            m, n = np.unravel_index(np.argmax(F64), F64.shape)
            assert FstatMap.F_mn.shape == (47, 47) and FstatMap.F_mn.dtype == np.float32
            assert FstatMap.maxF == pytest.approx(F64.max(), rel=REL_TOL)
            assert (FstatMap.t0_ML, FstatMap.tau_ML) == (t0s[m], taus[n])
            assert FstatMap.lnBtSG == pytest.approx(oracle.lnBtSG(F64), rel=REL_TOL)
            dx, dy = wr.t0Band / 47, wr.tauBand / 47
            assert FstatMap.t0_MP == wr.t0 + (oracle.t0_max_posterior_idx(F64) + 0.5) * dx
            assert FstatMap.tau_MP == wr.tau + (oracle.tau_max_posterior_idx(F64) + 0.5) * dy
            # the host-side methods of the result type agree with the device
            assert FstatMap.get_lnBtSG() == pytest.approx(FstatMap.lnBtSG, rel=1e-6)
        # window type 'none'
        wr = transientWindowRange_t(type=0)
        FstatMap, _ = tcw.call_compute_transient_fstat_map("b200", features, multi, wr)
        assert wr.type == 1 and FstatMap.F_mn.shape == (1, 1)
    finally:
        if ctx:
            ctx.detach()


def test_maps_differ_from_the_reference_maps_only_by_its_own_rounding(handle, oracle, golden):
    """Against the reference's own outputs (its pycuda kernels' FP32 maps in
    the golden file): every cell of the GPU map lies within the reference's
    own distance from FP64 plus 1e-5 relative of it -- the two differ only
    by the reference's FP32 rounding."""
    names = sorted({k.split("__")[0] for k in golden.files})
    worst_ref = 0.0
    for name in names:
        g = golden[f"{name}__grid"]
        window, TAtom, t0_data = int(g[0]), int(g[1]), int(g[2])
        if f"{name}__t0s" in golden.files:
            t0s, taus = golden[f"{name}__t0s"], golden[f"{name}__taus"]
        else:
            c = golden_case(golden, name)
            t0s, taus = c["t0s"], c["taus"]
        A = golden[f"{name}__atoms"]
        F, _ = handle.map_plain_host(A, TAtom, t0_data, window, t0s, taus, want_map=True)
        F64, cond = oracle.map_f64(A, TAtom, t0_data, window if window else 1,
                                   t0s if window else np.array([t0_data], np.uint32),
                                   taus if window else np.array([A.shape[0] * TAtom], np.uint32),
                                   with_cond=True)
        if f"{name}__F" in golden.files:
            Fref, rows = golden[f"{name}__F"], slice(None)
        else:
            Fref, rows = golden[f"{name}__F_rows16"], slice(None, None, 16)
        Fg, F64r, cr = F[rows].astype(np.float64), F64[rows], cond[rows]
        band = np.abs(cr / 1e4 - 1.0) < 1e-5
        ref_err = np.abs(Fref.astype(np.float64) - F64r)
        ok = np.abs(Fg - Fref) <= ref_err + REL_TOL * np.abs(F64r) + 1e-12
        assert np.all(ok | band), name
        worst_ref = max(worst_ref, float(np.max(np.where(band, 0, ref_err / np.abs(F64r)))))
    print(f"\nreference FP32 maps' own max rel err vs FP64 over the golden cases: {worst_ref:.3e}")
