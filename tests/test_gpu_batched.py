"""Batched plans (persistent kernel, CUDA graph) against the FP64 oracle and
against the plain per-template path."""

import numpy as np
import pytest

from _helpers import REL_TOL, argmax_ok
from pyfstat_gb300 import synth
from pyfstat_gb300.batched import TransientMapBatch, template_grids

pytestmark = pytest.mark.gpu


def small_templates(n=24, seed=3):
    """Mixed rect/exp templates with uneven atom counts, gaps and grids small
    enough for the CPU oracle."""
    return synth.batched_templates(n, seed=seed, nsft_range=(30, 260), gap_range=(0.0, 0.3),
                                   grid_range=(1, 90))


def oracle_reference(oracle, t):
    t0s, taus = template_grids(t)
    F64, cond = oracle.map_f64(t["atoms"], t["TAtom"], t["t0_data"], t["window"], t0s, taus,
                               with_cond=True)
    return F64, cond


@pytest.fixture(scope="module")
def batch():
    b = TransientMapBatch(small_templates())
    yield b
    b.close()


def test_batched_matches_fp64_oracle(batch, oracle):
    res = batch.run()
    templates = small_templates()
    for k, t in enumerate(templates):
        F64, cond = oracle_reference(oracle, t)
        band = np.abs(cond / 1e4 - 1) < 1e-5
        assert float(res["maxF"][k]) == pytest.approx(F64.max(), rel=REL_TOL), k
        if not band.any():
            assert argmax_ok(res["argmax"][k], F64), k
            assert float(res["lnBtSG"][k]) == pytest.approx(oracle.lnBtSG(F64), rel=REL_TOL,
                                                            abs=1e-6), k


def test_batched_equals_plain_path(batch):
    from pyfstat_gb300 import _lib

    res = batch.run()
    h = batch.handle
    for k, t in enumerate(small_templates()):
        t0s, taus = template_grids(t)
        F, r = h.map_plain_host(t["atoms"], t["TAtom"], t["t0_data"], t["window"], t0s, taus,
                                want_map=True, flags=_lib.TCW_FLAG_LNBTSG)
        # rect cells read the same prefix rows: identical; exp recurrences start
        # where each tile's rows start, so values agree to rounding only
        if t["window"] == 1:
            assert float(res["maxF"][k]) == float(r["maxF"]), k
            assert int(res["argmax"][k]) == int(r["argmax"]), k
        else:
            assert float(res["maxF"][k]) == pytest.approx(float(r["maxF"]), rel=2e-6), k
            assert float(F.reshape(-1)[int(res["argmax"][k])]) == pytest.approx(
                float(r["maxF"]), rel=2e-6), k
        assert float(res["lnBtSG"][k]) == pytest.approx(float(r["lnBtSG"]), rel=1e-6), k


@pytest.mark.parametrize("cfg", [
    dict(rect_tn=7, rect_tm=32, exp_tn=32, exp_rows=3, blocks_per_sm=2),
    dict(rect_tn=64, rect_tm=64, exp_tn=64, exp_rows=0, blocks_per_sm=4),
    dict(rect_tn=300, rect_tm=128, exp_tn=128, exp_rows=17, blocks_per_sm=16),
])
def test_tile_shapes_do_not_change_results(batch, cfg):
    ref = batch.run()
    b2 = TransientMapBatch(small_templates(), tile_config=cfg, handle=batch.handle)
    try:
        res = b2.run()
    finally:
        b2.close()
    rect = batch.desc["window"] == 1
    assert np.array_equal(res["maxF"][rect], ref["maxF"][rect])
    assert np.array_equal(res["argmax"][rect], ref["argmax"][rect])
    np.testing.assert_allclose(res["maxF"], ref["maxF"], rtol=2e-6)
    np.testing.assert_allclose(res["lnBtSG"], ref["lnBtSG"], rtol=1e-6)


def test_graph_replay_on_device_buffers(batch):
    torch = pytest.importorskip("torch")
    from pyfstat_gb300 import _lib

    dev = torch.device("cuda:0")
    d_atoms = torch.from_numpy(batch.atoms).to(dev)
    d_res = torch.zeros(batch.n_templates * 5, dtype=torch.float64, device=dev)
    side = torch.cuda.Stream(device=dev)
    side.wait_stream(torch.cuda.current_stream())
    batch.handle.set_stream(side.cuda_stream)
    ctx = torch.cuda.stream(side)
    ctx.__enter__()
    try:
        outs = []
        for _ in range(3):
            batch.run_device(d_atoms, d_res, use_graph=True)
            torch.cuda.synchronize()
            outs.append(d_res.cpu().numpy().view(_lib.RESULT_DTYPE).copy())
        # new atoms through the same captured graph (same buffer, new contents)
        d_atoms.mul_(2.0)
        batch.run_device(d_atoms, d_res, use_graph=True)
        torch.cuda.synchronize()
        scaled = d_res.cpu().numpy().view(_lib.RESULT_DTYPE).copy()
    finally:
        ctx.__exit__(None, None, None)
        batch.handle.set_stream(None)
    ref = batch.run()
    for o in outs:
        assert np.array_equal(o["maxF"], ref["maxF"])
        assert np.array_equal(o["argmax"], ref["argmax"])
    # F is invariant under a common scale of a2,b2,ab by s and Fa,Fb by s...
    # with s = 2 on all channels F scales by 2 (F ~ |F|^2 / M): maxF doubles
    np.testing.assert_allclose(scaled["maxF"][ref["maxF"] != 2], 2 * ref["maxF"][ref["maxF"] != 2],
                               rtol=1e-5)


def test_single_cell_and_single_atom_templates(oracle):
    t0_data, A = synth.merged_atoms(5, 1, 1, inject=None)
    t0_data2, A2 = synth.merged_atoms(6, 40, 1)
    templates = [
        dict(window=1, atoms=A, TAtom=1800, t0_data=t0_data, t0=t0_data, dt0=1800, N_t0=1,
             tau=1800, dtau=1800, N_tau=1),
        dict(window=2, atoms=A2, TAtom=1800, t0_data=t0_data2, t0=t0_data2, dt0=1800, N_t0=1,
             tau=1800 * 40, dtau=1, N_tau=1),
        dict(window=1, atoms=A2, TAtom=1800, t0_data=t0_data2, t0=t0_data2, dt0=1800, N_t0=1,
             tau=1800 * 40, dtau=1, N_tau=1),
    ]
    b = TransientMapBatch(templates)
    try:
        res = b.run()
    finally:
        b.close()
    assert res["maxF"][0] == 2.0  # one atom: ill-conditioned -> F = 2
    for k in (1, 2):
        t = templates[k]
        F64, _ = oracle_reference(oracle, t)
        assert float(res["maxF"][k]) == pytest.approx(F64[0, 0], rel=REL_TOL)


def test_autotuned_plan_matches_default_plan(tmp_path, monkeypatch):
    monkeypatch.setenv("PYFSTAT_GB300_TUNE_CACHE", str(tmp_path / "tiles.json"))
    tl = small_templates(n=32, seed=9)
    ref = TransientMapBatch(tl)
    tuned = TransientMapBatch(tl, tile_config="auto", handle=ref.handle)
    cfg = tuned.tile_config
    assert cfg["rect_tm"] in (32, 64, 128) and cfg["exp_tn"] in (32, 64, 128)
    a, b = ref.run(), tuned.run()
    rect = ref.desc["window"] == 1
    assert np.array_equal(a["maxF"][rect], b["maxF"][rect])
    np.testing.assert_allclose(b["maxF"], a["maxF"], rtol=2e-6)
    # exp cells round differently under another chunking (<= 2e-6 relative),
    # and the log-sum-exp partial sums are merged in another order
    np.testing.assert_allclose(b["lnBtSG"], a["lnBtSG"], rtol=2e-6)
    # a second construction reads the cache
    again = TransientMapBatch(tl, tile_config="auto", handle=ref.handle)
    assert again.tile_config == cfg
    for x in (again, tuned, ref):
        x.close()


def test_plan_maps_and_posteriors_equal_the_plain_path():
    """tcw_plan_run_maps: every template's map equals the plain per-template
    map (rect bit for bit, exp within the chunking rounding), and a
    TCW_FLAG_POSTERIORS plan's posterior indices equal the plain path's."""
    from pyfstat_gb300 import _lib

    tl = small_templates(n=16, seed=21)
    flags = _lib.TCW_FLAG_LNBTSG | _lib.TCW_FLAG_POSTERIORS
    batch = TransientMapBatch(tl, flags=flags)
    res, maps = batch.plan.run_maps_host(batch.atoms)
    off = 0
    for k, t in enumerate(tl):
        t0s, taus = template_grids(t)
        n = t0s.size * taus.size
        F, rec = batch.handle.map_plain_host(t["atoms"], t["TAtom"], t["t0_data"], t["window"],
                                             t0s, taus, want_map=True, flags=flags)
        Fb = maps[off:off + n].reshape(t0s.size, taus.size)
        if t["window"] == 1:
            assert np.array_equal(Fb, F)
        else:
            # both within ~2e-6 of FP64 (tier-1 bound), so within 4e-6 of each other
            np.testing.assert_allclose(Fb, F, rtol=4e-6)
        if t["window"] == 1 or np.array_equal(Fb, F):
            assert res["t0_mp_idx"][k] == rec["t0_mp_idx"]
            assert res["tau_mp_idx"][k] == rec["tau_mp_idx"]
        off += n
    # a posterior plan needs the maps
    with pytest.raises(_lib.TcwError):
        batch.run()
    batch.close()


def test_golden_cases_in_one_persistent_launch(oracle, golden):
    """Every golden case (clamps, u32 wrap, tiny grids, gaps, off-grid steps)
    as one template of a single batched plan with maps and posteriors: each
    map against the FP64 oracle, and maxF, argmax, lnBtSG and the posterior
    indices as for the plain path."""
    from _helpers import golden_case, golden_cases, index_ok, rel_err
    from pyfstat_gb300 import _lib

    cases = [golden_case(golden, n) for n in golden_cases(golden)]
    cases = [c for c in cases if c["window"] in (1, 2)]
    flags = _lib.TCW_FLAG_LNBTSG | _lib.TCW_FLAG_POSTERIORS
    batch = TransientMapBatch([dict(c, t0s=c["t0s"], taus=c["taus"]) for c in cases],
                              flags=flags)
    res, maps = batch.plan.run_maps_host(batch.atoms)
    off = 0
    for k, c in enumerate(cases):
        n = c["t0s"].size * c["taus"].size
        F = maps[off:off + n].reshape(c["t0s"].size, c["taus"].size)
        off += n
        F64, cond = oracle.map_f64(c["atoms"], c["TAtom"], c["t0_data"], c["window"], c["t0s"],
                                   c["taus"], with_cond=True)
        rel, nband = rel_err(F, F64, cond)
        assert rel.max() < REL_TOL, (c["name"], rel.max())
        assert float(res["maxF"][k]) == float(F.max()), c["name"]
        assert int(res["argmax"][k]) == int(np.argmax(F)), c["name"]
        if nband == 0:
            assert argmax_ok(res["argmax"][k], F64), c["name"]
            assert float(res["lnBtSG"][k]) == pytest.approx(oracle.lnBtSG(F64), rel=REL_TOL,
                                                            abs=1e-6), c["name"]
            e = np.exp(F64 - F64.max())
            assert index_ok(res["t0_mp_idx"][k], e.sum(axis=1)), c["name"]
            assert index_ok(res["tau_mp_idx"][k], e.sum(axis=0)), c["name"]
    batch.close()


def test_exp_template_with_more_than_65535_rows(oracle):
    """Row chunks of exponential tiles are 16-bit counts: a column of 70,000
    t0 rows must be split, not truncated (plain and batched paths)."""
    from pyfstat_gb300 import _lib

    t0_data, A = synth.merged_atoms(77, 120, 2, gap_frac=0.05)
    t0s = (t0_data + 3 * np.arange(70000)).astype(np.uint32)  # 3 s steps over ~58 h
    taus = np.array([1800, 9000, 36000, 90000], dtype=np.uint32)
    F64, cond = oracle.map_f64(A, 1800, t0_data, 2, t0s, taus, with_cond=True)
    band = np.abs(cond / 1e4 - 1) < 1e-5
    h = _lib.Handle(0)
    try:
        F, res = h.map_plain_host(A, 1800, t0_data, 2, t0s, taus, want_map=True)
        rel = np.where(band, 0, np.abs(F - F64) / np.abs(F64))
        assert rel.max() < REL_TOL
        tmpl = dict(atoms=A, TAtom=1800, t0_data=t0_data, window=2, t0s=t0s, taus=taus)
        b = TransientMapBatch([tmpl], handle=h)
        r = b.run()[0]
        b.close()
        assert abs(float(r["maxF"]) - F64.max()) <= REL_TOL * F64.max()
        assert argmax_ok(r["argmax"], F64)
    finally:
        h.close()


def test_all_gap_templates_give_the_fallback_everywhere(oracle):
    """Templates whose atoms are all zero (data gaps only): every cell is the
    F = 2 fallback, maxF = 2 and lnBtSG = ln 70 + 2, on both paths."""
    from pyfstat_gb300 import _lib

    A = np.zeros((50, 7), np.float32)
    t0_data = 700000000
    t0s = (t0_data + 1800 * np.arange(30)).astype(np.uint32)
    taus = (1800 + 3600 * np.arange(12)).astype(np.uint32)
    tl = [dict(atoms=A, TAtom=1800, t0_data=t0_data, window=w, t0s=t0s, taus=taus)
          for w in (1, 2)]
    b = TransientMapBatch(tl)
    res = b.run()
    for k, w in enumerate((1, 2)):
        F64 = oracle.map_f64(A, 1800, t0_data, w, t0s, taus)
        assert np.all(F64 == 2.0)
        F, r = b.handle.map_plain_host(A, 1800, t0_data, w, t0s, taus, want_map=True,
                                       flags=_lib.TCW_FLAG_LNBTSG)
        assert np.all(F == 2.0)
        for rec in (r, res[k]):
            assert float(rec["maxF"]) == 2.0 and int(rec["argmax"]) == 0
            assert float(rec["lnBtSG"]) == pytest.approx(np.log(70.0) + 2.0, rel=1e-12)
    b.close()


def test_one_shot_map_batched_equals_the_plan(batch):
    from pyfstat_gb300.batched import map_batched

    res = batch.run()
    max2F, argmax, lnB = map_batched(small_templates(), handle=batch.handle)
    assert np.array_equal(max2F, 2.0 * res["maxF"])
    assert np.array_equal(argmax, res["argmax"])
    assert np.array_equal(lnB, res["lnBtSG"])


@pytest.mark.parametrize("uncompensated", [False, True])
def test_pipelined_runs_equal_synchronous_runs(batch, uncompensated):
    """tcw_plan_run_host_async: each upload overlaps the previous run's map
    kernels (waits for them too where they read the atoms themselves: the
    uncompensated variant); every run's results equal a synchronous run on
    the same atoms."""
    from pyfstat_gb300 import _lib

    if uncompensated:
        batch = TransientMapBatch(small_templates(), handle=batch.handle,
                                  flags=_lib.TCW_FLAG_LNBTSG | _lib.TCW_FLAG_UNCOMPENSATED)
    rng = np.random.default_rng(5)
    arrays = []
    for _ in range(4):
        a = batch.atoms.copy()
        a[:, 3:] *= rng.uniform(0.5, 2.0, size=(a.shape[0], 4)).astype(np.float32)
        arrays.append(a)
    out = batch.run_pipelined(arrays)
    for a, r in zip(arrays, out):
        ref = batch.run(a)
        for key in ("maxF", "argmax", "lnBtSG"):
            assert np.array_equal(r[key], ref[key]), key
    assert not np.array_equal(out[0]["maxF"], out[1]["maxF"])
    # a synchronous run between pipelined ones, page-locked atoms
    from pyfstat_gb300 import _lib

    pinned = _lib.pinned_empty(arrays[2].shape)
    pinned[:] = arrays[2]
    batch.plan.run_host_async(pinned)
    mid = batch.run(arrays[3])
    batch.plan.run_host_async(arrays[0])
    r0, r1 = batch.plan.wait()
    assert np.array_equal(r0["maxF"], out[2]["maxF"])
    assert np.array_equal(mid["maxF"], out[3]["maxF"])
    assert np.array_equal(r1["maxF"], out[0]["maxF"])
    if uncompensated:
        batch.close()


def test_pipelined_run_rejects_posterior_plans_and_handle_survives(batch):
    from pyfstat_gb300 import _lib

    b2 = TransientMapBatch(small_templates(), handle=batch.handle,
                           flags=_lib.TCW_FLAG_LNBTSG | _lib.TCW_FLAG_POSTERIORS)
    try:
        with pytest.raises(_lib.TcwError) as e:
            b2.plan.run_host_async(b2.atoms)
        assert e.value.code == _lib.TCW_ERR_INVALID_ARG
        assert b2.plan.wait() == []
    finally:
        b2.close()
    out = batch.run_pipelined([batch.atoms])
    ref = batch.run()
    assert np.array_equal(out[0]["maxF"], ref["maxF"])


def random_templates(seed):
    """Random geometries in the style of the host tests' random grids: t0
    grids off the atom grid and starting before the data (u32 wrap of
    t0 - t0_data), taus with dtau = 0 included, gap runs of zero atoms."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(24):
        t0_data, A = synth.merged_atoms(1000 * seed + k, int(rng.integers(20, 300)),
                                        int(rng.integers(1, 3)),
                                        gap_frac=float(rng.uniform(0, 0.5)))
        A = A.copy()
        for _ in range(int(rng.integers(0, 4))):
            s = int(rng.integers(0, A.shape[0]))
            A[s:s + int(rng.integers(1, 40))] = 0
        nt0, ntau = int(rng.integers(1, 60)), int(rng.integers(1, 60))
        t0 = int(t0_data + rng.integers(-5000, 3000))
        t0s = (t0 + np.arange(nt0) * int(rng.integers(1, 4000))).astype(np.uint32)
        taus = (int(rng.integers(1, 5000)) + np.arange(ntau) * int(rng.integers(0, 8000))
                ).astype(np.uint32)
        out.append(dict(window=1 + k % 2, atoms=A, TAtom=1800, t0_data=t0_data, t0s=t0s,
                        taus=taus))
    return out


@pytest.mark.parametrize("seed,cfg", [
    (1, None),
    (2, dict(rect_tn=5, rect_tm=32, exp_tn=32, exp_rows=7, blocks_per_sm=3)),
    (3, dict(rect_tn=64, rect_tm=128, exp_tn=64, exp_rows=0, blocks_per_sm=8)),
])
def test_random_geometries_in_one_launch(oracle, seed, cfg):
    """Random geometries (u32 wrap, off-grid steps, dtau = 0, gaps) of both
    windows in one persistent launch, against the FP64 oracle."""
    templates = random_templates(seed)
    b = TransientMapBatch(templates, tile_config=cfg)
    try:
        res = b.run()
    finally:
        b.close()
    for k, t in enumerate(templates):
        F64, cond = oracle.map_f64(t["atoms"], 1800, t["t0_data"], t["window"], t["t0s"],
                                   t["taus"], with_cond=True)
        band = np.abs(cond / 1e4 - 1) < 1e-5
        assert float(res["maxF"][k]) == pytest.approx(F64.max(), rel=REL_TOL), (seed, k)
        if not band.any():
            assert argmax_ok(res["argmax"][k], F64), (seed, k)
            assert float(res["lnBtSG"][k]) == pytest.approx(oracle.lnBtSG(F64), rel=REL_TOL,
                                                            abs=1e-6), (seed, k)
