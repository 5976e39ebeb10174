"""Host logic of the tile autotuner: workload signature, template sampling
and sub-batch extraction (no GPU)."""

import numpy as np

from pyfstat_gb300 import _lib, autotune, synth
from pyfstat_gb300.batched import pack_templates


def templates(n=40, seed=7):
    return synth.batched_templates(n, seed=seed, nsft_range=(20, 120), grid_range=(4, 60))


def test_subset_equals_packing_the_chosen_templates():
    tl = templates()
    atoms, desc, t0s, taus = pack_templates(tl)
    idx = np.array([1, 4, 5, 17, 38])
    sd, st0, stau, sa = autotune.subset(desc, t0s, taus, atoms, idx)
    ra, rd, rt0, rtau = pack_templates([tl[i] for i in idx])
    assert np.array_equal(sd, rd)
    assert np.array_equal(st0, rt0) and np.array_equal(stau, rtau)
    assert np.array_equal(sa, ra)


def test_sample_covers_both_windows_and_the_budget():
    _, desc, _, _ = pack_templates(templates())
    cells = desc["N_t0"].astype(np.float64) * desc["N_tau"]
    idx = autotune.sample_templates(desc, budget_cells=2000.0, seed=3)
    for w in (_lib.TCW_WINDOW_RECT, _lib.TCW_WINDOW_EXP):
        sel = idx[desc["window"][idx] == w]
        assert sel.size >= 1
        # the sample reaches the budget unless it takes every template of the type
        assert cells[sel].sum() >= 2000.0 or sel.size == np.sum(desc["window"] == w)
    # a budget above the total takes every template
    idx_all = autotune.sample_templates(desc, budget_cells=1e12)
    assert np.array_equal(np.sort(idx_all), np.arange(desc.shape[0]))
    # seeded
    assert np.array_equal(idx, autotune.sample_templates(desc, budget_cells=2000.0, seed=3))


def test_signature_depends_on_the_mix_not_on_the_order():
    tl = templates()
    _, desc, _, _ = pack_templates(tl)
    _, desc_rev, _, _ = pack_templates(tl[::-1])
    assert autotune.signature(desc) == autotune.signature(desc_rev)
    _, desc_rect, _, _ = pack_templates([t for t in tl if t["window"] == 1])
    assert autotune.signature(desc_rect) != autotune.signature(desc)
    assert "w2:0" in autotune.signature(desc_rect)


def test_cache_round_trip(tmp_path, monkeypatch):
    p = tmp_path / "tiles.json"
    monkeypatch.setenv("PYFSTAT_GB300_TUNE_CACHE", str(p))
    assert autotune.cache_path() == str(p)
    autotune._store_cache(str(p), {"k": {"rect_tm": 64}})
    assert autotune._load_cache(str(p)) == {"k": {"rect_tm": 64}}
    assert autotune._load_cache(str(tmp_path / "missing.json")) == {}
