"""Sharding across ranks (host logic, CPU): cost partition, exact merges of
row-split templates, and a world_size-2 gloo run of the gather."""

import socket

import numpy as np
import pytest

from pyfstat_gb300 import _lib, shard, synth
from pyfstat_gb300.batched import template_grids


def test_partition_covers_each_template_once_and_balances():
    rng = np.random.default_rng(0)
    costs = rng.uniform(1, 100, 257)
    for ws in (1, 2, 3, 8):
        parts = shard.partition(costs, ws)
        allidx = np.sort(np.concatenate(parts))
        assert np.array_equal(allidx, np.arange(costs.size))
        loads = np.array([costs[p].sum() for p in parts])
        # LPT bound: no rank exceeds the mean by more than the largest cost
        assert loads.max() <= costs.sum() / ws + costs.max()
        assert all(np.all(np.diff(p) > 0) for p in parts)
    assert all(np.array_equal(a, b) for a, b in zip(shard.partition(costs, 4),
                                                   shard.partition(costs, 4)))
    with pytest.raises(ValueError):
        shard.partition(costs, 0)


def test_cost_grows_with_cells_and_exponential_windows():
    t = synth.batched_templates(2, seed=5, nsft_range=(100, 100), grid_range=(50, 50))
    rect, exp = t[0], t[1]
    assert rect["window"] == 1 and exp["window"] == 2
    assert shard.template_cost(exp) > shard.template_cost(rect)
    big = dict(rect, N_t0=100)
    assert shard.template_cost(big) == 2 * shard.template_cost(rect)


def records_from_map(F):
    r = np.zeros(1, dtype=_lib.RESULT_DTYPE)[0]
    k = int(np.argmax(F))
    Fd = F.astype(np.float64).reshape(-1)
    m = Fd.max()
    r["maxF"] = F.reshape(-1)[k]
    r["argmax"] = k
    r["lnBtSG"] = np.log(70.0 / Fd.size) + m + np.log(np.sum(np.exp(Fd - m)))
    return r


@pytest.mark.parametrize("n_blocks", [1, 2, 3, 7])
def test_merge_of_row_blocks_equals_the_whole_map(n_blocks):
    rng = np.random.default_rng(n_blocks)
    N_t0, N_tau = 23, 11
    # integer-valued F with many exact ties across blocks
    F = rng.integers(0, 6, (N_t0, N_tau)).astype(np.float32) * 7.0
    edges = np.linspace(0, N_t0, n_blocks + 1).round().astype(int)
    parts = [(lo, hi - lo, records_from_map(F[lo:hi]))
             for lo, hi in zip(edges[:-1], edges[1:]) if hi > lo]
    merged = shard.merge_split(parts, N_t0, N_tau)
    full = records_from_map(F)
    assert merged["argmax"] == full["argmax"] == int(np.argmax(F))
    assert merged["maxF"] == full["maxF"]
    assert merged["lnBtSG"] == pytest.approx(float(full["lnBtSG"]), rel=1e-13, abs=1e-12)
    assert merged["t0_mp_idx"] == -1 and merged["tau_mp_idx"] == -1


def test_split_rows_runs_as_templates_and_merges_to_the_full_result(oracle):
    from _shard_worker import oracle_compute

    t = synth.batched_templates(2, seed=8, nsft_range=(60, 60), grid_range=(30, 30))[1]
    t0s, taus = template_grids(t)
    blocks = shard.split_rows(t, 4)
    assert sum(p["N_t0"] for _, p in blocks) == t0s.shape[0]
    res = oracle_compute([p for _, p in blocks])
    merged = shard.merge_split([(off, p["N_t0"], r) for (off, p), r in zip(blocks, res)],
                               t0s.shape[0], taus.shape[0])
    full = oracle_compute([t])[0]
    assert merged["argmax"] == full["argmax"]
    assert merged["maxF"] == full["maxF"]
    assert merged["lnBtSG"] == pytest.approx(float(full["lnBtSG"]), rel=1e-13)


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_gloo_world_size_2_gathers_every_template(tmp_path, oracle):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    import _shard_worker as W

    out = tmp_path / "res.npy"
    mp.start_processes(W.worker, args=(2, free_port(), str(out)), nprocs=2, join=True,
                       start_method="spawn")
    got = np.load(out).view(_lib.RESULT_DTYPE).reshape(-1)
    want = W.oracle_compute(W.templates())
    assert np.array_equal(got["argmax"], want["argmax"])
    assert np.array_equal(got["maxF"], want["maxF"])
    np.testing.assert_allclose(got["lnBtSG"], want["lnBtSG"], rtol=1e-14)
