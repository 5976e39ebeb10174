"""The sharded path with its default GPU compute function on one GPU: a
world-size-1 gloo group runs shard.run_sharded (partition, batched GPU
compute, gather) and row-split templates are merged with shard.merge_split;
both against the FP64 oracle."""

import socket

import numpy as np
import pytest

from _helpers import REL_TOL, argmax_ok
from pyfstat_gb300 import shard, synth
from pyfstat_gb300.batched import template_grids

pytestmark = pytest.mark.gpu


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _templates():
    return synth.batched_templates(12, seed=77, nsft_range=(60, 300), grid_range=(20, 90),
                                   gap_range=(0.0, 0.3))


def _check_against_oracle(oracle, t, rec, label):
    t0s, taus = template_grids(t)
    F64 = oracle.map_f64(t["atoms"], t["TAtom"], t["t0_data"], t["window"], t0s, taus)
    assert float(rec["maxF"]) == pytest.approx(F64.max(), rel=REL_TOL), label
    assert argmax_ok(int(rec["argmax"]), F64, label=label), label
    assert float(rec["lnBtSG"]) == pytest.approx(oracle.lnBtSG(F64), rel=REL_TOL), label


def test_run_sharded_default_gpu_compute_world_size_1(oracle):
    torch = pytest.importorskip("torch")
    import torch.distributed as dist

    torch.cuda.set_device(0)
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{_free_port()}", rank=0,
                            world_size=1)
    try:
        ts = _templates()
        res = shard.run_sharded(ts)  # compute defaults to shard.gpu_compute
    finally:
        dist.destroy_process_group()
    assert res is not None and res.shape == (len(ts),)
    for k, t in enumerate(ts):
        _check_against_oracle(oracle, t, res[k], f"sharded template {k}")


def test_row_split_templates_merge_on_gpu(oracle):
    ts = _templates()
    for k in (0, 1, 4, 5):
        t = ts[k]
        t0s, taus = template_grids(t)
        whole = shard.gpu_compute([t])[0]
        for n_blocks in (2, 3, 7):
            blocks = shard.split_rows(t, n_blocks)
            recs = shard.gpu_compute([b for _, b in blocks])
            merged = shard.merge_split(
                [(off, int(b["N_t0"]), r) for (off, b), r in zip(blocks, recs)], len(t0s),
                len(taus))
            # rectangular cells do not depend on the row blocking, so max and first
            # argmax merge exactly; exponential columns restart their sliding sums
            # at each block's first row (rounding-level differences)
            if t["window"] == 1:
                assert float(merged["maxF"]) == float(whole["maxF"])
                assert int(merged["argmax"]) == int(whole["argmax"])
            else:
                assert float(merged["maxF"]) == pytest.approx(float(whole["maxF"]), rel=2e-6)
            assert float(merged["lnBtSG"]) == pytest.approx(float(whole["lnBtSG"]), rel=1e-6)
            _check_against_oracle(oracle, t, merged, f"split template {k} / {n_blocks}")
