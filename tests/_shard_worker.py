"""Rank body of the gloo sharding test (spawned processes; CPU only)."""

import os
import sys

import numpy as np


def oracle_compute(templates):
    """Per-template result records from the oracle's FP32 port (CPU stand-in
    for the GPU compute of a rank): maxF, first-occurrence argmax and an FP64
    log-sum-exp lnBtSG of the FP32 map."""
    import oracle as O
    from pyfstat_gb300 import _lib
    from pyfstat_gb300.batched import template_grids

    out = np.zeros(len(templates), dtype=_lib.RESULT_DTYPE)
    for k, t in enumerate(templates):
        t0s, taus = template_grids(t)
        fn = O.rect_map_f32 if t["window"] == 1 else O.exp_map_f32
        F = fn(t["atoms"], t["TAtom"], t["t0_data"], t0s, taus, nthreads=1)
        mx, am = O.max_argmax(F)
        Fd = F.astype(np.float64).reshape(-1)
        m = Fd.max()
        out[k]["maxF"] = mx
        out[k]["argmax"] = am
        out[k]["lnBtSG"] = np.log(70.0 / Fd.size) + m + np.log(np.sum(np.exp(Fd - m)))
    return out


def templates():
    from pyfstat_gb300 import synth

    return synth.batched_templates(9, seed=21, nsft_range=(20, 90), grid_range=(3, 40))


def worker(rank, world_size, port, result_path):
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, repo)
    sys.path.insert(0, os.path.join(repo, "oracle"))
    import torch.distributed as dist

    from pyfstat_gb300 import shard

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world_size)
    try:
        res = shard.run_sharded(templates(), compute=oracle_compute)
        if rank == 0:
            np.save(result_path, res.view(np.uint8))
        else:
            assert res is None
    finally:
        dist.destroy_process_group()
