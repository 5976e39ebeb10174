"""Tile-shape autotuner for batched plans.

The two map kernels of a plan are tuned independently (the timed run
launches them one after the other): the rectangular kernel over
(rows per tile, columns per tile) and the exponential kernel over (columns
per block, rows per thread chunk).  Timing uses ``tcw_plan_run_timed`` (CUDA
events between the kernels) on a seeded sample of the batch's templates of
about ``budget_cells`` cells per window type, best of ``repeats`` runs.  The
default budget (4e9 cells, some 15 ms of kernel time per window type) takes
whole batches of the benchmark's size: the persistent kernels' tails weigh
on a small sample far more than on the full batch (a 4e8-cell sample of the
4096-template batch gives each warp about two exponential tiles) and make
short row chunks look better than they are (19.5 ms with whole columns
against 21.3 ms with 1024-row chunks on the full batch).

Choices are cached per device name and workload signature (window mix and
log2-bucketed mean grid sizes and atom counts) in a JSON file:
``$PYFSTAT_GB300_TUNE_CACHE`` or ``~/.cache/pyfstat_gb300/tiles.json``.
"""

import json
import os

import numpy as np

from . import _lib

RECT_CANDIDATES = [(tm, tn) for tm in (32, 64, 128) for tn in (32, 64, 128, 256)]
# batched plans run exponential tiles as 32-column warp tiles: only the rows
# per tile (0 = whole columns) are tuned
EXP_CANDIDATES = [(32, rows) for rows in (0, 64, 256, 1024)]


def cache_path():
    p = os.environ.get("PYFSTAT_GB300_TUNE_CACHE")
    if p:
        return p
    return os.path.join(os.path.expanduser("~"), ".cache", "pyfstat_gb300", "tiles.json")


def signature(desc):
    """Workload key: per window type the template count bucket and the log2
    buckets of the mean N_t0, N_tau and numAtoms."""
    parts = []
    for w in (_lib.TCW_WINDOW_RECT, _lib.TCW_WINDOW_EXP):
        sel = desc[desc["window"] == w]
        if sel.shape[0] == 0:
            parts.append(f"w{w}:0")
            continue
        b = [int(np.round(np.log2(max(1.0, float(np.mean(sel[f]))))))
             for f in ("N_t0", "N_tau", "numAtoms")]
        nb = int(np.round(np.log2(sel.shape[0])))
        parts.append(f"w{w}:{nb}:{b[0]}:{b[1]}:{b[2]}")
    return "|".join(parts)


def _load_cache(path):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store_cache(path, cache):
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        tmp = path + f".{os.getpid()}.tmp"
        with open(tmp, "w") as f:
            json.dump(cache, f, indent=1, sort_keys=True)
        os.replace(tmp, path)
    except OSError:
        pass


def sample_templates(desc, budget_cells, seed=0):
    """Indices of a seeded random sample of templates, per window type, whose
    cells add up to about ``budget_cells`` (all templates when fewer)."""
    rng = np.random.default_rng(seed)
    keep = []
    for w in (_lib.TCW_WINDOW_RECT, _lib.TCW_WINDOW_EXP):
        idx = np.flatnonzero(desc["window"] == w)
        if idx.size == 0:
            continue
        idx = rng.permutation(idx)
        cells = np.cumsum(desc["N_t0"][idx].astype(np.float64) * desc["N_tau"][idx])
        n = int(np.searchsorted(cells, budget_cells)) + 1
        keep.append(np.sort(idx[:min(n, idx.size)]))
    return np.concatenate(keep) if keep else np.zeros(0, dtype=np.int64)


def subset(desc, t0s, taus, atoms, idx):
    """A self-contained (desc, t0s, taus, atoms) for the templates ``idx``."""
    sub = np.zeros(idx.size, dtype=_lib.DESC_DTYPE)
    a_parts, g_parts, u_parts = [], [], []
    a0 = g0 = u0 = 0
    for j, k in enumerate(idx):
        d = desc[k]
        na, nt0, ntau = int(d["numAtoms"]), int(d["N_t0"]), int(d["N_tau"])
        a_parts.append(atoms[int(d["atom_offset"]):int(d["atom_offset"]) + na])
        g_parts.append(t0s[int(d["t0_offset"]):int(d["t0_offset"]) + nt0])
        u_parts.append(taus[int(d["tau_offset"]):int(d["tau_offset"]) + ntau])
        sub[j] = (a0, g0, u0, na, d["TAtom"], d["t0_data"], d["window"], nt0, ntau)
        a0 += na
        g0 += nt0
        u0 += ntau
    return (sub, np.ascontiguousarray(np.concatenate(g_parts), np.uint32),
            np.ascontiguousarray(np.concatenate(u_parts), np.uint32),
            np.ascontiguousarray(np.concatenate(a_parts), np.float32))


def _time_plan(handle, desc, t0s, taus, cfg, flags, d_atoms, d_res, repeats):
    plan = _lib.Plan(handle, desc, t0s, taus, cfg, flags)
    try:
        plan.run_timed(d_atoms, d_res)  # warm-up (first-touch of the workspace)
        best = None
        for _ in range(repeats):
            ms = plan.run_timed(d_atoms, d_res)
            best = ms if best is None else tuple(min(a, b) for a, b in zip(best, ms))
        return best, plan.tile_config
    finally:
        plan.close()


def tune(desc, t0s, taus, atoms, handle, flags=_lib.TCW_FLAG_LNBTSG, budget_cells=4e9,
         repeats=2, use_cache=True, verbose=False):
    """Best tile config (dict) for this batch on ``handle``'s device."""
    import torch

    desc = np.ascontiguousarray(desc, dtype=_lib.DESC_DTYPE)
    name = _lib.device_info(handle.device)["name"]
    key = f"{name}|flags{int(flags)}|{signature(desc)}"
    path = cache_path()
    if use_cache:
        hit = _load_cache(path).get(key)
        if hit:
            return dict(hit)

    idx = sample_templates(desc, budget_cells)
    sd, st0, stau, sa = subset(desc, np.asarray(t0s, np.uint32), np.asarray(taus, np.uint32),
                               np.asarray(atoms, np.float32), idx)
    dev = torch.device("cuda", handle.device)
    d_atoms = torch.from_numpy(sa).to(dev)
    d_res = torch.zeros(sd.shape[0] * 5, dtype=torch.float64, device=dev)
    torch.cuda.synchronize(dev)
    has_rect = bool(np.any(sd["window"] == _lib.TCW_WINDOW_RECT))
    has_exp = bool(np.any(sd["window"] == _lib.TCW_WINDOW_EXP))

    best_rect, best_exp = None, None
    log = []
    if has_rect:
        for tm, tn in RECT_CANDIDATES:
            ms, _ = _time_plan(handle, sd, st0, stau, dict(rect_tm=tm, rect_tn=tn), flags,
                               d_atoms, d_res, repeats)
            log.append(("rect", tm, tn, ms[1]))
            if best_rect is None or ms[1] < best_rect[0]:
                best_rect = (ms[1], tm, tn)
    if has_exp:
        for tn, rows in EXP_CANDIDATES:
            ms, _ = _time_plan(handle, sd, st0, stau, dict(exp_tn=tn, exp_rows=rows), flags,
                               d_atoms, d_res, repeats)
            log.append(("exp", tn, rows, ms[2]))
            if best_exp is None or ms[2] < best_exp[0]:
                best_exp = (ms[2], tn, rows)
    cfg = {}
    if best_rect:
        cfg.update(rect_tm=best_rect[1], rect_tn=best_rect[2])
    if best_exp:
        cfg.update(exp_tn=best_exp[1], exp_rows=best_exp[2])
    if verbose:
        for row in log:
            print("autotune", *row)
    if use_cache:
        cache = _load_cache(path)
        cache[key] = cfg
        _store_cache(path, cache)
    return cfg
