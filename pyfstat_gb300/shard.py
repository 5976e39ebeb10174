"""Sharding transient-map work across processes (one GPU per process).

Every template, and every block of t0 rows inside a template, is
independent, so the work partitions with no exchange on the data path:

* :func:`partition` assigns whole templates to ranks by estimated cost
  (longest-processing-time greedy, deterministic);
* :func:`split_rows` cuts one large template into row blocks that run as
  templates of their own, and :func:`merge_split` combines their results
  exactly: max/argmax as a max over (maxF, -flat index) pairs (the first
  occurrence in row-major order wins, as numpy's argmax), lnBtSG as an FP64
  log-sum-exp merge of the blocks' (log-sum-exp) partials;
* :func:`gather_results` collects the per-template 40-byte result records on
  rank 0 over a ``torch.distributed`` process group (a host-side gather of
  scalars; gloo or NCCL);
* :func:`run_sharded` ties them together around a compute function (by
  default the batched GPU path on this rank's device).

Posterior indices (t0_MP, tau_MP) need whole-map row and column sums; for a
template split by rows they are not merged and come back as -1.
"""

import math

import numpy as np

from . import _lib


def template_cost(t):
    """Relative cost estimate of a template: its cells, times the mean window
    length in atoms for exponential windows (a window of 3 tau, capped by the
    data), which sets the per-cell work of the recurrences' tails."""
    N_t0, N_tau = int(t["N_t0"]), int(t["N_tau"])
    cells = float(N_t0) * float(N_tau)
    if int(t["window"]) != _lib.TCW_WINDOW_EXP:
        return cells
    na = float(np.asarray(t["atoms"]).shape[0]) if "atoms" in t else float(t["numAtoms"])
    if "taus" in t:
        mean_tau = float(np.mean(np.asarray(t["taus"], dtype=np.float64)))
    else:
        mean_tau = float(t["tau"]) + 0.5 * float(t["dtau"]) * (N_tau - 1)
    span = min(na, 3.0 * mean_tau / float(t["TAtom"]))
    return cells * (1.0 + span / 256.0)


def partition(costs, world_size):
    """Template indices per rank, balancing the summed costs (LPT greedy:
    largest first onto the least-loaded rank; ties to the lower rank).
    Each rank's indices come back sorted."""
    costs = np.asarray(costs, dtype=np.float64)
    if world_size < 1:
        raise ValueError("world_size must be >= 1")
    order = np.lexsort((np.arange(costs.size), -costs))
    load = np.zeros(world_size)
    owner = np.empty(costs.size, dtype=np.int64)
    for i in order:
        r = int(np.argmin(load))
        owner[i] = r
        load[r] += costs[i]
    return [np.flatnonzero(owner == r) for r in range(world_size)]


def split_rows(t, n_blocks):
    """Cut template ``t`` (explicit or uniform grid) into up to ``n_blocks``
    templates over consecutive blocks of t0 rows.  Returns the list of
    (row_offset, template) pairs."""
    from .batched import template_grids

    t0s, taus = template_grids(t)
    N_t0 = t0s.shape[0]
    n_blocks = max(1, min(int(n_blocks), N_t0))
    edges = np.linspace(0, N_t0, n_blocks + 1).round().astype(np.int64)
    out = []
    for b in range(n_blocks):
        lo, hi = int(edges[b]), int(edges[b + 1])
        if hi <= lo:
            continue
        part = {k: v for k, v in t.items() if k not in ("t0", "dt0", "N_t0", "tau", "dtau",
                                                       "N_tau", "t0s", "taus")}
        part.update(t0s=t0s[lo:hi].copy(), taus=taus.copy(), N_t0=hi - lo, N_tau=taus.shape[0])
        out.append((lo, part))
    return out


def lse_partial(result, N_t0, N_tau):
    """The log-sum-exp of F over a (sub)map, from its lnBtSG
    (lnBtSG = ln(70 / (N_t0 N_tau)) + logsumexp F)."""
    return float(result["lnBtSG"]) - math.log(70.0 / (float(N_t0) * float(N_tau)))


def merge_split(parts, N_t0, N_tau):
    """Merge results of row blocks of one template.

    ``parts``: list of (row_offset, n_rows, result record) for blocks that
    cover the rows [0, N_t0) once.  Returns one result record of the whole
    template (posterior indices -1)."""
    best = None
    lses = []
    for off, n_rows, r in parts:
        flat = int(r["argmax"])
        gflat = (flat // N_tau + int(off)) * N_tau + flat % N_tau
        key = (float(r["maxF"]), -gflat)
        if best is None or key > best:
            best = key
        lses.append(lse_partial(r, n_rows, N_tau))
    m = max(lses)
    lse = m + math.log(sum(math.exp(x - m) for x in lses))
    out = np.zeros(1, dtype=_lib.RESULT_DTYPE)[0]
    out["maxF"] = best[0]
    out["argmax"] = -best[1]
    out["lnBtSG"] = math.log(70.0 / (float(N_t0) * float(N_tau))) + lse
    out["t0_mp_idx"] = -1
    out["tau_mp_idx"] = -1
    out["status"] = max(int(r["status"]) for _, _, r in parts)
    return out


def gather_results(local_idx, local_res, n_templates, group=None):
    """All ranks' (indices, result records) into one array of ``n_templates``
    records on rank 0 (None on the other ranks).  Collective over ``group``."""
    import torch
    import torch.distributed as dist

    ws = dist.get_world_size(group)
    rank = dist.get_rank(group)
    idx = np.asarray(local_idx, dtype=np.int64)
    res = np.ascontiguousarray(local_res, dtype=_lib.RESULT_DTYPE)
    # fixed-size exchange: counts first, then padded index and record buffers
    backend = dist.get_backend(group)
    dev = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else None
    cnt = torch.tensor([idx.size], dtype=torch.int64, device=dev)
    counts = [torch.zeros(1, dtype=torch.int64, device=dev) for _ in range(ws)]
    dist.all_gather(counts, cnt, group=group)
    cap = max(int(c.item()) for c in counts)
    ib = torch.full((cap,), -1, dtype=torch.int64)
    ib[:idx.size] = torch.from_numpy(idx)
    rb = torch.zeros((cap, _lib.RESULT_DTYPE.itemsize), dtype=torch.uint8)
    rb[:idx.size] = torch.from_numpy(res.view(np.uint8).reshape(idx.size,
                                                                 _lib.RESULT_DTYPE.itemsize))
    if dev is not None:
        ib, rb = ib.to(dev), rb.to(dev)
    ibs = [torch.empty_like(ib) for _ in range(ws)]
    rbs = [torch.empty_like(rb) for _ in range(ws)]
    dist.all_gather(ibs, ib, group=group)
    dist.all_gather(rbs, rb, group=group)
    if rank != 0:
        return None
    out = np.zeros(n_templates, dtype=_lib.RESULT_DTYPE)
    seen = np.zeros(n_templates, dtype=bool)
    for r in range(ws):
        n = int(counts[r].item())
        ii = ibs[r][:n].cpu().numpy()
        rr = np.ascontiguousarray(rbs[r][:n].cpu().numpy()).view(_lib.RESULT_DTYPE).reshape(-1)
        if np.any(seen[ii]):
            raise RuntimeError("a template was computed by more than one rank")
        out[ii] = rr
        seen[ii] = True
    if not np.all(seen):
        raise RuntimeError(f"{int((~seen).sum())} templates were not computed by any rank")
    return out


def gpu_compute(templates, device=None):
    """Batched GPU results of ``templates`` on this process's device."""
    from .batched import TransientMapBatch

    if not templates:
        return np.zeros(0, dtype=_lib.RESULT_DTYPE)
    import torch

    dev = torch.cuda.current_device() if device is None else device
    batch = TransientMapBatch(templates, device=dev)
    try:
        return batch.run()
    finally:
        batch.close()


def run_sharded(templates, compute=None, group=None):
    """Compute all templates across the ranks of ``group`` (this rank's share
    by :func:`partition`), gather the records on rank 0 in template order.
    ``compute(list_of_templates) -> records`` defaults to :func:`gpu_compute`."""
    import torch.distributed as dist

    compute = compute or gpu_compute
    ws = dist.get_world_size(group)
    rank = dist.get_rank(group)
    shares = partition([template_cost(t) for t in templates], ws)
    mine = shares[rank]
    res = compute([templates[i] for i in mine])
    return gather_results(mine, res, len(templates), group=group)
