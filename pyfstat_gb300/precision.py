"""Precision report of transient maps at scale.

For each template, the FP32 maps of the library's default path (double-word
compensated window sums, error-free FP32 D, FP64 lnBtSG), of the same with D
in native FP64 (``TCW_FLAG_FP64_DET``) and of the uncompensated FP32 variant
(``TCW_FLAG_UNCOMPENSATED``) are compared cell by cell with the full-FP64
direct-summation map of ``tcw_map_f64`` on the same device:

* every t0 row for the first ``full_templates`` templates (then max2F, the
  argmax and lnBtSG are compared too), every ``row_stride``-th row plus the
  last row and the row of the library's argmax for the others;
* cells whose FP64 condition number lies within 1e-5 (relative) of the
  reference's 1e4 threshold are excluded from the 2F error (F or the
  fallback value 2 are both legitimate there) and counted.

    python -m pyfstat_gb300.precision [--templates 64] [--full-templates 4]
        [--row-stride 16] [--json out.json] [--md out.md]

Default workload: :func:`pyfstat_gb300.synth.precision_templates` (64 x one
year of 1800 s SFTs from 2 detectors with 5 % gaps, exponential window,
8192 t0 x 4096 tau).
"""

import argparse
import json
import math
import time

import numpy as np

from . import _lib, synth
from .batched import template_grids

THRESHOLD = 1e4
BAND = 1e-5
LEVELS = (1e-7, 1e-6, 1e-5, 1e-4)
# the library's default (double-word sums, error-free FP32 D), the same with
# D in native FP64, and plain FP32 throughout
VARIANTS = (("compensated", _lib.TCW_FLAG_LNBTSG),
            ("compensated_fp64D", _lib.TCW_FLAG_LNBTSG | _lib.TCW_FLAG_FP64_DET),
            ("uncompensated", _lib.TCW_FLAG_LNBTSG | _lib.TCW_FLAG_UNCOMPENSATED))


def _variant_errors(torch, Fv, F64, band, res_v, full, rows_np, N_t0, N_tau):
    Fd = Fv.double()
    den = F64.abs().clamp_min(1e-300)
    rel = (Fd - F64).abs() / den
    rel = torch.where(band, torch.zeros_like(rel), rel)
    out = {"max_rel_2F": float(rel.max()),
           "mean_rel_2F": float(rel.mean()),
           "cells_above": {f"{lv:g}": int((rel > lv).sum()) for lv in LEVELS}}
    flat = int(torch.argmax(rel))
    r, n = divmod(flat, N_tau)
    out["worst_cell"] = {"t0_idx": int(rows_np[r]), "tau_idx": int(n), "F": float(Fd[r, n]),
                         "F64": float(F64[r, n])}
    rec = res_v.cpu().numpy().view(_lib.RESULT_DTYPE)[0]
    if full:
        f64max = float(F64.max())
        out["max2F"] = 2.0 * float(rec["maxF"])
        out["max2F_rel_err"] = abs(2.0 * float(rec["maxF"]) - 2.0 * f64max) / (2.0 * f64max)
        am = int(rec["argmax"])
        a64 = int(torch.argmax(F64))
        # an argmax is correct when it is F64's or an exact-tie-within-rounding of it
        out["argmax"] = am
        out["argmax_f64"] = a64
        out["argmax_ok"] = bool(am == a64 or
                                abs(float(F64.view(-1)[am]) - f64max) <= BAND * f64max)
        lnB64 = math.log(70.0 / (N_t0 * N_tau)) + float(torch.logsumexp(F64.view(-1), 0))
        out["lnBtSG"] = float(rec["lnBtSG"])
        out["lnBtSG_f64"] = lnB64
        out["lnBtSG_abs_err"] = abs(float(rec["lnBtSG"]) - lnB64)
    return out


def template_report(handle, t, full, row_stride, torch, dev):
    """Errors of one template's FP32 maps (all variants) against FP64."""
    t0s, taus = template_grids(t)
    N_t0, N_tau = t0s.shape[0], taus.shape[0]
    A = torch.from_numpy(np.ascontiguousarray(t["atoms"], np.float32)).to(dev)
    d_t0 = torch.from_numpy(t0s.view(np.int32)).to(dev)
    d_tau = torch.from_numpy(taus.view(np.int32)).to(dev)
    maps = {}
    t_map = {}
    for name, flags in VARIANTS:
        F = torch.empty((N_t0, N_tau), dtype=torch.float32, device=dev)
        res = torch.zeros(5, dtype=torch.float64, device=dev)
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        handle.map_plain(A, A.shape[0], t["TAtom"], t["t0_data"], t["window"], d_t0, N_t0, d_tau,
                         N_tau, F, res, flags=flags)
        torch.cuda.synchronize(dev)
        t_map[name] = time.perf_counter() - t0
        maps[name] = (F, res)
    if full:
        rows = np.arange(N_t0, dtype=np.uint32)
    else:
        am = int(maps["compensated"][1].cpu().numpy().view(_lib.RESULT_DTYPE)[0]["argmax"])
        rows = np.unique(np.concatenate([np.arange(0, N_t0, row_stride), [N_t0 - 1, am // N_tau]]))
        rows = rows.astype(np.uint32)
    F64 = torch.empty((rows.shape[0], N_tau), dtype=torch.float64, device=dev)
    cond = torch.empty_like(F64)
    t0 = time.perf_counter()
    handle.map_f64(A, A.shape[0], t["TAtom"], t["t0_data"], t["window"], d_t0, N_t0, d_tau, N_tau,
                   F64, rows=None if full else rows, d_cond=cond)
    torch.cuda.synchronize(dev)
    t_f64 = time.perf_counter() - t0
    band = (cond / THRESHOLD - 1.0).abs() < BAND
    ridx = torch.from_numpy(rows.astype(np.int64)).to(dev)
    out = {"numAtoms": int(A.shape[0]), "N_t0": N_t0, "N_tau": N_tau, "rows": int(rows.shape[0]),
           "full": bool(full), "cells_compared": int(rows.shape[0]) * N_tau,
           "cells_in_threshold_band": int(band.sum()),
           "fallback_cells_f64": int((cond >= THRESHOLD).sum()),
           "seconds": {"f64_reference": t_f64, **{f"map_{k}": v for k, v in t_map.items()}}}
    for name, (F, res) in maps.items():
        Fv = F.index_select(0, ridx)
        out[name] = _variant_errors(torch, Fv, F64, band, res, full, rows, N_t0, N_tau)
    return out


def summarise(reports):
    s = {"templates": len(reports), "cells_compared": sum(r["cells_compared"] for r in reports),
         "cells_in_threshold_band": sum(r["cells_in_threshold_band"] for r in reports)}
    for v, _ in VARIANTS:
        s[v] = {"max_rel_2F": max(r[v]["max_rel_2F"] for r in reports),
                "cells_above": {k: sum(r[v]["cells_above"][k] for r in reports)
                                for k in reports[0][v]["cells_above"]}}
        full = [r for r in reports if r["full"]]
        if full:
            s[v]["max2F_rel_err_max"] = max(r[v]["max2F_rel_err"] for r in full)
            s[v]["argmax_ok"] = sum(r[v]["argmax_ok"] for r in full)
            s[v]["lnBtSG_abs_err_max"] = max(r[v]["lnBtSG_abs_err"] for r in full)
            s[v]["full_templates"] = len(full)
    return s


def markdown(summary, reports, args):
    lines = ["# Precision at scale: exponential-window maps vs the full-FP64 GPU reference", "",
             f"Workload: {args.templates} templates, {reports[0]['numAtoms']}+ merged atoms "
             f"(one year of 1800 s SFTs, 2 detectors, 5 % gaps), {reports[0]['N_t0']} t0 x "
             f"{reports[0]['N_tau']} tau; all rows for the first {args.full_templates} templates, "
             f"every {args.row_stride}th row (plus the argmax row and the last row) for the rest.",
             "", f"Cells compared: {summary['cells_compared']:,}; cells excluded for a condition "
             f"number within {BAND:g} of the 1e4 threshold: {summary['cells_in_threshold_band']}.",
             "", "| variant | max rel err 2F | cells > 1e-7 | > 1e-6 | > 1e-5 | > 1e-4 | "
             "max2F rel err (full) | argmax ok (full) | lnBtSG abs err (full) |",
             "|---|---|---|---|---|---|---|---|---|"]
    for v, _ in VARIANTS:
        x = summary[v]
        c = x["cells_above"]
        lines.append(f"| {v} | {x['max_rel_2F']:.3e} | {c['1e-07']} | {c['1e-06']} | {c['1e-05']} "
                     f"| {c['0.0001']} | {x.get('max2F_rel_err_max', float('nan')):.3e} | "
                     f"{x.get('argmax_ok', 0)}/{x.get('full_templates', 0)} | "
                     f"{x.get('lnBtSG_abs_err_max', float('nan')):.3e} |")
    lines += ["", "Per template (max rel err of 2F per variant; map times of one template):", "",
              "| k | rows | compensated | compensated, FP64 D | uncompensated | map ms (default / "
              "FP64 D / uncomp.) | FP64 reference s |", "|---|---|---|---|---|---|---|"]
    for k, r in enumerate(reports):
        sec = r["seconds"]
        lines.append(f"| {k} | {r['rows']} | {r['compensated']['max_rel_2F']:.3e} | "
                     f"{r['compensated_fp64D']['max_rel_2F']:.3e} | "
                     f"{r['uncompensated']['max_rel_2F']:.3e} | "
                     f"{1e3 * sec['map_compensated']:.1f} / {1e3 * sec['map_compensated_fp64D']:.1f}"
                     f" / {1e3 * sec['map_uncompensated']:.1f} | {sec['f64_reference']:.2f} |")
    return "\n".join(lines) + "\n"


def main(argv=None):
    import torch

    p = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    p.add_argument("--templates", type=int, default=64)
    p.add_argument("--full-templates", type=int, default=4)
    p.add_argument("--row-stride", type=int, default=16)
    p.add_argument("--seed", type=int, default=777)
    p.add_argument("--device", type=int, default=0)
    p.add_argument("--json", default="")
    p.add_argument("--md", default="")
    args = p.parse_args(argv)
    dev = torch.device("cuda", args.device)
    torch.cuda.set_device(dev)
    handle = _lib.Handle(args.device)
    # run on torch's stream so that torch reads the results in order
    handle.set_stream(torch.cuda.current_stream(dev).cuda_stream or 0x1)
    reports = []
    for k, t in enumerate(synth.precision_templates(args.templates, seed=args.seed)):
        r = template_report(handle, t, k < args.full_templates, args.row_stride, torch, dev)
        reports.append(r)
        print(f"template {k}: rows {r['rows']} " + " ".join(
            f"{v} {r[v]['max_rel_2F']:.3e}" for v, _ in VARIANTS) +
              f" (FP64 reference {r['seconds']['f64_reference']:.2f} s)", flush=True)
    summary = summarise(reports)
    print(json.dumps(summary))
    if args.json:
        with open(args.json, "w") as f:
            json.dump({"summary": summary, "templates": reports, "args": vars(args)}, f, indent=1)
    if args.md:
        with open(args.md, "w") as f:
            f.write(markdown(summary, reports, args))
    handle.close()
    return summary


if __name__ == "__main__":
    main()
