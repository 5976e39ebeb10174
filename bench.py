"""Benchmark: batched transient-CW F-statistic maps on GB300.

Workload (N=1): 4096 templates, SFT counts uniform in 200..4000 with 0-30 %
of SFTs dropped as gaps, half rectangular and half exponential windows,
(t0, tau) grid sizes uniform in 256..2048 per axis -- about 5.4e9 cells per
step -- synthetic seeded atoms (pyfstat_gb300.synth).  A step is one pass of
the batched fused path over all templates (one CUDA graph of five launches:
repack -> persistent exp map kernel on one branch, prefix -> persistent rect
map kernel on the other, then finalize), giving max2F, argmax and FP64
lnBtSG per template.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line.  Under torchrun each rank runs its own 4096 templates
(weak scaling, no collective on the data path); rank 0 prints.
"""

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = ("2F-map cells/s, batched+fused vs plain per-template kernel, "
          "2F rel err ≤1e-5")
UNIT = "cells/s"
# ncu summaries of the map kernels on this workload; each holds a line
# "traffic_bytes_per_launch = N" (DRAM read + write bytes of one launch)
TRAFFIC_FILES = {"rect_map_kernel": os.path.join(REPO, "profiles", "rect_map_kernel_batched.md"),
                 "exp_map_kernel": os.path.join(REPO, "profiles", "exp_map_kernel_batched.md")}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--templates", type=int, default=4096)
    p.add_argument("--seed", type=int, default=12345)
    p.add_argument("--cpu-seconds", type=float, default=12.0,
                   help="target CPU time of the bounded CPU-baseline sample")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-grad", action="store_true",
                   help="skip the differentiation workload (forward/backward timing)")
    p.add_argument("--plain-templates", type=int, default=256,
                   help="templates timed with the plain per-template kernel")
    p.add_argument("--window", choices=["both", "rect", "exp"], default="both",
                   help="restrict the workload to one window type (breakdown runs)")
    p.add_argument("--case", choices=["plain-rect", "plain-exp", "single-480", "grad"],
                   default=None,
                   help="instead of the benchmark: time one single-template map with the map "
                        "written (8192 t0 x 4096 tau over one year of two-detector data; the "
                        "134 MB map exceeds L2), for the memory-side profile of the plain kernel; "
                        "single-480: the 480 x 480 rect and 480 x 512 log-tau exp single-template "
                        "maps on device buffers (--steps calls each); grad: the differentiation "
                        "workload alone (the first --templates of its 256 templates, --steps "
                        "repetitions)")
    p.add_argument("--tile", type=str, default="auto",
                   help="tile config as JSON, 'auto' for the autotuner (default), "
                        "'default' for the library defaults")
    return p.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def workload(n_templates, seed):
    from pyfstat_gb300 import synth

    return synth.batched_templates(n_templates, seed=seed)


# ------------------------------------------------------------------ clocks


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during a region."""

    FIELDS = ("uuid,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, uuid=None):
        self.uuid = uuid
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=2)
        rows = []
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) != 9:
                continue
            if self.uuid and parts[0] != self.uuid:
                continue
            rows.append(parts)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows)}


def gpu_uuid(torch, dev):
    try:
        u = str(torch.cuda.get_device_properties(dev).uuid)
        return u if u.startswith("GPU-") else "GPU-" + u
    except Exception:
        return None


# ------------------------------------------------------------------ CPU baseline


def template_cost(t):
    """CPU cost model of one template on the reference's path: rectangular
    maps cost O(1) per cell (plus the running sums along tau); exponential
    maps sum every atom of each cell's window (up to 3 tau / TAtom atoms)."""
    from pyfstat_gb300.batched import template_grids

    t0s, taus = template_grids(t)
    cells = float(len(t0s)) * len(taus)
    if t["window"] == 1:
        return cells
    win = np.minimum(3.0 * taus.astype(np.float64) / t["TAtom"], t["atoms"].shape[0])
    return float(len(t0s)) * float(np.sum(np.maximum(win, 1.0)))


def cpu_baseline(templates, seconds, threads, seed=2024):
    """The reference's per-template CPU path restated in C (oracle port: the
    pycuda kernels' FP32 arithmetic, OpenMP over rows/cells) plus its numpy
    max/argmax/lnBtSG, timed on a stratified random sample of the workload:
    rectangular and exponential templates drawn alternately (seeded) until
    ~`seconds` of CPU time.  The whole workload's time is estimated per window
    type by a ratio estimator on the cost model (template_cost): sampled
    seconds x (the window type's total cost / the sample's cost).  Returns
    (cells/s of the whole workload, details)."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle as O
    from pyfstat_gb300.batched import template_grids

    O.build()
    rng = np.random.default_rng(seed)
    groups = {w: [k for k, t in enumerate(templates) if t["window"] == w] for w in (1, 2)}
    order = {w: list(rng.permutation(ix)) for w, ix in groups.items() if ix}
    cost = {w: {k: template_cost(templates[k]) for k in ix} for w, ix in groups.items()}
    spent = {w: 0.0 for w in order}
    scost = {w: 0.0 for w in order}
    scells = {w: 0 for w in order}
    used = {w: 0 for w in order}
    t_start = time.perf_counter()
    while any(order.values()):
        for w in list(order):
            if not order[w]:
                continue
            k = order[w].pop()
            t = templates[k]
            t0s, taus = template_grids(t)
            fn = O.rect_map_f32 if w == 1 else O.exp_map_f32
            a = time.perf_counter()
            F = fn(t["atoms"], t["TAtom"], t["t0_data"], t0s, taus, nthreads=threads)
            O.max_argmax(F)
            O.lnBtSG(F)
            spent[w] += time.perf_counter() - a
            scost[w] += cost[w][k]
            scells[w] += F.size
            used[w] += 1
        if time.perf_counter() - t_start > seconds and all(used[w] >= 2 for w in order):
            break
    total_cells = sum(float(t["N_t0"]) * t["N_tau"] if "N_t0" in t else
                      float(len(template_grids(t)[0])) * len(template_grids(t)[1])
                      for t in templates)
    est = {w: spent[w] * sum(cost[w].values()) / scost[w] for w in order}
    value = total_cells / sum(est.values())
    names = {1: "rect", 2: "exp"}
    detail = {
        "sample": (f"stratified seeded sample: {used.get(1, 0)} rect + {used.get(2, 0)} exp "
                   f"templates ({sum(scells.values())} cells, {sum(spent.values()):.1f} s); "
                   "whole-workload time per window type = sampled time x total cost / sampled "
                   "cost (cost: cells for rect, cells x window length for exp)"),
        "per_window_cells_per_s": {names[w]: scells[w] / spent[w] for w in order},
        "estimated_workload_s": {names[w]: est[w] for w in order},
        "templates_sampled": {names[w]: used[w] for w in order},
    }
    return value, detail


def dropin_per_call(h, reps=20):
    """Median wall time (ms) of one drop-in call, host arrays in and out: the
    480 x 480 rectangular single-template map through the PyFstat-facing
    dispatcher (windowRange, BtSG), and the 480 t0 x 512 log-spaced tau
    exponential map through the C-ABI host entry (tcw_map_plain_host)."""
    from pyfstat_gb300 import _lib, synth
    from pyfstat_gb300 import tcw_fstat_map_funcs as tcw
    from pyfstat_gb300.window import transientWindowRange_t

    def median_ms(fn):
        for _ in range(3):
            fn()
        ts = []
        for _ in range(reps):
            t0 = time.perf_counter()
            fn()
            ts.append(time.perf_counter() - t0)
        return 1e3 * statistics.median(ts)

    features, ctx = tcw.init_transient_fstat_map_features("b200")
    multi = synth.multi_detector_atoms(0, 480, 1)
    wr = dict(type=1, t0=700000000, t0Band=479 * 1800, dt0=1800, tau=1800, tauBand=479 * 1800,
              dtau=1800)
    rect_ms = median_ms(lambda: tcw.call_compute_transient_fstat_map(
        "b200", features, multi, transientWindowRange_t(**wr), BtSG=True))
    ctx.detach()
    c = synth.plain_exp_case()
    flags = _lib.TCW_FLAG_LNBTSG | _lib.TCW_FLAG_POSTERIORS
    exp_ms = median_ms(lambda: h.map_plain_host(c["atoms"], c["TAtom"], c["t0_data"], 2,
                                                c["t0s"], c["taus"], want_map=True, flags=flags))
    return {"rect_480x480_dispatcher_ms": rect_ms, "exp_480x512log_c_abi_ms": exp_ms,
            "note": "median of 20 calls, full F map and result back on the host"}


def plain_configs(h, dev, torch, stream, hbm, reps=200):
    """The single-template workloads on device buffers (map written, lnBtSG
    and posteriors), timed with CUDA events over ``reps`` calls: the 480 x 480
    rectangular map of one 480-SFT detector and the 480 t0 x 512 log-spaced
    tau exponential map of two merged detectors.  HBM figures use the
    algorithmic bytes: 28 B per atom read + 4 B per map cell written."""
    from pyfstat_gb300 import _lib, synth

    out = {}
    for name, c in (("rect_480x480", synth.plain_rect_case()),
                    ("exp_480x512log", synth.plain_exp_case())):
        A = torch.from_numpy(c["atoms"]).to(dev)
        t0s = torch.from_numpy(c["t0s"].view(np.int32)).to(dev)
        taus = torch.from_numpy(c["taus"].view(np.int32)).to(dev)
        N_t0, N_tau = len(c["t0s"]), len(c["taus"])
        F = torch.empty((N_t0, N_tau), dtype=torch.float32, device=dev)
        r = torch.zeros(5, dtype=torch.float64, device=dev)
        flags = _lib.TCW_FLAG_LNBTSG | _lib.TCW_FLAG_POSTERIORS

        def call():
            h.map_plain(A, A.shape[0], c["TAtom"], c["t0_data"], c["window"], t0s, N_t0, taus,
                        N_tau, F, r, flags=flags)

        for _ in range(min(10, reps)):
            call()
        torch.cuda.synchronize(dev)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            call()
        e1.record(stream)
        torch.cuda.synchronize(dev)
        ms = e0.elapsed_time(e1) / reps
        cells = N_t0 * N_tau
        nbytes = 28.0 * A.shape[0] + 4.0 * cells
        gbs = nbytes / (ms * 1e-3) / 1e9
        out[name] = {"ms_per_call": ms, "cells_per_s": cells / (ms * 1e-3),
                     "algorithmic_bytes": nbytes, "hbm_gbs": gbs,
                     "frac_of_hbm": gbs / hbm if hbm else None,
                     "note": "device buffers, map written, lnBtSG and posteriors; all "
                             "launches of one call (map, finalize, posteriors) in the time"}
    return out


# Algorithmic FP64 work per cell of the differentiable statistics: the
# forward pass is the map's per-cell math (55 flops with an FMA as 2) in
# FP64; the backward pass recomputes the window sums and runs their adjoint
# (twice the forward).
GRAD_FP64_FLOPS = {"forward": 55.0, "backward": 110.0}


def grad_case(torch, dev, peaks, reps=3, n_templates=256):
    """Differentiation workload: 256 templates x 2000 SFTs x 2 detectors,
    exponential windows, 1024 t0 x 1024 tau; forward (lnBtSG and soft-max 2F)
    and backward (gradients of both w.r.t. atoms and tau), CUDA events."""
    from pyfstat_gb300 import synth
    from pyfstat_gb300.autograd import DiffBatch

    tl = []
    for k in range(n_templates):
        t0_data, A = synth.merged_atoms(5000 + k, 2000, 2)
        tl.append(dict(atoms=A, TAtom=1800, t0_data=t0_data, t0=t0_data + 450, dt0=3600,
                       N_t0=1024, N_tau=1024, tau_min=30075.0,
                       tau_max=30075.0 + 1200.0 * 1023))
    b = DiffBatch(tl, device=dev.index, temperature=0.1)
    atoms = torch.from_numpy(b.atoms).to(dev)
    tmin = np.array([t["tau_min"] for t in tl])
    tmax = np.array([t["tau_max"] for t in tl])
    one = torch.ones(n_templates, dtype=torch.float64, device=dev)
    lnB, soft = b.forward_raw(atoms, tmin, tmax)
    b.backward_raw(atoms, tmin, tmax, lnB, soft, one, one)
    torch.cuda.synchronize(dev)
    s = torch.cuda.current_stream(dev)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    fwd, bwd = [], []
    for _ in range(reps):
        ev[0].record(s)
        lnB, soft = b.forward_raw(atoms, tmin, tmax)
        ev[1].record(s)
        b.backward_raw(atoms, tmin, tmax, lnB, soft, one, one)
        ev[2].record(s)
        torch.cuda.synchronize(dev)
        fwd.append(ev[0].elapsed_time(ev[1]))
        bwd.append(ev[1].elapsed_time(ev[2]))
    cells = n_templates * 1024 * 1024
    out = {"workload": f"{n_templates} templates x 2000 SFTs x 2 detectors (exp), 1024 t0 x "
                       "1024 tau "
                       "(tau from 30075 s in steps of 1200 s), temperature 0.1",
           "cells": cells}
    for name, ms in (("forward", statistics.median(fwd)), ("backward", statistics.median(bwd))):
        cps = cells / (ms * 1e-3)
        ach = cps * GRAD_FP64_FLOPS[name] / 1e12
        out[name] = {"ms": ms, "cells_per_s": cps,
                     "roofline": {"bound": "fp64", "achieved": ach,
                                  "peak": peaks["fp64_tflops"], "unit": "TFLOP/s",
                                  "frac": ach / peaks["fp64_tflops"],
                                  "fp64_flops_per_cell": GRAD_FP64_FLOPS[name]}}
    return out


def cpu_per_call(threads, reps=3):
    """The same two single-template maps with the oracle port (the reference
    kernels' FP32 arithmetic) plus its numpy lnBtSG / posteriors, best of 3."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle as O
    from pyfstat_gb300 import synth

    O.build()
    out = {}
    for name, c, fn in (("rect_480x480_ms", synth.plain_rect_case(), O.rect_map_f32),
                        ("exp_480x512log_ms", synth.plain_exp_case(), O.exp_map_f32)):
        best = None
        for _ in range(reps):
            t0 = time.perf_counter()
            F = fn(c["atoms"], c["TAtom"], c["t0_data"], c["t0s"], c["taus"], nthreads=threads)
            O.max_argmax(F)
            O.lnBtSG(F)
            O.t0_max_posterior_idx(F)
            dt = 1e3 * (time.perf_counter() - t0)
            best = dt if best is None else min(best, dt)
        out[name] = best
    return out


def cpu_model():
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith(("model name", "cpu part")):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform

    return platform.processor() or platform.machine()


# Sources whose compiled code the map-kernel profiles describe; each committed
# summary records their hash ("kernel_source_sha16 = ...") at capture time.
KERNEL_SOURCES = ("tcw_kernels.cu", "tcw_cell.h", "tcw_internal.h")


def kernel_source_hash():
    """First 16 hex digits of the SHA-256 of the map kernels' sources."""
    import hashlib

    h = hashlib.sha256()
    for name in KERNEL_SOURCES:
        with open(os.path.join(REPO, "pyfstat_gb300", "csrc", name), "rb") as f:
            h.update(name.encode() + b"\0" + f.read())
    return h.hexdigest()[:16]


def profile_text(kernel):
    try:
        with open(TRAFFIC_FILES[kernel]) as f:
            return f.read()
    except (OSError, KeyError):
        return ""


def profile_is_current(kernel):
    """True when the kernel's committed ncu summary was captured from the
    sources built now (its recorded source hash equals the current one)."""
    for line in profile_text(kernel).splitlines():
        if line.strip().startswith("kernel_source_sha16"):
            return line.split("=")[1].strip() == kernel_source_hash()
    return False


def traffic_per_launch(kernel):
    """DRAM bytes per launch of a map kernel from its committed ncu summary,
    or None when there is none or it was captured from other sources."""
    if not profile_is_current(kernel):
        return None
    return profile_figure(kernel, "traffic_bytes_per_launch")


def launches_per_step(n_rect, n_exp):
    """Kernels one plan step launches: prefix (rect templates), repack and
    map (exp templates), map (rect templates), finalize."""
    return (2 if n_rect else 0) + (2 if n_exp else 0) + 1


# Algorithmic per-cell demand of the fused batched map (the reference's
# per-cell math; compensation not counted): FP32 flops (an FMA counts 2),
# MUFU ops (sqrt, rcp, ex2) and FP64 operations: D = AB - C^2 as two
# (a multiply and a fused multiply-add) plus the lnBtSG accumulation as one
# -- 3 operations per cell, the count the scope table fixes.  The measured
# FP64 peak counts an FMA as 2 flops, so in consistent flop units the FP64
# demand is 4 (mul 1 + fma 2 + add 1); the bench line states the fraction
# both ways ("frac" with 3, "frac_fp64_flops" with 4).
DEMAND = {1: {"fp32": 34.0, "mufu": 3.0, "fp64": 3.0},
          2: {"fp32": 55.0, "mufu": 3.0, "fp64": 3.0}}
FP64_FLOPS_PER_CELL = 4.0
KERNEL_WINDOW = {"rect_map_kernel": 1, "exp_map_kernel": 2}


def profile_figure(kernel, key):
    """A "key = value" figure from the kernel's committed ncu summary."""
    for line in profile_text(kernel).splitlines():
        if line.strip().startswith(key):
            try:
                return float(line.split("=")[1].split()[0])
            except (ValueError, IndexError):
                return None
    return None


def rect_reused_fraction(desc, t0s, taus, n_sample=64, seed=99):
    """Fraction of the rect cells whose window end equals the previous
    column's in the row (the rect map kernel reuses their F instead of
    evaluating it), on a seeded sample of the batch's rect templates; the
    end index is the kernel's (rect_end: the reference's u32 arithmetic,
    clamps, and the running maximum of wrapped rows)."""
    idx = np.flatnonzero(desc["window"] == 1)
    if idx.size == 0:
        return None
    idx = np.random.default_rng(seed).permutation(idx)[:n_sample]
    same = total = 0
    for k in idx:
        d = desc[k]
        T, t0d, N = int(d["TAtom"]), int(d["t0_data"]), int(d["numAtoms"])
        g0 = t0s[int(d["t0_offset"]):int(d["t0_offset"]) + int(d["N_t0"])].astype(np.uint64)
        tu = taus[int(d["tau_offset"]):int(d["tau_offset"]) + int(d["N_tau"])].astype(np.uint64)
        m32 = np.uint64(0xFFFFFFFF)

        def end(t1):
            q = (((t1 - np.uint64(t0d) + np.uint64(T // 2)) & m32) // np.uint64(T) - 1) & m32
            i = q.astype(np.int64)
            i = np.where(i >= 2 ** 31, i - 2 ** 32, i)  # the cast to int
            return np.clip(i, 0, N - 1)

        e = end((g0[:, None] + tu[None, :]) & m32)
        wr = g0 + tu[0] + np.uint64(T // 2) < np.uint64(t0d)
        e = np.where(wr[:, None], np.maximum(e, end((g0 + tu[0]) & m32)[:, None]), e)
        same += int(np.sum(e[:, 1:] == e[:, :-1]))
        total += e.size
    return same / total


def roofline_block(batch, rect_ms, exp_ms, prefix_ms, fin_ms, peaks, clk, n_sms):
    """Roofline of the dominant map kernel: cells/s against the minimum over
    {FP32, MUFU, FP64, HBM} of measured peak / per-cell algorithmic demand,
    stated in the binding unit (algorithmic TFLOP/s or GB/s per second of
    kernel time against that unit's measured peak; the fraction is the same
    in cells/s); with the FP32-flop view and the instruction-issue view of
    the same kernel."""
    hbm = None
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            hbm = json.load(f).get("hbm_gbs")
    except (OSError, ValueError):
        pass
    desc = batch.desc
    kernels = {}
    for name, w in KERNEL_WINDOW.items():
        sel = desc["window"] == w
        cells = float(np.sum(desc["N_t0"][sel].astype(np.float64) * desc["N_tau"][sel]))
        ms = rect_ms if w == 1 else exp_ms
        if cells == 0 or ms <= 0:
            continue
        # bytes read per launch: the template's atoms once (28 B per atom) + results
        nbytes = 28.0 * float(np.sum(desc["numAtoms"][sel])) + 40.0 * float(np.sum(sel))
        d = DEMAND[w]
        bounds = {"fp32": peaks["fp32_tflops"] * 1e12 / d["fp32"],
                  "mufu": peaks["mufu_tops"] * 1e12 / d["mufu"],
                  "fp64": peaks["fp64_tflops"] * 1e12 / d["fp64"]}
        if hbm:
            bounds["hbm"] = hbm * 1e9 / (nbytes / cells)
        bound = min(bounds, key=bounds.get)
        cps = cells / (ms * 1e-3)
        # the binding unit's algorithmic work per second against its peak
        if bound == "hbm":
            unit, ach, pk = "GB/s", cps * (nbytes / cells) / 1e9, hbm
        elif bound == "mufu":
            unit, ach, pk = "Tops/s", cps * d["mufu"] / 1e12, peaks["mufu_tops"]
        else:
            unit, ach, pk = "TFLOP/s", cps * d[bound] / 1e12, peaks[f"{bound}_tflops"]
        k = {"ms": ms, "cells": cells, "cells_per_s": cps, "bound": bound,
             "bound_unit": unit, "achieved": ach, "peak": pk,
             "roofline_cells_per_s": bounds[bound], "frac": cps / bounds[bound],
             "unit_bounds_cells_per_s": bounds, "algorithmic_per_cell": d,
             "algorithmic_bytes_per_launch": nbytes,
             "fp32_view": {"achieved_tflops": cps * d["fp32"] / 1e12,
                           "peak_tflops": peaks["fp32_tflops"],
                           "frac": cps * d["fp32"] / 1e12 / peaks["fp32_tflops"]}}
        if bound == "fp64":
            k["unit_note"] = ("achieved = 3 FP64 operations per cell (scope-table count: D as "
                              "mul + fma, lnBtSG as add) x cells/s; peak = measured FP64 FMA "
                              "rate with an FMA counted as 2 flops")
            k["frac_fp64_flops"] = cps * FP64_FLOPS_PER_CELL / (peaks["fp64_tflops"] * 1e12)
        if w == 1:
            reused = rect_reused_fraction(desc, batch.t0s, batch.taus)
            if reused is not None:
                k["cells_reusing_F"] = reused
                k["reuse_note"] = ("a cell whose window end equals its left neighbour's has "
                                   "that cell's window and F, which the kernel reuses; the "
                                   "per-cell FP64 count assumes every cell forms D, so frac "
                                   "can exceed 1 (sampled on 64 rect templates)")
        current = profile_is_current(name)
        k["profile_source_current"] = current
        ipc = profile_figure(name, "warp_instructions_per_cell")
        if ipc and clk and clk.get("sm_mhz"):
            issue = 4.0 * n_sms * clk["sm_mhz"] * 1e6 / ipc
            k["issue_view"] = {"warp_instructions_per_cell": ipc,
                               "issue_bound_cells_per_s": issue, "frac": cps / issue,
                               "stale": not current}
        kernels[name] = k
    dom = max(kernels, key=lambda n: kernels[n]["ms"])
    d = kernels[dom]
    return {"bound": d["bound"], "achieved": d["achieved"], "peak": d["peak"],
            "unit": d["bound_unit"], "frac": d["frac"], "traffic": traffic_per_launch(dom),
            "kernel_source_sha16": kernel_source_hash(),
            "achieved_cells_per_s": d["cells_per_s"], "roofline_cells_per_s": d["roofline_cells_per_s"],
            "kernel": dom, "kernels": kernels, "prefix_ms": prefix_ms, "finalize_ms": fin_ms,
            "peak_source": "FP32/FP64/MUFU of measured (tcw_probe_peaks on this GPU), HBM of "
                           "measured (MEASURED_PEAKS.json)",
            "measured_peaks": dict(peaks, hbm_gbs=hbm)}


# ------------------------------------------------------------------ arms


def run_reference(args, ws, rank):
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    templates = workload(args.templates, args.seed)
    for w in range(args.warmup):
        cpu_baseline(templates, min(2.0, args.cpu_seconds), threads, seed=1000 + w)
    vals, details = [], []
    t_all = time.perf_counter()
    for k in range(args.steps):
        v, d = cpu_baseline(templates, args.cpu_seconds, threads, seed=2024 + k)
        vals.append(v)
        details.append(d)
    elapsed = time.perf_counter() - t_all
    value = float(statistics.median(vals))
    d = details[-1]
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * elapsed / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"batched {args.templates} templates, rect+exp, "
                   "SFTs 200-4000, 0-30% gaps, grids 256-2048^2",
                   "sample": "each step: a different seeded stratified sample of the same "
                             "workload, its time extrapolated to all templates"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": d["sample"],
                         "per_window_cells_per_s": d["per_window_cells_per_s"],
                         "estimated_workload_s": d["estimated_workload_s"],
                         "step_values": vals},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args, ws, rank, local):
    import torch

    from pyfstat_gb300 import _lib
    from pyfstat_gb300.batched import TransientMapBatch, template_grids

    if ws > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local if ws > 1 else 0)
    torch.cuda.set_device(dev)

    templates = workload(args.templates, args.seed + 1000003 * rank)
    if args.window != "both":
        keep = 1 if args.window == "rect" else 2
        templates = [t for t in templates if t["window"] == keep]
    tile = None
    if args.tile == "auto":
        tile = "auto"
    elif args.tile and args.tile != "default":
        tile = json.loads(args.tile)
    batch = TransientMapBatch(templates, device=dev.index, tile_config=tile)
    h = batch.handle
    # a side stream: graphs cannot be captured on the legacy default stream
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(stream)
    h.set_stream(stream.cuda_stream)
    n_cells = batch.n_cells
    n_t = batch.n_templates
    d_atoms = torch.from_numpy(batch.atoms).to(dev)
    d_res = torch.zeros(n_t * 5, dtype=torch.float64, device=dev)

    def barrier():
        torch.cuda.synchronize(dev)
        if ws > 1:
            torch.distributed.barrier()

    for _ in range(max(3, args.warmup)):
        batch.run_device(d_atoms, d_res, use_graph=True)
    barrier()
    clocks = ClockSampler(gpu_uuid(torch, dev))
    clocks.start()
    time.sleep(0.3)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    barrier()
    e0.record(stream)
    for _ in range(args.steps):
        batch.run_device(d_atoms, d_res, use_graph=True)
    e1.record(stream)
    barrier()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1) / args.steps
    if ws > 1:
        t = torch.tensor([ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    # whole-job cells and copied bytes: ranks hold different (seeded) template sets
    total_cells, total_in, total_out = n_cells, batch.atoms.nbytes, 40 * n_t
    if ws > 1:
        t = torch.tensor([float(n_cells), float(total_in), float(total_out)],
                         dtype=torch.float64, device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.SUM)
        total_cells, total_in, total_out = (float(v) for v in t.tolist())
    value = total_cells / (ms * 1e-3)
    res = d_res.cpu().numpy().view(_lib.RESULT_DTYPE)
    assert np.all(np.isfinite(res["lnBtSG"])) and np.all(res["maxF"] > 0)

    # per-kernel durations (events between the launches, same stream)
    kms = np.array([batch.plan.run_timed(d_atoms, d_res) for _ in range(args.steps)])
    prefix_ms, rect_ms, exp_ms, fin_ms = (float(x) for x in kms.mean(axis=0))

    # end to end through the public API with pinned host buffers
    pinned = torch.empty(batch.atoms.shape, dtype=torch.float32, pin_memory=True)
    pinned.numpy()[:] = batch.atoms
    host_atoms = pinned.numpy()
    batch.run_pipelined([host_atoms] * args.warmup)
    barrier()
    t0 = time.perf_counter()
    out = batch.run_pipelined([host_atoms] * args.steps)[-1]
    e2e_s = (time.perf_counter() - t0) / args.steps
    # the same, one blocking call per step (upload, run, download, wait)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        out_serial = batch.run(host_atoms)
    e2e_serial_s = (time.perf_counter() - t0) / args.steps
    assert np.array_equal(out_serial["argmax"], res["argmax"])
    if ws > 1:
        t = torch.tensor([e2e_s, e2e_serial_s], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_s, e2e_serial_s = (float(x) for x in t.tolist())
    assert np.array_equal(out["argmax"], res["argmax"])

    # plain per-template kernel (map written, one call per template) on a subset
    plain = None
    if rank == 0 and args.plain_templates > 0:
        sub = templates[:args.plain_templates]
        maxcells = max(int(t["N_t0"]) * int(t["N_tau"]) for t in sub)
        d_map = torch.empty(maxcells, dtype=torch.float32, device=dev)
        d_r1 = torch.zeros(5, dtype=torch.float64, device=dev)
        dev_t = []
        for t in sub:
            t0s, taus = template_grids(t)
            dev_t.append((torch.from_numpy(t["atoms"]).to(dev),
                          torch.from_numpy(t0s.view(np.int32)).to(dev),
                          torch.from_numpy(taus.view(np.int32)).to(dev), t))
        def plain_pass():
            for A, t0s, taus, t in dev_t:
                h.map_plain(A, A.shape[0], t["TAtom"], t["t0_data"], t["window"], t0s,
                            t0s.shape[0], taus, taus.shape[0], d_map, d_r1,
                            flags=_lib.TCW_FLAG_LNBTSG)
        plain_pass()
        torch.cuda.synchronize(dev)
        p0 = torch.cuda.Event(enable_timing=True)
        p1 = torch.cuda.Event(enable_timing=True)
        p0.record(stream)
        plain_pass()
        p1.record(stream)
        torch.cuda.synchronize(dev)
        pcells = sum(int(t["N_t0"]) * int(t["N_tau"]) for t in sub)
        pval = pcells / (p0.elapsed_time(p1) * 1e-3)
        plain = {"value": pval, "unit": UNIT, "templates": len(sub),
                 "ratio_batched_over_plain": n_cells / (ms * 1e-3) / pval,
                 "note": "one tcw_map_plain call per template, full F map written"}

    if rank != 0:
        if ws > 1:
            torch.distributed.destroy_process_group()
        return

    # the same plan with the determinant in native FP64 (TCW_FLAG_FP64_DET)
    p64 = _lib.Plan(h, batch.desc, batch.t0s, batch.taus, batch.tile_config,
                    _lib.TCW_FLAG_LNBTSG | _lib.TCW_FLAG_FP64_DET)
    k64 = np.array([p64.run_timed(d_atoms, d_res) for _ in range(max(2, args.steps))])
    p64.close()
    _, r64_ms, e64_ms, _ = (float(x) for x in k64[1:].mean(axis=0))
    fp64_det = {"rect_ms": r64_ms, "exp_ms": e64_ms,
                "note": "map kernels with D = AB - C^2 in native FP64 instead of the "
                        "error-free FP32 products of the default path"}
    per_call = dropin_per_call(h)
    peaks = _lib.probe_peaks(dev.index)
    hbm_peak = None
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            hbm_peak = json.load(f).get("hbm_gbs")
    except (OSError, ValueError):
        pass
    single = plain_configs(h, dev, torch, stream, hbm_peak)
    grad = grad_case(torch, dev, peaks) if not args.no_grad else None
    roofline = roofline_block(batch, rect_ms, exp_ms, prefix_ms, fin_ms, peaks, clk,
                              torch.cuda.get_device_properties(dev).multi_processor_count)
    n_rect = int(np.sum(batch.desc["window"] == 1))
    atoms_bytes = batch.atoms.nbytes

    cpu = None
    if not args.no_cpu_baseline and ws == 1:
        threads = os.cpu_count() or 1
        v, d = cpu_baseline(templates, args.cpu_seconds, threads)
        v1, d1 = cpu_baseline(templates, args.cpu_seconds / 3.0, 1)
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": d["sample"] + "; oracle port of the reference pycuda kernels' FP32 "
                         "arithmetic + numpy reductions",
               "per_window_cells_per_s": d["per_window_cells_per_s"],
               "value_1thread": v1,
               "sample_1thread": d1["sample"],
               "per_call_ms": cpu_per_call(threads),
               "cpu": cpu_model()}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"batched {n_t} templates per GPU ({n_rect} rect, "
                   f"{n_t - n_rect} exp), SFTs 200-4000 with 0-30% gaps, grids 256-2048 per "
                   "axis, one CUDA graph per step",
                   "cells_per_step_per_gpu": n_cells, "atoms_bytes": atoms_bytes,
                   "l2": "inputs and per-template prefix rows larger than L2",
                   "tile_config": batch.tile_config, "parallelism": f"templates x{ws} ranks"},
        "roofline": roofline,
        "cpu_baseline": cpu,
        "e2e": {"value": total_cells / e2e_s, "unit": UNIT,
                "h2d_bytes_per_step": int(total_in), "d2h_bytes_per_step": int(total_out),
                "api": "TransientMapBatch.run_pipelined (tcw_plan_run_host_async), pinned "
                       "host atoms uploaded every step, each upload overlapping the previous "
                       "step's map kernels; results downloaded every step"},
        "e2e_serial": {"value": total_cells / e2e_serial_s, "unit": UNIT,
                       "api": "TransientMapBatch.run (tcw_plan_run_host), one blocking call "
                              "per step"},
        "plain_per_template": plain,
        "fp64_determinant_variant": fp64_det,
        "dropin_per_call": per_call,
        "single_template_device": single,
        "grad": grad,
        "gpu_launches": launches_per_step(n_rect, n_t - n_rect) * args.steps,
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


def run_case(args):
    """One plain single-template map (map written), CUDA-event timed: the
    write bandwidth it reaches against the measured HBM copy peak."""
    import torch

    from pyfstat_gb300 import _lib, synth
    from pyfstat_gb300.batched import template_grids

    t = dict(synth.precision_templates(1)[0], window=1 if args.case == "plain-rect" else 2)
    t0s, taus = template_grids(t)
    N_t0, N_tau = len(t0s), len(taus)
    dev = torch.device("cuda", 0)
    h = _lib.Handle(0)
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(stream)
    h.set_stream(stream.cuda_stream)
    A = torch.from_numpy(np.ascontiguousarray(t["atoms"], np.float32)).to(dev)
    d_t0 = torch.from_numpy(t0s.view(np.int32)).to(dev)
    d_tau = torch.from_numpy(taus.view(np.int32)).to(dev)
    F = torch.empty((N_t0, N_tau), dtype=torch.float32, device=dev)
    res = torch.zeros(5, dtype=torch.float64, device=dev)

    def call():
        h.map_plain(A, A.shape[0], t["TAtom"], t["t0_data"], t["window"], d_t0, N_t0, d_tau,
                    N_tau, F, res, flags=_lib.TCW_FLAG_LNBTSG)

    for _ in range(max(3, args.warmup)):
        call()
    torch.cuda.synchronize(dev)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        call()
    e1.record(stream)
    torch.cuda.synchronize(dev)
    ms = e0.elapsed_time(e1) / args.steps
    map_bytes = 4.0 * N_t0 * N_tau
    hbm = None
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            hbm = json.load(f).get("hbm_gbs")
    except (OSError, ValueError):
        pass
    gbs = map_bytes / (ms * 1e-3) / 1e9
    print(json.dumps({"case": args.case, "N_t0": N_t0, "N_tau": N_tau,
                      "numAtoms": int(A.shape[0]), "ms_per_call": ms,
                      "cells_per_s": N_t0 * N_tau / (ms * 1e-3), "map_bytes": map_bytes,
                      "map_write_gbs": gbs, "hbm_peak_gbs": hbm,
                      "frac_of_hbm": (gbs / hbm) if hbm else None}), flush=True)
    h.close()


def run_single_480(args):
    """The two single-template workloads alone (for their ncu captures)."""
    import torch

    from pyfstat_gb300 import _lib

    dev = torch.device("cuda", 0)
    h = _lib.Handle(0)
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(stream)
    h.set_stream(stream.cuda_stream)
    hbm = None
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            hbm = json.load(f).get("hbm_gbs")
    except (OSError, ValueError):
        pass
    print(json.dumps({"case": "single-480",
                      **plain_configs(h, dev, torch, stream, hbm, reps=max(1, args.steps))}),
          flush=True)
    h.close()


def main():
    args = parse()
    ws, rank, local = dist_env()
    if args.case == "single-480":
        if rank == 0:
            run_single_480(args)
        return
    if args.case == "grad":
        if rank == 0:
            import torch

            from pyfstat_gb300 import _lib

            peaks = _lib.probe_peaks(0)
            g = grad_case(torch, torch.device("cuda", 0), peaks, reps=max(1, args.steps),
                          n_templates=min(256, args.templates))
            print(json.dumps({"case": "grad", **g}), flush=True)
        return
    if args.case:
        if rank == 0:
            run_case(args)
        return
    if args.impl == "reference":
        run_reference(args, ws, rank)
    else:
        run_ours(args, ws, rank, local)


if __name__ == "__main__":
    main()
