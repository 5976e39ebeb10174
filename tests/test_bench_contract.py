"""The benchmark's one-line JSON output: the reference arm on the CPU (the
oracle port of the reference's CPU path) and, on a GPU, this library's arm
on a small batch.  Checks the keys and types the line promises, not the
numbers."""

import json
import os
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def run_bench(*args, timeout=600):
    r = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), *args], cwd=REPO,
                       capture_output=True, text=True, timeout=timeout)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]
    return json.loads(lines[0])


def check_common(d, steps, warmup):
    assert d["metric"] and d["unit"] == "cells/s"
    assert d["value"] > 0 and d["ms_per_step"] > 0
    assert d["n_gpus"] == 1 and d["steps"] == steps and d["warmup"] == warmup
    assert d["higher_is_better"] is True and d["scaling"] == "weak"
    assert d["vs_baseline"] is None
    assert d["dtype"] == "f32" and d["data"] == "synthetic"
    assert isinstance(d["config"]["workload"], str)


def test_reference_arm_line():
    d = run_bench("--impl", "reference", "--steps", "1", "--warmup", "0", "--templates", "8",
                  "--cpu-seconds", "0.5")
    check_common(d, 1, 0)
    assert d["impl"] == "reference"
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["unit"] == "cells/s"
    assert cb["cores"] >= 1 and cb["kind"] in ("port", "reference") and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "cells/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}


@pytest.mark.gpu
def test_gpu_arm_line():
    d = run_bench("--steps", "2", "--warmup", "3", "--templates", "64", "--plain-templates", "4",
                  "--cpu-seconds", "0.5", "--tile", "default")
    check_common(d, 2, 3)
    assert "impl" not in d or d["impl"] == "ours"
    r = d["roofline"]
    assert r["bound"] in ("fp64", "fp32", "mufu", "hbm")
    assert r["unit"] in ("TFLOP/s", "GB/s", "Tops/s")
    assert 0 < r["achieved"] and 0 < r["peak"]
    assert r["frac"] == pytest.approx(r["achieved"] / r["peak"], rel=1e-9)
    assert r["traffic"] is None or r["traffic"] > 0
    cb = d["cpu_baseline"]
    assert cb["value"] > 0 and cb["cores"] >= 1 and cb["kind"] == "port"
    e = d["e2e"]
    assert e["value"] > 0 and e["unit"] == "cells/s"
    assert e["h2d_bytes_per_step"] > 0 and e["d2h_bytes_per_step"] > 0
    assert d["gpu_launches"] >= 2 * 5
    c = d["clocks"]
    assert "sm_mhz" in c and "sm_max_mhz" in c and isinstance(c["reasons"], list)
    for name in ("rect_480x480", "exp_480x512log"):
        s = d["single_template_device"][name]
        assert s["cells_per_s"] > 0 and s["hbm_gbs"] > 0
    g = d["grad"]
    for name in ("forward", "backward"):
        assert g[name]["ms"] > 0 and g[name]["roofline"]["bound"] == "fp64"
        assert 0 < g[name]["roofline"]["frac"] < 2
    assert isinstance(r["kernels"][r["kernel"]]["profile_source_current"], bool)


@pytest.mark.gpu
def test_gpu_single_template_case_line():
    for case in ("plain-rect", "plain-exp"):
        r = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--case", case,
                            "--steps", "2", "--warmup", "3"], cwd=REPO, capture_output=True,
                           text=True, timeout=600)
        assert r.returncode == 0, r.stderr[-2000:]
        d = json.loads([l for l in r.stdout.splitlines() if l.startswith("{")][-1])
        assert d["case"] == case and d["N_t0"] == 8192 and d["N_tau"] == 4096
        assert d["ms_per_call"] > 0 and d["map_bytes"] == 4.0 * 8192 * 4096
        assert d["map_write_gbs"] == pytest.approx(d["map_bytes"] / d["ms_per_call"] / 1e6)


def test_rect_reused_fraction():
    """The bench line's share of rect cells whose window end equals their
    left neighbour's: a template whose taus all reach past the data repeats
    the last atom as every window end after the first column, and one with
    a tau step of whole SFTs inside the data repeats none."""
    import numpy as np

    sys.path.insert(0, REPO)
    import bench
    from pyfstat_gb300 import _lib

    T, n = 1800, 100
    desc = np.zeros(2, dtype=_lib.DESC_DTYPE)
    t0d = 700000000
    t0s = np.concatenate([t0d + T * np.arange(10), t0d + T * np.arange(10)]).astype(np.uint32)
    taus = np.concatenate([(n * T + T * np.arange(8)),            # past the data: clamped
                           (T + T * np.arange(8))]).astype(np.uint32)  # one SFT apart
    for k in range(2):
        desc[k] = (0, 10 * k, 8 * k, n, T, t0d, 1, 10, 8)
    one = bench.rect_reused_fraction(desc[:1], t0s, taus)
    assert abs(one - 7 / 8) < 1e-12
    two = bench.rect_reused_fraction(desc[1:], t0s, taus)
    assert two == 0.0
