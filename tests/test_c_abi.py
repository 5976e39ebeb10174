"""The C ABI from a plain C program (gcc, no Python in the client): without a
GPU the handle creation fails with a status code and message; on the GPU the
map's result record agrees with the FP64 oracle."""

import json
import os
import shutil
import subprocess

import numpy as np
import pytest

from _helpers import REL_TOL, argmax_ok
from pyfstat_gb300 import build as B
from pyfstat_gb300 import synth

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def client(tmp_path_factory):
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    lib = B.build()
    out = tmp_path_factory.mktemp("cabi") / "client"
    subprocess.run(["gcc", "-O2", "-std=c11", "-I", os.path.join(REPO, "include"),
                    os.path.join(REPO, "tests", "c_abi_client.c"), "-o", str(out),
                    "-L", os.path.dirname(lib), "-ltcw_b200",
                    f"-Wl,-rpath,{os.path.dirname(lib)}"], check=True)
    return out


def run_client(client, tmp_path, case, window):
    p = tmp_path / "atoms.bin"
    with open(p, "wb") as f:
        np.array([case["atoms"].shape[0], 1800, case["t0_data"], case["t0s"].size,
                  case["taus"].size], np.uint32).tofile(f)
        case["t0s"].astype(np.uint32).tofile(f)
        case["taus"].astype(np.uint32).tofile(f)
        np.ascontiguousarray(case["atoms"], np.float32).tofile(f)
    out = subprocess.run([str(client), str(p), str(window)], capture_output=True, text=True,
                         check=True)
    return json.loads(out.stdout)


def small_case():
    t0_data, A = synth.merged_atoms(9, 80, 2, gap_frac=0.1)
    return dict(atoms=A, t0_data=t0_data,
                t0s=(t0_data + 1800 * np.arange(40)).astype(np.uint32),
                taus=(1800 + 1800 * np.arange(30)).astype(np.uint32))


def test_client_links_and_reports_status_without_a_device(client, tmp_path):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present (covered by the GPU test)")
    r = run_client(client, tmp_path, small_case(), 2)
    assert r["abi"] >= 1 and r["create"] < 0 and r["error"]


@pytest.mark.gpu
@pytest.mark.parametrize("window", [1, 2])
def test_client_map_matches_fp64_oracle(client, tmp_path, oracle, window):
    c = small_case()
    r = run_client(client, tmp_path, c, window)
    assert r["map"] == 0, r
    F64 = oracle.map_f64(c["atoms"], 1800, c["t0_data"], window, c["t0s"], c["taus"])
    assert abs(r["maxF"] - F64.max()) <= REL_TOL * F64.max()
    assert argmax_ok(r["argmax"], F64)
    assert r["lnBtSG"] == pytest.approx(oracle.lnBtSG(F64), rel=REL_TOL)
    assert abs(r["F00"] - F64[0, 0]) <= REL_TOL * abs(F64[0, 0])
    # the batched plan from C: template `window - 1` is this window's map
    assert r["plan"] == 0, r
    assert r["pipelined_equal"] is True
    k = window - 1
    assert abs(r["plan_maxF"][k] - F64.max()) <= REL_TOL * F64.max()
    assert argmax_ok(r["plan_argmax"][k], F64)
