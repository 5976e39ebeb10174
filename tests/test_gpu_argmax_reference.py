"""Argmax and max-posterior indices against the reference's own recorded
outputs.

tests/golden holds, per case, the reference's pycuda kernels' FP32 map (in
full, or every 16th row of the two 480-row workloads) and what the
reference's own ``pyTransientFstatMap`` computed from it: ``get_maxF_idx``
(pyfstat/tcw_fstat_map_funcs.py:186-194, first occurrence in row-major
order) and ``get_t0_max_posterior`` / ``get_tau_max_posterior`` (:219-287).

The reference's FP32 map differs from exact arithmetic by its own rounding
(err_ref, measured per case against the FP64 oracle on the stored cells).
Where the maximum is unique beyond that -- no other cell of the FP64 map
within 2 (err_ref + 1e-5) of the top, relatively -- the reference's index
is the true one and the GPU index must equal it exactly.  Only where cells
tie within the reference's own error (e.g. windows holding the same atoms,
or near-singular cells whose F the reference rounds by more than the gap)
is any tied index accepted; every such case is counted and printed.
"""

import numpy as np
import pytest

from _helpers import REL_TOL, THRESHOLD_BAND, argmax_ok, golden_case, index_ok
from pyfstat_gb300 import synth

pytestmark = pytest.mark.gpu

FLAGS = 0x1 | 0x2  # lnBtSG and posteriors


@pytest.fixture(scope="module")
def handle():
    from pyfstat_gb300 import _lib

    h = _lib.Handle(0)
    yield h
    h.close()


def _cases(golden):
    names = sorted({k.split("__")[0] for k in golden.files})
    out = []
    for name in names:
        g = golden[f"{name}__grid"]
        if f"{name}__t0s" in golden.files:  # explicit grid (log-spaced tau)
            c = dict(name=name, window=int(g[0]), TAtom=int(g[1]), t0_data=int(g[2]),
                     atoms=golden[f"{name}__atoms"], t0s=golden[f"{name}__t0s"],
                     taus=golden[f"{name}__taus"])
            for k in ("F_rows16", "maxF", "argmax", "lnBtSG"):
                c[k] = golden[f"{name}__{k}"]
        else:
            c = golden_case(golden, name)
        out.append(c)
    return out


def _unique_margin(values, margin):
    """Index of the maximum of ``values`` if every other entry lies more than
    ``margin`` (relative) below it, else None."""
    v = np.asarray(values, dtype=np.float64).reshape(-1)
    k = int(np.argmax(v))
    if v.size == 1:
        return k
    rest = np.delete(v, k)
    return k if rest.max() < v[k] - margin * abs(v[k]) else None


def _unique_log_margin(sums, log_margin):
    """Index of the largest of the positive ``sums`` if it exceeds every
    other one by more than a factor e^log_margin, else None."""
    v = np.asarray(sums, dtype=np.float64).reshape(-1)
    k = int(np.argmax(v))
    if v.size == 1:
        return k
    second = np.delete(v, k).max()
    if second <= 0.0:
        return k
    return k if np.log(v[k]) - np.log(second) > log_margin else None


def test_argmax_and_posteriors_equal_the_reference_where_unique(handle, oracle, golden):
    strict, tied = [], []
    for c in _cases(golden):
        name = c["name"]
        F, res = handle.map_plain_host(c["atoms"], c["TAtom"], c["t0_data"], c["window"],
                                       c["t0s"], c["taus"], want_map=True, flags=FLAGS)
        F64, cond = oracle.map_f64(c["atoms"], c["TAtom"], c["t0_data"], c["window"],
                                   c["t0s"], c["taus"], with_cond=True)
        if "F" in c:
            Fref, rows = c["F"], slice(None)
        else:
            Fref, rows = c["F_rows16"], slice(None, None, 16)
        band = np.abs(cond[rows] / 1e4 - 1.0) < THRESHOLD_BAND
        err = np.abs(Fref.astype(np.float64) - F64[rows]) / np.abs(F64[rows])
        err_ref = float(np.max(np.where(band, 0.0, err)))
        margin = 2.0 * (err_ref + REL_TOL)
        k = _unique_margin(F64, margin)
        if k is not None:
            # the reference's recorded index is the true maximum ...
            assert int(c["argmax"]) == k, (name, int(c["argmax"]), k)
            # ... and the GPU's equals it
            assert int(res["argmax"]) == int(c["argmax"]), (name, int(res["argmax"]))
            strict.append(name)
        else:
            assert argmax_ok(res["argmax"], F64, label=f"{name} argmax vs reference"), name
            tied.append(name)
        if "t0_MP" not in c:
            continue
        # posterior bin centres t0 + (k + 1/2) t0Band / N_t0 with t0Band = (N_t0 - 1) dt0
        # (the reference's windowRange of these cases, tcw:248-251, :283-286)
        e = np.exp(F64 - F64.max())
        for key, sums, idx, x0, dx, N in (
                ("t0_MP", e.sum(axis=1), int(res["t0_mp_idx"]), c["t0"], c["dt0"], c["N_t0"]),
                ("tau_MP", e.sum(axis=0), int(res["tau_mp_idx"]), c["tau"], c["dtau"],
                 c["N_tau"])):
            gpu_mp = x0 + (idx + 0.5) * (N - 1) * dx / N
            # the sums weigh exp(F - maxF): an absolute error of up to dF in
            # every F (and in maxF) scales each sum by a factor within
            # e^(+-2 dF), so a sum is the reference's maximum for sure when it
            # exceeds every other by more than e^(4 dF), dF = (err_ref + 1e-5) maxF
            dF = (err_ref + REL_TOL) * max(1.0, abs(F64.max()))
            m = _unique_log_margin(sums, 4.0 * dF)
            if m is not None:
                assert gpu_mp == pytest.approx(float(c[key]), abs=1e-6), (name, key)
                strict.append(f"{name} {key}")
            else:
                assert index_ok(idx, sums, label=f"{name} {key} vs reference"), (name, key)
                tied.append(f"{name} {key}")
    print(f"\nindices equal to the reference's exactly: {len(strict)}; "
          f"tied within the reference's own FP32 error: {len(tied)} {tied}")
    # the two 480-row workloads have a unique maximum: no tie branch there
    assert "workload_rect480" in strict and "workload_exp480x512log" in strict
    assert not any(t.startswith("workload_") for t in tied), tied


@pytest.mark.parametrize("case", ["rect", "exp"])
def test_workload_480_argmax_is_the_unique_fp64_maximum(handle, oracle, case):
    c = synth.plain_rect_case() if case == "rect" else synth.plain_exp_case()
    F, res = handle.map_plain_host(c["atoms"], c["TAtom"], c["t0_data"], c["window"], c["t0s"],
                                   c["taus"], want_map=True, flags=FLAGS)
    F64 = oracle.map_f64(c["atoms"], c["TAtom"], c["t0_data"], c["window"], c["t0s"], c["taus"])
    k = _unique_margin(F64, 1e-3)
    assert k is not None and int(res["argmax"]) == k
    e = np.exp(F64 - F64.max())
    assert int(res["t0_mp_idx"]) == _unique_margin(e.sum(axis=1), 1e-6)
    assert int(res["tau_mp_idx"]) == _unique_margin(e.sum(axis=0), 1e-6)
