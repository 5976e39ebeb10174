"""Pin the CPU oracle against the reference's own outputs (tests/golden/).

The golden fixtures hold maps of the reference pycuda kernels compiled for the
host and the reference's own numpy post-processing (make_golden.py).  The FP32
port must reproduce those maps bit for bit; the post-processing restatement
must reproduce the reference's numbers; the FP64 arbiter must agree with the
reference to within the reference's own FP32 error on well-conditioned cells.
"""

import numpy as np
import pytest

from _helpers import golden_case, golden_cases, sha256


def _port_map(O, c):
    fn = O.rect_map_f32 if c["window"] == 1 else O.exp_map_f32
    return fn(c["atoms"], c["TAtom"], c["t0_data"], c["t0s"], c["taus"])


def test_golden_has_cases(golden):
    names = golden_cases(golden)
    assert len(names) >= 30
    assert "workload_rect480" in names


@pytest.mark.parametrize("threads", [1, 4])
def test_port_bit_exact_on_every_golden_case(oracle, golden, threads):
    for name in golden_cases(golden):
        c = golden_case(golden, name)
        fn = oracle.rect_map_f32 if c["window"] == 1 else oracle.exp_map_f32
        F = fn(c["atoms"], c["TAtom"], c["t0_data"], c["t0s"], c["taus"], nthreads=threads)
        assert np.array_equal(sha256(F), c["sha256"]), name
        if "F" in c:
            assert np.array_equal(F.view(np.uint32), c["F"].view(np.uint32)), name
        else:
            assert np.array_equal(F[::16].view(np.uint32), c["F_rows16"].view(np.uint32)), name


def test_port_bit_exact_log_tau_exp_workload(oracle, golden):
    name = "workload_exp480x512log"
    A = golden[f"{name}__atoms"]
    _, TAtom, t0_data = (int(v) for v in golden[f"{name}__grid"])
    F = oracle.exp_map_f32(A, TAtom, t0_data, golden[f"{name}__t0s"], golden[f"{name}__taus"])
    assert np.array_equal(sha256(F), golden[f"{name}__sha256"])
    m, k = oracle.max_argmax(F)
    assert float(m) == float(golden[f"{name}__maxF"]) and k == int(golden[f"{name}__argmax"])
    assert oracle.lnBtSG(F) == pytest.approx(float(golden[f"{name}__lnBtSG"]), rel=1e-12)


def test_postprocessing_matches_reference(oracle, golden):
    for name in golden_cases(golden):
        c = golden_case(golden, name)
        if "F" not in c:
            continue
        F = c["F"]
        m, k = oracle.max_argmax(F)
        assert float(m) == float(c["maxF"]), name
        assert k == int(c["argmax"]), name
        assert oracle.lnBtSG(F) == pytest.approx(float(c["lnBtSG"]), rel=1e-12, abs=1e-9), name
        dx = (c["N_t0"] - 1) * c["dt0"] / c["N_t0"]
        dy = (c["N_tau"] - 1) * c["dtau"] / c["N_tau"]
        t0_MP = c["t0"] + (oracle.t0_max_posterior_idx(F) + 0.5) * dx
        tau_MP = c["tau"] + (oracle.tau_max_posterior_idx(F) + 0.5) * dy
        assert t0_MP == pytest.approx(float(c["t0_MP"]), abs=1e-6), name
        assert tau_MP == pytest.approx(float(c["tau_MP"]), abs=1e-6), name


def test_f64_arbiter_agrees_with_reference_where_well_conditioned(oracle, golden):
    for name in golden_cases(golden):
        c = golden_case(golden, name)
        F64, cond = oracle.map_f64(c["atoms"], c["TAtom"], c["t0_data"], c["window"], c["t0s"],
                                   c["taus"], with_cond=True)
        Fref = c["F"] if "F" in c else None
        if Fref is None:
            F64, cond, Fref = F64[::16], cond[::16], c["F_rows16"]
        good = cond < 50.0
        rel = np.abs(Fref[good] - F64[good]) / np.abs(F64[good])
        assert rel.size == 0 or rel.max() < 2e-4, (name, rel.max())
        # both sides fall back to F = 2 on the same ill-conditioned cells
        clear = (cond > 1.01e4) | ~np.isfinite(cond)
        assert np.all(F64[clear] == 2.0) and np.all(Fref[clear] == 2.0), name


def test_index_semantics_u32_wraparound(oracle):
    t0_data, TAtom, N = 700000000, 1800, 40
    # in range
    assert oracle.idx_start(t0_data, t0_data, TAtom, N) == 0
    assert oracle.idx_start(t0_data + 900, t0_data, TAtom, N) == 1  # rounds half up
    assert oracle.idx_start(t0_data + 899, t0_data, TAtom, N) == 0
    # before the data: the unsigned difference wraps and the index clamps high
    assert oracle.idx_start(t0_data - 5 * 1800, t0_data, TAtom, N) == N - 1
    # within half a bin before the data: wraps back to 0
    assert oracle.idx_start(t0_data - 600, t0_data, TAtom, N) == 0
    # end index: quotient 0 minus one wraps to -1, clamps to 0
    assert oracle.idx_end(t0_data, t0_data, TAtom, N) == 0
    assert oracle.idx_end(t0_data + 1800, t0_data, TAtom, N) == 0
    assert oracle.idx_end(t0_data + 3600, t0_data, TAtom, N) == 1
    assert oracle.idx_end(t0_data + 10 ** 6, t0_data, TAtom, N) == N - 1


@pytest.mark.skipif(not __import__("oracle").RefKernels.available(),
                    reason="reference kernels not built here (make -C oracle ref)")
def test_port_matches_live_reference_kernels(oracle):
    from pyfstat_gb300 import synth
    from pyfstat_gb300.window import uniform_grid

    ref = oracle.RefKernels()
    for window in (1, 2):
        t0_data, A = synth.merged_atoms(42, 150, 2, gap_frac=0.2)
        # uniform grid starting before the data (u32 wrap-around rows included)
        t0, dt0, tau, dtau = t0_data - 2000, 1300, 900, 2300
        t0s = uniform_grid(t0, dt0, 60)
        taus = uniform_grid(tau, dtau, 50)
        Fr = ref.map_uniform(window, A, 1800, t0_data, t0, dt0, tau, dtau, 60, 50)
        fn = oracle.rect_map_f32 if window == 1 else oracle.exp_map_f32
        Fp = fn(A, 1800, t0_data, t0s, taus)
        assert np.array_equal(Fr.view(np.uint32), Fp.view(np.uint32))
