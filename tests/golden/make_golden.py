"""Generate the golden fixtures in tests/golden/ from the reference itself.

Run where a PyFstat checkout is available, with PYFSTAT_REF naming it, after
the host build of its pycuda kernels (``make -C oracle ref REF=$PYFSTAT_REF``):

    PYFSTAT_REF=<checkout> python tests/golden/make_golden.py

For every case it records
  * the F map of the reference's own kernels compiled for the host
    (oracle/_ref/libtcw_ref.so, FP32, reference arithmetic): in full for small
    cases; for the two 480-row workloads every 16th row plus a SHA-256 of the
    whole map's bytes;
  * maxF, argmax, lnBtSG, t0_MP and tau_MP from the reference's own
    ``pyTransientFstatMap`` (pyfstat/tcw_fstat_map_funcs.py, imported on its
    own: its top-level imports are only importlib, logging, os, time, numpy).
The atoms come from pyfstat_gb300.synth (seeded) and are stored with the case.
"""

import hashlib
import importlib.util
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "oracle"))

import oracle as O  # noqa: E402
from pyfstat_gb300 import synth  # noqa: E402
from pyfstat_gb300.window import transientWindowRange_t, uniform_grid  # noqa: E402

REF = os.environ.get("PYFSTAT_REF")
if not REF:
    sys.exit("set PYFSTAT_REF to the PyFstat checkout the fixtures are generated from")


def load_reference_tcw():
    path = os.path.join(REF, "pyfstat", "tcw_fstat_map_funcs.py")
    spec = importlib.util.spec_from_file_location("ref_tcw_fstat_map_funcs", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def ref_postprocess(tcw, F, wr):
    """maxF, argmax, lnBtSG, t0_MP, tau_MP exactly as the reference computes them."""
    fm = tcw.pyTransientFstatMap(N_t0Range=F.shape[0], N_tauRange=F.shape[1])
    fm.F_mn = F
    fm.maxF = F.max()
    idx = fm.get_maxF_idx()
    lnB = fm.get_lnBtSG()
    t0_MP = fm.get_t0_max_posterior(wr)
    tau_MP = fm.get_tau_max_posterior(wr)
    return dict(maxF=np.float64(fm.maxF), argmax=np.int64(idx[0] * F.shape[1] + idx[1]),
                lnBtSG=np.float64(lnB), t0_MP=np.float64(t0_MP), tau_MP=np.float64(tau_MP))


def uniform_case(name, window, atoms, TAtom, t0_data, t0, dt0, tau, dtau, N_t0, N_tau,
                 full=True):
    return dict(name=name, window=window, atoms=atoms, TAtom=TAtom, t0_data=t0_data, t0=t0,
                dt0=dt0, tau=tau, dtau=dtau, N_t0=N_t0, N_tau=N_tau, full=full)


def small_cases():
    cases = []
    rng = np.random.default_rng(7)
    # tiny grids and atom counts (1, 2, 31 atoms; 1, 2, 3, 33 grid points)
    for nsft in (1, 2, 31):
        t0_data, A = synth.merged_atoms(100 + nsft, nsft, 1, inject=None)
        for N in (1, 2, 3, 33):
            for window in (1, 2):
                cases.append(uniform_case(f"tiny_w{window}_a{nsft}_g{N}", window, A, 1800,
                                          t0_data, t0_data, 1800, 1800, 1800, N, N))
    # grid larger than the data span (index clamps engage)
    t0_data, A = synth.merged_atoms(3, 40, 1, inject=None)
    for window in (1, 2):
        cases.append(uniform_case(f"clamp_w{window}", window, A, 1800, t0_data, t0_data,
                                  1800, 1800, 3600, 64, 48))
    # t0 before the data start: u32 wrap-around in the reference index arithmetic
    for window in (1, 2):
        cases.append(uniform_case(f"wrap_w{window}", window, A, 1800, t0_data,
                                  t0_data - 5 * 1800, 1800, 1800, 1800, 20, 20))
        cases.append(uniform_case(f"wraphalf_w{window}", window, A, 1800, t0_data,
                                  t0_data - 600, 1800, 1800, 1800, 8, 8))
    # t0 and tau steps not multiples of TAtom
    t0_data, A = synth.merged_atoms(4, 300, 2, gap_frac=0.1)
    for window in (1, 2):
        cases.append(uniform_case(f"offgrid_w{window}", window, A, 1800, t0_data,
                                  t0_data + 450, 700, 1000, 1300, 90, 70))
    # gaps (zero atoms) with the injection inside, rect and exp
    t0_data, A = synth.merged_atoms(5, 400, 1, gap_frac=0.3)
    for window in (1, 2):
        cases.append(uniform_case(f"gaps_w{window}", window, A, 1800, t0_data, t0_data, 1800,
                                  3600, 1800, 120, 100))
    # window type "none": one rectangular cell spanning all data (tcw:742-749)
    t0_data, A = synth.merged_atoms(6, 200, 1)
    cases.append(uniform_case("none_equiv", 1, A, 1800, t0_data, t0_data, 1800,
                              A.shape[0] * 1800, 1800, 1, 1))
    # the reference test's geometry (1 day of 1800 s SFTs, H1; test_tcw:36-50)
    t0_data, A = synth.merged_atoms(1, 48, 1, inject=(12, 24))
    day = 86400
    for window in (1, 2):
        cases.append(uniform_case(f"reftest_w{window}", window, A, 1800, t0_data, t0_data,
                                  1800, 2 * 1800, 1800, (day - 2 * 1800) // 1800 + 1,
                                  (day - 2 * 1800) // 1800 + 1))
    del rng
    return cases


def main():
    if not O.RefKernels.available():
        raise SystemExit("build the reference harness first: make -C oracle ref")
    tcw = load_reference_tcw()
    ref = O.RefKernels()
    cases = small_cases()
    c0 = synth.plain_rect_case()
    cases.append(uniform_case("workload_rect480", 1, c0["atoms"], 1800, c0["t0_data"],
                              c0["t0"], 1800, 1800, 1800, 480, 480, full=False))
    out = {}
    for c in cases:
        A = c["atoms"]
        F = ref.map_uniform(c["window"], A, c["TAtom"], c["t0_data"], c["t0"], c["dt0"],
                            c["tau"], c["dtau"], c["N_t0"], c["N_tau"])
        wr = transientWindowRange_t(type=c["window"], t0=c["t0"],
                                    t0Band=(c["N_t0"] - 1) * c["dt0"], dt0=c["dt0"],
                                    tau=c["tau"], tauBand=(c["N_tau"] - 1) * c["dtau"],
                                    dtau=c["dtau"])
        post = ref_postprocess(tcw, F, wr)
        rec = dict(atoms=A, grid=np.array([c["window"], c["TAtom"], c["t0_data"], c["t0"],
                                           c["dt0"], c["tau"], c["dtau"], c["N_t0"],
                                           c["N_tau"]], dtype=np.int64),
                   sha256=np.frombuffer(hashlib.sha256(F.tobytes()).digest(), np.uint8))
        if c["full"]:
            rec["F"] = F
        else:
            rec["F_rows16"] = F[::16]
        rec.update(post)
        for k, v in rec.items():
            out[f"{c['name']}__{k}"] = v
    # log-spaced exponential workload (2 detectors merged): explicit tau grid
    e = synth.plain_exp_case()
    F = ref.map_grid(2, e["atoms"], 1800, e["t0_data"], e["t0s"], e["taus"])
    fm = tcw.pyTransientFstatMap(N_t0Range=F.shape[0], N_tauRange=F.shape[1])
    fm.F_mn = F
    fm.maxF = F.max()
    idx = fm.get_maxF_idx()
    name = "workload_exp480x512log"
    out[f"{name}__atoms"] = e["atoms"]
    out[f"{name}__t0s"] = e["t0s"]
    out[f"{name}__taus"] = e["taus"]
    out[f"{name}__grid"] = np.array([2, 1800, e["t0_data"]], dtype=np.int64)
    out[f"{name}__sha256"] = np.frombuffer(hashlib.sha256(F.tobytes()).digest(), np.uint8)
    out[f"{name}__F_rows16"] = F[::16]
    out[f"{name}__maxF"] = np.float64(fm.maxF)
    out[f"{name}__argmax"] = np.int64(idx[0] * F.shape[1] + idx[1])
    out[f"{name}__lnBtSG"] = np.float64(fm.get_lnBtSG())
    path = os.path.join(HERE, "reference_maps.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path}: {len(cases) + 1} cases, {os.path.getsize(path) / 1e3:.0f} kB")
    assert np.array_equal(uniform_grid(c0["t0"], 1800, 480), c0["t0s"])


if __name__ == "__main__":
    main()
