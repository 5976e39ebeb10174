"""Shared helpers of the test-suite (case loading, error metrics, host-cell calls)."""

import ctypes
import hashlib

import numpy as np

from pyfstat_gb300.window import uniform_grid

P = ctypes.c_void_p

# Cells whose FP64 conditioning number lies this close (relatively) to the
# reference's cut cond < 1e4 may legitimately fall on either side of it under
# any rounding change; they are counted separately, not compared.
THRESHOLD_BAND = 1e-5
# Parity bar on F (and 2F) against the FP64 oracle.
REL_TOL = 1e-5


def golden_cases(golden):
    """Names of the uniform-grid golden cases."""
    names = sorted({k.split("__")[0] for k in golden.files})
    return [n for n in names if f"{n}__dt0" not in golden.files and golden[f"{n}__grid"].size == 9]


def golden_case(golden, name):
    g = golden[f"{name}__grid"]
    window, TAtom, t0_data, t0, dt0, tau, dtau, N_t0, N_tau = (int(v) for v in g)
    c = dict(name=name, window=window, TAtom=TAtom, t0_data=t0_data, t0=t0, dt0=dt0, tau=tau,
             dtau=dtau, N_t0=N_t0, N_tau=N_tau, atoms=golden[f"{name}__atoms"],
             t0s=uniform_grid(t0, dt0, N_t0), taus=uniform_grid(tau, dtau, N_tau))
    for k in ("F", "F_rows16", "maxF", "argmax", "lnBtSG", "t0_MP", "tau_MP", "sha256"):
        key = f"{name}__{k}"
        if key in golden.files:
            c[k] = golden[key]
    return c


def sha256(a):
    return np.frombuffer(hashlib.sha256(np.ascontiguousarray(a).tobytes()).digest(), np.uint8)


def rel_err(F, F64, cond):
    """Elementwise |F - F64| / |F64| with threshold-band cells set to 0; also
    returns the number of threshold-band cells."""
    F = np.asarray(F, dtype=np.float64)
    rel = np.abs(F - F64) / np.maximum(np.abs(F64), 1e-30)
    band = np.abs(cond / 1e4 - 1.0) < THRESHOLD_BAND
    rel = np.where(band, 0.0, rel)
    return rel, int(band.sum())


def hc_map(lib, c, comp=True, row_chunk=0):
    """Map of the host build of the device arithmetic for case dict ``c``."""
    A = np.ascontiguousarray(c["atoms"], np.float32)
    t0s = np.ascontiguousarray(c["t0s"], np.uint32)
    taus = np.ascontiguousarray(c["taus"], np.uint32)
    F = np.empty((len(t0s), len(taus)), np.float32)
    ok = np.empty(F.shape, np.uint8)
    args = [A.ctypes.data_as(P), ctypes.c_uint32(A.shape[0]), ctypes.c_uint32(c["TAtom"]),
            ctypes.c_uint32(c["t0_data"]), t0s.ctypes.data_as(P), ctypes.c_uint32(len(t0s)),
            taus.ctypes.data_as(P), ctypes.c_uint32(len(taus)), ctypes.c_int(int(comp))]
    if c["window"] == 1:
        lib.hc_rect_map(*args, F.ctypes.data_as(P), ok.ctypes.data_as(P))
    else:
        lib.hc_exp_map(*args, ctypes.c_uint32(row_chunk), F.ctypes.data_as(P),
                       ok.ctypes.data_as(P))
    return F, ok.astype(bool)


# How often argmax_ok / index_ok compared against a unique maximum (exact
# index equality) and how often they took the tie branch, over the session;
# conftest.py prints the counts at the end of the run.
ARGMAX_COUNTS = {"unique": 0, "tie": 0}
ARGMAX_TIE_LABELS = []


def argmax_ok(idx, F64, tol=REL_TOL, label=None):
    """The flat argmax ``idx`` is the oracle's when the oracle's maximum is
    unique within the tolerance; where several cells tie within it (windows
    holding the same atoms, e.g. one merged bin between gaps) any of them.
    Each call is counted as a unique-maximum or a tie-branch comparison."""
    F64 = np.asarray(F64, dtype=np.float64).reshape(-1)
    top = F64.max()
    tied = np.flatnonzero(F64 >= top - 2 * tol * abs(top))
    if tied.size == 1:
        ARGMAX_COUNTS["unique"] += 1
        return int(idx) == int(tied[0])
    ARGMAX_COUNTS["tie"] += 1
    ARGMAX_TIE_LABELS.append(f"{label or '?'} ({tied.size} cells)")
    return int(idx) in set(int(i) for i in tied)


def index_ok(idx, values, tol=REL_TOL, label=None):
    """Same rule for the argmax of a 1-D marginal (posterior row/column sums)."""
    return argmax_ok(idx, values, tol, label)
