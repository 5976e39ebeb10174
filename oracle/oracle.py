"""CPU oracle for the transient-CW F-statistic map -- TEST INFRASTRUCTURE ONLY.

Only tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module, and only as the checker or the timed CPU
baseline.  The product path (``pyfstat_gb300``) never imports it.

Contents
--------
* ctypes bindings to ``liboracle.so`` (``tcw_oracle.c``):
  - ``rect_map_f32`` / ``exp_map_f32``: the reference pycuda kernels' FP32
    arithmetic restated in C (cudaTransientFstatRectWindow.cu:16-128,
    cudaTransientFstatExpWindow.cu:16-134) -- the "port" CPU baseline;
  - ``map_f64`` / ``cells_f64`` / ``cell_sums_f64``: the same per-cell math in
    FP64 -- the parity arbiter.
* ``lnBtSG``, ``max_argmax``, ``t0_max_posterior``, ``tau_max_posterior``: the
  numpy post-processing of ``pyTransientFstatMap`` (tcw_fstat_map_funcs.py:
  186-287) restated, evaluated in the precision of the map passed in.
* ``RefKernels``: bindings to ``_ref/libtcw_ref.so``, the reference's own
  kernel sources compiled for the host (only where that build exists).
"""

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_LIB_PATH = os.path.join(HERE, "_ref", "libtcw_ref.so")

WIN_RECT = 1
WIN_EXP = 2

_u32p = ctypes.POINTER(ctypes.c_uint32)
_f32p = ctypes.POINTER(ctypes.c_float)
_f64p = ctypes.POINTER(ctypes.c_double)

_lib = None


def build(ref=False):
    """Compile liboracle.so (and, if ``ref``, the reference harness)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True)


def _load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(
            os.path.join(HERE, "tcw_oracle.c")
        ):
            build()
        lib = ctypes.CDLL(LIB_PATH)
        sig_map32 = [_f32p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                     _u32p, ctypes.c_uint32, _u32p, ctypes.c_uint32, _f32p, ctypes.c_int]
        for name in ("tcwo_rect_map_f32", "tcwo_exp_map_f32"):
            fn = getattr(lib, name)
            fn.argtypes = sig_map32
            fn.restype = ctypes.c_int
        lib.tcwo_map_f64.argtypes = [_f32p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                     ctypes.c_int, _u32p, ctypes.c_uint32, _u32p,
                                     ctypes.c_uint32, _f64p, _f64p, ctypes.c_int]
        lib.tcwo_map_f64.restype = ctypes.c_int
        lib.tcwo_cells_f64.argtypes = [_f32p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                       ctypes.c_int, _u32p, _u32p, ctypes.c_uint64, _f64p,
                                       _f64p, ctypes.c_int]
        lib.tcwo_cells_f64.restype = ctypes.c_int
        lib.tcwo_cell_sums_f64.argtypes = [_f32p, ctypes.c_uint32, ctypes.c_uint32,
                                           ctypes.c_uint32, ctypes.c_int, _u32p, _u32p,
                                           ctypes.c_uint64, _f64p]
        lib.tcwo_cell_sums_f64.restype = ctypes.c_int
        lib.tcwo_exp_map_f64_realtau.argtypes = [_f32p, ctypes.c_uint32, ctypes.c_uint32,
                                                 ctypes.c_uint32, _u32p, ctypes.c_uint32, _f64p,
                                                 ctypes.c_uint32, _f64p, ctypes.c_int]
        lib.tcwo_exp_map_f64_realtau.restype = ctypes.c_int
        for name in ("tcwo_idx_start", "tcwo_idx_end"):
            fn = getattr(lib, name)
            fn.argtypes = [ctypes.c_uint32] * 4
            fn.restype = ctypes.c_uint32
        _lib = lib
    return _lib


def _c(arr, dtype):
    return np.ascontiguousarray(arr, dtype=dtype)


def _atoms(atoms7):
    a = _c(atoms7, np.float32)
    if a.ndim != 2 or a.shape[1] != 7:
        raise ValueError("atoms must be a (numAtoms, 7) float32 matrix")
    return a


def rect_map_f32(atoms7, TAtom, t0_data, t0s, taus, nthreads=0):
    """Reference FP32 arithmetic, rectangular window (Rect.cu:16-128)."""
    return _map_f32("tcwo_rect_map_f32", atoms7, TAtom, t0_data, t0s, taus, nthreads)


def exp_map_f32(atoms7, TAtom, t0_data, t0s, taus, nthreads=0):
    """Reference FP32 arithmetic, exponential window (Exp.cu:16-134)."""
    return _map_f32("tcwo_exp_map_f32", atoms7, TAtom, t0_data, t0s, taus, nthreads)


def _map_f32(name, atoms7, TAtom, t0_data, t0s, taus, nthreads):
    lib = _load()
    a = _atoms(atoms7)
    t0s = _c(t0s, np.uint32)
    taus = _c(taus, np.uint32)
    out = np.empty((len(t0s), len(taus)), dtype=np.float32)
    rc = getattr(lib, name)(a.ctypes.data_as(_f32p), a.shape[0], int(TAtom), int(t0_data),
                            t0s.ctypes.data_as(_u32p), len(t0s), taus.ctypes.data_as(_u32p),
                            len(taus), out.ctypes.data_as(_f32p), int(nthreads))
    if rc != 0:
        raise ValueError(f"oracle {name} failed with status {rc}")
    return out


def map_f64(atoms7, TAtom, t0_data, window, t0s, taus, with_cond=False, nthreads=0):
    """FP64 arbiter map F[m, n] (and the conditioning number if asked)."""
    lib = _load()
    a = _atoms(atoms7)
    t0s = _c(t0s, np.uint32)
    taus = _c(taus, np.uint32)
    F = np.empty((len(t0s), len(taus)), dtype=np.float64)
    cond = np.empty_like(F) if with_cond else None
    rc = lib.tcwo_map_f64(a.ctypes.data_as(_f32p), a.shape[0], int(TAtom), int(t0_data),
                          int(window), t0s.ctypes.data_as(_u32p), len(t0s),
                          taus.ctypes.data_as(_u32p), len(taus), F.ctypes.data_as(_f64p),
                          cond.ctypes.data_as(_f64p) if with_cond else None, int(nthreads))
    if rc != 0:
        raise ValueError(f"oracle map_f64 failed with status {rc}")
    return (F, cond) if with_cond else F


def cells_f64(atoms7, TAtom, t0_data, window, t0s, taus, with_cond=False, nthreads=0):
    """FP64 F for the cells (t0s[k], taus[k])."""
    lib = _load()
    a = _atoms(atoms7)
    t0s = _c(t0s, np.uint32)
    taus = _c(taus, np.uint32)
    if t0s.shape != taus.shape:
        raise ValueError("t0s and taus must have the same shape")
    F = np.empty(t0s.shape, dtype=np.float64)
    cond = np.empty_like(F) if with_cond else None
    rc = lib.tcwo_cells_f64(a.ctypes.data_as(_f32p), a.shape[0], int(TAtom), int(t0_data),
                            int(window), t0s.ctypes.data_as(_u32p), taus.ctypes.data_as(_u32p),
                            t0s.size, F.ctypes.data_as(_f64p),
                            cond.ctypes.data_as(_f64p) if with_cond else None, int(nthreads))
    if rc != 0:
        raise ValueError(f"oracle cells_f64 failed with status {rc}")
    return (F, cond) if with_cond else F


def cell_sums_f64(atoms7, TAtom, t0_data, window, t0s, taus):
    """FP64 window sums (A, B, C, Fa_re, Fa_im, Fb_re, Fb_im) per cell."""
    lib = _load()
    a = _atoms(atoms7)
    t0s = _c(t0s, np.uint32)
    taus = _c(taus, np.uint32)
    out = np.empty((t0s.size, 7), dtype=np.float64)
    rc = lib.tcwo_cell_sums_f64(a.ctypes.data_as(_f32p), a.shape[0], int(TAtom), int(t0_data),
                                int(window), t0s.ctypes.data_as(_u32p),
                                taus.ctypes.data_as(_u32p), t0s.size, out.ctypes.data_as(_f64p))
    if rc != 0:
        raise ValueError(f"oracle cell_sums_f64 failed with status {rc}")
    return out


def exp_map_f64_realtau(atoms7, TAtom, t0_data, t0s, taus, nthreads=0):
    """FP64 exponential-window map on a real-valued tau grid (differentiable variant)."""
    lib = _load()
    a = _atoms(atoms7)
    t0s = _c(t0s, np.uint32)
    taus = _c(taus, np.float64)
    F = np.empty((len(t0s), len(taus)), dtype=np.float64)
    rc = lib.tcwo_exp_map_f64_realtau(a.ctypes.data_as(_f32p), a.shape[0], int(TAtom),
                                      int(t0_data), t0s.ctypes.data_as(_u32p), len(t0s),
                                      taus.ctypes.data_as(_f64p), len(taus),
                                      F.ctypes.data_as(_f64p), int(nthreads))
    if rc != 0:
        raise ValueError(f"oracle exp_map_f64_realtau failed with status {rc}")
    return F


def idx_start(t0, t0_data, TAtom, numAtoms):
    return int(_load().tcwo_idx_start(t0, t0_data, TAtom, numAtoms))


def idx_end(t1, t0_data, TAtom, numAtoms):
    return int(_load().tcwo_idx_end(t1, t0_data, TAtom, numAtoms))


# ------------------------------------------------------------------ post-processing
# Restatements of pyTransientFstatMap's reductions (tcw_fstat_map_funcs.py:186-287).


def max_argmax(F):
    """maxF and the first-occurrence row-major flat argmax (tcw:810-813)."""
    k = int(np.argmax(F))
    return F.reshape(-1)[k], k


def lnBtSG(F):
    """ln(70 / (N_t0 N_tau)) + maxF + ln sum exp(F - maxF)  (tcw:196-217)."""
    maxF = F.max()
    s = np.sum(np.exp(-(maxF - F)))
    logBhat = maxF + np.log(s)  # in the map's precision, as the reference does
    return np.log(70.0 / np.prod(F.shape)) + logBhat


def t0_max_posterior_idx(F):
    """Index of the max of sum_n exp(F - maxF) over rows (tcw:247-251)."""
    return int(np.argmax(np.sum(np.exp(-(F.max() - F)), axis=1)))


def tau_max_posterior_idx(F):
    """Index of the max of sum_m exp(F - maxF) over columns (tcw:282-286)."""
    return int(np.argmax(np.sum(np.exp(-(F.max() - F)), axis=0)))


def softmax2F(F, T=0.1):
    """T * ln sum exp(2F / T) in FP64 (the smooth max of 2F at temperature T)."""
    z = 2.0 * np.asarray(F, dtype=np.float64) / T
    zmax = z.max()
    return T * (zmax + np.log(np.sum(np.exp(z - zmax))))


# ------------------------------------------------------------------ reference kernels


class RefKernels:
    """The reference's pycuda kernels compiled for the host (oracle/_ref)."""

    def __init__(self, path=REF_LIB_PATH):
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        lib = ctypes.CDLL(path)
        u = ctypes.c_uint
        sig = [_f32p, u, u, u, u, u, u, u, u, u, _f32p, ctypes.c_int]
        lib.ref_rect_uniform.argtypes = sig
        lib.ref_exp_uniform.argtypes = sig
        lib.ref_cells.argtypes = [_f32p, u, u, u, ctypes.c_int, _u32p, _u32p, ctypes.c_long,
                                  _f32p, ctypes.c_int]
        self.lib = lib

    @staticmethod
    def available(path=REF_LIB_PATH):
        return os.path.exists(path)

    def map_uniform(self, window, atoms7, TAtom, t0_data, t0, dt0, tau, dtau, N_t0, N_tau,
                    nthreads=0):
        a = _atoms(atoms7)
        out = np.empty((N_t0, N_tau), dtype=np.float32)
        fn = self.lib.ref_rect_uniform if window == WIN_RECT else self.lib.ref_exp_uniform
        fn(a.ctypes.data_as(_f32p), a.shape[0], TAtom, t0_data, t0, dt0, tau, dtau, N_t0,
           N_tau, out.ctypes.data_as(_f32p), int(nthreads))
        return out

    def map_grid(self, window, atoms7, TAtom, t0_data, t0s, taus, nthreads=0):
        t0s = _c(t0s, np.uint32)
        taus = _c(taus, np.uint32)
        T0, TA = np.meshgrid(t0s, taus, indexing="ij")
        return self.cells(window, atoms7, TAtom, t0_data, T0.ravel(), TA.ravel(),
                          nthreads).reshape(len(t0s), len(taus))

    def cells(self, window, atoms7, TAtom, t0_data, t0s, taus, nthreads=0):
        a = _atoms(atoms7)
        t0s = _c(t0s, np.uint32)
        taus = _c(taus, np.uint32)
        out = np.empty(t0s.size, dtype=np.float32)
        self.lib.ref_cells(a.ctypes.data_as(_f32p), a.shape[0], TAtom, t0_data, window,
                           t0s.ctypes.data_as(_u32p), taus.ctypes.data_as(_u32p), t0s.size,
                           out.ctypes.data_as(_f32p), int(nthreads))
        return out
