"""Transient-CW F-statistic maps with a GB300 'b200' version.

Mirrors the interface of PyFstat's ``pyfstat/tcw_fstat_map_funcs.py`` --
``fstatmap_versions`` (:320-327), ``init_transient_fstat_map_features``
(:361-492), ``call_compute_transient_fstat_map`` (:495-544) and the result
type ``pyTransientFstatMap`` (:50-317) -- with the same names, argument
meanings and error behaviour, and adds the key ``'b200'`` whose compute runs
in hand-written sm_103a CUDA through the C ABI of include/tcw_b200.h.

The 'lal' and 'pycuda' keys delegate to an installed PyFstat when one can be
imported (they need lalpulsar / pycuda); they are reported unavailable
otherwise, exactly as PyFstat's own feature probing does.
"""

import importlib
import logging
import os
from time import time

import numpy as np

from . import _lib
from .atoms import merge_multi_atoms_binned, vector_arrays
from .window import (TRANSIENT_EXPONENTIAL, TRANSIENT_LAST, TRANSIENT_NONE,
                     TRANSIENT_RECTANGULAR, expand_window_range, grid_sizes)

logger = logging.getLogger(__name__)


class pyTransientFstatMap:
    """F(t0, tau) map and its summaries (F, not 2F), as in PyFstat.

    Attributes: ``F_mn`` (float32 [N_t0, N_tau]), ``maxF``, ``t0_ML``,
    ``tau_ML``, ``lnBtSG``, ``t0_MP``, ``tau_MP`` (the last three NaN until
    computed).
    """

    def __init__(self, N_t0Range=None, N_tauRange=None, transientFstatMap_t=None,
                 from_file=None):
        if transientFstatMap_t and from_file:
            raise ValueError(
                "Please choose either a transientFstatMap_t or file to init from.")
        elif transientFstatMap_t:
            self._init_from_lalpulsar_type(transientFstatMap_t)
        elif from_file:
            self.read_from_file(from_file)
        else:
            if not N_t0Range or not N_tauRange:
                raise ValueError(
                    "Need either a transientFstatMap_t or a pair of (N_t0Range, N_tauRange)!.")
            self.F_mn = np.zeros((N_t0Range, N_tauRange), dtype=np.float32)
            # a negative start guarantees at least one update of the ML point
            self.maxF = float(-1.0)
            self.t0_ML = float(0.0)
            self.tau_ML = float(0.0)
        self.lnBtSG = np.nan
        self.t0_MP = np.nan
        self.tau_MP = np.nan

    def _init_from_lalpulsar_type(self, transientFstatMap_t):
        self.F_mn = transientFstatMap_t.F_mn.data
        self.maxF = transientFstatMap_t.maxF
        self.t0_ML = transientFstatMap_t.t0_ML
        self.tau_ML = transientFstatMap_t.tau_ML

    def read_from_file(self, file):
        """Load a ``t0 tau 2F`` text map (lalpulsar write_transientFstatMap_to_fp
        format; parsed natively, semantics of tcw:159-184)."""
        from .formats import read_map_text

        self.F_mn, self.t0_ML, self.tau_ML, self.maxF = read_map_text(file)

    def get_maxF_idx(self):
        """(m, n) of the first maximum of F_mn (row-major order)."""
        return np.unravel_index(np.argmax(self.F_mn), self.F_mn.shape)

    def get_lnBtSG(self):
        """ln of the transient Bayes factor B_tSG marginalised over (t0, tau).

        ln(70 / (N_t0 N_tau)) + maxF + ln sum exp(F - maxF)   (rhohMax = 1).
        """
        terms = np.exp(self.F_mn - self.maxF)
        self.lnBtSG = np.log(70.0 / np.prod(self.F_mn.shape)) + self.maxF + np.log(np.sum(terms))
        return self.lnBtSG

    def get_t0_max_posterior(self, windowRange):
        """Centre of the t0 bin maximising sum_n exp(F - maxF); bins of t0Band / N_t0."""
        marg = np.sum(np.exp(self.F_mn - self.maxF), axis=1)
        width = windowRange.t0Band / self.F_mn.shape[0]
        self.t0_MP = windowRange.t0 + (np.argmax(marg) + 0.5) * width
        return self.t0_MP

    def get_tau_max_posterior(self, windowRange):
        """Centre of the tau bin maximising sum_m exp(F - maxF); bins of tauBand / N_tau."""
        marg = np.sum(np.exp(self.F_mn - self.maxF), axis=0)
        width = windowRange.tauBand / self.F_mn.shape[1]
        self.tau_MP = windowRange.tau + (np.argmax(marg) + 0.5) * width
        return self.tau_MP

    def write_F_mn_to_file(self, tCWfile, windowRange, header=[]):
        """Write ``t0 tau 2F`` lines (lalpulsar write_transientFstatMap_to_fp
        format, tcw:289-317), formatted natively."""
        from .formats import write_map_text
        from .window import uniform_grid

        N_t0, N_tau = self.F_mn.shape
        t0s = uniform_grid(int(windowRange.t0), int(windowRange.dt0), N_t0)
        taus = uniform_grid(int(windowRange.tau), int(windowRange.dtau), N_tau)
        write_map_text(tCWfile, self.F_mn, t0s, taus, header)


# ------------------------------------------------------------------ versions


def _reference_function(name):
    mod = importlib.import_module("pyfstat.tcw_fstat_map_funcs")
    return getattr(mod, name)


fstatmap_versions = {
    "lal": lambda multiFstatAtoms, windowRange, BtSG: _reference_function(
        "lalpulsar_compute_transient_fstat_map")(multiFstatAtoms, windowRange, BtSG),
    "pycuda": lambda multiFstatAtoms, windowRange, BtSG: _reference_function(
        "pycuda_compute_transient_fstat_map")(multiFstatAtoms, windowRange, BtSG),
    "b200": lambda multiFstatAtoms, windowRange, BtSG: b200_compute_transient_fstat_map(
        multiFstatAtoms, windowRange, BtSG),
}
"""Name -> callable(multiFstatAtoms, windowRange, BtSG) of every supported version."""


def _optional_import(modulename):
    try:
        importlib.import_module(modulename)
        return True
    except ImportError:
        return False


# The library is compiled for sm_103a only (architecture-specific code: it
# loads on compute capability 10.3 and nowhere else).
B200_COMPUTE_CAPABILITY = (10, 3)


def _b200_available():
    """True iff the library loads and a device it can run on is present
    (the 'b200' row of _get_transient_fstat_map_features, tcw:351-358)."""
    try:
        n = _lib.device_count()
    except Exception as e:  # library missing or not loadable
        logger.debug(f"b200 library not available: {e}")
        return False
    for d in range(n):
        if tuple(_lib.device_info(d)["cc"]) == B200_COMPUTE_CAPABILITY:
            return True
    return False


def _get_transient_fstat_map_features():
    """Which versions can run here (the keys of ``fstatmap_versions``)."""
    features = {}
    features["lal"] = _optional_import("lal") and _optional_import("lalpulsar")
    features["pycuda"] = all(
        _optional_import(m) for m in ("pycuda", "pycuda.driver", "pycuda.gpuarray",
                                      "pycuda.tools", "pycuda.compiler"))
    features["b200"] = _b200_available()
    return features


class B200Context:
    """Device context of the 'b200' version: one library handle.

    ``detach()`` releases it (the same call PyFstat makes on a pycuda
    context, core.py:499-505 and tests/test_tcw_fstat_map_funcs.py:130-132).
    """

    def __init__(self, device):
        self.device = device
        self.handle = _lib.Handle(device)

    def detach(self):
        global _current_context
        if self.handle is not None:
            self.handle.close()
            self.handle = None
        if _current_context is self:
            _current_context = None

    pop = detach


_current_context = None


def _select_device(cudaDeviceName):
    n = _lib.device_count()
    names = [_lib.device_info(d)["name"].replace(" ", "-").replace("_", "-") for d in range(n)]
    for d, name in enumerate(names):
        logger.info("device {}: model: {}".format(d, name))
    if "CUDA_DEVICE" in os.environ:
        devnum = int(os.environ["CUDA_DEVICE"])
        if devnum >= n:
            raise RuntimeError(
                "Requested CUDA device number {} exceeds number of available devices!"
                " Please change through environment variable $CUDA_DEVICE.".format(devnum))
    else:
        devnum = 0
    if cudaDeviceName:
        matches = [d for d, name in enumerate(names) if cudaDeviceName in name]
        if not matches:
            raise RuntimeError('Requested CUDA device "{}" not found. Available devices: [{}]'
                               .format(cudaDeviceName, ",".join(names)))
        devnum = matches[0]
        if len(matches) > 1:
            logger.warning('Found {} CUDA devices matching name "{}". Choosing first one with '
                           'index {}.'.format(len(matches), cudaDeviceName, devnum))
        os.environ["CUDA_DEVICE"] = str(devnum)
    return devnum


def init_transient_fstat_map_features(feature="lal", cudaDeviceName=None):
    """Probe the versions and set up the requested one.

    Returns ``(features, gpu_context)``; ``gpu_context`` is a
    :class:`B200Context` for 'b200', PyFstat's pycuda context for 'pycuda',
    ``None`` for 'lal'.
    """
    global _current_context
    features = _get_transient_fstat_map_features()
    logger.debug("Got the following features for transient F-stat maps:")
    logger.debug(features)
    if feature == "b200":
        if not features["b200"]:
            raise RuntimeError(
                "b200 use was requested, but the CUDA library or a compute capability 10.3"
                " device is not available.")
        devnum = _select_device(cudaDeviceName)
        if _current_context is not None:
            _current_context.detach()
        _current_context = B200Context(devnum)
        gpu_context = _current_context
        _print_GPU_memory_MB("Available", devnum)
    elif feature == "pycuda":
        if not features["pycuda"]:
            raise RuntimeError("pycuda use was requested, but imports failed.")
        _, gpu_context = _reference_function("init_transient_fstat_map_features")(
            "pycuda", cudaDeviceName)
    elif feature == "lal":
        gpu_context = None
    else:
        raise ValueError(
            "Unknown transient F-stat map computation feature" f"'{feature}' requested.")
    return features, gpu_context


def call_compute_transient_fstat_map(version, features, multiFstatAtoms=None, windowRange=None,
                                     BtSG=False):
    """Compute a transient F-stat map with ``version``; returns (FstatMap, seconds)."""
    if version in fstatmap_versions:
        if features[version]:
            time0 = time()
            FstatMap = fstatmap_versions[version](multiFstatAtoms, windowRange, BtSG)
            timingFstatMap = time() - time0
        else:
            raise Exception(
                "Required module(s) for transient F-stat map"
                ' method "{}" not available!'.format(version))
    else:
        raise Exception('Transient F-stat map method "{}"' " not implemented!".format(version))
    return FstatMap, timingFstatMap


def reshape_FstatAtomsVector(atomsVector):
    """Dictionary of 1-D arrays per atom quantity (tcw_fstat_map_funcs.py:590-639)."""
    ts, mat, _ = vector_arrays(atomsVector)
    return {
        "timestamp": ts.astype(np.uint32),
        "a2_alpha": mat[:, 0].copy(),
        "b2_alpha": mat[:, 1].copy(),
        "ab_alpha": mat[:, 2].copy(),
        "Fa_alpha_re": mat[:, 3].copy(),
        "Fa_alpha_im": mat[:, 4].copy(),
        "Fb_alpha_re": mat[:, 5].copy(),
        "Fb_alpha_im": mat[:, 6].copy(),
    }


def _print_GPU_memory_MB(key, device=None):
    """Debug log of free / total device memory (tcw:648-653), at the same
    points of a map computation as the reference logs it."""
    if not logger.isEnabledFor(logging.DEBUG):
        return
    if device is None:
        device = _current_context.device if _current_context is not None else 0
    try:
        free, total = _lib.device_memory(device)
    except Exception as e:  # logging never fails a computation
        logger.debug(f"{key} GPU memory: unavailable ({e})")
        return
    logger.debug("{} GPU memory: {:.4f} / {:.4f} MB free".format(
        key, free / 2.0**20, total / 2.0**20))


def _context():
    global _current_context
    if _current_context is None or _current_context.handle is None:
        devnum = int(os.environ.get("CUDA_DEVICE", 0))
        _current_context = B200Context(devnum)
    return _current_context


def b200_compute_transient_fstat_map(multiFstatAtoms, windowRange, BtSG=False):
    """GB300 version of the transient F-stat map (drop-in for the pycuda one).

    Same flow as pycuda_compute_transient_fstat_map (tcw:656-834): binned
    merge of the detectors' atoms, window type 'none' as one rectangular cell
    over all data, grid sizes floor(Band/d)+1, the full F map, maxF and the ML
    point; with ``BtSG`` also lnBtSG (FP64, on the GPU) and the t0 / tau
    max-posterior estimates.
    """
    if windowRange.type >= TRANSIENT_LAST:
        raise ValueError("Unknown window-type ({}) passed as input. Allowed are [0,{}]."
                         .format(windowRange.type, TRANSIENT_LAST - 1))
    TAtom = int(multiFstatAtoms.data[0].TAtom)
    t0_data, atoms = merge_multi_atoms_binned(multiFstatAtoms, TAtom)
    numAtoms = atoms.shape[0]
    logger.debug("Transient F-stat map: t0_data={:d}, t1_data={:d}".format(
        t0_data, t0_data + (numAtoms - 1) * TAtom + TAtom))
    if windowRange.type == TRANSIENT_NONE:
        windowRange.type = TRANSIENT_RECTANGULAR
        windowRange.t0 = t0_data
        windowRange.t0Band = 0
        windowRange.dt0 = TAtom
        windowRange.tau = numAtoms * TAtom
        windowRange.tauBand = 0
        windowRange.dtau = TAtom
    N_t0, N_tau = grid_sizes(windowRange)
    FstatMap = pyTransientFstatMap(N_t0, N_tau)
    if windowRange.type not in (TRANSIENT_RECTANGULAR, TRANSIENT_EXPONENTIAL):
        raise ValueError("Invalid transient window type {} not in [{}, {}].".format(
            windowRange.type, TRANSIENT_NONE, TRANSIENT_LAST - 1))
    t0s, taus = expand_window_range(windowRange)
    flags = _lib.TCW_FLAG_LNBTSG | (_lib.TCW_FLAG_POSTERIORS if BtSG else 0)
    ctx = _context()
    _print_GPU_memory_MB("Initial", ctx.device)
    F, res = ctx.handle.map_plain_host(atoms, TAtom, t0_data, int(windowRange.type), t0s, taus,
                                       want_map=True, flags=flags)
    _print_GPU_memory_MB("Final", ctx.device)
    FstatMap.F_mn = F
    FstatMap.maxF = np.float32(res["maxF"])
    m, n = divmod(int(res["argmax"]), N_tau)
    FstatMap.t0_ML = windowRange.t0 + m * windowRange.dt0
    FstatMap.tau_ML = windowRange.tau + n * windowRange.dtau
    logger.debug("Done computing transient F-stat map. maxF={:.4f}, t0_ML={}, tau_ML={}".format(
        FstatMap.maxF, FstatMap.t0_ML, FstatMap.tau_ML))
    if BtSG:
        FstatMap.lnBtSG = float(res["lnBtSG"])
        FstatMap.t0_MP = windowRange.t0 + (int(res["t0_mp_idx"]) + 0.5) * (
            windowRange.t0Band / N_t0)
        FstatMap.tau_MP = windowRange.tau + (int(res["tau_mp_idx"]) + 0.5) * (
            windowRange.tauBand / N_tau)
        logger.debug(f"Also computed: lnBtSG={FstatMap.lnBtSG:.4f},"
                     f" t0_MP={FstatMap.t0_MP}, tau_MP={FstatMap.tau_MP}")
    return FstatMap
