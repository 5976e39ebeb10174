"""Transient window ranges: the ``lalpulsar.transientWindowRange_t`` equivalent.

Fields and enum values follow lalpulsar's struct as PyFstat sets it
(core.py:821-891, tests/test_tcw_fstat_map_funcs.py:40-50): ``type`` in
{TRANSIENT_NONE, TRANSIENT_RECTANGULAR, TRANSIENT_EXPONENTIAL} and the UINT4
seconds ``t0, t0Band, dt0, tau, tauBand, dtau``.  Any object with those
attributes (a real lalpulsar struct included) is accepted by the b200 path.
"""

import numpy as np

TRANSIENT_NONE = 0
TRANSIENT_RECTANGULAR = 1
TRANSIENT_EXPONENTIAL = 2
TRANSIENT_LAST = 3

_U32_MAX = 0xFFFFFFFF


class transientWindowRange_t:
    """Uniform (t0, tau) grid of a transient search, all times in integer s."""

    def __init__(self, type=TRANSIENT_NONE, t0=0, t0Band=0, dt0=0, tau=0, tauBand=0, dtau=0):
        self.type = type
        self.t0 = t0
        self.t0Band = t0Band
        self.dt0 = dt0
        self.tau = tau
        self.tauBand = tauBand
        self.dtau = dtau

    def __repr__(self):
        return ("transientWindowRange_t(type={}, t0={}, t0Band={}, dt0={}, tau={}, "
                "tauBand={}, dtau={})".format(self.type, self.t0, self.t0Band, self.dt0,
                                              self.tau, self.tauBand, self.dtau))


def grid_sizes(windowRange):
    """N_t0Range, N_tauRange = floor(Band / d) + 1 (tcw_fstat_map_funcs.py:775-780)."""
    N_t0 = int(np.floor(1.0 * windowRange.t0Band / windowRange.dt0) + 1)
    N_tau = int(np.floor(1.0 * windowRange.tauBand / windowRange.dtau) + 1)
    return N_t0, N_tau


def uniform_grid(start, step, n):
    """u32 values start + k*step (mod 2**32, as the reference kernels compute)."""
    k = np.arange(n, dtype=np.uint64)
    return ((np.uint64(start) + k * np.uint64(step)) & np.uint64(_U32_MAX)).astype(np.uint32)


def expand_window_range(windowRange):
    """Explicit (t0s, taus) u32 arrays of a uniform windowRange grid."""
    N_t0, N_tau = grid_sizes(windowRange)
    return (uniform_grid(windowRange.t0, windowRange.dt0, N_t0),
            uniform_grid(windowRange.tau, windowRange.dtau, N_tau))
