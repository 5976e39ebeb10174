"""GB300-native transient-CW F-statistic maps: a 'b200' version for PyFstat.

``pyfstat_gb300.tcw_fstat_map_funcs`` mirrors PyFstat's module of the same
name (version table, feature probing, dispatcher, ``pyTransientFstatMap``)
and adds the ``'b200'`` version; ``pyfstat_gb300.batched`` runs thousands of
templates in one persistent launch.  The compute is the CUDA library
``libtcw_b200.so`` (C ABI in include/tcw_b200.h); there is no CPU fallback.
"""

from .window import (TRANSIENT_EXPONENTIAL, TRANSIENT_LAST, TRANSIENT_NONE,  # noqa: F401
                     TRANSIENT_RECTANGULAR, transientWindowRange_t)

__all__ = ["tcw_fstat_map_funcs", "batched", "atoms", "window", "synth",
           "transientWindowRange_t", "TRANSIENT_NONE", "TRANSIENT_RECTANGULAR",
           "TRANSIENT_EXPONENTIAL", "TRANSIENT_LAST"]
