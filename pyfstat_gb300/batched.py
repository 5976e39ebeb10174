"""Batched transient F-statistic maps: many templates in one persistent launch.

A transient grid search evaluates one map per Doppler template
(grid_based_searches.py:1186-1189 calls get_det_stat per point, which calls
call_compute_transient_fstat_map once each).  :class:`TransientMapBatch`
takes all templates at once: the geometry (atom counts, windows, grids) is
fixed in a plan; each run takes the concatenated atoms and returns, per
template, maxF (2F = 2 maxF), the flat argmax and lnBtSG (FP64), without
writing any map.  A run is one CUDA graph of five launches on two branches:
(repack -> persistent exponential-window map kernel) and (prefix ->
persistent rectangular-window map kernel), joined by a finalize kernel
(plus the posterior kernels when maps are written).
"""

import numpy as np

from . import _lib
from .window import uniform_grid


def template_grids(t):
    """(t0s, taus) u32 arrays of a template dict (explicit or uniform grid)."""
    if "t0s" in t and "taus" in t:
        return (np.ascontiguousarray(t["t0s"], np.uint32),
                np.ascontiguousarray(t["taus"], np.uint32))
    return (uniform_grid(t["t0"], t["dt0"], t["N_t0"]),
            uniform_grid(t["tau"], t["dtau"], t["N_tau"]))


def pack_templates(templates):
    """Concatenate templates into (atoms (rows, 7) f32, desc, t0s, taus).

    Each template is a dict with ``atoms`` ((numAtoms, 7) float32 binned atoms
    starting at ``t0_data``), ``TAtom``, ``t0_data``, ``window`` (1 rect,
    2 exp) and either explicit ``t0s``/``taus`` or a uniform grid
    ``t0, dt0, N_t0, tau, dtau, N_tau``.
    """
    n = len(templates)
    desc = np.zeros(n, dtype=_lib.DESC_DTYPE)
    atoms_parts, t0_parts, tau_parts = [], [], []
    a_off = g0 = g1 = 0
    for k, t in enumerate(templates):
        A = np.ascontiguousarray(t["atoms"], np.float32)
        if A.ndim != 2 or A.shape[1] != 7:
            raise ValueError(f"template {k}: atoms must be (numAtoms, 7)")
        t0s, taus = template_grids(t)
        desc[k] = (a_off, g0, g1, A.shape[0], int(t["TAtom"]), int(t["t0_data"]),
                   int(t["window"]), t0s.shape[0], taus.shape[0])
        atoms_parts.append(A)
        t0_parts.append(t0s)
        tau_parts.append(taus)
        a_off += A.shape[0]
        g0 += t0s.shape[0]
        g1 += taus.shape[0]
    return (np.ascontiguousarray(np.concatenate(atoms_parts)), desc,
            np.concatenate(t0_parts).astype(np.uint32), np.concatenate(tau_parts).astype(np.uint32))


class TransientMapBatch:
    """Plan and run batched maps on one GPU.

    Parameters
    ----------
    templates: list of template dicts (see :func:`pack_templates`); their
        atoms become the default input of :meth:`run`.
    device: CUDA device ordinal.
    tile_config: dict of tile shapes (``rect_tn, rect_tm, exp_tn, exp_rows,
        blocks_per_sm``), or ``"auto"`` for the autotuner's choice.
    flags: ``_lib.TCW_FLAG_*`` precision flags.
    """

    def __init__(self, templates, device=0, tile_config=None, flags=_lib.TCW_FLAG_LNBTSG,
                 handle=None):
        self.atoms, self.desc, self.t0s, self.taus = pack_templates(templates)
        self.handle = handle if handle is not None else _lib.Handle(device)
        if tile_config == "auto":
            from .autotune import tune

            tile_config = tune(self.desc, self.t0s, self.taus, self.atoms, handle=self.handle,
                               flags=flags)
        self.plan = _lib.Plan(self.handle, self.desc, self.t0s, self.taus, tile_config, flags)
        self.n_templates = self.desc.shape[0]
        self.n_cells = self.plan.n_cells

    @property
    def tile_config(self):
        return self.plan.tile_config

    def run(self, atoms=None):
        """Host atoms in (default: the templates' own), per-template results out."""
        return self.plan.run_host(self.atoms if atoms is None else atoms)

    def run_pipelined(self, atom_batches):
        """One run per host atom array (same layout as the templates' own),
        pipelined: each upload overlaps the previous run's map kernels
        (pinned arrays make the copies asynchronous).  Returns the
        per-template results of every run, in order."""
        for a in atom_batches:
            self.plan.run_host_async(a)
        return self.plan.wait()

    def run_device(self, d_atoms, d_results, use_graph=True):
        """Device buffers (torch tensors or raw pointers); asynchronous on the
        handle's stream.  ``d_results`` holds n_templates records of 40 bytes."""
        self.plan.run(d_atoms, d_results, use_graph)

    @staticmethod
    def max2F(results):
        return 2.0 * results["maxF"].astype(np.float64)

    def close(self):
        self.plan.close()


def map_batched(templates, handle=None, device=0):
    """One-shot batched maps through the C ABI's ``tcw_map_batched`` (host
    buffers; no plan kept): (max2F float32, argmax int64, lnBtSG float64)
    per template."""
    import ctypes

    atoms, desc, t0s, taus = pack_templates(templates)
    h = handle if handle is not None else _lib.Handle(device)
    n = desc.shape[0]
    max2F = np.empty(n, dtype=np.float32)
    argmax = np.empty(n, dtype=np.int64)
    lnB = np.empty(n, dtype=np.float64)
    _lib.check(_lib.load().tcw_map_batched(
        h.ptr, desc.ctypes.data, n, t0s.ctypes.data, t0s.shape[0], taus.ctypes.data,
        taus.shape[0], atoms.ctypes.data, ctypes.POINTER(_lib.TcwTileConfig)(),
        max2F.ctypes.data, argmax.ctypes.data, lnB.ctypes.data), h.ptr)
    return max2F, argmax, lnB
