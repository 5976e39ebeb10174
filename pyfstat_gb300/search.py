"""Batched transient searches over many Doppler (frequency-evolution) points.

The reference evaluates a grid point by point: ``TransientGridSearch.run``
loops over the points and ``_get_single_cand_results`` computes one
transient F-stat map per point (pyfstat/grid_based_searches.py:1080-1200),
each through ``call_compute_transient_fstat_map`` (with a kernel launch, a
full map download and host reductions per point); transient BSGL computes
one more map per detector and reads one cell of each
(pyfstat/core.py:1503-1546); the semi-coherent search computes per-segment
2F as a rectangular map with one t0 row per segment and tauBand = 0
(core.py:2000-2019, :2240-2289).

Here all points (and all detectors of all points) of a batch are templates
of one batched plan, run in one persistent launch (or one per chunk of
points when the maps to be written would exceed a device-memory budget):

* :class:`TransientGridBatch` -- maxTwoF, t0_ML, tau_ML, and with ``BtSG``
  lnBtSG, t0_MP, tau_MP (posteriors from the written maps on the GPU), and
  with ``BSGL`` the per-detector 2F at the multi-detector argmax
  (``twoF<IFO>atMaxTwoF``) and log10BSGL;  ``twoF`` (all data, one
  rectangular cell, the window type 'none' of tcw:742-749) is computed for
  every point;
* :func:`semicoherent_twoF` -- per-segment 2F of every point (and every
  detector), their sums, and the semi-coherent log10BSGL.

The BSGL combination restates the line-robust statistic of Keitel, Prix,
Papa, Leaci and Siddiqi, Phys. Rev. D 89, 064023 (2014), which lalpulsar's
``ComputeBSGL`` implements (called at core.py:1409, :1542, :2276 with the
setup of core.py:793-819):

    ln B_S/GL = F + ln(1 + oLG) - ln( exp(F*0) + sum_X oLGX exp(F^X) ),

F = twoF / 2, F^X = twoFX / 2, oLG = sum_X oLGX, with the exact log-sum-exp
(``useLogCorrection``) or only its largest term; log10BSGL = ln B / ln 10.
lalpulsar is not available to check the constants; pass ``bsgl=`` to use
another combination (e.g. lalpulsar's own when it is installed).
"""

import math

import numpy as np

from . import _lib
from .atoms import MultiFstatAtomVector, merge_multi_atoms_binned
from .batched import TransientMapBatch
from .window import (TRANSIENT_EXPONENTIAL, TRANSIENT_NONE, TRANSIENT_RECTANGULAR,
                     grid_sizes, uniform_grid)


# ------------------------------------------------------------------ BSGL


def fstar0_semicoherent(nsegs, p_val_threshold=1e-6):
    """F*0 of a semi-coherent search of ``nsegs`` segments: the value where
    the chi^2_{4 nsegs} tail probability reaches ``p_val_threshold`` on the
    grid linspace(0, 1000, 10000) (core.py:797-808); 15 for one segment."""
    import scipy.special

    if nsegs <= 1:
        return 15.0
    grid = np.linspace(0, 1000, 10000)
    p = scipy.special.gammaincc(2 * nsegs, grid)
    f = grid[np.argmin(np.abs(p - p_val_threshold))]
    if f == grid[-1]:
        raise ValueError("Max Fstar0 exceeded")
    return float(f)


def compute_log10BSGL(twoF, twoFX, Fstar0=15.0, oLGX=None, use_log_correction=True):
    """log10 B_S/GL of (arrays of) multi-detector 2F and per-detector 2F^X
    (last axis: detectors); uniform line-to-Gaussian odds oLGX = 1/N_det by
    default, as core.py:811-812."""
    twoF = np.asarray(twoF, dtype=np.float64)
    twoFX = np.asarray(twoFX, dtype=np.float64)
    ndet = twoFX.shape[-1]
    oLGX = np.full(ndet, 1.0 / ndet) if oLGX is None else np.asarray(oLGX, dtype=np.float64)
    oLG = float(np.sum(oLGX))
    with np.errstate(divide="ignore"):
        terms = np.concatenate([np.broadcast_to(Fstar0, twoF.shape + (1,)),
                                0.5 * twoFX + np.log(oLGX)], axis=-1)
    top = np.max(terms, axis=-1)
    if use_log_correction:
        den = top + np.log(np.sum(np.exp(terms - top[..., None]), axis=-1))
    else:
        den = top
    return (0.5 * twoF + math.log1p(oLG) - den) / math.log(10.0)


# ------------------------------------------------------------------ points


def _as_multi(point):
    """A MultiFstatAtomVector-like object from a point given as one, as a list
    of per-detector FstatAtomVectors, or as one FstatAtomVector."""
    if hasattr(point, "data") and hasattr(point, "length") and not hasattr(point, "TAtom"):
        return point
    if isinstance(point, (list, tuple)):
        return MultiFstatAtomVector(list(point))
    return MultiFstatAtomVector([point])


def _merged(multi):
    TAtom = int(multi.data[0].TAtom)
    t0_data, A = merge_multi_atoms_binned(multi, TAtom)
    return TAtom, t0_data, A


def _grid_for(windowRange, TAtom, t0_data, numAtoms):
    """(window type, t0s, taus, (t0, dt0, t0Band, tau, dtau, tauBand)) of the
    map of one point; window type 'none' is one rectangular cell over all
    data (tcw:742-749)."""
    wtype = int(windowRange.type)
    if wtype == TRANSIENT_NONE:
        t0, dt0, t0Band, tau, dtau, tauBand = t0_data, TAtom, 0, numAtoms * TAtom, TAtom, 0
        wtype = TRANSIENT_RECTANGULAR
    elif wtype in (TRANSIENT_RECTANGULAR, TRANSIENT_EXPONENTIAL):
        t0, dt0, t0Band = int(windowRange.t0), int(windowRange.dt0), int(windowRange.t0Band)
        tau, dtau, tauBand = int(windowRange.tau), int(windowRange.dtau), int(windowRange.tauBand)
    else:
        raise ValueError(f"Unknown window-type ({wtype}) passed as input. Allowed are [0,2].")

    class _R:
        pass

    r = _R()
    r.t0, r.dt0, r.t0Band, r.tau, r.dtau, r.tauBand = t0, dt0, t0Band, tau, dtau, tauBand
    N_t0, N_tau = grid_sizes(r)
    return wtype, uniform_grid(t0, dt0, N_t0), uniform_grid(tau, dtau, N_tau), r


def chunks_by_cells(cells, budget_cells):
    """Consecutive index ranges [a, b) whose summed cells stay within
    ``budget_cells`` (a range holds at least one item)."""
    out, a, acc = [], 0, 0
    for i, c in enumerate(cells):
        if i > a and acc + c > budget_cells:
            out.append((a, i))
            a, acc = i, 0
        acc += c
    if a < len(cells):
        out.append((a, len(cells)))
    return out


def _device_maps_run(templates, flags, device, tile_config=None, handle=None):
    """Results and device maps (torch) of one batched plan over ``templates``."""
    import torch

    batch = TransientMapBatch(templates, device=device, tile_config=tile_config, flags=flags,
                              handle=handle)
    dev = torch.device("cuda", device)
    h = batch.handle
    h.set_stream(torch.cuda.current_stream(dev).cuda_stream or 0x1)
    d_atoms = torch.from_numpy(batch.atoms).to(dev)
    d_res = torch.zeros(batch.n_templates * 5, dtype=torch.float64, device=dev)
    d_maps = torch.empty(max(1, batch.n_cells), dtype=torch.float32, device=dev)
    batch.plan.run_maps(d_atoms, d_res, d_maps, use_graph=False)
    torch.cuda.synchronize(dev)
    res = d_res.cpu().numpy().view(_lib.RESULT_DTYPE).copy()
    cells = batch.desc["N_t0"].astype(np.int64) * batch.desc["N_tau"]
    offs = np.concatenate([[0], np.cumsum(cells)[:-1]])
    batch.close()
    return res, d_maps, offs


class TransientGridBatch:
    """Transient statistics of many Doppler points in one batched launch.

    Parameters
    ----------
    points: list of per-point atoms -- each a MultiFstatAtomVector-like
        object (``.data[X]`` per detector, each with ``TAtom``), a list of
        per-detector FstatAtomVectors, or a single FstatAtomVector.
    windowRange: transientWindowRange-like (type, t0, t0Band, dt0, tau,
        tauBand, dtau), shared by all points.
    BtSG: also lnBtSG and the t0 / tau max-posterior estimates.
    BSGL: also per-detector 2F at the argmax and log10BSGL.
    detector_names: IFO names for the ``twoF<IFO>atMaxTwoF`` columns.
    map_budget_bytes: device memory for the maps written per launch (BtSG
        posteriors, BSGL cells); points are processed in consecutive chunks
        within it (default 8 GiB).
    """

    def __init__(self, points, windowRange, BtSG=False, BSGL=False, detector_names=None,
                 device=0, tile_config=None, Fstar0=15.0, oLGX=None, use_log_correction=True,
                 bsgl=None, flags=_lib.TCW_FLAG_LNBTSG, map_budget_bytes=8 << 30):
        self.multis = [_as_multi(p) for p in points]
        self.windowRange = windowRange
        self.BtSG = bool(BtSG)
        self.BSGL = bool(BSGL)
        ndet = self.multis[0].length if self.multis else 0
        self.detector_names = (list(detector_names) if detector_names is not None
                               else [f"X{k}" for k in range(ndet)])
        self.device = device
        self.tile_config = tile_config
        self.flags = int(flags)
        # device memory for written maps per launch (posteriors, BSGL cells):
        # larger searches run as several batched launches
        self.map_budget_cells = max(1, int(map_budget_bytes) // 4)
        self.bsgl = bsgl or (lambda twoF, twoFX: compute_log10BSGL(
            twoF, twoFX, Fstar0=Fstar0, oLGX=oLGX, use_log_correction=use_log_correction))
        # provenance of the output columns: the maps, their reductions and the
        # per-detector 2F follow the reference's algorithm and are checked
        # against the FP64 oracle; the BSGL combination is a restatement of
        # the published statistic that lalpulsar's ComputeBSGL implements,
        # which is absent here, so its constants are not pinned to it
        self.metadata = {"bsgl_parity": "unpinned" if bsgl is None else "caller-supplied",
                         "bsgl": "Keitel et al. PRD 89 064023 (2014), Fstar0=%g" % Fstar0,
                         "maps_parity": "FP64 oracle, 2F rel err <= 1e-5"}

    def output_keys(self):
        keys = ["twoF", "maxTwoF", "t0_ML", "tau_ML"]
        if self.BSGL:
            keys += [f"twoF{ifo}atMaxTwoF" for ifo in self.detector_names] + ["log10BSGL"]
        if self.BtSG:
            keys += ["lnBtSG", "t0_MP", "tau_MP"]
        return keys

    def run(self):
        """Structured array of one row per point with :meth:`output_keys`."""
        npts = len(self.multis)
        out = np.zeros(npts, dtype=[(k, np.float64) for k in self.output_keys()])
        if npts == 0:
            return out
        merged = [_merged(m) for m in self.multis]
        grids = [_grid_for(self.windowRange, TA, t0d, A.shape[0]) for TA, t0d, A in merged]
        maps_tmpl, full_tmpl = [], []
        for (TA, t0d, A), (w, t0s, taus, _) in zip(merged, grids):
            maps_tmpl.append(dict(atoms=A, TAtom=TA, t0_data=t0d, window=w, t0s=t0s, taus=taus))
            full_tmpl.append(dict(atoms=A, TAtom=TA, t0_data=t0d, window=TRANSIENT_RECTANGULAR,
                                  t0s=np.array([t0d], np.uint32),
                                  taus=np.array([A.shape[0] * TA], np.uint32)))
        # all-data 2F (one cell per point) and the transient maps: one plan per
        # chunk of points (one chunk unless the written maps would exceed the
        # memory budget)
        flags = self.flags | (_lib.TCW_FLAG_POSTERIORS if self.BtSG else 0)
        rmap = np.zeros(npts, dtype=_lib.RESULT_DTYPE)
        rfull = np.zeros(npts, dtype=_lib.RESULT_DTYPE)
        cells = [int(g[1].size) * int(g[2].size) + 1 for g in grids]
        budget = self.map_budget_cells if self.BtSG else float("inf")
        for a, b in chunks_by_cells(cells, budget):
            tmpl = maps_tmpl[a:b] + full_tmpl[a:b]
            if self.BtSG:
                res, _, _ = _device_maps_run(tmpl, flags, self.device, self.tile_config)
            else:
                batch = TransientMapBatch(tmpl, device=self.device, tile_config=self.tile_config,
                                          flags=flags)
                res = batch.run()
                batch.close()
            rmap[a:b], rfull[a:b] = res[:b - a], res[b - a:]
        out["twoF"] = 2.0 * rfull["maxF"].astype(np.float64)
        maxTwoF = 2.0 * rmap["maxF"].astype(np.float64)
        out["maxTwoF"] = np.where(np.isnan(maxTwoF), 0.0, maxTwoF)
        ms, ns = [], []
        for k, (w, t0s, taus, r) in enumerate(grids):
            m, n = divmod(int(rmap["argmax"][k]), taus.size)
            ms.append(m)
            ns.append(n)
            out["t0_ML"][k] = r.t0 + m * r.dt0
            out["tau_ML"][k] = r.tau + n * r.dtau
            if self.BtSG:
                out["lnBtSG"][k] = rmap["lnBtSG"][k]
                out["t0_MP"][k] = r.t0 + (int(rmap["t0_mp_idx"][k]) + 0.5) * (r.t0Band / t0s.size)
                out["tau_MP"][k] = r.tau + (int(rmap["tau_mp_idx"][k]) + 0.5) * (
                    r.tauBand / taus.size)
        if self.BSGL:
            twoFX = self._per_detector_at(merged, grids, ms, ns)
            for x, ifo in enumerate(self.detector_names):
                out[f"twoF{ifo}atMaxTwoF"] = twoFX[:, x]
            out["log10BSGL"] = self.bsgl(out["maxTwoF"], twoFX)
        return out

    def _per_detector_at(self, merged, grids, ms, ns):
        """2F^X at the multi-detector argmax cell of every point: one-row
        templates (t0 of the argmax row, taus up to the argmax column) of each
        detector's own binned atoms, so that the rectangular running sums
        along tau are those of the full single-detector map (core.py:1531-1541)."""
        import torch

        tmpl, where = [], []
        for k, multi in enumerate(self.multis):
            w, t0s, taus, _ = grids[k]
            for x in range(multi.length):
                TA, t0d, A = _merged(MultiFstatAtomVector([multi.data[x]]))
                tmpl.append(dict(atoms=A, TAtom=TA, t0_data=t0d, window=w,
                                 t0s=t0s[ms[k]:ms[k] + 1].copy(), taus=taus[:ns[k] + 1].copy()))
                where.append((k, x, ns[k]))
        twoFX = np.zeros((len(self.multis), len(self.detector_names)))
        for a, b in chunks_by_cells([n + 1 for _, _, n in where], self.map_budget_cells):
            _, d_maps, offs = _device_maps_run(tmpl[a:b], self.flags, self.device,
                                               self.tile_config)
            idx = np.array([offs[j - a] + where[j][2] for j in range(a, b)], dtype=np.int64)
            vals = d_maps[torch.from_numpy(idx).to(d_maps.device)].cpu().numpy()
            for j in range(a, b):
                k, x, _ = where[j]
                twoFX[k, x] = 2.0 * float(vals[j - a])
        return twoFX


def semicoherent_twoF(points, tboundaries, BSGL=False, detector_names=None, device=0,
                      record_segments=False, Fstar0=None, oLGX=None, bsgl=None):
    """Semi-coherent 2F of many points from per-segment rectangular windows.

    Segment k covers [tboundaries[0] + k Tcoh, + Tcoh) with
    Tcoh = (tboundaries[-1] - tboundaries[0]) / nsegs, i.e. the window range
    t0 = tboundaries[0], t0Band = tboundaries[-1] - tboundaries[0] - Tcoh,
    dt0 = tau = Tcoh, tauBand = 0 (core.py:2000-2019).  Returns a dict with
    ``twoF`` (sum of per-segment 2F, NaNs counted as 0, core.py:2192-2198),
    with ``BSGL`` also ``twoFX`` (points x detectors) and ``log10BSGL``
    (F*0 from :func:`fstar0_semicoherent`), and with ``record_segments`` the
    per-segment values."""
    tb = np.asarray(tboundaries, dtype=np.int64)
    nsegs = tb.size - 1
    if nsegs < 1:
        raise ValueError("need at least two segment boundaries")
    Tcoh = int((tb[-1] - tb[0]) // nsegs)
    t0s = uniform_grid(int(tb[0]), Tcoh, nsegs)
    taus = np.array([Tcoh], dtype=np.uint32)
    multis = [_as_multi(p) for p in points]
    npts = len(multis)
    ndet = multis[0].length if npts else 0
    tmpl = []
    for m in multis:
        TA, t0d, A = _merged(m)
        tmpl.append(dict(atoms=A, TAtom=TA, t0_data=t0d, window=TRANSIENT_RECTANGULAR, t0s=t0s,
                         taus=taus))
        if BSGL:
            for x in range(m.length):
                TA, t0d, A = _merged(MultiFstatAtomVector([m.data[x]]))
                tmpl.append(dict(atoms=A, TAtom=TA, t0_data=t0d, window=TRANSIENT_RECTANGULAR,
                                 t0s=t0s, taus=taus))
    b = TransientMapBatch(tmpl, device=device)
    _, maps = b.plan.run_maps_host(b.atoms)
    b.close()
    per = 2.0 * maps.reshape(len(tmpl), nsegs).astype(np.float64)
    per = np.nan_to_num(per, nan=0.0)
    stride = 1 + (ndet if BSGL else 0)
    seg = per[0::stride]
    out = {"twoF": seg.sum(axis=1)}
    if record_segments:
        out["twoF_per_segment"] = seg
    if BSGL:
        segX = np.stack([per[1 + x::stride] for x in range(ndet)], axis=1)
        out["twoFX"] = segX.sum(axis=2)
        if record_segments:
            out["twoFX_per_segment"] = segX
        f0 = fstar0_semicoherent(nsegs) if Fstar0 is None else Fstar0
        comb = bsgl or (lambda a, bx: compute_log10BSGL(a, bx, Fstar0=f0, oLGX=oLGX))
        l10 = comb(out["twoF"], out["twoFX"])
        out["log10BSGL"] = np.where(np.isnan(l10), 0.0, l10)
        if detector_names is not None:
            out["detector_names"] = list(detector_names)
        # the BSGL combination restates the published statistic; lalpulsar's
        # ComputeBSGL is absent here, so its constants are not pinned to it
        out["bsgl_parity"] = "unpinned" if bsgl is None else "caller-supplied"
    return out
