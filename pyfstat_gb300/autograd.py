"""Differentiable transient statistics of exponential- and rectangular-window maps.

For each template, the tau grid is continuous:
tau_n = tau_min + n (tau_max - tau_min) / (N_tau - 1).  The forward pass
returns

* ``lnBtSG = ln(70 / (N_t0 N_tau)) + logsumexp_mn F_mn``, the marginalised
  transient Bayes factor (as in pyfstat/tcw_fstat_map_funcs.py:196-217);
* ``softmax2F = T logsumexp_mn (2 F_mn / T)``, a smooth maximum of 2F that
  tends to max 2F as the temperature T -> 0 (T = 0.1 by default).

:func:`transient_stats` is a ``torch.autograd.Function``: gradients flow to
the atoms (columns a2, b2, ab, Fa_re, Fa_im, Fb_re, Fb_im) and to tau_min /
tau_max.  The backward pass recomputes the window sums on the GPU (no map is
stored).  Window boundaries change in steps with tau and are not
differentiated; only the window weights are -- so rectangular windows, whose
sums do not depend on tau between boundaries, have zero tau gradients.
"""

import numpy as np
import torch

from . import _lib
from .window import uniform_grid


class DiffBatch:
    """Geometry of a batch of templates for differentiation.

    ``templates``: dicts with ``atoms`` ((numAtoms, 7) float32 binned atoms,
    used for row offsets and as the default input), ``TAtom``, ``t0_data``,
    ``N_tau``, a non-decreasing t0 grid (``t0s`` or ``t0, dt0, N_t0``) and
    optionally ``window`` (2 exponential, the default; 1 rectangular).
    """

    def __init__(self, templates, device=0, temperature=0.1, handle=None):
        self.temperature = float(temperature)
        n = len(templates)
        self.desc = np.zeros(n, dtype=_lib.DIFF_DESC_DTYPE)
        t0_parts, rows = [], 0
        g0 = 0
        for k, t in enumerate(templates):
            t0s = (np.ascontiguousarray(t["t0s"], np.uint32) if "t0s" in t
                   else uniform_grid(t["t0"], t["dt0"], t["N_t0"]))
            na = int(np.asarray(t["atoms"]).shape[0])
            self.desc[k] = (rows, g0, na, int(t["TAtom"]), int(t["t0_data"]), t0s.shape[0],
                            int(t["N_tau"]), int(t.get("window", _lib.TCW_WINDOW_EXP)),
                            float(t.get("tau_min", 1.0)), float(t.get("tau_max", 1.0)))
            t0_parts.append(t0s)
            rows += na
            g0 += t0s.shape[0]
        self.t0s = np.ascontiguousarray(np.concatenate(t0_parts), dtype=np.uint32)
        self.n_rows = rows
        self.n_templates = n
        self.atoms = np.ascontiguousarray(
            np.concatenate([np.asarray(t["atoms"], np.float32) for t in templates]))
        self.handle = handle if handle is not None else _lib.Handle(device)

    def _desc_with(self, tau_min, tau_max):
        d = self.desc.copy()
        d["tau_min"] = np.asarray(tau_min, dtype=np.float64)
        d["tau_max"] = np.asarray(tau_max, dtype=np.float64)
        return d

    def _stream(self):
        # Run on torch's current stream so that torch reads the outputs in
        # order.  Torch reports its default stream as handle 0, which the
        # library takes to mean "the handle's own stream"; 0x1 names the
        # legacy default stream (cudaStreamLegacy) explicitly.
        s = torch.cuda.current_stream().cuda_stream
        self.handle.set_stream(s if s else 0x1)

    def forward_raw(self, d_atoms, tau_min, tau_max):
        """(lnBtSG, softmax2F) as FP64 device tensors; d_atoms float32 (rows, 7)."""
        dev = d_atoms.device
        d = self._desc_with(tau_min, tau_max)
        lnB = torch.empty(self.n_templates, dtype=torch.float64, device=dev)
        soft = torch.empty(self.n_templates, dtype=torch.float64, device=dev)
        self._stream()
        _lib.check(_lib.load().tcw_map_forward(
            self.handle.ptr, d.ctypes.data, self.n_templates, d_atoms.data_ptr(),
            self.t0s.ctypes.data, self.t0s.shape[0], self.temperature, lnB.data_ptr(),
            soft.data_ptr()), self.handle.ptr)
        return lnB, soft

    def backward_raw(self, d_atoms, tau_min, tau_max, lnB, soft, g_lnB, g_soft):
        """(dL/datoms (rows, 7) FP64, dL/dtau (n, 2) FP64) on the device."""
        dev = d_atoms.device
        d = self._desc_with(tau_min, tau_max)
        ga = torch.empty((self.n_rows, 7), dtype=torch.float64, device=dev)
        gt = torch.empty((self.n_templates, 2), dtype=torch.float64, device=dev)
        g_lnB = g_lnB.to(torch.float64).contiguous()
        g_soft = g_soft.to(torch.float64).contiguous()
        self._stream()
        _lib.check(_lib.load().tcw_map_backward(
            self.handle.ptr, d.ctypes.data, self.n_templates, d_atoms.data_ptr(),
            self.t0s.ctypes.data, self.t0s.shape[0], self.temperature, lnB.data_ptr(),
            soft.data_ptr(), g_lnB.data_ptr(), g_soft.data_ptr(), ga.data_ptr(), self.n_rows,
            gt.data_ptr()), self.handle.ptr)
        return ga, gt


# the exponential-window name of the same class
ExpDiffBatch = DiffBatch


class _TransientStats(torch.autograd.Function):
    @staticmethod
    def forward(ctx, atoms, tau_min, tau_max, batch):
        a32 = atoms.detach().to(torch.float32).contiguous()
        tmin = tau_min.detach().cpu().numpy().astype(np.float64)
        tmax = tau_max.detach().cpu().numpy().astype(np.float64)
        lnB, soft = batch.forward_raw(a32, tmin, tmax)
        ctx.batch = batch
        ctx.tau = (tmin, tmax)
        ctx.save_for_backward(a32, lnB, soft)
        ctx.atoms_dtype = atoms.dtype
        return lnB, soft

    @staticmethod
    def backward(ctx, g_lnB, g_soft):
        a32, lnB, soft = ctx.saved_tensors
        if g_lnB is None:
            g_lnB = torch.zeros_like(lnB)
        if g_soft is None:
            g_soft = torch.zeros_like(soft)
        ga, gt = ctx.batch.backward_raw(a32, *ctx.tau, lnB, soft, g_lnB, g_soft)
        return ga.to(ctx.atoms_dtype), gt[:, 0].cpu(), gt[:, 1].cpu(), None


def transient_stats(atoms, tau_min, tau_max, batch):
    """(lnBtSG, softmax2F) per template, differentiable in atoms, tau_min, tau_max.

    ``atoms``: (rows, 7) CUDA tensor (float32 or float64; computed from its
    float32 values), ``tau_min`` / ``tau_max``: CPU float64 tensors of one
    value per template, ``batch``: :class:`DiffBatch`.
    """
    return _TransientStats.apply(atoms, tau_min, tau_max, batch)
