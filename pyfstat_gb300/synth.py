"""Seeded synthetic F-statistic atoms for the benchmark and tests.

The transient map has no public dataset; inputs are synthetic atoms with the
shapes and value distributions of the benchmark workloads:

* timestamps ``t_k = T0 + k*Tsft`` (+ a per-detector offset), T0 = 700000000
  as in PyFstat's tests/test_tcw_fstat_map_funcs.py:36, Tsft = 1800 s;
* antenna terms ``a = 0.4 + 0.3 cos(2 pi t / 86164 s + phi_a)``,
  ``b = 0.3 sin(2 pi t / 86164 s + phi_b)``, ``phi ~ U(0, 2 pi)``;
* ``a2 = a^2, b2 = b^2, ab = a b`` (FP32);
  ``Fa = sqrt(a2/2) (x + i y)``, ``Fb = sqrt(b2/2) (u + i v)`` (complex64),
  ``x, y, u, v ~ N(0, 1)`` from ``numpy.random.default_rng(seed)``;
* an injected signal adds ``amp*a`` to ``x`` and ``amp*b`` to ``u`` (amp = 3)
  for SFTs 200..320 inclusive;
* optional random gaps (SFTs dropped).

Draw order per detector: ``phi_a, phi_b = rng.uniform(0, 2 pi, 2)``, then
``x, y, u, v = rng.standard_normal((4, nsft))``, then the gap mask
``rng.random(nsft)``.  Detector X of a multi-detector set uses
``default_rng([seed, X])`` and a timestamp offset of ``X * Tsft / 3`` s, so
that floor and nearest-bin merging agree.
"""

import numpy as np

from .atoms import FstatAtomVector, MultiFstatAtomVector, merge_multi_atoms_binned
from .window import uniform_grid

T0_DEFAULT = 700000000
TSFT_DEFAULT = 1800
SIDEREAL_DAY = 86164.0
INJECT_RANGE = (200, 320)


def detector_atoms(rng, nsft, Tsft=TSFT_DEFAULT, T0=T0_DEFAULT, offset=0, amp=3.0,
                   inject=INJECT_RANGE, gap_frac=0.0):
    """One detector's atoms as an :class:`FstatAtomVector`."""
    k = np.arange(nsft, dtype=np.int64)
    t = T0 + int(offset) + k * int(Tsft)
    phi_a, phi_b = rng.uniform(0.0, 2.0 * np.pi, 2)
    om = 2.0 * np.pi / SIDEREAL_DAY
    a = 0.4 + 0.3 * np.cos(om * t + phi_a)
    b = 0.3 * np.sin(om * t + phi_b)
    x, y, u, v = rng.standard_normal((4, nsft))
    if inject is not None and amp:
        s, e = inject
        sl = slice(s, min(e + 1, nsft))
        x[sl] += amp * a[sl]
        u[sl] += amp * b[sl]
    a2 = (a * a).astype(np.float32)
    b2 = (b * b).astype(np.float32)
    ab = (a * b).astype(np.float32)
    Fa = (np.sqrt(a2.astype(np.float64) / 2.0) * (x + 1j * y)).astype(np.complex64)
    Fb = (np.sqrt(b2.astype(np.float64) / 2.0) * (u + 1j * v)).astype(np.complex64)
    keep = np.ones(nsft, dtype=bool)
    if gap_frac > 0:
        keep = rng.random(nsft) >= gap_frac
        keep[0] = True  # keep the span fixed
        keep[-1] = True
    return FstatAtomVector(t[keep].astype(np.uint32), a2[keep], b2[keep], ab[keep], Fa[keep],
                           Fb[keep], Tsft)


def multi_detector_atoms(seed, nsft, ndet=1, Tsft=TSFT_DEFAULT, T0=T0_DEFAULT, amp=3.0,
                         inject=INJECT_RANGE, gap_frac=0.0):
    """A :class:`MultiFstatAtomVector` of ``ndet`` detectors.

    A single detector uses ``default_rng(seed)`` (the single-template 480-SFT generator);
    detector X of several uses ``default_rng([seed, X])``.
    """
    vecs = []
    for X in range(ndet):
        rng = np.random.default_rng(seed if ndet == 1 else [seed, X])
        vecs.append(detector_atoms(rng, nsft, Tsft=Tsft, T0=T0, offset=(X * Tsft) // 3,
                                   amp=amp, inject=inject, gap_frac=gap_frac))
    return MultiFstatAtomVector(vecs)


def merged_atoms(seed, nsft, ndet=1, Tsft=TSFT_DEFAULT, T0=T0_DEFAULT, amp=3.0,
                 inject=INJECT_RANGE, gap_frac=0.0):
    """(t0_data, (NBins, 7) float32) after the binned merge."""
    multi = multi_detector_atoms(seed, nsft, ndet, Tsft, T0, amp, inject, gap_frac)
    return merge_multi_atoms_binned(multi, Tsft)


# ----------------------------------------------------------------- named workloads


def plain_rect_case(seed=0, nsft=480, Tsft=TSFT_DEFAULT):
    """Rectangular map, 1 template, 1 detector, 480 SFTs; t0 grid 480 x Tsft,
    tau = Tsft * (1..480)."""
    t0_data, atoms = merged_atoms(seed, nsft, 1, Tsft)
    t0s = uniform_grid(t0_data, Tsft, nsft)
    taus = uniform_grid(Tsft, Tsft, nsft)
    return dict(window=1, atoms=atoms, TAtom=Tsft, t0_data=t0_data, t0s=t0s, taus=taus,
                t0=t0_data, dt0=Tsft, tau=Tsft, dtau=Tsft)


def log_tau_grid(Tsft, max_sfts, n):
    """``n`` log-spaced taus in [Tsft, max_sfts*Tsft], rounded to integer s."""
    return np.round(Tsft * np.logspace(0.0, np.log10(max_sfts), n)).astype(np.uint32)


def plain_exp_case(seed=0, nsft=480, Tsft=TSFT_DEFAULT):
    """Exponential map, 1 template, 2 detectors merged (2 x 480 atoms with
    interleaved timestamps -> 480 bins); 480 t0 x 512 log-spaced taus in
    [1, 1440] SFT lengths."""
    t0_data, atoms = merged_atoms(seed, nsft, 2, Tsft)
    t0s = uniform_grid(t0_data, Tsft, nsft)
    taus = log_tau_grid(Tsft, 3 * nsft, 512)
    return dict(window=2, atoms=atoms, TAtom=Tsft, t0_data=t0_data, t0s=t0s, taus=taus)


def batched_templates(n_templates=4096, seed=12345, nsft_range=(200, 4000),
                      gap_range=(0.0, 0.3), grid_range=(256, 2048), Tsft=TSFT_DEFAULT,
                      ndet=1):
    """Batched workload: per-template SFT count, gap fraction, window and grid.

    Template k uses atoms seed ``seed + k`` (the single-detector generator with a random
    phase per template); even k rectangular, odd k exponential.  Grids are
    uniform windowRange grids covering the data span:
    ``dt0 = max(1, span // N_t0)``, ``tau = Tsft + n * dtau`` with
    ``dtau = max(1, (span - Tsft) // (N_tau - 1))``.
    Returns a list of dicts (atoms matrix, TAtom, t0_data, window, grid).
    """
    meta = np.random.default_rng(seed)
    nsfts = meta.integers(nsft_range[0], nsft_range[1] + 1, n_templates)
    gaps = meta.uniform(gap_range[0], gap_range[1], n_templates)
    nt0 = meta.integers(grid_range[0], grid_range[1] + 1, n_templates)
    ntau = meta.integers(grid_range[0], grid_range[1] + 1, n_templates)
    out = []
    for k in range(n_templates):
        t0_data, atoms = merged_atoms(seed + k, int(nsfts[k]), ndet, Tsft,
                                      gap_frac=float(gaps[k]))
        span = atoms.shape[0] * Tsft
        N_t0 = int(nt0[k])
        N_tau = int(ntau[k])
        dt0 = max(1, span // N_t0)
        dtau = max(1, (span - Tsft) // max(1, N_tau - 1))
        out.append(dict(window=1 if k % 2 == 0 else 2, atoms=atoms, TAtom=Tsft,
                        t0_data=t0_data, t0=t0_data, dt0=dt0, tau=Tsft, dtau=dtau,
                        N_t0=N_t0, N_tau=N_tau))
    return out


def precision_templates(n_templates=64, seed=777, nsft=17532, ndet=2, gap_frac=0.05,
                        N_t0=8192, N_tau=4096, Tsft=TSFT_DEFAULT):
    """Precision-at-scale workload: ``n_templates`` exponential-window
    templates of one year of data (17532 SFTs of 1800 s per detector, two
    detectors merged, 5 % of SFTs dropped as gaps), each on an 8192 t0 x 4096
    tau grid covering the span: ``dt0 = span // N_t0``,
    ``tau = Tsft + n * dtau`` with ``dtau = (span - Tsft) // (N_tau - 1)``.
    Template k uses atoms seed ``seed + k``."""
    out = []
    for k in range(n_templates):
        t0_data, atoms = merged_atoms(seed + k, nsft, ndet, Tsft, gap_frac=gap_frac)
        span = atoms.shape[0] * Tsft
        out.append(dict(window=2, atoms=atoms, TAtom=Tsft, t0_data=t0_data, t0=t0_data,
                        dt0=max(1, span // N_t0), tau=Tsft,
                        dtau=max(1, (span - Tsft) // max(1, N_tau - 1)), N_t0=N_t0,
                        N_tau=N_tau))
    return out
