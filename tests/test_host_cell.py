"""The device cell arithmetic (pyfstat_gb300/csrc/tcw_cell.h), built for the
host, against the FP64 oracle and the reference's golden maps -- no GPU.

This checks the algorithm the kernels run (quantised compensated prefixes,
two-pointer exponential recurrences, error-free determinant, u32 index
semantics); the GPU tests check the kernels themselves.
"""

import ctypes

import numpy as np
import pytest

from _helpers import REL_TOL, golden_case, golden_cases, hc_map, rel_err
from pyfstat_gb300 import synth

P = ctypes.c_void_p


def test_fastdiv_matches_integer_division(hostcell):
    rng = np.random.default_rng(0)
    xs = np.concatenate([np.arange(0, 200000, dtype=np.uint64),
                         rng.integers(0, 2 ** 32, 500000, dtype=np.uint64),
                         2 ** 32 - 1 - np.arange(20000, dtype=np.uint64)]).astype(np.uint32)
    for d in [1, 2, 3, 5, 7, 60, 900, 1799, 1800, 1801, 3600, 65535, 65536, 86400, 2 ** 31 - 1,
              2 ** 31, 2 ** 31 + 1, 2 ** 32 - 1]:
        q = np.empty_like(xs)
        hostcell.hc_fastdiv(ctypes.c_uint32(d), xs.ctypes.data_as(P), ctypes.c_uint64(xs.size),
                            q.ctypes.data_as(P))
        assert np.array_equal(q, xs // np.uint32(d)), d


def test_rect_walk_reuse_equals_per_cell(hostcell):
    """The rect map kernel's walk -- a column whose window end equals the
    previous column's reuses its F, a 32-column chunk inside every row's
    clamped run repeats it -- gives bit-identical maps to computing every
    cell: random gappy atoms, TAtom other than 1800, t0 grids starting
    before the data (u32 wrap of the reference's end index), tau steps
    below TAtom (shared ends), taus past the data (clamped runs) and
    shuffled tau grids (no run test passes)."""
    from _helpers import P

    checked = runs = 0
    for seed in range(40):
        rng = np.random.default_rng(900 + seed)
        TAtom = 1800 if seed % 3 else int(rng.integers(2, 5000))
        t0_data, A = synth.merged_atoms(seed, int(rng.integers(5, 300)), int(rng.integers(1, 3)),
                                        Tsft=TAtom, gap_frac=float(rng.uniform(0, 0.4)))
        n = A.shape[0]
        nt0, ntau = int(rng.integers(1, 100)), int(rng.integers(1, 150))
        t0 = int(t0_data + rng.integers(-3 * TAtom if seed % 5 == 0 else 0, n * TAtom))
        t0s = (t0 + np.arange(nt0) * int(rng.integers(1, 2 * TAtom))).astype(np.uint32)
        step = int(rng.integers(0, 2 * TAtom)) if seed % 2 else int(rng.integers(1, TAtom // 2 + 2))
        taus = (int(rng.integers(1, 2 * TAtom)) + np.arange(ntau) * step).astype(np.uint32)
        if seed % 7 == 3:
            taus = rng.permutation(taus)
        out = []
        for fn in ("hc_rect_walk_map", "hc_rect_map"):
            F = np.empty((nt0, ntau), np.float32)
            args = [A.ctypes.data_as(P), ctypes.c_uint32(n), ctypes.c_uint32(TAtom),
                    ctypes.c_uint32(t0_data), t0s.ctypes.data_as(P), ctypes.c_uint32(nt0),
                    taus.ctypes.data_as(P), ctypes.c_uint32(ntau)]
            if fn == "hc_rect_map":
                ok = np.empty((nt0, ntau), np.uint8)
                getattr(hostcell, fn)(*args, ctypes.c_int(1), F.ctypes.data_as(P),
                                      ok.ctypes.data_as(P))
            else:
                getattr(hostcell, fn)(*args, F.ctypes.data_as(P))
            out.append(F)
        assert np.array_equal(out[0].view(np.uint32), out[1].view(np.uint32)), seed
        checked += out[0].size
        runs += int(np.sum(out[1][:, 1:] == out[1][:, :-1]))
    assert checked > 100000 and runs > 10000


def test_exp_window_bounds_match_reference_loop(hostcell, oracle):
    """[lo, hi] = atoms with t0 <= t_i <= t0 + 3 tau inside [i_t0, i_t1] (Exp.cu:80-90)."""
    rng = np.random.default_rng(1)
    n, TAtom, t0_data = 50, 1800, 700000000
    t0s = (t0_data + rng.integers(-20000, 100000, 4000)).astype(np.uint32)
    taus = rng.integers(1, 40000, 4000).astype(np.uint32)
    lohi = np.empty((4000, 2), np.int32)
    hostcell.hc_exp_window(ctypes.c_uint32(n), ctypes.c_uint32(TAtom), ctypes.c_uint32(t0_data),
                           t0s.ctypes.data_as(P), taus.ctypes.data_as(P), ctypes.c_uint64(4000),
                           lohi.ctypes.data_as(P))
    for k in range(4000):
        t0, tau = int(t0s[k]), int(taus[k])
        t1 = (t0 + 3 * tau) & 0xFFFFFFFF
        a = oracle.idx_start(t0, t0_data, TAtom, n)
        b = oracle.idx_end(t1, t0_data, TAtom, n)
        idx = [i for i in range(a, b + 1) if t0 <= t0_data + i * TAtom <= t1]
        if idx:
            assert (lohi[k, 0], lohi[k, 1]) == (idx[0], idx[-1]), k
        else:
            assert lohi[k, 0] > lohi[k, 1], k


@pytest.mark.parametrize("case", ["rect", "exp"])
def test_workload_maps_within_tolerance_of_fp64(hostcell, oracle, case):
    c = synth.plain_rect_case() if case == "rect" else synth.plain_exp_case()
    F64, cond = oracle.map_f64(c["atoms"], c["TAtom"], c["t0_data"], c["window"], c["t0s"],
                               c["taus"], with_cond=True)
    F, _ = hc_map(hostcell, c)
    rel, nband = rel_err(F, F64, cond)
    assert rel.max() < REL_TOL
    assert np.argmax(F) == np.argmax(F64)
    assert nband <= 2


def test_uncompensated_variant_is_worse(hostcell, oracle):
    """The plain-FP32 variant (precision report) misses the bar on the exp workload."""
    c = synth.plain_exp_case()
    F64, cond = oracle.map_f64(c["atoms"], c["TAtom"], c["t0_data"], 2, c["t0s"], c["taus"],
                               with_cond=True)
    F, _ = hc_map(hostcell, c, comp=False)
    rel, _ = rel_err(F, F64, cond)
    assert rel.max() > REL_TOL


@pytest.mark.parametrize("row_chunk", [0, 1, 5, 33])
def test_exp_row_chunks_agree(hostcell, oracle, row_chunk):
    t0_data, A = synth.merged_atoms(9, 200, 2, gap_frac=0.15)
    c = dict(window=2, atoms=A, TAtom=1800, t0_data=t0_data,
             t0s=(t0_data + np.arange(120) * 1500 - 700).astype(np.uint32),
             taus=np.round(1800 * np.logspace(0, 2.4, 70)).astype(np.uint32))
    F64, cond = oracle.map_f64(A, 1800, t0_data, 2, c["t0s"], c["taus"], with_cond=True)
    F, _ = hc_map(hostcell, c, row_chunk=row_chunk)
    rel, _ = rel_err(F, F64, cond)
    assert rel.max() < REL_TOL


def test_golden_edge_cases(hostcell, oracle, golden):
    """Every golden case (tiny grids, clamps, u32 wrap, off-grid steps, gaps,
    the window-'none' cell, the reference test geometry): within tolerance of
    FP64, same F = 2 fallback cells as the reference away from the threshold."""
    for name in golden_cases(golden):
        c = golden_case(golden, name)
        F64, cond = oracle.map_f64(c["atoms"], c["TAtom"], c["t0_data"], c["window"], c["t0s"],
                                   c["taus"], with_cond=True)
        F, _ = hc_map(hostcell, c)
        rel, _ = rel_err(F, F64, cond)
        assert rel.max() < REL_TOL, (name, rel.max())
        Fref = c["F"] if "F" in c else None
        if Fref is not None:
            clear = (cond > 1.01e4) | ~np.isfinite(cond)
            assert np.all(F[clear] == 2.0) and np.all(Fref[clear] == 2.0), name


def test_random_gappy_grids(hostcell, oracle):
    """Random grids (off the atom grid, starting before the data, dtau = 0
    included) over atoms with long runs of zero (gap) bins."""
    for seed in range(16):
        rng = np.random.default_rng(seed)
        t0_data, A = synth.merged_atoms(seed, int(rng.integers(20, 300)), int(rng.integers(1, 3)),
                                        gap_frac=float(rng.uniform(0, 0.5)))
        A = A.copy()
        for _ in range(int(rng.integers(0, 4))):
            s = int(rng.integers(0, A.shape[0]))
            A[s:s + int(rng.integers(1, 40))] = 0
        for window in (1, 2):
            nt0, ntau = int(rng.integers(1, 60)), int(rng.integers(1, 60))
            t0 = int(t0_data + rng.integers(-5000, 3000))
            t0s = (t0 + np.arange(nt0) * int(rng.integers(1, 4000))).astype(np.uint32)
            taus = (int(rng.integers(1, 5000)) + np.arange(ntau) * int(rng.integers(0, 8000))
                    ).astype(np.uint32)
            c = dict(window=window, atoms=A, TAtom=1800, t0_data=t0_data, t0s=t0s, taus=taus)
            F64, cond = oracle.map_f64(A, 1800, t0_data, window, t0s, taus, with_cond=True)
            F, _ = hc_map(hostcell, c, row_chunk=int(rng.integers(0, 10)))
            rel, _ = rel_err(F, F64, cond)
            assert rel.max() < REL_TOL, (seed, window, rel.max())
            port = oracle.rect_map_f32 if window == 1 else oracle.exp_map_f32
            Fr = port(A, 1800, t0_data, t0s, taus)
            clear = (cond > 1.01e4) | ~np.isfinite(cond)
            assert np.all(F[clear] == 2.0) and np.all(Fr[clear] == 2.0), (seed, window)


@pytest.mark.parametrize("dt0", [667, 1800, 4861])
def test_exp_long_columns_many_removals(hostcell, oracle, dt0):
    """Long exponential columns: the sliding window sum adds and removes
    thousands of atoms per column (short taus remove one or more atoms on
    almost every row, long ones clamp at the data end) and stays within the
    tolerance of FP64 on every cell."""
    t0_data, A = synth.merged_atoms(31, 1500, 2, gap_frac=0.1)
    span = A.shape[0] * 1800
    nt0 = min(700, span // dt0)
    t0s = (t0_data - 900 + np.arange(nt0) * dt0).astype(np.uint32)
    taus = np.unique(np.round(1800 * np.logspace(0, np.log10(span / 1800), 40))).astype(np.uint32)
    c = dict(window=2, atoms=A, TAtom=1800, t0_data=t0_data, t0s=t0s, taus=taus)
    F64, cond = oracle.map_f64(A, 1800, t0_data, 2, t0s, taus, with_cond=True)
    F, _ = hc_map(hostcell, c)
    rel, _ = rel_err(F, F64, cond)
    assert rel.max() < REL_TOL, rel.max()


def test_exp_row_table_column_equals_generic_column(hostcell):
    """The row-table column (tabulated window starts and first non-zero atoms,
    division-free window ends; what the GPU runs on regular rows) gives
    bit-identical maps to the generic column on the same row chunks: random
    grids (regular ones and ones starting before the data, which fall back to
    the generic arithmetic), TAtom other than 1800, non-uniform t0 grids."""
    from _helpers import P

    checked = 0
    for seed in range(30):
        rng = np.random.default_rng(500 + seed)
        TAtom = 1800 if seed % 3 else int(rng.integers(2, 5000))
        t0_data, A = synth.merged_atoms(seed, int(rng.integers(5, 250)), int(rng.integers(1, 3)),
                                        Tsft=TAtom, gap_frac=float(rng.uniform(0, 0.4)))
        A = A.copy()
        for _ in range(int(rng.integers(0, 3))):
            s = int(rng.integers(0, A.shape[0]))
            A[s:s + int(rng.integers(1, 30))] = 0
        nt0, ntau = int(rng.integers(1, 150)), int(rng.integers(1, 60))
        if seed % 4 == 0:  # non-uniform, sorted t0 grid inside the data
            t0s = np.sort(rng.integers(t0_data, t0_data + A.shape[0] * TAtom, nt0))
        else:
            t0 = int(t0_data + rng.integers(-3 * TAtom if seed % 5 == 0 else 0, 2 * TAtom))
            t0s = t0 + np.arange(nt0) * int(rng.integers(1, 3 * TAtom))
        t0s = t0s.astype(np.uint32)
        taus = (int(rng.integers(1, 4 * TAtom)) + np.arange(ntau) *
                int(rng.integers(0, 5 * TAtom))).astype(np.uint32)
        row_chunk = int(rng.integers(0, 40))
        out = []
        for comp in (1, 2):
            F = np.empty((nt0, ntau), np.float32)
            hostcell.hc_exp_map(A.ctypes.data_as(P), ctypes.c_uint32(A.shape[0]),
                                ctypes.c_uint32(TAtom), ctypes.c_uint32(t0_data),
                                t0s.ctypes.data_as(P), ctypes.c_uint32(nt0),
                                taus.ctypes.data_as(P), ctypes.c_uint32(ntau), ctypes.c_int(comp),
                                ctypes.c_uint32(row_chunk), F.ctypes.data_as(P),
                                None)
            out.append(F)
        assert np.array_equal(out[0].view(np.uint32), out[1].view(np.uint32)), seed
        checked += out[0].size
    assert checked > 50000


def test_exp_chunk_paths_long_columns(hostcell):
    """The row-table walk's chunk paths over several 128-row tables per
    column: clamped chunks (long taus), steady rows after the first window
    with an atom and after the first window with data (zero atoms at the end
    of the data, so the first windows of a column hold none), rows sharing a
    window start (t0 steps below TAtom), and t0 grids that fall back in
    places (no steady rows there) -- bit-identical to the generic column."""
    from _helpers import P

    checked = 0
    for seed in range(12):
        rng = np.random.default_rng(4400 + seed)
        TAtom = 1800 if seed % 2 else int(rng.integers(600, 3000))
        t0_data, A = synth.merged_atoms(seed, int(rng.integers(150, 400)), 2, Tsft=TAtom,
                                        gap_frac=0.2)
        A = A.copy()
        A[-int(rng.integers(1, 40)):] = 0  # no data at the end
        n = A.shape[0]
        nt0 = int(rng.integers(300, 700))
        span = n * TAtom
        step = max(1, int(span / nt0 * rng.uniform(0.3, 1.2)))
        t0s = t0_data + np.arange(nt0, dtype=np.int64) * step
        if seed % 3 == 0:  # a stretch that falls back by a few steps
            k = int(rng.integers(50, nt0 - 50))
            t0s[k:k + 20] -= 3 * step
        t0s = np.clip(t0s, t0_data, t0_data + span).astype(np.uint32)
        taus = np.unique(np.round(TAtom * np.logspace(0, np.log10(3 * n), 24))).astype(np.uint32)
        out = []
        for comp in (1, 2):
            F = np.empty((nt0, taus.size), np.float32)
            hostcell.hc_exp_map(A.ctypes.data_as(P), ctypes.c_uint32(n), ctypes.c_uint32(TAtom),
                                ctypes.c_uint32(t0_data), t0s.ctypes.data_as(P),
                                ctypes.c_uint32(nt0), taus.ctypes.data_as(P),
                                ctypes.c_uint32(taus.size), ctypes.c_int(comp), ctypes.c_uint32(0),
                                F.ctypes.data_as(P), None)
            out.append(F)
        assert np.array_equal(out[0].view(np.uint32), out[1].view(np.uint32)), seed
        checked += out[0].size
    assert checked > 50000


def test_exp_real_tau_window_sums_match_fp64(hostcell):
    """The forward pass of the differentiable statistics: double-word window
    sums on a real tau grid (window ends from the split 3 tau + TAtom/2 =
    Q' TAtom + R'', R'' real) against FP64 sums over the reference's window
    (t0 <= t_i <= t0 + 3 tau, i <= floor((t0 + 3 tau - t0_data + TAtom/2) /
    TAtom) - 1; the FP64 torch reference's mask), on grids with real taus
    and, for every data window, relative to the sum of |terms|."""
    import _torch_ref as R
    from _helpers import P

    for seed in range(6):
        rng = np.random.default_rng(900 + seed)
        t0_data, A = synth.merged_atoms(seed, int(rng.integers(20, 160)), 2,
                                        gap_frac=float(rng.uniform(0, 0.3)))
        nt0, ntau = int(rng.integers(3, 40)), int(rng.integers(2, 30))
        t0s = (t0_data + int(rng.integers(0, 900)) +
               np.arange(nt0) * int(rng.integers(300, 4000))).astype(np.uint32)
        tau_min = float(rng.uniform(500, 5000))
        taus = tau_min + np.arange(ntau) * float(rng.uniform(10, 3000))
        W = np.empty((nt0, ntau, 7), np.float64)
        ok = np.empty((nt0, ntau), np.uint8)
        assert hostcell.hc_exp_real_sums(
            A.ctypes.data_as(P), ctypes.c_uint32(A.shape[0]), ctypes.c_uint32(1800),
            ctypes.c_uint32(t0_data), t0s.ctypes.data_as(P), ctypes.c_uint32(nt0),
            taus.ctypes.data_as(P), ctypes.c_uint32(ntau), W.ctypes.data_as(P),
            ok.ctypes.data_as(P)) == 0
        mask = R.window_mask(A.shape[0], 1800, t0_data, t0s, taus, window=2)
        t_i = t0_data + np.arange(A.shape[0]) * 1800.0
        dt = np.clip(t_i[None, None, :] - t0s.astype(np.float64)[:, None, None], 0, None)
        w = np.where(mask, np.exp(-dt / taus[None, :, None]), 0.0)
        for c in range(7):
            wk = w * w if c < 3 else w
            # the double-word sums leave out the window's common factor
            # e^(-k (t_lo - t0) / tau): compare after scaling to the first atom
            ref = np.einsum("mni,i->mn", wk, A[:, c].astype(np.float64))
            absref = np.einsum("mni,i->mn", wk, np.abs(A[:, c]).astype(np.float64))
            lo = np.argmax(mask, axis=2)
            t_lo = t0_data + lo * 1800.0
            k = 2.0 if c < 3 else 1.0
            scale = np.exp(-k * (t_lo - t0s.astype(np.float64)[:, None]) / taus[None, :])
            has = mask.any(axis=2) & (ok == 1)
            got = W[:, :, c] * scale
            err = np.abs(got - ref)[has] / np.maximum(absref[has], 1e-300)
            assert err.size == 0 or err.max() < 1e-11, (seed, c, err.max())
        # a window without data in the reference mask (or only zero atoms) is not valid
        nodata = ~(mask & ((A[:, 0] != 0) | (A[:, 1] != 0))[None, None, :]).any(axis=2)
        assert np.all(ok[nodata] == 0), seed
        assert np.all(ok[~nodata] == 1), seed


def _sum_forms(hostcell, x, Eh, El, rh, rl):
    from _helpers import P

    arrs = [np.ascontiguousarray(a, np.float32) for a in (x, Eh, El, rh, rl)]
    out = np.empty((arrs[0].size, 8), np.float32)
    hostcell.hc_sum_forms(*[a.ctypes.data_as(P) for a in arrs], ctypes.c_uint64(arrs[0].size),
                          out.ctypes.data_as(P))
    return out


def _split(v):
    h = v.astype(np.float32)
    return h, (v - h.astype(np.float64)).astype(np.float32)


def test_entering_sum_forms(hostcell):
    """The exponential columns' entering step W = x + r W: the magnitude-ordered
    Fast2Sum forms (A, B, C) give TwoSum's double-word bit for bit, and the
    plain Fast2Sum form (Fa, Fb) misses at most 2^-24 |x| of the exact value,
    and nothing when the decayed sum outweighs x."""
    from fractions import Fraction

    rng = np.random.default_rng(31)
    n = 20000
    r = np.exp(-rng.uniform(1e-4, 3.0, n))
    rh, rl = _split(r)
    # window sums from much smaller to much larger than the entering term
    mag = 10.0 ** rng.uniform(-3, 4, n)
    Ev = mag * rng.choice([-1.0, 1.0], n) * rng.uniform(0.5, 1.0, n)
    Eh, El = _split(Ev)
    x = (rng.uniform(-1, 1, n) * 10.0 ** rng.uniform(-2, 1, n)).astype(np.float32)
    out = _sum_forms(hostcell, x, Eh, El, rh, rl)
    assert np.array_equal(out[:, 0:2].view(np.uint32), out[:, 2:4].view(np.uint32))
    # non-negative operands (the (A,B) pair)
    xn, En = np.abs(x), np.abs(Ev)
    Enh, Enl = _split(En)
    outn = _sum_forms(hostcell, xn, Enh, Enl, rh, rl)
    assert np.array_equal(outn[:, 0:2].view(np.uint32), outn[:, 4:6].view(np.uint32))
    # plain Fast2Sum: compare hi + lo with TwoSum's (both as exact rationals)
    worst = 0.0
    for i in range(0, n, 7):
        two = Fraction(float(out[i, 0])) + Fraction(float(out[i, 1]))
        fast = Fraction(float(out[i, 6])) + Fraction(float(out[i, 7]))
        miss = abs(float(fast - two))
        p = abs(float(rh[i]) * float(Eh[i]))
        if p >= 2.0 * abs(float(x[i])):
            assert miss == 0.0, i
        worst = max(worst, miss / max(abs(float(x[i])), 1e-30))
    assert worst <= 2.0 ** -24 * 1.01, worst
