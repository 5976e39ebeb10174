"""Differentiable exponential-window statistics on the GPU: values against the
FP64 oracle / torch reference, gradients against FP64 torch autograd and
central FP64 finite differences (bar: 1e-4 relative)."""

import time

import numpy as np
import pytest

import _torch_ref as R
from pyfstat_gb300 import synth

pytestmark = pytest.mark.gpu


# Window boundaries move with tau and are not differentiated, so the grids
# keep every window end t1 = t0 + 3 tau mid-way between atom-index
# boundaries (multiples of TAtom/2 = 900 s from t0_data): t0 = t0_data + 450
# + m 1800, 3 tau_min = 225 (mod 900), tau steps multiples of 300 s.  A
# perturbation of tau by ~1 s then moves no boundary.
def templates_small():
    out = []
    for k, (nsft, N_t0, N_tau, step) in enumerate([(60, 14, 11, 1500), (90, 30, 17, 2400),
                                                   (40, 9, 1, 300)]):
        t0_data, A = synth.merged_atoms(20 + k, nsft, 2, gap_frac=0.15)
        tau_min = 1875.0 + 900.0 * k
        out.append(dict(atoms=A, TAtom=1800, t0_data=t0_data,
                        t0s=(t0_data + 1800 * np.arange(N_t0) + 450).astype(np.uint32),
                        N_tau=N_tau, tau_min=tau_min, tau_max=tau_min + step * (N_tau - 1)))
    return out


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    return torch


def test_values_and_gradients_match_torch_fp64_reference(torch_cuda):
    torch = torch_cuda
    from pyfstat_gb300.autograd import ExpDiffBatch, transient_stats

    T = 0.1
    tl = templates_small()
    batch = ExpDiffBatch(tl, temperature=T)
    dev = torch.device("cuda:0")
    atoms = torch.from_numpy(batch.atoms).to(dev).requires_grad_(True)
    tmin = torch.tensor([t["tau_min"] for t in tl], dtype=torch.float64, requires_grad=True)
    tmax = torch.tensor([t["tau_max"] for t in tl], dtype=torch.float64, requires_grad=True)
    lnB, soft = transient_stats(atoms, tmin, tmax, batch)
    gl = torch.tensor([1.0, -0.5, 0.25], dtype=torch.float64, device=dev)
    gs = torch.tensor([0.3, 1.0, -2.0], dtype=torch.float64, device=dev)
    ((lnB * gl).sum() + (soft * gs).sum()).backward()
    ga = atoms.grad.double().cpu().numpy()
    lnB_v, soft_v = lnB.detach().cpu().numpy(), soft.detach().cpu().numpy()
    row = 0
    for k, t in enumerate(tl):
        x = torch.from_numpy(t["atoms"].astype(np.float64)).requires_grad_(True)
        a = torch.tensor(t["tau_min"], dtype=torch.float64, requires_grad=True)
        b = torch.tensor(t["tau_max"], dtype=torch.float64, requires_grad=True)
        rl, rs, _ = R.stats(x, 1800, t["t0_data"], t["t0s"], a, b, t["N_tau"], T)
        assert float(lnB_v[k]) == pytest.approx(float(rl.detach()), rel=1e-9)
        assert float(soft_v[k]) == pytest.approx(float(rs.detach()), rel=1e-9)
        (rl * float(gl[k]) + rs * float(gs[k])).backward()
        n = t["atoms"].shape[0]
        g_ref = x.grad.numpy()
        g_gpu = ga[row:row + n]
        scale = np.abs(g_ref).max()
        np.testing.assert_allclose(g_gpu, g_ref, rtol=1e-6, atol=1e-9 * scale)
        if t["N_tau"] > 1:
            assert float(tmax.grad[k]) == pytest.approx(float(b.grad), rel=1e-6, abs=1e-15)
        assert float(tmin.grad[k]) == pytest.approx(float(a.grad), rel=1e-6, abs=1e-15)
        row += n


def test_gradients_match_central_finite_differences(torch_cuda):
    torch = torch_cuda
    from pyfstat_gb300.autograd import ExpDiffBatch

    T = 0.1
    tl = templates_small()[:2]
    batch = ExpDiffBatch(tl, temperature=T)
    dev = torch.device("cuda:0")
    atoms = torch.from_numpy(batch.atoms).to(dev)
    tmin = np.array([t["tau_min"] for t in tl])
    tmax = np.array([t["tau_max"] for t in tl])
    lnB, soft = batch.forward_raw(atoms, tmin, tmax)
    one = torch.ones(2, dtype=torch.float64, device=dev)
    zero = torch.zeros(2, dtype=torch.float64, device=dev)
    ga_l, gt_l = batch.backward_raw(atoms, tmin, tmax, lnB, soft, one, zero)
    ga_s, gt_s = batch.backward_raw(atoms, tmin, tmax, lnB, soft, zero, one)
    torch.cuda.synchronize()
    for k, t in enumerate(tl):
        # tau_max: the GPU forward in FP64 at tau_max +- h tau_max
        h = 1e-6 * tmax[k]
        p, m = tmax.copy(), tmax.copy()
        p[k] += h
        m[k] -= h
        lp, sp = batch.forward_raw(atoms, tmin, p)
        lm, sm = batch.forward_raw(atoms, tmin, m)
        fd_l = (float(lp[k]) - float(lm[k])) / (2 * h)
        fd_s = (float(sp[k]) - float(sm[k])) / (2 * h)
        assert fd_l == pytest.approx(float(gt_l[k, 1]), rel=1e-4, abs=1e-12)
        assert fd_s == pytest.approx(float(gt_s[k, 1]), rel=1e-4, abs=1e-12)
        # atoms: FP64 reference function (atoms are FP32 on the GPU, too coarse for h = 1e-6)
        x0 = torch.from_numpy(t["atoms"].astype(np.float64))
        row = int(batch.desc["atom_offset"][k])
        rng = np.random.default_rng(k)
        for _ in range(5):
            i, ch = int(rng.integers(0, x0.shape[0])), int(rng.integers(0, 7))
            vals = []
            for sgn in (1, -1):
                xv = x0.clone()
                xv[i, ch] += sgn * 1e-6
                with torch.no_grad():
                    a, b, _ = R.stats(xv, 1800, t["t0_data"], t["t0s"], torch.tensor(tmin[k]),
                                      torch.tensor(tmax[k]), t["N_tau"], T)
                vals.append((float(a), float(b)))
            fl = (vals[0][0] - vals[1][0]) / 2e-6
            fs = (vals[0][1] - vals[1][1]) / 2e-6
            assert float(ga_l[row + i, ch]) == pytest.approx(fl, rel=1e-4, abs=1e-7)
            assert float(ga_s[row + i, ch]) == pytest.approx(fs, rel=1e-4, abs=1e-6)


def _config3_templates(tau_min):
    """256 templates, 2000 SFTs x 2 detectors, 1024 t0 x 3600 s (~ the 2000-SFT
    span) x 1024 tau from ``tau_min`` in steps of 1200 s (boundary-safe grids,
    see templates_small: 3 tau_min = 225 mod 900)."""
    tl = []
    for k in range(256):
        t0_data, A = synth.merged_atoms(5000 + k, 2000, 2)
        tl.append(dict(atoms=A, TAtom=1800, t0_data=t0_data, t0=t0_data + 450, dt0=3600,
                       N_t0=1024, N_tau=1024, tau_min=tau_min, tau_max=tau_min + 1200.0 * 1023))
    return tl


def _fp32_step(x, h):
    """Central-difference points around the FP32 value x: (x - h', x + h'')
    as FP32 values and their exact FP64 distance."""
    lo = np.float32(np.float64(x) - h)
    hi = np.float32(np.float64(x) + h)
    return lo, hi, float(np.float64(hi) - np.float64(lo))


@pytest.mark.parametrize("grid", ["short_tau", "interior_tau"])
def test_differentiation_workload_256x2000x1024sq(torch_cuda, grid):
    """256 templates, 2000 SFTs x 2 detectors, 1024 x 1024 (t0, tau): forward
    and backward of all templates; for 3 of them, every gradient against
    central FP64 finite differences of the GPU's FP64 forward (bar 1e-4
    relative): d/d tau_min, d/d tau_max and d/d atom for 8 atoms x all 7
    channels (the 4 atoms with the largest adjoint and 4 random ones).

    Two tau grids on the same atoms: "short_tau" starts at 1875 s, where
    windows of a few SFTs are near-singular and their huge F puts the weight
    of both statistics in the first tau column (so the tau_min derivatives
    carry it and the tau_max ones nearly vanish); "interior_tau" starts at
    30075 s (windows of >= 50 SFTs, well conditioned), so the weight lies in
    interior tau columns and d/d tau_max is non-zero for both statistics."""
    torch = torch_cuda
    from pyfstat_gb300.autograd import ExpDiffBatch

    tau_min0 = 1875.0 if grid == "short_tau" else 30075.0
    tl = _config3_templates(tau_min0)
    batch = ExpDiffBatch(tl, temperature=0.1)
    dev = torch.device("cuda:0")
    atoms = torch.from_numpy(batch.atoms).to(dev)
    tmin = np.array([t["tau_min"] for t in tl])
    tmax = np.array([t["tau_max"] for t in tl])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    lnB, soft = batch.forward_raw(atoms, tmin, tmax)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    one = torch.ones(256, dtype=torch.float64, device=dev)
    zero = torch.zeros(256, dtype=torch.float64, device=dev)
    ga_s, gt_s = batch.backward_raw(atoms, tmin, tmax, lnB, soft, zero, one)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    ga_l, gt_l = batch.backward_raw(atoms, tmin, tmax, lnB, soft, one, zero)
    torch.cuda.synchronize()
    print(f"\n[{grid}] 256 templates x 2000 SFTs x 2 detectors, 1024 x 1024: forward "
          f"{1e3 * (t1 - t0):.1f} ms, backward {1e3 * (t2 - t1):.1f} ms for "
          f"{256 * 1024 * 1024:.3g} cells")
    assert torch.isfinite(ga_s).all() and torch.isfinite(ga_l).all()
    assert torch.isfinite(gt_s).all() and torch.isfinite(gt_l).all()
    ga_s, ga_l = ga_s.cpu().numpy(), ga_l.cpu().numpy()

    # finite differences on a batch of the 3 checked templates (independent
    # of the others, so its forward gives the same values)
    ks = (0, 17, 255)
    sub = ExpDiffBatch([tl[k] for k in ks], temperature=0.1, handle=batch.handle)
    s_atoms = torch.from_numpy(sub.atoms).to(dev)
    s_min, s_max = tmin[list(ks)], tmax[list(ks)]
    l0, s0 = sub.forward_raw(s_atoms, s_min, s_max)
    for j, k in enumerate(ks):
        assert float(l0[j]) == pytest.approx(float(lnB[k]), rel=1e-12)
        assert float(s0[j]) == pytest.approx(float(soft[k]), rel=1e-12)

    # tau: tau_min moves by ~2 s (short) / 1e-5 relative, tau_max by ~1.2 s,
    # so no window boundary moves
    for which, base, rel_h in (("min", s_min, 1e-3 if grid == "short_tau" else 3e-5),
                               ("max", s_max, 1e-6)):
        hh = rel_h * base
        args_p = (s_min + hh, s_max) if which == "min" else (s_min, s_max + hh)
        args_m = (s_min - hh, s_max) if which == "min" else (s_min, s_max - hh)
        lp, sp = sub.forward_raw(s_atoms, *args_p)
        lm, sm = sub.forward_raw(s_atoms, *args_m)
        col = 0 if which == "min" else 1
        for j, k in enumerate(ks):
            fd_l = (float(lp[j]) - float(lm[j])) / (2 * hh[j])
            fd_s = (float(sp[j]) - float(sm[j])) / (2 * hh[j])
            print(f"template {k}: d/dtau_{which}: lnBtSG adjoint {float(gt_l[k, col]):.9e} "
                  f"FD {fd_l:.9e}; softmax2F adjoint {float(gt_s[k, col]):.9e} FD {fd_s:.9e}")
            informative = which == "min" or grid == "interior_tau"
            if informative:
                # non-vacuous: both sides are clearly non-zero
                assert abs(fd_l) > 1e-9 and abs(fd_s) > 1e-9, (which, k, fd_l, fd_s)
                assert fd_l == pytest.approx(float(gt_l[k, col]), rel=1e-4)
                assert fd_s == pytest.approx(float(gt_s[k, col]), rel=1e-4)
            else:
                # the weight sits in the first column: the derivative nearly
                # vanishes; adjoint and FD still agree to 1e-4 of the tau_min one
                scale_l, scale_s = abs(float(gt_l[k, 0])), abs(float(gt_s[k, 0]))
                assert abs(fd_l - float(gt_l[k, col])) <= 1e-4 * max(abs(fd_l), scale_l)
                assert abs(fd_s - float(gt_s[k, col])) <= 1e-4 * max(abs(fd_s), scale_s)

    # atoms: 8 atoms per template x 7 channels; the same (atom, channel) slot is
    # perturbed in all 3 templates at once (their results are independent)
    rng = np.random.default_rng(3)
    picks, rows = [], []
    for j, k in enumerate(ks):
        r0 = int(batch.desc["atom_offset"][k])
        n = int(batch.desc["numAtoms"][k])
        mag = np.abs(ga_s[r0:r0 + n]).sum(axis=1) + np.abs(ga_l[r0:r0 + n]).sum(axis=1)
        top = list(np.argsort(mag)[-4:][::-1])
        rest = [int(i) for i in rng.permutation(np.flatnonzero(mag > 0)) if i not in top][:4]
        picks.append([int(i) for i in top] + rest)
        rows.append((r0, int(sub.desc["atom_offset"][j])))
    base = sub.atoms.copy()
    checked = 0
    for slot in range(8):
        for ch in range(7):
            xp, xm, steps = base.copy(), base.copy(), []
            for j in range(3):
                i = picks[j][slot]
                x = base[rows[j][1] + i, ch]
                # short taus: a few dozen FP32 ulps, small enough for the
                # truncation error of the near-singular cells that carry the
                # weight (F up to ~1e4, strongly non-linear in the atoms);
                # interior taus (smooth): 1e-4 of the value, so that the
                # forward's round-off (~1e-14 of its value) stays far below
                # the difference
                h = (2e-6 if grid == "short_tau" else 1e-4) * abs(float(x)) if x != 0 else 1e-9
                lo, hi, step = _fp32_step(x, h)
                xm[rows[j][1] + i, ch] = lo
                xp[rows[j][1] + i, ch] = hi
                steps.append(step)
            lp, sp = sub.forward_raw(torch.from_numpy(xp).to(dev), s_min, s_max)
            lm, sm = sub.forward_raw(torch.from_numpy(xm).to(dev), s_min, s_max)
            lp, sp, lm, sm = (v.cpu().numpy() for v in (lp, sp, lm, sm))
            for j, k in enumerate(ks):
                i = picks[j][slot]
                r0 = rows[j][0]
                n = int(batch.desc["numAtoms"][k])
                for fd, g in (((lp[j] - lm[j]) / steps[j], ga_l[r0:r0 + n]),
                              ((sp[j] - sm[j]) / steps[j], ga_s[r0:r0 + n])):
                    scale = np.abs(g).max()
                    assert float(g[i, ch]) == pytest.approx(float(fd), rel=1e-4,
                                                           abs=1e-6 * scale), (k, i, ch)
                    checked += 1
    print(f"[{grid}] atom gradients checked against FP64 finite differences: {checked} "
          f"(3 templates x 8 atoms x 7 channels x 2 statistics)")


def test_rect_and_exp_templates_in_one_batch(torch_cuda):
    """Rectangular windows: values and atom gradients against the FP64 torch
    reference (and its finite differences); tau gradients are zero (the sums do
    not depend on tau between window boundaries)."""
    torch = torch_cuda
    from pyfstat_gb300.autograd import DiffBatch, transient_stats

    T = 0.1
    tl = templates_small()
    rect = []
    for k, (nsft, N_t0, N_tau) in enumerate([(70, 20, 13), (45, 7, 9)]):
        t0_data, A = synth.merged_atoms(40 + k, nsft, 2, gap_frac=0.1)
        rect.append(dict(atoms=A, TAtom=1800, t0_data=t0_data, window=1,
                         t0s=(t0_data + 1800 * np.arange(N_t0) + 450).astype(np.uint32),
                         N_tau=N_tau, tau_min=2700.0 + 450.0, tau_max=3150.0 + 1800.0 * (N_tau - 1)))
    mixed = [rect[0], tl[0], rect[1], tl[1]]
    batch = DiffBatch(mixed, temperature=T)
    dev = torch.device("cuda:0")
    atoms = torch.from_numpy(batch.atoms).to(dev).requires_grad_(True)
    tmin = torch.tensor([t["tau_min"] for t in mixed], dtype=torch.float64, requires_grad=True)
    tmax = torch.tensor([t["tau_max"] for t in mixed], dtype=torch.float64, requires_grad=True)
    lnB, soft = transient_stats(atoms, tmin, tmax, batch)
    gl = torch.tensor([0.7, -0.2, 1.0, 0.4], dtype=torch.float64, device=dev)
    gs = torch.tensor([0.5, 1.0, -1.5, 0.1], dtype=torch.float64, device=dev)
    ((lnB * gl).sum() + (soft * gs).sum()).backward()
    ga = atoms.grad.double().cpu().numpy()
    lnB_v, soft_v = lnB.detach().cpu().numpy(), soft.detach().cpu().numpy()
    row = 0
    for k, t in enumerate(mixed):
        w = t.get("window", 2)
        x = torch.from_numpy(t["atoms"].astype(np.float64)).requires_grad_(True)
        a = torch.tensor(t["tau_min"], dtype=torch.float64, requires_grad=True)
        b = torch.tensor(t["tau_max"], dtype=torch.float64, requires_grad=True)
        rl, rs, _ = R.stats(x, 1800, t["t0_data"], t["t0s"], a, b, t["N_tau"], T, window=w)
        assert float(lnB_v[k]) == pytest.approx(float(rl.detach()), rel=1e-9)
        assert float(soft_v[k]) == pytest.approx(float(rs.detach()), rel=1e-9)
        (rl * float(gl[k]) + rs * float(gs[k])).backward()
        n = t["atoms"].shape[0]
        g_ref = x.grad.numpy()
        scale = np.abs(g_ref).max()
        np.testing.assert_allclose(ga[row:row + n], g_ref, rtol=1e-6, atol=1e-9 * scale)
        if w == 1:
            assert float(tmin.grad[k]) == 0.0 and float(tmax.grad[k]) == 0.0
            # atoms: central FP64 finite differences of the reference function
            x0 = torch.from_numpy(t["atoms"].astype(np.float64))
            rng = np.random.default_rng(k)
            for _ in range(4):
                i, ch = int(rng.integers(0, n)), int(rng.integers(0, 7))
                vals = []
                for sgn in (1, -1):
                    xv = x0.clone()
                    xv[i, ch] += sgn * 1e-6
                    with torch.no_grad():
                        p, q, _ = R.stats(xv, 1800, t["t0_data"], t["t0s"],
                                          torch.tensor(t["tau_min"]), torch.tensor(t["tau_max"]),
                                          t["N_tau"], T, window=1)
                    vals.append(float(p) * float(gl[k]) + float(q) * float(gs[k]))
                fd = (vals[0] - vals[1]) / 2e-6
                assert float(ga[row + i, ch]) == pytest.approx(fd, rel=1e-4, abs=1e-6 * scale)
        row += n


def test_invalid_window_type_is_a_status_error(torch_cuda):
    torch = torch_cuda
    from pyfstat_gb300 import _lib
    from pyfstat_gb300.autograd import DiffBatch

    t = templates_small()[0]
    b = DiffBatch([dict(t, window=3)])
    atoms = torch.from_numpy(b.atoms).to("cuda:0")
    with pytest.raises(_lib.TcwError):
        b.forward_raw(atoms, [t["tau_min"]], [t["tau_max"]])
    # the handle stays usable
    b.desc["window"] = 2
    lnB, soft = b.forward_raw(atoms, [t["tau_min"]], [t["tau_max"]])
    torch.cuda.synchronize()
    assert np.isfinite(float(lnB[0])) and np.isfinite(float(soft[0]))
