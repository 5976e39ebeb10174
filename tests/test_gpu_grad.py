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


def test_differentiation_workload_256x2000x1024sq(torch_cuda):
    """256 templates, 2000 SFTs x 2 detectors, 1024 x 1024 (t0, tau): forward
    and backward run; tau gradients of a few templates against central FP64
    finite differences of the GPU forward: d softmax2F / d tau_min (at
    T = 0.1 the soft-max sits on its largest cells, whose tau moves with
    tau_min) and d lnBtSG / d tau_max (a sum over all cells)."""
    torch = torch_cuda
    from pyfstat_gb300.autograd import ExpDiffBatch

    tl = []
    for k in range(256):
        t0_data, A = synth.merged_atoms(5000 + k, 2000, 2)
        # 1024 t0 x 3600 s ~ the 2000-SFT span; tau in [1875 s, ~span/3] in
        # steps of 1200 s (boundary-safe grids, see templates_small)
        tl.append(dict(atoms=A, TAtom=1800, t0_data=t0_data, t0=t0_data + 450, dt0=3600,
                       N_t0=1024, N_tau=1024, tau_min=1875.0, tau_max=1875.0 + 1200.0 * 1023))
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
    ga, gt_s = batch.backward_raw(atoms, tmin, tmax, lnB, soft, zero, one)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    _, gt_l = batch.backward_raw(atoms, tmin, tmax, lnB, soft, one, zero)
    torch.cuda.synchronize()
    print(f"\n256 templates x 2000 SFTs x 2 detectors, 1024 x 1024: forward "
          f"{1e3 * (t1 - t0):.1f} ms, backward {1e3 * (t2 - t1):.1f} ms for "
          f"{256 * 1024 * 1024:.3g} cells")
    assert torch.isfinite(ga).all() and torch.isfinite(gt_s).all()
    for k in (0, 17, 255):
        # tau_min moves by ~2 s and tau_max by ~1.2 s: no window boundary moves.
        # The cells that carry weight in both statistics lie in the first tau
        # column here, so the tau_min derivatives are the informative ones;
        # the tau_max ones are checked too (they may vanish).
        fd = {}
        for which, base, hh in (("min", tmin, 1e-3 * tmin[k]), ("max", tmax, 1e-6 * tmax[k])):
            p, m = base.copy(), base.copy()
            p[k] += hh
            m[k] -= hh
            args_p = (p, tmax) if which == "min" else (tmin, p)
            args_m = (m, tmax) if which == "min" else (tmin, m)
            lp, sp = batch.forward_raw(atoms, *args_p)
            lm, sm = batch.forward_raw(atoms, *args_m)
            fd[which] = ((float(lp[k]) - float(lm[k])) / (2 * hh),
                         (float(sp[k]) - float(sm[k])) / (2 * hh))
        print(f"template {k}: tau_min: d lnBtSG adjoint {float(gt_l[k, 0]):.9e} FD "
              f"{fd['min'][0]:.9e}, d softmax2F adjoint {float(gt_s[k, 0]):.9e} FD "
              f"{fd['min'][1]:.9e}; tau_max: d lnBtSG {float(gt_l[k, 1]):.3e} / {fd['max'][0]:.3e}")
        assert fd["min"][0] != 0.0 and fd["min"][1] != 0.0
        assert fd["min"][0] == pytest.approx(float(gt_l[k, 0]), rel=1e-4)
        assert fd["min"][1] == pytest.approx(float(gt_s[k, 0]), rel=1e-4)
        assert fd["max"][0] == pytest.approx(float(gt_l[k, 1]), rel=1e-4, abs=1e-12)
        assert fd["max"][1] == pytest.approx(float(gt_s[k, 1]), rel=1e-4, abs=1e-12)


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
