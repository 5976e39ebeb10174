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
        assert float(lnB_v[k]) == pytest.approx(float(rl), rel=1e-9)
        assert float(soft_v[k]) == pytest.approx(float(rs), rel=1e-9)
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
    and backward run; tau_max gradients of a few templates against central
    FP64 finite differences of the GPU forward."""
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
    ga, gt = batch.backward_raw(atoms, tmin, tmax, lnB, soft, zero, one)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    print(f"\n256 templates x 2000 SFTs x 2 detectors, 1024 x 1024: forward {1e3 * (t1 - t0):.1f} ms, backward "
          f"{1e3 * (t2 - t1):.1f} ms for {256 * 1024 * 1024:.3g} cells")
    assert torch.isfinite(ga).all() and torch.isfinite(gt).all()
    for k in (0, 17, 255):
        h = 1e-6 * tmax[k]
        p, m = tmax.copy(), tmax.copy()
        p[k] += h
        m[k] -= h
        _, sp = batch.forward_raw(atoms, tmin, p)
        _, sm = batch.forward_raw(atoms, tmin, m)
        fd = (float(sp[k]) - float(sm[k])) / (2 * h)
        print(f"template {k}: d softmax2F / d tau_max adjoint {float(gt[k, 1]):.9e}, "
              f"central FD {fd:.9e}")
        assert fd == pytest.approx(float(gt[k, 1]), rel=1e-4, abs=1e-12)
