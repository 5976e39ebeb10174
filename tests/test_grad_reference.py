"""The FP64 torch-autograd reference of the differentiable statistics is
itself checked on the CPU: its map equals the FP64 oracle's on a continuous
tau grid, and its autograd gradients equal central FP64 finite differences."""

import numpy as np
import pytest
import torch

import _torch_ref as R
from pyfstat_gb300 import synth


def small_case(seed=11, nsft=60, ndet=2, N_t0=14, N_tau=11):
    t0_data, A = synth.merged_atoms(seed, nsft, ndet, gap_frac=0.1)
    t0s = (t0_data + 1800 * np.arange(N_t0) + 300).astype(np.uint32)
    return dict(atoms=A, TAtom=1800, t0_data=t0_data, t0s=t0s, N_tau=N_tau,
                tau_min=1800.0 * 1.3, tau_max=1800.0 * 21.7)


def test_torch_reference_map_equals_oracle(oracle):
    c = small_case()
    taus = np.linspace(c["tau_min"], c["tau_max"], c["N_tau"])
    F64 = oracle.exp_map_f64_realtau(c["atoms"], 1800, c["t0_data"], c["t0s"], taus)
    x = torch.from_numpy(c["atoms"].astype(np.float64))
    _, _, F = R.stats(x, 1800, c["t0_data"], c["t0s"], torch.tensor(c["tau_min"]),
                      torch.tensor(c["tau_max"]), c["N_tau"])
    np.testing.assert_allclose(F.numpy(), F64, rtol=1e-10, atol=0)


def test_torch_reference_gradients_match_finite_differences():
    c = small_case()
    x = torch.from_numpy(c["atoms"].astype(np.float64)).requires_grad_(True)
    tmin = torch.tensor(c["tau_min"], dtype=torch.float64, requires_grad=True)
    tmax = torch.tensor(c["tau_max"], dtype=torch.float64, requires_grad=True)
    lnB, soft, _ = R.stats(x, 1800, c["t0_data"], c["t0s"], tmin, tmax, c["N_tau"])
    (gx_l, gmax_l) = torch.autograd.grad(lnB, (x, tmax), retain_graph=True)
    (gx_s, gmax_s) = torch.autograd.grad(soft, (x, tmax))

    def f(xv, tmx):
        with torch.no_grad():
            a, b, _ = R.stats(xv, 1800, c["t0_data"], c["t0s"], torch.tensor(c["tau_min"]),
                              torch.tensor(tmx), c["N_tau"])
        return float(a), float(b)

    h = 1e-6
    rng = np.random.default_rng(0)
    for _ in range(6):
        i, ch = int(rng.integers(0, x.shape[0])), int(rng.integers(0, 7))
        xp = x.detach().clone()
        xm = x.detach().clone()
        xp[i, ch] += h
        xm[i, ch] -= h
        (lp, sp), (lm, sm) = f(xp, c["tau_max"]), f(xm, c["tau_max"])
        assert (lp - lm) / (2 * h) == pytest.approx(float(gx_l[i, ch]), rel=1e-4, abs=1e-7)
        assert (sp - sm) / (2 * h) == pytest.approx(float(gx_s[i, ch]), rel=1e-4, abs=1e-6)
    ht = h * c["tau_max"]
    (lp, sp), (lm, sm) = f(x.detach(), c["tau_max"] + ht), f(x.detach(), c["tau_max"] - ht)
    assert (lp - lm) / (2 * ht) == pytest.approx(float(gmax_l), rel=1e-4, abs=1e-12)
    assert (sp - sm) / (2 * ht) == pytest.approx(float(gmax_s), rel=1e-4, abs=1e-12)


def test_torch_reference_rect_map_equals_oracle(oracle):
    c = small_case(seed=12)
    tau_min, step = 2700.0, 900.0
    taus = tau_min + step * np.arange(c["N_tau"])
    F64 = oracle.map_f64(c["atoms"], 1800, c["t0_data"], 1, c["t0s"], taus.astype(np.uint32))
    x = torch.from_numpy(c["atoms"].astype(np.float64))
    _, _, F = R.stats(x, 1800, c["t0_data"], c["t0s"], torch.tensor(tau_min),
                      torch.tensor(tau_min + step * (c["N_tau"] - 1)), c["N_tau"], window=1)
    np.testing.assert_allclose(F.numpy(), F64, rtol=1e-10, atol=0)
