"""FP64 torch-autograd reference of the differentiable exponential-window
statistics (test infrastructure): the transient map written as dense FP64
tensor algebra over (t0, tau, atom), with the reference's window and
conditioning rules (pyfstat/pyCUDAkernels/cudaTransientFstatExpWindow.cu:
27-66, :80-129) on a continuous tau grid.  Small sizes only."""

import numpy as np
import torch


def window_mask(numAtoms, TAtom, t0_data, t0s, taus, window=2):
    """[m, n, i] True where atom i is in the window of (t0s[m], taus[n]):
    exponential windows as Exp.cu:27-90 (t1 = t0 + 3 tau, t0 <= t_i <= t1),
    rectangular ones as Rect.cu:21-69 (i_t0 <= i <= i_t1, t1 = t0 + tau)."""
    t0s = np.asarray(t0s, dtype=np.float64)
    taus = np.asarray(taus, dtype=np.float64)
    half = TAtom // 2
    i = np.arange(numAtoms, dtype=np.float64)
    t_i = t0_data + i * TAtom
    # i_t0 for t0 >= t0_data - TAtom/2 (no u32 wrap): floor((t0 - t0_data + half) / TAtom)
    i_t0 = np.clip(np.floor((t0s - t0_data + half) / TAtom), 0, numAtoms - 1)
    t1 = t0s[:, None] + (3.0 if window == 2 else 1.0) * taus[None, :]
    i_t1 = np.clip(np.floor((t1 - t0_data + half) / TAtom) - 1.0, 0, numAtoms - 1)
    if window == 1:
        return (i[None, None, :] >= i_t0[:, None, None]) & (i[None, None, :] <= i_t1[:, :, None])
    m = ((i[None, None, :] >= i_t0[:, None, None]) & (i[None, None, :] <= i_t1[:, :, None])
         & (t_i[None, None, :] >= t0s[:, None, None]) & (t_i[None, None, :] <= t1[:, :, None])
         & (t1[:, :, None] >= t0_data))
    return m


def stats(atoms, TAtom, t0_data, t0s, tau_min, tau_max, N_tau, T=0.1, window=2):
    """(lnBtSG, softmax2F, F) as FP64 torch values, differentiable in atoms,
    tau_min and tau_max (torch FP64 tensors); ``window`` 2 exponential, 1
    rectangular."""
    n = torch.arange(N_tau, dtype=torch.float64)
    taus = tau_min + n * (tau_max - tau_min) / max(1, N_tau - 1) if N_tau > 1 else tau_min + 0 * n
    numAtoms = atoms.shape[0]
    mask = torch.from_numpy(window_mask(numAtoms, TAtom, t0_data, t0s, taus.detach().numpy(),
                                        window))
    t_i = t0_data + torch.arange(numAtoms, dtype=torch.float64) * TAtom
    t0 = torch.from_numpy(np.asarray(t0s, dtype=np.float64))
    dt = (t_i[None, None, :] - t0[:, None, None]).clamp(min=0.0)
    if window == 1:
        w = torch.where(mask, torch.ones((), dtype=torch.float64),
                        torch.zeros((), dtype=torch.float64))
    else:
        w = torch.where(mask, torch.exp(-dt / taus[None, :, None]),
                        torch.zeros((), dtype=torch.float64))
    w2 = w * w
    A = torch.einsum("mni,i->mn", w2, atoms[:, 0])
    B = torch.einsum("mni,i->mn", w2, atoms[:, 1])
    C = torch.einsum("mni,i->mn", w2, atoms[:, 2])
    Far = torch.einsum("mni,i->mn", w, atoms[:, 3])
    Fai = torch.einsum("mni,i->mn", w, atoms[:, 4])
    Fbr = torch.einsum("mni,i->mn", w, atoms[:, 5])
    Fbi = torch.einsum("mni,i->mn", w, atoms[:, 6])
    with torch.no_grad():
        sumAB = A + B
        disc = torch.sqrt((A - B) ** 2 + 4.0 * C * C)
        denom = sumAB - disc
        cond = torch.where(denom > 0, (sumAB + disc) / torch.where(denom > 0, denom, 1.0),
                           torch.full_like(denom, float("inf")))
        D0 = A * B - C * C
        ok = (cond < 1e4) & (D0 > 0)
    D = torch.where(ok, A * B - C * C, torch.ones_like(A))
    N = B * (Far ** 2 + Fai ** 2) + A * (Fbr ** 2 + Fbi ** 2) - 2.0 * C * (Far * Fbr + Fai * Fbi)
    F = torch.where(ok, N / D, torch.full_like(A, 2.0))
    N_t0 = len(t0s)
    lnB = np.log(70.0 / (N_t0 * N_tau)) + torch.logsumexp(F.reshape(-1), 0)
    soft = T * torch.logsumexp(2.0 * F.reshape(-1) / T, 0)
    return lnB, soft, F
