"""Child process of the debug-checks test: loads the library named by
PYFSTAT_GB300_LIB (a -DTCW_DEBUG_CHECKS build), runs every kernel family on
small cases and prints the number of failed device-side index checks."""

import ctypes
import os
import sys

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "tests"))


def main():
    import torch

    from _helpers import golden_case, golden_cases
    from pyfstat_gb300 import _lib, synth
    from pyfstat_gb300.autograd import DiffBatch
    from pyfstat_gb300.batched import TransientMapBatch

    lib = _lib.load()
    h = _lib.Handle(0)
    golden = np.load(os.path.join(REPO, "tests", "golden", "reference_maps.npz"))
    flags = _lib.TCW_FLAG_LNBTSG | _lib.TCW_FLAG_POSTERIORS
    cases = [golden_case(golden, n) for n in golden_cases(golden)]
    for c in cases:  # plain path, all windows incl. 'none' (host entry point)
        h.map_plain_host(c["atoms"], c["TAtom"], c["t0_data"], c["window"], c["t0s"], c["taus"],
                         want_map=True, flags=flags)
    cases = [c for c in cases if c["window"] in (1, 2)]
    b = TransientMapBatch([dict(c) for c in cases], flags=flags, handle=h)
    b.plan.run_maps_host(b.atoms)  # batched maps + posteriors
    b.close()
    b = TransientMapBatch(synth.batched_templates(24, seed=4, nsft_range=(20, 200),
                                                  grid_range=(1, 120)), handle=h)
    b.run()  # persistent fused kernels through the graph
    b.close()
    dev = torch.device("cuda", 0)
    h.set_stream(torch.cuda.current_stream(dev).cuda_stream or 0x1)
    for c in cases[:6]:  # FP64 reference map
        A = torch.from_numpy(np.ascontiguousarray(c["atoms"], np.float32)).to(dev)
        t0s = torch.from_numpy(c["t0s"].astype(np.uint32).view(np.int32)).to(dev)
        taus = torch.from_numpy(c["taus"].astype(np.uint32).view(np.int32)).to(dev)
        F = torch.empty((c["t0s"].size, c["taus"].size), dtype=torch.float64, device=dev)
        h.map_f64(A, A.shape[0], c["TAtom"], c["t0_data"], c["window"], t0s, c["t0s"].size,
                  taus, c["taus"].size, F)
    tl = []
    for k, w in enumerate((2, 1, 2, 1)):  # adjoint, both windows
        t0_data, A = synth.merged_atoms(60 + k, 50 + 10 * k, 2, gap_frac=0.1)
        tl.append(dict(atoms=A, TAtom=1800, t0_data=t0_data, window=w,
                       t0s=(t0_data + 450 + 1800 * np.arange(9 + k)).astype(np.uint32),
                       N_tau=7 + k, tau_min=2000.0, tau_max=2000.0 + 1100.0 * (6 + k)))
    db = DiffBatch(tl, handle=h)
    dA = torch.from_numpy(db.atoms).to(dev)
    tmin = [t["tau_min"] for t in tl]
    tmax = [t["tau_max"] for t in tl]
    lnB, soft = db.forward_raw(dA, tmin, tmax)
    one = torch.ones(len(tl), dtype=torch.float64, device=dev)
    db.backward_raw(dA, tmin, tmax, lnB, soft, one, one)
    torch.cuda.synchronize(dev)
    c = cases[0]  # the no-allocation entry point
    A = torch.from_numpy(np.ascontiguousarray(c["atoms"], np.float32)).to(dev)
    t0s = torch.from_numpy(c["t0s"].astype(np.uint32).view(np.int32)).to(dev)
    taus = torch.from_numpy(c["taus"].astype(np.uint32).view(np.int32)).to(dev)
    Fm = torch.empty((c["t0s"].size, c["taus"].size), dtype=torch.float32, device=dev)
    res = torch.zeros(5, dtype=torch.float64, device=dev)
    _lib.map_plain_noalloc(torch.cuda.current_stream(dev).cuda_stream, A, A.shape[0], c["TAtom"],
                           c["t0_data"], c["window"], t0s, c["t0s"].size, taus, c["taus"].size,
                           Fm, res)
    torch.cuda.synchronize(dev)
    n = ctypes.c_uint32(0)
    rc = lib.tcw_debug_check_failures(ctypes.byref(n))
    print("DCHECK", rc, n.value, flush=True)
    h.close()


if __name__ == "__main__":
    main()
