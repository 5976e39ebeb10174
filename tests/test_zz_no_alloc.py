"""The entry point for callers that cannot allocate device memory.

Host programs that forbid raw device allocations (a caller-managed memory
pool, code that must not synchronise the device as cudaMalloc/cudaFree may,
real-time loops with pre-budgeted memory) call tcw_map_plain_noalloc: its
scratch is a fixed static device array instead of allocated workspace.  Its
results must equal the handle-based tcw_map_plain's, on two calls in a row
(the second call reuses the scratch the first one left behind).  This file is
collected last so that a run stopping at the first failure has run the rest.
"""

import ctypes

import numpy as np
import pytest

from pyfstat_gb300 import synth

pytestmark = pytest.mark.gpu

FLAGS = 0x1 | 0x2  # lnBtSG and posteriors


def _cases():
    return [synth.plain_rect_case(), synth.plain_exp_case()]


@pytest.mark.parametrize("case", [0, 1], ids=["rect", "exp"])
def test_noalloc_matches_plain_entry_point_on_two_calls(case):
    torch = pytest.importorskip("torch")
    from pyfstat_gb300 import _lib

    lib = _lib.load()
    c = _cases()[case]
    dev = torch.device("cuda:0")
    torch.cuda.set_device(dev)
    stream = torch.cuda.Stream(device=dev)
    A = torch.from_numpy(c["atoms"]).to(dev)
    t0s = torch.from_numpy(c["t0s"].view(np.int32)).to(dev)
    taus = torch.from_numpy(c["taus"].view(np.int32)).to(dev)
    shape = (len(c["t0s"]), len(c["taus"]))
    torch.cuda.synchronize()

    # existing entry point (handle, allocated workspace)
    h = _lib.Handle(0)
    try:
        F_ref = torch.empty(shape, dtype=torch.float32, device=dev)
        r_ref = torch.zeros(5, dtype=torch.float64, device=dev)
        h.set_stream(stream.cuda_stream)
        h.map_plain(A, A.shape[0], c["TAtom"], c["t0_data"], c["window"], t0s, shape[0], taus,
                    shape[1], F_ref, r_ref, flags=FLAGS)
        torch.cuda.synchronize()
    finally:
        h.close()
    ref = r_ref.cpu().numpy().view(_lib.RESULT_DTYPE)[0]
    Fr = F_ref.cpu().numpy()

    outs = []
    for _ in range(2):
        F = torch.full(shape, -1.0, dtype=torch.float32, device=dev)
        r = torch.zeros(5, dtype=torch.float64, device=dev)
        rc = lib.tcw_map_plain_noalloc(ctypes.c_void_p(stream.cuda_stream), A.data_ptr(),
                                       A.shape[0], c["TAtom"], c["t0_data"], c["window"],
                                       t0s.data_ptr(), shape[0], taus.data_ptr(), shape[1],
                                       F.data_ptr(), r.data_ptr(), FLAGS)
        assert rc == 0, _lib.strerror(rc)
        torch.cuda.synchronize()
        outs.append((F.cpu().numpy(), r.cpu().numpy().view(_lib.RESULT_DTYPE)[0]))

    for F, res in outs:
        np.testing.assert_allclose(F, Fr, rtol=1e-6, atol=0)
        assert float(res["maxF"]) == pytest.approx(float(ref["maxF"]), rel=1e-6)
        assert int(res["argmax"]) == int(ref["argmax"])
        assert float(res["lnBtSG"]) == pytest.approx(float(ref["lnBtSG"]), rel=1e-9)
        assert int(res["t0_mp_idx"]) == int(ref["t0_mp_idx"])
        assert int(res["tau_mp_idx"]) == int(ref["tau_mp_idx"])


def test_noalloc_rejects_problems_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    from pyfstat_gb300 import _lib

    dev = torch.device("cuda:0")
    n = 300000  # 64 B x 300001 prefix rows > 16 MiB
    A = torch.zeros((n, 7), dtype=torch.float32, device=dev)
    grid = torch.zeros(4, dtype=torch.int32, device=dev)
    r = torch.zeros(5, dtype=torch.float64, device=dev)
    with pytest.raises(_lib.TcwError) as e:
        _lib.map_plain_noalloc(None, A, n, 1800, 700000000, 1, grid, 4, grid, 4, None, r)
    assert e.value.code == _lib.TCW_ERR_OVERFLOW
