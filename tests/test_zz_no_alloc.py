"""The entry point for callers that cannot allocate device memory.

Host programs that forbid raw device allocations (a caller-managed memory
pool, code that must not synchronise the device as cudaMalloc/cudaFree may,
real-time loops with pre-budgeted memory) call tcw_map_plain_noalloc: its
scratch is a fixed static device array instead of allocated workspace.  Its
results must equal the handle-based tcw_map_plain's, on two calls in a row
(the second call reuses the scratch the first one left behind), and on a
sequence of differently shaped calls, each also checked against the FP64
oracle.  This file is
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


def _run_pair(lib, dev, stream, c, flags):
    """The map of case ``c`` through the handle-based entry point and through
    tcw_map_plain_noalloc, on the same stream: (F_handle, res_handle, F, res)."""
    import torch

    from pyfstat_gb300 import _lib

    A = torch.from_numpy(np.ascontiguousarray(c["atoms"], np.float32)).to(dev)
    t0s = torch.from_numpy(np.ascontiguousarray(c["t0s"], np.uint32).view(np.int32)).to(dev)
    taus = torch.from_numpy(np.ascontiguousarray(c["taus"], np.uint32).view(np.int32)).to(dev)
    shape = (len(c["t0s"]), len(c["taus"]))
    out = []
    h = _lib.Handle(0)
    try:
        F = torch.full(shape, -1.0, dtype=torch.float32, device=dev)
        r = torch.zeros(5, dtype=torch.float64, device=dev)
        h.set_stream(stream.cuda_stream)
        h.map_plain(A, A.shape[0], c["TAtom"], c["t0_data"], c["window"], t0s, shape[0], taus,
                    shape[1], F, r, flags=flags)
        torch.cuda.synchronize()
        out += [F.cpu().numpy(), r.cpu().numpy().view(_lib.RESULT_DTYPE)[0]]
    finally:
        h.close()
    F = torch.full(shape, -1.0, dtype=torch.float32, device=dev)
    r = torch.zeros(5, dtype=torch.float64, device=dev)
    rc = lib.tcw_map_plain_noalloc(ctypes.c_void_p(stream.cuda_stream), A.data_ptr(),
                                   A.shape[0], c["TAtom"], c["t0_data"], c["window"],
                                   t0s.data_ptr(), shape[0], taus.data_ptr(), shape[1],
                                   F.data_ptr(), r.data_ptr(), flags)
    assert rc == 0, _lib.strerror(rc)
    torch.cuda.synchronize()
    out += [F.cpu().numpy(), r.cpu().numpy().view(_lib.RESULT_DTYPE)[0]]
    return out


def _long_column_case():
    """An exponential map with 1.1 million t0 rows: more than 16 x 65535, so
    a column's rows are split into several row tiles (a lane's row chunk is
    a 16-bit count)."""
    t0_data, A = synth.merged_atoms(9, 700, 1, gap_frac=0.1)
    return dict(name="long_column", window=2, atoms=A, TAtom=1800, t0_data=t0_data,
                t0s=(t0_data + np.arange(1_100_000)).astype(np.uint32),
                taus=np.array([1800, 3600, 18000, 36000], np.uint32))


def test_noalloc_sequence_of_geometries_against_oracle(oracle):
    """Calls of different windows and sizes in a row, each reading scratch
    that the previous, differently shaped call left behind (longer tile
    lists, more partials, exponential atom rows where rectangular prefix
    rows now go): each result equals the handle-based entry point's bit for
    bit and agrees with the FP64 oracle within the parity bar."""
    torch = pytest.importorskip("torch")
    from _helpers import REL_TOL, argmax_ok, rel_err
    from pyfstat_gb300 import _lib

    lib = _lib.load()
    dev = torch.device("cuda:0")
    torch.cuda.set_device(dev)
    stream = torch.cuda.Stream(device=dev)
    t0_data, A = synth.merged_atoms(11, 120, 1, gap_frac=0.2)
    small_rect = dict(name="small_rect", window=1, atoms=A, TAtom=1800, t0_data=t0_data,
                      t0s=(t0_data + 900 * np.arange(60)).astype(np.uint32),
                      taus=(1800 + 2700 * np.arange(50)).astype(np.uint32))
    seq = [(dict(synth.plain_exp_case(), name="exp480x512log"), 0x1 | 0x2),
           (small_rect, 0x1),
           (dict(synth.plain_rect_case(), name="rect480"), 0x1 | 0x2),
           (_long_column_case(), 0x1),
           (dict(synth.plain_exp_case(), name="exp480x512log again"), 0x1 | 0x2),
           (small_rect, 0x1 | 0x2)]
    for c, flags in seq:
        Fh, rh, F, r = _run_pair(lib, dev, stream, c, flags)
        assert np.array_equal(F.view(np.uint32), Fh.view(np.uint32)), c["name"]
        assert r.tobytes() == rh.tobytes(), c["name"]
        F64, cond = oracle.map_f64(c["atoms"], c["TAtom"], c["t0_data"], c["window"],
                                   c["t0s"], c["taus"], with_cond=True)
        rel, nband = rel_err(F, F64, cond)
        assert rel.max() < REL_TOL, (c["name"], rel.max())
        assert float(r["maxF"]) == float(F.max()) and int(r["argmax"]) == int(np.argmax(F))
        if nband == 0:
            assert argmax_ok(r["argmax"], F64, label=f"noalloc {c['name']}"), c["name"]
            assert float(r["lnBtSG"]) == pytest.approx(oracle.lnBtSG(F64), rel=REL_TOL)


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
