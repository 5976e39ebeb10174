"""The full-FP64 GPU reference map (tcw_map_f64): against the FP64 CPU oracle
on the golden cases and, at the precision-at-scale size (one year of data,
8192 t0 x 4096 tau), on 10^4 random cells plus whole rows and columns; then
the library's default FP32 path against it over the whole map."""

import math

import numpy as np
import pytest

from _helpers import REL_TOL, golden_case, golden_cases, rel_err
from pyfstat_gb300 import _lib, synth
from pyfstat_gb300.batched import template_grids

pytestmark = pytest.mark.gpu

# FP64 direct sums on the GPU vs on the CPU: the same cells summed in FP64
# (exponential weights by recursion on the GPU, by exp() per atom on the CPU).
F64_REL_TOL = 1e-10


@pytest.fixture(scope="module")
def torch_dev():
    torch = pytest.importorskip("torch")
    return torch, torch.device("cuda:0")


@pytest.fixture(scope="module")
def h(torch_dev):
    torch, dev = torch_dev
    handle = _lib.Handle(0)
    handle.set_stream(torch.cuda.current_stream(dev).cuda_stream or 0x1)
    yield handle
    handle.close()


def gpu_f64(h, torch, dev, c, rows=None):
    t0s = np.ascontiguousarray(c["t0s"], np.uint32)
    taus = np.ascontiguousarray(c["taus"], np.uint32)
    A = torch.from_numpy(np.ascontiguousarray(c["atoms"], np.float32)).to(dev)
    d_t0 = torch.from_numpy(t0s.view(np.int32)).to(dev)
    d_tau = torch.from_numpy(taus.view(np.int32)).to(dev)
    nr = len(t0s) if rows is None else len(rows)
    F = torch.empty((nr, len(taus)), dtype=torch.float64, device=dev)
    cond = torch.empty_like(F)
    h.map_f64(A, A.shape[0], c["TAtom"], c["t0_data"], c["window"], d_t0, len(t0s), d_tau,
              len(taus), F, rows=rows, d_cond=cond)
    torch.cuda.synchronize(dev)
    return F, cond


def test_golden_cases_match_cpu_fp64_oracle(golden, oracle, h, torch_dev):
    torch, dev = torch_dev
    for name in golden_cases(golden):
        c = golden_case(golden, name)
        if c["window"] not in (1, 2):
            continue
        F, cond = gpu_f64(h, torch, dev, c)
        F64, cond64 = oracle.map_f64(c["atoms"], c["TAtom"], c["t0_data"], c["window"], c["t0s"],
                                     c["taus"], with_cond=True)
        rel, _ = rel_err(F.cpu().numpy(), F64, cond64)
        assert rel.max() < F64_REL_TOL, name


def test_row_subset_equals_full_rows(h, torch_dev):
    torch, dev = torch_dev
    c = synth.plain_exp_case()
    F, _ = gpu_f64(h, torch, dev, c)
    rows = np.array([479, 0, 17, 17, 250], dtype=np.uint32)
    Fr, _ = gpu_f64(h, torch, dev, c, rows=rows)
    assert torch.equal(Fr, F[torch.from_numpy(rows.astype(np.int64)).to(dev)])


def test_rows_outside_the_grid_are_rejected(h, torch_dev):
    torch, dev = torch_dev
    c = synth.plain_exp_case()
    with pytest.raises(_lib.TcwError):
        gpu_f64(h, torch, dev, c, rows=np.array([0, 480], dtype=np.uint32))


def test_precision_scale_template(oracle, h, torch_dev):
    """One template of the precision workload (17532 SFTs x 2 detectors, 5 %
    gaps, exp window, 8192 x 4096): the GPU FP64 map against the CPU FP64
    oracle on 10^4 random cells, 3 whole rows and 3 whole columns; the
    library's default map, max2F, argmax and lnBtSG against the GPU FP64 map."""
    torch, dev = torch_dev
    t = synth.precision_templates(1)[0]
    t0s, taus = template_grids(t)
    c = dict(t, t0s=t0s, taus=taus)
    N_t0, N_tau = len(t0s), len(taus)
    F64d, condd = gpu_f64(h, torch, dev, c)

    rng = np.random.default_rng(4)
    ms = rng.integers(0, N_t0, 10000)
    ns = rng.integers(0, N_tau, 10000)
    rows = [0, N_t0 // 2 + 1, N_t0 - 1]
    cols = [0, N_tau // 2 - 1, N_tau - 1]
    for r in rows:
        ms = np.concatenate([ms, np.full(N_tau, r)])
        ns = np.concatenate([ns, np.arange(N_tau)])
    for col in cols:
        ms = np.concatenate([ms, np.arange(N_t0)])
        ns = np.concatenate([ns, np.full(N_t0, col)])
    Fc, condc = oracle.cells_f64(t["atoms"], t["TAtom"], t["t0_data"], 2, t0s[ms], taus[ns],
                                 with_cond=True)
    flat = torch.from_numpy(ms * N_tau + ns).to(dev)
    Fg = F64d.view(-1)[flat].cpu().numpy()
    rel, _ = rel_err(Fg, Fc, condc)
    assert rel.max() < F64_REL_TOL

    A = torch.from_numpy(t["atoms"]).to(dev)
    d_t0 = torch.from_numpy(t0s.view(np.int32)).to(dev)
    d_tau = torch.from_numpy(taus.view(np.int32)).to(dev)
    F = torch.empty((N_t0, N_tau), dtype=torch.float32, device=dev)
    res = torch.zeros(5, dtype=torch.float64, device=dev)
    h.map_plain(A, A.shape[0], 1800, t["t0_data"], 2, d_t0, N_t0, d_tau, N_tau, F, res,
                flags=_lib.TCW_FLAG_LNBTSG)
    torch.cuda.synchronize(dev)
    band = (condd / 1e4 - 1.0).abs() < 1e-5
    relg = ((F.double() - F64d).abs() / F64d.abs().clamp_min(1e-300)).masked_fill(band, 0.0)
    print(f"\nprecision-scale template: max rel err 2F {float(relg.max()):.3e} over "
          f"{N_t0 * N_tau} cells ({int(band.sum())} in the threshold band)")
    assert float(relg.max()) < REL_TOL
    rec = res.cpu().numpy().view(_lib.RESULT_DTYPE)[0]
    top = float(F64d.max())
    assert abs(float(rec["maxF"]) - top) <= REL_TOL * top
    am = int(rec["argmax"])
    assert am == int(torch.argmax(F64d)) or float(F64d.view(-1)[am]) >= top * (1 - 2 * REL_TOL)
    lnB64 = math.log(70.0 / (N_t0 * N_tau)) + float(torch.logsumexp(F64d.view(-1), 0))
    assert abs(float(rec["lnBtSG"]) - lnB64) <= REL_TOL * abs(lnB64)
