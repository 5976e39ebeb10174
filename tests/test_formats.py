"""File formats (host, no GPU): text maps byte-identical to the reference's
line format, reader semantics of read_from_file, atoms text and binary dumps
round trips."""

import numpy as np
import pytest

from pyfstat_gb300 import _lib, formats
from pyfstat_gb300.tcw_fstat_map_funcs import pyTransientFstatMap
from pyfstat_gb300.window import uniform_grid


def reference_lines(F, t0s, taus, header):
    """The line format of write_F_mn_to_file (tcw_fstat_map_funcs.py:289-317)."""
    out = ["# {:s}\n".format(h) for h in header] + ["# t0[s]     tau[s]     2F\n"]
    for m, F_m in enumerate(F):
        for n, this_F in enumerate(F_m):
            out.append("  %10d %10d %- 11.8g\n" % (int(t0s[m]), int(taus[n]), 2.0 * this_F))
    return "".join(out)


def test_text_map_is_byte_identical_to_the_reference_format(tmp_path):
    rng = np.random.default_rng(1)
    F = (rng.standard_normal((7, 5)) * 10.0 ** rng.integers(-6, 6, (7, 5))).astype(np.float32)
    F[0, 0] = 0.0
    F[1, 1] = 2.0
    F[2, 2] = np.float32(1e-30)
    F[3, 3] = np.float32(3e30)
    t0s = uniform_grid(4294000000, 123456, 7)  # the last rows pass 2**31
    taus = uniform_grid(1800, 1800, 5)
    p = tmp_path / "map.txt"
    formats.write_map_text(p, F, t0s, taus, header=["a header", "second"])
    assert p.read_text() == reference_lines(F, t0s, taus, ["a header", "second"])


def test_text_map_reader_matches_genfromtxt_semantics(tmp_path):
    rng = np.random.default_rng(2)
    F = rng.uniform(0, 50, (6, 4)).astype(np.float32)
    F[4, 1] = F[2, 3] = 60.0  # first occurrence decides ML
    t0s = uniform_grid(700000000, 3600, 6)
    taus = uniform_grid(1800, 900, 4)
    p = tmp_path / "m.txt"
    formats.write_map_text(p, F, t0s, taus)
    Fr, t0_ML, tau_ML, maxF = formats.read_map_text(p)
    table = np.genfromtxt(p, comments="#")
    assert np.array_equal(Fr, (0.5 * table[:, 2]).reshape(6, 4))
    k = int(np.argmax(table[:, 2]))
    assert (t0_ML, tau_ML, maxF) == (table[k, 0], table[k, 1], 0.5 * table[k, 2])
    assert t0_ML == t0s[2] and tau_ML == taus[3]


def test_map_object_round_trip(tmp_path):
    class WR:
        t0, dt0, tau, dtau = 700000000, 1800, 3600, 1800

    m = pyTransientFstatMap(N_t0Range=5, N_tauRange=3)
    m.F_mn = np.arange(15, dtype=np.float32).reshape(5, 3) * 0.5
    p = tmp_path / "obj.txt"
    m.write_F_mn_to_file(p, WR, header=["h"])
    r = pyTransientFstatMap(N_t0Range=1, N_tauRange=1)
    r.read_from_file(p)
    assert np.allclose(r.F_mn, m.F_mn)
    assert r.maxF == 7.0 and r.t0_ML == 700000000 + 4 * 1800 and r.tau_ML == 3600 + 2 * 1800


def test_reader_rejects_malformed_lines(tmp_path):
    p = tmp_path / "bad.txt"
    p.write_text("# header\n  1 2 3\n  4 5\n")
    with pytest.raises(_lib.TcwError):
        formats.read_map_text_columns(p)
    with pytest.raises(_lib.TcwError):
        formats.read_map_text_columns(tmp_path / "missing.txt")


def test_atoms_text_round_trip_and_comment_handling(tmp_path):
    rng = np.random.default_rng(3)
    ts = (700000000 + 1800 * np.arange(50)).astype(np.uint32)
    A = rng.standard_normal((50, 7)).astype(np.float32)
    p = tmp_path / "CFS_Fstatatoms_x.dat"
    formats.write_atoms_text(p, ts, A, header=["data from a test"])
    text = p.read_text().splitlines()
    assert text[0].startswith("%%") and text[1] == "%% tGPS a2 b2 ab Fa_re Fa_im Fb_re Fb_im"
    ts2, A2 = formats.read_atoms_text(p)
    assert np.array_equal(ts2, ts) and np.array_equal(A2, A)
    # a second detector's block appended after its own header
    formats.write_atoms_text(tmp_path / "b.dat", ts[:3], A[:3])
    with open(p, "a") as fa:
        fa.write((tmp_path / "b.dat").read_text())
    ts3, A3 = formats.read_atoms_text(p)
    assert ts3.size == 53 and np.array_equal(A3[50:], A[:3])
    tab = formats.atoms_table(ts2, A2)
    assert np.array_equal(tab["Fb_alpha_im"], A[:, 6]) and tab["timestamp"].dtype == np.uint32


def test_binary_map_dump_round_trip(tmp_path):
    F = np.random.default_rng(4).uniform(0, 9, (33, 17)).astype(np.float32)
    p = tmp_path / "map.bin"
    formats.dump_map(p, F, window=2, t0=1, dt0=2, tau=3, dtau=4, maxF=float(F.max()),
                     lnBtSG=1.5, argmax=int(np.argmax(F)))
    h, G = formats.load_map(p)
    assert np.array_equal(np.asarray(G), F)
    assert (int(h["N_t0"]), int(h["N_tau"]), int(h["window"]), int(h["dtau"])) == (33, 17, 2, 4)
    assert h["lnBtSG"] == 1.5 and h["argmax"] == np.argmax(F)
    (tmp_path / "junk.bin").write_bytes(b"x" * 100)
    with pytest.raises(ValueError):
        formats.load_map(tmp_path / "junk.bin")
