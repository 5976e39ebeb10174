"""On-disk formats of the transient-map path.

* Text maps ``t0 tau 2F`` in the lalpulsar write_transientFstatMap_to_fp
  layout (pyfstat/tcw_fstat_map_funcs.py:289-317 writes, :159-184 reads),
  formatted and parsed by the native library.
* F-statistic atom text files (core.py:1879-1910; columns tGPS a2 b2 ab
  Fa_re Fa_im Fb_re Fb_im, comment lines starting with '%'), parsed by the
  native library.
* A binary map dump for batched runs: a 64-byte little-endian header
  (:data:`MAP_HEADER`: magic ``TCWMAP01``; N_t0, N_tau, window, t0, dt0,
  tau, dtau; maxF, lnBtSG, flat argmax) followed by the FP32 F map (F, not
  2F) row-major; read back with a memory map.
"""

import ctypes

import numpy as np

from . import _lib

MAP_MAGIC = b"TCWMAP01"
MAP_HEADER = np.dtype([("magic", "S8"), ("N_t0", "<u4"), ("N_tau", "<u4"), ("window", "<i4"),
                       ("t0", "<u4"), ("dt0", "<u4"), ("tau", "<u4"), ("dtau", "<u4"),
                       ("pad", "<u4"), ("maxF", "<f8"), ("lnBtSG", "<f8"), ("argmax", "<i8")])
assert MAP_HEADER.itemsize == 64


def _path(p):
    return str(p).encode()


# ------------------------------------------------------------------ text maps


def write_map_text(path, F, t0s, taus, header=()):
    """Write ``F`` (N_t0, N_tau; F, not 2F) as ``t0 tau 2F`` lines with the
    reference's header lines (``# <line>`` each, then the column line)."""
    F = np.ascontiguousarray(F, dtype=np.float32)
    t0s = np.ascontiguousarray(t0s, dtype=np.uint32)
    taus = np.ascontiguousarray(taus, dtype=np.uint32)
    if F.shape != (t0s.size, taus.size):
        raise ValueError("F must have shape (len(t0s), len(taus))")
    if isinstance(header, str):
        header = [header]
    with open(path, "w") as fp:
        for line in header:
            fp.write("# {:s}\n".format(line))
        fp.write("# t0[s]     tau[s]     2F\n")
    _lib.check(_lib.load().tcw_write_map_text(_path(path), F.ctypes.data, t0s.size, taus.size,
                                              t0s.ctypes.data, taus.ctypes.data, 1))


def read_map_text_columns(path):
    """(t0, tau, 2F) FP64 columns of a text map."""
    lib = _lib.load()
    n = ctypes.c_uint64(0)
    _lib.check(lib.tcw_read_map_text(_path(path), ctypes.byref(n), None, None, None, 0))
    cols = [np.empty(n.value, dtype=np.float64) for _ in range(3)]
    _lib.check(lib.tcw_read_map_text(_path(path), ctypes.byref(n), cols[0].ctypes.data,
                                     cols[1].ctypes.data, cols[2].ctypes.data, n.value))
    return tuple(cols)


def read_map_text(path):
    """(F_mn, t0_ML, tau_ML, maxF) with the semantics of the reference's
    read_from_file: the map is 2F/2 reshaped to (unique t0s, unique taus),
    the ML values come from the first largest 2F line."""
    t0, tau, twoF = read_map_text_columns(path)
    n_t0 = np.unique(t0).size
    n_tau = np.unique(tau).size
    F = (0.5 * twoF).reshape(n_t0, n_tau)
    k = int(np.argmax(twoF))
    return F, t0[k], tau[k], 0.5 * twoF[k]


# ------------------------------------------------------------------ atoms


def read_atoms_text(path):
    """(timestamps u32, atoms (n, 7) float32) of an atoms text file; several
    detectors' blocks come back concatenated in file order."""
    lib = _lib.load()
    n = ctypes.c_uint64(0)
    _lib.check(lib.tcw_read_atoms_text(_path(path), ctypes.byref(n), None, None, 0))
    ts = np.empty(n.value, dtype=np.uint32)
    A = np.empty((n.value, 7), dtype=np.float32)
    _lib.check(lib.tcw_read_atoms_text(_path(path), ctypes.byref(n), ts.ctypes.data,
                                       A.ctypes.data, n.value))
    return ts, A


def write_atoms_text(path, timestamps, atoms7, header=(), comments="%%"):
    """Write atoms in the same column layout, after ``comments``-prefixed
    header lines."""
    ts = np.ascontiguousarray(timestamps, dtype=np.uint32)
    A = np.ascontiguousarray(atoms7, dtype=np.float32)
    if A.shape != (ts.size, 7):
        raise ValueError("atoms must have shape (len(timestamps), 7)")
    with open(path, "w") as fp:
        for line in header:
            fp.write(f"{comments} {line}\n")
    _lib.check(_lib.load().tcw_write_atoms_text(_path(path), ts.ctypes.data, A.ctypes.data,
                                                ts.size, 1))


def atoms_table(timestamps, atoms7):
    """The dict-of-arrays layout of reshape_FstatAtomsVector (tcw:590-639)."""
    A = np.asarray(atoms7, dtype=np.float32)
    return {"timestamp": np.asarray(timestamps, dtype=np.uint32),
            "a2_alpha": A[:, 0], "b2_alpha": A[:, 1], "ab_alpha": A[:, 2],
            "Fa_alpha_re": A[:, 3], "Fa_alpha_im": A[:, 4],
            "Fb_alpha_re": A[:, 5], "Fb_alpha_im": A[:, 6]}


# ------------------------------------------------------------------ binary maps


def dump_map(path, F, window=0, t0=0, dt0=0, tau=0, dtau=0, maxF=np.nan, lnBtSG=np.nan,
             argmax=-1):
    """Write a binary map dump (header + FP32 F row-major)."""
    F = np.ascontiguousarray(F, dtype=np.float32)
    if F.ndim != 2:
        raise ValueError("F must be 2-D")
    h = np.zeros(1, dtype=MAP_HEADER)
    h[0] = (MAP_MAGIC, F.shape[0], F.shape[1], window, t0, dt0, tau, dtau, 0, maxF, lnBtSG,
            argmax)
    with open(path, "wb") as fp:
        fp.write(h.tobytes())
        F.tofile(fp)


def load_map(path, mmap=True):
    """(header record, F) of a binary map dump; F is a read-only memory map
    unless ``mmap`` is False."""
    h = np.fromfile(path, dtype=MAP_HEADER, count=1)
    if h.size != 1 or h[0]["magic"] != MAP_MAGIC:
        raise ValueError(f"{path}: not a transient map dump")
    shape = (int(h[0]["N_t0"]), int(h[0]["N_tau"]))
    if mmap:
        F = np.memmap(path, dtype=np.float32, mode="r", offset=MAP_HEADER.itemsize, shape=shape)
    else:
        F = np.fromfile(path, dtype=np.float32, offset=MAP_HEADER.itemsize).reshape(shape)
    return h[0], F
