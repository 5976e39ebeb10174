"""F-statistic atoms containers and the binned multi-detector merge.

The containers duck-type lalpulsar's ``FstatAtom`` / ``FstatAtomVector`` /
``MultiFstatAtomVector`` (fields ``timestamp, a2_alpha, b2_alpha, ab_alpha,
Fa_alpha, Fb_alpha``; ``length``, ``TAtom``, ``data``), which is what
PyFstat's ``tcw_fstat_map_funcs`` consumes (tcw_fstat_map_funcs.py:590-639,
:704-728), but keep the per-timestamp quantities in numpy arrays so that no
per-atom Python loop is needed on the way to the GPU.  Real lalpulsar structs
are accepted too (read attribute by attribute).

``merge_multi_atoms_binned`` restates lalpulsar's
``XLALmergeMultiFstatAtomsBinned`` (lalsuite, lalpulsar >= 7.13 as pinned by
PyFstat's setup.py:45; not vendored in PyFstat), called by the pycuda path at
tcw_fstat_map_funcs.py:706:
  * bin width ``deltaT`` (PyFstat passes ``multiFstatAtoms.data[0].TAtom``);
  * ``tMin`` / ``tMax`` = earliest first / latest last timestamp over detectors;
  * ``NBins = round((tMax - tMin) / deltaT) + 1``;
  * each atom goes to bin ``floor((t - tMin) / deltaT)`` (``rule="floor"``, the
    default) or the nearest bin (``rule="round"``) -- lalpulsar's exact
    rounding cannot be checked here, so both are offered and the synthetic
    multi-detector data use offsets for which the two agree;
  * all atoms falling in a bin are summed in FP32, detector by detector;
  * empty (gap) bins are zero atoms; bin timestamps are ``tMin + i*deltaT``.
"""

import numpy as np

ATOM_CHANNELS = ("a2_alpha", "b2_alpha", "ab_alpha", "Fa_alpha_re", "Fa_alpha_im",
                 "Fb_alpha_re", "Fb_alpha_im")


class FstatAtom:
    """One atom (a view of one row of an :class:`FstatAtomVector`)."""

    __slots__ = ("_vec", "_k")

    def __init__(self, vec, k):
        self._vec = vec
        self._k = k

    @property
    def timestamp(self):
        return int(self._vec.timestamps[self._k])

    @property
    def a2_alpha(self):
        return float(self._vec.a2[self._k])

    @property
    def b2_alpha(self):
        return float(self._vec.b2[self._k])

    @property
    def ab_alpha(self):
        return float(self._vec.ab[self._k])

    @property
    def Fa_alpha(self):
        return complex(self._vec.Fa[self._k])

    @property
    def Fb_alpha(self):
        return complex(self._vec.Fb[self._k])


class _AtomSeq:
    def __init__(self, vec):
        self._vec = vec

    def __len__(self):
        return self._vec.length

    def __getitem__(self, k):
        if isinstance(k, slice):
            return [FstatAtom(self._vec, i) for i in range(*k.indices(self._vec.length))]
        if k < 0:
            k += self._vec.length
        if not 0 <= k < self._vec.length:
            raise IndexError(k)
        return FstatAtom(self._vec, k)

    def __iter__(self):
        return (FstatAtom(self._vec, k) for k in range(self._vec.length))


class FstatAtomVector:
    """Atoms of one detector: timestamps (u32), a2, b2, ab (f32), Fa, Fb (c64)."""

    def __init__(self, timestamps, a2, b2, ab, Fa, Fb, TAtom):
        self.timestamps = np.ascontiguousarray(timestamps, dtype=np.uint32)
        n = self.timestamps.shape[0]
        self.a2 = np.ascontiguousarray(a2, dtype=np.float32)
        self.b2 = np.ascontiguousarray(b2, dtype=np.float32)
        self.ab = np.ascontiguousarray(ab, dtype=np.float32)
        self.Fa = np.ascontiguousarray(Fa, dtype=np.complex64)
        self.Fb = np.ascontiguousarray(Fb, dtype=np.complex64)
        for arr in (self.a2, self.b2, self.ab, self.Fa, self.Fb):
            if arr.shape != (n,):
                raise ValueError("all atom quantities must be 1-D of the same length")
        self.TAtom = int(TAtom)

    @property
    def length(self):
        return int(self.timestamps.shape[0])

    @property
    def data(self):
        return _AtomSeq(self)

    def as_matrix(self):
        """(length, 7) float32 [a2, b2, ab, Fa_re, Fa_im, Fb_re, Fb_im]."""
        return atoms_matrix(self.a2, self.b2, self.ab, self.Fa, self.Fb)


class MultiFstatAtomVector:
    """Atoms of several detectors (``data[X]`` is an :class:`FstatAtomVector`)."""

    def __init__(self, vectors):
        self.data = list(vectors)

    @property
    def length(self):
        return len(self.data)


def atoms_matrix(a2, b2, ab, Fa, Fb):
    """Stack atoms into the (numAtoms, 7) float32 matrix of tcw:711-721."""
    Fa = np.asarray(Fa)
    Fb = np.asarray(Fb)
    return np.ascontiguousarray(
        np.column_stack((np.asarray(a2, np.float32), np.asarray(b2, np.float32),
                         np.asarray(ab, np.float32), Fa.real.astype(np.float32),
                         Fa.imag.astype(np.float32), Fb.real.astype(np.float32),
                         Fb.imag.astype(np.float32))), dtype=np.float32)


def vector_arrays(vec):
    """(timestamps u32, (n,7) f32 matrix, TAtom) of a vector of either kind.

    Our own containers are read directly; a lalpulsar ``FstatAtomVector`` is
    read attribute by attribute (the only per-atom loop left, for foreign
    structs, mirroring reshape_FstatAtomsVector at tcw:627-632).
    """
    if isinstance(vec, FstatAtomVector):
        return vec.timestamps, vec.as_matrix(), vec.TAtom
    n = int(vec.length)
    ts = np.empty(n, dtype=np.uint32)
    mat = np.empty((n, 7), dtype=np.float32)
    for k, atom in enumerate(vec.data):
        ts[k] = atom.timestamp
        Fa = complex(atom.Fa_alpha)
        Fb = complex(atom.Fb_alpha)
        mat[k] = (atom.a2_alpha, atom.b2_alpha, atom.ab_alpha, Fa.real, Fa.imag, Fb.real,
                  Fb.imag)
    return ts, mat, int(vec.TAtom)


def merge_multi_atoms_binned(multiAtoms, deltaT, rule="floor"):
    """Merge detectors into one binned atoms series.

    Returns ``(t0_data, matrix)`` with ``matrix`` the (NBins, 7) float32 atoms
    of consecutive bins starting at ``t0_data`` (see module docstring).
    """
    if multiAtoms is None or multiAtoms.length < 1:
        raise ValueError("need at least one detector's atoms")
    deltaT = int(deltaT)
    if deltaT <= 0:
        raise ValueError(f"invalid bin width deltaT={deltaT}")
    parts = [vector_arrays(multiAtoms.data[X]) for X in range(multiAtoms.length)]
    for ts, _, _ in parts:
        if ts.shape[0] == 0:
            raise ValueError("empty atoms vector")
    tMin = min(int(ts[0]) for ts, _, _ in parts)
    tMax = max(int(ts[-1]) for ts, _, _ in parts)
    nbins = int(np.round((tMax - tMin) / deltaT)) + 1
    out = np.zeros((nbins, 7), dtype=np.float32)
    for ts, mat, _ in parts:
        off = (ts.astype(np.int64) - tMin).astype(np.float64) / deltaT
        idx = np.floor(off) if rule == "floor" else np.floor(off + 0.5)
        idx = idx.astype(np.int64)
        if idx.min() < 0 or idx.max() >= nbins:
            raise ValueError("atom timestamp outside the binned range")
        np.add.at(out, idx, mat)
    return tMin, out


def binned_timestamps(t0_data, nbins, deltaT):
    return (np.uint32(t0_data) + np.arange(nbins, dtype=np.uint32) * np.uint32(deltaT)).astype(
        np.uint32)
