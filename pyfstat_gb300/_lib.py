"""ctypes binding of the C ABI in include/tcw_b200.h (libtcw_b200.so).

The library is the only compute path: if it cannot be loaded there is no
fallback, and every entry point raises.
"""

import ctypes
import os
import threading

import numpy as np

from . import build as _build

TCW_OK = 0
TCW_ERR_INVALID_ARG = -1
TCW_ERR_CUDA = -2
TCW_ERR_NO_DEVICE = -3
TCW_ERR_ALLOC = -4
TCW_ERR_TIMEOUT = -5
TCW_ERR_UNSUPPORTED = -6
TCW_ERR_OVERFLOW = -7
TCW_ERR_IO = -8
TCW_ERR_FORMAT = -9

TCW_WINDOW_NONE = 0
TCW_WINDOW_RECT = 1
TCW_WINDOW_EXP = 2

TCW_FLAG_LNBTSG = 0x1
TCW_FLAG_POSTERIORS = 0x2
TCW_FLAG_FP64_DET = 0x4
TCW_FLAG_UNCOMPENSATED = 0x8

# Every function the header declares, with (restype, argtypes).
_c_u32 = ctypes.c_uint32
_c_u64 = ctypes.c_uint64
_vp = ctypes.c_void_p


class TcwResult(ctypes.Structure):
    _fields_ = [("lnBtSG", ctypes.c_double), ("argmax", ctypes.c_int64),
                ("t0_mp_idx", ctypes.c_int64), ("tau_mp_idx", ctypes.c_int64),
                ("maxF", ctypes.c_float), ("status", ctypes.c_int32)]


class TcwTemplateDesc(ctypes.Structure):
    _fields_ = [("atom_offset", _c_u64), ("t0_offset", _c_u64), ("tau_offset", _c_u64),
                ("numAtoms", _c_u32), ("TAtom", _c_u32), ("t0_data", _c_u32),
                ("window", ctypes.c_int32), ("N_t0", _c_u32), ("N_tau", _c_u32)]


class TcwTileConfig(ctypes.Structure):
    _fields_ = [("rect_tn", _c_u32), ("rect_tm", _c_u32), ("exp_tn", _c_u32),
                ("exp_rows", _c_u32), ("blocks_per_sm", _c_u32)]

    def as_dict(self):
        return {k: int(getattr(self, k)) for k, _ in self._fields_}


RESULT_DTYPE = np.dtype([("lnBtSG", "<f8"), ("argmax", "<i8"), ("t0_mp_idx", "<i8"),
                         ("tau_mp_idx", "<i8"), ("maxF", "<f4"), ("status", "<i4")])
DESC_DTYPE = np.dtype([("atom_offset", "<u8"), ("t0_offset", "<u8"), ("tau_offset", "<u8"),
                       ("numAtoms", "<u4"), ("TAtom", "<u4"), ("t0_data", "<u4"),
                       ("window", "<i4"), ("N_t0", "<u4"), ("N_tau", "<u4")])
DIFF_DESC_DTYPE = np.dtype([("atom_offset", "<u8"), ("t0_offset", "<u8"), ("numAtoms", "<u4"),
                            ("TAtom", "<u4"), ("t0_data", "<u4"), ("N_t0", "<u4"),
                            ("N_tau", "<u4"), ("window", "<u4"), ("tau_min", "<f8"),
                            ("tau_max", "<f8")])
assert DIFF_DESC_DTYPE.itemsize == 56
assert RESULT_DTYPE.itemsize == ctypes.sizeof(TcwResult) == 40
assert DESC_DTYPE.itemsize == ctypes.sizeof(TcwTemplateDesc) == 48

SIGNATURES = {
    "tcw_abi_version": (ctypes.c_int, []),
    "tcw_strerror": (ctypes.c_char_p, [ctypes.c_int]),
    "tcw_last_error": (ctypes.c_char_p, [_vp]),
    "tcw_device_count": (ctypes.c_int, [ctypes.POINTER(ctypes.c_int)]),
    "tcw_device_info": (ctypes.c_int, [ctypes.c_int, ctypes.c_char_p, ctypes.c_size_t,
                                       ctypes.POINTER(ctypes.c_int),
                                       ctypes.POINTER(ctypes.c_int),
                                       ctypes.POINTER(ctypes.c_size_t)]),
    "tcw_device_memory": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_size_t),
                                         ctypes.POINTER(ctypes.c_size_t)]),
    "tcw_create": (ctypes.c_int, [ctypes.POINTER(_vp), ctypes.c_int]),
    "tcw_destroy": (ctypes.c_int, [_vp]),
    "tcw_get_stream": (ctypes.c_int, [_vp, ctypes.POINTER(_vp)]),
    "tcw_set_stream": (ctypes.c_int, [_vp, _vp]),
    "tcw_sync": (ctypes.c_int, [_vp, ctypes.c_int]),
    "tcw_map_plain": (ctypes.c_int, [_vp, _vp, _c_u32, _c_u32, _c_u32, ctypes.c_int, _vp, _c_u32,
                                     _vp, _c_u32, _vp, _vp, ctypes.c_int]),
    "tcw_map_plain_host": (ctypes.c_int, [_vp, _vp, _c_u32, _c_u32, _c_u32, ctypes.c_int, _vp,
                                          _c_u32, _vp, _c_u32, _vp, _vp, ctypes.c_int]),
    "tcw_plan_create": (ctypes.c_int, [_vp, _vp, _c_u32, _vp, _c_u64, _vp, _c_u64,
                                       ctypes.POINTER(TcwTileConfig), ctypes.c_int,
                                       ctypes.POINTER(_vp)]),
    "tcw_plan_destroy": (ctypes.c_int, [_vp]),
    "tcw_plan_info": (ctypes.c_int, [_vp, ctypes.POINTER(_c_u64), ctypes.POINTER(_c_u32),
                                     ctypes.POINTER(_c_u64), ctypes.POINTER(TcwTileConfig)]),
    "tcw_plan_run": (ctypes.c_int, [_vp, _vp, _vp, _vp, ctypes.c_int]),
    "tcw_map_batched": (ctypes.c_int, [_vp, _vp, _c_u32, _vp, _c_u64, _vp, _c_u64, _vp,
                                       ctypes.POINTER(TcwTileConfig), _vp, _vp, _vp]),
    "tcw_plan_run_maps": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, ctypes.c_int]),
    "tcw_plan_run_maps_host": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp]),
    "tcw_plan_run_host": (ctypes.c_int, [_vp, _vp, _vp, _vp]),
    "tcw_plan_run_host_async": (ctypes.c_int, [_vp, _vp, _vp, _vp]),
    "tcw_pinned_alloc": (ctypes.c_int, [ctypes.POINTER(_vp), ctypes.c_size_t]),
    "tcw_pinned_free": (ctypes.c_int, [_vp]),
    "tcw_plan_run_timed": (ctypes.c_int, [_vp, _vp, _vp, _vp, ctypes.POINTER(ctypes.c_float)]),
    "tcw_debug_fail_alloc": (ctypes.c_int, [_vp, ctypes.c_int]),
    "tcw_map_plain_noalloc": (ctypes.c_int, [_vp, _vp, _c_u32, _c_u32, _c_u32, ctypes.c_int, _vp,
                                             _c_u32, _vp, _c_u32, _vp, _vp, ctypes.c_int]),
    "tcw_debug_check_failures": (ctypes.c_int, [ctypes.POINTER(_c_u32)]),
    "tcw_map_f64": (ctypes.c_int, [_vp, _vp, _c_u32, _c_u32, _c_u32, ctypes.c_int, _vp, _c_u32,
                                   _vp, _c_u32, _vp, _c_u32, _vp, _vp]),
    "tcw_map_forward": (ctypes.c_int, [_vp, _vp, _c_u32, _vp, _vp, _c_u64, ctypes.c_double,
                                           _vp, _vp]),
    "tcw_map_backward": (ctypes.c_int, [_vp, _vp, _c_u32, _vp, _vp, _c_u64, ctypes.c_double,
                                            _vp, _vp, _vp, _vp, _vp, _c_u64, _vp]),
    "tcw_write_map_text": (ctypes.c_int, [ctypes.c_char_p, _vp, _c_u32, _c_u32, _vp, _vp,
                                          ctypes.c_int]),
    "tcw_read_map_text": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(_c_u64), _vp, _vp, _vp,
                                         _c_u64]),
    "tcw_read_atoms_text": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(_c_u64), _vp, _vp,
                                           _c_u64]),
    "tcw_write_atoms_text": (ctypes.c_int, [ctypes.c_char_p, _vp, _vp, _c_u64, ctypes.c_int]),
    "tcw_probe_peaks": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                       ctypes.POINTER(ctypes.c_double),
                                       ctypes.POINTER(ctypes.c_double),
                                       ctypes.POINTER(ctypes.c_double)]),
}

_lib = None
_lock = threading.Lock()


class TcwError(RuntimeError):
    def __init__(self, code, message):
        super().__init__(f"{message} [{code}]")
        self.code = code


def load(build_if_missing=True):
    """Load (building first if needed and possible) the CUDA library."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = os.environ.get("PYFSTAT_GB300_LIB") or _build.LIB_PATH
        if path == _build.LIB_PATH and build_if_missing and not _build.up_to_date():
            _build.build()
        if not os.path.exists(path):
            raise RuntimeError(f"{path} is missing: build it with pyfstat_gb300.build.build()")
        lib = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def strerror(code):
    return load().tcw_strerror(code).decode()


def check(rc, handle=None):
    if rc != TCW_OK:
        lib = load()
        msg = lib.tcw_strerror(rc).decode()
        if handle:
            detail = lib.tcw_last_error(handle).decode()
            if detail:
                msg = f"{msg}: {detail}"
        raise TcwError(rc, msg)


def device_count():
    n = ctypes.c_int(0)
    rc = load().tcw_device_count(ctypes.byref(n))
    return n.value if rc == TCW_OK else 0


def device_info(device):
    name = ctypes.create_string_buffer(256)
    major, minor = ctypes.c_int(0), ctypes.c_int(0)
    mem = ctypes.c_size_t(0)
    check(load().tcw_device_info(device, name, 256, ctypes.byref(major), ctypes.byref(minor),
                                 ctypes.byref(mem)))
    return dict(name=name.value.decode(), cc=(major.value, minor.value), total_mem=mem.value)


def device_memory(device):
    """(free, total) bytes of device memory."""
    f, t = ctypes.c_size_t(0), ctypes.c_size_t(0)
    check(load().tcw_device_memory(int(device), ctypes.byref(f), ctypes.byref(t)))
    return f.value, t.value


def probe_peaks(device=0):
    """Measured FP32 / FP64 / packed-FP32x2 TFLOP/s and MUFU ex2 Tops/s of ``device``."""
    a, b, c, d = ctypes.c_double(), ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    check(load().tcw_probe_peaks(int(device), ctypes.byref(a), ctypes.byref(b), ctypes.byref(c),
                                 ctypes.byref(d)))
    return dict(fp32_tflops=a.value, fp64_tflops=b.value, mufu_tops=c.value,
                fp32x2_tflops=d.value)


def _ptr(a):
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return a.data_ptr()  # torch tensor


class _PinnedBlock:
    """Owner of one page-locked host allocation (freed when collected)."""

    def __init__(self, nbytes):
        p = _vp()
        check(load().tcw_pinned_alloc(ctypes.byref(p), int(nbytes)))
        self.ptr = p.value

    def __del__(self):
        try:
            if self.ptr:
                load().tcw_pinned_free(self.ptr)
                self.ptr = None
        except Exception:
            pass


def pinned_empty(shape, dtype=np.float32):
    """An uninitialised numpy array in page-locked host memory."""
    dtype = np.dtype(dtype)
    shape = (shape,) if np.isscalar(shape) else tuple(shape)
    nbytes = int(np.prod(shape)) * dtype.itemsize
    block = _PinnedBlock(nbytes)
    buf = (ctypes.c_char * max(nbytes, 1)).from_address(block.ptr)
    arr = np.frombuffer(buf, dtype=dtype, count=int(np.prod(shape))).reshape(shape)
    arr_owner = arr.view()
    # keep the allocation alive as long as any view of it is
    buf._tcw_block = block
    return arr_owner


class Handle:
    """A library handle on one device (its own stream and workspace)."""

    def __init__(self, device=0):
        lib = load()
        h = _vp()
        check(lib.tcw_create(ctypes.byref(h), int(device)))
        self._h = h
        self.device = int(device)

    @property
    def ptr(self):
        if self._h is None:
            raise RuntimeError("handle already destroyed")
        return self._h

    def close(self):
        if getattr(self, "_h", None):
            load().tcw_destroy(self._h)
            self._h = None

    detach = close

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_stream(self, stream_ptr):
        check(load().tcw_set_stream(self.ptr, stream_ptr), self.ptr)

    def stream(self):
        s = _vp()
        check(load().tcw_get_stream(self.ptr, ctypes.byref(s)), self.ptr)
        return s.value

    def sync(self, timeout_ms=60000):
        check(load().tcw_sync(self.ptr, int(timeout_ms)), self.ptr)

    def fail_alloc(self, n):
        check(load().tcw_debug_fail_alloc(self.ptr, int(n)), self.ptr)

    # ------------------------------------------------------------- plain map
    def map_plain_host(self, atoms7, TAtom, t0_data, window, t0s, taus, want_map=True,
                       flags=TCW_FLAG_LNBTSG):
        """Host arrays in, (F map or None, result record) out."""
        atoms7 = np.ascontiguousarray(atoms7, dtype=np.float32)
        if atoms7.ndim != 2 or atoms7.shape[1] != 7:
            raise ValueError("atoms must be a (numAtoms, 7) float32 matrix")
        t0s = np.ascontiguousarray(t0s, dtype=np.uint32)
        taus = np.ascontiguousarray(taus, dtype=np.uint32)
        if window == TCW_WINDOW_NONE:
            shape = (1, 1)
        else:
            shape = (t0s.shape[0], taus.shape[0])
        F = np.empty(shape, dtype=np.float32) if want_map else None
        res = np.zeros(1, dtype=RESULT_DTYPE)
        rc = load().tcw_map_plain_host(self.ptr, atoms7.ctypes.data, atoms7.shape[0], int(TAtom),
                                       int(t0_data), int(window), t0s.ctypes.data, t0s.shape[0],
                                       taus.ctypes.data, taus.shape[0], _ptr(F), res.ctypes.data,
                                       int(flags))
        check(rc, self.ptr)
        return F, res[0]

    def map_plain(self, d_atoms, numAtoms, TAtom, t0_data, window, d_t0s, N_t0, d_taus, N_tau,
                  d_Fmn, d_result, flags=TCW_FLAG_LNBTSG):
        """Device pointers (ints or torch tensors); asynchronous on the handle's stream."""
        rc = load().tcw_map_plain(self.ptr, _p(d_atoms), int(numAtoms), int(TAtom),
                                  int(t0_data), int(window), _p(d_t0s), int(N_t0), _p(d_taus),
                                  int(N_tau), _p(d_Fmn), _p(d_result), int(flags))
        check(rc, self.ptr)

    def map_f64(self, d_atoms, numAtoms, TAtom, t0_data, window, d_t0s, N_t0, d_taus, N_tau,
                d_F, rows=None, d_cond=None):
        """Full-FP64 direct-summation map of the listed t0 rows (host indices;
        None = all rows) into device FP64 ``d_F`` (n_rows x N_tau); asynchronous
        on the handle's stream."""
        if rows is None:
            rp, nr = None, int(N_t0)
        else:
            rows = np.ascontiguousarray(rows, dtype=np.uint32)
            rp, nr = rows.ctypes.data, rows.shape[0]
        rc = load().tcw_map_f64(self.ptr, _p(d_atoms), int(numAtoms), int(TAtom), int(t0_data),
                                int(window), _p(d_t0s), int(N_t0), _p(d_taus), int(N_tau), rp, nr,
                                _p(d_F), _p(d_cond))
        check(rc, self.ptr)


NOALLOC_SCRATCH_BYTES = 16 << 20


def map_plain_noalloc(stream, d_atoms, numAtoms, TAtom, t0_data, window, d_t0s, N_t0, d_taus,
                      N_tau, d_Fmn, d_result, flags=TCW_FLAG_LNBTSG):
    """The plain map without any device allocation, for callers that may not
    allocate: its scratch is a fixed static device array
    (NOALLOC_SCRATCH_BYTES); larger problems raise TcwError(TCW_ERR_OVERFLOW).
    Runs asynchronously on ``stream`` (a raw cudaStream_t pointer) on the
    current device.  Calls whose work overlaps on the GPU share the scratch
    and must be serialised."""
    rc = load().tcw_map_plain_noalloc(stream, _p(d_atoms), int(numAtoms), int(TAtom),
                                      int(t0_data), int(window), _p(d_t0s), int(N_t0),
                                      _p(d_taus), int(N_tau), _p(d_Fmn), _p(d_result),
                                      int(flags))
    if rc == TCW_ERR_OVERFLOW:
        raise TcwError(rc, "problem needs more scratch than the no-allocation entry point's "
                           f"{NOALLOC_SCRATCH_BYTES} bytes (or times exceed the u32 range)")
    check(rc)


def _p(x):
    if x is None:
        return None
    if isinstance(x, int):
        return x
    return _ptr(x)


class Plan:
    """A batched plan (geometry, grids, tile schedule) on one handle's device."""

    def __init__(self, handle, desc, t0s, taus, tile_config=None, flags=0):
        desc = np.ascontiguousarray(desc, dtype=DESC_DTYPE)
        t0s = np.ascontiguousarray(t0s, dtype=np.uint32)
        taus = np.ascontiguousarray(taus, dtype=np.uint32)
        cfg = None
        if tile_config is not None:
            cfg = TcwTileConfig(**{k: int(v) for k, v in dict(tile_config).items()})
        p = _vp()
        rc = load().tcw_plan_create(handle.ptr, desc.ctypes.data, desc.shape[0], t0s.ctypes.data,
                                    t0s.shape[0], taus.ctypes.data, taus.shape[0],
                                    ctypes.byref(cfg) if cfg is not None else None, int(flags),
                                    ctypes.byref(p))
        check(rc, handle.ptr)
        self._p = p
        self.handle = handle
        self.n_templates = desc.shape[0]
        n_cells, n_items, n_rows = _c_u64(), _c_u32(), _c_u64()
        tc = TcwTileConfig()
        check(load().tcw_plan_info(p, ctypes.byref(n_cells), ctypes.byref(n_items),
                                   ctypes.byref(n_rows), ctypes.byref(tc)))
        self.n_cells = n_cells.value
        self.n_items = n_items.value
        self.n_atom_rows = n_rows.value
        self.tile_config = tc.as_dict()

    def run(self, d_atoms, d_results, use_graph=True):
        check(load().tcw_plan_run(self.handle.ptr, self._p, _p(d_atoms), _p(d_results),
                                  int(bool(use_graph))), self.handle.ptr)

    def run_maps(self, d_atoms, d_results, d_maps, use_graph=True):
        """As :meth:`run`, also writing all templates' FP32 maps into ``d_maps``
        (``n_cells`` floats; template k's map at the sum of the earlier
        templates' N_t0 * N_tau, row-major)."""
        check(load().tcw_plan_run_maps(self.handle.ptr, self._p, _p(d_atoms), _p(d_results),
                                       _p(d_maps), int(bool(use_graph))), self.handle.ptr)

    def run_timed(self, d_atoms, d_results):
        """One run with per-kernel CUDA events: (prefix, rect map, exp map, finalize) ms."""
        ms = (ctypes.c_float * 4)()
        check(load().tcw_plan_run_timed(self.handle.ptr, self._p, _p(d_atoms), _p(d_results), ms),
              self.handle.ptr)
        return tuple(float(x) for x in ms)

    def run_host(self, atoms7):
        atoms7 = np.ascontiguousarray(atoms7, dtype=np.float32)
        if atoms7.shape[0] < self.n_atom_rows:
            raise ValueError("atoms array shorter than the plan's atom rows")
        res = np.zeros(self.n_templates, dtype=RESULT_DTYPE)
        check(load().tcw_plan_run_host(self.handle.ptr, self._p, atoms7.ctypes.data,
                                       res.ctypes.data), self.handle.ptr)
        return res

    def run_host_async(self, atoms7):
        """Pipelined :meth:`run_host`: enqueues the upload, the run and the
        download of the results into a page-locked slot of this plan, and
        returns at once.  The atoms are kept alive until :meth:`wait`, which
        returns the results of the runs enqueued since the last wait, in
        order.  Pass page-locked atoms (:func:`pinned_empty`) for the upload
        to overlap the previous run's map kernels."""
        atoms7 = np.ascontiguousarray(atoms7, dtype=np.float32)
        if atoms7.shape[0] < self.n_atom_rows:
            raise ValueError("atoms array shorter than the plan's atom rows")
        if not hasattr(self, "_inflight"):
            self._inflight, self._slots = [], []
        k = len(self._inflight)
        if k == len(self._slots):
            self._slots.append(pinned_empty(self.n_templates, RESULT_DTYPE))
        slot = self._slots[k]
        check(load().tcw_plan_run_host_async(self.handle.ptr, self._p, atoms7.ctypes.data,
                                             slot.ctypes.data), self.handle.ptr)
        self._inflight.append(atoms7)

    def wait(self, timeout_ms=600000):
        """Waits for the pipelined runs; their results (copies), in order."""
        self.handle.sync(timeout_ms)
        n = len(getattr(self, "_inflight", []))
        out = [self._slots[k].copy() for k in range(n)]
        self._inflight = []
        return out

    def run_maps_host(self, atoms7):
        """Host atoms in; (results, maps) out, maps a flat float32 array of
        ``n_cells`` values (template k's map at the sum of the earlier
        templates' cells)."""
        atoms7 = np.ascontiguousarray(atoms7, dtype=np.float32)
        if atoms7.shape[0] < self.n_atom_rows:
            raise ValueError("atoms array shorter than the plan's atom rows")
        res = np.zeros(self.n_templates, dtype=RESULT_DTYPE)
        maps = np.empty(self.n_cells, dtype=np.float32)
        check(load().tcw_plan_run_maps_host(self.handle.ptr, self._p, atoms7.ctypes.data,
                                            res.ctypes.data, maps.ctypes.data), self.handle.ptr)
        return res, maps

    def close(self):
        if getattr(self, "_p", None):
            load().tcw_plan_destroy(self._p)
            self._p = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
