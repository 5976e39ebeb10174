"""The C-ABI library builds, loads and exports every function the header
declares; calls that need no GPU behave (no compute without a GPU)."""

import ctypes
import os
import re

import pytest

from conftest import REPO

HEADER = os.path.join(REPO, "include", "tcw_b200.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(tcw_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from pyfstat_gb300 import _lib, build

    build.build()
    return _lib.load()


def test_header_declares_the_entry_points():
    names = declared_functions()
    for required in ("tcw_create", "tcw_destroy", "tcw_map_plain", "tcw_map_plain_host",
                     "tcw_plan_create", "tcw_plan_run", "tcw_plan_run_host", "tcw_sync",
                     "tcw_strerror"):
        assert required in names


def test_library_exports_every_declared_symbol(lib):
    from pyfstat_gb300 import _lib

    for name in declared_functions():
        assert hasattr(lib, name), name
        assert name in _lib.SIGNATURES, f"{name} has no ctypes signature"


def test_struct_layouts():
    from pyfstat_gb300 import _lib

    assert ctypes.sizeof(_lib.TcwResult) == 40
    assert ctypes.sizeof(_lib.TcwTemplateDesc) == 48
    assert ctypes.sizeof(_lib.TcwTileConfig) == 20


def test_calls_without_a_gpu(lib):
    from pyfstat_gb300 import _lib

    assert lib.tcw_abi_version() == 1
    for code in range(-7, 1):
        assert lib.tcw_strerror(code)
    assert b"unknown" in lib.tcw_strerror(-99)
    assert lib.tcw_destroy(None) == _lib.TCW_ERR_INVALID_ARG
    assert lib.tcw_sync(None, 0) == _lib.TCW_ERR_INVALID_ARG
    f, t = ctypes.c_size_t(), ctypes.c_size_t()
    assert lib.tcw_device_memory(0, None, ctypes.byref(t)) == _lib.TCW_ERR_INVALID_ARG
    if _lib.device_count() == 0:
        assert lib.tcw_device_memory(0, ctypes.byref(f), ctypes.byref(t)) == \
            _lib.TCW_ERR_NO_DEVICE
        h = ctypes.c_void_p()
        assert lib.tcw_create(ctypes.byref(h), 0) == _lib.TCW_ERR_NO_DEVICE
        assert not h.value
        with pytest.raises(_lib.TcwError):
            _lib.Handle(0)


def test_no_fallback_without_gpu():
    """The b200 feature is reported unavailable without a device; asking for
    it raises instead of falling back to the CPU."""
    from pyfstat_gb300 import _lib
    from pyfstat_gb300 import tcw_fstat_map_funcs as tcw

    if _lib.device_count() > 0:
        pytest.skip("a GPU is present")
    features = tcw._get_transient_fstat_map_features()
    assert features["b200"] is False
    with pytest.raises(RuntimeError, match="b200 use was requested"):
        tcw.init_transient_fstat_map_features("b200")
    with pytest.raises(Exception, match="not available"):
        tcw.call_compute_transient_fstat_map("b200", features, None, None)


def test_release_build_has_no_device_checks():
    import ctypes

    from pyfstat_gb300 import _lib

    n = ctypes.c_uint32(7)
    assert _lib.load().tcw_debug_check_failures(ctypes.byref(n)) == _lib.TCW_ERR_UNSUPPORTED
    assert n.value == 0


def test_missing_library_fails_loudly(tmp_path):
    """With the CUDA library absent the product path raises; there is no
    other implementation to fall back to."""
    import subprocess
    import sys

    code = ("from pyfstat_gb300 import _lib\n"
            "try:\n"
            "    _lib.load()\n"
            "except RuntimeError as e:\n"
            "    print('raised', e)\n"
            "else:\n"
            "    print('loaded')\n")
    env = dict(os.environ, PYFSTAT_GB300_LIB=str(tmp_path / "absent.so"))
    r = subprocess.run([sys.executable, "-c", code], cwd=REPO, env=env, capture_output=True,
                       text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.startswith("raised") and "missing" in r.stdout
