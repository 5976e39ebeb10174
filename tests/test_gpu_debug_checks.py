"""A debug build of the library (-DTCW_DEBUG_CHECKS: every load/store index of
the map, adjoint and FP64-reference kernels checked on the device, failures
counted instead of trapped) runs every kernel family on the golden cases and
small batches without a single failed check."""

import os
import subprocess
import sys

import pytest

from pyfstat_gb300 import build as B

pytestmark = pytest.mark.gpu
REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_all_kernels_pass_device_index_checks(tmp_path):
    lib = B.build(extra_flags=("-DTCW_DEBUG_CHECKS",), lib_path=str(tmp_path / "libtcw_b200.so"))
    env = dict(os.environ, PYFSTAT_GB300_LIB=lib)
    out = subprocess.run([sys.executable, os.path.join(REPO, "tests", "_debug_checks_run.py")],
                         env=env, capture_output=True, text=True, timeout=900)
    assert out.returncode == 0, out.stderr[-3000:]
    line = [l for l in out.stdout.splitlines() if l.startswith("DCHECK")][-1]
    _, rc, n = line.split()
    assert int(rc) == 0 and int(n) == 0, line
