import os
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def pytest_terminal_summary(terminalreporter):
    """Reports how many argmax / posterior-index comparisons had a unique
    maximum (exact index equality) and how many took the tie branch."""
    mod = sys.modules.get("_helpers")
    if mod is None:
        return
    c = mod.ARGMAX_COUNTS
    if c["unique"] or c["tie"]:
        terminalreporter.write_line(
            f"argmax comparisons: {c['unique']} unique maximum (exact index), "
            f"{c['tie']} tie branch" +
            (f" [{'; '.join(mod.ARGMAX_TIE_LABELS[:20])}]" if c["tie"] else ""))


@pytest.fixture(scope="session")
def oracle():
    import oracle as O

    O.build()
    return O


@pytest.fixture(scope="session")
def hostcell(tmp_path_factory):
    """Host build of the device cell arithmetic (tests/host_cell.cpp)."""
    import ctypes

    out = tmp_path_factory.mktemp("hostcell") / "libhostcell.so"
    src = os.path.join(REPO, "tests", "host_cell.cpp")
    subprocess.run(["g++", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-std=c++17",
                    "-o", str(out), src, "-lm"], check=True)
    return ctypes.CDLL(str(out))


@pytest.fixture(scope="session")
def golden():
    import numpy as np

    return np.load(os.path.join(REPO, "tests", "golden", "reference_maps.npz"))
