"""In-tree build of the CUDA library ``pyfstat_gb300/libtcw_b200.so`` for sm_103a.

Two translation units (kernels, C-ABI layer) are compiled in parallel with
nvcc and linked into one shared library; nothing is installed anywhere.
"""

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB_NAME = "libtcw_b200.so"
LIB_PATH = os.path.join(HERE, LIB_NAME)
BUILD_DIR = os.path.join(HERE, "_build")
SOURCES = ("tcw_kernels.cu", "tcw_abi.cu", "tcw_probe.cu", "tcw_noalloc.cu", "tcw_diff.cu",
           "tcw_f64.cu", "tcw_io.cpp")
HEADERS = ("tcw_cell.h", "tcw_internal.h")
GENCODE = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc_path():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build " + LIB_NAME)
    return cand


def _inputs():
    inc = os.path.join(os.path.dirname(HERE), "include", "tcw_b200.h")
    return [os.path.join(CSRC, s) for s in SOURCES + HEADERS] + [inc]


def up_to_date():
    if not os.path.exists(LIB_PATH):
        return False
    t = os.path.getmtime(LIB_PATH)
    return all(os.path.getmtime(p) <= t for p in _inputs())


def build(force=False, verbose=False, extra_flags=(), lib_path=None, build_dir=None):
    """Compile the library if any source is newer than it; return its path.

    ``lib_path`` / ``build_dir`` build a variant (e.g. with
    ``extra_flags=("-DTCW_DEBUG_CHECKS",)``) elsewhere; the default is the
    in-tree library."""
    if lib_path is None:
        if not force and up_to_date():
            return LIB_PATH
        lib_path = LIB_PATH
    build_dir = build_dir or (BUILD_DIR if lib_path == LIB_PATH else lib_path + ".objs")
    nvcc = nvcc_path()
    os.makedirs(build_dir, exist_ok=True)
    common = [GENCODE, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-O2", *extra_flags]

    def compile_one(src):
        obj = os.path.join(build_dir, os.path.splitext(src)[0] + ".o")
        cmd = [nvcc, *common, "-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        return obj

    with ThreadPoolExecutor(len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = lib_path + ".tmp"
    cmd = [nvcc, GENCODE, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib_path)
    return lib_path


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
