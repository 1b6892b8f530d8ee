"""Build the CUDA library in-tree: ``measure_ia_gb300/libmeasureia_gb300.so``.

nvcc compiles each translation unit for sm_103a in parallel, then links a
shared library that exports the C ABI of ``include/measure_ia_gb300.h``.

    python -m measure_ia_gb300.build
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB_NAME = "libmeasureia_gb300.so"
LIB_PATH = os.path.join(HERE, LIB_NAME)
BUILD_DIR = os.path.join(HERE, "_build")
SOURCES = ["mia_prep.cu", "mia_pairs.cu", "mia_post.cu", "mia_lightcone.cu", "mia_capi.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden"]


def nvcc_path():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale(lib, deps):
    if not os.path.exists(lib):
        return True
    t = os.path.getmtime(lib)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False, defines=(), out=None):
    """Compile if any source is newer than the library.  Returns the library path.

    ``defines`` adds -D options and ``out`` names another output library
    (tuning builds)."""
    lib_path = out or LIB_PATH
    build_dir = BUILD_DIR if not defines else os.path.join(BUILD_DIR, "_".join(d.replace("=", "") for d in defines))
    srcs = [os.path.join(CSRC, s) for s in SOURCES]
    hdrs = [os.path.join(CSRC, "mia_internal.cuh"), os.path.join(HERE, "..", "include", "measure_ia_gb300.h")]
    if not force and not _stale(lib_path, srcs + hdrs + [os.path.abspath(__file__)]):
        return lib_path
    os.makedirs(build_dir, exist_ok=True)
    nvcc = nvcc_path()

    def compile_one(src):
        obj = os.path.join(build_dir, os.path.basename(src) + ".o")
        cmd = [nvcc, *ARCH, *FLAGS, *[f"-D{d}" for d in defines], "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr, file=sys.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = lib_path + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, lib_path)
    return lib_path


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
