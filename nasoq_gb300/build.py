"""Builds libnasoq_gb300.so in-tree: the host symbolic analysis, the sm_103a
CUDA kernels, the C ABI (include/nasoq_gb300.h) and the C++ drop-in classes,
linked against the CUDA toolkit's static METIS library.

    python -m nasoq_gb300.build        # or nasoq_gb300.build.build()
    python -m nasoq_gb300.build clean  # recompile every object

Objects are reused when they are newer than their source and every header;
NASOQ_GB300_REBUILD=1 (or build(clean=True)) recompiles everything.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import platform
import re
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libnasoq_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def cuda_home():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nv = shutil.which("nvcc")
    if nv:
        return os.path.dirname(os.path.dirname(os.path.realpath(nv)))
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build nasoq_gb300")


def metis_lib(cuda):
    tdir = "sbsa-linux" if platform.machine() in ("aarch64", "arm64") else "x86_64-linux"
    cands = [os.path.join(cuda, "targets", tdir, "lib", "libmetis_static.a"),
             os.path.join(cuda, "lib64", "libmetis_static.a")]
    cands += glob.glob(os.path.join(cuda, "targets", "*", "lib", "libmetis_static.a"))
    for c in cands:
        if os.path.exists(c):
            return c
    raise RuntimeError("libmetis_static.a not found in the CUDA toolkit")


def sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))


def _deps(src):
    """Files an object depends on: its source, every header of the package
    and of include/, and the .cu files it includes (batch_fp64.cu)."""
    deps = [src] + glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.hpp")) \
        + glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(ROOT, "include", "**", "*.h"), recursive=True)
    with open(src) as f:
        deps += [os.path.join(CSRC, m) for m in re.findall(r'#include "([^"/]+\.cu)"', f.read())]
    return deps


def _compile(nvcc, src, flags, clean=False):
    obj = os.path.join(OBJ, os.path.basename(src) + ".o")
    if not clean and os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in _deps(src)):
        return obj
    lang = ["-x", "cu"] if src.endswith(".cu") else ["-x", "c++"]
    cmd = [nvcc] + lang + flags + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False, clean: bool = False) -> str:
    clean = clean or os.environ.get("NASOQ_GB300_REBUILD", "") not in ("", "0")
    cuda = cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(OBJ, exist_ok=True)
    flags = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O3", "-I" + os.path.join(ROOT, "include"),
                    "-I" + CSRC, "--expt-relaxed-constexpr", "-DNDEBUG"]
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(nvcc, s, flags, clean), srcs))
    link = [nvcc] + ARCH + ["-shared", "-o", LIB] + objs + [metis_lib(cuda), "-cudart", "static", "-lpthread"]
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(link)}\n{r.stdout}\n{r.stderr}")
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True, clean=len(sys.argv) > 1 and sys.argv[1] == "clean")
    sys.exit(0)
