"""Build the CUDA library (lib/libpdx.so) and the CLI (bin/PDLSM-FEM) in-tree.

Every translation unit is compiled by nvcc for sm_103a only, in parallel, and
linked into one shared library with a plain C ABI (include/pdx.h).  Host code
is compiled without floating-point contraction so that the setup steps that
compare distances (family membership, crack tests) agree between x86 and Arm.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "lib")
BIN = os.path.join(HERE, "bin")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _compile(src: str) -> str:
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(
            os.path.getmtime(src), *(os.path.getmtime(os.path.join(CSRC, h))
                                     for h in os.listdir(CSRC) if h.endswith((".h", ".cuh")))):
        return obj
    flags = ["-std=c++17", "-O3", "-Xcompiler", "-fPIC,-ffp-contract=off", "-c"]
    if src.endswith(".cu"):
        flags += ARCH + ["-lineinfo", "--extended-lambda", "-Xptxas", "-warn-spills"]
    cmd = [nvcc()] + flags + [src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIB, exist_ok=True)
    os.makedirs(BIN, exist_ok=True)
    srcs = sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(_compile, srcs))
    lib = os.path.join(LIB, "libpdx.so")
    cmd = [nvcc()] + ARCH + ["-shared", "-o", lib] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {r.stdout}\n{r.stderr}")
    exe = os.path.join(BIN, "PDLSM-FEM")
    cmd = [nvcc(), "-std=c++17", "-O2", os.path.join(HERE, "app", "main.cpp"), "-o", exe, "-L" + LIB, "-lpdx",
           "-Xlinker", "-rpath,$ORIGIN/../lib"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"CLI link failed: {r.stdout}\n{r.stderr}")
    if verbose:
        print("built", lib, exe)
    return lib


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
