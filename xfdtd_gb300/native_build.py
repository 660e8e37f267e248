"""Builds the two native libraries in-tree, into xfdtd_gb300/_lib/:

  libxfdtd_cuda.so  the GPU engine and its C-ABI (include/xfdtd_cuda.h),
                    hand-written CUDA for sm_103a, CUDA runtime linked
                    statically;
  libxfdtd.so       the C++ scene API mirroring the reference
                    (host/include/xfdtd/xfdtd.h) and its C-ABI
                    (include/xfdtd_sim.h), linked against libxfdtd_cuda.so.

The engine is one nvcc job (two to three minutes); its device code is not
split across parallel jobs (--split-compile), which optimises parts of the
module apart: built that way, the 280^3 dielectric-sphere step took 0.445
ms instead of 0.427 ms with the same kernel variants, and the adjoint's
reverse kernels executed 30 % more instructions.  nvcc cross-compiles, so
the build also runs on a machine without a GPU.
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIB_DIR = os.path.join(HERE, "_lib")
CUDA_LIB = os.path.join(LIB_DIR, "libxfdtd_cuda.so")
HOST_LIB = os.path.join(LIB_DIR, "libxfdtd.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def _nvcc() -> str:
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build xfdtd_gb300")


def cuda_cmd(out: str = CUDA_LIB, extra=()) -> list:
    srcs = [os.path.join(HERE, "csrc", f) for f in ("engine.cu", "nffft_noalloc.cu")]
    return [_nvcc(), ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-shared", *extra, "-o", out,
            *srcs, "-ldl"]


def host_cmd() -> list:
    srcs = sorted(glob.glob(os.path.join(HERE, "host", "src", "*.cpp")))
    # no FMA contraction (GCC contracts by default on aarch64): the host
    # arithmetic (coefficients, profiles, far-field post-processing) rounds
    # as the reference's does, on either architecture
    return ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-pthread", "-Wall",
            "-Wno-unused-variable",
            "-I", os.path.join(HERE, "host", "include"), *srcs,
            "-L", LIB_DIR, "-lxfdtd_cuda", "-Wl,-rpath,$ORIGIN", "-o", HOST_LIB]


def _newer(target: str, deps) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def build(force: bool = False, verbose: bool = False) -> None:
    os.makedirs(LIB_DIR, exist_ok=True)
    cu_deps = glob.glob(os.path.join(HERE, "csrc", "*")) + [os.path.join(ROOT, "include", "xfdtd_cuda.h")]
    host_deps = (glob.glob(os.path.join(HERE, "host", "src", "*.cpp"))
                 + glob.glob(os.path.join(HERE, "host", "include", "xfdtd", "*.h"))
                 + glob.glob(os.path.join(ROOT, "include", "*.h")))
    if force or not _newer(CUDA_LIB, cu_deps):
        _run(cuda_cmd(), verbose)
    if force or not _newer(HOST_LIB, host_deps + [CUDA_LIB]):
        _run(host_cmd(), verbose)


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
