"""Builds libfvc.so (the CUDA kernels and the C ABI) in-tree for sm_103a.

    python -m frustumvolumecaching_gb300.build

Two translation units compiled in parallel by nvcc; host code without fused
multiply-add contraction so its float setup matches the oracle's.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
OUT_DIR = os.path.join(PKG, "_lib")
LIB = os.path.join(OUT_DIR, "libfvc.so")
SOURCES = ["fvc_kernels.cu", "fvc_render.cu", "fvc_capi.cu", "fvc_noalloc.cu"]
HEADERS = ["fvc_kernels.h", "fvc_device.cuh", "fvc_detmath.h", "fvc_tc.cuh", os.path.join("..", "..", "include", "fvc.h")]
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(os.path.join(CSRC, f)) < t for f in SOURCES + HEADERS)


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = LIB + ".tmp"
    cmd = [nvcc(), ARCH, "-O3", "-std=c++17", "-lineinfo", "--threads", "4", "-shared", "-Xcompiler", "-fPIC",
           "-Xcompiler", "-ffp-contract=off", "-o", tmp] + [os.path.join(CSRC, f) for f in SOURCES]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed:\n" + r.stdout + r.stderr)
    if verbose:
        sys.stderr.write(r.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
