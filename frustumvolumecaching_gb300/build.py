"""Builds libfvc.so (the CUDA kernels and the C ABI) in-tree for sm_103a, and
the `eval` program on the C++ renderer API (include/fvc.hpp).

    python -m frustumvolumecaching_gb300.build

The CUDA translation units are compiled in parallel by nvcc; host code
without fused multiply-add contraction so its float setup matches the
oracle's.  eval is plain g++ against libfvc.so and the CUDA runtime.
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
SOURCES = ["fvc_kernels.cu", "fvc_render.cu", "fvc_capi.cu", "fvc_noalloc.cu", "fvc_backward.cu", "fvc_ingp.cpp"]
HEADERS = ["fvc_kernels.h", "fvc_device.cuh", "fvc_detmath.h", "fvc_tc.cuh", "fvc_ingp.h", os.path.join("..", "..", "include", "fvc.h")]
INCLUDE = os.path.join(PKG, "..", "include")
EVAL_SRC = os.path.join(PKG, "cpp", "eval.cpp")
EVAL = os.path.join(OUT_DIR, "eval")
PATH_SRC = os.path.join(PKG, "cpp", "render_path.cpp")
PATH_EXE = os.path.join(OUT_DIR, "render_path")
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
    # tuning macros of the kernels (e.g. -DFVC_TC_CTAS_PER_SM=5), for launch-shape sweeps
    cmd[1:1] = os.environ.get("FVC_NVCC_DEFINES", "").split()
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed:\n" + r.stdout + r.stderr)
    if verbose:
        sys.stderr.write(r.stderr)
    os.replace(tmp, LIB)
    return LIB


def cuda_root() -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc())))


def _build_program(src: str, exe: str, extra_deps: list, force: bool) -> str:
    """g++ build of a program on the C++ renderer API; needs libfvc.so first."""
    lib = build()
    deps = [src, os.path.join(INCLUDE, "fvc.hpp"), os.path.join(INCLUDE, "fvc.h"), lib, *extra_deps]
    if not force and os.path.exists(exe) and all(os.path.getmtime(d) < os.path.getmtime(exe) for d in deps):
        return exe
    cuda = cuda_root()
    cudalib = next((d for d in (os.path.join(cuda, "lib64"), os.path.join(cuda, "lib")) if os.path.isdir(d)), None)
    if cudalib is None:
        raise RuntimeError("CUDA runtime library directory not found under " + cuda)
    tmp = exe + ".tmp"
    cmd = [os.environ.get("CXX", "g++"), "-std=c++17", "-O2", "-Wall", "-I", INCLUDE, "-I", os.path.join(cuda, "include"),
           src, "-o", tmp, "-L", OUT_DIR, "-lfvc", "-L", cudalib, "-lcudart",
           "-Wl,-rpath,$ORIGIN", "-Wl,-rpath," + cudalib]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("g++ failed:\n" + r.stdout + r.stderr)
    os.replace(tmp, exe)
    return exe


def build_eval(force: bool = False) -> str:
    """The eval program (src/eval.cu's command line)."""
    return _build_program(EVAL_SRC, EVAL, [], force)


def build_render_path(force: bool = False) -> str:
    """The headless camera-path renderer (the real-time viewer's path rendering)."""
    return _build_program(PATH_SRC, PATH_EXE, [os.path.join(INCLUDE, "fvc_camera_path.hpp"),
                                               os.path.join(PKG, "csrc", "fvc_sampling.h")], force)


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
    print(build_eval(force="--force" in sys.argv))
    print(build_render_path(force="--force" in sys.argv))
