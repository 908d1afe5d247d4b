"""Builds the native library fcl_gb300/_build/libfclgpu.so for sm_103a.

Device translation units are compiled with -fmad=false: the FP64 paths must not
fuse multiply-adds (the reference's FP64 arithmetic is unfused), and FP32 code that
wants fusion calls fmaf explicitly.  Host code is compiled with -ffp-contract=off
for the same reason (gcc contracts by default on aarch64).
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
LIB = os.path.join(BUILD, "libfclgpu.so")

ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def _nvcc() -> str:
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _headers() -> list[str]:
    return glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))


def _stale(obj: str, src: str, deps: list[str]) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(p) > t for p in [src, *deps, __file__])


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def build(verbose: bool = False, jobs: int = 8) -> str:
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    deps = _headers()
    cu = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    cpp = sorted(glob.glob(os.path.join(CSRC, "*.cpp")))
    cmds = []
    objs = []
    for src in cu:
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(obj)
        if _stale(obj, src, deps):
            cmds.append([nvcc, ARCH, "-O3", "-lineinfo", "-std=c++17", "-fmad=false", "--expt-relaxed-constexpr",
                         "-Xcompiler", "-fPIC,-ffp-contract=off,-fvisibility=hidden", "-I", CSRC, "-I", INCLUDE,
                         "-c", src, "-o", obj])
    for src in cpp:
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(obj)
        if _stale(obj, src, deps):
            cmds.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math",
                         "-fvisibility=hidden", "-I", CSRC, "-I", INCLUDE, "-c", src, "-o", obj])
    if cmds:
        with ThreadPoolExecutor(max_workers=jobs) as ex:
            list(ex.map(_run, cmds))
    if cmds or not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        _run([nvcc, ARCH, "-shared", "-o", LIB, *objs, "-lpthread"])
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
