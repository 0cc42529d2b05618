"""Builds the lattice library, banjo_gb300/_build/libgbl.so, in tree.

nvcc compiles the CUDA translation unit for sm_103a only; the host builders
are plain C++. The arithmetic flags are part of the contract, not tuning: no
FMA contraction (-fmad=false on the device, -ffp-contract=off on the host),
IEEE division and square root, denormals kept, because the float path is held
to the reference CPU lane bit for bit.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libgbl.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
DEVICE_FP = ["-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false"]
HOST_FP = "-ffp-contract=off,-fno-fast-math"

SOURCES_CU = ["gbl_device.cu", "gbl_noalloc.cu"]
SOURCES_CPP = ["gbl_host.cpp"]
HEADERS = ["gbl_internal.hpp", "gbl_math.cuh", "gbl_kernels.cuh"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the lattice library needs the CUDA toolkit to build")


def _stale(target: str, inputs: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(p) > t for p in inputs)


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    inc = ["-I", os.path.join(ROOT, "include"), "-I", CSRC]
    deps = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(ROOT, "include", "gbl.h"), __file__]
    objs, procs = [], []
    for src in SOURCES_CU + SOURCES_CPP:
        path = os.path.join(CSRC, src)
        obj = os.path.join(OUT, src + ".o")
        objs.append(obj)
        if not force and not _stale(obj, [path] + deps):
            continue
        if src.endswith(".cu"):
            cmd = [nvcc, *ARCH, "-lineinfo", "-O3", "-std=c++17", *DEVICE_FP, "-Xcompiler", "-fPIC," + HOST_FP,
                   *inc, "-c", path, "-o", obj]
        else:
            cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-Wall", "-Wextra",
                   *inc, "-I", "/usr/local/cuda/include", "-c", path, "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + out)
        if verbose and out.strip():
            print(out, file=sys.stderr)
    if force or _stale(LIB, objs):
        cmd = [nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed: " + " ".join(cmd) + "\n" + r.stdout)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
