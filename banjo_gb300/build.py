"""Builds the lattice library, banjo_gb300/_build/libgbl.so, in tree.

nvcc compiles the CUDA translation unit for sm_103a only; the host builders
are plain C++. The arithmetic flags are part of the contract, not tuning: no
FMA contraction (-fmad=false on the device, -ffp-contract=off on the host),
IEEE division and square root, denormals kept, because the float path is held
to the reference CPU lane bit for bit.

Beside it, libgbl_checked.so is the same library with the kernels compiled
with GBL_BOUNDS_CHECK: every index read out of device data is checked before
use and a violation is recorded instead of made (gbl_bounds_report), the
stand-in for a memory checker on machines where none may run. A process picks
it with GBL_LIBRARY=checked.
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
LIB_CHECKED = os.path.join(OUT, "libgbl_checked.so")

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
    # (source, object, extra flags): every source once, and the kernels' unit
    # again with the bounds checks compiled in.
    units = [(src, os.path.join(OUT, src + ".o"), []) for src in SOURCES_CU + SOURCES_CPP]
    checked_obj = os.path.join(OUT, "gbl_device_checked.cu.o")
    units.append(("gbl_device.cu", checked_obj, ["-DGBL_BOUNDS_CHECK"]))
    for src, obj, extra in units:
        path = os.path.join(CSRC, src)
        if not extra:
            objs.append(obj)
        if not force and not _stale(obj, [path] + deps):
            continue
        if src.endswith(".cu"):
            cmd = [nvcc, *ARCH, "-lineinfo", "-O3", "-std=c++17", *DEVICE_FP, "-Xcompiler", "-fPIC," + HOST_FP,
                   *extra, *inc, "-c", path, "-o", obj]
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
    checked_objs = [checked_obj if o.endswith("gbl_device.cu.o") else o for o in objs]
    for lib, parts in ((LIB, objs), (LIB_CHECKED, checked_objs)):
        if force or _stale(lib, parts):
            cmd = [nvcc, *ARCH, "-shared", "-o", lib, *parts, "-lcudart"]
            r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
            if r.returncode != 0:
                raise RuntimeError("link failed: " + " ".join(cmd) + "\n" + r.stdout)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
