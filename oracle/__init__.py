"""CPU checkers of the lattice substep (test infrastructure only).

`run_port` drives the CPU restatement (oracle/oracle.cpp, built to
oracle/_build/liboracle.so); `run_reference` drives the reference harness
(oracle/_ref/ref_harness, built from the reference's own sources where the
reference tree is present). Both take a case dict of numpy arrays
(banjo_gb300.scenes) and return a dict of output arrays. Nothing in the product
imports this package.
"""
from __future__ import annotations

import ctypes
import os
import struct
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(HERE, "_build", "liboracle.so")
REF_BIN = os.path.join(HERE, "_ref", "ref_harness")

_TYPES = {"d": np.float64, "f": np.float32, "I": np.uint32, "Q": np.uint64, "B": np.uint8}
_CODES = {np.dtype(np.float64): "d", np.dtype(np.float32): "f", np.dtype(np.uint32): "I",
          np.dtype(np.uint64): "Q", np.dtype(np.uint8): "B"}


def build_port() -> str:
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    return PORT_LIB


def reference_root() -> str:
    """Where the reference's source tree is read from: the BANJO_REFERENCE_ROOT
    environment variable, else a checkout named `reference` beside this
    repository."""
    env = os.environ.get("BANJO_REFERENCE_ROOT")
    if env:
        return env
    return os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")


def reference_present() -> bool:
    return os.path.isdir(os.path.join(reference_root(), "src", "fastlattice"))


def build_reference(ref_root: str | None = None) -> str | None:
    """Builds oracle/_ref from the reference's sources when they are present."""
    ref_root = ref_root or reference_root()
    if not os.path.isdir(os.path.join(ref_root, "src", "fastlattice")):
        return None
    jobs = str(max(1, min(8, os.cpu_count() or 1)))
    subprocess.run(["make", "-s", "-C", HERE, "-j", jobs, "ref", f"REF={ref_root}"], check=True)
    return REF_BIN


def write_case(case: dict, path: str) -> None:
    with open(path, "wb") as f:
        for name, value in case.items():
            arr = np.ascontiguousarray(value)
            code = _CODES[arr.dtype]
            raw = name.encode()
            f.write(struct.pack("<I", len(raw)))
            f.write(raw)
            f.write(code.encode())
            f.write(struct.pack("<Q", arr.size))
            f.write(arr.tobytes())


def read_case(path: str) -> dict:
    out = {}
    with open(path, "rb") as f:
        data = f.read()
    pos = 0
    while pos < len(data):
        (n,) = struct.unpack_from("<I", data, pos)
        pos += 4
        name = data[pos:pos + n].decode()
        pos += n
        code = chr(data[pos])
        pos += 1
        (count,) = struct.unpack_from("<Q", data, pos)
        pos += 8
        dt = np.dtype(_TYPES[code])
        out[name] = np.frombuffer(data, dtype=dt, count=count, offset=pos).copy()
        pos += count * dt.itemsize
    return out


_lib = None


def _port():
    global _lib
    if _lib is None:
        if not os.path.exists(PORT_LIB):
            build_port()
        lib = ctypes.CDLL(PORT_LIB)
        lib.oracle_case_new.restype = ctypes.c_void_p
        lib.oracle_case_free.argtypes = [ctypes.c_void_p]
        lib.oracle_case_put.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_char, ctypes.c_uint64, ctypes.c_void_p]
        lib.oracle_case_count.argtypes = [ctypes.c_void_p, ctypes.c_char_p]
        lib.oracle_case_count.restype = ctypes.c_longlong
        lib.oracle_case_type.argtypes = [ctypes.c_void_p, ctypes.c_char_p]
        lib.oracle_case_type.restype = ctypes.c_char
        lib.oracle_case_get.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_void_p, ctypes.c_uint64]
        lib.oracle_run.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        lib.oracle_last_error.restype = ctypes.c_char_p
        _lib = lib
    return _lib


OUTPUT_NAMES = ["sched_bond_order", "sched_color", "sched_range_begin", "sched_range_end", "sched_bond_block_begin",
                "sched_color_count", "sched_boundary_bond_count", "state_nbr_other", "state_max_degree", "u", "u_prev",
                "v", "alive", "failure_mode", "damage", "plastic_extension", "plastic_strain", "prev_tensile",
                "prev_compressive", "prev_shear", "sphere_out", "first_failure_bonds", "break_step", "status_u64",
                "status_f64", "source_names", "source_ledgers", "wall_seconds", "threads", "substep_seconds",
                "bond_projections", "plastic_increments", "substep_projections"]


# The arrays the phase-diff mode records after each requested phase (case keys
# "phase_substep" and "phase_mask"), as "phase<p>__<array>" outputs.
PHASE_ARRAYS = ["u", "u_prev", "v", "alive", "failure_mode", "damage", "plastic_extension", "plastic_strain",
                "prev_tensile", "prev_compressive", "prev_shear", "sphere_out"]


def run_port(case: dict, precision: str = "float", threads: int = 1, per_substep: bool = False) -> dict:
    """Runs the CPU restatement on a case; returns its outputs."""
    lib = _port()
    cin = lib.oracle_case_new()
    cout = lib.oracle_case_new()
    try:
        for name, value in case.items():
            arr = np.ascontiguousarray(value)
            if lib.oracle_case_put(cin, name.encode(), _CODES[arr.dtype].encode(), arr.size,
                                   arr.ctypes.data_as(ctypes.c_void_p)) != 0:
                raise RuntimeError(lib.oracle_last_error().decode())
        rc = lib.oracle_run(cin, cout, 1 if precision == "double" else 0, int(threads), 1 if per_substep else 0)
        if rc != 0:
            raise RuntimeError("oracle: " + lib.oracle_last_error().decode())
        out = {}
        names = list(OUTPUT_NAMES)
        if "phase_mask" in case:
            mask = int(np.asarray(case["phase_mask"]).reshape(-1)[0])
            names += [f"phase{p}__{a}" for p in range(32) if (mask >> p) & 1 for a in PHASE_ARRAYS]
        for name in names:
            count = lib.oracle_case_count(cout, name.encode())
            if count < 0:
                continue
            dt = np.dtype(_TYPES[lib.oracle_case_type(cout, name.encode()).decode()])
            arr = np.empty(count, dtype=dt)
            lib.oracle_case_get(cout, name.encode(), arr.ctypes.data_as(ctypes.c_void_p), arr.nbytes)
            out[name] = arr
        return out
    finally:
        lib.oracle_case_free(cin)
        lib.oracle_case_free(cout)


def run_reference(case: dict, precision: str = "float", parallel: bool = False, threads: int = 0,
                  per_substep: bool = False) -> dict:
    """Runs the reference's own CPU lane (oracle/_ref) on a case."""
    if not os.path.exists(REF_BIN):
        raise FileNotFoundError("reference harness is not built (oracle/_ref)")
    with tempfile.TemporaryDirectory() as tmp:
        cin, cout = os.path.join(tmp, "in.case"), os.path.join(tmp, "out.case")
        write_case(case, cin)
        args = [REF_BIN, cin, cout, precision, "parallel" if parallel else "serial", str(threads)]
        if per_substep:
            args.append("--per-substep")
        subprocess.run(args, check=True)
        return read_case(cout)
