"""Records the long-horizon notched-bar fixture from the reference itself.

The 128x32x32 notched bar (energy-scaled law compiled in FP64, plastic flow,
horizon 2, x = 0 face pinned, x = nx-1 face pulled along +x with a load ramped
linearly from 0 to twice the failure load over 10,000 rigid steps of 10
substeps, re-set every step) is run for the whole ramp by the reference's own
threaded CPU lane (oracle/_ref/ref_harness: makeParallelCpuLatticeBackend,
compiled from the reference's sources), one substep per run call so that the
substep at which every bond broke is recorded. A 100,000-substep run takes
about three and a half hours on six threads of an x86-64 host (the double
lane, which the FP32 error is measured against, about the same), so each is
recorded once:

    python tests/golden/make_cascade_long.py [--threads 6] [--precision float|double]

writing tests/golden/cascade_long.npz or cascade_long_double.npz.

The fixture keeps what the GPU test compares: the final positions and
velocities in full (float32 for the float lane: its values are floats widened,
so the narrowing is exact), aliveness, failure modes and the RunStatus, and
for the large per-bond arrays (damage, plastic state, peaks, the substep each
bond broke) a SHA-256 digest of their bytes plus a few counts. The case
itself is rebuilt by banjo_gb300.scenes.notched_bar; a digest of its arrays is
stored so that a change of the generator is caught rather than compared.
"""
from __future__ import annotations

import argparse
import hashlib
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from banjo_gb300 import scenes  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
RAMP_STEPS = 10000
DIGESTED = ("damage", "plastic_extension", "plastic_strain", "prev_tensile", "prev_compressive", "prev_shear",
            "break_step", "u_prev")


def case_digest(case: dict) -> str:
    h = hashlib.sha256()
    for name in sorted(case):
        arr = np.ascontiguousarray(case[name])
        h.update(name.encode())
        h.update(str(arr.dtype).encode())
        h.update(arr.tobytes())
    return h.hexdigest()


def array_digest(arr, float_lane: bool) -> str:
    arr = np.ascontiguousarray(arr)
    if float_lane and arr.dtype == np.float64:
        arr = arr.astype(np.float32)
    return hashlib.sha256(arr.tobytes()).hexdigest()


def main() -> None:
    p = argparse.ArgumentParser()
    p.add_argument("--threads", type=int, default=6)
    p.add_argument("--precision", default="float", choices=["float", "double"])
    p.add_argument("--steps", type=int, default=RAMP_STEPS, help="rigid steps run (the ramp is always 10,000)")
    args = p.parse_args()
    oracle.build_reference()
    case = scenes.notched_bar(ramp_steps=RAMP_STEPS, steps=args.steps)
    t0 = time.time()
    out = oracle.run_reference(case, precision=args.precision, parallel=True, threads=args.threads, per_substep=True)
    wall = time.time() - t0
    float_lane = args.precision == "float"
    narrow = (lambda a: a.astype(np.float32)) if float_lane else (lambda a: a)
    rec = {
        "precision": np.array([args.precision]),
        "rigid_steps": np.array([args.steps], dtype=np.uint64),
        "case_sha256": np.array([case_digest(case)]),
        "u": narrow(out["u"]),
        "v": narrow(out["v"]),
        "alive": out["alive"],
        "failure_mode": out["failure_mode"],
        "status_u64": out["status_u64"],
        "status_f64": out["status_f64"],
        "broken_per_step": np.bincount(out["break_step"][out["break_step"] != 0xFFFFFFFF] // 10,
                                       minlength=args.steps).astype(np.uint32),
        "threads": np.array([args.threads], dtype=np.uint32),
        "wall_seconds": np.array([wall]),
    }
    for name in DIGESTED:
        rec["sha256__" + name] = np.array([array_digest(out[name], float_lane)])
    suffix = "" if float_lane else "_double"
    if args.steps != RAMP_STEPS:
        suffix += f"_{args.steps}"
    path = os.path.join(HERE, f"cascade_long{suffix}.npz")
    np.savez_compressed(path, **rec)
    print(f"{path}: {int(out['status_u64'][4])} bonds broken, {wall:.0f} s on {args.threads} threads")


if __name__ == "__main__":
    main()
