"""Runs cases through the bounds-checked build of the library.

Run as a child process with GBL_LIBRARY=checked (tests/test_gpu_bounds_checked.py
does): every golden fixture, a sliced impact and a batch of uneven drop
trials go through libgbl_checked.so, whose kernels check every index they
read out of device data before using it and record, instead of making, any
out-of-range access. Prints one JSON line: the bounds record and, per case,
whether the outputs still equal the reference's (fixtures) or the CPU
restatement's. Exits 0 when it could run every case.
"""
from __future__ import annotations

import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, HERE)

from _util import (LEDGER_RTOL, SCHEDULE_KEYS, STATE_KEYS, golden_names, load_golden, mismatches,  # noqa: E402
                   status_mismatches)


def main() -> int:
    import oracle
    from banjo_gb300 import lattice, scenes

    if not lattice.LIB_PATH.endswith("libgbl_checked.so"):
        print(json.dumps({"error": "GBL_LIBRARY=checked is not set"}))
        return 2
    lattice.bounds_clear()
    parity = {}
    for name in golden_names():
        case, ref, precision = load_golden(name)
        out = lattice.run_case(case, precision=precision, per_substep=True)
        parity[name] = (mismatches(ref, out, SCHEDULE_KEYS + STATE_KEYS + ["break_step"]) == [] and
                        status_mismatches(ref, out, ledger_rtol=LEDGER_RTOL) == [])
    oracle.build_port()
    impact = scenes.impact_block(nx=48, ny=24, nz=48, blocks=4, radius=0.25, steps=2)
    cpu = oracle.run_port(impact, threads=8, per_substep=True)
    gpu = lattice.run_case(impact, per_substep=True)
    parity["impact_48x24x48"] = (mismatches(cpu, gpu, STATE_KEYS + ["break_step"]) == [] and
                                 status_mismatches(cpu, gpu, ledger_rtol=LEDGER_RTOL) == [])
    trials = [scenes.drop_trial(nx, ny, nz, compliance=10.0 ** (-7 + 0.5 * k), break_strain=1.0e-3 + 5e-4 * k,
                                drop_height=h, steps=12)
              for k, ((nx, ny, nz), h) in enumerate(zip([(8, 6, 8), (12, 5, 9), (6, 6, 6), (10, 7, 5)],
                                                        [0.004, 0.005, 0.02, 0.006]))]
    together = lattice.run_batch(trials)
    for k, (case, out) in enumerate(zip(trials, together)):
        cpu = oracle.run_port(case, threads=4)
        parity[f"batch_member_{k}"] = (mismatches(cpu, out, STATE_KEYS) == [] and
                                       status_mismatches(cpu, out, ledger_rtol=LEDGER_RTOL) == [])
    print(json.dumps({"report": lattice.bounds_report(), "parity": parity}))
    return 0


if __name__ == "__main__":
    sys.exit(main())
