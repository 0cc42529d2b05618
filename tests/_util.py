"""Shared helpers of the test suite: golden fixtures and exact comparisons."""
from __future__ import annotations

import glob
import os

import numpy as np

from oracle.compare import (LEDGER_RTOL, LEDGERS, SCHEDULE_KEYS, STATE_KEYS, STATUS_F64, STATUS_U64,  # noqa: F401
                            mismatches, same_bits, status_mismatches)

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden_names() -> list[str]:
    """The lattice-run fixtures (material_*.npz hold material compiles, and
    cascade_long*.npz the long-horizon record, which keeps digests instead of
    the case and full outputs)."""
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz"))
                  if not os.path.basename(p).startswith(("material_", "cascade_long")))


def load_golden(name: str):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    case = {k[len("case__"):]: z[k] for k in z.files if k.startswith("case__")}
    ref = {k[len("ref__"):]: z[k] for k in z.files if k.startswith("ref__")}
    return case, ref, str(z["precision"][0])
