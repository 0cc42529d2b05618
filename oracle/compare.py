"""Bit-for-bit comparison of lattice run outputs (test infrastructure).

The tests and the benchmark's parity checks hold the GPU's outputs to the
CPU checkers' with these helpers: every state array bit for bit, the
RunStatus slot by slot, and the two FP64 ledgers the reference folds one bond
at a time within the tolerance below. Outputs are the dicts oracle.run_port,
oracle.run_reference and banjo_gb300.lattice.run_case return.
"""
from __future__ import annotations

import numpy as np

# Outputs held bit for bit between runners (status excludes wall time and the
# launch count, which differ by construction).
STATE_KEYS = ["u", "u_prev", "v", "alive", "failure_mode", "damage", "plastic_extension", "plastic_strain",
              "prev_tensile", "prev_compressive", "prev_shear", "sphere_out", "first_failure_bonds", "source_names",
              "source_ledgers"]
SCHEDULE_KEYS = ["sched_bond_order", "sched_color", "sched_range_begin", "sched_range_end",
                 "sched_bond_block_begin", "sched_color_count", "sched_boundary_bond_count"]
STATUS_U64 = {"total_steps": 0, "first_failure_step": 1, "last_failure_step": 2, "failure_rounds": 3,
              "broken_bonds": 4, "last_energy_gain_step": 5, "last_damage_gain_step": 6, "exit_reason": 7,
              "rank_deficient_nodes": 8, "impulse_contacts": 9, "candidate_overflow": 10, "ball_support_events": 11,
              "node_contacts": 13, "node_pair_tests": 14, "node_rebuilds": 15, "node_pairs_listed": 16,
              "node_pair_overflow": 17, "energy_audited": 18}
STATUS_F64 = {"removed_energy_j": 0, "max_damage": 1, "plastic_work_j": 2, "max_tensile": 3, "max_compressive": 4,
              "max_shear": 5, "max_plastic_stretch": 6, "impulse_x": 7, "impulse_y": 8, "impulse_z": 9,
              "contact_dissipated": 10, "max_penetration": 11, "max_correction": 12, "max_center_shift": 13,
              "external_work": 14, "external_impulse_x": 15, "external_impulse_y": 16, "external_impulse_z": 17,
              "external_steps": 18, "node_dissipated": 20, "node_max_overlap": 21, "node_max_correction": 22,
              "node_momentum_x": 23, "node_momentum_y": 24, "node_momentum_z": 25, "damping_dissipated": 26,
              "striker_dissipated": 27}


def same_bits(a, b) -> bool:
    a = np.asarray(a)
    b = np.asarray(b)
    if a.dtype.kind == "f" and b.dtype.kind == "f" and a.dtype != b.dtype:
        # A float32 fixture against a float64 output of the float lane: the
        # widening is exact, so compare the widened bits.
        a = a.astype(np.float64)
        b = b.astype(np.float64)
    return a.shape == b.shape and a.dtype == b.dtype and np.array_equal(a.view(np.uint8), b.view(np.uint8))


def mismatches(expected: dict, actual: dict, keys) -> list[str]:
    bad = []
    for k in keys:
        if k not in expected or k not in actual:
            if k in expected or k in actual:
                bad.append(k + " (missing)")
            continue
        if not same_bits(expected[k], actual[k]):
            bad.append(k)
    return bad


# The two FP64 ledgers the reference folds one bond at a time. The GPU sums
# them in a fixed parallel order (deterministic, but not the serial order), so
# against a serial runner they are held to the tolerance the reference gave its
# own CUDA backend for them, 1e-12 relative (tests/fast_lattice_tests.cpp:517-521).
LEDGERS = ("removed_energy_j", "plastic_work_j")
LEDGER_RTOL = 1e-12


def _slot(status, i):
    """A status slot; records written before the node-contact or audit slots
    existed (both off) read zero there."""
    return status[i] if i < len(status) else 0


def status_mismatches(expected: dict, actual: dict, skip=(), ledger_rtol: float = 0.0) -> list[str]:
    bad = []
    for name, i in STATUS_U64.items():
        e, a = int(_slot(expected["status_u64"], i)), int(_slot(actual["status_u64"], i))
        if name not in skip and e != a:
            bad.append(f"{name}: {e} != {a}")
    for name, i in STATUS_F64.items():
        if name in skip:
            continue
        e, a = float(_slot(expected["status_f64"], i)), float(_slot(actual["status_f64"], i))
        if name in LEDGERS and ledger_rtol > 0.0:
            if abs(e - a) > ledger_rtol * max(abs(e), 1e-300):
                bad.append(f"{name}: {e!r} != {a!r} beyond {ledger_rtol:g} relative")
            continue
        if not (e == a or (np.isnan(e) and np.isnan(a))):
            bad.append(f"{name}: {e!r} != {a!r}")
    return bad


def ledger_report(expected: dict, actual: dict) -> dict:
    """Each FP64 ledger's relative difference beside the most that another
    summation order of its n non-negative addends can move it, 2 n 2^-53
    relative (each order's rounding error is at most (n - 1) 2^-53 of the sum
    of the addends, which for non-negative terms is the sum itself). n is the
    broken-bond count for the removed energy and the restatement's count of
    plastic increments for the plastic work; `within` holds when a ledger
    meets the larger of that bound and LEDGER_RTOL."""
    n_removed = int(_slot(expected["status_u64"], STATUS_U64["broken_bonds"]))
    n_plastic = int(np.asarray(expected.get("plastic_increments", [0]))[0])
    out, ok = {}, True
    for name, n in (("removed_energy_j", n_removed), ("plastic_work_j", n_plastic)):
        i = STATUS_F64[name]
        e, a = float(_slot(expected["status_f64"], i)), float(_slot(actual["status_f64"], i))
        rel = abs(e - a) / max(abs(e), 1e-300) if e != a else 0.0
        bound = max(LEDGER_RTOL, 2.0 * n * 2.0 ** -53)
        out[name] = {"rel_error": rel, "addends": n, "order_bound": bound}
        ok = ok and rel <= bound
    out["within"] = ok
    return out
