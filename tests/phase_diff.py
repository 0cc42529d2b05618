"""Phase-diff: the device against the CPU restatement after every phase of a substep.

The debug mode the survey of the reference's test strategy asks for in place
of a memory checker: run a case to a substep, then run that one substep on
the device phase by phase (gbl_debug_substep, outside the captured graph) and
in the restatement (oracle/oracle.cpp's phase hook), each side recording the
lattice's state at the end of every phase, and compare the two bit for bit
phase by phase. The first phase whose arrays differ names the kernel to read.

The device fuses or moves some work (the support projection inside the sweep,
the restart beside the first contact pass, the strain and end sample outside
the contact halo beside the second), so only the phases where both sides have
finished the same work are compared, and at each only the arrays that work
has settled (SYNC below): nodes after the kick, everything after the first
contact pass (the restart is done by then on both), nodes after the sweep
with its support projection, the velocity update, the damping and the second
contact pass, everything after the end sample and after the ledger. The
sphere is compared after the contact passes only when it is on: without it
the device kicks the sphere in the ledger, the reference before the passes.

    python tests/phase_diff.py --case impact_small --substep 12

runs one of the golden fixtures' cases (or a scene: --scene impact|contact)
and prints the first divergent phase and arrays, or that every phase agrees.
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, HERE)

NODES = ["u", "u_prev", "v"]
BONDS = ["alive", "failure_mode", "damage", "plastic_extension", "plastic_strain", "prev_tensile",
         "prev_compressive", "prev_shear"]
# Phase number (latticePhaseName, FastLattice.cpp:15-28) -> arrays settled there on both sides.
SYNC = {3: NODES, 4: NODES + BONDS + ["sphere_out"], 7: NODES, 8: NODES, 9: NODES, 10: NODES + ["sphere_out"],
        15: NODES, 12: NODES + BONDS, 13: NODES + BONDS + ["sphere_out"]}
PHASE_NAMES = {3: "kick_classify", 4: "contact_pass_1", 7: "support_project", 8: "velocity_update", 9: "damping",
               10: "contact_pass_2", 12: "end_sample_bonds", 13: "sphere_exit", 15: "node_contact_narrow"}


def phases_for(case: dict) -> list[int]:
    """The comparable phases this case's settings run, ascending."""
    from banjo_gb300 import scenes

    s = np.asarray(case["settings"])
    out = [3, 4, 7, 8]
    if float(s[scenes.K_DAMP]) > 0.0:
        out.append(9)
    out += [10, 12, 13]
    if s.size > scenes.K_NODE_CONTACT and float(s[scenes.K_NODE_CONTACT]) != 0.0:
        out.append(15)
    return sorted(out)


def compare(expected: dict, actual: dict, phases, sphere: bool = True) -> dict:
    """Per phase, the arrays whose bits differ (phase -> list of names);
    both dicts hold "phase<p>__<array>" entries. `sphere`: the case runs the
    sphere (its state is compared after the contact passes too)."""
    from oracle.compare import same_bits

    bad = {}
    for p in phases:
        arrays = [a for a in SYNC[p] if sphere or p == 13 or a != "sphere_out"]
        names = [a for a in arrays if not same_bits(expected[f"phase{p}__{a}"], actual[f"phase{p}__{a}"])]
        if names:
            bad[p] = names
    return bad


def first_divergence(bad: dict):
    """The first phase that differs and its arrays, or None."""
    if not bad:
        return None
    p = min(bad)
    return p, PHASE_NAMES.get(p, str(p)), bad[p]


def port_phases(case: dict, substep: int, phases, precision: str = "float", threads: int = 4) -> dict:
    """The restatement's state after each phase of substep `substep`."""
    import oracle

    c = dict(case)
    c["steps"] = np.array([substep + 1], dtype=np.uint64)
    c["phase_substep"] = np.array([substep], dtype=np.uint64)
    mask = 0
    for p in phases:
        mask |= 1 << p
    c["phase_mask"] = np.array([mask], dtype=np.uint32)
    out = oracle.run_port(c, precision=precision, threads=threads)
    return {k: v for k, v in out.items() if k.startswith("phase")}


def device_phases(case: dict, substep: int, phases, precision: str = "float") -> dict:
    """The device's state after each phase of substep `substep`: the case run
    to that substep through the C ABI, then the substep phase by phase."""
    from banjo_gb300 import lattice

    n = int(case["node_count"][0])
    sched = lattice.build_lattice_schedule(n, case["bond_a"], case["bond_b"], case["node_block_begin"])
    state = lattice.build_lattice_state(case, sched)
    be = lattice.make_gb300_lattice_backend(sched, precision)
    settings = lattice.step_settings(case["settings"])
    settings.direct_arithmetic = 1 if precision == "double" else 0
    be.upload(state, settings, lattice.sphere_state(case["sphere"]))
    if case.get("forces") is not None:
        be.set_external_forces(case["forces"], int(case["force_substeps"][0]))
    if "wrench_names" in case:
        be.set_external_wrenches(lattice.case_wrenches(case), int(case["wrench_substeps"][0]))
    if substep:
        be.run(lattice.RunControl(max_steps=substep))
    states = [lattice.build_lattice_state(case, sched) for _ in phases]
    spheres = be.debug_substep(phases, states)
    out = {}
    for p, st, sp in zip(phases, states, spheres):
        for a in NODES + BONDS:
            out[f"phase{p}__{a}"] = getattr(st, a).copy()
        out[f"phase{p}__sphere_out"] = lattice.pack_sphere(sp)
    return out


def phase_diff(case: dict, substep: int, precision: str = "float", threads: int = 4):
    """(phases compared, {phase: differing arrays}) for the device against
    the restatement at substep `substep` of the case."""
    if "force_ramp_steps" in case:
        raise ValueError("phase-diff runs cases whose loads are set once (no ramp)")
    from banjo_gb300 import scenes

    phases = phases_for(case)
    expected = port_phases(case, substep, phases, precision, threads)
    actual = device_phases(case, substep, phases, precision)
    sphere = float(np.asarray(case["settings"])[scenes.K_SPHERE]) != 0.0
    return phases, compare(expected, actual, phases, sphere)


def main() -> int:
    from _util import golden_names, load_golden
    from banjo_gb300 import scenes

    p = argparse.ArgumentParser()
    p.add_argument("--case", help="a golden fixture's case: " + ", ".join(golden_names()))
    p.add_argument("--scene", choices=["impact", "contact"])
    p.add_argument("--substep", type=int, default=10)
    args = p.parse_args()
    precision = "float"
    if args.case:
        case, _, precision = load_golden(args.case)
    elif args.scene == "impact":
        case = scenes.impact_block(nx=48, ny=24, nz=48, blocks=4, radius=0.1, steps=3)
    elif args.scene == "contact":
        case = scenes.contact_drop(nx=24, ny=10, nz=18, speed=6.0, steps=40)
    else:
        raise SystemExit("name a --case or a --scene")
    phases, bad = phase_diff(case, args.substep, precision)
    first = first_divergence(bad)
    if first is None:
        print(f"substep {args.substep}: every phase agrees ({', '.join(PHASE_NAMES[p] for p in phases)})")
        return 0
    print(f"substep {args.substep}: first divergence after phase {first[0]} ({first[1]}): {', '.join(first[2])}")
    return 1


if __name__ == "__main__":
    sys.exit(main())
