"""Generates the golden fixtures of tests/golden from the reference itself.

Each fixture is one lattice case (inputs, as banjo_gb300.scenes builds them) and
the outputs of the reference's own CPU lane on it: the reference harness
(oracle/_ref/ref_harness, compiled from the reference's sources) runs
buildLatticeSchedule, buildLatticeState and CpuLatticeBackend<float|double> and
records the schedule, the final state, the RunStatus and the substep at which
every bond broke. Run where the reference tree is present:

    python tests/golden/make_golden.py

Float-lane positions and velocities are stored as float32: the float backend
widens float values, so the narrowing is exact.
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from banjo_gb300 import scenes  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
INF = float("inf")


def cases() -> dict:
    out = {}
    # The cantilever workload itself (32x8x8), 24 rigid steps: fracture from substep 19.
    out["cantilever_24"] = (scenes.cantilever(steps=24), "float")
    # Sphere impact on a 4-slab block with plastic flow, through shattering.
    out["impact_small"] = (scenes.impact_block(nx=16, ny=10, nz=12, blocks=4, radius=0.03, speed=12.0, steps=30,
                                               seed_point=5, seed_strength=21), "float")
    # The same in the double (direct arithmetic) lane, shorter.
    out["impact_small_double"] = (scenes.impact_block(nx=16, ny=10, nz=12, blocks=4, radius=0.03, speed=12.0,
                                                      steps=10, seed_point=5, seed_strength=21), "double")
    # A batched-trial box dropped a few millimetres onto the ground.
    out["drop_small"] = (scenes.drop_trial(10, 6, 8, compliance=1e-6, break_strain=2e-3, drop_height=0.003, steps=20),
                         "float")
    # Radial bond damping on, and a ledge plane with finite footprints (reach cap) over the ground.
    damped = scenes.drop_trial(12, 6, 10, compliance=3e-7, break_strain=1.5e-3, drop_height=0.004, steps=20)
    ground = scenes.plane((0.0, 0.0, 0.0), node_radius=0.005)
    ledge = scenes.plane((0.0, 0.002, 0.0), node_radius=0.005, restitution=0.3,
                         footprints=((-0.04, 0.0, 0.02, 0.06), (0.04, 0.0, 0.02, 0.06)))
    damped["settings"] = scenes.settings(damping_fraction=0.05, planes=[ledge, ground])
    out["damped_ledge"] = (damped, "float")
    # The notched bar (energy-scaled law, plastic flow, horizon 2, pinned end,
    # ramped end load), small, through its first failure rounds.
    out["bar_small"] = (scenes.notched_bar(24, 8, 8, ramp_steps=800, steps=20), "float")
    out["bar_small_double"] = (scenes.notched_bar(16, 6, 6, ramp_steps=800, steps=6), "double")
    # Node-to-node contact: the reference's two-cell pairs (an unbonded pair
    # closing at 4 m/s; a bonded pair held overlapping by its bond; the same
    # pair with its bond failed; unequal masses closing unevenly), and a box
    # thrown onto the ground that cracks, with the cracked faces in contact.
    out["contact_pair_closing"] = (scenes.two_cells(0.02, v0=2.0, v1=-2.0, steps=6000), "double")
    out["contact_pair_bonded"] = (scenes.two_cells(0.006, bonded=True, steps=2000), "double")
    out["contact_pair_dead"] = (scenes.two_cells(0.006, bonded=True, dead=True, steps=2000), "double")
    out["contact_pair_momentum"] = (scenes.two_cells(0.02, v0=4.0, v1=-1.0, mass_ratio=3.0, steps=8000), "double")
    out["contact_drop"] = (scenes.contact_drop(), "float")
    out["contact_drop_measure"] = (scenes.contact_drop(mode=1, steps=20), "float")
    # Plate bending: a sheet one cell thick on two ledges, struck at its
    # centre, breaking by the fibre strain of its bending; float and double.
    out["plate_strike"] = (scenes.plate_strike(), "float")
    out["plate_strike_double"] = (scenes.plate_strike(nx=16, nz=16, steps=25), "double")
    # The energy audit: what the striker passes and the damping sweep take out
    # of the lattice, measured as kinetic-energy differences (sphere impact,
    # radial damping and plastic flow on); float and double.
    for name, precision, steps in (("audit_impact", "float", 12), ("audit_impact_double", "double", 6)):
        audited = scenes.impact_block(nx=16, ny=10, nz=12, blocks=4, radius=0.03, speed=12.0, steps=steps,
                                      seed_point=5, seed_strength=21)
        audited["settings"] = audited["settings"].copy()
        audited["settings"][scenes.K_DAMP] = 0.05
        audited["settings"][scenes.K_AUDIT] = 1.0
        out[name] = (audited, precision)
    # External wrenches: a pinned bar twisted and pushed by two named sources,
    # each spread over its nodes from the current geometry at every kick and
    # keeping its own ledger; breaking from substep 9.
    out["wrench_bar"] = (scenes.wrenched_bar(), "float")
    out["wrench_bar_double"] = (scenes.wrenched_bar(steps=20), "double")
    # Checkpoint and resume: the run downloaded mid-way (after failures, with
    # damage, plastic flow and contact under way) and uploaded into a fresh
    # backend, which starts afresh from the state as the reference's upload
    # does (the resumed run is not the uninterrupted one).
    resumed = scenes.impact_block(nx=16, ny=10, nz=12, blocks=4, radius=0.03, speed=12.0, steps=30, seed_point=5,
                                  seed_strength=21)
    resumed["checkpoint_at"] = np.array([11], dtype=np.uint64)
    out["resume_impact"] = (resumed, "float")
    resumed = scenes.contact_drop()
    resumed["checkpoint_at"] = np.array([10], dtype=np.uint64)
    out["resume_contact_drop"] = (resumed, "float")
    # A loaded run resumed: external loads are not part of the state, so the
    # fresh backend runs on without them (the caller would set them again).
    resumed = scenes.cantilever(nx=16, ny=6, nz=6, steps=5)
    resumed["checkpoint_at"] = np.array([27], dtype=np.uint64)
    out["resume_loaded"] = (resumed, "float")
    # Caps: a slab with more sphere candidates than a slab's list holds
    # (1024), and node contact with more pairs per owner than its slots (24).
    out["candidate_overflow"] = (scenes.impact_block(nx=40, ny=4, nz=40, blocks=1, radius=0.4, speed=6.0, steps=1,
                                                     substeps=6, seed_point=3, seed_strength=4, gap=0.0005), "float")
    dense = scenes.contact_drop(nx=8, ny=5, nz=6, speed=2.0, steps=6)
    settings = dense["settings"].copy()
    settings[scenes.K_NODE_CONTACT:scenes.K_NODE_CONTACT + 9] = scenes.node_contact(
        2, 0.012, 0.01, node_count=int(dense["node_count"][0]))
    dense["settings"] = settings
    dense["alive"] = np.zeros(int(dense["bond_count"][0]), dtype=np.uint8)
    out["contact_pair_overflow"] = (dense, "float")
    return out


def material() -> None:
    """The reference's own compile of the bar material (MaterialCompiler.cpp), for
    the restatement in banjo_gb300.scenes.compile_energy_scaled."""
    m = list(scenes.BAR_MATERIAL) + [0.01, 2.0]  # + cell, horizon
    ref = oracle.run_reference({"material": np.asarray(m, dtype=np.float64)})
    path = os.path.join(HERE, "material_bar.npz")
    np.savez_compressed(path, material=np.asarray(m), compiled=ref["compiled"])
    print("material_bar:", ref["compiled"])


def main() -> None:
    oracle.build_reference()
    material()
    only = set(sys.argv[1:])
    for name, (case, precision) in cases().items():
        if only and name not in only:
            continue
        ref = oracle.run_reference(case, precision=precision, per_substep=True)
        data = {"case__" + k: np.asarray(v) for k, v in case.items()}
        for k, v in ref.items():
            if k in ("wall_seconds", "threads", "state_adj_bonds"):
                continue
            if precision == "float" and k in ("u", "u_prev", "v", "damage", "prev_tensile", "prev_compressive",
                                              "prev_shear", "plastic_extension", "plastic_strain"):
                narrowed = v.astype(np.float32)
                assert np.array_equal(narrowed.astype(np.float64), v), k
                v = narrowed
            data["ref__" + k] = v
        data["precision"] = np.array([precision])
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, **data)
        su = ref["status_u64"]
        print(f"{name}: N={case['node_count'][0]} B={case['bond_count'][0]} substeps={su[0]} "
              f"broken={su[4]} rounds={su[3]} first={su[1]} size={os.path.getsize(path) // 1024} KiB")


if __name__ == "__main__":
    main()
