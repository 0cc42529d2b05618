"""The CPU checker against the reference itself on seeded random scenes.

The fixtures and the combined cases fix their sizes and seeds. Here a seeded
generator draws them: lattice sizes, slab counts, strength and impact seeds,
striker radius and speed, plastic flow on or off, compliance and break strain,
and the scene kind -- a sphere impact on a block, a drop onto the ground, a
thrown box with node-to-node contact, a plate strike with plate bending, a
pinned beam under its load, a small notched bar under its ramp. The checker
must reproduce the reference harness bit for bit on each, in both lanes:
every state array, the substep each bond broke, every RunStatus counter. The
draw is fixed (seed 2026), so a failure names a case that can be rerun; the
device is held to the checker on the same draw (tests/test_gpu_random.py). A
second draw (seed 7) layers the optional features on at random -- radial bond
damping, the energy audit, plastic hardening, a named wrench -- and holds the
checker alone to the harness. They run where the harness is built (the
reference tree is present).
"""
import os

import numpy as np
import pytest

import oracle
from _util import STATE_KEYS, mismatches, status_mismatches

pytestmark = pytest.mark.skipif(not os.path.exists(oracle.REF_BIN), reason="the reference harness is not built here")

KINDS = ("impact", "drop", "contact", "plate", "beam", "bar")


def _draw(rng, kind):
    """One scene of `kind` with parameters drawn from `rng`: (label, case)."""
    from banjo_gb300 import scenes

    if kind == "impact":
        nx, ny, nz = (int(v) for v in rng.integers(8, 19, size=3))
        blocks = int(rng.integers(1, min(4, nz) + 1))
        radius = float(rng.uniform(0.02, 0.05))
        speed = float(rng.uniform(6.0, 14.0))
        yf = float(rng.choice([0.0, 0.6]))
        case = scenes.impact_block(nx=nx, ny=ny, nz=nz, blocks=blocks, radius=radius, speed=speed, steps=2,
                                   seed_point=int(rng.integers(1, 100)), seed_strength=int(rng.integers(1, 100)),
                                   yield_fraction=yf)
        label = f"impact {nx}x{ny}x{nz} slabs {blocks} r {radius:.3f} v {speed:.1f} yield {yf}"
    elif kind == "drop":
        nx, ny, nz = (int(v) for v in rng.integers(6, 15, size=3))
        compliance = float(10.0 ** rng.uniform(-8.0, -5.0))
        strain = float(rng.uniform(1e-3, 5e-3))
        height = float(rng.uniform(0.0005, 0.003))
        case = scenes.drop_trial(nx, ny, nz, compliance=compliance, break_strain=strain, drop_height=height, steps=6)
        label = f"drop {nx}x{ny}x{nz} c {compliance:.1e} e {strain:.4f} h {height:.4f}"
    elif kind == "contact":
        nx, ny, nz = (int(v) for v in rng.integers(6, 13, size=3))
        speed = float(rng.uniform(2.0, 6.0))
        case = scenes.contact_drop(nx=nx, ny=ny, nz=nz, speed=speed, steps=int(rng.integers(15, 31)))
        label = f"contact {nx}x{ny}x{nz} v {speed:.2f}"
    elif kind == "plate":
        nx, nz = (int(v) for v in rng.integers(10, 21, size=2))
        speed = float(rng.uniform(5.0, 10.0))
        case = scenes.plate_strike(nx=nx, nz=nz, steps=20, radius=float(rng.uniform(0.02, 0.04)), speed=speed,
                                   seed_strength=int(rng.integers(1, 100)))
        label = f"plate {nx}x1x{nz} v {speed:.1f}"
    elif kind == "beam":
        nx = int(rng.integers(8, 21))
        ny, nz = (int(v) for v in rng.integers(3, 7, size=2))
        case = scenes.cantilever(nx=nx, ny=ny, nz=nz, steps=3)
        label = f"beam {nx}x{ny}x{nz}"
    else:
        nx = int(rng.integers(12, 25)) & ~1
        case = scenes.notched_bar(nx=nx, ny=8, nz=8, ramp_steps=int(rng.integers(2, 6)), steps=3)
        label = f"bar {nx}x8x8"
    return label, case


def _cases():
    rng = np.random.default_rng(2026)
    out = []
    for k in range(24):
        kind = KINDS[k % len(KINDS)]
        out.append(_draw(rng, kind))
    return out


CASES = _cases()


@pytest.mark.parametrize("precision", ["float", "double"])
@pytest.mark.parametrize("index", range(len(CASES)), ids=[label for label, _ in CASES])
def test_checker_matches_reference_on_random_scenes(index, precision):
    _, case = CASES[index]
    ref = oracle.run_reference(case, precision=precision, per_substep=True)
    port = oracle.run_port(case, precision=precision, per_substep=True, threads=4)
    assert mismatches(ref, port, STATE_KEYS + ["break_step"]) == []
    assert status_mismatches(ref, port) == []


def test_random_scenes_fracture():
    """The draw is not all quiet lattices: most of its float runs break bonds."""
    broke = 0
    for _, case in CASES:
        out = oracle.run_port(case, per_substep=False, threads=4)
        broke += int(out["status_u64"][4]) > 0
    assert broke >= len(CASES) // 2


# A second draw, for the checker alone: the same kinds with the optional
# features layered on at random -- radial bond damping, the energy audit,
# hardening of the plastic flow, and a named wrench (force and torque) on the
# movable nodes of the top face for part of the run.
def _with_features(rng, case):
    from banjo_gb300 import scenes

    case = dict(case)
    s = np.asarray(case["settings"], np.float64).copy()
    if s.size < scenes.SETTINGS_WIDTH:
        s = np.concatenate([s, np.zeros(scenes.SETTINGS_WIDTH - s.size)])
    notes = []
    if rng.random() < 0.6:
        s[scenes.K_DAMP] = float(rng.uniform(0.01, 0.1))
        notes.append(f"damping {s[scenes.K_DAMP]:.3f}")
    if rng.random() < 0.6:
        s[scenes.K_AUDIT] = 1.0
        notes.append("audit")
    if s[scenes.K_YIELD] > 0 and rng.random() < 0.7:
        s[scenes.K_HARDEN] = float(rng.uniform(0.05, 0.3))
        notes.append(f"hardening {s[scenes.K_HARDEN]:.2f}")
    case["settings"] = s
    if rng.random() < 0.7:
        pos = np.asarray(case["ref_pos"], np.float64).reshape(-1, 3)
        movable = np.ones(len(pos), dtype=bool)
        if "pinned" in case:
            movable &= np.asarray(case["pinned"]) == 0
        top = np.flatnonzero((pos[:, 1] >= pos[:, 1].max() - 1e-9) & movable)
        if top.size:
            mass = 1e-3 * top.size
            force = rng.uniform(-1.0, 1.0, size=3) * mass * float(rng.uniform(5.0, 50.0))
            torque = rng.uniform(-1.0, 1.0, size=3) * float(np.abs(force).max()) * 0.01
            substeps = int(min(int(case["steps"][0]), int(rng.integers(5, 31))))
            case = scenes.wrenches(case, [("drive", top, pos[top].mean(axis=0), force, torque)], substeps)
            notes.append(f"wrench {substeps}")
    return case, notes


def _feature_cases():
    rng = np.random.default_rng(7)
    out = []
    for k in range(15):
        kind = KINDS[k % (len(KINDS) - 1)]  # the notched bar's ramp already re-sets its loads every step
        label, case = _draw(rng, kind)
        case, notes = _with_features(rng, case)
        out.append((label + (" + " + ", ".join(notes) if notes else ""), case))
    return out


FEATURE_CASES = _feature_cases()


@pytest.mark.parametrize("precision", ["float", "double"])
@pytest.mark.parametrize("index", range(len(FEATURE_CASES)), ids=[label for label, _ in FEATURE_CASES])
def test_checker_matches_reference_on_random_scenes_with_features(index, precision):
    _, case = FEATURE_CASES[index]
    ref = oracle.run_reference(case, precision=precision, per_substep=True)
    port = oracle.run_port(case, precision=precision, per_substep=True, threads=4)
    assert mismatches(ref, port, STATE_KEYS + ["break_step"]) == []
    assert status_mismatches(ref, port) == []
