"""The notched bar over its whole 10,000-step ramp against the reference's run.

tests/golden/cascade_long.npz holds the reference's own threaded CPU lane
(makeParallelCpuLatticeBackend, compiled from its sources) on the 128x32x32
notched bar -- energy-scaled law and plastic flow compiled in FP64, horizon 2,
x = 0 face pinned, the x = nx-1 face pulled along +x by a load ramped from 0 to
twice the failure load over 10,000 rigid steps of 10 substeps, re-set every
step (src/material/MaterialCompiler.cpp:110-125, 179-214;
src/fastlattice/ExternalLoads.hpp:28-50). The device runs the same ramp
through the C ABI and must end bit for bit where the reference ended: final
positions and velocities, aliveness and failure modes, the damage, plastic and
peak-strain arrays (by SHA-256 digest), the count of bonds broken in every one
of the 10,000 steps, and every RunStatus counter, the FP64 ledgers within the
bound another summation order allows. (The bar breaks bonds in 9,986 of the
steps, so the substep each bond broke, which the record also digests, would
take a download after almost every one of the 100,000 substeps; the per-step
counts and the final arrays are compared instead.)

Where tests/golden/cascade_long_double.npz (the reference's FP64 lane on the
same ramp) is present, the device's FP32 error against it at the end of the
horizon is reported: it is a measurement, not a pass condition, since a
rupture cascade is chaotic and FP32 and FP64 part ways once bonds fail.
"""
import hashlib
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

from _util import STATUS_F64, STATUS_U64  # noqa: E402

pytestmark = pytest.mark.gpu

FIXTURE = os.path.join(HERE, "golden", "cascade_long.npz")
FIXTURE_FP64 = os.path.join(HERE, "golden", "cascade_long_double.npz")
PER_STEP = 10


def _digest(arr) -> str:
    arr = np.ascontiguousarray(arr)
    if arr.dtype == np.float64:
        arr = arr.astype(np.float32)  # the float lane's values, widened: exact
    return hashlib.sha256(arr.tobytes()).hexdigest()


def _run_ramp(device, case):
    """The ramp on the device, one rigid step per run call; the bonds broken
    in each step from the status."""
    n = int(case["node_count"][0])
    sched = device.build_lattice_schedule(n, case["bond_a"], case["bond_b"], case["node_block_begin"])
    state = device.build_lattice_state(case, sched)
    be = device.make_gb300_lattice_backend(sched)
    be.upload(state, device.step_settings(case["settings"]), device.sphere_state(case["sphere"]))
    base = case["forces"]
    ramp = int(case["force_ramp_steps"][0])
    scale0 = float(case["force_ramp_scale"][0])
    steps = int(case["steps"][0]) // PER_STEP
    broken_per_step = np.zeros(steps, dtype=np.uint32)
    broken = 0
    st = None
    for step in range(steps):
        be.set_external_forces((scale0 * step / ramp) * base, PER_STEP)
        st = be.run(device.RunControl(max_steps=PER_STEP))
        broken_per_step[step] = st.broken_bonds - broken
        broken = st.broken_bonds
    be.download(state)
    return state, st, broken_per_step


def test_full_ramp_reproduces_the_reference(device):
    if not os.path.exists(FIXTURE):
        pytest.skip("the long-horizon record is not present")
    from banjo_gb300 import scenes
    from make_cascade_long import case_digest

    ref = np.load(FIXTURE)
    steps = int(ref["rigid_steps"][0])
    case = scenes.notched_bar(ramp_steps=10000, steps=steps)
    assert case_digest(case) == str(ref["case_sha256"][0]), "the scene generator changed since the record was made"
    want_per_step = ref["broken_per_step"]
    state, st, per_step = _run_ramp(device, case)

    assert np.array_equal(per_step, want_per_step)
    assert np.array_equal(state.u.astype(np.float32), ref["u"])
    assert np.array_equal(state.v.astype(np.float32), ref["v"])
    assert np.array_equal(state.alive, ref["alive"])
    assert np.array_equal(state.failure_mode, ref["failure_mode"])
    got = {"damage": state.damage, "plastic_extension": state.plastic_extension,
           "plastic_strain": state.plastic_strain, "prev_tensile": state.prev_tensile,
           "prev_compressive": state.prev_compressive, "prev_shear": state.prev_shear, "u_prev": state.u_prev}
    bad = [name for name, arr in got.items() if _digest(arr) != str(ref["sha256__" + name][0])]
    assert bad == []

    status = device.status_arrays(st)
    for name, i in STATUS_U64.items():
        if name == "last_energy_gain_step":
            # The reference's threaded lane tests the energy gain once per
            # failure round, its serial lane per bond
            # (ParallelCpuLatticeBackend.cpp:1913-1919): the device follows
            # the serial lane.
            continue
        assert int(status["status_u64"][i]) == int(ref["status_u64"][i]), name
    n_removed = int(ref["status_u64"][STATUS_U64["broken_bonds"]])
    for name, i in STATUS_F64.items():
        e, a = float(ref["status_f64"][i]), float(status["status_f64"][i])
        if name in ("removed_energy_j", "plastic_work_j"):
            # Non-negative addends: another order moves the sum by at most
            # 2 n 2^-53 of itself. n is the broken-bond count for the removed
            # energy; for the plastic work, one increment per substep of each
            # bond whose plastic extension ends non-zero (the bonds that
            # flowed in the ramp's tension).
            flowed = int(np.count_nonzero(state.plastic_extension))
            n = n_removed if name == "removed_energy_j" else flowed * steps * PER_STEP
            assert abs(e - a) <= max(1e-12, 2.0 * n * 2.0 ** -53) * abs(e), name
        else:
            assert e == a or (np.isnan(e) and np.isnan(a)), name

    if os.path.exists(FIXTURE_FP64):
        ref64 = np.load(FIXTURE_FP64)
        x0 = case["ref_pos"].reshape(-1, 3)
        extent = float(np.max(x0.max(axis=0) - x0.min(axis=0)))
        du = float(np.abs(state.u - ref64["u"]).max())
        alive_diff = int(np.count_nonzero(state.alive != ref64["alive"]))
        rel = lambda a, b: abs(a - b) / max(abs(b), 1e-300)  # noqa: E731
        print(f"notched bar, {steps} steps: FP32 device vs FP64 reference: max |du| / extent = {du / extent:.3e}, "
              f"bonds whose state differs {alive_diff} of {state.alive.size}, broken {int(st.broken_bonds)} vs "
              f"{int(ref64['status_u64'][4])}, removed energy rel {rel(st.removed_energy_j, float(ref64['status_f64'][0])):.3e}, "
              f"plastic work rel {rel(st.plastic_work_j, float(ref64['status_f64'][2])):.3e}")
