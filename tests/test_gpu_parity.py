"""GPU parity: the CUDA path against the reference's outputs and the CPU checker.

Bar (the reference's own CUDA test, tests/fast_lattice_tests.cpp:480-524):
positions, velocities, damage and every other state array bit for bit, the
same bonds broken at the same substep, the same first-failure list and every
RunStatus counter. The two FP64 ledgers the reference folds bond by bond
(removed energy, plastic work) are summed on the device in a fixed parallel
order -- deterministic run to run -- and held to 1e-12 relative, the bound the
reference set for its own CUDA backend.
"""
import numpy as np
import pytest

from _util import LEDGER_RTOL, SCHEDULE_KEYS, STATE_KEYS, golden_names, load_golden, mismatches, status_mismatches

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", golden_names())
def test_gpu_reproduces_reference_fixture(device, name):
    case, ref, precision = load_golden(name)
    out = device.run_case(case, precision=precision, per_substep=True)
    assert mismatches(ref, out, SCHEDULE_KEYS + STATE_KEYS + ["break_step"]) == []
    assert status_mismatches(ref, out, ledger_rtol=LEDGER_RTOL) == []


def test_gpu_cantilever_full_run_matches_checker(device, port):
    """The cantilever workload (32x8x8, 240 steps x 10 substeps) end to end."""
    from banjo_gb300 import scenes

    case = scenes.cantilever()
    cpu = port.run_port(case, threads=8)
    gpu = device.run_case(case)
    assert int(cpu["status_u64"][4]) > 0
    assert mismatches(cpu, gpu, STATE_KEYS) == []
    assert status_mismatches(cpu, gpu, ledger_rtol=LEDGER_RTOL) == []
    # The throughput numerator: bonds alive at each sweep times iterations.
    assert int(gpu["bond_projections"][0]) == int(cpu["bond_projections"][0]) > 0


def test_gpu_sliced_impact_matches_checker(device, port):
    """32 slabs, sphere contact, plastic flow, ground plane: every sweep level kind."""
    from banjo_gb300 import scenes

    case = scenes.impact_block(nx=48, ny=24, nz=64, blocks=32, radius=0.08, speed=10.0, steps=12, seed_point=2,
                               seed_strength=20)
    cpu = port.run_port(case, threads=8, per_substep=True)
    gpu = device.run_case(case, per_substep=True)
    assert int(cpu["status_u64"][4]) > 0 and int(cpu["status_u64"][9]) > 0
    assert mismatches(cpu, gpu, STATE_KEYS + ["break_step"]) == []
    assert status_mismatches(cpu, gpu, ledger_rtol=LEDGER_RTOL) == []
    assert int(gpu["bond_projections"][0]) == int(cpu["bond_projections"][0]) > 0


def test_gpu_candidate_overflow_over_several_slabs(device, port):
    """A sphere large against its slabs: more than 1024 candidates in several
    slabs of one lattice at once, so every slab's CTA adds to the one overflow
    counter in the same substep (CpuLatticeBackend.cpp:379-385)."""
    from banjo_gb300 import scenes

    case = scenes.impact_block(nx=48, ny=24, nz=48, blocks=4, radius=0.25, steps=3)
    cpu = port.run_port(case, threads=8, per_substep=True)
    gpu = device.run_case(case, per_substep=True)
    assert int(cpu["status_u64"][10]) > 10000  # candidate_overflow
    assert mismatches(cpu, gpu, STATE_KEYS + ["break_step"]) == []
    assert status_mismatches(cpu, gpu, ledger_rtol=LEDGER_RTOL) == []


def test_gpu_double_lane_matches_checker(device, port):
    from banjo_gb300 import scenes

    case = scenes.cantilever(nx=16, ny=6, nz=6, steps=8)
    cpu = port.run_port(case, precision="double", per_substep=True)
    gpu = device.run_case(case, precision="double", per_substep=True)
    assert mismatches(cpu, gpu, STATE_KEYS + ["break_step"]) == []
    assert status_mismatches(cpu, gpu, ledger_rtol=LEDGER_RTOL) == []


def test_gpu_runs_are_deterministic(device):
    from banjo_gb300 import scenes

    case = scenes.impact_block(nx=24, ny=12, nz=24, blocks=6, radius=0.04, speed=12.0, steps=5)
    a = device.run_case(case)
    b = device.run_case(case)
    assert mismatches(a, b, STATE_KEYS) == []


def test_status_accumulates_across_run_calls(device, port):
    """A run split into several calls equals one call (fast_lattice_tests.cpp:994-998)."""
    from banjo_gb300 import scenes

    case = scenes.cantilever(steps=4)
    whole = device.run_case(case)
    n = int(case["node_count"][0])
    sched = device.build_lattice_schedule(n, case["bond_a"], case["bond_b"], case["node_block_begin"])
    state = device.build_lattice_state(case, sched)
    be = device.make_gb300_lattice_backend(sched)
    be.upload(state, device.step_settings(case["settings"]), device.sphere_state(case["sphere"]))
    be.set_external_forces(case["forces"], int(case["force_substeps"][0]))
    for chunk in (7, 13, 20):
        st = be.run(device.RunControl(max_steps=chunk))
    assert st.total_steps == 40
    be.download(state)
    assert np.array_equal(state.u, whole["u"]) and np.array_equal(state.alive, whole["alive"])
    assert st.broken_bonds == int(whole["status_u64"][4])
    assert st.removed_energy_j == float(whole["status_f64"][0])  # same fixed order in both runs


def _backend(device, case):
    n = int(case["node_count"][0])
    sched = device.build_lattice_schedule(n, case["bond_a"], case["bond_b"], case["node_block_begin"])
    state = device.build_lattice_state(case, sched)
    be = device.make_gb300_lattice_backend(sched)
    be.upload(state, device.step_settings(case["settings"]), device.sphere_state(case["sphere"]))
    return sched, state, be


def test_exit_rules_and_abandon(device):
    from banjo_gb300 import scenes

    case = scenes.drop_trial(8, 6, 8, compliance=1e-6, break_strain=5e-3, drop_height=0.5, steps=1)
    _, _, be = _backend(device, case)
    st = be.run(device.RunControl(max_steps=50, no_failure_steps=7))
    assert st.exit_reason == 2 and st.total_steps == 7
    st = be.run(device.RunControl(max_steps=5))
    assert st.exit_reason == 3 and st.total_steps == 12
    flag = np.ones(1, dtype=np.uint8)
    st = be.run(device.RunControl(max_steps=100, abandon=flag))
    assert st.exit_reason == 7 and st.total_steps == 12


def test_external_force_rules(device):
    from banjo_gb300 import scenes

    case = scenes.cantilever(nx=6, ny=3, nz=3, steps=1)
    _, _, be = _backend(device, case)
    n = int(case["node_count"][0])
    bad = np.zeros((n, 3))
    bad[0, 1] = -1.0  # node 0 is pinned: no movable mass
    with pytest.raises(ValueError, match="movable"):
        be.set_external_forces(bad, 10)
    with pytest.raises(ValueError):
        be.set_external_forces(np.zeros((n - 1, 3)), 10)
    nonfinite = np.zeros((n, 3))
    nonfinite[5, 0] = np.inf
    with pytest.raises(ValueError, match="finite"):
        be.set_external_forces(nonfinite, 10)
    with pytest.raises(ValueError):
        be.set_external_forces(None, 3)
    be.set_external_forces(None, 0)


def test_refused_features(device):
    """What the device lane refuses at upload, as the reference's parallel lane
    refuses what it does not run: the Verlet integrator (serial double only,
    ParallelCpuLatticeBackend.cpp:1380-1381), node contact with no cutoff, and
    a double backend asked for the float lane's arithmetic."""
    from banjo_gb300 import scenes

    case = scenes.cantilever(nx=6, ny=3, nz=3, steps=1)
    sched, state, be = _backend(device, case)
    be.run(device.RunControl(max_steps=3))
    be.download(state)
    before = state.u.copy()
    s = device.step_settings(case["settings"])
    s.bond_integrator = 1
    with pytest.raises(ValueError, match="XPBD"):
        be.upload(state, s, device.sphere_state(case["sphere"]))
    # A refused upload leaves the lattice it had (lattice_verlet_tests.cpp:165-185).
    assert be.status().total_steps == 3
    be.download(state)
    assert np.array_equal(state.u, before)
    s = device.step_settings(case["settings"])
    s.node_contact.mode = 2  # radius and skin left at zero
    with pytest.raises(ValueError, match="cutoff"):
        be.upload(state, s, device.sphere_state(case["sphere"]))
    dbl = device.make_gb300_lattice_backend(sched, "double")
    with pytest.raises(ValueError, match="direct"):
        dbl.upload(state, device.step_settings(case["settings"]), device.sphere_state(case["sphere"]))


def test_frames_and_phase_profile(device):
    from banjo_gb300 import scenes

    case = scenes.cantilever(nx=10, ny=4, nz=4, steps=3)
    sched, state, be = _backend(device, case)
    st = be.run(device.RunControl(max_steps=25, capture_stride=10, max_frames=2))
    frames = be.take_frames()
    assert [f["step"] for f in frames] == [0, 10] and st.frames_captured == 2
    _, state2, be2 = _backend(device, case)
    be2.run(device.RunControl(max_steps=10))
    be2.download(state2)
    assert np.array_equal(frames[1]["u"], state2.u.astype(np.float32))
    # Profiling advances the state exactly like a run.
    _, state3, be3 = _backend(device, case)
    phases = be3.profile_phases(10)
    be3.download(state3)
    assert np.array_equal(state3.u, state2.u)
    assert phases["sweep_interior"] > 0 and phases["end_sample_bonds"] > 0


def test_frames_match_the_checker_at_their_substeps(device, port):
    """FrameCapture (FastLattice.hpp:247-253; captured before the substep it
    is named for, CpuLatticeBackend.cpp:274-278): every frame of a sliced
    impact -- positions as float, aliveness, damage, the sphere -- equals the
    CPU checker's state after that many substeps."""
    from banjo_gb300 import scenes

    case = scenes.impact_block(nx=32, ny=16, nz=24, blocks=4, radius=0.06, steps=3)
    _, _, be = _backend(device, case)
    be.run(device.RunControl(max_steps=30, capture_stride=7, max_frames=10))
    frames = be.take_frames()
    assert [f["step"] for f in frames] == [0, 7, 14, 21, 28]
    broke = 0
    for f in frames:
        sub = dict(case)
        sub["steps"] = np.array([f["step"]], dtype=np.uint64)
        cpu = port.run_port(sub, threads=4)
        assert np.array_equal(f["u"], cpu["u"].astype(np.float32)), f["step"]
        assert np.array_equal(f["alive"], cpu["alive"]), f["step"]
        assert np.array_equal(f["damage"], cpu["damage"].astype(np.float32)), f["step"]
        assert np.array_equal(f["sphere"], cpu["sphere_out"]), f["step"]
        broke = int(cpu["status_u64"][4])
    assert broke > 0
