"""The batch: many lattices stepped by shared launches.

Each lattice of a batch keeps its own state, control block and ledgers, and
every kernel's work for one lattice depends on that lattice's data alone, so a
lattice's results in a batch are bit for bit its results alone -- ledgers
included, since each lattice's fixed summation order depends only on its own
bond count. These tests hold the batch to exactly that, and one member to the
CPU checker directly.
"""
import numpy as np
import pytest

from _util import LEDGER_RTOL, STATE_KEYS, mismatches, status_mismatches


def _drop_trials():
    from banjo_gb300 import scenes

    # Uneven sizes; three land (and break) within 120 substeps, two are still
    # falling at the end.
    shapes = [(8, 6, 8), (12, 5, 9), (6, 6, 6), (10, 7, 5), (5, 4, 13)]
    heights = [0.004, 0.005, 0.02, 0.006, 0.03]
    cases = []
    for k, ((nx, ny, nz), height) in enumerate(zip(shapes, heights)):
        cases.append(scenes.drop_trial(nx, ny, nz, compliance=10.0 ** (-7 + 0.5 * k), break_strain=1.0e-3 + 5e-4 * k,
                                       drop_height=height, steps=12))
    return cases


@pytest.mark.gpu
def test_batch_members_equal_each_lattice_alone(device):
    cases = _drop_trials()
    together = device.run_batch(cases)
    broke = 0
    for case, out in zip(cases, together):
        alone = device.run_case(case)
        assert mismatches(alone, out, STATE_KEYS) == []
        assert status_mismatches(alone, out) == []  # exact: same per-lattice order
        broke += int(out["status_u64"][4]) > 0
    assert broke == 3


@pytest.mark.gpu
def test_batch_member_matches_checker(device, port):
    cases = _drop_trials()
    together = device.run_batch(cases)
    cpu = port.run_port(cases[3], threads=4)
    assert mismatches(cpu, together[3], STATE_KEYS) == []
    assert status_mismatches(cpu, together[3], ledger_rtol=LEDGER_RTOL) == []


@pytest.mark.gpu
def test_batch_sphere_impacts_equal_alone(device):
    """Sphere contact, candidate lists per (lattice, slab), plasticity and the
    ground plane, for lattices of different slab counts and sizes."""
    from banjo_gb300 import scenes

    cases = [scenes.impact_block(nx=24, ny=12, nz=24, blocks=6, radius=0.04, speed=12.0, steps=6),
             scenes.impact_block(nx=32, ny=12, nz=16, blocks=8, radius=0.04, speed=12.0, steps=6, seed_point=5,
                                 seed_strength=9),
             scenes.impact_block(nx=16, ny=12, nz=40, blocks=4, radius=0.04, speed=12.0, steps=6, seed_point=7,
                                 seed_strength=4)]
    together = device.run_batch(cases)
    # The same lattices swept whole in one CTA each with their positions
    # staged in shared memory (plastic flow and the ground plane included).
    staged = device.run_batch(cases, tuning={"whole_max_bonds": 1 << 24, "staged_max_nodes": 14336})
    for case, out, st in zip(cases, together, staged):
        alone = device.run_case(case)
        assert int(out["status_u64"][9]) > 0  # the sphere touched this lattice
        assert mismatches(alone, out, STATE_KEYS) == []
        assert status_mismatches(alone, out) == []
        assert mismatches(alone, st, STATE_KEYS) == []
        assert status_mismatches(alone, st) == []


@pytest.mark.gpu
def test_batch_lattices_stop_on_their_own_exit_rules(device):
    """A lattice that meets an exit rule stops; the others go on."""
    cases = _drop_trials()
    control = device.RunControl(max_steps=150, no_failure_steps=100, quiet_steps=8)
    together = device.run_batch(cases, control=control)
    totals = set()
    for case, out in zip(cases, together):
        n = int(case["node_count"][0])
        sched = device.build_lattice_schedule(n, case["bond_a"], case["bond_b"], case["node_block_begin"])
        state = device.build_lattice_state(case, sched)
        be = device.make_gb300_lattice_backend(sched)
        be.upload(state, device.step_settings(case["settings"]), device.sphere_state(case["sphere"]))
        st = be.run(control)
        be.download(state)
        assert int(out["status_u64"][0]) == st.total_steps
        assert int(out["status_u64"][7]) == st.exit_reason
        assert np.array_equal(out["u"], state.u) and np.array_equal(out["alive"], state.alive)
        totals.add(st.total_steps)
    assert len(totals) >= 2  # some lattices stopped earlier than others


@pytest.mark.gpu
def test_batch_loads_and_status_per_lattice(device):
    """Per-lattice external loads, and a second run call continuing the first."""
    from banjo_gb300 import scenes

    a = scenes.cantilever(nx=12, ny=4, nz=4, steps=2)
    b = scenes.cantilever(nx=20, ny=5, nz=3, steps=2)
    cases = [a, b]
    whole = [device.run_case(c) for c in cases]
    batch = device.Batch()
    states = []
    for c in cases:
        n = int(c["node_count"][0])
        sched = device.build_lattice_schedule(n, c["bond_a"], c["bond_b"], c["node_block_begin"])
        state = device.build_lattice_state(c, sched)
        batch.add(sched, state, device.sphere_state(c["sphere"]))
        states.append(state)
    batch.settle(device.step_settings(a["settings"]))
    for k, c in enumerate(cases):
        batch.set_external_forces(k, c["forces"], int(c["force_substeps"][0]))
    assert len(batch) == 2
    batch.run(device.RunControl(max_steps=7))
    batch.run(device.RunControl(max_steps=13))
    for k, (c, w) in enumerate(zip(cases, whole)):
        batch.download(k, states[k])
        st = batch.status(k)
        assert st.total_steps == 20
        assert np.array_equal(states[k].u, w["u"]) and np.array_equal(states[k].alive, w["alive"])
        assert st.external_load.work_j == float(w["status_f64"][14])
    with pytest.raises(ValueError):
        batch.status(2)


def test_batch_refuses_mixed_settings(gbl):
    from banjo_gb300 import scenes

    a = scenes.drop_trial(6, 4, 6, compliance=1e-6, break_strain=2e-3, drop_height=0.1, steps=1)
    b = scenes.impact_block(nx=8, ny=6, nz=8, blocks=2, radius=0.02, steps=1)
    with pytest.raises(ValueError, match="share"):
        gbl.run_batch([a, b])


@pytest.mark.gpu
@pytest.mark.parametrize("shape", ["tune", {"sweep_threads": 256, "whole_max_bonds": 1 << 24},
                                   {"sweep_threads": 1024, "whole_max_bonds": 1}, {"group_bytes": 1 << 16},
                                   {"staged_max_nodes": 14336}, {"sweep_threads": 256, "staged_max_nodes": 300}])
def test_batch_launch_shapes_leave_results_unchanged(device, shape):
    """The autotuner's choices (one-CTA sweep size and reach, group size) and
    its timing runs change nothing: every shape runs the same levels."""
    cases = _drop_trials()
    base = device.run_batch(cases)
    shaped = device.run_batch(cases, tuning=shape)
    for a, b in zip(base, shaped):
        assert mismatches(a, b, STATE_KEYS) == []
        assert status_mismatches(a, b) == []


@pytest.mark.gpu
def test_batch_tuned_mid_run_equals_untuned(device):
    """Tuning between runs restores every position it moved."""
    cases = _drop_trials()
    whole = device.run_batch(cases)
    batch = device.Batch()
    states = []
    for c in cases:
        sched = device.build_lattice_schedule(int(c["node_count"][0]), c["bond_a"], c["bond_b"], c["node_block_begin"])
        state = device.build_lattice_state(c, sched)
        batch.add(sched, state, device.sphere_state(c["sphere"]))
        states.append(state)
    batch.settle(device.step_settings(cases[0]["settings"]))
    total = max(int(c["steps"][0]) for c in cases)
    batch.run(device.RunControl(max_steps=total // 2))
    chosen = batch.tune()
    assert chosen["candidates"] > 1 and chosen["sweep_ms"] > 0.0
    batch.run(device.RunControl(max_steps=total - total // 2))
    for k, state in enumerate(states):
        batch.download(k, state)
        assert np.array_equal(state.u, whole[k]["u"]) and np.array_equal(state.alive, whole[k]["alive"])
