"""Edge cases of the lattice path on the GPU, each against the CPU checker.

A lattice without bonds (every node supported on its own), a single bond (a
sweep of one level), every bond dead from the start, and the same lattices
inside one batch with an ordinary one (single-level and bond-less lattices
next to a multi-level one).
"""
import numpy as np
import pytest

from _util import LEDGER_RTOL, STATE_KEYS, mismatches, status_mismatches

pytestmark = pytest.mark.gpu


def _cases():
    from banjo_gb300 import scenes

    lone = scenes.drop_trial(1, 1, 1, compliance=1e-6, break_strain=2e-3, drop_height=0.002, steps=3)
    pair = scenes.drop_trial(2, 1, 1, compliance=1e-6, break_strain=2e-3, drop_height=0.002, steps=3)
    dead = scenes.drop_trial(6, 4, 5, compliance=1e-6, break_strain=2e-3, drop_height=0.002, steps=3)
    dead["alive"] = np.zeros(int(dead["bond_count"][0]), dtype=np.uint8)
    ordinary = scenes.drop_trial(7, 5, 6, compliance=1e-7, break_strain=1e-3, drop_height=0.004, steps=3)
    return {"lone": lone, "pair": pair, "dead": dead, "ordinary": ordinary}


@pytest.mark.parametrize("name", ["lone", "pair", "dead"])
def test_edge_lattice_matches_checker(device, port, name):
    case = _cases()[name]
    cpu = port.run_port(case, threads=2, per_substep=True)
    gpu = device.run_case(case, per_substep=True)
    assert float(np.abs(gpu["u"]).max()) > 0.0  # it fell and met the ground
    assert mismatches(cpu, gpu, STATE_KEYS + ["break_step"]) == []
    assert status_mismatches(cpu, gpu, ledger_rtol=LEDGER_RTOL) == []


def test_edge_lattices_in_one_batch(device):
    cases = list(_cases().values())
    together = device.run_batch(cases)
    for case, out in zip(cases, together):
        alone = device.run_case(case)
        assert mismatches(alone, out, STATE_KEYS) == []
        assert status_mismatches(alone, out) == []


def test_queued_request_cancelled(device):
    """A request still waiting for memory leaves without touching the others."""
    cases = _cases()
    big, small = cases["ordinary"], cases["pair"]
    sizes = {}
    held = {}
    for name, c in (("big", big), ("small", small)):
        n = int(c["node_count"][0])
        sched = device.build_lattice_schedule(n, c["bond_a"], c["bond_b"], c["node_block_begin"])
        state = device.build_lattice_state(c, sched)
        held[name] = (sched, state)
        sizes[name] = device.footprint(state.node_count, state.bond_count, state.view.max_degree, 1)
    server = device.Server(device.step_settings(big["settings"]), sizes["big"])  # room for one at a time
    t_big = server.submit(*held["big"], device.sphere_state(big["sphere"]), 30)
    t_wait = server.submit(*held["small"], device.sphere_state(small["sphere"]), 30)
    server.step(5)
    assert server.poll(t_big).phase == device.REQUEST_RUNNING
    assert server.poll(t_wait).phase == device.REQUEST_QUEUED
    server.cancel(t_wait)
    while server.poll(t_big).phase != device.REQUEST_DONE:
        server.step(10)
    _, status = server.take(t_big, held["big"][1])
    alone = device.run_case(dict(big, steps=np.array([30], dtype=np.uint64)))
    assert np.array_equal(held["big"][1].u, alone["u"])
    assert status.total_steps == 30
    st = server.stats()
    assert st.queued == 0 and st.running == 0 and st.bytes_in_use == 0
