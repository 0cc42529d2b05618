"""Node-to-node contact on the GPU (LatticePhysics.hpp:1441-1647) against the
CPU checker, which is pinned to the reference on the contact fixtures.

Bar: the state bit for bit, the same bonds broken at the same substep, and
every RunStatus counter including the node-contact accumulators (the narrow
phase runs in the reference's serial pair order, so its FP64 sums are the
serial sums). The golden fixtures themselves run in test_gpu_parity.
"""
import numpy as np
import pytest

from _util import LEDGER_RTOL, STATE_KEYS, mismatches, status_mismatches

pytestmark = pytest.mark.gpu

NODE_CONTACTS, NODE_REBUILDS, NODE_LISTED = 13, 15, 16


def _drop(**kw):
    from banjo_gb300 import scenes

    return scenes.contact_drop(**kw)


def test_contact_drop_matches_checker(device, port):
    """A cracking box with its crack faces meeting: rebuilds after every
    failure round, thousands of pairs, hundreds of responses per substep."""
    case = _drop(nx=24, ny=10, nz=18, speed=6.0, steps=40)
    cpu = port.run_port(case, threads=4, per_substep=True)
    gpu = device.run_case(case, per_substep=True)
    assert int(cpu["status_u64"][4]) > 0 and int(cpu["status_u64"][NODE_CONTACTS]) > 100
    assert mismatches(cpu, gpu, STATE_KEYS + ["break_step"]) == []
    assert status_mismatches(cpu, gpu, ledger_rtol=LEDGER_RTOL) == []


def test_contact_drop_double_lane_matches_checker(device, port):
    from banjo_gb300 import scenes

    case = _drop(nx=12, ny=6, nz=10, speed=5.0, steps=20)
    case["settings"] = case["settings"].copy()
    case["settings"][scenes.K_DIRECT] = 1
    cpu = port.run_port(case, precision="double", threads=2, per_substep=True)
    gpu = device.run_case(case, precision="double", per_substep=True)
    assert int(cpu["status_u64"][NODE_CONTACTS]) > 0
    assert mismatches(cpu, gpu, STATE_KEYS + ["break_step"]) == []
    assert status_mismatches(cpu, gpu, ledger_rtol=LEDGER_RTOL) == []


def test_contact_with_sphere_matches_checker(device, port):
    """Sphere contact and node contact in one substep: the end phase waits for
    the node-contact pass (no halo split)."""
    from banjo_gb300 import scenes

    case = scenes.impact_block(nx=20, ny=10, nz=14, blocks=2, radius=0.03, speed=14.0, steps=3, substeps=10,
                               seed_point=5, seed_strength=21)
    n = int(case["node_count"][0])
    s = case["settings"].copy()
    s[scenes.K_NODE_CONTACT:scenes.K_NODE_CONTACT + 9] = scenes.node_contact(2, 0.005, 0.0025, restitution=0.1,
                                                                           node_count=n)
    case["settings"] = s
    cpu = port.run_port(case, threads=4, per_substep=True)
    gpu = device.run_case(case, per_substep=True)
    assert int(cpu["status_u64"][4]) > 0 and int(cpu["status_u64"][9]) > 0
    assert int(cpu["status_u64"][NODE_LISTED]) > 0
    assert mismatches(cpu, gpu, STATE_KEYS + ["break_step"]) == []
    assert status_mismatches(cpu, gpu, ledger_rtol=LEDGER_RTOL) == []


def test_contact_lattices_in_one_batch(device):
    """Uneven cracking boxes with contact on, one batch: each equals itself alone."""
    cases = [_drop(nx=nx, ny=ny, nz=nz, speed=sp, steps=25) for nx, ny, nz, sp in
             ((10, 6, 8, 4.0), (18, 8, 12, 6.0), (7, 5, 6, 3.0), (22, 9, 14, 5.0))]
    shared = cases[-1]["settings"]
    for c in cases:
        c["settings"] = shared  # one table size for all: the list does not depend on it
    together = device.run_batch(cases)
    for case, out in zip(cases, together):
        alone = device.run_case(case)
        assert mismatches(alone, out, STATE_KEYS) == []
        assert status_mismatches(alone, out) == []
    assert sum(int(o["status_u64"][NODE_CONTACTS]) > 0 for o in together) >= 3


def test_contact_requests_served_equal_alone(device):
    """Node contact in the served form: the pair-list scratch is charged at
    admission, each result equals its lattice run alone."""
    cases = [_drop(nx=nx, ny=ny, nz=nz, speed=sp, steps=20) for nx, ny, nz, sp in
             ((10, 6, 8, 4.0), (14, 7, 9, 6.0), (8, 5, 6, 3.0))]
    shared = cases[0]["settings"]
    for c in cases:
        c["settings"] = shared
    server = device.Server(device.step_settings(shared), 1 << 33)
    held, tickets = [], []
    for c in cases:
        n = int(c["node_count"][0])
        sched = device.build_lattice_schedule(n, c["bond_a"], c["bond_b"], c["node_block_begin"])
        state = device.build_lattice_state(c, sched)
        held.append(state)
        tickets.append(server.submit(sched, state, device.sphere_state(c["sphere"]), int(c["steps"][0]),
                                     borrow=True))
    while any(server.poll(t).phase != device.REQUEST_DONE for t in tickets):
        server.step(7)
    for c, t, state in zip(cases, tickets, held):
        _, status = server.take(t, state)
        alone = device.run_case(c)
        assert np.array_equal(state.u, alone["u"]) and np.array_equal(state.alive, alone["alive"])
        assert status.node_contact.contacts == int(alone["status_u64"][NODE_CONTACTS])
    assert server.stats().bytes_in_use == 0


def test_plate_and_contact_batch_equal_alone(device):
    """Plate bending, node contact and the ledge supports together, in one
    batch of struck sheets of uneven size: each equals itself alone."""
    from banjo_gb300 import scenes

    cases = [scenes.plate_strike(nx=nx, nz=nz, steps=25, speed=sp) for nx, nz, sp in
             ((16, 16, 8.0), (24, 12, 10.0), (12, 20, 6.0))]
    s = cases[0]["settings"].copy()
    s[scenes.K_NODE_CONTACT:scenes.K_NODE_CONTACT + 9] = scenes.node_contact(2, 0.005, 0.0025, node_count=600)
    for c in cases:
        c["settings"] = s
    together = device.run_batch(cases)
    for case, out in zip(cases, together):
        alone = device.run_case(case)
        assert mismatches(alone, out, STATE_KEYS) == []
        assert status_mismatches(alone, out) == []
    assert all(int(o["status_u64"][4]) > 0 for o in together)
