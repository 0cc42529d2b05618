"""External wrenches on the device (LatticeBackend::setExternalWrenches).

A wrench is a named node region driven by a force and a torque about a world
point; the reference spreads it over the region's nodes by mass about their
mass centre, from the current positions at every kick, and keeps a ledger per
source (ExternalLoads.hpp:52-77, 79-148, 171-238). The device does the same,
its region sums folded in the reference's order, so state and source ledgers
are held bit for bit: to the reference's own fixtures (wrench_bar*, in the
fixture parity test) and to the CPU checker here. The refusal and ordering
rules follow the reference's own wrench tests
(tests/lattice_external_load_tests.cpp:307-422).
"""
import numpy as np
import pytest

from _util import LEDGER_RTOL, STATE_KEYS, mismatches, status_mismatches

pytestmark = pytest.mark.gpu

CELL = 0.04
ORIGIN = (2.0, 0.6, -1.0)


def _cube(steps=1, bonded=False):
    """A 3x3x3 cube of equal point masses at -40, 0, +40 mm about the world
    point ORIGIN, no gravity; unbonded unless `bonded`."""
    from banjo_gb300 import scenes

    case = scenes._box_case(3, 3, 3, CELL, ORIGIN, 1e-7, [scenes.INF] * 6)
    case["mass"] = np.full(27, 0.25)
    case["origin"] = np.asarray(ORIGIN, dtype=np.float64)
    if not bonded:
        case["alive"] = np.zeros(int(case["bond_count"][0]), dtype=np.uint8)
    case["settings"] = scenes.settings(gravity=(0.0, 0.0, 0.0))
    case["steps"] = np.array([steps], dtype=np.uint64)
    return case


def _player(nodes=None, source="player-a", force=(20.0, -10.0, 5.0), torque=(0.5, -0.75, 1.25)):
    point = np.asarray(ORIGIN) + np.array([0.02, -0.03, 0.04])
    return (source, np.arange(27) if nodes is None else nodes, point, force, torque)


def _backend(device, case, precision="float"):
    n = int(case["node_count"][0])
    sched = device.build_lattice_schedule(n, case["bond_a"], case["bond_b"], case["node_block_begin"])
    state = device.build_lattice_state(case, sched)
    be = device.make_gb300_lattice_backend(sched, precision)
    s = device.step_settings(case["settings"])
    s.direct_arithmetic = 1 if precision == "double" else 0
    be.upload(state, s, device.sphere_state(case["sphere"]))
    return state, be


@pytest.mark.parametrize("precision", ["float", "double"])
def test_cube_wrench_matches_checker_and_carries_its_resultant(device, port, precision):
    from banjo_gb300 import scenes

    case = scenes.wrenches(_cube(), [_player()], 1)
    cpu = port.run_port(case, precision=precision)
    gpu = device.run_case(case, precision=precision)
    assert mismatches(cpu, gpu, STATE_KEYS) == []
    assert status_mismatches(cpu, gpu, ledger_rtol=LEDGER_RTOL) == []
    # The kick delivered the wrench: the cube's momentum is dt F, and the one
    # source ledger holds the run's whole external work.
    dt = float(np.float32(scenes.DT_SUBSTEP)) if precision == "float" else scenes.DT_SUBSTEP
    p = (0.25 * gpu["v"].reshape(-1, 3)).sum(axis=0)
    assert np.allclose(p, dt * np.array([20.0, -10.0, 5.0]), rtol=0, atol=1e-6 * dt * 23)
    ledger = gpu["source_ledgers"].reshape(-1, 15)
    assert bytes(gpu["source_names"]) == b"player-a\0" and ledger[0, 0] == 1
    assert ledger[0, 14] == gpu["status_f64"][14]


def test_wrench_order_and_sources(device):
    """Two sources given in either order, their node lists in either order,
    give the same run; each keeps its own span; an upload clears them."""
    from banjo_gb300 import scenes

    case = _cube(bonded=True)
    v = np.zeros((27, 3))
    p = case["ref_pos"].reshape(-1, 3) - np.asarray(ORIGIN)
    v[:] = np.array([3.0, -2.0, 1.0]) + np.cross(np.array([0.0, 30.0, 0.0]), p)
    case["vel"] = v.reshape(-1)
    a = _player(np.arange(9), force=(8.0, 2.0, 1.0), torque=(0.1, 0.2, -0.3))
    b = _player(np.arange(9, 27), source="player-b", force=(-3.0, -4.0, 0.5), torque=(-0.1, 0.05, 0.2))
    state1, one = _backend(device, case, "double")
    state2, two = _backend(device, case, "double")
    one.set_external_wrenches([b, a], 64)
    two.set_external_wrenches([(a[0], a[1][::-1]) + a[2:], (b[0], b[1][::-1]) + b[2:]], 64)
    for be in (one, two):
        be.run(device.RunControl(max_steps=20))
        st = be.run(device.RunControl(max_steps=108))
    one.download(state1)
    two.download(state2)
    assert np.array_equal(state1.u, state2.u) and np.array_equal(state1.v, state2.v)
    assert st.external_load.steps == 64
    sources = one.external_sources()
    assert [s for s, _ in sources] == ["player-a", "player-b"]
    assert all(g.steps == 64 for _, g in sources)
    total = sum(g.work_j for _, g in sources)
    assert abs(total - st.external_load.work_j) <= 1e-12 * abs(st.external_load.work_j)
    after = one.run(device.RunControl(max_steps=1))
    assert after.external_load.steps == 64 and all(g.steps == 64 for _, g in one.external_sources())
    settings = device.step_settings(case["settings"])
    settings.direct_arithmetic = 1
    one.upload(state1, settings, device.sphere_state(case["sphere"]))
    one.run(device.RunControl(max_steps=1))
    assert one.external_sources() == []


@pytest.mark.parametrize("precision", ["float", "double"])
def test_bad_wrenches_keep_the_load(device, precision):
    case = _cube()
    _, be = _backend(device, case, precision)
    original = _player()
    be.set_external_wrenches([original], 4)
    name, nodes, point, force, torque = original
    bad = [
        [(name, np.append(nodes, nodes[0]), point, force, torque)],  # a node twice
        [(name, np.append(nodes[1:], 27), point, force, torque)],     # outside the lattice
        [(name, np.zeros(0, np.uint32), point, force, torque)],       # empty
        [("", nodes, point, force, torque)],                          # unnamed
        [(name, nodes, point, force, (np.nan, 0.0, 0.0))],            # not finite
        [(name, nodes, point, (1.7e308, 1.7e308, 0.0), torque)],      # norm overflows
        [original, original],                                         # the same source twice
        [original, ("player-b",) + original[1:]],                     # overlapping regions
    ]
    for wrenches in bad:
        with pytest.raises(ValueError):
            be.set_external_wrenches(wrenches, 20)
    with pytest.raises(ValueError):
        be.set_external_wrenches([original], 0)
    st = be.run(device.RunControl(max_steps=4))
    sources = be.external_sources()
    assert len(sources) == 1 and sources[0][0] == "player-a" and sources[0][1].steps == 4
    be.set_external_wrenches([], 0)
    assert be.run(device.RunControl(max_steps=20)).external_load.steps == st.external_load.steps == 4


def test_unrepresentable_torque_refuses(device):
    """A torque on a region that cannot turn (one node: no lever arm) is
    refused when set, and the load in place stays."""
    case = _cube()
    _, be = _backend(device, case)
    be.set_external_wrenches([_player()], 2)
    with pytest.raises(ValueError):
        be.set_external_wrenches([_player(np.array([4]), source="hand")], 4)
    be.run(device.RunControl(max_steps=3))
    assert [(s, g.steps) for s, g in be.external_sources()] == [("player-a", 2)]


def test_forces_replace_wrenches(device):
    case = _cube()
    _, be = _backend(device, case)
    be.set_external_wrenches([_player()], 10)
    be.run(device.RunControl(max_steps=2))
    be.set_external_forces(np.tile([0.0, 1.0, 0.0], 27), 3)
    st = be.run(device.RunControl(max_steps=5))
    assert st.external_load.steps == 5
    assert [g.steps for _, g in be.external_sources()] == [2]


def test_wrenched_lattices_in_a_batch_equal_each_alone(device):
    """Bars of three sizes, each driven by its own wrenches, stepped by shared
    launches: each member's state and source ledgers are its run alone."""
    from banjo_gb300 import scenes

    cases = [scenes.wrenched_bar(steps=24), scenes.wrenched_bar(nx=12, ny=5, nz=7, steps=24, twist=(0.03, 0.0, 0.0)),
             scenes.wrenched_bar(nx=20, ny=6, nz=5, steps=24, hand=(0.0, 0.0, -3.0))]
    together = device.run_batch(cases)
    broke = 0
    for case, out in zip(cases, together):
        alone = device.run_case(case)
        assert "source_ledgers" in out
        assert mismatches(alone, out, STATE_KEYS) == []
        assert status_mismatches(alone, out) == []
        broke += int(out["status_u64"][4]) > 0
    assert broke >= 1
