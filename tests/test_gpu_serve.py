"""The served form: requests admitted while others run, under a memory budget.

Each request's result must be the one it gets alone, whatever else is on the
device when it arrives, runs and leaves: the state bit for bit and every
RunStatus counter (its ledgers sum in an order fixed by its own bonds).
"""
import numpy as np
import pytest

from _util import STATE_KEYS, mismatches, status_mismatches

# A served request reports no first-failure list.
SERVED_KEYS = [k for k in STATE_KEYS if k != "first_failure_bonds"]

pytestmark = pytest.mark.gpu


def _requests():
    from banjo_gb300 import scenes

    shapes = [(8, 6, 8), (12, 5, 9), (6, 6, 6), (10, 7, 5), (5, 4, 13), (9, 9, 4)]
    heights = [0.004, 0.005, 0.02, 0.006, 0.03, 0.004]
    substeps = [110, 95, 40, 120, 25, 87]
    cases = []
    for k, ((nx, ny, nz), h, s) in enumerate(zip(shapes, heights, substeps)):
        c = scenes.drop_trial(nx, ny, nz, compliance=10.0 ** (-7 + 0.4 * k), break_strain=1.0e-3 + 4e-4 * k,
                              drop_height=h, steps=1)
        c["steps"] = np.array([s], dtype=np.uint64)
        cases.append(c)
    return cases


def _prepared(device, case):
    n = int(case["node_count"][0])
    sched = device.build_lattice_schedule(n, case["bond_a"], case["bond_b"], case["node_block_begin"])
    state = device.build_lattice_state(case, sched)
    return sched, state


def _result(device, state, sphere, status):
    out = {"u": state.u.copy(), "u_prev": state.u_prev.copy(), "v": state.v.copy(), "alive": state.alive.copy(),
           "failure_mode": state.failure_mode.copy(), "damage": state.damage.copy(),
           "plastic_extension": state.plastic_extension.copy(), "plastic_strain": state.plastic_strain.copy(),
           "prev_tensile": state.prev_tensile.copy(), "prev_compressive": state.prev_compressive.copy(),
           "prev_shear": state.prev_shear.copy(), "sphere_out": device.pack_sphere(sphere)}
    out.update(device.status_arrays(status))
    return out


def _serve(device, cases, budget, arrivals, chunk=7, borrow=False, lane_threshold=None):
    """Submits case k before step arrivals[k]; steps until every request is done."""
    server = device.Server(device.step_settings(cases[0]["settings"]), budget)
    if lane_threshold is not None:
        server.set_lane_threshold(lane_threshold)
    tickets, states, peak = {}, {}, 0
    step = 0
    while len(tickets) < len(cases) or any(server.poll(t).phase != device.REQUEST_DONE for t in tickets.values()):
        for k, at in enumerate(arrivals):
            if at == step and k not in tickets:
                sched, state = _prepared(device, cases[k])
                states[k] = state
                tickets[k] = server.submit(sched, state, device.sphere_state(cases[k]["sphere"]),
                                           int(cases[k]["steps"][0]), borrow=borrow)
        st = server.step(chunk)
        peak = max(peak, st.running)
        assert st.bytes_in_use <= budget
        step += 1
        assert step < 1000
    outs = {}
    for k, t in tickets.items():
        info = server.poll(t)
        assert info.substeps_done == int(cases[k]["steps"][0])
        assert info.admitted_s >= info.submitted_s and info.finished_s >= info.admitted_s
        sphere, status = server.take(t, states[k])
        outs[k] = _result(device, states[k], sphere, status)
    return outs, peak


def test_served_results_equal_each_request_alone(device):
    cases = _requests()
    outs, peak = _serve(device, cases, budget=1 << 34, arrivals=[0, 0, 1, 3, 3, 6])
    assert peak >= 3  # requests overlapped on the device
    broke = 0
    for k, case in enumerate(cases):
        alone = device.run_case(case)
        assert mismatches(alone, outs[k], SERVED_KEYS) == [], k
        assert status_mismatches(alone, outs[k]) == [], k
        broke += int(outs[k]["status_u64"][4]) > 0
    assert broke >= 3


def test_budget_limits_admission(device):
    cases = _requests()
    sizes = []
    for c in cases:
        sched, state = _prepared(device, c)
        sizes.append(device.footprint(state.node_count, state.bond_count, state.view.max_degree, 1))
    budget = sorted(sizes)[-1] + sorted(sizes)[-2]  # never more than two of the largest at once
    outs, peak = _serve(device, cases, budget=budget, arrivals=[0] * len(cases))
    assert 1 <= peak < len(cases)
    for k, case in enumerate(cases):
        alone = device.run_case(case)
        assert mismatches(alone, outs[k], SERVED_KEYS) == [], k


def test_oversize_request_and_cancel(device):
    cases = _requests()
    sched, state = _prepared(device, cases[0])
    small = device.Server(device.step_settings(cases[0]["settings"]), 1024)
    with pytest.raises(ValueError, match="budget"):
        small.submit(sched, state, device.sphere_state(cases[0]["sphere"]), 10)
    server = device.Server(device.step_settings(cases[0]["settings"]), 1 << 34)
    held = [_prepared(device, c) for c in cases[:3]]
    t = [server.submit(s, st, device.sphere_state(c["sphere"]), int(c["steps"][0])) for (s, st), c in
         zip(held, cases[:3])]
    server.step(5)
    server.cancel(t[1])  # running: leaves between substeps
    with pytest.raises(ValueError):
        server.poll(t[1])
    while server.poll(t[0]).phase != device.REQUEST_DONE or server.poll(t[2]).phase != device.REQUEST_DONE:
        server.step(16)
    for k in (0, 2):
        sphere, status = server.take(t[k], held[k][1])
        out = _result(device, held[k][1], sphere, status)
        alone = device.run_case(cases[k])
        assert mismatches(alone, out, SERVED_KEYS) == []
    st = server.stats()
    assert st.running == 0 and st.queued == 0 and st.bytes_in_use == 0


def test_borrowed_requests_equal_each_request_alone(device):
    """Borrowed states (read by the device at admission, some after waiting
    for memory) give the results the same requests get alone."""
    cases = _requests()
    sizes = []
    for c in cases:
        sched, state = _prepared(device, c)
        sizes.append(device.footprint(state.node_count, state.bond_count, state.view.max_degree, 1))
    budget = sorted(sizes)[-1] + sorted(sizes)[-2]
    outs, peak = _serve(device, cases, budget=budget, arrivals=[0, 0, 0, 1, 1, 2], borrow=True)
    assert 1 <= peak < len(cases)
    for k, case in enumerate(cases):
        alone = device.run_case(case)
        assert mismatches(alone, outs[k], SERVED_KEYS) == [], k
        assert status_mismatches(alone, outs[k]) == [], k


def test_two_lanes_equal_each_request_alone(device):
    """With the large lane's threshold inside the requests' sizes, the larger
    requests run on the helper thread's lane while the smaller ones step
    beside them, several chunks per step: every result is still the one the
    request gets alone."""
    cases = _requests()
    sizes = sorted(int(c["bond_count"][0]) for c in cases)
    threshold = sizes[len(sizes) // 2]
    outs, peak = _serve(device, cases, budget=1 << 34, arrivals=[0, 1, 1, 2, 4, 4], chunk=5,
                        lane_threshold=threshold)
    assert peak >= 3
    assert sum(int(c["bond_count"][0]) >= threshold for c in cases) >= 2
    for k, case in enumerate(cases):
        alone = device.run_case(case)
        assert mismatches(alone, outs[k], SERVED_KEYS) == [], k
        assert status_mismatches(alone, outs[k]) == [], k
