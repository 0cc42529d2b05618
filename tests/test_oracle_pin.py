"""The CPU checker is pinned to the reference itself.

The golden fixtures hold the outputs of the reference's own CPU lane
(tests/golden/make_golden.py runs oracle/_ref, built from the reference's
sources). The restatement must reproduce every one of them bit for bit:
schedule, final state, the substep each bond broke at, and the RunStatus.
Where the reference harness is built (this container), it is also compared
directly on cases that have no fixture.
"""
import os

import numpy as np
import pytest

from _util import SCHEDULE_KEYS, STATE_KEYS, golden_names, load_golden, mismatches, status_mismatches


@pytest.mark.parametrize("name", golden_names())
def test_port_reproduces_reference_fixture(port, name):
    case, ref, precision = load_golden(name)
    out = port.run_port(case, precision=precision, per_substep=True)
    assert mismatches(ref, out, SCHEDULE_KEYS + STATE_KEYS + ["break_step", "state_nbr_other"]) == []
    assert status_mismatches(ref, out) == []


@pytest.mark.parametrize("name", golden_names())
def test_threaded_port_is_bit_identical(port, name):
    case, ref, precision = load_golden(name)
    out = port.run_port(case, precision=precision, threads=4, per_substep=True)
    assert mismatches(ref, out, STATE_KEYS + ["break_step"]) == []
    assert status_mismatches(ref, out) == []


def test_resume_fixtures_are_not_the_uninterrupted_run(port):
    """The reference's download does not write the neighbour slots'
    aliveness back into the LatticeState (LatticeWorking.hpp:126-142), so a
    lattice uploaded from a downloaded state counts its failed bonds' slots in
    the strain again, and every derived array starts afresh: a resumed run is
    its own run (here its positions differ from the uninterrupted run's), and
    the fixture exercises the re-upload, not a copy of the uninterrupted
    result."""
    case, ref, precision = load_golden("resume_impact")
    case = {k: v for k, v in case.items() if k != "checkpoint_at"}
    whole = port.run_port(case, precision=precision)
    assert mismatches(ref, whole, ["u", "v", "alive"]) != []


def test_fixtures_contain_fracture():
    # The two-cell contact pairs hold at most one bond and are about contact,
    # not fracture; every other fixture runs through bond failure.
    broken = {n: int(load_golden(n)[1]["status_u64"][4]) for n in golden_names() if not n.startswith("contact_pair")}
    assert len(broken) >= 5
    assert all(b > 0 for b in broken.values()), broken


def test_audit_fixtures_carry_the_audit():
    """The reference records the audit only when asked (RunStatus::energy_audited,
    CpuLatticeBackend.cpp:114): the damping sweep removes energy, the striker
    passes move it; every other fixture's audit slots are zero."""
    damping, striker, audited = 26, 27, 18
    for name in golden_names():
        ref = load_golden(name)[1]
        u, d = ref["status_u64"], ref["status_f64"]
        if name.startswith("audit_"):
            assert int(u[audited]) == 1 and d[damping] > 0 and d[striker] != 0, name
        else:
            assert (len(u) <= audited or int(u[audited]) == 0) and (len(d) <= damping or
                                                                      (d[damping] == 0 and d[striker] == 0)), name


def test_contact_fixtures_hold_the_reference_rules():
    """The reference's own assertions on its two-cell contact pairs
    (fast_lattice_tests.cpp:800-896), on the fixtures its code produced."""
    u64 = lambda n: load_golden(n)[1]["status_u64"]  # noqa: E731
    f64 = lambda n: load_golden(n)[1]["status_f64"]  # noqa: E731
    contacts, rebuilds, listed, dissipated, correction = 13, 15, 16, 20, 22
    closing = load_golden("contact_pair_closing")[1]
    assert u64("contact_pair_closing")[contacts] > 0
    x = closing["u"].reshape(-1, 3)[:, 0] + np.array([-0.01, 0.01])
    assert x[1] - x[0] > 0.01 - 2 * 1e-5  # apart by at least the touch distance less the margin
    assert u64("contact_pair_bonded")[rebuilds] > 0
    assert u64("contact_pair_bonded")[listed] == 0 and u64("contact_pair_bonded")[contacts] == 0
    assert u64("contact_pair_dead")[listed] > 0 and f64("contact_pair_dead")[correction] > 0.0
    m = f64("contact_pair_momentum")
    assert u64("contact_pair_momentum")[contacts] > 0 and m[dissipated] > 0.0
    assert max(abs(m[23]), abs(m[24]), abs(m[25])) < 1e-14 * 2.5e-3  # below 1e-14 of the pair's momentum
    drop = u64("contact_drop")
    assert drop[contacts] > 0 and drop[listed] > 0 and int(drop[4]) > 0


def _reference_built():
    import oracle

    return os.path.exists(oracle.REF_BIN)


@pytest.mark.skipif(not _reference_built(), reason="reference harness not built here (no reference tree)")
@pytest.mark.parametrize("blocks", [1, 3, 8])
def test_port_matches_reference_on_slab_counts(port, blocks):
    from banjo_gb300 import scenes

    case = scenes.impact_block(nx=12, ny=8, nz=16, blocks=blocks, radius=0.025, speed=9.0, steps=6, seed_point=9,
                               seed_strength=31)
    ref = port.run_reference(case, per_substep=True)
    out = port.run_port(case, per_substep=True)
    assert mismatches(ref, out, SCHEDULE_KEYS + STATE_KEYS + ["break_step"]) == []
    assert status_mismatches(ref, out) == []


@pytest.mark.skipif(not _reference_built(), reason="reference harness not built here (no reference tree)")
def test_port_matches_reference_with_loads_in_double(port):
    from banjo_gb300 import scenes

    case = scenes.cantilever(nx=12, ny=4, nz=4, steps=6)
    ref = port.run_reference(case, precision="double", per_substep=True)
    out = port.run_port(case, precision="double", per_substep=True)
    assert mismatches(ref, out, STATE_KEYS + ["break_step"]) == []
    assert status_mismatches(ref, out) == []


def test_float_lane_tracks_double_lane(port):
    """CPU float vs CPU double before fracture: |du| < 1e-6 m, the reference's
    own bound (tests/fast_lattice_tests.cpp:441-445)."""
    from banjo_gb300 import scenes

    case = scenes.cantilever(steps=1)
    f = port.run_port(case, precision="float")
    d = port.run_port(case, precision="double")
    assert int(d["status_u64"][4]) == 0
    assert np.max(np.abs(f["u"] - d["u"])) < 1e-6
