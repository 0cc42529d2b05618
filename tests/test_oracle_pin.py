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


def test_fixtures_contain_fracture():
    broken = {n: int(load_golden(n)[1]["status_u64"][4]) for n in golden_names()}
    assert len(broken) >= 5
    assert all(b > 0 for b in broken.values()), broken


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
