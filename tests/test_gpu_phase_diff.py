"""The phase-diff debug mode on the device: at chosen substeps of cases that
exercise every phase kind -- a sliced sphere impact with plastic flow, node
contact between crack faces, damping with a two-plane ledge, a wrench load --
the device's state after every comparable phase equals the restatement's bit
for bit (tests/phase_diff.py says which phases and arrays compare)."""
import pytest

import phase_diff

pytestmark = pytest.mark.gpu


def _check(case, substep, precision="float"):
    phases, bad = phase_diff.phase_diff(case, substep, precision)
    assert bad == {}, phase_diff.first_divergence(bad)
    return phases


@pytest.mark.parametrize("substep", [0, 9, 23])
def test_impact_every_phase(device, port, substep):
    from banjo_gb300 import scenes

    case = scenes.impact_block(nx=48, ny=24, nz=48, blocks=4, radius=0.1, steps=3)
    assert 4 in _check(case, substep)


def test_node_contact_every_phase(device, port):
    from banjo_gb300 import scenes

    case = scenes.contact_drop(nx=24, ny=10, nz=18, speed=6.0, steps=40)
    assert 15 in _check(case, 25)


def test_damped_ledge_and_double_lane(device, port):
    from _util import load_golden

    case, _, precision = load_golden("damped_ledge")
    assert 9 in _check(case, 30, precision)
    case, _, precision = load_golden("impact_small_double")
    assert precision == "double"
    _check(case, 12, precision)


def test_wrench_every_phase(device, port):
    from _util import load_golden

    case, _, precision = load_golden("wrench_bar")
    _check(case, 15, precision)
