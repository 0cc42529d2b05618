"""The CPU checker against the reference itself on features combined.

Each fixture exercises one feature; these cases switch several on at once
(wrenches with the energy audit and damping, node contact with the audit, a
sphere impact with a wrench on the struck block) and hold the checker to the
reference harness bit for bit, both lanes. They run where the harness is built
(the reference tree is present); the device meets the same features through
the fixtures.
"""
import os

import numpy as np
import pytest

import oracle
from _util import STATE_KEYS, mismatches, status_mismatches

pytestmark = pytest.mark.skipif(not os.path.exists(oracle.REF_BIN), reason="the reference harness is not built here")


def _audited(case, damping=0.05):
    from banjo_gb300 import scenes

    case = dict(case)
    case["settings"] = case["settings"].copy()
    if len(case["settings"]) <= scenes.K_AUDIT:
        case["settings"] = np.concatenate([case["settings"], np.zeros(scenes.SETTINGS_WIDTH - len(case["settings"]))])
    case["settings"][scenes.K_DAMP] = damping
    case["settings"][scenes.K_AUDIT] = 1.0
    return case


def _cases():
    from banjo_gb300 import scenes

    out = {"wrenched_bar_audited": _audited(scenes.wrenched_bar(steps=16)),
           "contact_drop_audited": _audited(scenes.contact_drop(steps=12), damping=0.02)}
    impact = scenes.impact_block(nx=16, ny=10, nz=12, blocks=4, radius=0.03, speed=12.0, steps=2, seed_point=5,
                                 seed_strength=21)
    i = np.arange(int(impact["node_count"][0]))
    side = np.flatnonzero(i % 16 == 0)  # the x = 0 face, pushed sideways while the sphere strikes
    pos = impact["ref_pos"].reshape(-1, 3)
    out["impact_wrenched_audited"] = _audited(
        scenes.wrenches(impact, [("push", side, pos[side].mean(axis=0), (3.0, 0.0, 0.0), (0.0, 0.01, 0.0))], 20))
    return out


CASES = _cases()


@pytest.mark.parametrize("precision", ["float", "double"])
@pytest.mark.parametrize("name", sorted(CASES))
def test_checker_matches_reference_with_features_combined(name, precision):
    case = CASES[name]
    ref = oracle.run_reference(case, precision=precision, per_substep=True)
    port = oracle.run_port(case, precision=precision, per_substep=True, threads=4)
    assert mismatches(ref, port, STATE_KEYS + ["break_step"]) == []
    assert status_mismatches(ref, port) == []
    assert int(ref["status_u64"][18]) == 1 and ref["status_f64"][26] > 0  # audited, damping measured
