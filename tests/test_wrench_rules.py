"""The CPU checker's external wrenches against the reference's own rules.

The checker restates setExternalWrenches and the per-kick spread
(ExternalLoads.hpp:52-77, 171-238). Here it must refuse what the reference's
wrench tests refuse (tests/lattice_external_load_tests.cpp:387-422) and, where
the reference harness is built, agree with the reference itself bit for bit on
a moving two-source cube (:347-385) and refuse the same sets.
"""
import os

import numpy as np
import pytest

import oracle
from _util import STATE_KEYS, mismatches, status_mismatches

ORIGIN = np.array([2.0, 0.6, -1.0])


def _cube(steps=4):
    from banjo_gb300 import scenes

    case = scenes._box_case(3, 3, 3, 0.04, tuple(ORIGIN), 1e-7, [scenes.INF] * 6)
    case["mass"] = np.full(27, 0.25)
    case["origin"] = ORIGIN.copy()
    case["settings"] = scenes.settings(gravity=(0.0, 0.0, 0.0))
    case["steps"] = np.array([steps], dtype=np.uint64)
    p = case["ref_pos"].reshape(-1, 3) - ORIGIN
    case["vel"] = (np.array([3.0, -2.0, 1.0]) + np.cross(np.array([0.0, 30.0, 0.0]), p)).reshape(-1)
    return case


def _wrench(source="player-a", nodes=None, force=(20.0, -10.0, 5.0), torque=(0.5, -0.75, 1.25)):
    return (source, np.arange(27) if nodes is None else np.asarray(nodes), ORIGIN + np.array([0.02, -0.03, 0.04]),
            force, torque)


def _with(wrenches, substeps=4):
    from banjo_gb300 import scenes

    return scenes.wrenches(_cube(), wrenches, substeps)


BAD = {
    "node twice": [_wrench(nodes=np.append(np.arange(27), 0))],
    "outside": [_wrench(nodes=np.append(np.arange(1, 27), 27))],
    "unnamed": [_wrench(source="")],
    "not finite": [_wrench(torque=(np.nan, 0.0, 0.0))],
    "norm overflows": [_wrench(force=(1.7e308, 1.7e308, 0.0))],
    "same source twice": [_wrench(), _wrench()],
    "overlap": [_wrench(), _wrench(source="player-b")],
    "no lever arm": [_wrench(nodes=[4])],
}

_HARNESS = os.path.exists(oracle.REF_BIN)


@pytest.mark.parametrize("name", sorted(BAD))
def test_checker_refuses_what_the_reference_refuses(name):
    case = _with(BAD[name])
    with pytest.raises(RuntimeError):
        oracle.run_port(case)
    if _HARNESS:
        with pytest.raises(Exception):
            oracle.run_reference(case)


@pytest.mark.skipif(not _HARNESS, reason="the reference harness is not built here")
@pytest.mark.parametrize("precision", ["float", "double"])
def test_checker_matches_reference_on_two_moving_sources(precision):
    a = _wrench(nodes=np.arange(9)[::-1], force=(8.0, 2.0, 1.0), torque=(0.1, 0.2, -0.3))
    b = _wrench(source="player-b", nodes=np.arange(9, 27), force=(-3.0, -4.0, 0.5), torque=(-0.1, 0.05, 0.2))
    case = _with([b, a], substeps=3)  # the run outlasts the span by one substep
    ref = oracle.run_reference(case, precision=precision, per_substep=True)
    port = oracle.run_port(case, precision=precision, per_substep=True)
    assert mismatches(ref, port, STATE_KEYS) == []
    assert status_mismatches(ref, port) == []
    assert bytes(ref["source_names"]) == b"player-a\0player-b\0"
    assert list(ref["source_ledgers"].reshape(-1, 15)[:, 0]) == [3.0, 3.0]
