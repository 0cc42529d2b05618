"""Linear isotropic hardening against its closed form.

The reference checks its plastic return map on one bond held at a prescribed
extension (tests/lattice_plasticity_tests.cpp:191-230): loaded in one step to
four times the yield extension, the permanent extension must be
p = (target - yield) / (1 + H) within 1e-13 of the rest length, and the
plastic work (yield p + H p^2 / 2) / compliance within 1e-9 relative, for
H = 0, 0.02 and 0.1 (iron: 200 MPa yield over 211 GPa, 10 mm cell). Here the
same bond is a whole lattice: two nodes 10 mm apart, both pinned so that the
sweep cannot move them, no gravity, fracture off; one substep of the double
lane (direct arithmetic) runs the end sample's plastic return on the
prescribed extension. The checker is held to the closed form, and to the
reference harness bit for bit where the harness is built; the device meets the
same return map through the double-lane fixtures with plastic flow.
"""
import os

import numpy as np
import pytest

import oracle

REST = 0.01
COMPLIANCE = 4.7393364928909956e-10
YIELD_STRETCH = 200.0e6 / 211.0e9
INF = float("inf")


def one_bond_case(hardening: float, extension: float) -> dict:
    """Two pinned nodes, one bond along x stretched by `extension`, one substep."""
    from banjo_gb300 import scenes

    case = scenes._box_case(2, 1, 1, REST, (0.0, 0.0, 0.0), COMPLIANCE, [INF] * 6)
    assert int(case["bond_count"][0]) == 1
    pos = case["pos"].reshape(-1, 3).copy()
    pos[1, 0] += extension
    case["pos"] = pos.reshape(-1)
    case.update({
        "pinned": np.ones(2, dtype=np.uint8),
        "settings": scenes.settings(gravity=(0.0, 0.0, 0.0), direct=1, yield_stretch=YIELD_STRETCH,
                                    hardening=hardening),
        "steps": np.array([1], dtype=np.uint64),
    })
    return case


def closed_form(hardening: float, target: float) -> tuple[float, float]:
    y = YIELD_STRETCH * REST
    p = (target - y) / (1.0 + hardening)
    return p, (y * p + 0.5 * hardening * p * p) / COMPLIANCE


@pytest.mark.parametrize("hardening", [0.0, 0.02, 0.1])
def test_checker_hardening_follows_the_closed_form(port, hardening):
    target = 4.0 * YIELD_STRETCH * REST
    out = port.run_port(one_bond_case(hardening, target), precision="double")
    p, work = closed_form(hardening, target)
    assert abs(float(out["plastic_extension"][0]) - p) <= 1e-13 * REST
    assert abs(float(out["status_f64"][2]) - work) <= 1e-9 * work
    assert float(out["plastic_strain"][0]) == pytest.approx(p, rel=1e-12)  # monotone: accumulated = permanent
    assert int(out["status_u64"][4]) == 0  # fracture off


def test_checker_below_yield_leaves_no_permanent_extension(port):
    """Elastic below yield: the plastic state stays exactly zero."""
    out = port.run_port(one_bond_case(0.1, 0.5 * YIELD_STRETCH * REST), precision="double")
    assert float(out["plastic_extension"][0]) == 0.0 and float(out["status_f64"][2]) == 0.0


@pytest.mark.skipif(not os.path.exists(oracle.REF_BIN), reason="the reference harness is not built here")
@pytest.mark.parametrize("hardening", [0.0, 0.02, 0.1])
def test_reference_harness_gives_the_same_return(hardening):
    case = one_bond_case(hardening, 4.0 * YIELD_STRETCH * REST)
    ref = oracle.run_reference(case, precision="double")
    port = oracle.run_port(case, precision="double")
    for key in ("plastic_extension", "plastic_strain", "u", "v"):
        assert np.array_equal(np.asarray(ref[key]).view(np.uint8), np.asarray(port[key]).view(np.uint8)), key
    assert float(ref["status_f64"][2]) == float(port["status_f64"][2])
