"""The library's box-lattice builder against the scene generator.

The scene generator (numpy) is pinned to the reference's generator through the
golden fixtures; the library's C++ builder must produce the same lattice bit
for bit, so that either can feed a run.
"""
import numpy as np
import pytest

from banjo_gb300 import scenes


@pytest.mark.parametrize("dims,blocks", [((5, 4, 3), 1), ((7, 3, 9), 3), ((1, 6, 2), 2), ((12, 5, 8), 8)])
def test_box_matches_scene_generator(gbl, dims, blocks):
    nx, ny, nz = dims
    thr = (1e-3, 2e-3, scenes.INF, scenes.INF, 3e-3, scenes.INF)
    case = scenes._box_case(nx, ny, nz, 0.01, (0.1, -0.2, 0.3), 1e-6, list(thr), blocks=blocks)
    box = gbl.build_box(nx, ny, nz, 0.01, center=(0.1, -0.2, 0.3), compliance=1e-6, threshold=thr, slabs=blocks)
    for key in ("ref_pos", "pos", "vel", "mass", "bond_a", "bond_b", "rest_length", "compliance", "threshold"):
        want = np.asarray(case[key])
        got = box.array(key)
        assert got.shape == want.shape and np.array_equal(got.view(np.uint8), want.astype(got.dtype).view(np.uint8)), key
    assert np.array_equal(box.node_block_begin, case["node_block_begin"])


def test_box_horizon_rule_matches_scene_offsets(gbl):
    box = gbl.build_box(6, 5, 5, 0.02, horizon=2, max_offset_sq=0)
    a, b, d2 = scenes.box_bonds(6, 5, 5, max_d2=None, horizon=2)
    assert np.array_equal(box.array("bond_a"), a) and np.array_equal(box.array("bond_b"), b)
    assert np.array_equal(box.array("rest_length"), np.sqrt(d2.astype(np.float64)) * 0.02)


def test_box_state_equals_case_state(gbl):
    case = scenes.drop_trial(9, 6, 7, compliance=3e-7, break_strain=2e-3, drop_height=0.35)
    n = int(case["node_count"][0])
    sched = gbl.build_lattice_schedule(n, case["bond_a"], case["bond_b"], case["node_block_begin"])
    want = gbl.build_lattice_state(case, sched)
    lift = 0.35 + 0.5 * 6 * 0.01
    box = gbl.build_box(9, 6, 7, 0.01, center=(0.0, lift, 0.0), compliance=3e-7,
                        threshold=(2e-3, 2e-3, scenes.INF, scenes.INF, scenes.INF, scenes.INF))
    bsched = gbl.box_schedule(box)
    got = gbl.box_state(box, bsched)
    for key in ("x0", "u", "v", "mass", "inv_mass", "nbr_bond", "nbr_other", "nbr_rest", "rest_edge", "rest_length",
                "compliance", "threshold", "bond_a", "bond_b"):
        assert np.array_equal(getattr(got, key), getattr(want, key)), key
    assert np.array_equal(bsched.arrays()["sched_bond_order"], sched.arrays()["sched_bond_order"])
