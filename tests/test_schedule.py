"""Host builders of the library: the schedule and the canonical state.

The greedy colouring and the slab grouping are integer work and must equal the
reference's bit for bit (golden fixtures); the colouring properties restate
tests/fast_lattice_tests.cpp:110-143 (one colour never shares a node, every
bond swept once, owner = lower slab, bonds join adjacent slabs only).
"""
import numpy as np
import pytest

from _util import SCHEDULE_KEYS, golden_names, load_golden, mismatches


@pytest.mark.parametrize("name", golden_names())
def test_schedule_and_state_equal_reference(gbl, name):
    case, ref, _ = load_golden(name)
    s = gbl.build_lattice_schedule(case["node_count"][0], case["bond_a"], case["bond_b"], case["node_block_begin"])
    assert mismatches(ref, s.arrays(), SCHEDULE_KEYS) == []
    st = gbl.build_lattice_state(case, s)
    assert np.array_equal(st.nbr_other, ref["state_nbr_other"])
    assert st.view.max_degree == int(ref["state_max_degree"][0])


@pytest.mark.parametrize("blocks", [1, 4, 16])
def test_schedule_is_a_proper_colouring(gbl, blocks):
    from banjo_gb300 import scenes

    nx, ny, nz = 6, 2, 16
    a, b, _ = scenes.box_bonds(nx, ny, nz)
    slabs = scenes.slabs(nx, ny, nz, blocks)
    s = gbl.build_lattice_schedule(nx * ny * nz, a, b, slabs)
    arr = s.arrays()
    assert s.block_count == min(blocks, nz)
    assert 0 < s.color_count <= 64
    order = arr["sched_bond_order"]
    seen = np.zeros(a.size, dtype=np.int64)
    block_of = np.searchsorted(slabs, np.arange(nx * ny * nz), side="right") - 1
    C = s.color_count
    for blk in range(s.block_count):
        for boundary in (0, 1):
            for c in range(C):
                key = (blk * 2 + boundary) * C + c
                lo, hi = arr["sched_range_begin"][key], arr["sched_range_end"][key]
                bonds = order[lo:hi]
                ends = np.concatenate([a[bonds], b[bonds]])
                assert np.unique(ends).size == ends.size, "one colour never shares a node"
                seen[bonds] += 1
                ba, bb = block_of[a[bonds]], block_of[b[bonds]]
                assert np.all(np.minimum(ba, bb) == blk), "owner is the lower slab"
                assert np.all((ba != bb) == (boundary == 1)), "boundary flag matches the slabs"
                assert np.all(np.abs(ba - bb) <= 1), "bonds join adjacent slabs only"
    assert np.all(seen == 1), "every bond is swept exactly once"


def test_schedule_refuses_thin_slabs(gbl):
    from banjo_gb300 import scenes

    a, b, _ = scenes.box_bonds(4, 4, 6)
    thin = np.array([0, 16, 32, 96], dtype=np.uint32)  # one-layer slabs cannot hold a diagonal across two
    a2 = np.append(a, [0]).astype(np.uint32)
    b2 = np.append(b, [40]).astype(np.uint32)  # joins slab 0 and slab 2
    with pytest.raises(ValueError, match="slab"):
        gbl.build_lattice_schedule(96, a2, b2, thin)


def test_schedule_refuses_invalid_bonds(gbl):
    with pytest.raises(ValueError, match="invalid nodes"):
        gbl.build_lattice_schedule(4, [0, 1], [1, 1], [0, 4])
    with pytest.raises(ValueError, match="invalid nodes"):
        gbl.build_lattice_schedule(4, [0, 1], [1, 7], [0, 4])
    with pytest.raises(ValueError, match="block offsets"):
        gbl.build_lattice_schedule(4, [0], [1], [0, 3])


def test_state_builder_geometry(gbl):
    from banjo_gb300 import scenes

    case = scenes.cantilever(nx=5, ny=3, nz=3, steps=1)
    s = gbl.build_lattice_schedule(case["node_count"][0], case["bond_a"], case["bond_b"], case["node_block_begin"])
    st = gbl.build_lattice_state(case, s)
    order = s.arrays()["sched_bond_order"]
    ref = case["ref_pos"].reshape(-1, 3)
    edge = ref[case["bond_b"][order]] - ref[case["bond_a"][order]]
    assert np.array_equal(st.rest_edge.reshape(-1, 3), edge)
    e2 = np.sum(edge * edge, axis=1)
    assert np.array_equal(st.weight, 1.0 / e2)
    assert np.all(st.inv_mass[case["pinned"] == 1] == 0.0)
    assert np.all(st.inv_mass[case["pinned"] == 0] == 1.0 / 1e-3)
    # Padded slots carry no bond; every bond sits in one slot of each end.
    N, D = int(case["node_count"][0]), st.view.max_degree
    slots = st.nbr_bond.reshape(D, N)
    assert np.all(st.nbr_bond[st.bond_slot_a] == np.arange(st.bond_count))
    assert np.all(st.nbr_bond[st.bond_slot_b] == np.arange(st.bond_count))
    assert np.sum(slots != 0xFFFFFFFF) == 2 * st.bond_count
