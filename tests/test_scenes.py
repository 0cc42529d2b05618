"""Synthetic workloads: the shapes and counts the benchmark configurations name."""
import numpy as np

from banjo_gb300 import scenes


def test_offsets_are_face_and_edge_neighbours_in_walk_order():
    offs = scenes.half_offsets(1, 2)
    # dz, dy, dx ascending over the positive half-space (src/matter/Lattice.cpp:49-52).
    assert offs == [(1, 0, 0, 1), (-1, 1, 0, 2), (0, 1, 0, 1), (1, 1, 0, 2), (0, -1, 1, 2), (-1, 0, 1, 2),
                    (0, 0, 1, 1), (1, 0, 1, 2), (0, 1, 1, 2)]
    # Horizon rule of the reference generator: |o| <= 2 gives 6 + 12 + 8 + 6 = 32 per interior node.
    assert len(scenes.half_offsets(2, None)) == 16


def test_cantilever_counts_and_pin():
    c = scenes.cantilever()
    assert int(c["node_count"][0]) == 2048
    assert int(c["bond_count"][0]) == 15648
    assert int(c["pinned"].sum()) == 8 * 8
    assert np.all(c["threshold"].reshape(-1, 6)[:, :2] == 2e-3)
    assert np.all(np.isinf(c["threshold"].reshape(-1, 6)[:, 2:]))
    f = c["forces"].reshape(-1, 3)
    assert np.all(f[c["pinned"] == 1] == 0.0)
    assert np.allclose(f[c["pinned"] == 0, 1], -9.81e-3)


def test_node_index_and_interior_degree():
    a, b, _ = scenes.box_bonds(5, 5, 5)
    deg = np.bincount(np.concatenate([a, b]), minlength=125)
    centre = 2 + 5 * (2 + 5 * 2)
    assert deg[centre] == 18
    assert np.all(a < b)


def test_slabs_match_reference_rule():
    s = scenes.slabs(256, 128, 128, 32)
    assert s.size == 33 and s[0] == 0 and s[-1] == 256 * 128 * 128
    assert np.all(np.diff(s) == 4 * 256 * 128)


def test_streams_are_deterministic_and_uniform():
    u = scenes.uniform(7, 0, 10000)
    assert np.array_equal(u, scenes.uniform(7, 0, 10000))
    assert np.array_equal(u[100:200], scenes.uniform(7, 100, 100))
    assert 0.0 <= u.min() and u.max() < 1.0
    assert abs(u.mean() - 0.5) < 0.02
    ln = scenes.lognormal(20, 20000, 1.5e-3, 0.3)
    assert abs(np.median(ln) / 1.5e-3 - 1.0) < 0.02
    assert abs(np.std(np.log(ln)) - 0.3) < 0.01


def test_trial_parameters_ranges():
    e, c, s, h = scenes.trial_parameters(4096)
    assert e.min() >= 8 and e.max() <= 48
    assert c.min() >= 1e-8 and c.max() <= 1e-5
    assert s.min() >= 1e-3 and s.max() <= 5e-3
    assert h.min() >= 0.1 and h.max() <= 1.0
    assert abs(np.mean(e) - 28) < 0.6


def test_wrench_case_round_trip():
    """A case's wrenches unpack as they were packed (the layout every runner
    reads: names with a zero byte after each, counts, nodes, 9 numbers each)."""
    from banjo_gb300 import lattice, scenes

    case = scenes.wrenched_bar(nx=8, ny=4, nz=4, steps=5)
    got = lattice.case_wrenches(case)
    assert [w[0] for w in got] == ["hand", "grip"]
    assert int(case["wrench_substeps"][0]) == 5
    grip = got[1]
    i = np.asarray(grip[1])
    assert np.all(i % 8 == 7) and list(i) == sorted(i, reverse=True)  # the end face, given unsorted
    assert np.allclose(grip[3], (0.0, -4.0, 0.0)) and np.allclose(grip[4], (0.04, 0.0, 0.0))
    assert case["wrench_vectors"].size == 18 and case["wrench_nodes"].size == sum(len(w[1]) for w in got)
