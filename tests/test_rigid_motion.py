"""A rigid motion strains nothing (fast_lattice_tests.cpp:165-224).

The reference's known-answer test rotates a lattice's current positions by
0.37 rad about a tilted axis and shifts them, leaving the rest configuration
untouched, and requires every bond's strain sample to stay below 1e-9 -- for a
solid block, a sheet one cell thick (the rank-deficient neighbourhood the
pseudo-inverse handles) and a slab two cells thick. Here the same motion is
given to box lattices in the direct (double) arithmetic, run one substep with
no gravity and no load, and the bonds' recorded peaks must stay below 1e-9:
on the CPU restatement, and on the device equal to it bit for bit.
"""
import numpy as np
import pytest

CASES = [("solid block", (6, 3, 4), 0.02), ("sheet one cell thick", (12, 1, 8), 0.01),
         ("two cells thick", (12, 2, 8), 0.01)]


def _rigid_case(dims, cell):
    from banjo_gb300 import scenes

    nx, ny, nz = dims
    inf = scenes.INF
    case = scenes._box_case(nx, ny, nz, cell, (0.0, 0.0, 0.0), 1e-7, [inf] * 6)
    angle = 0.37
    axis = np.array([0.3, 0.8, 0.5])
    axis /= np.linalg.norm(axis)
    c, s, t = np.cos(angle), np.sin(angle), 1.0 - np.cos(angle)
    x, y, z = axis
    rot = np.array([[t * x * x + c, t * x * y - s * z, t * x * z + s * y],
                    [t * x * y + s * z, t * y * y + c, t * y * z - s * x],
                    [t * x * z - s * y, t * y * z + s * x, t * z * z + c]])
    ref = case["ref_pos"].reshape(-1, 3)
    case["pos"] = (ref @ rot.T + np.array([0.31, -0.17, 0.09])).reshape(-1)
    case["settings"] = scenes.settings(gravity=(0.0, 0.0, 0.0), direct=1)
    case["steps"] = np.array([1], dtype=np.uint64)
    return case


def _worst(out):
    return max(float(np.abs(out[k]).max()) for k in ("prev_tensile", "prev_compressive", "prev_shear"))


@pytest.mark.parametrize("name,dims,cell", CASES)
def test_rigid_motion_strains_nothing_on_the_checker(port, name, dims, cell):
    out = port.run_port(_rigid_case(dims, cell), precision="double")
    assert int(out["status_u64"][4]) == 0
    assert _worst(out) < 1e-9, name


@pytest.mark.gpu
@pytest.mark.parametrize("name,dims,cell", CASES)
def test_rigid_motion_strains_nothing_on_the_device(device, port, name, dims, cell):
    from _util import STATE_KEYS, mismatches

    case = _rigid_case(dims, cell)
    cpu = port.run_port(case, precision="double")
    gpu = device.run_case(case, precision="double")
    assert _worst(gpu) < 1e-9, name
    assert mismatches(cpu, gpu, STATE_KEYS) == []
