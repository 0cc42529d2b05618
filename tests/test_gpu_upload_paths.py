"""The upload paths and host copy modes give the same lattice.

Upload's conversion kernels read the caller's arrays in place where the
device reads pageable host memory (a Grace host's chip-to-chip link;
GBL_UPLOAD=in_place, the default below 1 GiB of arrays), or the arrays are
copied in chunks into device staging buffers and converted there
(GBL_UPLOAD=staged, the default above). Downloads and copies to the device
of 64 MB or more go through two page-locked staging slices of 64 MB
(GBL_HOST_COPY unset or "pinned"), or through the driver's own staging
(GBL_HOST_COPY=driver). Runs of the same case under each choice, each in its own process (the choices
are made once per process), must agree bit for bit. The larger case moves
several slices each way, so the alternation of the two slices is exercised
both ways.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
KEYS = ("u", "u_prev", "v", "alive", "failure_mode", "damage", "prev_tensile", "prev_compressive", "prev_shear",
        "plastic_extension", "plastic_strain")
SCRIPT = """
import sys
import numpy as np
sys.path.insert(0, {root!r})
from banjo_gb300 import lattice, scenes
case = scenes.impact_block({shape}, radius=0.03, speed=12.0, steps=4)
out = lattice.run_case(case)
np.savez(sys.argv[1], **{{k: out[k] for k in {keys!r}}})
"""
SMALL = "nx=24, ny=12, nz=16, blocks=3"
# 294,912 nodes and 2,585,504 bonds: 643 MiB up (eleven slices) and 144 MiB down (three).
LARGE = "nx=96, ny=48, nz=64, blocks=8"


def _run(path, shape, staged, host_copy=None):
    env = dict(os.environ)
    env.pop("GBL_UPLOAD", None)
    env.pop("GBL_HOST_COPY", None)
    env["GBL_UPLOAD"] = "staged" if staged else "in_place"
    if host_copy:
        env["GBL_HOST_COPY"] = host_copy
    subprocess.run([sys.executable, "-c", SCRIPT.format(root=ROOT, keys=KEYS, shape=shape), str(path)], env=env,
                   check=True, timeout=600)
    return np.load(path)


def _same(a, b):
    return [k for k in KEYS if not np.array_equal(a[k].view(np.uint8), b[k].view(np.uint8))]


def test_staged_and_in_place_uploads_agree(tmp_path):
    a = _run(tmp_path / "in_place.npz", SMALL, staged=False)
    b = _run(tmp_path / "staged.npz", SMALL, staged=True)
    assert int((a["alive"] == 0).sum()) > 0  # the case fractures
    assert _same(a, b) == []


def test_host_copy_modes_agree_over_many_slices(tmp_path):
    a = _run(tmp_path / "in_place_pinned.npz", LARGE, staged=False, host_copy="pinned")
    b = _run(tmp_path / "staged_pinned.npz", LARGE, staged=True, host_copy="pinned")
    c = _run(tmp_path / "staged_driver.npz", LARGE, staged=True, host_copy="driver")
    assert int((a["alive"] == 0).sum()) > 0
    assert _same(a, b) == []
    assert _same(a, c) == []
