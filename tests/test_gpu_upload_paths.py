"""The two upload paths give the same lattice.

Where the device reads pageable host memory (a Grace host's chip-to-chip
link), upload's conversion kernels read the caller's arrays in place;
elsewhere, or with GBL_STAGED_UPLOAD=1, the arrays are copied in chunks into
device staging buffers first. Both runs of the same case, each in its own
process (the choice is made once per process), must agree bit for bit.
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
case = scenes.impact_block(nx=24, ny=12, nz=16, blocks=3, radius=0.03, speed=12.0, steps=4)
out = lattice.run_case(case)
np.savez(sys.argv[1], **{{k: out[k] for k in {keys!r}}})
"""


def _run(path, staged):
    env = dict(os.environ)
    env.pop("GBL_STAGED_UPLOAD", None)
    if staged:
        env["GBL_STAGED_UPLOAD"] = "1"
    subprocess.run([sys.executable, "-c", SCRIPT.format(root=ROOT, keys=KEYS), str(path)], env=env, check=True,
                   timeout=600)
    return np.load(path)


def test_staged_and_in_place_uploads_agree(tmp_path):
    a = _run(tmp_path / "in_place.npz", staged=False)
    b = _run(tmp_path / "staged.npz", staged=True)
    assert int((a["alive"] == 0).sum()) > 0  # the case fractures
    for k in KEYS:
        assert np.array_equal(a[k].view(np.uint8), b[k].view(np.uint8)), k
