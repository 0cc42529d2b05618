"""The bounds-checked build: no index out of range, and the same results.

libgbl_checked.so is the library with every data-driven index of its kernels
checked before use (bond ends, neighbour slots, candidate, dirty, event, load,
halo and isolated-node lists); a violation is recorded and the access skipped,
never trapped. The memory checker is not available on these machines, so this
build stands in for it: the golden fixtures, a sliced impact whose slabs
overflow the candidate cap, and a batch of uneven trials run through it in a
child process, which must record no violation and still reproduce every
reference and restatement output bit for bit.
"""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def test_checked_build_records_no_violation_and_keeps_parity(device):
    from banjo_gb300 import build

    assert os.path.exists(build.LIB_CHECKED)
    env = dict(os.environ, GBL_LIBRARY="checked")
    r = subprocess.run([sys.executable, os.path.join(HERE, "bounds_checked_run.py")], env=env, capture_output=True,
                       text=True, timeout=1200)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["report"]["checked"] is True
    assert line["report"]["violations"] == 0, line["report"]
    bad = [name for name, ok in line["parity"].items() if not ok]
    assert bad == []
    assert len(line["parity"]) > 10
