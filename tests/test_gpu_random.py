"""The device against the CPU checker on the seeded random scenes.

The same 24 scenes the checker is held to the reference harness on
(tests/test_oracle_random.py: impacts with and without plastic flow, drops,
thrown boxes with node contact, plate strikes, pinned beams, notched bars,
sizes and seeds drawn with seed 2026), run on the device and compared with the
checker bit for bit: every state array, the substep each bond broke, every
RunStatus counter, the FP64 ledgers within 1e-12.
"""
import pytest

from _util import LEDGER_RTOL, STATE_KEYS, mismatches, status_mismatches
from test_oracle_random import CASES

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("index", range(len(CASES)), ids=[label for label, _ in CASES])
def test_device_matches_checker_on_random_scenes(device, port, index):
    _, case = CASES[index]
    cpu = port.run_port(case, per_substep=True, threads=4)
    gpu = device.run_case(case, per_substep=True)
    assert mismatches(cpu, gpu, STATE_KEYS + ["break_step"]) == []
    assert status_mismatches(cpu, gpu, ledger_rtol=LEDGER_RTOL) == []
