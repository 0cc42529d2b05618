"""The notched bar (energy-scaled law, plastic flow, horizon 2, pinned end,
ramped end load): the device against the CPU checker bit for bit over a long
ramp, and its FP32 error against the FP64 restatement reported.
"""
import numpy as np
import pytest

from _util import LEDGER_RTOL, STATE_KEYS, mismatches, status_mismatches

pytestmark = pytest.mark.gpu


def test_bar_long_ramp_matches_checker(device, port):
    from banjo_gb300 import scenes

    case = scenes.notched_bar(32, 10, 10, ramp_steps=800, steps=60)
    cpu = port.run_port(case, threads=8)
    gpu = device.run_case(case)
    assert int(cpu["status_u64"][4]) > 0 and float(cpu["status_f64"][2]) > 0.0  # bonds broke, plastic work done
    assert mismatches(cpu, gpu, STATE_KEYS) == []
    assert status_mismatches(cpu, gpu, ledger_rtol=LEDGER_RTOL) == []


def test_bar_fp32_against_fp64(device, port):
    """Before the first failure the FP32 lane tracks the FP64 one closely."""
    from banjo_gb300 import scenes

    case = scenes.notched_bar(24, 8, 8, ramp_steps=100000, steps=1)
    case["steps"] = np.array([13], dtype=np.uint64)  # one unloaded step, then loaded substeps up to the first failure
    gpu = device.run_case(case)
    cpu64 = port.run_port(case, precision="double", threads=4)
    assert int(gpu["status_u64"][4]) == 0 and int(cpu64["status_u64"][4]) == 0
    ref = case["ref_pos"].reshape(-1, 3)
    extent = float(np.max(ref.max(axis=0) - ref.min(axis=0)))
    err = np.abs(gpu["u"].astype(np.float64) - cpu64["u"]).max() / extent
    umax = np.abs(cpu64["u"]).max()
    print(f"notched bar, 13 substeps: max |u32 - u64| / extent = {err:.3e}; relative to the largest displacement "
          f"{err * extent / umax:.3e}")
    assert umax > 0.0 and err * extent <= 1e-4 * umax
