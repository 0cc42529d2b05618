"""The energy audit (StepSettings::audit_energy) on the device.

With the audit on, the reference measures what the striker passes and the
radial damping sweep take out of the lattice as differences of its total
kinetic energy across each phase, folded serially in node order
(CpuLatticeBackend.cpp:388-422, LatticePhysics.hpp:1676-1682). The device folds
in the same order, so the two audit ledgers are held bit for bit -- against the
reference's own fixtures (audit_impact*, in the fixture parity test), against
the CPU checker here, alone and in a batch. The audit measures only: the state
it leaves is the state of the same run without it.
"""
import pytest

from _util import LEDGER_RTOL, STATE_KEYS, mismatches, status_mismatches

pytestmark = pytest.mark.gpu

DAMPING, STRIKER, AUDITED = 26, 27, 18


def _audited_impact(nx=24, ny=12, nz=24, blocks=6, steps=6, seed_point=2, audit=True):
    from banjo_gb300 import scenes

    case = scenes.impact_block(nx=nx, ny=ny, nz=nz, blocks=blocks, radius=0.04, speed=12.0, steps=steps,
                               seed_point=seed_point, seed_strength=9)
    case["settings"] = case["settings"].copy()
    case["settings"][scenes.K_DAMP] = 0.05
    case["settings"][scenes.K_AUDIT] = 1.0 if audit else 0.0
    return case


def test_audit_matches_checker(device, port):
    case = _audited_impact()
    cpu = port.run_port(case, threads=8, per_substep=True)
    gpu = device.run_case(case, per_substep=True)
    assert int(gpu["status_u64"][AUDITED]) == 1
    assert gpu["status_f64"][DAMPING] > 0 and gpu["status_f64"][STRIKER] != 0
    assert mismatches(cpu, gpu, STATE_KEYS + ["break_step"]) == []
    assert status_mismatches(cpu, gpu, ledger_rtol=LEDGER_RTOL) == []


def test_audit_double_lane_matches_checker(device, port):
    case = _audited_impact(nx=16, ny=10, nz=12, blocks=4, steps=3)
    cpu = port.run_port(case, precision="double", per_substep=True)
    gpu = device.run_case(case, precision="double", per_substep=True)
    assert mismatches(cpu, gpu, STATE_KEYS + ["break_step"]) == []
    assert status_mismatches(cpu, gpu, ledger_rtol=LEDGER_RTOL) == []


def test_audit_measures_only(device):
    on = device.run_case(_audited_impact())
    off = device.run_case(_audited_impact(audit=False))
    assert mismatches(on, off, STATE_KEYS) == []
    assert int(off["status_u64"][AUDITED]) == 0
    assert off["status_f64"][DAMPING] == 0 and off["status_f64"][STRIKER] == 0


def test_audit_in_a_batch_equals_alone(device):
    cases = [_audited_impact(), _audited_impact(nx=32, ny=12, nz=16, blocks=8, seed_point=5),
             _audited_impact(nx=16, ny=12, nz=40, blocks=4, seed_point=7)]
    together = device.run_batch(cases)
    for case, out in zip(cases, together):
        alone = device.run_case(case)
        assert out["status_f64"][DAMPING] > 0
        assert mismatches(alone, out, STATE_KEYS) == []
        assert status_mismatches(alone, out) == []  # exact, audit ledgers included
