"""The phase-diff tool's comparison, on the CPU: two restatement runs that
differ only in the sweep (a planted difference in the oracle's input: one
projection iteration fewer) must agree through the kick and the first contact
pass and part at the sweep, the first phase the difference touches."""
import numpy as np

import phase_diff


def test_planted_sweep_difference_is_found_at_the_sweep(port):
    from banjo_gb300 import scenes

    case = scenes.impact_block(nx=24, ny=12, nz=16, blocks=4, radius=0.05, steps=1)
    fewer = dict(case)
    fewer["settings"] = case["settings"].copy()
    fewer["settings"][scenes.K_ITER] = case["settings"][scenes.K_ITER] - 1
    phases = phase_diff.phases_for(case)
    a = phase_diff.port_phases(case, 0, phases, threads=2)
    b = phase_diff.port_phases(fewer, 0, phases, threads=2)
    bad = phase_diff.compare(a, b, phases)
    first = phase_diff.first_divergence(bad)
    assert first is not None and first[0] == 7 and "u" in first[2]
    assert 3 not in bad and 4 not in bad


def test_identical_runs_agree_at_every_phase(port):
    from banjo_gb300 import scenes

    case = scenes.impact_block(nx=24, ny=12, nz=16, blocks=4, radius=0.05, steps=1)
    phases = phase_diff.phases_for(case)
    a = phase_diff.port_phases(case, 3, phases, threads=1)
    b = phase_diff.port_phases(case, 3, phases, threads=3)
    assert phase_diff.compare(a, b, phases) == {}
    assert set(phases) == {3, 4, 7, 8, 10, 12, 13}
    assert np.any(a["phase13__u"] != a["phase3__u"])
