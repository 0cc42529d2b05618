"""The bar material's compile against the reference's own compiler.

tests/golden/material_bar.npz holds what the reference's MaterialCompiler
(withPlasticFlow(withEnergyScaledFailure(compileElasticLatticeReference(...))))
returns for the bar material, written by tests/golden/make_golden.py; the
restatement that builds the notched-bar scene must give the same doubles.
"""
import os

import numpy as np

from banjo_gb300 import scenes

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "material_bar.npz")


def test_energy_scaled_compile_matches_reference():
    z = np.load(GOLDEN)
    m = z["material"]
    ref = z["compiled"]
    got = scenes.compile_energy_scaled(tuple(m[:7]), cell=float(m[7]), horizon=int(m[8]))
    # compliance, tensile start/end, compressive and shear ramps (disabled),
    # energy-scaled stretch, strength bound, yield stretch, hardening
    want = [got["bond_compliance"], got["damage_start"], got["damage_end"], np.inf, np.inf, np.inf, np.inf,
            got["energy_scaled_stretch"], 1.0 if got["strength_bound_active"] else 0.0, got["yield_stretch"],
            got["hardening"]]
    assert np.array_equal(np.asarray(want, dtype=np.float64).view(np.uint64), ref.view(np.uint64))


def test_notched_bar_counts():
    full = scenes.notched_bar(notch=False, steps=1)
    assert int(full["node_count"][0]) == 128 * 32 * 32 and int(full["bond_count"][0]) == 1996924
    bar = scenes.notched_bar(steps=1)
    assert int(bar["node_count"][0]) == 128 * 32 * 32 - 16 * 32
    # Interior nodes of a horizon-2 lattice carry 16 unique bonds.
    assert int(bar["bond_count"][0]) < 1996924
