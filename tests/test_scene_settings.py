"""The impact scene's step settings builder (gbl_impact_settings), checked
rule by rule against buildSettings (src/fastlattice/TileImpactScene.cpp:259-336)
and makePlane/addFootprint (:83-105). The reference builds these from a scene
that needs its physics engine, so the rules are held here one by one."""
import math

import pytest


def _scene(lattice, **kw):
    s = lattice.ImpactScene()
    s.dt = 1.0 / 2400.0
    s.gravity[:] = (0.0, -9.81, 0.0)
    s.constraint_iterations = 4
    s.ball_tile = lattice.ContactPair(0.3, 0.25, 0.4)
    s.tile_tile = lattice.ContactPair(0.6, 0.5, 0.1)
    s.tile_ground = lattice.ContactPair(0.7, 0.6, 0.2)
    s.cell_size = 0.01
    s.node_contact_radius_factor = 0.5
    s.node_contact_skin_factor = 0.25
    s.node_contact_mode = 2
    s.ball_radius = 0.2
    s.yield_stretch = 1.2e-3
    s.plastic_hardening_ratio = 0.05
    s.ground_y = -0.3
    s.support_y = 0.1
    s.origin[:] = (0.5, 0.2, -0.1)
    s.node_count = 3000
    for k, v in kw.items():
        setattr(s, k, v)
    return s


def test_flat_scene_settings():
    from banjo_gb300 import lattice

    sc = _scene(lattice, bond_damping=30.0)
    s = lattice.impact_settings(sc)
    assert s.dt == sc.dt and tuple(s.gravity) == (0.0, -9.81, 0.0) and s.constraint_iterations == 4
    assert s.damping_fraction == 1.0 - math.exp(-30.0 * sc.dt)
    assert s.sphere_enabled == 1 and s.direct_arithmetic == 0 and s.plate_half_thickness == 0.0
    c = s.contact
    assert (c.static_friction, c.dynamic_friction, c.restitution) == (0.3, 0.25, 0.4)
    assert c.restitution_speed_threshold == 0.5 and c.contact_margin == 1e-5
    assert c.node_contact_radius == 0.5 * 0.01 and c.prefilter_slack == 0.05 * 0.2
    n = s.node_contact
    assert n.mode == 2 and n.radius == 0.5 * 0.01 and n.skin == 0.25 * 0.01 and n.margin == 1e-5
    assert (n.static_friction, n.dynamic_friction, n.restitution) == (0.6, 0.5, 0.1)
    assert n.bucket_mask == 8191  # smallest power of two >= 2 x 3000, minus one
    assert (s.plastic_yield_stretch, s.plastic_hardening) == (1.2e-3, 0.05)
    assert s.plane_count == 1
    g = s.planes[0]
    assert tuple(g.point) == (0.0 - 0.5, -0.3 - 0.2, 0.0 + 0.1)
    assert tuple(g.normal) == (0.0, 1.0, 0.0) and tuple(g.tangent) == (1.0, 0.0, 0.0)
    assert tuple(g.bitangent) == (0.0, 0.0, 1.0)
    assert (g.static_friction, g.dynamic_friction, g.restitution) == (0.7, 0.6, 0.2)
    assert g.node_radius == 0.005 and g.footprint_count == 1 and g.reach_capped == 0
    assert math.isinf(g.footprints[0].half_t) and math.isinf(g.footprints[0].half_b)


def test_bridge_scene_settings():
    from banjo_gb300 import lattice

    sc = _scene(lattice, bridge=1, multi_body=1, double_precision=1, constraint_iterations=0, ledge_count=2)
    sc.ledges[0] = lattice.Ledge((-0.3, 0.05, 0.0), (0.2, 0.1, 0.4))
    sc.ledges[1] = lattice.Ledge((0.3, 0.05, 0.1), (0.2, 0.1, 0.6))
    s = lattice.impact_settings(sc)
    assert s.constraint_iterations == 1 and s.sphere_enabled == 0 and s.direct_arithmetic == 1
    assert s.damping_fraction == 0.0 and s.plane_count == 2
    ledges, ground = s.planes[0], s.planes[1]
    assert tuple(ledges.point) == (-0.5, 0.1 - 0.2, 0.1) and ledges.reach_capped == 1
    assert ledges.footprint_count == 2
    f0, f1 = ledges.footprints[0], ledges.footprints[1]
    assert (f0.center_t, f0.center_b, f0.half_t, f0.half_b) == (-0.3 - 0.5, 0.0 + 0.1, 0.1, 0.2)
    assert (f1.center_t, f1.center_b, f1.half_t, f1.half_b) == (0.3 - 0.5, 0.1 + 0.1, 0.1, 0.3)
    assert tuple(ground.point) == (-0.5, -0.5, 0.1) and ground.reach_capped == 0 and ground.footprint_count == 1


def test_too_many_ledges_refused():
    from banjo_gb300 import lattice

    sc = _scene(lattice, bridge=1, ledge_count=5)
    with pytest.raises(Exception, match="footprints"):
        lattice.impact_settings(sc)
