"""Synthetic lattice workloads for the bonded-lattice substep.

Each builder returns a *case*: a dict of numpy arrays named as the lattice case
files name them (node/bond arrays of a LatticeAsset + ActiveMatter, packed
StepSettings<double> and SphereState<double>, the run length). The same dict
feeds the GPU backend, the CPU checker and the reference harness, so all three
see identical inputs.

Bonds follow the reference's box generator walk (src/matter/BoxLattice.cpp:117-155:
node index order, offsets dz, dy, dx over [-h, h] in the positive half-space,
src/matter/Lattice.cpp:49-52) filtered to the 6 face + 12 edge neighbours
(|o|^2 <= 2), so an interior node has 9 unique bonds. Node index is
x + nx*(y + ny*z) (src/matter/BoxLattice.hpp:22-26). Positions are cell
centres of a box centred on its own origin (BoxLattice.cpp:82-86).

Seeds are counter-based splitmix64 streams (the mixing function of
src/matter/Lattice.cpp:28-33): draw k of stream s is mix(s + (k+1)*golden).
"""
from __future__ import annotations

import math

import numpy as np

# Settings packing (oracle/case_layout.hpp, the one order every runner uses).
K_DT, K_GRAVITY, K_ITER, K_DAMP, K_SPHERE, K_DIRECT = 0, 1, 4, 5, 6, 7
K_YIELD, K_HARDEN, K_PLATE, K_CONTACT, K_PLANE_COUNT, K_PLANES = 8, 9, 10, 11, 18, 19
PLANE_WIDTH = 34
K_NODE_CONTACT = 19 + 2 * PLANE_WIDTH  # 9 slots; a record that ends here has node contact off
K_AUDIT = K_NODE_CONTACT + 9  # StepSettings::audit_energy; a record that ends here has it off
SETTINGS_WIDTH = K_AUDIT + 1
SPHERE_WIDTH = 12

GOLDEN = np.uint64(0x9E3779B97F4A7C15)
DT_SUBSTEP = (1.0 / 240.0) / 10.0
INF = float("inf")


def splitmix64(values: np.ndarray) -> np.ndarray:
    """The splitmix64 output mix on uint64 values (wrapping arithmetic), in place
    on a copy so that tens of millions of draws stay cheap."""
    z = np.array(values, dtype=np.uint64, copy=True)
    t = np.empty_like(z)
    with np.errstate(over="ignore"):
        for shift, mult in ((30, 0xBF58476D1CE4E5B9), (27, 0x94D049BB133111EB)):
            np.right_shift(z, np.uint64(shift), out=t)
            np.bitwise_xor(z, t, out=z)
            np.multiply(z, np.uint64(mult), out=z)
        np.right_shift(z, np.uint64(31), out=t)
        np.bitwise_xor(z, t, out=z)
    return z


def uniform(seed: int, start: int, count: int) -> np.ndarray:
    """Draws start..start+count-1 of stream `seed`, uniform in [0, 1)."""
    state = np.arange(start + 1, start + count + 1, dtype=np.uint64)
    with np.errstate(over="ignore"):
        np.multiply(state, GOLDEN, out=state)
        np.add(state, np.uint64(seed), out=state)
    z = splitmix64(state)
    np.right_shift(z, np.uint64(11), out=z)
    out = z.astype(np.float64)
    out *= 1.0 / 9007199254740992.0
    return out


def lognormal(seed: int, count: int, median: float, sigma: float) -> np.ndarray:
    """Box-Muller normals from draw pairs (2k, 2k+1) of the stream."""
    u = uniform(seed, 0, 2 * count)
    u1 = 1.0 - u[0::2]  # (0, 1]
    np.log(u1, out=u1)
    u1 *= -2.0
    np.sqrt(u1, out=u1)
    u2 = u[1::2] * (2.0 * math.pi)
    np.cos(u2, out=u2)
    u1 *= u2
    u1 *= sigma
    np.exp(u1, out=u1)
    u1 *= median
    return u1


def half_offsets(horizon: int = 1, max_d2: int | None = 2):
    """Positive-half integer offsets in the generator's walk order.

    With max_d2 set, the walk over [-horizon, horizon]^3 keeps |o|^2 <= max_d2
    (horizon 1, max_d2 2: the 6 face + 12 edge neighbours, 9 per node); with
    max_d2 None it is the reference's own horizon rule |o| <= horizon
    (src/matter/BoxLattice.cpp:123-129).
    """
    out = []
    for dz in range(-horizon, horizon + 1):
        for dy in range(-horizon, horizon + 1):
            for dx in range(-horizon, horizon + 1):
                if not (dz > 0 or (dz == 0 and dy > 0) or (dz == 0 and dy == 0 and dx > 0)):
                    continue
                d2 = dx * dx + dy * dy + dz * dz
                if max_d2 is not None:
                    if d2 > max_d2:
                        continue
                elif math.sqrt(d2) > horizon + 1e-9:
                    continue
                out.append((dx, dy, dz, d2))
    return out


def box_nodes(nx: int, ny: int, nz: int, h: float, center=(0.0, 0.0, 0.0)) -> np.ndarray:
    """Cell-centre positions (3N float64), node index x + nx*(y + ny*z)."""
    idx = np.arange(nx * ny * nz, dtype=np.int64)
    x = idx % nx
    y = (idx // nx) % ny
    z = idx // (nx * ny)
    pos = np.empty((idx.size, 3), dtype=np.float64)
    pos[:, 0] = (x.astype(np.float64) + 0.5 - 0.5 * nx) * h + center[0]
    pos[:, 1] = (y.astype(np.float64) + 0.5 - 0.5 * ny) * h + center[1]
    pos[:, 2] = (z.astype(np.float64) + 0.5 - 0.5 * nz) * h + center[2]
    return pos.reshape(-1)


def box_bonds(nx: int, ny: int, nz: int, max_d2: int | None = 2, horizon: int = 1):
    """Bond endpoints and grid distance^2, in the reference generator's order."""
    n = nx * ny * nz
    offs = half_offsets(horizon, max_d2)
    K = len(offs)
    idx3 = np.arange(n, dtype=np.int64).reshape(nz, ny, nx)
    other = np.full((nz, ny, nx, K), -1, dtype=np.int64)

    def span(d, size):  # source range whose neighbour at offset d is inside
        return slice(max(0, -d), min(size, size - d))

    for k, (dx, dy, dz, _) in enumerate(offs):
        sz, sy, sx = span(dz, nz), span(dy, ny), span(dx, nx)
        other[sz, sy, sx, k] = idx3[sz, sy, sx] + (dx + nx * (dy + ny * dz))
    flat = other.reshape(-1)
    mask = flat >= 0
    a = (np.nonzero(mask)[0] // K).astype(np.uint32)
    b = flat[mask].astype(np.uint32)
    d2 = np.tile(np.asarray([o[3] for o in offs], dtype=np.int8), n)[mask]
    return a, b, d2


def slabs(nx: int, ny: int, nz: int, requested: int, layers_per_block: int = 1) -> np.ndarray:
    """Node offsets of at most `requested` z-slabs (src/matter/BoxLattice.cpp:175-195)."""
    blocks = max(1, requested)
    blocks = min(blocks, max(1, nz // layers_per_block))
    layer = nx * ny
    begin = [(nz * b // blocks) * layer for b in range(blocks + 1)]
    begin[-1] = layer * nz
    return np.asarray(begin, dtype=np.uint32)


def plane(point, normal=(0.0, 1.0, 0.0), tangent=(1.0, 0.0, 0.0), bitangent=(0.0, 0.0, 1.0),
          restitution=0.0, static_friction=0.5, dynamic_friction=0.4, node_radius=0.005,
          footprints=((0.0, 0.0, INF, INF),)) -> np.ndarray:
    """A support plane packed as the settings record holds it."""
    p = np.zeros(PLANE_WIDTH, dtype=np.float64)
    p[0:3], p[3:6], p[6:9], p[9:12] = point, normal, tangent, bitangent
    p[12], p[13], p[14], p[15] = restitution, static_friction, dynamic_friction, node_radius
    capped = any(math.isfinite(f[2]) or math.isfinite(f[3]) for f in footprints)
    p[16] = 1.0 if capped else 0.0
    p[17] = len(footprints)
    for k, f in enumerate(footprints):
        p[18 + 4 * k: 22 + 4 * k] = f
    return p


def contact_bucket_mask(node_count: int) -> int:
    """The hash table size rule of latticeContactBucketMask (LatticePhysics.hpp:239-243):
    the smallest power of two >= 2 N, at least 64 and at most 2^22, minus one."""
    size = 64
    while size < 2 * node_count and size < (1 << 22):
        size <<= 1
    return size - 1


def node_contact(mode=2, radius=0.005, skin=0.0025, margin=1e-5, restitution=0.0, threshold=0.5,
                 static_friction=0.5, dynamic_friction=0.4, node_count=0) -> tuple:
    """NodeContactSettings (LatticePhysics.hpp:188-202) as the packed record's
    9 slots: mode (0 off, 1 measure, 2 on), contact radius, Verlet skin, margin,
    restitution and its speed threshold, static and dynamic friction, and the
    hash mask for `node_count` nodes."""
    return (mode, radius, skin, margin, restitution, threshold, static_friction, dynamic_friction,
            contact_bucket_mask(node_count))


def settings(dt=DT_SUBSTEP, gravity=(0.0, -9.81, 0.0), iterations=4, damping_fraction=0.0, sphere_enabled=0,
             direct=0, yield_stretch=0.0, hardening=0.0, contact=(0.5, 0.4, 0.0, 0.5, 0.005, 1e-5, 0.01),
             planes=(), node_contact=None, audit_energy=False) -> np.ndarray:
    s = np.zeros(SETTINGS_WIDTH, dtype=np.float64)
    s[K_AUDIT] = 1.0 if audit_energy else 0.0
    if node_contact is not None:
        s[K_NODE_CONTACT:K_NODE_CONTACT + 9] = node_contact
    s[K_DT] = dt
    s[K_GRAVITY:K_GRAVITY + 3] = gravity
    s[K_ITER] = iterations
    s[K_DAMP] = damping_fraction
    s[K_SPHERE] = sphere_enabled
    s[K_DIRECT] = direct
    s[K_YIELD] = yield_stretch
    s[K_HARDEN] = hardening
    s[K_CONTACT:K_CONTACT + 7] = contact
    s[K_PLANE_COUNT] = len(planes)
    for k, p in enumerate(planes):
        s[K_PLANES + PLANE_WIDTH * k: K_PLANES + PLANE_WIDTH * (k + 1)] = p
    return s


def sphere(center=(0.0, 0.0, 0.0), velocity=(0.0, 0.0, 0.0), radius=0.0, density=7870.0) -> np.ndarray:
    s = np.zeros(SPHERE_WIDTH, dtype=np.float64)
    s[0:3] = center
    s[3:6] = velocity
    if radius > 0.0:
        mass = density * 4.0 / 3.0 * math.pi * radius ** 3
        s[9], s[10], s[11] = radius, mass, 0.4 * mass * radius * radius
    return s


def _box_case(nx, ny, nz, h, center, compliance, thresholds, mass=1e-3, blocks=1, max_d2=2):
    a, b, d2 = box_bonds(nx, ny, nz, max_d2=max_d2, horizon=1)
    ref = box_nodes(nx, ny, nz, h, center)
    n = nx * ny * nz
    nb = a.size
    thr = np.empty((nb, 6), dtype=np.float64)
    thr[:] = thresholds if np.ndim(thresholds) == 1 else 0.0
    if np.ndim(thresholds) == 2:
        thr[:] = thresholds
    comp = np.broadcast_to(np.asarray(compliance, dtype=np.float64), (nb,)).copy()
    return {
        "node_count": np.array([n], dtype=np.uint32),
        "bond_count": np.array([nb], dtype=np.uint32),
        "ref_pos": ref,
        "pos": ref.copy(),
        "vel": np.zeros(3 * n, dtype=np.float64),
        "mass": np.full(n, mass, dtype=np.float64),
        "bond_a": a,
        "bond_b": b,
        "rest_length": np.sqrt(d2.astype(np.float64)) * h,
        "compliance": comp,
        "threshold": thr.reshape(-1),
        "node_block_begin": slabs(nx, ny, nz, blocks),
        "origin": np.zeros(3, dtype=np.float64),
        "sphere": sphere(),
    }


def cantilever(nx=32, ny=8, nz=8, h=0.01, steps=240, substeps=10):
    """A cantilever beam, x=0 face pinned, gravity as an external load.

    Compliance 1e-7 on every bond, tensile damage start = end = 2e-3 (a step),
    compression and shear disabled (+inf). The pin is the XPBD lane's own way to
    hold a node: inv_mass 0 with its mass kept; gravity then cannot be a global
    StepSettings acceleration (it would move the pinned face), so it is applied
    to every movable node as setExternalForces(m*g) for the whole run.
    """
    case = _box_case(nx, ny, nz, h, (0.0, 0.0, 0.0), 1e-7, [2e-3, 2e-3, INF, INF, INF, INF])
    n = nx * ny * nz
    x = np.arange(n) % nx
    pinned = (x == 0).astype(np.uint8)
    forces = np.zeros((n, 3), dtype=np.float64)
    forces[pinned == 0, 1] = 1e-3 * -9.81
    case.update({
        "pinned": pinned,
        "forces": forces.reshape(-1),
        "force_substeps": np.array([steps * substeps], dtype=np.uint64),
        "settings": settings(gravity=(0.0, 0.0, 0.0)),
        "steps": np.array([steps * substeps], dtype=np.uint64),
        "substeps_per_step": np.array([substeps], dtype=np.uint64),
    })
    return case


def impact_block(nx=256, ny=128, nz=128, h=0.01, blocks=32, steps=120, substeps=10, seed_point=2,
                 seed_strength=20, median=1.5e-3, sigma=0.3, yield_fraction=0.6, radius=0.2, speed=10.0,
                 gap=0.002):
    """A block on an infinite ground plane struck by a rigid iron sphere.

    Per-bond break strain lognormal (median, sigma) as tensile start = end,
    compression and shear disabled, plastic yield stretch = yield_fraction x
    median (StepSettings carries one yield per lattice), hardening 0. The
    sphere starts `gap` above the top face over a point drawn uniformly from the
    inner half of the top face.
    """
    nb_est = None  # noqa: F841 (documentation: B is known only after the walk)
    case = _box_case(nx, ny, nz, h, (0.0, 0.0, 0.0), 1e-7, [INF] * 6, blocks=blocks)
    nb = int(case["bond_count"][0])
    strength = lognormal(seed_strength, nb, median, sigma)
    thr = np.full((nb, 6), INF, dtype=np.float64)
    thr[:, 0] = strength
    thr[:, 1] = strength
    case["threshold"] = thr.reshape(-1)
    top = (ny - 1 + 0.5 - 0.5 * ny) * h + 0.5 * h
    bottom = (0.5 - 0.5 * ny) * h - 0.5 * h
    p = uniform(seed_point, 0, 2)
    cx = (p[0] - 0.5) * 0.5 * nx * h
    cz = (p[1] - 0.5) * 0.5 * nz * h
    case.update({
        "settings": settings(sphere_enabled=1, yield_stretch=yield_fraction * median,
                             contact=(0.5, 0.4, 0.0, 0.5, 0.5 * h, 1e-5, 0.05 * radius),
                             planes=[plane((0.0, bottom, 0.0), node_radius=0.5 * h)]),
        "sphere": sphere((cx, top + gap + radius, cz), (0.0, -speed, 0.0), radius),
        "steps": np.array([steps * substeps], dtype=np.uint64),
        "substeps_per_step": np.array([substeps], dtype=np.uint64),
    })
    return case


def plate_strike(nx=24, nz=24, h=0.01, steps=40, radius=0.03, speed=8.0, median=2e-3, sigma=0.2, seed_strength=7,
                 yield_fraction=0.0, span=0.5, plate=True, gap=0.001):
    """A sheet one cell thick (nx x 1 x nz) resting on two ledges at its x
    ends (finite footprints, `span` of its length clear between them), struck
    at the centre by a rigid sphere, with plate bending on (half the cell as
    the half thickness): the fibre strain of the bending sheet is what breaks
    its bonds. Per-bond tensile break strain lognormal (median, sigma);
    compression and shear disabled."""
    case = _box_case(nx, 1, nz, h, (0.0, 0.0, 0.0), 1e-7, [INF] * 6)
    nb = int(case["bond_count"][0])
    strength = lognormal(seed_strength, nb, median, sigma)
    thr = np.full((nb, 6), INF, dtype=np.float64)
    thr[:, 0] = strength
    thr[:, 1] = strength
    case["threshold"] = thr.reshape(-1)
    length = nx * h
    ledge = 0.5 * (1.0 - span) * length  # each ledge's width under the sheet
    centre = 0.5 * length - 0.5 * ledge
    ledges = plane((0.0, -0.5 * h, 0.0), node_radius=0.5 * h,
                   footprints=((-centre, 0.0, 0.5 * ledge, INF), (centre, 0.0, 0.5 * ledge, INF)))
    s = settings(sphere_enabled=1, yield_stretch=yield_fraction * median,
                 contact=(0.5, 0.4, 0.0, 0.5, 0.5 * h, 1e-5, 0.05 * radius), planes=[ledges])
    if plate:
        s[K_PLATE] = 0.5 * h
    case.update({
        "settings": s,
        "sphere": sphere((0.0, 0.5 * h + gap + radius, 0.0), (0.0, -speed, 0.0), radius),
        "steps": np.array([steps], dtype=np.uint64),
    })
    return case


def wrenches(case: dict, regions, substeps: int) -> dict:
    """Adds external wrenches to a case (LatticeBackend::setExternalWrenches,
    FastLattice.hpp:153-157, 278-288): `regions` holds (source name, node
    indices, point, force, torque) per wrench, applied for `substeps`."""
    names = bytearray()
    counts, nodes, vectors = [], [], []
    for source, idx, point, force, torque in regions:
        names += source.encode() + b"\0"
        idx = np.asarray(idx, dtype=np.uint32)
        counts.append(idx.size)
        nodes.append(idx)
        vectors.append(np.concatenate([np.asarray(point, float), np.asarray(force, float), np.asarray(torque, float)]))
    case = dict(case)
    case["wrench_names"] = np.frombuffer(bytes(names), dtype=np.uint8).copy()
    case["wrench_node_count"] = np.asarray(counts, dtype=np.uint32)
    case["wrench_nodes"] = np.concatenate(nodes) if nodes else np.zeros(0, np.uint32)
    case["wrench_vectors"] = np.concatenate(vectors) if vectors else np.zeros(0)
    case["wrench_substeps"] = np.array([substeps], dtype=np.uint64)
    return case


def wrenched_bar(nx=16, ny=6, nz=6, h=0.01, steps=40, grip=(0.0, -4.0, 0.0), twist=(0.04, 0.0, 0.0),
                 hand=(0.0, 0.0, 2.5)):
    """A bar pinned at its x=0 face, no gravity, driven by two named wrenches:
    "grip" on the free end face (a force and a twist about the bar's axis,
    applied at the face's centre) and "hand" (a sideways push on the top row
    at mid-length, no torque). Compliance 1e-7, tensile step at 2e-3. The
    caller's node lists are given unsorted, as the reference sorts them."""
    case = _box_case(nx, ny, nz, h, (0.0, 0.0, 0.0), 1e-7, [2e-3, 2e-3, INF, INF, INF, INF])
    n = nx * ny * nz
    i = np.arange(n)
    x, y = i % nx, (i // nx) % ny
    pos = case["ref_pos"].reshape(-1, 3)
    end = np.flatnonzero(x == nx - 1)[::-1]
    top = np.flatnonzero((y == ny - 1) & (np.abs(x - (nx - 1) / 2.0) < 1.0))
    case.update({
        "pinned": (x == 0).astype(np.uint8),
        "settings": settings(gravity=(0.0, 0.0, 0.0)),
        "steps": np.array([steps], dtype=np.uint64),
        "substeps_per_step": np.array([1], dtype=np.uint64),
    })
    return wrenches(case, [("hand", top, pos[top].mean(axis=0), hand, (0.0, 0.0, 0.0)),
                           ("grip", end, pos[end].mean(axis=0), grip, twist)], steps)


def drop_trial(nx, ny, nz, compliance, break_strain, drop_height, h=0.01, steps=240, substeps=10):
    """One batched trial: a box released at rest `drop_height` above the ground."""
    case = _box_case(nx, ny, nz, h, (0.0, 0.0, 0.0), compliance, [break_strain, break_strain, INF, INF, INF, INF])
    lift = drop_height + 0.5 * ny * h
    ref = case["ref_pos"].reshape(-1, 3).copy()
    ref[:, 1] += lift
    case["ref_pos"] = ref.reshape(-1)
    case["pos"] = case["ref_pos"].copy()
    case.update({
        "settings": settings(planes=[plane((0.0, 0.0, 0.0), node_radius=0.5 * h)]),
        "steps": np.array([steps * substeps], dtype=np.uint64),
        "substeps_per_step": np.array([substeps], dtype=np.uint64),
    })
    return case


def two_cells(separation, bonded=False, mode=2, v0=0.0, v1=0.0, mass_ratio=1.0, dead=False, cell=0.01,
              steps=2000, density=2500.0):
    """Two cells on the x axis, `separation` apart, closing (or not) at v0 and
    v1, in the double lane with node-to-node contact: the pair the reference's
    contact tests step (fast_lattice_tests.cpp:690-896). Contact radius half a
    cell (two cells touch one cell apart), skin a quarter cell, dt 1e-6 s, one
    iteration, no gravity. `bonded` joins them by a bond at rest at
    `separation` whose thresholds are out of reach; `dead` starts that bond
    failed. Node 1 is `mass_ratio` times heavier."""
    ref = np.array([-0.5 * separation, 0.0, 0.0, 0.5 * separation, 0.0, 0.0])
    mass = density * cell ** 3
    nb = 1 if bonded else 0
    case = {
        "node_count": np.array([2], dtype=np.uint32),
        "bond_count": np.array([nb], dtype=np.uint32),
        "ref_pos": ref,
        "pos": ref.copy(),
        "vel": np.array([v0, 0.0, 0.0, v1, 0.0, 0.0]),
        "mass": np.array([mass, mass * mass_ratio]),
        "bond_a": np.zeros(nb, dtype=np.uint32),
        "bond_b": np.ones(nb, dtype=np.uint32),
        "rest_length": np.full(nb, float(separation)),
        "compliance": np.full(nb, 1e-7),
        "threshold": np.tile([1.0, 2.0, 1.0, 2.0, 1.0, 2.0], nb).astype(np.float64),
        "node_block_begin": np.array([0, 2], dtype=np.uint32),
        "origin": np.zeros(3, dtype=np.float64),
        "sphere": sphere(radius=1.0),
        "settings": settings(dt=1e-6, gravity=(0.0, 0.0, 0.0), iterations=1, direct=1,
                             node_contact=node_contact(mode, 0.5 * cell, 0.25 * cell, node_count=2)),
        "steps": np.array([steps], dtype=np.uint64),
    }
    if bonded and dead:
        case["alive"] = np.zeros(1, dtype=np.uint8)
    return case


def contact_drop(nx=10, ny=6, nz=8, compliance=1e-6, break_strain=1.5e-3, drop_height=0.002, speed=3.0, h=0.01,
                 steps=30, mode=2, restitution=0.2):
    """A box thrown onto the ground at `speed` hard enough to break bonds, with
    node-to-node contact on: every failed bond puts its pair in the contact
    list, and the cracked faces meet again."""
    case = drop_trial(nx, ny, nz, compliance=compliance, break_strain=break_strain, drop_height=drop_height, h=h,
                      steps=steps, substeps=1)
    n = nx * ny * nz
    vel = case["vel"].reshape(-1, 3)
    vel[:, 1] = -speed
    case["vel"] = vel.reshape(-1)
    case["settings"] = settings(planes=[plane((0.0, 0.0, 0.0), node_radius=0.5 * h)],
                                node_contact=node_contact(mode, 0.5 * h, 0.25 * h, restitution=restitution,
                                                          node_count=n))
    return case


def trial_parameters(count=4096, seed=3, edge_lo=8, edge_hi=48):
    """Per-trial draws: edges uniform on [lo, hi], compliance log-uniform on
    [1e-8, 1e-5], break strain uniform on [1e-3, 5e-3], drop height uniform on
    [0.1, 1] m. Six draws per trial from one stream."""
    u = uniform(seed, 0, 6 * count).reshape(count, 6)
    span = edge_hi - edge_lo + 1
    edges = (edge_lo + np.minimum((u[:, 0:3] * span).astype(np.int64), span - 1)).astype(np.int64)
    compliance = 10.0 ** (-8.0 + 3.0 * u[:, 3])
    strain = 1e-3 + 4e-3 * u[:, 4]
    height = 0.1 + 0.9 * u[:, 5]
    return edges, compliance, strain, height


# ---------------------------------------------------------------------------
# The notched bar: an energy-scaled brittle material with plastic flow.
# ---------------------------------------------------------------------------
# Material constants of the bar: density (kg/m^3), Young's modulus (Pa),
# Poisson ratio, tensile strength (Pa), yield strength (Pa), hardening ratio,
# fracture energy (J/m^2).
BAR_MATERIAL = (2500.0, 70.0e9, 0.22, 45.0e6, 36.0e6, 0.0, 8.0)


def compile_energy_scaled(material=BAR_MATERIAL, cell=0.01, horizon=2) -> dict:
    """The reference's material compile for the energy-scaled law with plastic
    flow, in FP64: withPlasticFlow(withEnergyScaledFailure(
    compileElasticLatticeReference(m, cell, horizon), m, cell, horizon), m)
    (src/material/MaterialCompiler.cpp:44-66, 68-108, 110-125, 127-214), with
    the default solver calibration (damage x1, break x2; src/material/Material.hpp:30-35)
    and no declared compressive or shear strength (disabled ramps)."""
    density, young, _nu, tensile, yield_, hardening, gc = material
    damage_mult, break_mult = 1.0, 2.0
    compliance = 1.0 / (young * (cell * cell) / (cell * float(horizon)))

    def failure_strain(strain, mult, minimum=1.0e-5):
        return INF if strain <= 0.0 else max(minimum, strain * mult)

    tensile_strain = tensile / young
    start = failure_strain(tensile_strain, damage_mult)
    strength_end = max(start * 1.01, failure_strain(tensile_strain, break_mult))
    crossings = 0.0
    for dz in range(-horizon, horizon + 1):
        for dy in range(-horizon, horizon + 1):
            for dx in range(-horizon, horizon + 1):
                if not (dz > 0 or (dz == 0 and dy > 0) or (dz == 0 and dy == 0 and dx > 0)):
                    continue
                if math.sqrt(float(dx * dx + dy * dy + dz * dz)) > float(horizon) + 1.0e-9:
                    continue
                crossings += abs(float(dx))
    energy = math.sqrt(2.0 * float(horizon) * gc / (crossings * young * cell))
    bounded = max(1.0e-5, min(energy, strength_end))
    fraction = min(max(damage_mult / break_mult, 0.0), 1.0)
    ds = max(1.0e-5, bounded * fraction)
    de = max(ds * 1.01, bounded)
    return {"bond_compliance": compliance, "damage_start": ds, "damage_end": de, "energy_scaled_stretch": energy,
            "strength_bound_active": strength_end < energy,
            "yield_stretch": yield_ / young if yield_ > 0.0 else 0.0,
            "hardening": hardening if yield_ > 0.0 else 0.0, "density": density}


def notched_bar(nx=128, ny=32, nz=32, h=0.01, horizon=2, material=BAR_MATERIAL, ramp_steps=10000, load_factor=2.0,
                steps=10000, substeps=10, blocks=1, notch=True):
    """A bar along x with a one-cell-wide slot at mid-length through the lower
    half of its depth (cells x = nx/2, y < ny/2, every z, removed before
    bonding). Bonds follow the box generator's horizon walk
    (src/matter/BoxLattice.cpp:117-155) between the cells present, node
    indices in x + nx*(y + ny*z) order with the slot cells skipped; per-bond
    compliance is bond_compliance / horizon weight, weight 1/max(1, |o|^2)
    (:139-142); thresholds are the compiled ones (strength variation 0); node
    mass is density * h^3. The x = 0 face is pinned; the x = nx-1 face carries
    tension along +x, ramped linearly from 0 to load_factor x (tensile
    strength x cross-section) over ramp_steps rigid steps, the load re-set
    every step for that step's substeps. No gravity.
    """
    comp = compile_energy_scaled(material, h, horizon)
    n_all = nx * ny * nz
    idx = np.arange(n_all, dtype=np.int64)
    gx, gy, gz = idx % nx, (idx // nx) % ny, idx // (nx * ny)
    keep = np.ones(n_all, dtype=bool)
    if notch:
        keep &= ~((gx == nx // 2) & (gy < ny // 2))
    new_index = np.full(n_all, -1, dtype=np.int64)
    new_index[keep] = np.arange(int(keep.sum()))
    n = int(keep.sum())
    offs = half_offsets(horizon, None)
    a_list, b_list, comp_list = [], [], []
    other = np.full((n_all, len(offs)), -1, dtype=np.int64)
    for k, (dx, dy, dz, _) in enumerate(offs):
        ox, oy, oz = gx + dx, gy + dy, gz + dz
        inside = (ox >= 0) & (oy >= 0) & (oz >= 0) & (ox < nx) & (oy < ny) & (oz < nz)
        o = np.where(inside, ox + nx * (oy + ny * oz), 0)
        ok = inside & keep & keep[o]
        other[ok, k] = new_index[o[ok]]
    mask = other >= 0
    src = np.nonzero(mask)
    a = new_index[src[0]].astype(np.uint32)
    b = other[mask].astype(np.uint32)
    d2 = np.asarray([o[3] for o in offs], dtype=np.float64)[src[1]]
    dist = np.sqrt(d2)
    rest = dist * h
    weight = 1.0 / np.maximum(1.0, dist * dist)
    compliance = comp["bond_compliance"] / weight
    nb = a.size
    thr = np.empty((nb, 6), dtype=np.float64)
    thr[:, 0], thr[:, 1] = comp["damage_start"], comp["damage_end"]
    thr[:, 2:] = INF
    ref = box_nodes(nx, ny, nz, h).reshape(-1, 3)[keep].reshape(-1)
    mass = comp["density"] * (h * h * h)
    kx = gx[keep]
    pinned = (kx == 0).astype(np.uint8)
    loaded = kx == nx - 1
    forces = np.zeros((n, 3), dtype=np.float64)
    forces[loaded, 0] = material[3] * (ny * h) * (nz * h) / float(loaded.sum())
    layer = nx * ny
    slab_begin = [int(keep[: (nz * k // blocks) * layer].sum()) for k in range(blocks + 1)]
    slab_begin[-1] = n
    s = settings(gravity=(0.0, 0.0, 0.0), yield_stretch=comp["yield_stretch"], hardening=comp["hardening"])
    return {
        "node_count": np.array([n], dtype=np.uint32),
        "bond_count": np.array([nb], dtype=np.uint32),
        "ref_pos": ref,
        "pos": ref.copy(),
        "vel": np.zeros(3 * n, dtype=np.float64),
        "mass": np.full(n, mass, dtype=np.float64),
        "bond_a": a,
        "bond_b": b,
        "rest_length": rest,
        "compliance": compliance,
        "threshold": thr.reshape(-1),
        "node_block_begin": np.asarray(slab_begin, dtype=np.uint32),
        "origin": np.zeros(3, dtype=np.float64),
        "sphere": sphere(),
        "pinned": pinned,
        "forces": forces.reshape(-1),
        "force_ramp_steps": np.array([ramp_steps], dtype=np.uint64),
        "force_ramp_scale": np.array([load_factor], dtype=np.float64),
        "settings": s,
        "steps": np.array([steps * substeps], dtype=np.uint64),
        "substeps_per_step": np.array([substeps], dtype=np.uint64),
    }
