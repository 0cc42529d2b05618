// Host builders of the C ABI: the lattice schedule and the canonical state.
//
// buildSchedule restates buildLatticeSchedule (src/fastlattice/LatticeSchedule.cpp:71-155):
// a greedy edge colouring in asset bond order (lowest colour free at both
// ends, at most 64), slab ownership by the lower slab, and the permutation
// that groups bonds by (owner, boundary, colour) keeping asset order inside a
// group. The colouring is sequential by definition and is integer work, so it
// runs here, once per topology, and must match the reference bit for bit.
//
// buildState restates buildLatticeState (src/fastlattice/FastLattice.cpp:47-169).
// gbl_build_box and gbl_impact_settings are scene-side helpers (the box
// generator's walk; the impact scene's step settings).
#include "gbl_internal.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <mutex>

namespace gbl {

namespace {
thread_local std::string g_last_error;
}

void setLastError(const std::string &m) { g_last_error = m; }

Schedule Schedule::fromView(const gbl_schedule_view &v) {
    Schedule s;
    s.node_count = v.node_count;
    s.bond_count = v.bond_count;
    s.block_count = v.block_count;
    s.color_count = v.color_count;
    s.boundary_bond_count = v.boundary_bond_count;
    if (s.block_count == 0) invalid("lattice schedule needs at least one block");
    if (!v.node_block_begin || !v.range_begin || !v.range_end || !v.bond_block_begin ||
        (s.bond_count && (!v.bond_order || !v.bond_schedule_index || !v.bond_color)))
        invalid("lattice schedule view has null arrays");
    const std::size_t ranges = static_cast<std::size_t>(s.block_count) * 2 * std::max(s.color_count, 1U);
    s.node_block_begin.assign(v.node_block_begin, v.node_block_begin + s.block_count + 1);
    s.bond_block_begin.assign(v.bond_block_begin, v.bond_block_begin + s.block_count + 1);
    s.range_begin.assign(v.range_begin, v.range_begin + ranges);
    s.range_end.assign(v.range_end, v.range_end + ranges);
    if (s.bond_count) {
        s.bond_order.assign(v.bond_order, v.bond_order + s.bond_count);
        s.bond_schedule_index.assign(v.bond_schedule_index, v.bond_schedule_index + s.bond_count);
        s.bond_color.assign(v.bond_color, v.bond_color + s.bond_count);
    }
    if (s.node_block_begin.front() != 0 || s.node_block_begin.back() != s.node_count ||
        !std::is_sorted(s.node_block_begin.begin(), s.node_block_begin.end()))
        invalid("lattice schedule needs sorted node block offsets covering every node");
    for (std::size_t k = 0; k < ranges; ++k)
        if (s.range_begin[k] > s.range_end[k] || s.range_end[k] > s.bond_count)
            invalid("lattice schedule range exceeds the bonds");
    return s;
}

gbl_schedule_view Schedule::view() const {
    gbl_schedule_view v{};
    v.node_count = node_count;
    v.bond_count = bond_count;
    v.block_count = block_count;
    v.color_count = color_count;
    v.boundary_bond_count = boundary_bond_count;
    v.node_block_begin = node_block_begin.data();
    v.bond_order = bond_order.data();
    v.bond_schedule_index = bond_schedule_index.data();
    v.bond_block_begin = bond_block_begin.data();
    v.range_begin = range_begin.data();
    v.range_end = range_end.data();
    v.bond_color = bond_color.data();
    return v;
}

Schedule buildSchedule(std::uint32_t node_count, std::uint32_t bond_count, const std::uint32_t *a, const std::uint32_t *b,
                       const std::uint32_t *node_block_begin, std::uint32_t block_count) {
    if (block_count == 0 || !node_block_begin || (bond_count && (!a || !b)))
        invalid("lattice schedule needs sorted node block offsets covering every node");
    if (node_block_begin[0] != 0 || node_block_begin[block_count] != node_count ||
        !std::is_sorted(node_block_begin, node_block_begin + block_count + 1))
        invalid("lattice schedule needs sorted node block offsets covering every node");
    Schedule s;
    s.node_count = node_count;
    s.bond_count = bond_count;
    s.block_count = block_count;
    s.node_block_begin.assign(node_block_begin, node_block_begin + block_count + 1);

    std::vector<std::uint32_t> slab(node_count);
    for (std::uint32_t blk = 0; blk < block_count; ++blk)
        std::fill(slab.begin() + node_block_begin[blk], slab.begin() + node_block_begin[blk + 1], blk);

    // Greedy colouring; one 64-bit set of used colours per node.
    std::vector<std::uint64_t> taken(node_count, 0);
    std::vector<std::uint32_t> key(bond_count);
    std::vector<std::uint8_t> colour(bond_count);
    std::uint32_t colours = 0;
    for (std::uint32_t k = 0; k < bond_count; ++k) {
        const std::uint32_t na = a[k], nb = b[k];
        if (na >= node_count || nb >= node_count || na == nb) invalid("lattice bond joins invalid nodes");
        const std::uint64_t open = ~(taken[na] | taken[nb]);
        if (open == 0) runtime("lattice needs more than 64 bond colours");
        const unsigned c = static_cast<unsigned>(__builtin_ctzll(open));
        taken[na] |= 1ULL << c;
        taken[nb] |= 1ULL << c;
        colour[k] = static_cast<std::uint8_t>(c);
        colours = std::max(colours, c + 1);
        const std::uint32_t lo = std::min(slab[na], slab[nb]), hi = std::max(slab[na], slab[nb]);
        if (hi - lo > 1) invalid("slab decomposition needs slabs at least one neighbour horizon thick");
        const std::uint32_t boundary = hi != lo ? 1U : 0U;
        s.boundary_bond_count += boundary;
        key[k] = (lo * 2 + boundary) * 64 + c; // provisional: colours not known yet
    }
    s.color_count = colours;
    const std::uint32_t C = std::max(colours, 1U);
    const std::size_t ranges = static_cast<std::size_t>(block_count) * 2 * C;
    for (std::uint32_t k = 0; k < bond_count; ++k) key[k] = (key[k] / 64) * C + key[k] % 64;

    // Grouping with asset order kept inside a group: a counting sort by key.
    std::vector<std::uint32_t> first(ranges + 1, 0);
    for (std::uint32_t k = 0; k < bond_count; ++k) ++first[key[k] + 1];
    for (std::size_t q = 0; q < ranges; ++q) first[q + 1] += first[q];
    s.range_begin.assign(ranges, 0);
    s.range_end.assign(ranges, 0);
    for (std::size_t q = 0; q < ranges; ++q)
        if (first[q + 1] > first[q]) { s.range_begin[q] = first[q]; s.range_end[q] = first[q + 1]; }
    s.bond_order.resize(bond_count);
    {
        std::vector<std::uint32_t> fill(first.begin(), first.end() - 1);
        for (std::uint32_t k = 0; k < bond_count; ++k) s.bond_order[fill[key[k]]++] = k;
    }
    s.bond_schedule_index.resize(bond_count);
    s.bond_color.resize(bond_count);
    for (std::uint32_t q = 0; q < bond_count; ++q) {
        s.bond_schedule_index[s.bond_order[q]] = q;
        s.bond_color[q] = colour[s.bond_order[q]];
    }
    // Bond range of each owner slab; owners without bonds inherit the previous end.
    s.bond_block_begin.assign(block_count + 1, 0);
    for (std::uint32_t blk = 0; blk < block_count; ++blk) s.bond_block_begin[blk + 1] = first[(blk + 1) * 2 * C];
    return s;
}

gbl_state_view State::view() {
    gbl_state_view v{};
    std::memcpy(v.origin, origin, sizeof(origin));
    v.node_count = node_count;
    v.bond_count = bond_count;
    v.max_degree = max_degree;
    v.x0 = x0.data(); v.u = u.data(); v.u_prev = u_prev.data(); v.v = this->v.data();
    v.inv_mass = inv_mass.data(); v.mass = mass.data();
    v.adj_offsets = adj_offsets.data(); v.adj_bonds = adj_bonds.data();
    v.nbr_bond = nbr_bond.data(); v.nbr_other = nbr_other.data(); v.nbr_rest = nbr_rest.data();
    v.nbr_weight = nbr_weight.data(); v.nbr_alive = nbr_alive.data();
    v.bond_slot_a = bond_slot_a.data(); v.bond_slot_b = bond_slot_b.data();
    v.bond_a = bond_a.data(); v.bond_b = bond_b.data();
    v.rest_edge = rest_edge.data(); v.rest_length = rest_length.data();
    v.rest_length_sq_minus = rest_length_sq_minus.data(); v.weight = weight.data();
    v.compliance = compliance.data(); v.threshold = threshold.data();
    v.alive = alive.data(); v.failure_mode = failure_mode.data(); v.damage = damage.data();
    v.prev_tensile = prev_tensile.data(); v.prev_compressive = prev_compressive.data(); v.prev_shear = prev_shear.data();
    v.plastic_extension = plastic_extension.data(); v.plastic_strain = plastic_strain.data();
    return v;
}

State buildState(const gbl_matter_view &m, const Schedule &s, const double origin[3]) {
    const std::size_t N = m.node_count, B = m.bond_count;
    if (s.bond_order.size() != B || s.node_block_begin.back() != N)
        invalid("lattice schedule does not match the lattice");
    if (!m.reference_position || !m.position || !m.velocity || !m.mass ||
        (B && (!m.bond_a || !m.bond_b || !m.rest_length || !m.compliance || !m.threshold)))
        invalid("lattice state needs matching nodes, bonds and reference positions");
    State st;
    std::memcpy(st.origin, origin, sizeof(st.origin));
    st.node_count = m.node_count;
    st.bond_count = m.bond_count;
    st.x0.resize(3 * N); st.u.resize(3 * N); st.u_prev.resize(3 * N); st.v.resize(3 * N);
    st.inv_mass.resize(N); st.mass.resize(N);
    for (std::size_t i = 0; i < N; ++i) {
        for (int d = 0; d < 3; ++d) {
            const double ref = m.reference_position[3 * i + d];
            st.x0[3 * i + d] = ref - origin[d];
            st.u[3 * i + d] = m.position[3 * i + d] - ref;
            st.v[3 * i + d] = m.velocity[3 * i + d];
        }
        st.mass[i] = m.mass[i];
        st.inv_mass[i] = m.mass[i] > 0.0 ? 1.0 / m.mass[i] : 0.0;
    }
    st.u_prev = st.u;
    st.bond_a.resize(B); st.bond_b.resize(B); st.rest_edge.resize(3 * B); st.rest_length.resize(B);
    st.rest_length_sq_minus.resize(B); st.weight.resize(B); st.compliance.resize(B); st.threshold.resize(6 * B);
    st.alive.resize(B); st.failure_mode.resize(B); st.damage.resize(B);
    st.plastic_extension.assign(B, 0.0); st.plastic_strain.assign(B, 0.0);
    st.prev_tensile.assign(B, 0.0); st.prev_compressive.assign(B, 0.0); st.prev_shear.assign(B, 0.0);
    for (std::size_t q = 0; q < B; ++q) {
        const std::uint32_t o = s.bond_order[q];
        const std::uint32_t na = m.bond_a[o], nb = m.bond_b[o];
        if (na >= N || nb >= N) invalid("lattice bond joins invalid nodes");
        st.bond_a[q] = na;
        st.bond_b[q] = nb;
        double e[3];
        for (int d = 0; d < 3; ++d) e[d] = m.reference_position[3 * nb + d] - m.reference_position[3 * na + d];
        for (int d = 0; d < 3; ++d) st.rest_edge[3 * q + d] = e[d];
        const double rl = m.rest_length[o];
        st.rest_length[q] = rl;
        const double e2 = e[0] * e[0] + e[1] * e[1] + e[2] * e[2];
        st.rest_length_sq_minus[q] = e2 - rl * rl;
        st.weight[q] = e2 > 1.0e-18 ? 1.0 / e2 : 0.0;
        st.compliance[q] = m.compliance[o];
        for (int t = 0; t < 6; ++t) st.threshold[6 * q + t] = m.threshold[6 * static_cast<std::size_t>(o) + t];
        st.alive[q] = m.alive ? (m.alive[o] ? 1 : 0) : 1;
        st.failure_mode[q] = m.failure_mode ? m.failure_mode[o] : 0;
        st.damage[q] = m.damage ? m.damage[o] : 0.0;
    }
    // Adjacency in asset bond order (the CPU lane's summation order).
    std::vector<std::uint32_t> degree(N, 0);
    for (std::size_t o = 0; o < B; ++o) { ++degree[m.bond_a[o]]; ++degree[m.bond_b[o]]; }
    st.adj_offsets.assign(N + 1, 0);
    for (std::size_t i = 0; i < N; ++i) st.adj_offsets[i + 1] = st.adj_offsets[i] + degree[i];
    st.adj_bonds.resize(st.adj_offsets.back());
    {
        std::vector<std::uint32_t> cursor(st.adj_offsets.begin(), st.adj_offsets.end() - 1);
        for (std::size_t o = 0; o < B; ++o) {
            const std::uint32_t q = s.bond_schedule_index[o];
            st.adj_bonds[cursor[m.bond_a[o]]++] = q;
            st.adj_bonds[cursor[m.bond_b[o]]++] = q;
        }
    }
    std::uint32_t D = 0;
    for (std::size_t i = 0; i < N; ++i) D = std::max(D, degree[i]);
    st.max_degree = D;
    const std::size_t P = static_cast<std::size_t>(D) * N;
    st.nbr_bond.assign(P, GBL_NO_BOND); st.nbr_other.assign(P, 0); st.nbr_rest.assign(3 * P, 0.0);
    st.nbr_weight.assign(P, 0.0); st.nbr_alive.assign(P, 0);
    st.bond_slot_a.assign(B, 0); st.bond_slot_b.assign(B, 0);
    for (std::size_t i = 0; i < N; ++i)
        for (std::uint32_t k = 0; k < degree[i]; ++k) {
            const std::uint32_t q = st.adj_bonds[st.adj_offsets[i] + k];
            const std::size_t slot = static_cast<std::size_t>(k) * N + i;
            const bool is_a = st.bond_a[q] == i;
            st.nbr_bond[slot] = q;
            st.nbr_alive[slot] = st.alive[q];
            (is_a ? st.bond_slot_a : st.bond_slot_b)[q] = static_cast<std::uint32_t>(slot);
            st.nbr_other[slot] = is_a ? st.bond_b[q] : st.bond_a[q];
            const double sign = is_a ? 1.0 : -1.0;
            for (int d = 0; d < 3; ++d) st.nbr_rest[3 * slot + d] = sign * st.rest_edge[3 * q + d];
            st.nbr_weight[slot] = st.weight[q];
        }
    return st;
}

} // namespace gbl

extern "C" {

gbl_result gbl_last_error(char *buffer, size_t capacity) {
    if (!buffer || capacity == 0) return GBL_INVALID_ARGUMENT;
    const std::size_t n = std::min(capacity - 1, gbl::g_last_error.size());
    std::memcpy(buffer, gbl::g_last_error.data(), n);
    buffer[n] = '\0';
    return GBL_OK;
}

size_t gbl_struct_size(const char *name) {
    if (!name) return 0;
    const std::string n(name);
#define GBL_SIZE(T) if (n == #T) return sizeof(T);
    GBL_SIZE(gbl_schedule_view) GBL_SIZE(gbl_state_view) GBL_SIZE(gbl_footprint) GBL_SIZE(gbl_support_plane)
    GBL_SIZE(gbl_contact_settings) GBL_SIZE(gbl_node_contact_settings) GBL_SIZE(gbl_step_settings)
    GBL_SIZE(gbl_node_contact_accumulators) GBL_SIZE(gbl_tuning) GBL_SIZE(gbl_impact_scene)
    GBL_SIZE(gbl_sphere) GBL_SIZE(gbl_run_control) GBL_SIZE(gbl_contact_accumulators) GBL_SIZE(gbl_load_ledger)
    GBL_SIZE(gbl_run_status) GBL_SIZE(gbl_matter_view) GBL_SIZE(gbl_request_info) GBL_SIZE(gbl_server_stats)
    GBL_SIZE(gbl_box_spec) GBL_SIZE(gbl_external_wrench)
#undef GBL_SIZE
    return 0;
}

gbl_result gbl_build_schedule(uint32_t node_count, uint32_t bond_count, const uint32_t *bond_a, const uint32_t *bond_b,
                              const uint32_t *node_block_begin, uint32_t block_count, gbl_schedule **out) {
    return gbl::guard([&] {
        if (!out) gbl::invalid("null output");
        auto *s = new gbl_schedule{gbl::buildSchedule(node_count, bond_count, bond_a, bond_b, node_block_begin, block_count)};
        *out = s;
    });
}

gbl_result gbl_schedule_view_of(const gbl_schedule *schedule, gbl_schedule_view *view) {
    return gbl::guard([&] {
        if (!schedule || !view) gbl::invalid("null schedule");
        *view = schedule->s.view();
    });
}

void gbl_schedule_free(gbl_schedule *schedule) { delete schedule; }

gbl_result gbl_build_state(const gbl_matter_view *matter, const gbl_schedule *schedule, const double origin[3],
                           gbl_state **out) {
    return gbl::guard([&] {
        if (!matter || !schedule || !out) gbl::invalid("null argument");
        const double zero[3] = {0, 0, 0};
        *out = new gbl_state{gbl::buildState(*matter, schedule->s, origin ? origin : zero)};
    });
}

gbl_result gbl_state_view_of(gbl_state *state, gbl_state_view *view) {
    return gbl::guard([&] {
        if (!state || !view) gbl::invalid("null state");
        *view = state->s.view();
    });
}

gbl_result gbl_state_pin(gbl_state *state, const uint8_t *pinned) {
    return gbl::guard([&] {
        if (!state || !pinned) gbl::invalid("null argument");
        for (std::uint32_t i = 0; i < state->s.node_count; ++i)
            if (pinned[i]) state->s.inv_mass[i] = 0.0;
    });
}

void gbl_state_free(gbl_state *state) { delete state; }

} // extern "C"

// ---- Box lattices (the input generator of the reference's box scenes) ----

namespace gbl {

// generateBoxTileLattice's walk (src/matter/BoxLattice.cpp:117-155): nodes at
// cell centres, index x + nx*(y + ny*z) (BoxLattice.hpp:22-26, positions
// BoxLattice.cpp:82-86); for each node in index order, each integer offset of
// the positive half-space in dz, dy, dx order over [-h, h]
// (src/matter/Lattice.cpp:49-52) whose neighbour lies inside makes a bond
// (node, neighbour) of rest length spacing*|o|. The offset rule is the
// horizon |o| <= h, or |o|^2 <= max_offset_sq when that is set. Slabs:
// boxLatticeSlabs, BoxLattice.cpp:175-195.
struct Box {
    std::uint32_t node_count{}, bond_count{};
    std::vector<double> ref, pos, vel, mass, rest, compliance, threshold;
    std::vector<std::uint32_t> a, b, slabs;
};

Box buildBox(const gbl_box_spec &sp) {
    if (sp.nx == 0 || sp.ny == 0 || sp.nz == 0) invalid("box lattice needs at least one cell per axis");
    const std::uint64_t n64 = static_cast<std::uint64_t>(sp.nx) * sp.ny * sp.nz;
    if (n64 > kNodeLimit) invalid("box lattice exceeds 2^30 nodes");
    const int h = static_cast<int>(sp.horizon ? sp.horizon : 1);
    struct Offset { int dx, dy, dz, d2; };
    std::vector<Offset> offs;
    for (int dz = -h; dz <= h; ++dz)
        for (int dy = -h; dy <= h; ++dy)
            for (int dx = -h; dx <= h; ++dx) {
                if (!(dz > 0 || (dz == 0 && dy > 0) || (dz == 0 && dy == 0 && dx > 0))) continue;
                const int d2 = dx * dx + dy * dy + dz * dz;
                if (sp.max_offset_sq ? d2 > static_cast<int>(sp.max_offset_sq) : std::sqrt(double(d2)) > h + 1e-9) continue;
                offs.push_back({dx, dy, dz, d2});
            }
    Box bx;
    const std::uint32_t nx = sp.nx, ny = sp.ny, nz = sp.nz;
    const std::uint32_t n = static_cast<std::uint32_t>(n64);
    bx.node_count = n;
    bx.ref.resize(3 * static_cast<std::size_t>(n));
    for (std::uint32_t i = 0; i < n; ++i) {
        const std::uint32_t x = i % nx, y = (i / nx) % ny, z = i / (nx * ny);
        bx.ref[3 * i] = ((double(x) + 0.5) - 0.5 * nx) * sp.spacing + sp.center[0];
        bx.ref[3 * i + 1] = ((double(y) + 0.5) - 0.5 * ny) * sp.spacing + sp.center[1];
        bx.ref[3 * i + 2] = ((double(z) + 0.5) - 0.5 * nz) * sp.spacing + sp.center[2];
    }
    bx.pos = bx.ref;
    bx.vel.assign(bx.ref.size(), 0.0);
    bx.mass.assign(n, sp.node_mass);
    bx.a.reserve(static_cast<std::size_t>(n) * offs.size());
    bx.b.reserve(bx.a.capacity());
    std::vector<double> rest_of(offs.size());
    for (std::size_t k = 0; k < offs.size(); ++k) rest_of[k] = std::sqrt(double(offs[k].d2)) * sp.spacing;
    for (std::uint32_t i = 0; i < n; ++i) {
        const int x = static_cast<int>(i % nx), y = static_cast<int>((i / nx) % ny), z = static_cast<int>(i / (nx * ny));
        for (std::size_t k = 0; k < offs.size(); ++k) {
            const int X = x + offs[k].dx, Y = y + offs[k].dy, Z = z + offs[k].dz;
            if (X < 0 || Y < 0 || Z < 0 || X >= static_cast<int>(nx) || Y >= static_cast<int>(ny) ||
                Z >= static_cast<int>(nz))
                continue;
            bx.a.push_back(i);
            bx.b.push_back(static_cast<std::uint32_t>(X) + nx * (static_cast<std::uint32_t>(Y) + ny * Z));
            bx.rest.push_back(rest_of[k]);
        }
    }
    const std::size_t B = bx.a.size();
    if (B > 0xffffffffULL) invalid("box lattice has more than 2^32 - 1 bonds");
    bx.bond_count = static_cast<std::uint32_t>(B);
    bx.compliance.assign(B, sp.compliance);
    bx.threshold.resize(6 * B);
    for (std::size_t q = 0; q < B; ++q)
        for (int t = 0; t < 6; ++t) bx.threshold[6 * q + t] = sp.threshold[t];
    std::uint32_t blocks = std::max(1U, sp.slabs);
    blocks = std::min(blocks, std::max(1U, nz));
    const std::uint32_t layer = nx * ny;
    bx.slabs.resize(blocks + 1);
    for (std::uint32_t k = 0; k <= blocks; ++k)
        bx.slabs[k] = static_cast<std::uint32_t>((static_cast<std::uint64_t>(nz) * k / blocks) * layer);
    bx.slabs[blocks] = layer * nz;
    return bx;
}

} // namespace gbl

struct gbl_box {
    gbl::Box b;
};

extern "C" {

// buildSettings (TileImpactScene.cpp:259-336) with makePlane and addFootprint
// (:83-105): a horizontal plane's frame is normal +y, tangent +x, bitangent +z
// (makeSupportPlane, src/core/Plane.hpp:18-45, for that normal); a footprint
// with a finite half extent caps the plane's reach.
gbl_result gbl_impact_settings(const gbl_impact_scene *scene, gbl_step_settings *out) {
    return gbl::guard([&] {
        if (!scene || !out) gbl::invalid("null argument");
        const gbl_impact_scene &r = *scene;
        if (r.ledge_count > GBL_MAX_FOOTPRINTS) gbl::logic("too many support footprints");
        gbl_step_settings s{};
        s.dt = r.dt;
        for (int k = 0; k < 3; ++k) s.gravity[k] = r.gravity[k];
        s.constraint_iterations = std::max(1U, r.constraint_iterations);
        s.damping_fraction = r.bond_damping > 0.0 ? 1.0 - std::exp(-r.bond_damping * r.dt) : 0.0;
        s.sphere_enabled = r.multi_body ? 0 : 1;
        s.direct_arithmetic = r.double_precision ? 1 : 0;
        s.contact.static_friction = r.ball_tile.static_friction;
        s.contact.dynamic_friction = r.ball_tile.dynamic_friction;
        s.contact.restitution = r.ball_tile.restitution;
        s.contact.restitution_speed_threshold = 0.5;
        s.contact.node_contact_radius = r.node_contact_radius_factor * r.cell_size;
        s.contact.contact_margin = 1.0e-5;
        s.contact.prefilter_slack = 0.05 * r.ball_radius;
        s.audit_energy = r.audit_energy ? 1 : 0;
        s.plastic_yield_stretch = r.yield_stretch;
        s.plastic_hardening = r.plastic_hardening_ratio;
        s.plate_half_thickness = 0.0;
        s.node_contact.mode = r.node_contact_mode;
        s.node_contact.radius = r.node_contact_radius_factor * r.cell_size;
        s.node_contact.skin = r.node_contact_skin_factor * r.cell_size;
        s.node_contact.margin = 1.0e-5;
        s.node_contact.restitution = r.tile_tile.restitution;
        s.node_contact.restitution_speed_threshold = 0.5;
        s.node_contact.static_friction = r.tile_tile.static_friction;
        s.node_contact.dynamic_friction = r.tile_tile.dynamic_friction;
        std::uint32_t size = 64U; // latticeContactBucketMask (LatticePhysics.hpp:239-243)
        while (size < 2U * r.node_count && size < (1U << 22)) size <<= 1U;
        s.node_contact.bucket_mask = size - 1U;
        const double inf = std::numeric_limits<double>::infinity();
        const double node_radius = 0.5 * r.cell_size; // a cell centre rests half a cell above a surface
        auto plane = [&](double y) {
            gbl_support_plane p{};
            p.point[0] = 0.0 - r.origin[0];
            p.point[1] = y - r.origin[1];
            p.point[2] = 0.0 - r.origin[2];
            p.normal[1] = 1.0;
            p.tangent[0] = 1.0;
            p.bitangent[2] = 1.0;
            p.restitution = r.tile_ground.restitution;
            p.static_friction = r.tile_ground.static_friction;
            p.dynamic_friction = r.tile_ground.dynamic_friction;
            p.node_radius = node_radius;
            return p;
        };
        auto footprint = [](gbl_support_plane &p, double t, double b, double ht, double hb) {
            if (p.footprint_count >= GBL_MAX_FOOTPRINTS) gbl::logic("too many support footprints");
            p.footprints[p.footprint_count++] = {t, b, ht, hb};
            if (std::isfinite(ht) || std::isfinite(hb)) p.reach_capped = 1;
        };
        if (!r.bridge) {
            gbl_support_plane ground = plane(r.ground_y);
            footprint(ground, 0.0, 0.0, inf, inf);
            s.plane_count = 1;
            s.planes[0] = ground;
        } else {
            gbl_support_plane ledges = plane(r.support_y);
            for (std::uint32_t k = 0; k < r.ledge_count; ++k) {
                const gbl_ledge &l = r.ledges[k];
                footprint(ledges, l.center[0] - r.origin[0], l.center[2] - r.origin[2], 0.5 * l.dimensions[0],
                          0.5 * l.dimensions[2]);
            }
            gbl_support_plane ground = plane(r.ground_y);
            footprint(ground, 0.0, 0.0, inf, inf);
            s.plane_count = 2;
            s.planes[0] = ledges;
            s.planes[1] = ground;
        }
        *out = s;
    });
}

gbl_result gbl_build_box(const gbl_box_spec *spec, gbl_box **out) {
    return gbl::guard([&] {
        if (!spec || !out) gbl::invalid("null argument");
        *out = new gbl_box{gbl::buildBox(*spec)};
    });
}

gbl_result gbl_box_view_of(const gbl_box *box, gbl_matter_view *matter, const uint32_t **node_block_begin,
                           uint32_t *block_count) {
    return gbl::guard([&] {
        if (!box || !matter) gbl::invalid("null argument");
        const gbl::Box &b = box->b;
        gbl_matter_view m{};
        m.node_count = b.node_count;
        m.bond_count = b.bond_count;
        m.reference_position = b.ref.data();
        m.position = b.pos.data();
        m.velocity = b.vel.data();
        m.mass = b.mass.data();
        m.bond_a = b.a.data();
        m.bond_b = b.b.data();
        m.rest_length = b.rest.data();
        m.compliance = b.compliance.data();
        m.threshold = b.threshold.data();
        *matter = m;
        if (node_block_begin) *node_block_begin = b.slabs.data();
        if (block_count) *block_count = static_cast<uint32_t>(b.slabs.size() - 1);
    });
}

void gbl_box_free(gbl_box *box) { delete box; }

} // extern "C"
