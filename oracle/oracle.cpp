// CPU restatement of the reference's bonded-lattice XPBD fracture substep.
// TEST INFRASTRUCTURE ONLY -- see oracle.hpp. Every arithmetic expression keeps
// the reference's operand order and association (the reference's parity rule:
// no contraction, no reassociation), because the GPU path is held to it bit
// for bit and this file is the checker.
#include "oracle.hpp"

#include "case_layout.hpp"
#include "lsio.hpp"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <functional>
#include <limits>
#include <mutex>
#include <set>
#include <stdexcept>
#include <string>
#include <thread>
#include <type_traits>
#include <vector>

namespace orc {

constexpr std::uint32_t kNoBond = 0xffffffffU;
constexpr unsigned kPlanes = 2;
constexpr unsigned kFootprints = 4;
constexpr unsigned kCandidatesPerBlock = 1024;
constexpr std::uint64_t kNever = std::numeric_limits<std::uint64_t>::max();

// ---------------------------------------------------------------------------
// Vector algebra in the reference's expression order (LatticePhysics.hpp:39-98).
// ---------------------------------------------------------------------------
template <class R> struct V { R x, y, z; };
template <class R> V<R> add(V<R> a, V<R> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class R> V<R> sub(V<R> a, V<R> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class R> V<R> neg(V<R> a) { return {-a.x, -a.y, -a.z}; }
template <class R> V<R> scale(V<R> a, R s) { return {a.x * s, a.y * s, a.z * s}; }   // a * s and s * a
template <class R> V<R> divide(V<R> a, R s) { return {a.x / s, a.y / s, a.z / s}; }
template <class R> R dot(V<R> a, V<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class R> V<R> cross(V<R> a, V<R> b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class R> R len(V<R> a) { return std::sqrt(dot(a, a)); }
template <class R> R absR(R x) { return x < R(0) ? -x : x; }
template <class R> R maxR(R a, R b) { return (a < b) ? b : a; }
template <class R> R minR(R a, R b) { return (b < a) ? b : a; }
template <class R> V<R> unit(V<R> a) {
    const R m = len(a);
    return m > R(1.0e-12) ? divide(a, m) : V<R>{R(1), R(0), R(0)};
}
template <class R> V<R> ld(const std::vector<R> &p, std::size_t i) { return {p[3 * i], p[3 * i + 1], p[3 * i + 2]}; }
template <class R> void st(std::vector<R> &p, std::size_t i, V<R> v) {
    p[3 * i] = v.x; p[3 * i + 1] = v.y; p[3 * i + 2] = v.z;
}

// ---------------------------------------------------------------------------
// Schedule (LatticeSchedule.cpp:71-155): greedy edge colouring in bond order,
// owner = lower slab, stable sort by (owner, boundary, colour), ranges.
// ---------------------------------------------------------------------------
struct Schedule {
    std::uint32_t block_count{1}, color_count{}, boundary_bond_count{};
    std::vector<std::uint32_t> node_block_begin, bond_order, bond_schedule_index, bond_block_begin,
        range_begin, range_end;
    std::vector<std::uint8_t> bond_color;
};

Schedule buildSchedule(std::uint32_t node_count, const std::vector<std::uint32_t> &ba,
                       const std::vector<std::uint32_t> &bb, const std::vector<std::uint32_t> &blocks) {
    const std::uint32_t B = static_cast<std::uint32_t>(ba.size());
    if (blocks.size() < 2 || blocks.front() != 0 || blocks.back() != node_count ||
        !std::is_sorted(blocks.begin(), blocks.end()))
        throw std::invalid_argument("lattice schedule needs sorted node block offsets covering every node");
    Schedule s;
    s.block_count = static_cast<std::uint32_t>(blocks.size() - 1);
    s.node_block_begin = blocks;
    std::vector<std::uint32_t> block_of(node_count);
    for (std::uint32_t b = 0; b < s.block_count; ++b)
        for (std::uint32_t n = blocks[b]; n < blocks[b + 1]; ++n) block_of[n] = b;
    std::vector<std::uint64_t> used(node_count, 0);
    std::vector<std::uint8_t> color(B), boundary(B);
    std::vector<std::uint32_t> owner(B);
    std::uint32_t colors = 0;
    for (std::uint32_t k = 0; k < B; ++k) {
        const std::uint32_t a = ba[k], b = bb[k];
        if (a >= node_count || b >= node_count || a == b) throw std::invalid_argument("lattice bond joins invalid nodes");
        const std::uint64_t free_bits = ~(used[a] | used[b]);
        if (free_bits == 0) throw std::runtime_error("lattice needs more than 64 bond colours");
        unsigned c = 0;
        while (((free_bits >> c) & 1ULL) == 0) ++c;
        used[a] |= 1ULL << c;
        used[b] |= 1ULL << c;
        color[k] = static_cast<std::uint8_t>(c);
        colors = std::max(colors, c + 1U);
        const std::uint32_t lo = std::min(block_of[a], block_of[b]), hi = std::max(block_of[a], block_of[b]);
        if (hi - lo > 1) throw std::invalid_argument("slab decomposition needs slabs at least one neighbour horizon thick");
        owner[k] = lo;
        boundary[k] = hi != lo ? 1 : 0;
        if (boundary[k]) ++s.boundary_bond_count;
    }
    s.color_count = colors;
    // A stable sort on (owner, boundary, colour) is a counting sort on that key.
    const std::uint32_t C = std::max(colors, 1U);
    const std::size_t keys = static_cast<std::size_t>(s.block_count) * 2 * C;
    std::vector<std::uint32_t> start(keys + 1, 0);
    auto keyOf = [&](std::uint32_t k) { return (static_cast<std::size_t>(owner[k]) * 2 + boundary[k]) * C + color[k]; };
    for (std::uint32_t k = 0; k < B; ++k) ++start[keyOf(k) + 1];
    for (std::size_t q = 0; q < keys; ++q) start[q + 1] += start[q];
    s.bond_order.resize(B);
    std::vector<std::uint32_t> cursor(start.begin(), start.end() - 1);
    for (std::uint32_t k = 0; k < B; ++k) s.bond_order[cursor[keyOf(k)]++] = k;
    s.bond_schedule_index.resize(B);
    s.bond_color.resize(B);
    for (std::uint32_t q = 0; q < B; ++q) {
        s.bond_schedule_index[s.bond_order[q]] = q;
        s.bond_color[q] = color[s.bond_order[q]];
    }
    s.range_begin.assign(keys, 0);
    s.range_end.assign(keys, 0);
    for (std::size_t q = 0; q < keys; ++q)
        if (start[q + 1] > start[q]) { s.range_begin[q] = start[q]; s.range_end[q] = start[q + 1]; }
    s.bond_block_begin.assign(s.block_count + 1, 0);
    for (std::uint32_t q = 0; q < B; ++q) s.bond_block_begin[owner[s.bond_order[q]] + 1] = q + 1;
    for (std::uint32_t b = 1; b <= s.block_count; ++b)
        s.bond_block_begin[b] = std::max(s.bond_block_begin[b], s.bond_block_begin[b - 1]);
    return s;
}

// ---------------------------------------------------------------------------
// Working lattice (FastLattice.cpp:47-169 then LatticeWorking.hpp:53-124).
// ---------------------------------------------------------------------------
template <class R> struct Lattice {
    std::uint32_t N{}, B{}, blocks{}, C{}, D{};
    std::vector<R> x0, u, u_prev, v, inv_mass, mass, rinv, unmeasured, strain, approach;
    std::vector<std::uint8_t> node_valid, node_dirty, engaged, candidate;
    std::vector<std::uint32_t> node_block_begin, nbr_bond, nbr_other, bond_slot_a, bond_slot_b, bond_a, bond_b;
    std::vector<R> nbr_rest, nbr_weight;
    std::vector<std::uint8_t> nbr_alive;
    std::vector<R> rest_edge, rest_length, rsm, compliance, threshold;
    std::vector<std::uint8_t> alive, failure_mode;
    std::vector<R> damage, lambda, plastic_ext, plastic_strain, prev_t, prev_c, prev_s;
    std::vector<std::uint32_t> range_begin, range_end, candidate_list, candidate_count;
};

template <class R> std::vector<R> cast(const std::vector<double> &in) {
    std::vector<R> out(in.size());
    for (std::size_t i = 0; i < in.size(); ++i) out[i] = static_cast<R>(in[i]);
    return out;
}

template <class R>
Lattice<R> buildLattice(const lsio::Case &c, const Schedule &s) {
    Lattice<R> L;
    const auto N = c.scalar<std::uint32_t>("node_count");
    const auto B = c.scalar<std::uint32_t>("bond_count");
    const auto ref = c.get<double>("ref_pos"), pos = c.get<double>("pos"), vel = c.get<double>("vel");
    const auto mass = c.get<double>("mass");
    const auto ba = c.get<std::uint32_t>("bond_a"), bb = c.get<std::uint32_t>("bond_b");
    const auto rest = c.get<double>("rest_length"), comp = c.get<double>("compliance"), thr = c.get<double>("threshold");
    const auto origin = c.get<double>("origin");
    std::vector<std::uint8_t> alive0(B, 1);
    if (c.has("alive")) alive0 = c.get<std::uint8_t>("alive");
    L.N = N; L.B = B; L.blocks = s.block_count; L.C = s.color_count;
    std::vector<double> x0(3 * N), u(3 * N), vv(3 * N), inv(N);
    for (std::uint32_t i = 0; i < N; ++i)
        for (int k = 0; k < 3; ++k) {
            x0[3 * i + k] = ref[3 * i + k] - origin[k];
            u[3 * i + k] = pos[3 * i + k] - ref[3 * i + k];
            vv[3 * i + k] = vel[3 * i + k];
        }
    for (std::uint32_t i = 0; i < N; ++i) inv[i] = mass[i] > 0.0 ? 1.0 / mass[i] : 0.0;
    if (c.has("pinned")) {
        const auto pinned = c.get<std::uint8_t>("pinned");
        for (std::uint32_t i = 0; i < N; ++i) if (pinned[i]) inv[i] = 0.0;
    }
    // Bonds in schedule order; geometry from the reference positions in double.
    std::vector<double> redge(3 * static_cast<std::size_t>(B)), rlen(B), rsm(B), weight(B), cmp(B), th(6 * static_cast<std::size_t>(B));
    L.bond_a.resize(B); L.bond_b.resize(B); L.alive.resize(B); L.failure_mode.assign(B, 0);
    for (std::uint32_t q = 0; q < B; ++q) {
        const std::uint32_t o = s.bond_order[q];
        L.bond_a[q] = ba[o]; L.bond_b[q] = bb[o];
        const double ex = ref[3 * bb[o]] - ref[3 * ba[o]];
        const double ey = ref[3 * bb[o] + 1] - ref[3 * ba[o] + 1];
        const double ez = ref[3 * bb[o] + 2] - ref[3 * ba[o] + 2];
        redge[3 * q] = ex; redge[3 * q + 1] = ey; redge[3 * q + 2] = ez;
        rlen[q] = rest[o];
        const double e2 = ex * ex + ey * ey + ez * ez;
        rsm[q] = e2 - rest[o] * rest[o];
        weight[q] = e2 > 1.0e-18 ? 1.0 / e2 : 0.0;
        cmp[q] = comp[o];
        for (int k = 0; k < 6; ++k) th[6 * static_cast<std::size_t>(q) + k] = thr[6 * static_cast<std::size_t>(o) + k];
        L.alive[q] = alive0[o] ? 1 : 0;
    }
    // Adjacency in original bond order, padded k-major neighbour lists.
    std::vector<std::uint32_t> deg(N, 0), off(N + 1, 0);
    for (std::uint32_t o = 0; o < B; ++o) { ++deg[ba[o]]; ++deg[bb[o]]; }
    for (std::uint32_t i = 0; i < N; ++i) off[i + 1] = off[i] + deg[i];
    std::vector<std::uint32_t> adj(off[N]), cur(off.begin(), off.end() - 1);
    for (std::uint32_t o = 0; o < B; ++o) {
        const std::uint32_t q = s.bond_schedule_index[o];
        adj[cur[ba[o]]++] = q;
        adj[cur[bb[o]]++] = q;
    }
    std::uint32_t D = 0;
    for (std::uint32_t i = 0; i < N; ++i) D = std::max(D, off[i + 1] - off[i]);
    L.D = D;
    const std::size_t P = static_cast<std::size_t>(D) * N;
    L.nbr_bond.assign(P, kNoBond); L.nbr_other.assign(P, 0); L.nbr_alive.assign(P, 0);
    std::vector<double> nrest(3 * P, 0.0), nweight(P, 0.0);
    L.bond_slot_a.assign(B, 0); L.bond_slot_b.assign(B, 0);
    for (std::uint32_t i = 0; i < N; ++i)
        for (std::uint32_t k = 0; k < off[i + 1] - off[i]; ++k) {
            const std::uint32_t q = adj[off[i] + k];
            const std::size_t slot = static_cast<std::size_t>(k) * N + i;
            L.nbr_bond[slot] = q;
            L.nbr_alive[slot] = L.alive[q];
            const bool is_a = L.bond_a[q] == i;
            (is_a ? L.bond_slot_a : L.bond_slot_b)[q] = static_cast<std::uint32_t>(slot);
            L.nbr_other[slot] = is_a ? L.bond_b[q] : L.bond_a[q];
            const double sign = is_a ? 1.0 : -1.0;
            for (int d = 0; d < 3; ++d) nrest[3 * slot + d] = sign * redge[3 * static_cast<std::size_t>(q) + d];
            nweight[slot] = weight[q];
        }
    L.x0 = cast<R>(x0); L.u = cast<R>(u); L.u_prev = L.u; L.v = cast<R>(vv);
    L.inv_mass = cast<R>(inv); L.mass = cast<R>(mass);
    L.rinv.assign(9 * static_cast<std::size_t>(N), R(0));
    L.unmeasured.assign(3 * static_cast<std::size_t>(N), R(0));
    L.strain.assign(6 * static_cast<std::size_t>(N), R(0));
    L.approach.assign(kPlanes * static_cast<std::size_t>(N), R(0));
    L.node_valid.assign(N, 0); L.node_dirty.assign(N, 1);
    L.engaged.assign(kPlanes * static_cast<std::size_t>(N), 0); L.candidate.assign(N, 0);
    L.node_block_begin = s.node_block_begin;
    L.nbr_rest = cast<R>(nrest); L.nbr_weight = cast<R>(nweight);
    L.rest_edge = cast<R>(redge); L.rest_length = cast<R>(rlen); L.rsm = cast<R>(rsm);
    L.compliance = cast<R>(cmp); L.threshold = cast<R>(th);
    L.damage.assign(B, R(0)); L.lambda.assign(B, R(0)); L.plastic_ext.assign(B, R(0)); L.plastic_strain.assign(B, R(0));
    L.prev_t.assign(B, R(0)); L.prev_c.assign(B, R(0)); L.prev_s.assign(B, R(0));
    L.range_begin = s.range_begin; L.range_end = s.range_end;
    L.candidate_list.assign(static_cast<std::size_t>(s.block_count) * kCandidatesPerBlock, 0);
    L.candidate_count.assign(s.block_count, 0);
    return L;
}

// ---------------------------------------------------------------------------
// Settings and sphere (LatticePhysics.hpp:114-158, 248-284) cast to R the way
// LatticeWorking.hpp:213-288 casts them.
// ---------------------------------------------------------------------------
template <class R> struct Plane {
    V<R> point, normal, tangent, bitangent;
    R restitution, static_friction, dynamic_friction, node_radius;
    std::uint8_t reach_capped;
    std::uint32_t footprint_count;
    R fp[kFootprints][4];
};
template <class R> struct Settings {
    R dt;
    V<R> gravity;
    std::uint32_t iterations;
    R damping_fraction;
    std::uint8_t sphere_enabled, direct;
    R yield_stretch, hardening, plate_half_thickness;
    R c_static, c_dynamic, c_restitution, c_threshold, c_node_radius, c_margin, c_slack;
    std::uint32_t plane_count;
    Plane<R> planes[kPlanes];
    // NodeContactSettings (LatticePhysics.hpp:188-202); 0 off, 1 measure, 2 on.
    std::uint8_t nc_mode;
    R nc_radius, nc_skin, nc_margin, nc_restitution, nc_threshold, nc_static, nc_dynamic;
    std::uint32_t nc_mask;
    std::uint8_t audit; // StepSettings::audit_energy
};
template <class R> struct Sphere { V<R> center, velocity, angular; R radius, mass, inertia; };

template <class R> V<R> v3of(const std::vector<double> &s, int at) {
    return {static_cast<R>(s[at]), static_cast<R>(s[at + 1]), static_cast<R>(s[at + 2])};
}

template <class R> Settings<R> unpackSettings(const std::vector<double> &s) {
    if (s.size() != static_cast<std::size_t>(lsio::kSettingsWidth) &&
        s.size() != static_cast<std::size_t>(lsio::kAuditEnergy) &&
        s.size() != static_cast<std::size_t>(lsio::kNodeContact))
        throw std::invalid_argument("settings width");
    Settings<R> o{};
    o.dt = static_cast<R>(s[lsio::kDt]);
    o.gravity = v3of<R>(s, lsio::kGravity);
    o.iterations = static_cast<std::uint32_t>(s[lsio::kIterations]);
    o.damping_fraction = static_cast<R>(s[lsio::kDampingFraction]);
    o.sphere_enabled = static_cast<std::uint8_t>(s[lsio::kSphereEnabled]);
    o.direct = static_cast<std::uint8_t>(s[lsio::kDirectArithmetic]);
    o.yield_stretch = static_cast<R>(s[lsio::kPlasticYield]);
    o.hardening = static_cast<R>(s[lsio::kPlasticHardening]);
    o.plate_half_thickness = static_cast<R>(s[lsio::kPlateHalfThickness]);
    const int c = lsio::kContact;
    o.c_static = static_cast<R>(s[c]); o.c_dynamic = static_cast<R>(s[c + 1]);
    o.c_restitution = static_cast<R>(s[c + 2]); o.c_threshold = static_cast<R>(s[c + 3]);
    o.c_node_radius = static_cast<R>(s[c + 4]); o.c_margin = static_cast<R>(s[c + 5]);
    o.c_slack = static_cast<R>(s[c + 6]);
    o.plane_count = static_cast<std::uint32_t>(s[lsio::kPlaneCount]);
    for (unsigned p = 0; p < kPlanes; ++p) {
        const int b = lsio::kPlanes + static_cast<int>(p) * lsio::kPlaneWidth;
        Plane<R> &pl = o.planes[p];
        pl.point = v3of<R>(s, b + lsio::kPlanePoint);
        pl.normal = v3of<R>(s, b + lsio::kPlaneNormal);
        pl.tangent = v3of<R>(s, b + lsio::kPlaneTangent);
        pl.bitangent = v3of<R>(s, b + lsio::kPlaneBitangent);
        pl.restitution = static_cast<R>(s[b + lsio::kPlaneRestitution]);
        pl.static_friction = static_cast<R>(s[b + lsio::kPlaneStatic]);
        pl.dynamic_friction = static_cast<R>(s[b + lsio::kPlaneDynamic]);
        pl.node_radius = static_cast<R>(s[b + lsio::kPlaneNodeRadius]);
        pl.reach_capped = static_cast<std::uint8_t>(s[b + lsio::kPlaneReachCapped]);
        pl.footprint_count = static_cast<std::uint32_t>(s[b + lsio::kPlaneFootprintCount]);
        for (unsigned f = 0; f < kFootprints; ++f)
            for (int q = 0; q < 4; ++q) pl.fp[f][q] = static_cast<R>(s[b + lsio::kPlaneFootprints + 4 * static_cast<int>(f) + q]);
    }
    if (s.size() > static_cast<std::size_t>(lsio::kAuditEnergy)) o.audit = static_cast<std::uint8_t>(s[lsio::kAuditEnergy]);
    if (s.size() > static_cast<std::size_t>(lsio::kNodeContact)) {
        const int n = lsio::kNodeContact;
        o.nc_mode = static_cast<std::uint8_t>(s[n]);
        o.nc_radius = static_cast<R>(s[n + 1]); o.nc_skin = static_cast<R>(s[n + 2]);
        o.nc_margin = static_cast<R>(s[n + 3]); o.nc_restitution = static_cast<R>(s[n + 4]);
        o.nc_threshold = static_cast<R>(s[n + 5]); o.nc_static = static_cast<R>(s[n + 6]);
        o.nc_dynamic = static_cast<R>(s[n + 7]); o.nc_mask = static_cast<std::uint32_t>(s[n + 8]);
    }
    return o;
}

template <class R> Sphere<R> unpackSphere(const std::vector<double> &s) {
    return {v3of<R>(s, 0), v3of<R>(s, 3), v3of<R>(s, 6), static_cast<R>(s[9]), static_cast<R>(s[10]), static_cast<R>(s[11])};
}

struct ContactAcc {
    std::uint64_t impulse_contacts{}, candidate_overflow{}, ball_support_events{};
    double impulse_x{}, impulse_y{}, impulse_z{}, dissipated{}, max_penetration{}, max_correction{}, max_center_shift{};
};

// ---------------------------------------------------------------------------
// Element physics.
// ---------------------------------------------------------------------------
template <class R> V<R> position(const Lattice<R> &L, std::size_t i) { return add(ld(L.x0, i), ld(L.u, i)); }

template <class R> V<R> bondVector(const Lattice<R> &L, std::size_t j, bool direct) {
    const std::uint32_t a = L.bond_a[j], b = L.bond_b[j];
    if (direct) return sub(position(L, b), position(L, a));
    return add(ld(L.rest_edge, j), sub(ld(L.u, b), ld(L.u, a)));
}

// Cyclic Jacobi, 12 sweeps (LatticePhysics.hpp:455-493).
template <class R> void eigen3(const R m[9], R d[3], R v[9]) {
    R a[9];
    for (int k = 0; k < 9; ++k) a[k] = m[k];
    for (int k = 0; k < 9; ++k) v[k] = (k % 4 == 0) ? R(1) : R(0);
    for (int sweep = 0; sweep < 12; ++sweep) {
        const R off = absR(a[1]) + absR(a[2]) + absR(a[5]);
        if (!(off > R(0))) break;
        for (int p = 0; p < 2; ++p)
            for (int q = p + 1; q < 3; ++q) {
                const R apq = a[p * 3 + q];
                if (!(absR(apq) > R(0))) continue;
                const R app = a[p * 3 + p], aqq = a[q * 3 + q];
                const R theta = (aqq - app) / (R(2) * apq);
                const R sgn = theta >= R(0) ? R(1) : R(-1);
                const R t = sgn / (absR(theta) + std::sqrt(theta * theta + R(1)));
                const R c = R(1) / std::sqrt(t * t + R(1));
                const R sn = t * c;
                for (int k = 0; k < 3; ++k) {
                    const R akp = a[k * 3 + p], akq = a[k * 3 + q];
                    a[k * 3 + p] = c * akp - sn * akq;
                    a[k * 3 + q] = sn * akp + c * akq;
                }
                for (int k = 0; k < 3; ++k) {
                    const R apk = a[p * 3 + k], aqk = a[q * 3 + k];
                    a[p * 3 + k] = c * apk - sn * aqk;
                    a[q * 3 + k] = sn * apk + c * aqk;
                }
                for (int k = 0; k < 3; ++k) {
                    const R vkp = v[k * 3 + p], vkq = v[k * 3 + q];
                    v[k * 3 + p] = c * vkp - sn * vkq;
                    v[k * 3 + q] = sn * vkp + c * vkq;
                }
            }
    }
    d[0] = a[0]; d[1] = a[4]; d[2] = a[8];
}

// Truncating pseudo-inverse (LatticePhysics.hpp:506-531).
template <class R> int pinv3(const R m[9], R out[9], R unmeasured[3]) {
    R d[3], v[9];
    eigen3(m, d, v);
    R largest = absR(d[0]);
    if (absR(d[1]) > largest) largest = absR(d[1]);
    if (absR(d[2]) > largest) largest = absR(d[2]);
    const R floor_value = (sizeof(R) == 8 ? R(1.0e-9) : R(1.0e-5)) * largest;
    for (int k = 0; k < 9; ++k) out[k] = R(0);
    for (int k = 0; k < 3; ++k) unmeasured[k] = R(0);
    int rank = 0, dropped = -1;
    for (int c = 0; c < 3; ++c) {
        if (!(d[c] > floor_value)) { dropped = c; continue; }
        ++rank;
        const R inv = R(1) / d[c];
        for (int r = 0; r < 3; ++r)
            for (int col = 0; col < 3; ++col) out[r * 3 + col] += inv * v[r * 3 + c] * v[col * 3 + c];
    }
    if (rank == 2 && dropped >= 0)
        for (int k = 0; k < 3; ++k) unmeasured[k] = v[k * 3 + dropped];
    return rank;
}

// Bending strain of a sheet one cell thick (plateBendingStrain,
// LatticePhysics.hpp:575-777): the rest neighbourhood (every bond built, alive
// or not) says whether the node lies in a sheet and which way the sheet
// faces; a tilt fit and then a curvature fit over the live neighbours; a fit
// that explains no more than 0.9 of the out-of-plane motion claims no
// bending; the tension fibre of |K| at half the thickness, capped at the yield
// stretch, is added to E in the sheet's frame.
template <class R>
void plateBending(const Lattice<R> &L, std::size_t i, bool direct, R half_thickness, R yield_stretch, V<R> xi,
                  R *e) {
    const std::size_t N = L.N, D = L.D;
    R rest_cov[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (std::size_t k = 0; k < D; ++k) {
        const std::size_t slot = k * N + i;
        if (L.nbr_bond[slot] == kNoBond) continue;
        const R w = L.nbr_weight[slot];
        if (w <= R(0)) continue;
        const R rr[3] = {L.nbr_rest[3 * slot], L.nbr_rest[3 * slot + 1], L.nbr_rest[3 * slot + 2]};
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) rest_cov[r * 3 + c] += w * rr[r] * rr[c];
    }
    R rest_inv[9], flat[3];
    if (pinv3(rest_cov, rest_inv, flat) >= 3) return; // a solid neighbourhood, not a sheet
    const V<R> normal{flat[0], flat[1], flat[2]};
    if (!(dot(normal, normal) > R(0))) return;
    const R *inv = &L.rinv[9 * i];
    auto neighbour = [&](std::size_t k, R &w, V<R> &rest, V<R> &d) {
        const std::size_t slot = k * N + i;
        const bool present = L.nbr_bond[slot] != kNoBond;
        const std::size_t other = present ? L.nbr_other[slot] : i;
        w = (present && L.nbr_alive[slot]) ? L.nbr_weight[slot] : R(0);
        rest = present ? V<R>{L.nbr_rest[3 * slot], L.nbr_rest[3 * slot + 1], L.nbr_rest[3 * slot + 2]}
                       : V<R>{R(0), R(0), R(0)};
        const V<R> xo = direct ? position(L, other) : ld(L.u, other);
        d = direct ? sub(sub(xo, xi), rest) : sub(xo, xi);
    };
    // The tilt.
    R rhs[3] = {0, 0, 0};
    for (std::size_t k = 0; k < D; ++k) {
        R w;
        V<R> rest, d;
        neighbour(k, w, rest, d);
        const R out = w * dot(d, normal);
        rhs[0] += out * rest.x;
        rhs[1] += out * rest.y;
        rhs[2] += out * rest.z;
    }
    R tilt[3];
    for (int r = 0; r < 3; ++r) {
        R acc = R(0);
        for (int k = 0; k < 3; ++k) acc += inv[r * 3 + k] * rhs[k];
        tilt[r] = acc;
    }
    // The in-plane frame, from the axis the normal leans on least.
    const R ax = normal.x < R(0) ? -normal.x : normal.x;
    const R ay = normal.y < R(0) ? -normal.y : normal.y;
    const R az = normal.z < R(0) ? -normal.z : normal.z;
    const V<R> axis = (ax <= ay && ax <= az) ? V<R>{R(1), R(0), R(0)}
                    : (ay <= az)             ? V<R>{R(0), R(1), R(0)}
                                             : V<R>{R(0), R(0), R(1)};
    V<R> e1 = cross(normal, axis);
    const R e1len = len(e1);
    if (!(e1len > R(0))) return;
    e1 = scale(e1, R(1) / e1len);
    const V<R> e2 = cross(normal, e1);
    // The curvature, over what the tilt leaves.
    R A[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    R g[3] = {0, 0, 0};
    R out2 = R(0);
    for (std::size_t k = 0; k < D; ++k) {
        R w;
        V<R> rest, d;
        neighbour(k, w, rest, d);
        const R left = dot(d, normal) - (tilt[0] * rest.x + tilt[1] * rest.y + tilt[2] * rest.z);
        const R p1 = dot(rest, e1), p2 = dot(rest, e2);
        const R psi[3] = {R(0.5) * p1 * p1, p1 * p2, R(0.5) * p2 * p2};
        for (int r = 0; r < 3; ++r) {
            for (int c = 0; c < 3; ++c) A[r * 3 + c] += w * psi[r] * psi[c];
            g[r] += w * psi[r] * left;
        }
        out2 += w * left * left;
    }
    R ev[3], axes[9];
    eigen3(A, ev, axes);
    R biggest = absR(ev[0]);
    for (int k = 1; k < 3; ++k) biggest = absR(ev[k]) > biggest ? absR(ev[k]) : biggest;
    const R determined = R(1.0e-3) * biggest;
    R c[3] = {0, 0, 0};
    int along = 0;
    for (int k = 0; k < 3; ++k) {
        if (!(ev[k] > determined)) continue;
        ++along;
        R projected = R(0);
        for (int r = 0; r < 3; ++r) projected += axes[r * 3 + k] * g[r];
        const R amount = projected / ev[k];
        for (int r = 0; r < 3; ++r) c[r] += amount * axes[r * 3 + k];
    }
    if (along < 1) return;
    const R explained = c[0] * g[0] + c[1] * g[1] + c[2] * g[2];
    if (!(explained > R(0.9) * out2)) return;
    // |K| through the trace and the eigenvalue split of [[c0, c1], [c1, c2]].
    const R half_trace = R(0.5) * (c[0] + c[2]);
    const R det = c[0] * c[2] - c[1] * c[1];
    R under = half_trace * half_trace - det;
    if (under < R(0)) under = R(0);
    const R disc = std::sqrt(under);
    const R l1 = half_trace + disc, l2 = half_trace - disc;
    const R a1 = l1 < R(0) ? -l1 : l1, a2 = l2 < R(0) ? -l2 : l2;
    const R most = yield_stretch > R(0) ? yield_stretch : R(-1);
    R s1 = half_thickness * a1, s2 = half_thickness * a2;
    if (most > R(0)) {
        if (s1 > most) s1 = most;
        if (s2 > most) s2 = most;
    }
    const R alpha = R(0.5) * (s1 + s2), beta = R(0.5) * (s1 - s2);
    const R ratio = disc > R(0) ? beta / disc : R(0);
    const R b11 = alpha + ratio * (c[0] - half_trace);
    const R b12 = ratio * c[1];
    const R b22 = alpha + ratio * (c[2] - half_trace);
    const R u1[3] = {e1.x, e1.y, e1.z}, u2[3] = {e2.x, e2.y, e2.z};
    static const int rows[6] = {0, 1, 2, 0, 0, 1}, cols[6] = {0, 1, 2, 1, 2, 2};
    for (int q = 0; q < 6; ++q)
        e[q] += b11 * u1[rows[q]] * u1[cols[q]] + b22 * u2[rows[q]] * u2[cols[q]] +
                b12 * (u1[rows[q]] * u2[cols[q]] + u2[rows[q]] * u1[cols[q]]);
}

// Nonlocal node strain (LatticePhysics.hpp:791-907).
template <class R>
void nodeStrain(Lattice<R> &L, std::size_t i, bool direct, std::uint32_t &rank_deficient, R plate_half_thickness,
                R plate_yield) {
    const std::size_t N = L.N, D = L.D;
    if (L.node_dirty[i]) {
        R cov[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        std::uint32_t live = 0;
        for (std::size_t k = 0; k < D; ++k) {
            const std::size_t slot = k * N + i;
            if (L.nbr_bond[slot] == kNoBond) break;
            if (!L.nbr_alive[slot]) continue;
            const R w = L.nbr_weight[slot];
            if (w <= R(0)) continue;
            const R rr[3] = {L.nbr_rest[3 * slot], L.nbr_rest[3 * slot + 1], L.nbr_rest[3 * slot + 2]};
            for (int r = 0; r < 3; ++r)
                for (int c = 0; c < 3; ++c) cov[r * 3 + c] += w * rr[r] * rr[c];
            ++live;
        }
        std::uint8_t valid = 0;
        if (live >= 1) {
            R inv[9], un[3];
            const int rank = pinv3(cov, inv, un);
            if (rank >= 2) {
                for (int k = 0; k < 9; ++k) L.rinv[9 * i + k] = inv[k];
                for (int k = 0; k < 3; ++k) L.unmeasured[3 * i + k] = un[k];
                valid = 1;
            }
            if (rank < 3) ++rank_deficient;
        }
        L.node_valid[i] = valid;
        L.node_dirty[i] = 0;
    }
    if (!L.node_valid[i]) return;
    R acc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    const V<R> xi = direct ? position(L, i) : ld(L.u, i);
    for (std::size_t k = 0; k < D; ++k) {
        const std::size_t slot = k * N + i;
        const bool present = L.nbr_bond[slot] != kNoBond;
        const std::size_t other = present ? L.nbr_other[slot] : i;
        const R w = (present && L.nbr_alive[slot]) ? L.nbr_weight[slot] : R(0);
        const V<R> rest = present ? V<R>{L.nbr_rest[3 * slot], L.nbr_rest[3 * slot + 1], L.nbr_rest[3 * slot + 2]}
                                  : V<R>{R(0), R(0), R(0)};
        const V<R> xo = direct ? position(L, other) : ld(L.u, other);
        const V<R> cur = direct ? sub(sub(xo, xi), rest) : sub(xo, xi);
        const R cc[3] = {cur.x, cur.y, cur.z}, rr[3] = {rest.x, rest.y, rest.z};
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) acc[r * 3 + c] += w * cc[r] * rr[c];
    }
    const R *inv = &L.rinv[9 * i];
    R f[9];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
            R s = R(0);
            for (int k = 0; k < 3; ++k) s += acc[r * 3 + k] * inv[k * 3 + c];
            f[r * 3 + c] = s;
        }
    static const int rows[6] = {0, 1, 2, 0, 0, 1}, cols[6] = {0, 1, 2, 1, 2, 2};
    R e[6];
    for (int q = 0; q < 6; ++q) {
        R c = R(0);
        for (int k = 0; k < 3; ++k) c += f[k * 3 + rows[q]] * f[k * 3 + cols[q]];
        e[q] = R(0.5) * (f[rows[q] * 3 + cols[q]] + f[cols[q] * 3 + rows[q]] + c);
    }
    const R un[3] = {L.unmeasured[3 * i], L.unmeasured[3 * i + 1], L.unmeasured[3 * i + 2]};
    if (un[0] * un[0] + un[1] * un[1] + un[2] * un[2] > R(0)) {
        const R a[3] = {e[0] * un[0] + e[3] * un[1] + e[4] * un[2], e[3] * un[0] + e[1] * un[1] + e[5] * un[2],
                        e[4] * un[0] + e[5] * un[1] + e[2] * un[2]};
        const R s = a[0] * un[0] + a[1] * un[1] + a[2] * un[2];
        for (int q = 0; q < 6; ++q)
            e[q] += -un[rows[q]] * a[cols[q]] - a[rows[q]] * un[cols[q]] + s * un[rows[q]] * un[cols[q]];
        if (plate_half_thickness > R(0)) plateBending(L, i, direct, plate_half_thickness, plate_yield, xi, e);
    }
    for (int q = 0; q < 6; ++q) L.strain[6 * i + q] = e[q];
}

template <class R> void resolve(const R *e, V<R> d, R &normal, R &shear) {
    const V<R> tr{e[0] * d.x + e[3] * d.y + e[4] * d.z, e[3] * d.x + e[1] * d.y + e[5] * d.z,
                  e[4] * d.x + e[5] * d.y + e[2] * d.z};
    normal = dot(d, tr);
    shear = len(sub(tr, scale(d, normal)));
}

template <class R> R bondStretch(const Lattice<R> &L, std::size_t j, bool direct) {
    const V<R> delta = bondVector(L, j, direct);
    const R l = len(delta);
    const R rest = L.rest_length[j];
    if (direct) return l / rest - R(1);
    const V<R> du = sub(ld(L.u, L.bond_b[j]), ld(L.u, L.bond_a[j]));
    const V<R> r = ld(L.rest_edge, j);
    const R num = L.rsm[j] + R(2) * dot(r, du) + dot(du, du);
    return num / ((l + rest) * rest);
}

template <class R> void sampleBond(const Lattice<R> &L, std::size_t j, bool direct, R &t, R &c, R &s) {
    const R stretch = bondStretch(L, j, direct);
    t = stretch; c = -stretch; s = R(0);
    const V<R> edge = ld(L.rest_edge, j);
    const R rl = len(edge);
    if (rl > R(1.0e-9)) {
        const V<R> dir = scale(edge, R(1) / rl);
        const std::uint32_t ends[2] = {L.bond_a[j], L.bond_b[j]};
        for (int q = 0; q < 2; ++q) {
            const std::uint32_t n = ends[q];
            if (!L.node_valid[n]) continue;
            R nn, sh;
            resolve(&L.strain[6 * static_cast<std::size_t>(n)], dir, nn, sh);
            t = maxR(t, nn);
            c = maxR(c, -nn);
            s = maxR(s, sh);
        }
    }
}

template <class R> R progress(R value, R start, R end) {
    if (!std::isfinite(start) || value <= start) return R(0);
    if (!std::isfinite(end) || end <= start) return value > start ? R(1) : R(0);
    const R p = (value - start) / (end - start);
    return p < R(0) ? R(0) : (p > R(1) ? R(1) : p);
}

template <class R> R elasticExtension(const Lattice<R> &L, std::size_t j, bool direct) {
    return len(bondVector(L, j, direct)) - L.rest_length[j] - L.plastic_ext[j];
}

template <class R> R storedEnergy(const Lattice<R> &L, std::size_t j, bool direct) {
    const R c = L.compliance[j];
    if (c <= R(0)) return R(0);
    const R e = elasticExtension(L, j, direct);
    return R(0.5) * e * e / c;
}

template <class R> R plasticReturn(Lattice<R> &L, const Settings<R> &S, std::size_t j, bool direct) {
    if (!(S.yield_stretch > R(0))) return R(0);
    const R elastic = elasticExtension(L, j, direct);
    const R magnitude = absR(elastic);
    const R h = S.hardening;
    const R yield = S.yield_stretch * L.rest_length[j] + h * L.plastic_strain[j];
    if (!(magnitude > yield)) return R(0);
    const R inc = (magnitude - yield) / (R(1) + h);
    L.plastic_ext[j] = L.plastic_ext[j] + (elastic < R(0) ? -inc : inc);
    L.plastic_strain[j] = L.plastic_strain[j] + inc;
    const R c = L.compliance[j];
    if (!(c > R(0))) return R(0);
    const R yield_end = yield + h * inc;
    return R(0.5) * (yield + yield_end) * inc / c;
}

struct Outcome {
    bool broke;
    double removed;
    float peak_t, peak_c, peak_s;
    double plastic;
    float plastic_stretch;
    float damage;
};

// End-of-substep sample, plastic return and failure (LatticePhysics.hpp:1068-1114).
template <class R> Outcome endSample(Lattice<R> &L, const Settings<R> &S, std::size_t j, bool direct) {
    Outcome o{false, 0.0, 0.0F, 0.0F, 0.0F, 0.0, 0.0F, 0.0F};
    if (S.yield_stretch > R(0)) {
        o.plastic = static_cast<double>(plasticReturn(L, S, j, direct));
        o.plastic_stretch = static_cast<float>(absR(L.plastic_ext[j]) / L.rest_length[j]);
    }
    R t, c, s;
    sampleBond(L, j, direct, t, c, s);
    const R pt = maxR(R(0), maxR(L.prev_t[j], t));
    const R pc = maxR(R(0), maxR(L.prev_c[j], c));
    const R ps = maxR(R(0), maxR(L.prev_s[j], s));
    o.peak_t = static_cast<float>(pt); o.peak_c = static_cast<float>(pc); o.peak_s = static_cast<float>(ps);
    L.prev_t[j] = maxR(R(0), t); L.prev_c[j] = maxR(R(0), c); L.prev_s[j] = maxR(R(0), s);
    const R *th = &L.threshold[6 * j];
    const R dt_ = progress(pt, th[0], th[1]), dc = progress(pc, th[2], th[3]), ds = progress(ps, th[4], th[5]);
    R damage = dt_;
    std::uint8_t mode = 1;
    if (dc > damage) { damage = dc; mode = 2; }
    if (ds > damage) { damage = ds; mode = 3; }
    if (damage > L.damage[j]) { L.damage[j] = damage; L.failure_mode[j] = mode; }
    o.damage = static_cast<float>(L.damage[j]);
    if (L.damage[j] >= R(1)) {
        o.removed = static_cast<double>(storedEnergy(L, j, direct));
        o.broke = true;
        L.alive[j] = 0;
        L.nbr_alive[L.bond_slot_a[j]] = 0;
        L.nbr_alive[L.bond_slot_b[j]] = 0;
    }
    return o;
}

template <class R> void startSample(Lattice<R> &L, std::size_t j, bool direct) {
    R t, c, s;
    sampleBond(L, j, direct, t, c, s);
    L.prev_t[j] = maxR(R(0), t); L.prev_c[j] = maxR(R(0), c); L.prev_s[j] = maxR(R(0), s);
}

// The per-bond constants of the solve, formed once per run as the reference's
// threaded lane keeps them (ParallelCpuLatticeBackend.cpp:505-530, 717-745):
// alpha = compliance / dt^2 and the denominator wa + wb + alpha, the same
// expressions in the same order, so the same numbers.
template <class R> struct Kept {
    std::vector<R> alpha, denominator;
};

template <class R> Kept<R> keepSolveConstants(const Lattice<R> &L, R dt) {
    Kept<R> k;
    k.alpha.resize(L.B);
    k.denominator.resize(L.B);
    for (std::size_t j = 0; j < L.B; ++j) {
        const R alpha = L.compliance[j] / (dt * dt);
        k.alpha[j] = alpha;
        k.denominator[j] = L.inv_mass[L.bond_a[j]] + L.inv_mass[L.bond_b[j]] + alpha;
    }
    return k;
}

// bondSolve (LatticePhysics.hpp:1133-1168).
template <class R> void solveBond(Lattice<R> &L, const Kept<R> &k, std::size_t j, bool direct, bool first) {
    if (!L.alive[j]) return;
    const std::uint32_t a = L.bond_a[j], b = L.bond_b[j];
    const V<R> delta = bondVector(L, j, direct);
    const R cl = len(delta);
    if (cl <= R(1.0e-12)) return;
    const R original = L.rest_length[j];
    const R plastic = L.plastic_ext[j];
    const R rest = original + plastic;
    R constraint;
    if (direct) {
        constraint = cl - rest;
    } else {
        const V<R> du = sub(ld(L.u, b), ld(L.u, a));
        const V<R> r = ld(L.rest_edge, j);
        constraint = (L.rsm[j] + R(2) * dot(r, du) + dot(du, du) - plastic * (rest + original)) / (cl + rest);
    }
    const V<R> dir = divide(delta, cl);
    const R wa = L.inv_mass[a], wb = L.inv_mass[b];
    const R alpha = k.alpha[j];
    const R lambda = first ? R(0) : L.lambda[j];
    const R dl = (-constraint - alpha * lambda) / k.denominator[j];
    L.lambda[j] = lambda + dl;
    st(L.u, a, sub(ld(L.u, a), scale(dir, wa * dl)));
    st(L.u, b, add(ld(L.u, b), scale(dir, wb * dl)));
}

// Radial pair damping (LatticePhysics.hpp:1171-1184).
template <class R> void dampBond(Lattice<R> &L, std::size_t j, R fraction, bool direct) {
    if (!L.alive[j]) return;
    const std::uint32_t a = L.bond_a[j], b = L.bond_b[j];
    const R ma = L.mass[a], mb = L.mass[b];
    if (ma <= R(0) || mb <= R(0)) return;
    const V<R> n = unit(bondVector(L, j, direct));
    const V<R> va = ld(L.v, a), vb = ld(L.v, b);
    const R rel = dot(sub(vb, va), n);
    const R im = R(1) / ma + R(1) / mb;
    const R impulse = -fraction * rel / im;
    st(L.v, a, sub(va, scale(n, impulse / ma)));
    st(L.v, b, add(vb, scale(n, impulse / mb)));
}

// Support planes (LatticePhysics.hpp:1189-1276).
template <class R> bool insideFootprints(const Plane<R> &p, V<R> x) {
    const V<R> rel = sub(x, p.point);
    const R t = dot(rel, p.tangent), b = dot(rel, p.bitangent);
    for (std::uint32_t k = 0; k < p.footprint_count; ++k)
        if (absR(t - p.fp[k][0]) <= p.fp[k][2] && absR(b - p.fp[k][1]) <= p.fp[k][3]) return true;
    return false;
}

template <class R> R projectSupport(Lattice<R> &L, const Plane<R> &p, std::size_t i, R approach, R dt) {
    const V<R> x = position(L, i);
    if (!insideFootprints(p, x)) return R(0);
    const R distance = dot(sub(x, p.point), p.normal) - p.node_radius;
    if (distance > R(1.0e-8)) return R(0);
    if (p.reach_capped) {
        const R reach = R(8) * maxR(R(0), -approach) * dt + R(1.0e-5);
        if (-distance > reach) return R(0);
    }
    st(L.u, i, sub(ld(L.u, i), scale(p.normal, distance)));
    return -distance;
}

template <class R> void supportVelocity(Lattice<R> &L, const Plane<R> &p, std::size_t i, R approach) {
    V<R> vel = ld(L.v, i);
    const R restitution = -approach > R(0.5)
        ? (p.restitution < R(0) ? R(0) : (p.restitution > R(1) ? R(1) : p.restitution)) : R(0);
    const R target = approach < R(0) ? -restitution * approach : R(0);
    const R vn = dot(vel, p.normal);
    R corrected = vn;
    if (vn > target) corrected = target;
    else if (vn < R(0)) corrected = R(0);
    vel = add(vel, scale(p.normal, corrected - vn));
    const R normal_delta = corrected - minR(R(0), approach);
    if (normal_delta <= R(0)) { st(L.v, i, vel); return; }
    const V<R> tangent = sub(vel, scale(p.normal, dot(vel, p.normal)));
    const R speed = len(tangent);
    if (speed <= R(1.0e-12)) { st(L.v, i, vel); return; }
    const R fd = speed <= p.static_friction * normal_delta ? speed : minR(speed, p.dynamic_friction * normal_delta);
    vel = sub(vel, scale(tangent, fd / speed));
    st(L.v, i, vel);
}

template <class R> void nodeSupportProject(Lattice<R> &L, const Settings<R> &S, std::size_t i) {
    for (std::uint32_t p = 0; p < S.plane_count; ++p) {
        const R depth = projectSupport(L, S.planes[p], i, L.approach[p * L.N + i], S.dt);
        if (depth > R(0)) L.engaged[p * L.N + i] = 1;
    }
}
template <class R> void nodeSupportVelocity(Lattice<R> &L, const Settings<R> &S, std::size_t i) {
    for (std::uint32_t p = 0; p < S.plane_count; ++p) {
        if (!L.engaged[p * L.N + i]) continue;
        supportVelocity(L, S.planes[p], i, L.approach[p * L.N + i]);
    }
}
template <class R> void recordApproach(Lattice<R> &L, const Settings<R> &S, std::size_t i) {
    const V<R> vel = ld(L.v, i);
    for (std::uint32_t p = 0; p < S.plane_count; ++p) L.approach[p * L.N + i] = dot(vel, S.planes[p].normal);
}

// Sphere contact (LatticePhysics.hpp:1284-1428).
template <class R> bool sphereCandidate(const Lattice<R> &L, const Settings<R> &S, const Sphere<R> &sp, std::size_t i) {
    if (L.mass[i] <= R(0)) return false;
    const V<R> r = sub(position(L, i), sp.center);
    const R distance = len(r);
    const R gap = distance - (sp.radius + S.c_node_radius);
    const R bound = len(sub(ld(L.v, i), sp.velocity)) + len(sp.angular) * distance;
    const R reach = maxR(S.c_margin, bound * S.dt) + S.c_slack;
    return gap <= reach;
}
template <class R> R nodeKE(const Lattice<R> &L, std::size_t i) { const V<R> v = ld(L.v, i); return R(0.5) * L.mass[i] * dot(v, v); }
template <class R> R sphereKE(const Sphere<R> &s) {
    return R(0.5) * s.mass * dot(s.velocity, s.velocity) + R(0.5) * s.inertia * dot(s.angular, s.angular);
}

template <class R>
void sphereNode(Lattice<R> &L, const Settings<R> &S, Sphere<R> &sp, std::size_t i, bool correct, ContactAcc &acc) {
    if (L.mass[i] <= R(0)) return;
    const R dt = S.dt;
    const R ism = R(1) / sp.mass;
    const R iin = R(1) / sp.inertia;
    const R cr = sp.radius + S.c_node_radius;
    const V<R> r = sub(position(L, i), sp.center);
    const R distance = len(r);
    const V<R> normal = unit(r);
    const R gap = distance - cr;
    V<R> nv = ld(L.v, i);
    const V<R> rel = sub(sub(nv, sp.velocity), cross(sp.angular, r));
    const R vn = dot(rel, normal);
    if (gap > maxR(S.c_margin, -vn * dt)) return;
    if (-gap > R(acc.max_penetration)) acc.max_penetration = static_cast<double>(-gap);
    const R inm = R(1) / L.mass[i];
    auto eff = [&](V<R> d) { const V<R> rc = cross(r, d); return inm + ism + iin * dot(rc, rc); };
    const R restitution = -vn > S.c_threshold ? S.c_restitution : R(0);
    const R desired = gap > S.c_margin ? -gap / dt : -restitution * minR(vn, R(0));
    const R ni = maxR(R(0), (desired - vn) / eff(normal));
    if (ni > R(0)) {
        const R before = nodeKE(L, i);
        auto apply = [&](V<R> imp) {
            nv = add(nv, scale(imp, inm));
            st(L.v, i, nv);
            sp.velocity = sub(sp.velocity, scale(imp, ism));
            const V<R> ti = neg(cross(r, imp));
            sp.angular = add(sp.angular, scale(ti, iin));
            acc.impulse_x += static_cast<double>(imp.x);
            acc.impulse_y += static_cast<double>(imp.y);
            acc.impulse_z += static_cast<double>(imp.z);
        };
        apply(scale(normal, ni));
        const V<R> after = sub(sub(nv, sp.velocity), cross(sp.angular, r));
        const V<R> tangent = sub(after, scale(normal, dot(after, normal)));
        const R ts = len(tangent);
        if (ts > R(1.0e-12)) {
            const V<R> d = divide(tangent, ts);
            const R stick = ts / eff(d);
            const R fi = stick <= S.c_static * ni ? stick : minR(stick, S.c_dynamic * ni);
            apply(scale(d, -fi));
        }
        acc.dissipated += static_cast<double>(before - nodeKE(L, i));
        ++acc.impulse_contacts;
    }
    if (correct && gap < -S.c_margin) {
        const R corr = minR(-gap - S.c_margin, R(0.2) * maxR(S.c_node_radius, sp.radius * R(0.01)));
        const R sum = inm + ism;
        const V<R> ns = scale(normal, corr * inm / sum);
        const V<R> ss = neg(scale(normal, corr * ism / sum));
        st(L.u, i, add(ld(L.u, i), ns));
        sp.center = add(sp.center, ss);
        if (corr > R(acc.max_correction)) acc.max_correction = static_cast<double>(corr);
    }
}

template <class R> void spherePass(Lattice<R> &L, const Settings<R> &S, Sphere<R> &sp, int pass, ContactAcc &acc) {
    const V<R> c0 = sp.center;
    const R e0 = sphereKE(sp);
    for (std::uint32_t b = 0; b < L.blocks; ++b)
        for (std::uint32_t k = 0; k < L.candidate_count[b]; ++k) {
            const std::uint32_t i = L.candidate_list[b * kCandidatesPerBlock + k];
            sphereNode(L, S, sp, i, pass == 2, acc);
            if (pass == 1) {
                recordApproach(L, S, i);
                st(L.u, i, add(ld(L.u, i), scale(ld(L.v, i), S.dt)));
            }
        }
    acc.dissipated += static_cast<double>(e0 - sphereKE(sp));
    if (pass == 2)
        for (std::uint32_t b = 0; b < L.blocks; ++b)
            for (std::uint32_t k = 0; k < L.candidate_count[b]; ++k) nodeSupportVelocity(L, S, L.candidate_list[b * kCandidatesPerBlock + k]);
    const R shift = len(sub(sp.center, c0));
    if (shift > R(acc.max_center_shift)) acc.max_center_shift = static_cast<double>(shift);
}

template <class R> void sphereSupport(const Settings<R> &S, Sphere<R> &sp, ContactAcc &acc) {
    for (std::uint32_t p = 0; p < S.plane_count; ++p) {
        const Plane<R> &pl = S.planes[p];
        const V<R> foot = sub(sp.center, scale(pl.normal, sp.radius));
        if (!insideFootprints(pl, foot)) continue;
        const R distance = dot(sub(foot, pl.point), pl.normal);
        if (distance > R(0)) continue;
        const R vn0 = dot(sp.velocity, pl.normal);
        if (-distance > R(8) * maxR(R(0), -vn0) * S.dt + R(1.0e-5)) continue;
        const R vn = dot(sp.velocity, pl.normal);
        if (vn < R(0)) {
            const R restitution = -vn > R(0.5) ? pl.restitution : R(0);
            const R nd = -(R(1) + restitution) * vn;
            sp.velocity = add(sp.velocity, scale(pl.normal, nd));
            const V<R> tangent = sub(sp.velocity, scale(pl.normal, dot(sp.velocity, pl.normal)));
            const R speed = len(tangent);
            if (speed > R(1.0e-12)) {
                const R fd = speed <= pl.static_friction * nd ? speed : minR(speed, pl.dynamic_friction * nd);
                sp.velocity = sub(sp.velocity, scale(tangent, fd / speed));
            }
            ++acc.ball_support_events;
        }
        sp.center = sub(sp.center, scale(pl.normal, distance));
    }
}

// Exit rules (LatticePhysics.hpp:1766-1791).
unsigned exitReason(std::uint64_t completed, std::uint32_t broken, std::uint64_t last_failure, std::uint64_t quiet,
                    std::uint64_t min_steps, std::uint64_t no_failure, std::uint64_t energy_flat,
                    std::uint64_t last_energy_gain, std::uint64_t calm, std::uint64_t last_damage_gain,
                    double max_damage, double calm_margin, double removed, double removable) {
    if (removable > 0.0 && removed >= removable) return 6;
    if (broken > 0 && quiet > 0 && completed >= min_steps && completed > last_failure && completed - last_failure > quiet)
        return 1;
    if (broken == 0 && no_failure > 0 && completed >= no_failure) return 2;
    if (broken == 0 && calm > 0 && completed >= calm && max_damage < calm_margin && completed > last_damage_gain &&
        completed - last_damage_gain > calm)
        return 5;
    if (broken > 0 && energy_flat > 0 && completed >= min_steps && completed > last_energy_gain &&
        completed - last_energy_gain > energy_flat)
        return 4;
    return 0;
}

// ---------------------------------------------------------------------------
// The work pool of the threaded lane, dispatched as the reference's threaded
// backend dispatches (ParallelCpuLatticeBackend.cpp:135-320, grains at
// :1347-1356): a phase of `count` elements is cut into chunks of a fixed grain
// per phase, and the caller and the workers claim chunks from one atomic
// counter until none is left; below two chunks the caller runs the phase
// alone. Workers spin between phases (phases come every few microseconds
// inside a substep) and park on a condition variable after a stretch without
// work. Which thread runs a chunk never changes a value: elements of a phase
// are independent, and whatever a phase gathers per participant is folded
// afterwards in element order or by an order-free operation (integer sums,
// maxima).
//
// The claim word holds the job's chunk count in its high half and the next
// chunk in its low half, so one fetch-and-add both claims a chunk and says
// whether it belongs to the job in progress: a worker that wakes late can only
// ever claim a chunk of the current job, whose body the caller published
// before the claim word and keeps alive until every chunk is counted done.
// ---------------------------------------------------------------------------
class Pool {
public:
    explicit Pool(unsigned threads) : n_(std::max(1U, threads)) {
        for (unsigned t = 1; t < n_; ++t) workers_.emplace_back([this, t] { loop(t); });
    }
    ~Pool() {
        stop_.store(true);
        publish();
        for (auto &w : workers_) w.join();
    }
    Pool(const Pool &) = delete;
    Pool &operator=(const Pool &) = delete;
    [[nodiscard]] unsigned size() const { return n_; }

    // body(begin, end, participant) over [0, count) in chunks of `grain`
    // elements; the caller is participant 0.
    template <class F> void run(std::size_t count, std::size_t grain, F &&body) {
        if (count == 0) return;
        grain = std::max<std::size_t>(1, grain);
        const std::size_t chunks = (count + grain - 1) / grain;
        if (n_ == 1 || chunks < 2) {
            body(std::size_t{0}, count, 0U);
            return;
        }
        if (chunks > 0xffffffffULL) throw std::overflow_error("work pool: too many chunks");
        using Body = std::remove_reference_t<F>;
        fn_ = [](void *arg, std::size_t b, std::size_t e, unsigned t) { (*static_cast<Body *>(arg))(b, e, t); };
        arg_ = const_cast<void *>(static_cast<const void *>(&body));
        count_ = count;
        grain_ = grain;
        finished_.store(0, std::memory_order_relaxed);
        claim_.store(static_cast<std::uint64_t>(chunks) << 32, std::memory_order_release);
        publish();
        std::uint32_t mine = 0;
        for (;;) {
            const std::uint64_t word = claim_.fetch_add(1, std::memory_order_acq_rel);
            const std::uint32_t c = static_cast<std::uint32_t>(word);
            if (c >= chunks) break;
            const std::size_t b = static_cast<std::size_t>(c) * grain;
            body(b, std::min(count, b + grain), 0U);
            ++mine;
        }
        const std::uint32_t others = static_cast<std::uint32_t>(chunks) - mine;
        unsigned spins = 0;
        while (finished_.load(std::memory_order_acquire) != others)
            if (++spins % kSpinsBeforeYield == 0) std::this_thread::yield();
    }

private:
    static constexpr unsigned kSpinsBeforeYield = 4096;
    static constexpr auto kParkAfter = std::chrono::microseconds(500);

    // A new job (or the stop flag) for the workers; parked ones are woken.
    void publish() {
        seq_.fetch_add(1, std::memory_order_seq_cst);
        if (sleepers_.load(std::memory_order_seq_cst) != 0) {
            { std::lock_guard<std::mutex> g(park_m_); }
            park_cv_.notify_all();
        }
    }

    void loop(unsigned index) {
        std::uint64_t seen = seq_.load(std::memory_order_acquire);
        for (;;) {
            std::uint64_t now = seq_.load(std::memory_order_acquire);
            unsigned spins = 0;
            auto idle_since = std::chrono::steady_clock::now();
            while (now == seen) {
                if (++spins % kSpinsBeforeYield == 0) {
                    std::this_thread::yield();
                    if (std::chrono::steady_clock::now() - idle_since > kParkAfter) {
                        sleepers_.fetch_add(1, std::memory_order_seq_cst);
                        {
                            std::unique_lock<std::mutex> g(park_m_);
                            park_cv_.wait(g, [&] { return seq_.load(std::memory_order_seq_cst) != seen; });
                        }
                        sleepers_.fetch_sub(1, std::memory_order_seq_cst);
                        idle_since = std::chrono::steady_clock::now();
                    }
                }
                now = seq_.load(std::memory_order_acquire);
            }
            seen = now;
            if (stop_.load(std::memory_order_acquire)) return;
            std::uint32_t done = 0;
            for (;;) {
                const std::uint64_t word = claim_.fetch_add(1, std::memory_order_acq_rel);
                const std::uint32_t c = static_cast<std::uint32_t>(word);
                const std::uint32_t chunks = static_cast<std::uint32_t>(word >> 32);
                if (c >= chunks) break;
                const std::size_t b = static_cast<std::size_t>(c) * grain_;
                fn_(arg_, b, std::min(count_, b + grain_), index);
                ++done;
            }
            if (done) finished_.fetch_add(done, std::memory_order_release);
        }
    }

    unsigned n_;
    std::vector<std::thread> workers_;
    using Fn = void (*)(void *, std::size_t, std::size_t, unsigned);
    Fn fn_{nullptr};
    void *arg_{nullptr};
    std::size_t count_{0}, grain_{1};
    alignas(64) std::atomic<std::uint64_t> seq_{0};
    alignas(64) std::atomic<std::uint64_t> claim_{0};
    alignas(64) std::atomic<std::uint32_t> finished_{0};
    alignas(64) std::atomic<std::uint32_t> sleepers_{0};
    std::atomic<bool> stop_{false};
    std::mutex park_m_;
    std::condition_variable park_cv_;
};

// Grains per phase (elements per claimed chunk): about a microsecond of work
// each, as the reference sizes them (ParallelCpuLatticeBackend.cpp:1347-1356).
constexpr std::size_t kNodeGrain = 128;   // the cheap per-node phases
constexpr std::size_t kStrainGrain = 16;  // the nonlocal strain
constexpr std::size_t kBondGrain = 64;    // the per-bond samples
constexpr std::size_t kSolveGrain = 48;   // one colour stage of the sweep

// ---------------------------------------------------------------------------
// Node-to-node contact (LatticePhysics.hpp:1441-1647; the stage order is
// CpuLatticeBackend.cpp:424-436). Pairs of nodes that no live bond holds and
// that lie within 2 r + skin are listed per owner (the lower index) through a
// hashed grid of that cell size; the list is rebuilt before use when a bond
// failed in the previous substep or any node drifted more than skin / 2 since
// the last build. The narrow phase is one response per pair, in list order.
// ---------------------------------------------------------------------------
constexpr std::uint32_t kPairsPerNode = 24;

struct NodeAcc {
    std::uint64_t contacts{}, pair_tests{}, rebuilds{}, pairs_listed{}, pair_overflow{};
    double dissipated{}, max_overlap{}, max_correction{}, momentum[3]{};
};

// Teschner et al., "Optimized Spatial Hashing for Collision Detection of
// Deformable Objects" (2003): the three primes, exclusive-or, masked.
inline std::uint32_t cellBucket(std::int32_t x, std::int32_t y, std::int32_t z, std::uint32_t mask) {
    return ((static_cast<std::uint32_t>(x) * 73856093U) ^ (static_cast<std::uint32_t>(y) * 19349663U) ^
            (static_cast<std::uint32_t>(z) * 83492791U)) & mask;
}

template <class R> struct PairList {
    std::vector<std::int32_t> cell;        // 3 per node
    std::vector<R> built_u;                // u at the last build, 3 per node
    std::vector<std::uint32_t> bucket_at;  // bucket offsets (buckets + 1)
    std::vector<std::uint32_t> members;    // movable nodes by bucket, ascending within one
    std::vector<std::uint32_t> fill, other, bond, owners;
    bool rebuild{true};
};

template <class R> R contactCutoff(const Settings<R> &S) { return R(2) * S.nc_radius + S.nc_skin; }

// nodeContactStale: any node farther than skin / 2 from where the list was built.
template <class R> bool pairListStale(const Lattice<R> &L, const Settings<R> &S, const PairList<R> &P) {
    const R half = R(0.5) * S.nc_skin;
    const R limit = half * half;
    for (std::uint32_t i = 0; i < L.N; ++i) {
        const V<R> d = sub(ld(L.u, i), ld(P.built_u, i));
        if (dot(d, d) > limit) return true;
    }
    return false;
}

// The four broad-phase steps (cells, counting sort into the buckets, the
// per-owner gather, the owner list) in one pass each.
template <class R> void rebuildPairs(const Lattice<R> &L, const Settings<R> &S, PairList<R> &P, NodeAcc &acc) {
    const std::uint32_t N = L.N;
    P.cell.resize(3 * static_cast<std::size_t>(N));
    P.built_u.resize(3 * static_cast<std::size_t>(N));
    P.fill.assign(N, 0U);
    P.other.resize(kPairsPerNode * static_cast<std::size_t>(N));
    P.bond.resize(kPairsPerNode * static_cast<std::size_t>(N));
    const R cutoff = contactCutoff(S);
    const R inverse_cell = R(1) / cutoff;
    for (std::uint32_t i = 0; i < N; ++i) {
        const V<R> p = position(L, i);
        P.cell[3 * i] = static_cast<std::int32_t>(std::floor(p.x * inverse_cell));
        P.cell[3 * i + 1] = static_cast<std::int32_t>(std::floor(p.y * inverse_cell));
        P.cell[3 * i + 2] = static_cast<std::int32_t>(std::floor(p.z * inverse_cell));
        st(P.built_u, i, ld(L.u, i));
    }
    auto bucketOf = [&](std::uint32_t i) { return cellBucket(P.cell[3 * i], P.cell[3 * i + 1], P.cell[3 * i + 2], S.nc_mask); };
    const std::uint32_t buckets = S.nc_mask + 1U;
    P.bucket_at.assign(static_cast<std::size_t>(buckets) + 1, 0U);
    P.members.resize(N);
    for (std::uint32_t i = 0; i < N; ++i)
        if (!(L.mass[i] <= R(0))) ++P.bucket_at[bucketOf(i) + 1U];
    for (std::uint32_t b = 0; b < buckets; ++b) P.bucket_at[b + 1U] += P.bucket_at[b];
    std::vector<std::uint32_t> cursor(P.bucket_at.begin(), P.bucket_at.end() - 1);
    for (std::uint32_t i = 0; i < N; ++i)
        if (!(L.mass[i] <= R(0))) P.members[cursor[bucketOf(i)]++] = i;
    const R cutoff_sq = cutoff * cutoff;
    for (std::uint32_t i = 0; i < N; ++i) {
        if (L.mass[i] <= R(0)) continue;
        const V<R> p = position(L, i);
        const std::int32_t cx = P.cell[3 * i], cy = P.cell[3 * i + 1], cz = P.cell[3 * i + 2];
        std::uint32_t fill = 0;
        for (std::int32_t dz = -1; dz <= 1; ++dz)
            for (std::int32_t dy = -1; dy <= 1; ++dy)
                for (std::int32_t dx = -1; dx <= 1; ++dx) {
                    const std::int32_t gx = cx + dx, gy = cy + dy, gz = cz + dz;
                    const std::uint32_t b = cellBucket(gx, gy, gz, S.nc_mask);
                    for (std::uint32_t k = P.bucket_at[b]; k < P.bucket_at[b + 1U]; ++k) {
                        const std::uint32_t j = P.members[k];
                        if (j <= i || P.cell[3 * j] != gx || P.cell[3 * j + 1] != gy || P.cell[3 * j + 2] != gz) continue;
                        const V<R> r = sub(position(L, j), p);
                        if (dot(r, r) > cutoff_sq) continue;
                        // The pair's bond, if i lists one to j; a live one holds the pair.
                        std::uint32_t bond = kNoBond;
                        bool held = false;
                        for (std::uint32_t s = 0; s < L.D; ++s) {
                            const std::size_t slot = static_cast<std::size_t>(s) * N + i;
                            if (L.nbr_bond[slot] == kNoBond) break;
                            if (L.nbr_other[slot] != j) continue;
                            bond = L.nbr_bond[slot];
                            held = L.nbr_alive[slot] != 0;
                            break;
                        }
                        if (held) continue;
                        if (fill == kPairsPerNode) { ++acc.pair_overflow; continue; }
                        P.other[kPairsPerNode * static_cast<std::size_t>(i) + fill] = j;
                        P.bond[kPairsPerNode * static_cast<std::size_t>(i) + fill] = bond;
                        ++fill;
                    }
                }
        P.fill[i] = fill;
    }
    P.owners.clear();
    for (std::uint32_t i = 0; i < N; ++i)
        if (P.fill[i]) {
            P.owners.push_back(i);
            acc.pairs_listed += P.fill[i];
        }
    ++acc.rebuilds;
    P.rebuild = false;
}

// nodeContactPair: restitution-limited normal impulse, Coulomb friction and an
// overlap correction, each equal and opposite on the two nodes.
template <class R>
void contactPair(Lattice<R> &L, const Settings<R> &S, std::uint32_t a, std::uint32_t b, std::uint32_t bond, NodeAcc &acc) {
    if (bond != kNoBond && L.alive[bond]) return;
    const R ma = L.mass[a], mb = L.mass[b];
    if (ma <= R(0) || mb <= R(0)) return;
    ++acc.pair_tests;
    const V<R> r = sub(position(L, b), position(L, a));
    const R distance = len(r);
    const V<R> n = unit(r);
    const R gap = distance - R(2) * S.nc_radius;
    if (gap < R(0) && -gap > static_cast<R>(acc.max_overlap)) acc.max_overlap = static_cast<double>(-gap);
    if (S.nc_mode != 2) return;
    V<R> va = ld(L.v, a), vb = ld(L.v, b);
    const R vn = dot(sub(vb, va), n);
    if (gap > maxR(S.nc_margin, -vn * S.dt)) return;
    const R ia = R(1) / ma, ib = R(1) / mb;
    const R pair_inverse = ia + ib;
    const R restitution = -vn > S.nc_threshold ? S.nc_restitution : R(0);
    const R desired = gap > S.nc_margin ? -gap / S.dt : -restitution * minR(vn, R(0));
    const R impulse = maxR(R(0), (desired - vn) / pair_inverse);
    if (impulse > R(0)) {
        const V<R> va0 = va, vb0 = vb;
        const R before = R(0.5) * ma * dot(va, va) + R(0.5) * mb * dot(vb, vb);
        auto apply = [&](V<R> j) {
            vb = add(vb, scale(j, ib));
            va = sub(va, scale(j, ia));
        };
        apply(scale(n, impulse));
        const V<R> rel = sub(vb, va);
        const V<R> t = sub(rel, scale(n, dot(rel, n)));
        const R speed = len(t);
        if (speed > R(1.0e-12)) {
            const V<R> dir = divide(t, speed);
            const R stick = speed / pair_inverse;
            const R friction = stick <= S.nc_static * impulse ? stick : minR(stick, S.nc_dynamic * impulse);
            apply(scale(dir, -friction));
        }
        st(L.v, a, va);
        st(L.v, b, vb);
        acc.dissipated += static_cast<double>(before - (R(0.5) * ma * dot(va, va) + R(0.5) * mb * dot(vb, vb)));
        acc.momentum[0] += static_cast<double>(ma * (va.x - va0.x) + mb * (vb.x - vb0.x));
        acc.momentum[1] += static_cast<double>(ma * (va.y - va0.y) + mb * (vb.y - vb0.y));
        acc.momentum[2] += static_cast<double>(ma * (va.z - va0.z) + mb * (vb.z - vb0.z));
        ++acc.contacts;
    }
    if (gap < -S.nc_margin) {
        const R correction = minR(-gap - S.nc_margin, R(0.2) * S.nc_radius);
        const V<R> shift = scale(n, correction / pair_inverse);
        st(L.u, a, sub(ld(L.u, a), scale(shift, ia)));
        st(L.u, b, add(ld(L.u, b), scale(shift, ib)));
        if (correction > static_cast<R>(acc.max_correction)) acc.max_correction = static_cast<double>(correction);
    }
}

// nodeContactPass: owners ascending, then slots ascending.
template <class R> void contactPass(Lattice<R> &L, const Settings<R> &S, const PairList<R> &P, NodeAcc &acc) {
    for (const std::uint32_t a : P.owners)
        for (std::uint32_t k = 0; k < P.fill[a]; ++k) {
            const std::size_t slot = kPairsPerNode * static_cast<std::size_t>(a) + k;
            contactPair(L, S, a, P.other[slot], P.bond[slot], acc);
        }
}

struct Status {
    std::uint64_t total_steps{}, first_failure_step{kNever}, last_failure_step{kNever}, last_energy_gain_step{kNever},
        last_damage_gain_step{};
    std::uint32_t failure_rounds{}, broken_bonds{}, rank_deficient_nodes{};
    double removed_energy{}, max_damage{}, plastic_work{};
    float max_t{}, max_c{}, max_s{}, max_plastic_stretch{};
    unsigned exit_reason{}, launches{};
    ContactAcc contact{};
    double ext_work{}, ext_impulse[3]{};
    std::uint64_t ext_steps{};
    NodeAcc node{};
    double damping_dissipated{}, striker_dissipated{};
    bool energy_audited{};
    // Bond projections the sweeps ran: per substep, the bonds alive when its
    // sweep starts times the solver iterations. Not a reference counter: the
    // throughput measure both lanes report alike.
    std::uint64_t bond_projections{};
    // Non-zero addends folded into plastic_work: with the removed-energy
    // addends (one per broken bond) it bounds how far another summation
    // order of these non-negative terms can land, 2 n 2^-53 relative.
    std::uint64_t plastic_increments{};
};

// Double vector arithmetic of the load phase (core/Math.hpp:17-69).
struct D3 { double x, y, z; };
inline D3 operator+(D3 a, D3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline D3 operator-(D3 a, D3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline D3 operator*(double s, D3 a) { return {a.x * s, a.y * s, a.z * s}; }
inline double dotD(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline D3 crossD(D3 a, D3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline double normD(D3 a) { return std::hypot(a.x, a.y, a.z); }
inline bool finiteD(D3 a) { return std::isfinite(a.x) && std::isfinite(a.y) && std::isfinite(a.z); }

// An external wrench (FastLattice.hpp:153-157) and a source's load ledger
// (FastLattice.hpp:140-161).
struct Wrench { std::string source; std::vector<std::uint32_t> nodes; D3 point, force, torque; };
struct LoadLedger { double steps{}, elapsed{}; D3 req_imp{}, imp{}, req_ang{}, ang{}; double work{}; };
struct SourceLedger { std::string source; LoadLedger load; };

// External forces and wrenches (ExternalLoads.hpp:28-77 set/setWrenches,
// 79-148 kick, 171-238 wrenchNodes). Forces keep the run ledger's work,
// impulse and step count; wrench sources keep their own full ledgers.
template <class R> struct Loads {
    static constexpr std::size_t kNoSource = ~std::size_t(0);
    struct Node { std::uint32_t index; double req[3]; V<R> applied; std::size_t source = kNoSource; };
    std::vector<Node> nodes;
    std::vector<Wrench> wrenches;
    std::vector<SourceLedger> sources; // RunStatus::external_sources, in first-kick order
    std::uint64_t remaining{};
    double origin[3]{};

    D3 where(const Lattice<R> &L, std::uint32_t i) const {
        const V<R> p = add(ld(L.x0, i), ld(L.u, i));
        return D3{origin[0], origin[1], origin[2]} + D3{double(p.x), double(p.y), double(p.z)};
    }

    // A wrench's force and torque over its nodes by mass, about their mass
    // centre at the current positions (ExternalLoads.hpp:171-238).
    std::vector<Node> wrenchNodes(const std::vector<Wrench> &ws, const Lattice<R> &L) const {
        std::vector<Node> out;
        for (std::size_t k = 0; k < ws.size(); ++k) {
            const Wrench &w = ws[k];
            double mass = 0;
            std::vector<D3> points;
            const V<R> a0 = add(ld(L.x0, w.nodes.front()), ld(L.u, w.nodes.front()));
            const D3 anchor{double(a0.x), double(a0.y), double(a0.z)};
            for (const auto node : w.nodes) {
                if (!(L.mass[node] > 0) || !(L.inv_mass[node] > 0) || !std::isfinite(L.mass[node]) ||
                    !std::isfinite(L.inv_mass[node]))
                    throw std::invalid_argument("external wrench needs finite movable node masses");
                const V<R> p = add(ld(L.x0, node), ld(L.u, node));
                const D3 relative = D3{double(p.x), double(p.y), double(p.z)} - anchor;
                if (!finiteD(relative)) throw std::invalid_argument("external wrench node position is not finite");
                points.push_back(relative);
                mass += static_cast<double>(L.mass[node]);
            }
            if (!(mass > 0) || !std::isfinite(mass)) throw std::invalid_argument("external wrench mass overflow");
            D3 center{0, 0, 0};
            for (std::size_t i = 0; i < points.size(); ++i)
                center = center + (static_cast<double>(L.mass[w.nodes[i]]) / mass) * points[i];
            double tensor[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
            for (std::size_t i = 0; i < points.size(); ++i) {
                points[i] = points[i] - center;
                const double r[3] = {points[i].x, points[i].y, points[i].z};
                const double share = static_cast<double>(L.mass[w.nodes[i]]) / mass;
                for (unsigned a = 0; a < 3; ++a)
                    for (unsigned b = 0; b < 3; ++b)
                        tensor[3 * a + b] += share * (a == b ? r[(a + 1) % 3] * r[(a + 1) % 3] + r[(a + 2) % 3] * r[(a + 2) % 3]
                                                             : -r[a] * r[b]);
            }
            const D3 moment = w.torque + crossD(((w.point - D3{origin[0], origin[1], origin[2]}) - anchor) - center, w.force);
            if (!finiteD(center) || !finiteD(moment)) throw std::invalid_argument("external wrench moment overflow");
            double scale = 0;
            for (const double e : tensor) {
                if (!std::isfinite(e)) throw std::invalid_argument("external wrench inertia overflow");
                scale = std::max(scale, std::abs(e));
            }
            D3 alpha{0, 0, 0};
            if (scale > 0) {
                for (double &e : tensor) e /= scale;
                double eig[3], axes[9];
                eigen3(tensor, eig, axes);
                const double largest = std::max({std::abs(eig[0]), std::abs(eig[1]), std::abs(eig[2])});
                D3 unresolved = moment;
                for (unsigned axis = 0; axis < 3; ++axis) {
                    if (!(eig[axis] > 1e-10 * largest)) continue;
                    const D3 dir{axes[axis], axes[3 + axis], axes[6 + axis]};
                    const double component = dotD(dir, moment);
                    unresolved = unresolved - component * dir;
                    alpha = alpha + (component / mass / scale / eig[axis]) * dir;
                }
                if (normD(unresolved) > 1024 * std::numeric_limits<double>::epsilon() * normD(moment))
                    throw std::invalid_argument("external wrench torque is not represented by these nodes");
            } else if (normD(moment) > 0) {
                throw std::invalid_argument("external wrench torque needs a sampled lever arm");
            }
            if (!finiteD(alpha)) throw std::invalid_argument("external wrench acceleration overflow");
            D3 force_sum{0, 0, 0}, moment_sum{0, 0, 0};
            double absolute_force = 0, absolute_moment = 0;
            for (std::size_t i = 0; i < points.size(); ++i) {
                const double m = static_cast<double>(L.mass[w.nodes[i]]);
                const D3 f = (m / mass) * w.force + m * crossD(alpha, points[i]);
                const V<R> conv{static_cast<R>(f.x), static_cast<R>(f.y), static_cast<R>(f.z)};
                if (!finiteD(f) || !std::isfinite(conv.x) || !std::isfinite(conv.y) || !std::isfinite(conv.z))
                    throw std::invalid_argument("external wrench node force exceeds backend precision");
                out.push_back({w.nodes[i], {f.x, f.y, f.z}, conv, k});
                force_sum = force_sum + f;
                moment_sum = moment_sum + crossD(points[i], f);
                absolute_force += normD(f);
                absolute_moment += normD(crossD(points[i], f));
            }
            if (!finiteD(force_sum) || !finiteD(moment_sum) || !std::isfinite(absolute_force) ||
                !std::isfinite(absolute_moment) ||
                normD(force_sum - w.force) > 1e-10 * std::max(normD(w.force), absolute_force) ||
                normD(moment_sum - moment) > 1e-10 * std::max(normD(moment), absolute_moment))
                throw std::invalid_argument("external wrench resultant cannot be represented accurately");
        }
        return out;
    }

    void setWrenches(const std::vector<Wrench> &ws, std::uint64_t substeps, const Lattice<R> &L) {
        if (ws.empty()) {
            if (substeps != 0) throw std::invalid_argument("empty external load needs zero substeps");
            nodes.clear(); wrenches.clear(); remaining = 0; return;
        }
        if (!substeps) throw std::invalid_argument("external wrench needs a finite nonzero span");
        std::vector<Wrench> staged = ws;
        std::set<std::string> names;
        std::set<std::uint32_t> used;
        for (Wrench &w : staged) {
            if (w.source.empty() || !names.insert(w.source).second || w.nodes.empty())
                throw std::invalid_argument("external wrench needs distinct named nonempty regions");
            if (!finiteD(w.point) || !finiteD(w.force) || !finiteD(w.torque) || !std::isfinite(normD(w.force)) ||
                !std::isfinite(normD(w.torque)))
                throw std::invalid_argument("external wrench must be finite");
            std::sort(w.nodes.begin(), w.nodes.end());
            for (const auto node : w.nodes)
                if (node >= L.N || !used.insert(node).second)
                    throw std::invalid_argument("external wrench nodes repeat, overlap or exceed the lattice");
        }
        std::sort(staged.begin(), staged.end(), [](const Wrench &a, const Wrench &b) { return a.source < b.source; });
        staged.erase(std::remove_if(staged.begin(), staged.end(), [](const Wrench &w) {
            return w.force.x == 0 && w.force.y == 0 && w.force.z == 0 && w.torque.x == 0 && w.torque.y == 0 &&
                   w.torque.z == 0;
        }), staged.end());
        auto staged_nodes = wrenchNodes(staged, L);
        nodes = std::move(staged_nodes);
        wrenches = std::move(staged);
        remaining = nodes.empty() ? 0 : substeps;
    }

    void set(const std::vector<double> &f, std::uint64_t substeps, const Lattice<R> &L) {
        wrenches.clear();
        if (f.empty()) { nodes.clear(); remaining = 0; return; }
        if (f.size() != 3 * static_cast<std::size_t>(L.N) || substeps == 0)
            throw std::invalid_argument("external load needs one force per node and a finite nonzero span");
        std::vector<Node> staged;
        for (std::uint32_t i = 0; i < L.N; ++i) {
            const double fx = f[3 * i], fy = f[3 * i + 1], fz = f[3 * i + 2];
            const V<R> conv{static_cast<R>(fx), static_cast<R>(fy), static_cast<R>(fz)};
            if (!std::isfinite(fx) || !std::isfinite(fy) || !std::isfinite(fz) || !std::isfinite(std::hypot(fx, fy, fz)) ||
                !std::isfinite(conv.x) || !std::isfinite(conv.y) || !std::isfinite(conv.z))
                throw std::invalid_argument("external force is not finite in backend precision");
            if (fx == 0 && fy == 0 && fz == 0) continue;
            if (!(L.mass[i] > 0) || !(L.inv_mass[i] > 0) || !std::isfinite(L.mass[i]) || !std::isfinite(L.inv_mass[i]))
                throw std::invalid_argument("external force needs a finite positive movable node mass");
            staged.push_back({i, {fx, fy, fz}, conv});
        }
        nodes = std::move(staged);
        remaining = nodes.empty() ? 0 : substeps;
    }
    void kick(Lattice<R> &L, R dt, Status &st_) {
        if (!remaining) return;
        if (!wrenches.empty()) nodes = wrenchNodes(wrenches, L); // the current geometry
        double work = 0, imp[3] = {0, 0, 0};
        const double dtd = static_cast<double>(dt);
        std::vector<LoadLedger> change(wrenches.size());
        for (auto &c : change) { c.steps = 1; c.elapsed = dtd; }
        std::vector<V<R>> after(nodes.size());
        for (std::size_t k = 0; k < nodes.size(); ++k) {
            const Node &n = nodes[k];
            const V<R> before = ld(L.v, n.index);
            after[k] = add(before, scale(n.applied, dt * L.inv_mass[n.index]));
            if (!std::isfinite(after[k].x) || !std::isfinite(after[k].y) || !std::isfinite(after[k].z))
                throw std::overflow_error("external force kick exceeds backend precision");
            const double old[3] = {static_cast<double>(before.x), static_cast<double>(before.y), static_cast<double>(before.z)};
            const double nxt[3] = {static_cast<double>(after[k].x), static_cast<double>(after[k].y), static_cast<double>(after[k].z)};
            const double m = static_cast<double>(L.mass[n.index]);
            double ii[3];
            for (int q = 0; q < 3; ++q) ii[q] = m * (nxt[q] - old[q]);
            for (int q = 0; q < 3; ++q) imp[q] += ii[q];
            const double wk = ii[0] * (.5 * (old[0] + nxt[0])) + ii[1] * (.5 * (old[1] + nxt[1])) + ii[2] * (.5 * (old[2] + nxt[2]));
            work += wk;
            if (n.source != kNoSource) {
                LoadLedger &c = change[n.source];
                const D3 at = where(L, n.index);
                const D3 rq = dtd * D3{n.req[0], n.req[1], n.req[2]};
                const D3 im{ii[0], ii[1], ii[2]};
                c.req_imp = c.req_imp + rq;
                c.req_ang = c.req_ang + crossD(at, rq);
                c.imp = c.imp + im;
                c.ang = c.ang + crossD(at, im);
                c.work += wk;
            }
        }
        for (std::size_t k = 0; k < wrenches.size(); ++k) {
            auto found = std::find_if(sources.begin(), sources.end(),
                                      [&](const SourceLedger &s) { return s.source == wrenches[k].source; });
            if (found == sources.end()) {
                sources.push_back({wrenches[k].source, LoadLedger{}});
                found = sources.end() - 1;
            }
            LoadLedger &t = found->load;
            const LoadLedger &c = change[k];
            t.steps = t.steps + c.steps; t.elapsed = t.elapsed + c.elapsed;
            t.req_imp = t.req_imp + c.req_imp; t.imp = t.imp + c.imp;
            t.req_ang = t.req_ang + c.req_ang; t.ang = t.ang + c.ang;
            t.work = t.work + c.work;
        }
        for (std::size_t k = 0; k < nodes.size(); ++k) st(L.v, nodes[k].index, after[k]);
        st_.ext_steps += 1;
        for (int q = 0; q < 3; ++q) st_.ext_impulse[q] = st_.ext_impulse[q] + imp[q];
        st_.ext_work = st_.ext_work + work;
        --remaining;
    }
};

// The lattice's kinetic energy, folded serially in node order with each term
// formed in backend precision and widened (LatticePhysics.hpp:1676-1682): the
// energy audit's measure.
template <class R> double kineticEnergy(const Lattice<R> &L) {
    double total = 0.0;
    for (std::uint32_t i = 0; i < L.N; ++i) {
        const V<R> v = ld(L.v, i);
        total += static_cast<double>(R(0.5) * L.mass[i] * dot(v, v));
    }
    return total;
}

template <class R> class Runner {
public:
    Runner(Lattice<R> &L, const Settings<R> &S, Sphere<R> sp, unsigned threads) : L_(L), S_(S), sp_(sp), pool_(threads) {
        if (S_.nc_mode != 0 && !(contactCutoff(S_) > R(0))) throw std::invalid_argument("node contact needs 2 r + skin > 0");
        status.energy_audited = S_.audit != 0; // CpuLatticeBackend.cpp:114
        kept_ = keepSolveConstants(L_, S_.dt);
        live_upload_ = countAlive();
    }
    Status status;
    Loads<R> loads;
    std::vector<std::uint32_t> first_failure_bonds;
    std::vector<double> substep_seconds; // wall time of every substep run
    std::vector<std::uint64_t> substep_projections; // bond projections of every substep run
    // The phase-diff mode: called at the end of each phase of a substep with
    // the phase's number (latticePhaseName's, FastLattice.cpp:15-28).
    std::function<void(unsigned)> phase_hook;
    double energy_flat_fraction{1.0e-3};

    // CpuLatticeBackend.cpp:255-304 for one RunControl with exit rules off.
    void run(std::uint64_t max_steps) {
        status.exit_reason = 0;
        std::uint64_t done = 0;
        while (done < max_steps) {
            const std::uint64_t step = status.total_steps;
            const auto t0 = std::chrono::steady_clock::now();
            const bool failed = advance();
            substep_seconds.push_back(std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count());
            status.total_steps = step + 1;
            ++done;
            if (failed) {
                if (status.first_failure_step == kNever) status.first_failure_step = step;
                status.last_failure_step = step;
                ++status.failure_rounds;
            }
            status.exit_reason = exitReason(status.total_steps, status.broken_bonds, status.last_failure_step, 0, 0, 0, 0,
                                            status.last_energy_gain_step, 0, status.last_damage_gain_step,
                                            status.max_damage, 0.5, status.removed_energy, 0.0);
            if (status.exit_reason != 0) break;
        }
        if (status.exit_reason == 0 && done >= max_steps) status.exit_reason = 3;
        ++status.launches;
    }

private:
    template <class F> void nodes(F &&f) {
        pool_.run(L_.N, kNodeGrain, [&](std::size_t b, std::size_t e, unsigned) { for (std::size_t i = b; i < e; ++i) f(i); });
    }
    template <class F> void range(std::uint32_t b0, std::uint32_t e0, F &&f) {
        pool_.run(e0 - b0, kSolveGrain,
                  [&](std::size_t b, std::size_t e, unsigned) { for (std::size_t j = b; j < e; ++j) f(b0 + j); });
    }
    // The sweep order of CpuLatticeBackend.cpp:336-348, 395-407.
    template <class F> void sweepBlock(std::uint32_t block, std::uint32_t boundary, F &&f) {
        for (std::uint32_t c = 0; c < L_.C; ++c) {
            const std::size_t key = (static_cast<std::size_t>(block) * 2 + boundary) * L_.C + c;
            range(L_.range_begin[key], L_.range_end[key], f);
        }
    }
    template <class F> void sweepAll(F &&f) {
        for (std::uint32_t b = 0; b < L_.blocks; ++b) sweepBlock(b, 0, f);
        for (std::uint32_t b = 0; b < L_.blocks; b += 2) sweepBlock(b, 1, f);
        for (std::uint32_t b = 1; b < L_.blocks; b += 2) sweepBlock(b, 1, f);
    }
    void strainAll(bool direct) {
        std::vector<std::uint32_t> rd(pool_.size(), 0);
        pool_.run(L_.N, kStrainGrain, [&](std::size_t b, std::size_t e, unsigned t) {
            for (std::size_t i = b; i < e; ++i)
                nodeStrain(L_, i, direct, rd[t], S_.plate_half_thickness, S_.yield_stretch);
        });
        for (auto x : rd) status.rank_deficient_nodes += x;
    }

    // The start-of-substep sample after a failure, or after upload
    // (CpuLatticeBackend.cpp:363-370). The serial lane redoes every node's
    // strain and every live bond's start sample; only the nodes flagged dirty
    // (they lost a bond; every node after upload) can come out different --
    // every other node reads the positions and live neighbours it read at the
    // end of the previous substep, and a bond's end sample left exactly what
    // its start sample writes -- so those nodes and the live bonds at them are
    // redone, as the reference's threaded lane does
    // (ParallelCpuLatticeBackend.cpp:1718-1757).
    void restart(bool direct) {
        dirty_list_.clear();
        for (std::uint32_t i = 0; i < L_.N; ++i)
            if (L_.node_dirty[i]) dirty_list_.push_back(i);
        std::vector<std::uint32_t> rd(pool_.size(), 0);
        pool_.run(dirty_list_.size(), kStrainGrain, [&](std::size_t b, std::size_t e, unsigned t) {
            for (std::size_t k = b; k < e; ++k)
                nodeStrain(L_, dirty_list_[k], direct, rd[t], S_.plate_half_thickness, S_.yield_stretch);
        });
        for (auto x : rd) status.rank_deficient_nodes += x;
        if (bond_mark_.size() != L_.B) bond_mark_.assign(L_.B, 0U);
        touched_.clear();
        for (const std::uint32_t i : dirty_list_)
            for (std::uint32_t k = 0; k < L_.D; ++k) {
                const std::uint32_t j = L_.nbr_bond[static_cast<std::size_t>(k) * L_.N + i];
                if (j == kNoBond) break;
                if (!L_.alive[j] || bond_mark_[j]) continue;
                bond_mark_[j] = 1;
                touched_.push_back(j);
            }
        for (const std::uint32_t j : touched_) bond_mark_[j] = 0;
        pool_.run(touched_.size(), kBondGrain, [&](std::size_t b, std::size_t e, unsigned) {
            for (std::size_t k = b; k < e; ++k) startSample(L_, touched_[k], direct);
        });
    }

    // CpuLatticeBackend.cpp:357-439.
    bool advance() {
        const bool direct = S_.direct != 0;
        if (dirty_start_) {
            restart(direct);
            dirty_start_ = false;
        }
        loads.kick(L_, S_.dt, status);
        Sphere<R> kicked = sp_;
        kicked.velocity = add(kicked.velocity, scale(S_.gravity, S_.dt));
        nodes([&](std::size_t i) {
            V<R> vel = add(ld(L_.v, i), scale(S_.gravity, S_.dt));
            st(L_.v, i, vel);
            st(L_.u_prev, i, ld(L_.u, i));
            for (unsigned p = 0; p < kPlanes; ++p) L_.engaged[p * L_.N + i] = 0;
            const bool cand = S_.sphere_enabled && sphereCandidate(L_, S_, kicked, i);
            L_.candidate[i] = cand ? 1 : 0;
            if (!cand) {
                recordApproach(L_, S_, i);
                st(L_.u, i, add(ld(L_.u, i), scale(vel, S_.dt)));
            }
        });
        for (std::uint32_t b = 0; b < L_.blocks; ++b) {
            std::uint32_t count = 0;
            for (std::uint32_t i = L_.node_block_begin[b]; i < L_.node_block_begin[b + 1]; ++i) {
                if (!L_.candidate[i]) continue;
                if (count < kCandidatesPerBlock) L_.candidate_list[b * kCandidatesPerBlock + count] = i;
                else ++status.contact.candidate_overflow;
                ++count;
            }
            L_.candidate_count[b] = std::min(count, kCandidatesPerBlock);
        }
        sp_ = kicked;
        phase(3);
        if (S_.sphere_enabled) {
            const double before = S_.audit ? kineticEnergy(L_) : 0.0;
            spherePass(L_, S_, sp_, 1, status.contact);
            if (S_.audit) status.striker_dissipated += before - kineticEnergy(L_);
        }
        phase(4);
        const std::uint64_t swept = (live_upload_ - status.broken_bonds) * S_.iterations;
        status.bond_projections += swept;
        substep_projections.push_back(swept);
        for (std::uint32_t it = 0; it < S_.iterations; ++it) {
            const bool first = it == 0;
            auto solve = [&](std::size_t j) { solveBond(L_, kept_, j, direct, first); };
            sweepAll(solve);
            nodes([&](std::size_t i) { nodeSupportProject(L_, S_, i); });
        }
        phase(7);
        nodes([&](std::size_t i) {
            const V<R> vel = divide(sub(ld(L_.u, i), ld(L_.u_prev, i)), S_.dt);
            st(L_.v, i, vel);
            if (S_.damping_fraction <= R(0) && !L_.candidate[i]) nodeSupportVelocity(L_, S_, i);
        });
        phase(8);
        if (S_.damping_fraction > R(0)) {
            const double before = S_.audit ? kineticEnergy(L_) : 0.0;
            sweepAll([&](std::size_t j) { dampBond(L_, j, S_.damping_fraction, direct); });
            if (S_.audit) status.damping_dissipated += before - kineticEnergy(L_);
            nodes([&](std::size_t i) { if (!L_.candidate[i]) nodeSupportVelocity(L_, S_, i); });
            phase(9);
        }
        if (S_.sphere_enabled) {
            const double before = S_.audit ? kineticEnergy(L_) : 0.0;
            spherePass(L_, S_, sp_, 2, status.contact);
            if (S_.audit) status.striker_dissipated += before - kineticEnergy(L_);
        }
        phase(10);
        if (S_.nc_mode != 0) {
            if (pairs_.rebuild || pairListStale(L_, S_, pairs_)) rebuildPairs(L_, S_, pairs_, status.node);
            contactPass(L_, S_, pairs_, status.node);
            phase(15);
        }
        const bool failed = finishStep(direct);
        phase(13);
        return failed;
    }

    // CpuLatticeBackend.cpp:441-488. The bond loop runs in chunks on the pool;
    // the events each participant gathers are sorted by bond index and the
    // ledger folded in that order, which is the serial order (the reference's
    // threaded lane does the same, ParallelCpuLatticeBackend.cpp:1885-1910).
    bool finishStep(bool direct) {
        strainAll(direct);
        phase(11);
        const unsigned T = pool_.size();
        struct Event { std::uint32_t j; double removed, plastic; float damage; bool broke; };
        // One tally per participant, each on its own cache lines; a chunk
        // folds its peaks locally and merges them once.
        struct alignas(64) Tally {
            std::vector<Event> events;
            float t{0.0F}, c{0.0F}, s{0.0F}, p{0.0F};
            bool seen{false};
        };
        std::vector<Tally> tally(T);
        const double damage_floor = status.max_damage + 1.0e-6;
        pool_.run(L_.B, kBondGrain, [&](std::size_t b, std::size_t e, unsigned t) {
            Tally &my = tally[t];
            float lt = 0.0F, lc = 0.0F, ls = 0.0F, lp = 0.0F;
            bool seen = false;
            for (std::size_t j = b; j < e; ++j) {
                if (!L_.alive[j]) continue;
                const Outcome o = endSample(L_, S_, j, direct);
                if (!seen) { lt = o.peak_t; lc = o.peak_c; ls = o.peak_s; lp = o.plastic_stretch; seen = true; }
                lt = std::max(lt, o.peak_t); lc = std::max(lc, o.peak_c);
                ls = std::max(ls, o.peak_s); lp = std::max(lp, o.plastic_stretch);
                if (o.broke || o.plastic != 0.0 || o.damage > damage_floor)
                    my.events.push_back({static_cast<std::uint32_t>(j), o.removed, o.plastic, o.damage, o.broke});
            }
            if (!seen) return;
            if (!my.seen) { my.t = lt; my.c = lc; my.s = ls; my.p = lp; my.seen = true; }
            my.t = std::max(my.t, lt); my.c = std::max(my.c, lc); my.s = std::max(my.s, ls); my.p = std::max(my.p, lp);
        });
        for (unsigned t = 0; t < T; ++t) {
            if (!tally[t].seen) continue;
            status.max_t = std::max(status.max_t, tally[t].t); status.max_c = std::max(status.max_c, tally[t].c);
            status.max_s = std::max(status.max_s, tally[t].s);
            status.max_plastic_stretch = std::max(status.max_plastic_stretch, tally[t].p);
        }
        phase(12);
        std::vector<Event> ordered;
        for (unsigned t = 0; t < T; ++t) ordered.insert(ordered.end(), tally[t].events.begin(), tally[t].events.end());
        std::sort(ordered.begin(), ordered.end(), [](const Event &x, const Event &y) { return x.j < y.j; });
        bool any = false;
        const bool first_round = status.broken_bonds == 0;
        for (const Event &ev : ordered) {
            status.plastic_work += ev.plastic;
            status.plastic_increments += ev.plastic != 0.0;
            if (ev.damage > status.max_damage + 1.0e-6) {
                status.max_damage = ev.damage;
                status.last_damage_gain_step = status.total_steps;
            }
            if (!ev.broke) continue;
            any = true;
            if (first_round) first_failure_bonds.push_back(ev.j);
            status.removed_energy += ev.removed;
            if (ev.removed > energy_flat_fraction * std::max(status.removed_energy, 1.0e-12))
                status.last_energy_gain_step = status.total_steps;
            ++status.broken_bonds;
            L_.node_dirty[L_.bond_a[ev.j]] = 1;
            L_.node_dirty[L_.bond_b[ev.j]] = 1;
        }
        sp_.center = add(sp_.center, scale(sp_.velocity, S_.dt));
        sphereSupport(S_, sp_, status.contact);
        // A failure changes which pairs no live bond holds.
        if (any) dirty_start_ = pairs_.rebuild = true;
        return any;
    }

public:
    Sphere<R> sphere() const { return sp_; }
    void phase(unsigned p) {
        if (phase_hook) phase_hook(p);
    }

    // upload of the state a download wrote (LatticeWorking.hpp:53-124 on the
    // arrays LatticeWorking.hpp:126-142 writes back): positions, velocities
    // and bond state are the current ones, the neighbour slots' aliveness is
    // the state's as first built (download does not write it), every derived
    // array starts afresh, and so do the status, the loads, the first-failure
    // record and the pair list (CpuLatticeBackend.cpp:67-118).
    void reupload(const std::vector<std::uint8_t> &nbr_alive_built) {
        L_.nbr_alive = nbr_alive_built;
        std::fill(L_.rinv.begin(), L_.rinv.end(), R(0));
        std::fill(L_.unmeasured.begin(), L_.unmeasured.end(), R(0));
        std::fill(L_.strain.begin(), L_.strain.end(), R(0));
        std::fill(L_.approach.begin(), L_.approach.end(), R(0));
        std::fill(L_.node_valid.begin(), L_.node_valid.end(), 0);
        std::fill(L_.node_dirty.begin(), L_.node_dirty.end(), 1);
        std::fill(L_.engaged.begin(), L_.engaged.end(), 0);
        std::fill(L_.candidate.begin(), L_.candidate.end(), 0);
        std::fill(L_.lambda.begin(), L_.lambda.end(), R(0));
        std::fill(L_.candidate_list.begin(), L_.candidate_list.end(), 0U);
        std::fill(L_.candidate_count.begin(), L_.candidate_count.end(), 0U);
        status = Status{};
        status.energy_audited = S_.audit != 0;
        live_upload_ = countAlive();
        loads.nodes.clear();
        loads.wrenches.clear();
        loads.sources.clear();
        loads.remaining = 0;
        first_failure_bonds.clear();
        dirty_start_ = true;
        pairs_ = PairList<R>{};
    }

private:
    Lattice<R> &L_;
    Settings<R> S_;
    Sphere<R> sp_;
    Pool pool_;
    bool dirty_start_{true};
    PairList<R> pairs_;
    Kept<R> kept_;
    std::vector<std::uint32_t> dirty_list_, touched_;
    std::vector<std::uint8_t> bond_mark_;
    std::uint64_t live_upload_{}; // bonds alive at upload

    std::uint64_t countAlive() const {
        std::uint64_t n = 0;
        for (const std::uint8_t a : L_.alive) n += a != 0;
        return n;
    }
};

template <class R> std::vector<double> widen(const std::vector<R> &v) {
    return std::vector<double>(v.begin(), v.end());
}

// The wrenches of a case file (case_layout.hpp).
inline std::vector<Wrench> unpackWrenches(const lsio::Case &c) {
    const auto names = c.get<std::uint8_t>("wrench_names");
    const auto counts = c.get<std::uint32_t>("wrench_node_count");
    const auto nodes = c.get<std::uint32_t>("wrench_nodes");
    const auto vec = c.get<double>("wrench_vectors");
    std::vector<Wrench> out(counts.size());
    std::size_t at = 0, node = 0;
    for (std::size_t k = 0; k < out.size(); ++k) {
        Wrench &w = out[k];
        while (at < names.size() && names[at] != 0) w.source.push_back(static_cast<char>(names[at++]));
        ++at;
        w.nodes.assign(nodes.begin() + static_cast<std::ptrdiff_t>(node),
                       nodes.begin() + static_cast<std::ptrdiff_t>(node + counts[k]));
        node += counts[k];
        const double *v = vec.data() + lsio::kWrenchWidth * k;
        w.point = {v[0], v[1], v[2]};
        w.force = {v[3], v[4], v[5]};
        w.torque = {v[6], v[7], v[8]};
    }
    return out;
}

template <class R> void runCase(const lsio::Case &c, lsio::Case &out, unsigned threads, bool per_substep) {
    const auto N = c.scalar<std::uint32_t>("node_count");
    const Schedule s = buildSchedule(N, c.get<std::uint32_t>("bond_a"), c.get<std::uint32_t>("bond_b"),
                                     c.get<std::uint32_t>("node_block_begin"));
    out.put("sched_bond_order", s.bond_order);
    out.put("sched_color", s.bond_color);
    out.put("sched_range_begin", s.range_begin);
    out.put("sched_range_end", s.range_end);
    out.put("sched_bond_block_begin", s.bond_block_begin);
    out.putScalar<std::uint32_t>("sched_color_count", s.color_count);
    out.putScalar<std::uint32_t>("sched_boundary_bond_count", s.boundary_bond_count);
    Lattice<R> L = buildLattice<R>(c, s);
    out.put("state_nbr_other", L.nbr_other);
    out.putScalar<std::uint32_t>("state_max_degree", L.D);
    Settings<R> S = unpackSettings<R>(c.get<double>("settings"));
    if (std::is_same<R, double>::value) S.direct = 1;
    Runner<R> run(L, S, unpackSphere<R>(c.get<double>("sphere")), threads);
    const std::uint64_t steps = c.scalar<std::uint64_t>("steps");
    const std::uint64_t per_step = c.scalarOr<std::uint64_t>("substeps_per_step", 1);
    const bool ramp = c.has("force_ramp_steps");
    std::vector<double> base;
    if (c.has("origin")) {
        const auto o = c.get<double>("origin");
        for (int q = 0; q < 3; ++q) run.loads.origin[q] = o[q];
    }
    if (c.has("forces")) {
        base = c.get<double>("forces");
        if (!ramp) run.loads.set(base, c.scalar<std::uint64_t>("force_substeps"), L);
    }
    if (c.has("wrench_names")) run.loads.setWrenches(unpackWrenches(c), c.scalar<std::uint64_t>("wrench_substeps"), L);
    std::vector<std::uint32_t> break_step(L.B, 0xffffffffU);
    std::vector<std::uint8_t> alive_before = L.alive;
    const std::vector<std::uint8_t> nbr_alive_built = L.nbr_alive;
    const std::uint64_t resume_at = c.scalarOr<std::uint64_t>("checkpoint_at", 0);
    // The phase-diff mode: the state after each phase of `phase_mask` in
    // substep `phase_substep`, as "phase<p>__<array>" outputs.
    const bool phases = c.has("phase_substep");
    const std::uint64_t phase_at = phases ? c.scalar<std::uint64_t>("phase_substep") : 0;
    const std::uint32_t phase_mask = phases ? c.scalar<std::uint32_t>("phase_mask") : 0;
    const auto dump = [&](unsigned p) {
        if (p >= 32 || !((phase_mask >> p) & 1U)) return;
        const std::string k = "phase" + std::to_string(p) + "__";
        out.put(k + "u", widen(L.u)); out.put(k + "u_prev", widen(L.u_prev)); out.put(k + "v", widen(L.v));
        out.put(k + "alive", L.alive); out.put(k + "failure_mode", L.failure_mode);
        out.put(k + "damage", widen(L.damage)); out.put(k + "plastic_extension", widen(L.plastic_ext));
        out.put(k + "plastic_strain", widen(L.plastic_strain));
        out.put(k + "prev_tensile", widen(L.prev_t)); out.put(k + "prev_compressive", widen(L.prev_c));
        out.put(k + "prev_shear", widen(L.prev_s));
        const Sphere<R> sp = run.sphere();
        out.put(k + "sphere_out", std::vector<double>{sp.center.x, sp.center.y, sp.center.z, sp.velocity.x, sp.velocity.y,
                                                      sp.velocity.z, sp.angular.x, sp.angular.y, sp.angular.z, sp.radius,
                                                      sp.mass, sp.inertia});
    };
    const std::uint64_t chunk = per_substep ? 1 : (ramp ? per_step : steps);
    const auto t0 = std::chrono::steady_clock::now();
    for (std::uint64_t done = 0; done < steps;) {
        if (ramp && done % per_step == 0) {
            const double sc = c.scalar<double>("force_ramp_scale") * static_cast<double>(done / per_step) /
                              static_cast<double>(c.scalar<std::uint64_t>("force_ramp_steps"));
            std::vector<double> f(base.size());
            for (std::size_t i = 0; i < f.size(); ++i) f[i] = sc * base[i];
            run.loads.set(f, per_step, L);
        }
        std::uint64_t n = std::min(chunk, steps - done);
        if (resume_at) {
            if (done < resume_at) n = std::min(n, resume_at - done);
            else if (done == resume_at) run.reupload(nbr_alive_built); // checkpoint and resume
        }
        if (phases && done <= phase_at && phase_at < done + n) {
            if (done < phase_at) {
                n = phase_at - done;
            } else {
                n = 1;
                run.phase_hook = dump;
            }
        }
        run.run(n);
        run.phase_hook = nullptr;
        done += n;
        if (per_substep) {
            for (std::uint32_t k = 0; k < L.B; ++k)
                if (alive_before[k] && !L.alive[k]) break_step[k] = static_cast<std::uint32_t>(done - 1);
            alive_before = L.alive;
        }
    }
    const double wall = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    out.put("u", widen(L.u)); out.put("u_prev", widen(L.u_prev)); out.put("v", widen(L.v));
    out.put("alive", L.alive); out.put("failure_mode", L.failure_mode);
    out.put("damage", widen(L.damage)); out.put("plastic_extension", widen(L.plastic_ext));
    out.put("plastic_strain", widen(L.plastic_strain));
    out.put("prev_tensile", widen(L.prev_t)); out.put("prev_compressive", widen(L.prev_c)); out.put("prev_shear", widen(L.prev_s));
    const Sphere<R> sp = run.sphere();
    out.put("sphere_out", std::vector<double>{sp.center.x, sp.center.y, sp.center.z, sp.velocity.x, sp.velocity.y, sp.velocity.z,
                                              sp.angular.x, sp.angular.y, sp.angular.z, sp.radius, sp.mass, sp.inertia});
    out.put("first_failure_bonds", run.first_failure_bonds);
    if (per_substep) out.put("break_step", break_step);
    const Status &st_ = run.status;
    std::vector<std::uint64_t> u(lsio::kStatusU64Width, 0);
    u[lsio::kTotalSteps] = st_.total_steps; u[lsio::kFirstFailureStep] = st_.first_failure_step;
    u[lsio::kLastFailureStep] = st_.last_failure_step; u[lsio::kFailureRounds] = st_.failure_rounds;
    u[lsio::kBrokenBonds] = st_.broken_bonds; u[lsio::kLastEnergyGainStep] = st_.last_energy_gain_step;
    u[lsio::kLastDamageGainStep] = st_.last_damage_gain_step; u[lsio::kExitReason] = st_.exit_reason;
    u[lsio::kRankDeficientNodes] = st_.rank_deficient_nodes; u[lsio::kImpulseContacts] = st_.contact.impulse_contacts;
    u[lsio::kCandidateOverflow] = st_.contact.candidate_overflow; u[lsio::kBallSupportEvents] = st_.contact.ball_support_events;
    u[lsio::kLaunches] = st_.launches;
    u[lsio::kNodeContacts] = st_.node.contacts; u[lsio::kNodePairTests] = st_.node.pair_tests;
    u[lsio::kNodeRebuilds] = st_.node.rebuilds; u[lsio::kNodePairsListed] = st_.node.pairs_listed;
    u[lsio::kNodePairOverflow] = st_.node.pair_overflow;
    std::vector<double> d(lsio::kStatusF64Width, 0.0);
    d[lsio::kRemovedEnergy] = st_.removed_energy; d[lsio::kMaxDamage] = st_.max_damage; d[lsio::kPlasticWork] = st_.plastic_work;
    d[lsio::kMaxTensile] = st_.max_t; d[lsio::kMaxCompressive] = st_.max_c; d[lsio::kMaxShear] = st_.max_s;
    d[lsio::kMaxPlasticStretch] = st_.max_plastic_stretch;
    d[lsio::kImpulseX] = st_.contact.impulse_x; d[lsio::kImpulseY] = st_.contact.impulse_y; d[lsio::kImpulseZ] = st_.contact.impulse_z;
    d[lsio::kContactDissipated] = st_.contact.dissipated; d[lsio::kMaxPenetration] = st_.contact.max_penetration;
    d[lsio::kMaxCorrection] = st_.contact.max_correction; d[lsio::kMaxCenterShift] = st_.contact.max_center_shift;
    d[lsio::kExternalWork] = st_.ext_work; d[lsio::kExternalImpulseX] = st_.ext_impulse[0];
    d[lsio::kExternalImpulseY] = st_.ext_impulse[1]; d[lsio::kExternalImpulseZ] = st_.ext_impulse[2];
    d[lsio::kExternalSteps] = static_cast<double>(st_.ext_steps); d[lsio::kWallSeconds] = wall;
    d[lsio::kNodeDissipated] = st_.node.dissipated; d[lsio::kNodeMaxOverlap] = st_.node.max_overlap;
    d[lsio::kNodeMaxCorrection] = st_.node.max_correction; d[lsio::kNodeMomentumX] = st_.node.momentum[0];
    d[lsio::kNodeMomentumY] = st_.node.momentum[1]; d[lsio::kNodeMomentumZ] = st_.node.momentum[2];
    d[lsio::kDampingDissipated] = st_.damping_dissipated; d[lsio::kStrikerDissipated] = st_.striker_dissipated;
    u[lsio::kEnergyAudited] = st_.energy_audited ? 1 : 0;
    out.put("status_u64", u);
    out.put("status_f64", d);
    if (!run.loads.sources.empty()) {
        std::vector<std::uint8_t> names;
        std::vector<double> ledgers;
        for (const SourceLedger &sl : run.loads.sources) {
            names.insert(names.end(), sl.source.begin(), sl.source.end());
            names.push_back(0);
            const LoadLedger &g = sl.load;
            const double row[lsio::kSourceLedgerWidth] = {g.steps, g.elapsed, g.req_imp.x, g.req_imp.y, g.req_imp.z,
                                                    g.imp.x, g.imp.y, g.imp.z, g.req_ang.x, g.req_ang.y, g.req_ang.z,
                                                    g.ang.x, g.ang.y, g.ang.z, g.work};
            ledgers.insert(ledgers.end(), row, row + lsio::kSourceLedgerWidth);
        }
        out.put("source_names", names);
        out.put("source_ledgers", ledgers);
    }
    out.putScalar<double>("wall_seconds", wall);
    out.putScalar<std::uint32_t>("threads", threads);
    out.putScalar<std::uint64_t>("bond_projections", st_.bond_projections);
    out.putScalar<std::uint64_t>("plastic_increments", st_.plastic_increments);
    out.put("substep_seconds", run.substep_seconds);
    out.put("substep_projections", run.substep_projections);
}

thread_local std::string g_error;

} // namespace orc

extern "C" {

void *oracle_case_new(void) { return new lsio::Case(); }
void oracle_case_free(void *c) { delete static_cast<lsio::Case *>(c); }

int oracle_case_put(void *c, const char *name, char type, std::uint64_t count, const void *data) {
    try {
        lsio::Array a;
        a.type = type;
        a.bytes.resize(count * a.width());
        if (count) std::memcpy(a.bytes.data(), data, a.bytes.size());
        static_cast<lsio::Case *>(c)->arrays[name] = std::move(a);
        return 0;
    } catch (const std::exception &e) { orc::g_error = e.what(); return 1; }
}

long long oracle_case_count(void *c, const char *name) {
    const auto &m = static_cast<lsio::Case *>(c)->arrays;
    const auto it = m.find(name);
    return it == m.end() ? -1 : static_cast<long long>(it->second.count());
}

char oracle_case_type(void *c, const char *name) {
    const auto &m = static_cast<lsio::Case *>(c)->arrays;
    const auto it = m.find(name);
    return it == m.end() ? '\0' : it->second.type;
}

int oracle_case_get(void *c, const char *name, void *dst, std::uint64_t bytes) {
    const auto &m = static_cast<lsio::Case *>(c)->arrays;
    const auto it = m.find(name);
    if (it == m.end() || it->second.bytes.size() != bytes) { orc::g_error = std::string("no array of that size: ") + name; return 1; }
    if (bytes) std::memcpy(dst, it->second.bytes.data(), bytes);
    return 0;
}

int oracle_case_read(void *c, const char *path) {
    try { static_cast<lsio::Case *>(c)->read(path); return 0; }
    catch (const std::exception &e) { orc::g_error = e.what(); return 1; }
}

int oracle_case_write(void *c, const char *path) {
    try { static_cast<lsio::Case *>(c)->write(path); return 0; }
    catch (const std::exception &e) { orc::g_error = e.what(); return 1; }
}

int oracle_run(void *in_case, void *out_case, int precision, int threads, int per_substep) {
    try {
        const lsio::Case &in = *static_cast<lsio::Case *>(in_case);
        lsio::Case &out = *static_cast<lsio::Case *>(out_case);
        const unsigned t = threads < 1 ? 1U : static_cast<unsigned>(threads);
        if (precision == 1) orc::runCase<double>(in, out, t, per_substep != 0);
        else orc::runCase<float>(in, out, t, per_substep != 0);
        return 0;
    } catch (const std::exception &e) { orc::g_error = e.what(); return 1; }
}

const char *oracle_last_error(void) { return orc::g_error.c_str(); }

} // extern "C"
