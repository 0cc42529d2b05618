// Element arithmetic of the lattice substep, for the device.
//
// Every expression keeps the operand order and association of the reference's
// element physics (src/fastlattice/LatticePhysics.hpp), and the library is
// compiled with -fmad=false and IEEE division and square root, because the
// float path is held to the reference CPU lane bit for bit: a fused
// multiply-add or a reassociated sum changes the last bit, and a changed bit
// becomes a different fracture cascade within a few hundred substeps. The
// reference's own, now removed, CUDA backend held the same rule
// (tests/fast_lattice_tests.cpp:474-523).
#pragma once

#include <cstdint>

#if defined(__CUDACC__)
#define GBL_HD __host__ __device__ __forceinline__
#else
#define GBL_HD inline
#endif

namespace gbl {

constexpr std::uint32_t kNoBond = 0xffffffffU;
// Bond record flags, kept in the spare high bits of the two node indices
// (nodes are limited to 2^30): a broken bond; the last bond of node a, and of
// node b, in one sweep of the schedule (where that node's support projection
// runs).
constexpr std::uint32_t kDeadBit = 0x80000000U;  // in a
constexpr std::uint32_t kLastABit = 0x40000000U; // in a
constexpr std::uint32_t kLastBBit = 0x80000000U; // in b
constexpr std::uint32_t kNodeMask = 0x3fffffffU;
constexpr unsigned kPlanes = 2;
constexpr unsigned kFootprints = 4;
constexpr unsigned kCandidatesPerBlock = 1024;

template <class R> struct alignas(4 * sizeof(R)) Q4 { R x, y, z, w; };
template <class R> struct alignas(2 * sizeof(R)) Q2 { R x, y; };

template <class R> struct V3 { R x, y, z; };
template <class R> GBL_HD V3<R> mk(R x, R y, R z) { return {x, y, z}; }
template <class R> GBL_HD V3<R> xyz(const Q4<R> &q) { return {q.x, q.y, q.z}; }
template <class R> GBL_HD V3<R> operator+(V3<R> a, V3<R> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class R> GBL_HD V3<R> operator-(V3<R> a, V3<R> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class R> GBL_HD V3<R> operator-(V3<R> a) { return {-a.x, -a.y, -a.z}; }
// Scalar products store component * scalar, whichever side the scalar is on.
template <class R> GBL_HD V3<R> operator*(V3<R> a, R s) { return {a.x * s, a.y * s, a.z * s}; }
template <class R> GBL_HD V3<R> operator*(R s, V3<R> a) { return {a.x * s, a.y * s, a.z * s}; }
template <class R> GBL_HD V3<R> operator/(V3<R> a, R s) { return {a.x / s, a.y / s, a.z / s}; }
template <class R> GBL_HD R dot(V3<R> a, V3<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class R> GBL_HD V3<R> cross(V3<R> a, V3<R> b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class R> GBL_HD R sqrtR(R x) { return sqrt(x); }
template <class R> GBL_HD R length(V3<R> a) { return sqrtR(dot(a, a)); }
template <class R> GBL_HD R absR(R x) { return x < R(0) ? -x : x; }
template <class R> GBL_HD R maxR(R a, R b) { return (a < b) ? b : a; }
template <class R> GBL_HD R minR(R a, R b) { return (b < a) ? b : a; }
template <class R> GBL_HD bool finiteR(R x) { return isfinite(x); }
template <class R> GBL_HD V3<R> normalized(V3<R> a) {
    const R m = length(a);
    return m > R(1.0e-12) ? a / m : mk<R>(1, 0, 0);
}

// ---------------------------------------------------------------------------
// Settings as the device sees them (StepSettings<R>, LatticePhysics.hpp:114-158, 248-284).
// ---------------------------------------------------------------------------
template <class R> struct Plane {
    V3<R> point, normal, tangent, bitangent;
    R restitution, static_friction, dynamic_friction, node_radius;
    std::uint32_t reach_capped, footprint_count;
    R fp[kFootprints][4]; // center_t, center_b, half_t, half_b
};

template <class R> struct Settings {
    R dt;
    V3<R> gravity;
    std::uint32_t iterations;
    R damping_fraction;
    std::uint32_t sphere_enabled;
    R yield_stretch, hardening;
    R c_static, c_dynamic, c_restitution, c_threshold, c_node_radius, c_margin, c_slack;
    std::uint32_t plane_count;
    Plane<R> planes[kPlanes];
    // NodeContactSettings (LatticePhysics.hpp:188-202): 0 off, 2 on, any
    // other value measures (broad and narrow phase, no response).
    std::uint32_t nc_mode;
    R nc_radius, nc_skin, nc_margin, nc_restitution, nc_threshold, nc_static, nc_dynamic;
    R plate_half_thickness; // > 0: the bending strain of sheets one cell thick
    std::uint32_t audit;    // StepSettings::audit_energy
};

template <class R> struct Sphere { V3<R> center, velocity, angular; R radius, mass, inertia; };

// ---------------------------------------------------------------------------
// Symmetric 3x3 eigensystem by cyclic Jacobi, 12 sweeps, and the truncating
// pseudo-inverse (LatticePhysics.hpp:446-531).
// ---------------------------------------------------------------------------
template <class R> GBL_HD void jacobi3(const R m[9], R d[3], R v[9]) {
    R a[9];
    for (int k = 0; k < 9; ++k) a[k] = m[k];
    for (int k = 0; k < 9; ++k) v[k] = (k % 4 == 0) ? R(1) : R(0);
    for (int sweep = 0; sweep < 12; ++sweep) {
        const R off = absR(a[1]) + absR(a[2]) + absR(a[5]);
        if (!(off > R(0))) break;
        for (int p = 0; p < 2; ++p) {
            for (int q = p + 1; q < 3; ++q) {
                const R apq = a[p * 3 + q];
                if (!(absR(apq) > R(0))) continue;
                const R app = a[p * 3 + p], aqq = a[q * 3 + q];
                const R theta = (aqq - app) / (R(2) * apq);
                const R sg = theta >= R(0) ? R(1) : R(-1);
                const R t = sg / (absR(theta) + sqrtR(theta * theta + R(1)));
                const R c = R(1) / sqrtR(t * t + R(1));
                const R s = t * c;
                for (int k = 0; k < 3; ++k) {
                    const R kp = a[k * 3 + p], kq = a[k * 3 + q];
                    a[k * 3 + p] = c * kp - s * kq;
                    a[k * 3 + q] = s * kp + c * kq;
                }
                for (int k = 0; k < 3; ++k) {
                    const R pk = a[p * 3 + k], qk = a[q * 3 + k];
                    a[p * 3 + k] = c * pk - s * qk;
                    a[q * 3 + k] = s * pk + c * qk;
                }
                for (int k = 0; k < 3; ++k) {
                    const R kp = v[k * 3 + p], kq = v[k * 3 + q];
                    v[k * 3 + p] = c * kp - s * kq;
                    v[k * 3 + q] = s * kp + c * kq;
                }
            }
        }
    }
    d[0] = a[0];
    d[1] = a[4];
    d[2] = a[8];
}

template <class R> GBL_HD int pseudoInverse3(const R m[9], R out[9], R normal[3]) {
    R d[3], v[9];
    jacobi3(m, d, v);
    R top = absR(d[0]);
    if (absR(d[1]) > top) top = absR(d[1]);
    if (absR(d[2]) > top) top = absR(d[2]);
    const R floor_value = (sizeof(R) == 8 ? R(1.0e-9) : R(1.0e-5)) * top;
    for (int k = 0; k < 9; ++k) out[k] = R(0);
    for (int k = 0; k < 3; ++k) normal[k] = R(0);
    int rank = 0, dropped = -1;
    for (int c = 0; c < 3; ++c) {
        if (!(d[c] > floor_value)) {
            dropped = c;
            continue;
        }
        ++rank;
        const R inv = R(1) / d[c];
        for (int r = 0; r < 3; ++r)
            for (int k = 0; k < 3; ++k) out[r * 3 + k] += inv * v[r * 3 + c] * v[k * 3 + c];
    }
    if (rank == 2 && dropped >= 0)
        for (int k = 0; k < 3; ++k) normal[k] = v[k * 3 + dropped];
    return rank;
}

// G = dA R+, E = (G + G^T + G^T G) / 2, then the in-plane projection of a
// coplanar neighbourhood (LatticePhysics.hpp:859-906).
template <class R> GBL_HD void strainFromMoments(const R acc[9], const R inv[9], const R un[3], R e[6]) {
    R f[9];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
            R s = R(0);
            for (int k = 0; k < 3; ++k) s += acc[r * 3 + k] * inv[k * 3 + c];
            f[r * 3 + c] = s;
        }
    const int rows[6] = {0, 1, 2, 0, 0, 1};
    const int cols[6] = {0, 1, 2, 1, 2, 2};
    for (int q = 0; q < 6; ++q) {
        R c = R(0);
        for (int k = 0; k < 3; ++k) c += f[k * 3 + rows[q]] * f[k * 3 + cols[q]];
        e[q] = R(0.5) * (f[rows[q] * 3 + cols[q]] + f[cols[q] * 3 + rows[q]] + c);
    }
    if (un[0] * un[0] + un[1] * un[1] + un[2] * un[2] > R(0)) {
        const R a[3] = {e[0] * un[0] + e[3] * un[1] + e[4] * un[2], e[3] * un[0] + e[1] * un[1] + e[5] * un[2],
                        e[4] * un[0] + e[5] * un[1] + e[2] * un[2]};
        const R s = a[0] * un[0] + a[1] * un[1] + a[2] * un[2];
        for (int q = 0; q < 6; ++q)
            e[q] += -un[rows[q]] * a[cols[q]] - a[rows[q]] * un[cols[q]] + s * un[rows[q]] * un[cols[q]];
    }
}

// Normal and shear of a stored strain along a unit direction (LatticePhysics.hpp:910-919).
template <class R> GBL_HD void resolveAlong(const R e[6], V3<R> d, R &normal, R &shear) {
    const V3<R> t{e[0] * d.x + e[3] * d.y + e[4] * d.z, e[3] * d.x + e[1] * d.y + e[5] * d.z,
                  e[4] * d.x + e[5] * d.y + e[2] * d.z};
    normal = dot(d, t);
    shear = length(t - normal * d);
}

// BondFailure.cpp bondDamageProgress (LatticePhysics.hpp:962-968).
template <class R> GBL_HD R damageProgress(R value, R start, R end) {
    if (!finiteR(start) || value <= start) return R(0);
    if (!finiteR(end) || end <= start) return value > start ? R(1) : R(0);
    const R p = (value - start) / (end - start);
    return p < R(0) ? R(0) : (p > R(1) ? R(1) : p);
}

// ---------------------------------------------------------------------------
// Support planes (LatticePhysics.hpp:1189-1252).
// ---------------------------------------------------------------------------
template <class R> GBL_HD bool insideFootprints(const Plane<R> &p, V3<R> x) {
    const V3<R> rel = x - p.point;
    const R t = dot(rel, p.tangent), b = dot(rel, p.bitangent);
    for (std::uint32_t k = 0; k < p.footprint_count; ++k)
        if (absR(t - p.fp[k][0]) <= p.fp[k][2] && absR(b - p.fp[k][1]) <= p.fp[k][3]) return true;
    return false;
}

// Returns the depth removed; `u` is updated in place and `projected` says
// whether the projection ran (it also runs for a node a hair above the plane).
template <class R> GBL_HD R projectSupport(const Plane<R> &p, V3<R> x0, V3<R> &u, R approach, R dt, bool &projected) {
    const V3<R> x = x0 + u;
    if (!insideFootprints(p, x)) return R(0);
    const R distance = dot(x - p.point, p.normal) - p.node_radius;
    if (distance > R(1.0e-8)) return R(0);
    if (p.reach_capped) {
        const R reach = R(8) * maxR(R(0), -approach) * dt + R(1.0e-5);
        if (-distance > reach) return R(0);
    }
    u = u - distance * p.normal;
    projected = true;
    return -distance;
}

template <class R> GBL_HD V3<R> supportVelocity(const Plane<R> &p, V3<R> vel, R approach) {
    const R restitution = -approach > R(0.5)
        ? (p.restitution < R(0) ? R(0) : (p.restitution > R(1) ? R(1) : p.restitution)) : R(0);
    const R target = approach < R(0) ? -restitution * approach : R(0);
    const R vn = dot(vel, p.normal);
    R corrected = vn;
    if (vn > target) corrected = target;
    else if (vn < R(0)) corrected = R(0);
    vel = vel + (corrected - vn) * p.normal;
    const R normal_delta = corrected - minR(R(0), approach);
    if (normal_delta <= R(0)) return vel;
    const V3<R> tangent = vel - dot(vel, p.normal) * p.normal;
    const R speed = length(tangent);
    if (speed <= R(1.0e-12)) return vel;
    const R fd = speed <= p.static_friction * normal_delta ? speed : minR(speed, p.dynamic_friction * normal_delta);
    return vel - (fd / speed) * tangent;
}

// Rigid ball against the support planes (LatticePhysics.hpp:1796-1825).
template <class R, class Acc> GBL_HD void sphereSupport(const Settings<R> &S, Sphere<R> &sp, Acc &acc) {
    for (std::uint32_t p = 0; p < S.plane_count; ++p) {
        const Plane<R> &pl = S.planes[p];
        const V3<R> foot = sp.center - sp.radius * pl.normal;
        if (!insideFootprints(pl, foot)) continue;
        const R distance = dot(foot - pl.point, pl.normal);
        if (distance > R(0)) continue;
        const R vn0 = dot(sp.velocity, pl.normal);
        if (-distance > R(8) * maxR(R(0), -vn0) * S.dt + R(1.0e-5)) continue;
        const R vn = dot(sp.velocity, pl.normal);
        if (vn < R(0)) {
            const R restitution = -vn > R(0.5) ? pl.restitution : R(0);
            const R nd = -(R(1) + restitution) * vn;
            sp.velocity = sp.velocity + nd * pl.normal;
            const V3<R> tangent = sp.velocity - dot(sp.velocity, pl.normal) * pl.normal;
            const R speed = length(tangent);
            if (speed > R(1.0e-12)) {
                const R fd = speed <= pl.static_friction * nd ? speed : minR(speed, pl.dynamic_friction * nd);
                sp.velocity = sp.velocity - (fd / speed) * tangent;
            }
            ++acc.ball_support_events;
        }
        sp.center = sp.center - distance * pl.normal;
    }
}

// Exit rules (LatticePhysics.hpp:1766-1791).
GBL_HD unsigned exitReason(unsigned long long completed, unsigned broken, unsigned long long last_failure,
                           unsigned long long quiet, unsigned long long min_steps, unsigned long long no_failure,
                           unsigned long long energy_flat, unsigned long long last_energy_gain, unsigned long long calm,
                           unsigned long long last_damage_gain, double max_damage, double calm_margin, double removed,
                           double removable) {
    if (removable > 0.0 && removed >= removable) return 6U;
    if (broken > 0U && quiet > 0ULL && completed >= min_steps && completed > last_failure &&
        completed - last_failure > quiet)
        return 1U;
    if (broken == 0U && no_failure > 0ULL && completed >= no_failure) return 2U;
    if (broken == 0U && calm > 0ULL && completed >= calm && max_damage < calm_margin && completed > last_damage_gain &&
        completed - last_damage_gain > calm)
        return 5U;
    if (broken > 0U && energy_flat > 0ULL && completed >= min_steps && completed > last_energy_gain &&
        completed - last_energy_gain > energy_flat)
        return 4U;
    return 0U;
}

} // namespace gbl
