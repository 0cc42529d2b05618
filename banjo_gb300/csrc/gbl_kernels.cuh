// Kernels of the bonded-lattice substep.
//
// Device layout (one lattice, or many independent lattices concatenated):
//   nodes  u[i]   = (u.xyz, inv_mass)   v[i] = (v.xyz, mass)   x0[i] = (x0.xyz, 0)
//          up[i]  = u_prev              strain[2i..2i+1] = (e0..e3 | e4, e5, valid, 0)
//          rinv   9 x N, unm 3 x N      (component-major, coalesced per node)
//          nbr[k*N+i] = (rest.xyz, the slot's weight, negated once its bond has failed; 0 when padded)
//          nbr_other[k*N+i] (i itself for a padded slot), nbr_bond[k*N+i]
//   bonds  rec[d] = (a | dead | last-of-a, b | last-of-b, rest_length_sq_minus, rest_length)
//          geo[d] = (rest_edge.xyz, compliance)
//          prev[d] = (prev_tensile, prev_compressive, prev_shear, damage)
//          plastic[d] = (extension, strain), thr4/thr2 = six damage thresholds
// Bonds are stored level-major. A level is the set of bonds at one depth of
// the reference's serial sweep order (CpuLatticeBackend.cpp:336-348, 395-407),
// depth being one more than the deepest earlier bond at either end: a level
// shares no node, and every node meets its bonds in the serial order, so any
// thread mapping inside a level reproduces the serial sweep bit for bit.
// dev2sched maps storage index d to schedule index j; everything a caller
// sees (events, downloads, failure lists) is in schedule order.
#pragma once

#include "gbl_math.cuh"

#include <cfloat>
#include <cstdint>
#include <type_traits>

namespace gbl {

template <class R> struct BondRec;
template <> struct alignas(16) BondRec<float> { std::uint32_t a, b; float rsm, rest; };
template <> struct alignas(8) BondRec<double> { std::uint32_t a, b; double rsm, rest; };

template <class R> __device__ __forceinline__ std::uint32_t endA(const BondRec<R> &r) { return r.a & kNodeMask; }
template <class R> __device__ __forceinline__ std::uint32_t endB(const BondRec<R> &r) { return r.b & kNodeMask; }

// ---------------------------------------------------------------------------
// The bounds-checked build (GBL_BOUNDS_CHECK defined: libgbl_checked.so). Every
// index the kernels read out of device data -- bond ends, neighbour slots,
// candidate, dirty, event, load, halo and isolated-node lists -- is checked
// against the length of the array it indexes before it is used. A violation is
// counted in g_bounds_violation, with the first one's site, index and length,
// and the access is skipped; nothing traps, so the context stays usable and
// the host reads the record (gbl_bounds_report). In the normal build the check
// is the constant true.
// ---------------------------------------------------------------------------
enum BoundsSite : unsigned {
    kSiteSolve = 1, kSiteStrain, kSiteDirty, kSiteDirtyBond, kSiteEndSample, kSiteCandidate, kSiteEvent,
    kSiteEventEnd, kSiteLoad, kSiteIsolated, kSiteHalo, kSiteDamp
};
#ifdef GBL_BOUNDS_CHECK
__device__ unsigned long long g_bounds_violation[4]; // count, then the first's site, index, length
__device__ __noinline__ bool boundsViolated(std::uint64_t i, std::uint64_t n, unsigned site) {
    if (atomicAdd(&g_bounds_violation[0], 1ULL) == 0) {
        g_bounds_violation[1] = site;
        g_bounds_violation[2] = i;
        g_bounds_violation[3] = n;
    }
    return false;
}
__device__ __forceinline__ bool inBounds(std::uint64_t i, std::uint64_t n, unsigned site) {
    return i < n || boundsViolated(i, n, site);
}
#else
__device__ __forceinline__ constexpr bool inBounds(std::uint64_t, std::uint64_t, unsigned) { return true; }
#endif
template <class R> __device__ __forceinline__ bool endsInBounds(const BondRec<R> &r, std::uint32_t n, unsigned site) {
    return inBounds(endA(r), n, site) && inBounds(endB(r), n, site);
}

// Streaming loads for data read once per pass (bond records), so that they do
// not evict the node arrays the gathers keep re-reading from L2.
__device__ __forceinline__ BondRec<float> ldStream(const BondRec<float> *p) {
    const uint4 v = __ldcs(reinterpret_cast<const uint4 *>(p));
    return {v.x, v.y, __uint_as_float(v.z), __uint_as_float(v.w)};
}
__device__ __forceinline__ BondRec<double> ldStream(const BondRec<double> *p) {
    const uint2 ab = __ldcs(reinterpret_cast<const uint2 *>(p));
    const double *d = reinterpret_cast<const double *>(p);
    return {ab.x, ab.y, __ldcs(d + 1), __ldcs(d + 2)};
}
__device__ __forceinline__ Q4<float> ldStream(const Q4<float> *p) {
    const float4 v = __ldcs(reinterpret_cast<const float4 *>(p));
    return {v.x, v.y, v.z, v.w};
}
__device__ __forceinline__ Q4<double> ldStream(const Q4<double> *p) {
    const double2 *q = reinterpret_cast<const double2 *>(p);
    const double2 lo = __ldcs(q), hi = __ldcs(q + 1);
    return {lo.x, lo.y, hi.x, hi.y};
}
// L2-only loads for node data gathered once per pass by a different thread.
__device__ __forceinline__ Q4<float> ldShared(const Q4<float> *p) {
    const float4 v = __ldcg(reinterpret_cast<const float4 *>(p));
    return {v.x, v.y, v.z, v.w};
}
__device__ __forceinline__ Q4<double> ldShared(const Q4<double> *p) {
    const double2 *q = reinterpret_cast<const double2 *>(p);
    const double2 lo = __ldcg(q), hi = __ldcg(q + 1);
    return {lo.x, lo.y, hi.x, hi.y};
}

// Serial bookkeeping (ContactAccumulators, LatticePhysics.hpp:379-388).
struct ContactAcc {
    unsigned long long impulse_contacts;
    double impulse_x, impulse_y, impulse_z, dissipated, max_penetration, max_correction, max_center_shift;
    unsigned long long candidate_overflow, ball_support_events;
};

struct LoadLedger {
    unsigned long long steps;
    double elapsed, req_imp[3], imp[3], req_ang[3], ang[3], work;
};

// NodeContactAccumulators (LatticePhysics.hpp:204-221).
struct NodeAcc {
    unsigned long long contacts, pair_tests, rebuilds, pairs_listed, pair_overflow;
    double dissipated, max_overlap, max_correction, momentum[3];
};

// One device control block per lattice: the RunStatus accumulators, the
// RunControl exit rules, and the substep's transient counters.
struct Ctl {
    unsigned long long total_steps, first_failure_step, last_failure_step, last_energy_gain_step, last_damage_gain_step;
    unsigned failure_rounds, broken_bonds, rank_deficient, exit_reason;
    double removed_energy, max_damage, plastic_work;
    unsigned max_t, max_c, max_s, max_plastic; // non-negative float bit patterns
    ContactAcc contact;
    LoadLedger ext;
    // RunControl
    unsigned stop, error;
    unsigned long long quiet_steps, min_steps, no_failure_steps, energy_flat_steps, calm_steps;
    double energy_flat_fraction, calm_damage_margin, removable_energy;
    unsigned long long loads_remaining;
    unsigned long long step_limit; // a served lattice's substep count (0: none); reaching it is exit 3 (max steps)
    // transient
    unsigned full_restart, dirty_count, ffb_count, loads_kicked;
    unsigned event_count, ext_count; // broken bonds this substep; loaded nodes (set between runs)
    unsigned dmg_count, energy_gain;  // damage-record candidates; any broken bond passed the gain test
    double plastic_substep, removed_substep;
    // Node-to-node contact: its accumulators; whether the pair list is rebuilt
    // this substep (set at upload, after a failure round, or by the drift
    // test; cleared by the narrow phase), the list's length, and the bucket
    // fill of the build in progress.
    NodeAcc node;
    unsigned nc_rebuild, nc_pairs, nc_members;
    // The energy audit: the kinetic energy before the phase being measured,
    // and what the damping sweep and the striker passes took out.
    double ke_mark, damping_dissipated, striker_dissipated;
    // External wrenches: how many are set, and the count of sources kicked
    // since upload (a new source's place in the status order).
    unsigned wrench_count, source_seq;
    // Bond projections the sweeps ran: per substep, the bonds alive when its
    // sweep starts (alive at upload less those broken since) times the
    // solver iterations.
    unsigned long long projections, live_bonds;
};

// An external wrench on the device (ExternalWrench, FastLattice.hpp:153-157):
// its nodes (a range of the load list, sources in name order, nodes ascending),
// its source ledger slot, and its point, force and torque.
struct WrenchDev {
    std::uint32_t begin, end, slot, pad;
    double point[3], force[3], torque[3];
};
// A source's ledger (ExternalWrenchLedger) and its place in the status order.
struct SourceSlot {
    LoadLedger load;
    unsigned long long order;
};

constexpr unsigned kErrExternalOverflow = 1;
constexpr unsigned kErrWrench = 2;
constexpr unsigned kErrStageWait = 4; // a bounded wait for a bulk copy into shared memory ran out

template <class R> struct Dev {
    std::uint32_t N, B, D, blocks, words_b, tiles_b;
    Q4<R> *u, *v, *x0, *up, *strain;
    R *rinv, *unm, *approach;
    std::uint8_t *dirty, *engaged, *candidate;
    std::uint32_t *cand_bits;
    Q4<R> *nbr;
    std::uint32_t *nbr_other, *nbr_bond;
    std::uint32_t *slot_a, *slot_b;
    BondRec<R> *rec;
    Q4<R> *geo, *prev, *thr4;
    Q2<R> *thr2, *plastic;
    R *lambda;
    std::uint8_t *mode;
    // Substep ledger scratch. ev_*: broken bonds (bit per bond, per-tile count
    // then offset, ordered list, removed energy by bond and packed in list
    // order, in-tile inclusive prefix); dmg_*: bonds whose damage passed the
    // run maximum (the candidates of the damage-record scan); tile_*: per
    // end-sample tile FP64 partials and their prefix.
    std::uint32_t *ev_bits, *ev_tile, *ev_list;
    double *ev_removed, *ev_packed, *ev_prefix;
    uint2 *ev_ends;               // the two nodes of a broken bond, by schedule index
    std::uint32_t *dev2sched;     // bond storage order (level-major) -> schedule index
    std::uint32_t *isolated;      // nodes without bonds (their support projection has no sweep to ride on)
    std::uint32_t isolated_count;
    std::uint32_t *level_begin;   // sweep level boundaries in storage order (level_count + 1), when level_count fits
    std::uint32_t level_count;
    std::uint32_t *dmg_bits, *dmg_tile, *dmg_list;
    float *ev_damage, *dmg_value;
    double *tile_plastic, *tile_removed;
    std::uint32_t *blk_ev, *blk_dmg;   // per scan block of tiles: totals, then offsets
    double *blk_removed, *blk_plastic;
    std::uint32_t *node_block_begin, *cand_list, *cand_count, *dirty_list, *ffb;
    // Contact halo of the substep (stamped with the substep's number + 1): the
    // listed sphere candidates and their neighbours, and the end-sample tiles
    // holding a bond at one of them. Everything outside it is final before the
    // second contact pass, so its strain and end sample run beside that pass.
    std::uint32_t *halo_stamp, *late_tile_stamp;
    Q4<R> *ext_force;     // applied force (backend precision), w != 0 marks a loaded node
    double *ext_req;      // requested force, 3 per node
    double *ext_contrib;  // 13 per node: impulse 3, angular 3, work, requested 3, requested angular 3
    std::uint32_t *ext_nodes;
    WrenchDev *wrench;    // the set wrenches (their count is in the control block)
    SourceSlot *sources;  // every source kicked since upload
    // Node-to-node contact scratch, allocated when the settings turn contact
    // on: positions at the last build, each node's grid cell (w: its bucket),
    // the hashed grid (per bucket: count, then scatter cursor; first member;
    // members ascending within a bucket), pairs per owner and per 256-node
    // tile (then the tile's first pair), and the pair list in narrow-phase
    // order (owner, partner, bond or kNoBond).
    Q4<R> *nc_built;
    int4 *nc_cell;
    std::uint32_t *nc_count, *nc_start, *nc_members, *nc_fill, *nc_tile;
    std::uint32_t *nc_pa, *nc_pb, *nc_pbond;
    std::uint32_t nc_mask;
    double origin[3];
    Sphere<R> *sphere;
    Ctl *ctl;
    unsigned *running; // lattices of the engine still running this call; a lattice that stops takes itself off
};

constexpr int kThreads = 256;

// One CTA's share of a launch: a range of one lattice's nodes, bonds, tiles or
// scan blocks (what the range indexes is the kernel's).
struct Work {
    std::uint32_t lattice, begin, end;
};

// What a launch covers. With many lattices (Many = true) every CTA reads its
// item from `list` and its lattice's descriptor from `table`, so one launch
// advances any number of independent lattices. A launch over one lattice
// (Many = false) carries that lattice's descriptor in `one`, in the kernel's
// parameter space, and CTA b covers [base + b*per, min(base + (b+1)*per, end)):
// no dependent loads before the work itself.
template <class R> struct Grid {
    const Dev<R> *table;
    const Work *list;
    std::uint32_t base, end, per;
    Dev<R> one;
};

template <bool Many, class R> __device__ __forceinline__ Work item(const Grid<R> &g) {
    if (Many) return g.list[blockIdx.x];
    const std::uint32_t b = g.base + blockIdx.x * g.per;
    return Work{0U, b, b + g.per < g.end ? b + g.per : g.end};
}

// Items of a launch split into parts: {lattice, part, parts}.
template <bool Many, class R> __device__ __forceinline__ Work part(const Grid<R> &g) {
    if (Many) return g.list[blockIdx.x];
    return Work{0U, blockIdx.x, gridDim.x};
}

template <class R, bool Many> __device__ __forceinline__ Dev<R> descriptor(const Grid<R> &g, const Work &w) {
    if (Many) return g.table[w.lattice];
    return g.one;
}

// The descriptor as a reference a long kernel reads its fields through: for
// many lattices, the CTA's lattice's descriptor copied once into shared
// memory (its fields are then read from there as needed, not held in
// registers across the kernel); for one lattice, the launch's own. Every
// thread of the CTA must call it (it synchronises).
template <class R> struct SharedDesc {
    __align__(16) unsigned char bytes[sizeof(Dev<R>)];
};
template <class R, bool Many>
__device__ __forceinline__ const Dev<R> &descriptorIn(const Grid<R> &g, const Work &w, SharedDesc<R> &smem) {
    if (!Many) return g.one;
    const unsigned *src = reinterpret_cast<const unsigned *>(g.table + w.lattice);
    unsigned *dst = reinterpret_cast<unsigned *>(smem.bytes);
    for (unsigned k = threadIdx.x; k < sizeof(Dev<R>) / sizeof(unsigned); k += blockDim.x) dst[k] = src[k];
    __syncthreads();
    return *reinterpret_cast<const Dev<R> *>(smem.bytes);
}

template <class R> __device__ __forceinline__ V3<R> pos(const Dev<R> &L, std::uint32_t i) {
    return xyz(L.x0[i]) + xyz(L.u[i]);
}

// ---------------------------------------------------------------------------
// Nonlocal node strain (LatticePhysics.hpp:791-907, plate bending off).
// ---------------------------------------------------------------------------
// A slot's weight while its bond is alive, else 0 (LatticeArrays::nbr_alive
// gating nbr_weight); the raw weight stays in the slot, sign-flipped, for the
// rest geometry of plate bending.
template <class R> __device__ __forceinline__ R liveWeight(R w) { return signbit(w) ? R(0) : w; }

// Bending strain of a sheet one cell thick (plateBendingStrain,
// LatticePhysics.hpp:575-777): the rest neighbourhood (every bond built, alive
// or not) says whether the node lies in a sheet and which way it faces; a
// tilt fit and then a curvature fit over the live neighbours; a fit that
// explains no more than 0.9 of the out-of-plane motion claims no bending; the
// tension fibre of |K| at half the thickness, capped at the yield stretch, is
// added to E in the sheet's frame.
template <class R, bool Direct>
__device__ __noinline__ void plateBending(const Dev<R> &L, std::uint32_t i, V3<R> xi, R half_thickness,
                                          R yield_stretch, R *e) {
    const std::size_t N = L.N;
    R rest_cov[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (std::uint32_t k = 0; k < L.D; ++k) {
        const std::size_t slot = k * N + i;
        if (L.nbr_bond[slot] == kNoBond) continue;
        const Q4<R> q = L.nbr[slot];
        const R w = absR(q.w);
        if (w <= R(0)) continue;
        const R rr[3] = {q.x, q.y, q.z};
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) rest_cov[r * 3 + c] += w * rr[r] * rr[c];
    }
    R rest_inv[9], flat[3];
    if (pseudoInverse3(rest_cov, rest_inv, flat) >= 3) return; // a solid neighbourhood, not a sheet
    const V3<R> normal{flat[0], flat[1], flat[2]};
    if (!(dot(normal, normal) > R(0))) return;
    R inv[9];
    for (int k = 0; k < 9; ++k) inv[k] = L.rinv[k * N + i];
    auto neighbour = [&](std::uint32_t k, R &w, V3<R> &rest, V3<R> &d) {
        const std::size_t slot = k * N + i;
        const bool present = L.nbr_bond[slot] != kNoBond;
        const Q4<R> q = L.nbr[slot];
        std::uint32_t other = present ? L.nbr_other[slot] : i;
        if (!inBounds(other, N, kSiteStrain)) other = i;
        w = present ? liveWeight(q.w) : R(0);
        rest = present ? V3<R>{q.x, q.y, q.z} : V3<R>{R(0), R(0), R(0)};
        const V3<R> xo = Direct ? pos(L, other) : xyz(L.u[other]);
        d = Direct ? (xo - xi) - rest : xo - xi;
    };
    R rhs[3] = {0, 0, 0};
    for (std::uint32_t k = 0; k < L.D; ++k) {
        R w;
        V3<R> rest, d;
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
    const R ax = normal.x < R(0) ? -normal.x : normal.x;
    const R ay = normal.y < R(0) ? -normal.y : normal.y;
    const R az = normal.z < R(0) ? -normal.z : normal.z;
    const V3<R> axis = (ax <= ay && ax <= az) ? V3<R>{R(1), R(0), R(0)}
                     : (ay <= az)             ? V3<R>{R(0), R(1), R(0)}
                                              : V3<R>{R(0), R(0), R(1)};
    V3<R> e1 = cross(normal, axis);
    const R e1len = length(e1);
    if (!(e1len > R(0))) return;
    e1 = (R(1) / e1len) * e1;
    const V3<R> e2 = cross(normal, e1);
    R A[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    R g[3] = {0, 0, 0};
    R out2 = R(0);
    for (std::uint32_t k = 0; k < L.D; ++k) {
        R w;
        V3<R> rest, d;
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
    jacobi3(A, ev, axes);
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
    const R half_trace = R(0.5) * (c[0] + c[2]);
    const R det = c[0] * c[2] - c[1] * c[1];
    R under = half_trace * half_trace - det;
    if (under < R(0)) under = R(0);
    const R disc = sqrtR(under);
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
    const int rows[6] = {0, 1, 2, 0, 0, 1};
    const int cols[6] = {0, 1, 2, 1, 2, 2};
    for (int q = 0; q < 6; ++q)
        e[q] += b11 * u1[rows[q]] * u1[cols[q]] + b22 * u2[rows[q]] * u2[cols[q]] +
                b12 * (u1[rows[q]] * u2[cols[q]] + u2[rows[q]] * u1[cols[q]]);
}

template <class R, bool Direct, bool Plate = false>
__device__ void nodeStrain(const Dev<R> &L, std::uint32_t i, R plate_half_thickness = R(0), R plate_yield = R(0)) {
    const std::size_t N = L.N;
    if (L.dirty[i]) {
        R cov[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        std::uint32_t live = 0;
        for (std::uint32_t k = 0; k < L.D; ++k) {
            const Q4<R> q = L.nbr[k * N + i];
            const R w = liveWeight(q.w);
            if (w <= R(0)) continue; // dead, padded, or a degenerate rest edge
            const R rr[3] = {q.x, q.y, q.z};
            for (int r = 0; r < 3; ++r)
                for (int c = 0; c < 3; ++c) cov[r * 3 + c] += w * rr[r] * rr[c];
            ++live;
        }
        R valid = R(0);
        if (live >= 1U) {
            R inv[9], un[3];
            const int rank = pseudoInverse3(cov, inv, un);
            if (rank >= 2) {
                for (int k = 0; k < 9; ++k) L.rinv[k * N + i] = inv[k];
                for (int k = 0; k < 3; ++k) L.unm[k * N + i] = un[k];
                valid = R(1);
            }
            if (rank < 3) atomicAdd(&L.ctl->rank_deficient, 1U);
        }
        L.strain[2 * i + 1].z = valid;
        L.dirty[i] = 0;
        if (valid == R(0)) return;
    } else if (L.strain[2 * i + 1].z == R(0)) {
        return;
    }
    R acc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    const V3<R> xi = Direct ? pos(L, i) : xyz(L.u[i]);
#pragma unroll 2
    for (std::uint32_t k = 0; k < L.D; ++k) {
        const std::size_t slot = k * N + i;
        const Q4<R> q = L.nbr[slot];
        const std::uint32_t other = L.nbr_other[slot];
        if (!inBounds(other, N, kSiteStrain)) continue;
        const V3<R> rest{q.x, q.y, q.z};
        const V3<R> xo = Direct ? pos(L, other) : xyz(L.u[other]);
        const V3<R> cur = Direct ? (xo - xi) - rest : xo - xi;
        const R w = liveWeight(q.w);
        const R cc[3] = {cur.x, cur.y, cur.z};
        const R rr[3] = {rest.x, rest.y, rest.z};
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) acc[r * 3 + c] += w * cc[r] * rr[c];
    }
    R inv[9], un[3], e[6];
    for (int k = 0; k < 9; ++k) inv[k] = L.rinv[k * N + i];
    for (int k = 0; k < 3; ++k) un[k] = L.unm[k * N + i];
    strainFromMoments(acc, inv, un, e);
    // What a coplanar neighbourhood's plane cannot hold: the bending of a
    // sheet one cell thick (LatticePhysics.hpp:896-905).
    if (Plate && plate_half_thickness > R(0) && un[0] * un[0] + un[1] * un[1] + un[2] * un[2] > R(0))
        plateBending<R, Direct>(L, i, xi, plate_half_thickness, plate_yield, e);
    L.strain[2 * i] = Q4<R>{e[0], e[1], e[2], e[3]};
    L.strain[2 * i + 1] = Q4<R>{e[4], e[5], R(1), R(0)};
}

// The stamp of the running substep in the halo marks (never 0, the cleared value).
template <class R> __device__ __forceinline__ std::uint32_t substepStamp(const Dev<R> &L) {
    return static_cast<std::uint32_t>(L.ctl->total_steps) + 1U;
}

template <class R, bool Many, bool Direct, bool Plate>
__global__ void __launch_bounds__(kThreads) kStrainAll(const Grid<R> launch, int part, R plate, R yield) {
    const Work w = item<Many>(launch);
    __shared__ SharedDesc<R> desc;
    const Dev<R> &L = descriptorIn<R, Many>(launch, w, desc);
    if (L.ctl->stop) return;
    const std::uint32_t i = w.begin + threadIdx.x;
    if (i >= w.end) return;
    // part 0: every node; 1: the nodes outside the contact halo; 2: inside it.
    if (part != 0) {
        const bool halo = L.halo_stamp[i] == substepStamp(L);
        if (halo != (part == 2)) return;
    }
    nodeStrain<R, Direct, Plate>(L, i, plate, yield);
}

// The start-of-substep restart after an upload (every node) or after a failure
// round (the dirty nodes only: every other node's strain is unchanged, since
// positions have not moved since the end sample and its bonds are the same;
// src/fastlattice/ParallelCpuLatticeBackend.cpp:1718-1757 relies on the same fact).
// It reads the substep's starting positions: before the kick from u, or after
// it (beside the first contact pass) from u_prev, where the kick copied them.
template <class R, bool Many, bool Direct, bool Plate>
__global__ void __launch_bounds__(kThreads) kRestartStrain(const Grid<R> launch, int after_kick, R plate, R yield) {
    const Work w = item<Many>(launch);
    Dev<R> L = descriptor<R, Many>(launch, w);
    if (after_kick) L.u = L.up; // the kick kept the substep's starting positions there
    if (L.ctl->stop) return;
    // Items cover the node index range; a dirty list is never longer.
    const std::uint32_t t = w.begin + threadIdx.x;
    if (t >= w.end) return;
    if (L.ctl->full_restart) nodeStrain<R, Direct, Plate>(L, t, plate, yield);
    else if (t < L.ctl->dirty_count) {
        const std::uint32_t node = L.dirty_list[t];
        if (inBounds(node, L.N, kSiteDirty)) nodeStrain<R, Direct, Plate>(L, node, plate, yield);
    }
}

// ---------------------------------------------------------------------------
// Bond samples (LatticePhysics.hpp:921-959, 1116-1126).
// ---------------------------------------------------------------------------
template <class R, bool Direct>
__device__ __forceinline__ V3<R> bondVector(const Dev<R> &L, std::uint32_t a, std::uint32_t b, V3<R> edge) {
    if (Direct) return pos(L, b) - pos(L, a);
    return edge + (xyz(L.u[b]) - xyz(L.u[a]));
}

template <class R, bool Direct>
__device__ void sampleBond(const Dev<R> &L, std::uint32_t a, std::uint32_t b, const BondRec<R> &rec, V3<R> edge,
                           R len, R &t, R &c, R &s) {
    const R rest = rec.rest;
    R stretch;
    if (Direct) {
        stretch = len / rest - R(1);
    } else {
        const V3<R> du = xyz(L.u[b]) - xyz(L.u[a]);
        const R num = rec.rsm + R(2) * dot(edge, du) + dot(du, du);
        stretch = num / ((len + rest) * rest);
    }
    t = stretch;
    c = -stretch;
    s = R(0);
    const R rl = length(edge);
    if (rl > R(1.0e-9)) {
        const V3<R> dir = edge * (R(1) / rl);
        const std::uint32_t ends[2] = {a, b};
        for (int q = 0; q < 2; ++q) {
            const Q4<R> s0 = L.strain[2 * ends[q]], s1 = L.strain[2 * ends[q] + 1];
            if (s1.z == R(0)) continue;
            const R e[6] = {s0.x, s0.y, s0.z, s0.w, s1.x, s1.y};
            R nn, sh;
            resolveAlong(e, dir, nn, sh);
            t = maxR(t, nn);
            c = maxR(c, -nn);
            s = maxR(s, sh);
        }
    }
}

template <class R, bool Direct>
__device__ __forceinline__ void startSample(const Dev<R> &L, std::uint32_t j) {
    const BondRec<R> rec = L.rec[j];
    if (rec.a & kDeadBit) return;
    const Q4<R> g = L.geo[j];
    R t, c, s;
    const V3<R> edge{g.x, g.y, g.z};
    const R len = length(bondVector<R, Direct>(L, endA(rec), endB(rec), edge));
    sampleBond<R, Direct>(L, endA(rec), endB(rec), rec, edge, len, t, c, s);
    Q4<R> p = L.prev[j];
    p.x = maxR(R(0), t);
    p.y = maxR(R(0), c);
    p.z = maxR(R(0), s);
    L.prev[j] = p;
}

// Every live bond, after an upload: items cover the bond storage range.
template <class R, bool Many, bool Direct>
__global__ void __launch_bounds__(kThreads) kRestartBondsAll(const Grid<R> launch, int after_kick) {
    const Work w = item<Many>(launch);
    Dev<R> L = descriptor<R, Many>(launch, w);
    if (after_kick) L.u = L.up;
    if (L.ctl->stop || !L.ctl->full_restart) return;
    const std::uint32_t d = w.begin + threadIdx.x;
    if (d < w.end) startSample<R, Direct>(L, d);
}

// The live bonds at each dirty node, after a failure round: items cover the
// node index range (one thread per dirty-list entry, over its neighbour
// slots). A bond with both ends dirty is sampled twice to the same values.
template <class R, bool Many, bool Direct>
__global__ void __launch_bounds__(kThreads) kRestartBondsDirty(const Grid<R> launch, int after_kick) {
    const Work w = item<Many>(launch);
    Dev<R> L = descriptor<R, Many>(launch, w);
    if (after_kick) L.u = L.up;
    if (L.ctl->stop || L.ctl->full_restart) return;
    const std::uint32_t t = w.begin + threadIdx.x;
    if (t >= w.end || t >= L.ctl->dirty_count) return;
    const std::uint32_t node = L.dirty_list[t];
    if (!inBounds(node, L.N, kSiteDirty)) return;
    for (std::uint32_t k = 0; k < L.D; ++k) {
        const std::uint32_t d = L.nbr_bond[static_cast<std::size_t>(k) * L.N + node];
        if (d != kNoBond && inBounds(d, L.B, kSiteDirtyBond)) startSample<R, Direct>(L, d);
    }
}

// ---------------------------------------------------------------------------
// Kick and classify (LatticePhysics.hpp:1702-1719), with the external force
// kick before it (ExternalLoads.hpp:79-148).
// ---------------------------------------------------------------------------
template <class R>
__device__ __forceinline__ bool sphereCandidate(const Settings<R> &S, const Sphere<R> &sp, V3<R> x, V3<R> vel, R mass) {
    if (mass <= R(0)) return false;
    const V3<R> r = x - sp.center;
    const R distance = length(r);
    const R gap = distance - (sp.radius + S.c_node_radius);
    const R bound = length(vel - sp.velocity) + length(sp.angular) * distance;
    const R reach = maxR(S.c_margin, bound * S.dt) + S.c_slack;
    return gap <= reach;
}

template <class R, bool Many>
__global__ void __launch_bounds__(kThreads) kKick(const Grid<R> launch, Settings<R> S) {
    const Work w = item<Many>(launch);
    __shared__ SharedDesc<R> desc;
    const Dev<R> &L = descriptorIn<R, Many>(launch, w, desc);
    if (L.ctl->stop) return;
    const std::uint32_t i = w.begin + threadIdx.x; // items start on multiples of 256: warps cover whole bit words
    bool cand = false;
    if (i < w.end) {
        Q4<R> vq = L.v[i];
        const Q4<R> uq = L.u[i];
        V3<R> vel = xyz(vq);
        if (L.ctl->ext_count && L.ctl->loads_remaining > 0) {
            const Q4<R> f = L.ext_force[i];
            if (f.w != R(0)) {
                const V3<R> before = vel;
                const V3<R> after = before + (S.dt * uq.w) * V3<R>{f.x, f.y, f.z};
                if (!finiteR(after.x) || !finiteR(after.y) || !finiteR(after.z)) {
                    atomicOr(&L.ctl->error, kErrExternalOverflow);
                } else {
                    vel = after;
                    const double m = static_cast<double>(vq.w);
                    const double o[3] = {double(before.x), double(before.y), double(before.z)};
                    const double n[3] = {double(after.x), double(after.y), double(after.z)};
                    const double imp[3] = {m * (n[0] - o[0]), m * (n[1] - o[1]), m * (n[2] - o[2])};
                    const V3<R> p = xyz(L.x0[i]) + xyz(uq);
                    const double wp[3] = {L.origin[0] + double(p.x), L.origin[1] + double(p.y), L.origin[2] + double(p.z)};
                    const double dt = static_cast<double>(S.dt);
                    const double rq[3] = {dt * L.ext_req[3 * i], dt * L.ext_req[3 * i + 1], dt * L.ext_req[3 * i + 2]};
                    double *c = L.ext_contrib + 13 * static_cast<std::size_t>(i);
                    c[0] = imp[0]; c[1] = imp[1]; c[2] = imp[2];
                    c[3] = wp[1] * imp[2] - wp[2] * imp[1];
                    c[4] = wp[2] * imp[0] - wp[0] * imp[2];
                    c[5] = wp[0] * imp[1] - wp[1] * imp[0];
                    c[6] = imp[0] * (.5 * (o[0] + n[0])) + imp[1] * (.5 * (o[1] + n[1])) + imp[2] * (.5 * (o[2] + n[2]));
                    c[7] = rq[0]; c[8] = rq[1]; c[9] = rq[2];
                    c[10] = wp[1] * rq[2] - wp[2] * rq[1];
                    c[11] = wp[2] * rq[0] - wp[0] * rq[2];
                    c[12] = wp[0] * rq[1] - wp[1] * rq[0];
                }
            }
        }
        vel = vel + S.dt * S.gravity;
        L.v[i] = Q4<R>{vel.x, vel.y, vel.z, vq.w};
        L.up[i] = uq;
        L.engaged[i] = 0;
        L.engaged[L.N + i] = 0;
        if (S.sphere_enabled) {
            Sphere<R> kicked = *L.sphere;
            kicked.velocity = kicked.velocity + S.dt * S.gravity;
            cand = sphereCandidate(S, kicked, xyz(L.x0[i]) + xyz(uq), vel, vq.w);
        }
        L.candidate[i] = cand ? 1 : 0;
        if (!cand) {
            for (std::uint32_t p = 0; p < S.plane_count; ++p) L.approach[p * L.N + i] = dot(vel, S.planes[p].normal);
            const V3<R> un = xyz(uq) + S.dt * vel;
            L.u[i] = Q4<R>{un.x, un.y, un.z, uq.w};
        }
    }
    if (S.sphere_enabled) {
        const unsigned bits = __ballot_sync(0xffffffffU, cand);
        if ((threadIdx.x & 31) == 0 && i / 32 < (L.N + 31) / 32) L.cand_bits[i / 32] = bits;
    }
}

// ---------------------------------------------------------------------------
// External wrenches (ExternalLoads.hpp:171-238): each wrench's force and
// torque spread over its nodes by mass about their mass centre, from the
// current positions, before every kick. One CTA per wrench. The region's sums
// (mass, centre, inertia tensor, the resultant checks) are folded serially in
// node order as the reference folds them, each sum a chain on its own
// thread, from chunks the CTA stages in shared memory; the eigen-solve of the
// tensor is the reference's cyclic Jacobi in double. apply 1 writes the
// kick's forces (when loads remain); a wrench the current geometry cannot
// carry then stops the lattice before the kick changes anything, with
// kErrWrench set (the reference throws there). apply 0 only validates, into
// *verdict.
// ---------------------------------------------------------------------------
constexpr unsigned kWrenchThreads = 256;

__device__ inline double normD(double x, double y, double z) { return norm3d(x, y, z); }

template <class R>
__device__ __forceinline__ void wrenchSpread(const Dev<R> &L, const WrenchDev *ws, const std::uint32_t *lists,
                                             unsigned *verdict, int apply, unsigned index) {
    Ctl &c = *L.ctl;
    if (apply && (c.stop || c.loads_remaining == 0 || index >= c.wrench_count)) return;
    const WrenchDev w = ws[index];
    const std::uint32_t *list = lists + w.begin;
    const std::uint32_t n = w.end - w.begin;
    const unsigned t = threadIdx.x;
    __shared__ double sm[kWrenchThreads], sr[3][kWrenchThreads], sf[3][kWrenchThreads];
    __shared__ double mass, center[3], tensor[9], alpha[3], moment[3], sums[8];
    __shared__ int bad;
    if (t == 0) bad = 0;
    const std::uint32_t a0 = list[0];
    const V3<R> p0 = xyz(L.x0[a0]) + xyz(L.u[a0]);
    const double anchor[3] = {double(p0.x), double(p0.y), double(p0.z)};
    __syncthreads();
    // One pass over the region: stage(k, slot) for the chunk's nodes, then
    // fold(count) over the staged chunk.
    auto pass = [&](auto &&stage, auto &&fold) {
        for (std::uint32_t base = 0; base < n; base += kWrenchThreads) {
            if (base + t < n) stage(base + t, t);
            __syncthreads();
            fold(n - base < kWrenchThreads ? n - base : kWrenchThreads);
            __syncthreads();
        }
    };
    // Mass and position relative to the anchor; movable, finite nodes only.
    auto stageNode = [&](std::uint32_t k, unsigned j) {
        const std::uint32_t i = list[k];
        const Q4<R> u = L.u[i], v = L.v[i]; // w: inverse mass, mass
        const V3<R> p = xyz(L.x0[i]) + xyz(u);
        sm[j] = double(v.w);
        sr[0][j] = double(p.x) - anchor[0];
        sr[1][j] = double(p.y) - anchor[1];
        sr[2][j] = double(p.z) - anchor[2];
        if (!(v.w > R(0)) || !(u.w > R(0)) || !isfinite(v.w) || !isfinite(u.w) || !isfinite(sr[0][j]) ||
            !isfinite(sr[1][j]) || !isfinite(sr[2][j]))
            bad = 1;
    };
    double acc = 0.0;
    pass(stageNode, [&](unsigned m) {
        if (t == 0)
            for (unsigned j = 0; j < m; ++j) acc += sm[j];
    });
    if (t == 0) {
        mass = acc;
        if (!(acc > 0) || !isfinite(acc)) bad = 1;
    }
    __syncthreads();
    acc = 0.0;
    pass(stageNode, [&](unsigned m) {
        if (t < 3)
            for (unsigned j = 0; j < m; ++j) acc = acc + sr[t][j] * (sm[j] / mass);
    });
    if (t < 3) center[t] = acc;
    __syncthreads();
    acc = 0.0;
    pass(stageNode, [&](unsigned m) {
        if (t < 9) {
            const unsigned a = t / 3, b = t % 3;
            for (unsigned j = 0; j < m; ++j) {
                const double r[3] = {sr[0][j] - center[0], sr[1][j] - center[1], sr[2][j] - center[2]};
                const double share = sm[j] / mass;
                acc = acc + share * (a == b ? r[(a + 1) % 3] * r[(a + 1) % 3] + r[(a + 2) % 3] * r[(a + 2) % 3]
                                            : -r[a] * r[b]);
            }
        }
    });
    if (t < 9) tensor[t] = acc;
    __syncthreads();
    if (t == 0) {
        const double arm[3] = {((w.point[0] - L.origin[0]) - anchor[0]) - center[0],
                               ((w.point[1] - L.origin[1]) - anchor[1]) - center[1],
                               ((w.point[2] - L.origin[2]) - anchor[2]) - center[2]};
        moment[0] = w.torque[0] + (arm[1] * w.force[2] - arm[2] * w.force[1]);
        moment[1] = w.torque[1] + (arm[2] * w.force[0] - arm[0] * w.force[2]);
        moment[2] = w.torque[2] + (arm[0] * w.force[1] - arm[1] * w.force[0]);
        for (int q = 0; q < 3; ++q)
            if (!isfinite(center[q]) || !isfinite(moment[q])) bad = 1;
        double scale = 0.0;
        for (int e = 0; e < 9; ++e) {
            if (!isfinite(tensor[e])) bad = 1;
            const double x = fabs(tensor[e]);
            scale = scale < x ? x : scale;
        }
        double al[3] = {0.0, 0.0, 0.0};
        const double mn = normD(moment[0], moment[1], moment[2]);
        if (!bad && scale > 0) {
            double m9[9], eig[3], axes[9];
            for (int e = 0; e < 9; ++e) m9[e] = tensor[e] / scale;
            jacobi3(m9, eig, axes);
            double largest = fabs(eig[0]);
            largest = largest < fabs(eig[1]) ? fabs(eig[1]) : largest;
            largest = largest < fabs(eig[2]) ? fabs(eig[2]) : largest;
            double un[3] = {moment[0], moment[1], moment[2]};
            for (int axis = 0; axis < 3; ++axis) {
                if (!(eig[axis] > 1e-10 * largest)) continue;
                const double dir[3] = {axes[axis], axes[3 + axis], axes[6 + axis]};
                const double component = dir[0] * moment[0] + dir[1] * moment[1] + dir[2] * moment[2];
                const double sc = component / mass / scale / eig[axis];
                for (int q = 0; q < 3; ++q) {
                    un[q] = un[q] - dir[q] * component;
                    al[q] = al[q] + dir[q] * sc;
                }
            }
            if (normD(un[0], un[1], un[2]) > 1024 * DBL_EPSILON * mn) bad = 1;
        } else if (!bad && mn > 0) {
            bad = 1; // a torque with no sampled lever arm
        }
        for (int q = 0; q < 3; ++q) {
            if (!isfinite(al[q])) bad = 1;
            alpha[q] = al[q];
        }
    }
    __syncthreads();
    // Node forces, written for the kick, then the resultant checks.
    double part = 0.0;
    pass([&](std::uint32_t k, unsigned j) {
        stageNode(k, j);
        const double m = sm[j], share = m / mass;
        const double r[3] = {sr[0][j] - center[0], sr[1][j] - center[1], sr[2][j] - center[2]};
        const double cr[3] = {alpha[1] * r[2] - alpha[2] * r[1], alpha[2] * r[0] - alpha[0] * r[2],
                              alpha[0] * r[1] - alpha[1] * r[0]};
        double f[3];
        for (int q = 0; q < 3; ++q) {
            f[q] = w.force[q] * share + cr[q] * m;
            sr[q][j] = r[q];
            sf[q][j] = f[q];
        }
        const R fx = R(f[0]), fy = R(f[1]), fz = R(f[2]);
        if (!isfinite(f[0]) || !isfinite(f[1]) || !isfinite(f[2]) || !isfinite(fx) || !isfinite(fy) || !isfinite(fz))
            bad = 1;
        if (apply) {
            const std::uint32_t i = list[k];
            L.ext_force[i] = Q4<R>{fx, fy, fz, R(1)};
            L.ext_req[3 * static_cast<std::size_t>(i)] = f[0];
            L.ext_req[3 * static_cast<std::size_t>(i) + 1] = f[1];
            L.ext_req[3 * static_cast<std::size_t>(i) + 2] = f[2];
        }
    }, [&](unsigned m) {
        if (t >= 8) return;
        for (unsigned j = 0; j < m; ++j) {
            const double r[3] = {sr[0][j], sr[1][j], sr[2][j]}, f[3] = {sf[0][j], sf[1][j], sf[2][j]};
            const double mo[3] = {r[1] * f[2] - r[2] * f[1], r[2] * f[0] - r[0] * f[2], r[0] * f[1] - r[1] * f[0]};
            if (t < 3) part = part + f[t];
            else if (t < 6) part = part + mo[t - 3];
            else if (t == 6) part += normD(f[0], f[1], f[2]);
            else part += normD(mo[0], mo[1], mo[2]);
        }
    });
    if (t < 8) sums[t] = part;
    __syncthreads();
    if (t == 0) {
        for (int q = 0; q < 8; ++q)
            if (!isfinite(sums[q])) bad = 1;
        const double fn = normD(w.force[0], w.force[1], w.force[2]);
        const double mn = normD(moment[0], moment[1], moment[2]);
        const double df = normD(sums[0] - w.force[0], sums[1] - w.force[1], sums[2] - w.force[2]);
        const double dm = normD(sums[3] - moment[0], sums[4] - moment[1], sums[5] - moment[2]);
        if (df > 1e-10 * (fn < sums[6] ? sums[6] : fn) || dm > 1e-10 * (mn < sums[7] ? sums[7] : mn)) bad = 1;
        if (bad) {
            if (!apply) {
                atomicOr(verdict, 1U);
            } else if (!(atomicOr(&c.error, kErrWrench) & kErrWrench)) {
                c.stop = 1;
                atomicSub(L.running, 1U);
            }
        }
    }
}

// One lattice's wrenches: one CTA per wrench.
template <class R>
__global__ void __launch_bounds__(kWrenchThreads)
kWrench(const Dev<R> L, const WrenchDev *ws, const std::uint32_t *lists, unsigned *verdict, int apply) {
    wrenchSpread(L, ws, lists, verdict, apply, blockIdx.x);
}

// A batch's wrenches in one launch: one CTA per (lattice, wrench) item.
template <class R>
__global__ void __launch_bounds__(kWrenchThreads) kWrenchMany(const Grid<R> launch) {
    const Work w = launch.list[blockIdx.x];
    const Dev<R> &L = launch.table[w.lattice];
    wrenchSpread(L, L.wrench, L.ext_nodes, nullptr, 1, w.begin);
}

// Ordered candidate lists per slab, capped at 1024 (CpuLatticeBackend.cpp:375-386):
// one CTA per slab scans its bit words in node order.
template <class R, bool Many>
__global__ void __launch_bounds__(1024) kCandidates(const Grid<R> launch) {
    const Work w = item<Many>(launch);
    const Dev<R> L = descriptor<R, Many>(launch, w);
    if (L.ctl->stop) return;
    __shared__ std::uint32_t warp_total[32];
    __shared__ std::uint32_t carry;
    const std::uint32_t blk = w.begin; // one item per (lattice, slab)
    const std::uint32_t nb = L.node_block_begin[blk], ne = L.node_block_begin[blk + 1];
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const std::uint32_t w0 = nb / 32, w1 = ne == nb ? w0 : (ne - 1) / 32 + 1;
    for (std::uint32_t base = w0; base < w1; base += blockDim.x) {
        const std::uint32_t word = base + threadIdx.x;
        std::uint32_t bits = 0;
        if (word < w1) {
            bits = L.cand_bits[word];
            const std::uint32_t lo = word * 32, hi = lo + 32;
            if (nb > lo) bits &= ~0U << (nb - lo);
            if (ne < hi) bits &= (ne - lo) >= 32 ? ~0U : ((1U << (ne - lo)) - 1U);
        }
        const std::uint32_t n = __popc(bits);
        // Block exclusive scan of n.
        std::uint32_t x = n;
        for (int o = 1; o < 32; o <<= 1) {
            const std::uint32_t y = __shfl_up_sync(0xffffffffU, x, o);
            if ((threadIdx.x & 31) >= static_cast<unsigned>(o)) x += y;
        }
        if ((threadIdx.x & 31) == 31) warp_total[threadIdx.x / 32] = x;
        __syncthreads();
        if (threadIdx.x < 32) {
            std::uint32_t t = warp_total[threadIdx.x];
            for (int o = 1; o < 32; o <<= 1) {
                const std::uint32_t y = __shfl_up_sync(0xffffffffU, t, o);
                if (threadIdx.x >= static_cast<unsigned>(o)) t += y;
            }
            warp_total[threadIdx.x] = t;
        }
        __syncthreads();
        std::uint32_t before = carry + x - n + (threadIdx.x >= 32 ? warp_total[threadIdx.x / 32 - 1] : 0U);
        while (bits) {
            const int b = __ffs(bits) - 1;
            bits &= bits - 1;
            if (before < kCandidatesPerBlock) L.cand_list[blk * kCandidatesPerBlock + before] = word * 32 + b;
            ++before;
        }
        __syncthreads();
        if (threadIdx.x == 0) carry += warp_total[31];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const std::uint32_t total = carry;
        L.cand_count[blk] = total < kCandidatesPerBlock ? total : kCandidatesPerBlock;
        // Slabs of one lattice finish in any order: the count is shared.
        if (total > kCandidatesPerBlock)
            atomicAdd(&L.ctl->contact.candidate_overflow,
                      static_cast<unsigned long long>(total - kCandidatesPerBlock));
    }
}

// The contact halo of the substep: per (lattice, slab) item, its listed
// candidates, their neighbours, and the end-sample tiles of every bond at one
// of those nodes. Threads that mark the same entry write the same stamp.
template <class R, bool Many>
__global__ void __launch_bounds__(1024) kMarkHalo(const Grid<R> launch) {
    const Work w = item<Many>(launch);
    const Dev<R> L = descriptor<R, Many>(launch, w);
    if (L.ctl->stop) return;
    const std::uint32_t stamp = substepStamp(L);
    const std::uint32_t n = L.cand_count[w.begin];
    const std::uint32_t *list = L.cand_list + w.begin * kCandidatesPerBlock;
    for (std::uint32_t k = threadIdx.x; k < n; k += blockDim.x) {
        const std::uint32_t c = list[k];
        if (!inBounds(c, L.N, kSiteHalo)) continue;
        L.halo_stamp[c] = stamp;
        for (std::uint32_t q = 0; q < L.D; ++q) {
            const std::size_t slot = static_cast<std::size_t>(q) * L.N + c;
            const std::uint32_t o = L.nbr_other[slot];
            if (!inBounds(o, L.N, kSiteHalo)) continue;
            L.halo_stamp[o] = stamp;
            for (std::uint32_t r = 0; r < L.D; ++r) {
                const std::uint32_t bd = L.nbr_bond[static_cast<std::size_t>(r) * L.N + o];
                if (bd != kNoBond && inBounds(bd, L.B, kSiteHalo)) L.late_tile_stamp[bd / kThreads] = stamp;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Sphere contact (LatticePhysics.hpp:1322-1428): candidates in slab, then node
// order, one contact at a time -- every contact moves the sphere the next one
// sees, so that chain is serial by definition. It runs on one warp of one
// CTA per lattice; everything that does not depend on the sphere's changing
// state is computed by the whole CTA around it.
//
// A candidate's node data are staged in shared memory. In pass 1 the sphere
// centre cannot move (only pass 2 corrects positions), so the offset r, its
// length and unit normal, the gap, the inverse masses and the effective
// inverse mass along the normal are computed in parallel before the chain,
// with the reference's expressions; the chain then starts at the relative
// velocity. In pass 2 the parallel part is the node's position and masses.
// ---------------------------------------------------------------------------
template <class R> struct Staged {
    V3<R> p;       // position x0 + u (pass 2), or r = p - centre (pass 1)
    V3<R> normal;  // pass 1: normalized(r)
    R gap;         // pass 1: |r| - (sphere radius + node contact radius)
    R eff_n;       // pass 1: effective inverse mass along the normal
    R inm;         // 1 / mass
    R before;      // the node's kinetic energy as the pass reaches it
    Q4<R> u, v;    // u (w: inv_mass), v (w: mass)
};

// What one hit adds to the contact ledger's FP64 sums, in backend precision:
// the chain writes it to a log in shared memory and goes on, and the fold
// lanes widen and add it in log order (LatticePhysics.hpp:1354-1381), so the
// FP64 adds stay off the serial chain.
template <class R> struct ContactLog {
    R normal_imp[3], friction_imp[3];
    R lost;            // the node's kinetic energy before minus after
    unsigned friction; // friction_imp applies
};

// Bytes of shared memory per staging buffer of the contact pass: a slab's
// staged candidates and the log of its hits.
template <class R> constexpr unsigned sphereSlabBytes() {
    return kCandidatesPerBlock * static_cast<unsigned>(sizeof(Staged<R>) + sizeof(ContactLog<R>));
}

template <class R>
__device__ __forceinline__ void contactApply(V3<R> imp, V3<R> r, R inm, R ism, R iin, V3<R> &nv, Sphere<R> &sp) {
    nv = nv + inm * imp;
    sp.velocity = sp.velocity - ism * imp;
    const V3<R> ti = -cross(r, imp);
    sp.angular = sp.angular + iin * ti;
}

// A candidate against the current sphere state: 0 outside the contact gate
// (LatticePhysics.hpp:1338-1342; nothing happens), 1 a graze (past the gate,
// but no normal impulse and no position correction: it only raises the
// penetration record), 2 a hit (it changes the node and the sphere). The
// normal relative velocity and the normal impulse come back for the hit.
template <class R>
__device__ __forceinline__ int contactProbe(const Settings<R> &S, const Sphere<R> &sp, V3<R> nv, V3<R> r,
                                            V3<R> normal, R gap, R eff_n, bool correct, R &vn, R &ni) {
    const V3<R> rel = nv - sp.velocity - cross(sp.angular, r);
    vn = dot(rel, normal);
    if (gap > maxR(S.c_margin, -vn * S.dt)) return 0;
    const R restitution = -vn > S.c_threshold ? S.c_restitution : R(0);
    const R desired = gap > S.c_margin ? -gap / S.dt : -restitution * minR(vn, R(0));
    ni = maxR(R(0), (desired - vn) / eff_n);
    return (ni > R(0) || (correct && gap < -S.c_margin)) ? 2 : 1;
}

// The contact of one staged candidate past the gate, from its normal
// relative velocity and normal impulse on (LatticePhysics.hpp:1343-1386).
// `max_pen` and `max_corr` shadow acc.max_penetration and acc.max_correction
// in R: the ledger only ever holds a widened R, so the comparisons are the
// reference's. A hit's ledger sums go to `log`; it returns whether it hit.
template <class R>
__device__ __forceinline__ bool contactChain(const Settings<R> &S, Sphere<R> &sp, Staged<R> &c, V3<R> r, V3<R> normal,
                                             R gap, R ni, R ism, R iin, bool correct, ContactAcc &acc, R &max_pen,
                                             R &max_corr, ContactLog<R> &log) {
    V3<R> nv = xyz(c.v);
    if (-gap > max_pen) {
        max_pen = -gap;
        acc.max_penetration = static_cast<double>(-gap);
    }
    const R inm = c.inm;
    const R mass = c.v.w;
    const bool hit = ni > R(0);
    if (hit) {
        const V3<R> imp = ni * normal;
        contactApply(imp, r, inm, ism, iin, nv, sp);
        log.normal_imp[0] = imp.x;
        log.normal_imp[1] = imp.y;
        log.normal_imp[2] = imp.z;
        log.friction = 0;
        const V3<R> after = nv - sp.velocity - cross(sp.angular, r);
        const V3<R> tangent = after - dot(after, normal) * normal;
        const R ts = length(tangent);
        if (ts > R(1.0e-12)) {
            const V3<R> d = tangent / ts;
            const V3<R> rd = cross(r, d);
            const R stick = ts / (inm + ism + iin * dot(rd, rd));
            const R fi = stick <= S.c_static * ni ? stick : minR(stick, S.c_dynamic * ni);
            const V3<R> fimp = -fi * d;
            contactApply(fimp, r, inm, ism, iin, nv, sp);
            log.friction_imp[0] = fimp.x;
            log.friction_imp[1] = fimp.y;
            log.friction_imp[2] = fimp.z;
            log.friction = 1;
        }
        c.v = Q4<R>{nv.x, nv.y, nv.z, mass};
        log.lost = c.before - R(0.5) * mass * dot(nv, nv);
        ++acc.impulse_contacts;
    }
    if (correct && gap < -S.c_margin) {
        const R corr = minR(-gap - S.c_margin, R(0.2) * maxR(S.c_node_radius, sp.radius * R(0.01)));
        const R sum = inm + ism;
        const V3<R> ns = (corr * inm / sum) * normal;
        const V3<R> ss = -((corr * ism / sum) * normal);
        const V3<R> un = xyz(c.u) + ns;
        c.u = Q4<R>{un.x, un.y, un.z, c.u.w};
        sp.center = sp.center + ss;
        if (corr > max_corr) {
            max_corr = corr;
            acc.max_correction = static_cast<double>(corr);
        }
    }
    return hit;
}

constexpr unsigned kSphereThreads = 256;
// Staging buffers of the contact pass: with two, the chain of one slab runs on
// warp 0 while warp 1 folds the ledger log of the slab before it and the other
// warps write back the slab before it from the other buffer and then stage
// the slab after it into that buffer (a thread writes back and stages the
// same buffer slots, so no barrier is needed between); with one (when two do
// not fit the device's shared memory), one slab at a time.

// The chain runs on warp 0, with every lane holding the same sphere state and
// ledgers. Only a candidate that passes the contact gate changes anything, so
// the lanes test the next 32 candidates against the current state at once; the
// first that passes is applied (by every lane, identically) and the scan
// resumes after it. The candidates skipped were tested against exactly the
// state the serial order shows them, so the result is the serial chain's.
// Slabs are disjoint sets of nodes: staging one slab's candidates, running
// another's chain and writing back a third's touch different nodes.
//
// The ledger's four FP64 sums (impulse x, y, z and dissipated energy) are four
// independent serial folds; lanes 0-3 of warp 1 run one each over the hit
// logs, slab after slab, in the order the chain wrote them.
template <class R, bool Many>
__global__ void __launch_bounds__(kSphereThreads) kSpherePass(const Grid<R> launch, Settings<R> S, int pass,
                                                              unsigned buffers) {
    const Work w = item<Many>(launch);
    const Dev<R> L = descriptor<R, Many>(launch, w);
    extern __shared__ __align__(16) unsigned char sphere_smem[];
    Staged<R> *stage_base = reinterpret_cast<Staged<R> *>(sphere_smem);
    ContactLog<R> *log_base =
        reinterpret_cast<ContactLog<R> *>(sphere_smem + buffers * kCandidatesPerBlock * sizeof(Staged<R>));
    __shared__ Sphere<R> start;
    __shared__ unsigned log_count[2];
    __shared__ double folded[4];
    if (L.ctl->stop) return;
    const unsigned lane = threadIdx.x & 31U;
    const bool chain = threadIdx.x < 32;
    const bool fold = threadIdx.x >= 32 && threadIdx.x < 36;
    Sphere<R> sp{};
    ContactAcc acc{};
    V3<R> c0{};
    R e0 = R(0), max_pen = R(0), max_corr = R(0);
    double sum = 0.0; // the fold lane's ledger sum
    if (chain) {
        sp = *L.sphere;
        if (pass == 1) sp.velocity = sp.velocity + S.dt * S.gravity; // the kicked sphere becomes the state
        acc = L.ctl->contact;
        max_pen = R(acc.max_penetration);
        max_corr = R(acc.max_correction);
        c0 = sp.center;
        e0 = R(0.5) * sp.mass * dot(sp.velocity, sp.velocity) + R(0.5) * sp.inertia * dot(sp.angular, sp.angular);
        if (threadIdx.x == 0) start = sp;
    } else if (fold) {
        const ContactAcc &a = L.ctl->contact;
        sum = lane == 0 ? a.impulse_x : lane == 1 ? a.impulse_y : lane == 2 ? a.impulse_z : a.dissipated;
    }
    __syncthreads();
    // Constant over the pass: the sphere's mass and inertia never change.
    const R ism = R(1) / start.mass;
    const R iin = R(1) / start.inertia;
    const R cr = start.radius + S.c_node_radius;

    // A slab's candidates into a buffer, by threads [t0, t0 + nt).
    auto stageSlab = [&](std::uint32_t b, Staged<R> *st, unsigned t0, unsigned nt) {
        const std::uint32_t n = L.cand_count[b];
        const std::uint32_t *list = L.cand_list + b * kCandidatesPerBlock;
        for (std::uint32_t k = threadIdx.x - t0; k < n; k += nt) {
            const std::uint32_t i = list[k];
            Staged<R> c;
            if (!inBounds(i, L.N, kSiteCandidate)) {
                c = Staged<R>{}; // no mass: the chain passes it by
                st[k] = c;
                continue;
            }
            c.u = L.u[i];
            c.v = L.v[i];
            const R mass = c.v.w;
            const V3<R> p = xyz(L.x0[i]) + xyz(c.u);
            c.inm = R(1) / mass;
            c.before = R(0.5) * mass * dot(xyz(c.v), xyz(c.v));
            if (pass == 1) {
                const V3<R> r = p - start.center;
                const R distance = length(r);
                const V3<R> normal = normalized(r);
                const V3<R> rn = cross(r, normal);
                c.p = r;
                c.normal = normal;
                c.gap = distance - cr;
                c.eff_n = c.inm + ism + iin * dot(rn, rn);
            } else {
                c.p = p;
            }
            st[k] = c;
        }
    };
    // A slab's candidates back to the node arrays, by threads [t0, t0 + nt).
    auto writeBack = [&](std::uint32_t b, const Staged<R> *st, unsigned t0, unsigned nt) {
        const std::uint32_t n = L.cand_count[b];
        const std::uint32_t *list = L.cand_list + b * kCandidatesPerBlock;
        for (std::uint32_t k = threadIdx.x - t0; k < n; k += nt) {
            const std::uint32_t i = list[k];
            if (!inBounds(i, L.N, kSiteCandidate)) continue;
            const Q4<R> vq = st[k].v;
            const Q4<R> uq = st[k].u;
            if (pass == 1) {
                for (std::uint32_t p = 0; p < S.plane_count; ++p)
                    L.approach[p * L.N + i] = dot(xyz(vq), S.planes[p].normal);
                const V3<R> un = xyz(uq) + S.dt * xyz(vq);
                L.u[i] = Q4<R>{un.x, un.y, un.z, uq.w};
                L.v[i] = vq;
            } else {
                V3<R> vel = xyz(vq);
                for (std::uint32_t p = 0; p < S.plane_count; ++p)
                    if (L.engaged[p * L.N + i]) vel = supportVelocity(S.planes[p], vel, L.approach[p * L.N + i]);
                L.u[i] = uq;
                L.v[i] = Q4<R>{vel.x, vel.y, vel.z, vq.w};
            }
        }
    };
    // A slab's hit log into the fold lanes' sums (lane q: sum q).
    auto foldLog = [&](const ContactLog<R> *lg, unsigned n) {
        if (lane < 3) {
            for (unsigned e = 0; e < n; ++e) {
                sum += static_cast<double>(lg[e].normal_imp[lane]);
                if (lg[e].friction) sum += static_cast<double>(lg[e].friction_imp[lane]);
            }
        } else {
            for (unsigned e = 0; e < n; ++e) sum += static_cast<double>(lg[e].lost);
        }
    };
    // The serial chain over a staged slab, on warp 0; its hits go to `lg`.
    auto runChain = [&](std::uint32_t n, Staged<R> *st, ContactLog<R> *lg, unsigned &logged) {
        std::uint32_t k0 = 0;
        unsigned hits = 0;
        while (k0 < n) {
            const std::uint32_t k = k0 + lane;
            // hit: the contact changes the sphere or the node (an impulse, or
            // a position correction in pass 2). graze: it passes the gate but
            // only raises the penetration record, a maximum that any order
            // forms alike.
            bool hit = false, graze = false;
            R pen = R(0);
            V3<R> r{}, normal{};
            R gap = R(0), eff_n = R(0), vn = R(0), ni = R(0);
            if (k < n) {
                const Staged<R> &c = st[k];
                if (c.v.w > R(0)) {
                    if (pass == 1) {
                        r = c.p;
                        normal = c.normal;
                        gap = c.gap;
                        eff_n = c.eff_n;
                    } else {
                        r = c.p - sp.center;
                        const R distance = length(r);
                        normal = normalized(r);
                        const V3<R> rn = cross(r, normal);
                        eff_n = c.inm + ism + iin * dot(rn, rn);
                        gap = distance - cr;
                    }
                    const int probe = contactProbe(S, sp, xyz(c.v), r, normal, gap, eff_n, pass == 2, vn, ni);
                    hit = probe == 2;
                    graze = probe == 1;
                    pen = -gap;
                }
            }
            const unsigned mask = __ballot_sync(0xffffffffU, hit);
            const unsigned limit = mask ? static_cast<unsigned>(__ffs(mask) - 1) : 32U;
            // The grazes before the first hit raise the record as the serial
            // chain would have, one after another.
            const bool raises = graze && lane < limit && pen > max_pen;
            if (__any_sync(0xffffffffU, raises)) {
                R best = raises ? pen : max_pen;
                if constexpr (std::is_same<R, float>::value) {
                    // The record starts at zero and only grows, so a raising
                    // value is positive and its bits order as its value.
                    best = __uint_as_float(__reduce_max_sync(0xffffffffU, __float_as_uint(best)));
                } else {
                    for (int o = 16; o > 0; o >>= 1) {
                        const R other = __shfl_xor_sync(0xffffffffU, best, o);
                        best = other > best ? other : best;
                    }
                }
                if (best > max_pen) {
                    max_pen = best;
                    acc.max_penetration = static_cast<double>(best);
                }
            }
            if (mask == 0) {
                k0 += 32;
                continue;
            }
            const std::uint32_t j = k0 + limit;
            Staged<R> c = st[j];
            // The hit lane's geometry, computed in the scan against the state
            // the chain is in, to every lane.
            const int src = static_cast<int>(limit);
            const V3<R> hr{__shfl_sync(0xffffffffU, r.x, src), __shfl_sync(0xffffffffU, r.y, src),
                           __shfl_sync(0xffffffffU, r.z, src)};
            const V3<R> hn{__shfl_sync(0xffffffffU, normal.x, src), __shfl_sync(0xffffffffU, normal.y, src),
                           __shfl_sync(0xffffffffU, normal.z, src)};
            const R hgap = __shfl_sync(0xffffffffU, gap, src);
            const R hni = __shfl_sync(0xffffffffU, ni, src);
            ContactLog<R> entry;
            const bool logs = contactChain(S, sp, c, hr, hn, hgap, hni, ism, iin, pass == 2, acc, max_pen, max_corr,
                                           entry);
            __syncwarp();
            if (lane == 0) {
                st[j] = c;
                if (logs) lg[hits] = entry;
            }
            hits += logs ? 1U : 0U;
            k0 = j + 1;
        }
        if (lane == 0) logged = hits;
    };
    // The next slab with candidates after b (L.blocks: none).
    auto nextSlab = [&](std::uint32_t b) {
        while (b < L.blocks && L.cand_count[b] == 0) ++b;
        return b;
    };

    if (buffers == 2) {
        std::uint32_t cur = nextSlab(0);
        if (cur < L.blocks) stageSlab(cur, stage_base, 0, blockDim.x);
        __syncthreads();
        std::uint32_t prev = L.blocks;
        unsigned cb = 0;
        while (cur < L.blocks) {
            const std::uint32_t nxt = nextSlab(cur + 1);
            const unsigned ob = cb ^ 1U;
            if (chain) {
                runChain(L.cand_count[cur], stage_base + cb * kCandidatesPerBlock, log_base + cb * kCandidatesPerBlock,
                         log_count[cb]);
            } else if (threadIdx.x < 64) {
                if (fold && prev < L.blocks) foldLog(log_base + ob * kCandidatesPerBlock, log_count[ob]);
            } else {
                Staged<R> *other = stage_base + ob * kCandidatesPerBlock;
                if (prev < L.blocks) writeBack(prev, other, 64, blockDim.x - 64);
                if (nxt < L.blocks) stageSlab(nxt, other, 64, blockDim.x - 64);
            }
            __syncthreads();
            prev = cur;
            cur = nxt;
            cb = ob;
        }
        if (prev < L.blocks) {
            if (fold) foldLog(log_base + (cb ^ 1U) * kCandidatesPerBlock, log_count[cb ^ 1U]);
            writeBack(prev, stage_base + (cb ^ 1U) * kCandidatesPerBlock, 0, blockDim.x);
        }
    } else {
        for (std::uint32_t b = nextSlab(0); b < L.blocks; b = nextSlab(b + 1)) {
            stageSlab(b, stage_base, 0, blockDim.x);
            __syncthreads();
            if (chain) runChain(L.cand_count[b], stage_base, log_base, log_count[0]);
            __syncthreads();
            if (fold) foldLog(log_base, log_count[0]);
            writeBack(b, stage_base, 0, blockDim.x);
            __syncthreads();
        }
    }
    if (fold) folded[lane] = sum;
    __syncthreads();
    if (threadIdx.x == 0) {
        acc.impulse_x = folded[0];
        acc.impulse_y = folded[1];
        acc.impulse_z = folded[2];
        acc.dissipated = folded[3];
        const R e1 = R(0.5) * sp.mass * dot(sp.velocity, sp.velocity) + R(0.5) * sp.inertia * dot(sp.angular, sp.angular);
        acc.dissipated += static_cast<double>(e0 - e1);
        const R shift = length(sp.center - c0);
        if (shift > R(acc.max_center_shift)) acc.max_center_shift = static_cast<double>(shift);
        *L.sphere = sp;
        L.ctl->contact = acc;
    }
}

// ---------------------------------------------------------------------------
// XPBD projection of one level (LatticePhysics.hpp:1132-1168), one bond per
// thread over the level's contiguous storage range [begin, end).
//
// Support (LatticePhysics.hpp:1255-1261) rides on the sweep: the reference
// projects every node out of the support planes after the whole sweep; here a
// node is projected by the thread that ran its last bond of the sweep (the
// record's last-of flags), right after that bond. Nothing later in the sweep
// touches the node and the projection reads only the node itself, so the
// result is the reference's, and the separate pass over the nodes is gone. A
// broken or degenerate last bond still carries its nodes' projection.
// ---------------------------------------------------------------------------
template <class R>
__device__ __forceinline__ bool supportProject(const Dev<R> &L, const Settings<R> &S, std::uint32_t i, V3<R> &u) {
    const V3<R> x0 = xyz(L.x0[i]);
    bool projected = false;
    for (std::uint32_t p = 0; p < S.plane_count; ++p) {
        bool here = false;
        const R depth = projectSupport(S.planes[p], x0, u, L.approach[p * L.N + i], S.dt, here);
        if (depth > R(0)) L.engaged[p * L.N + i] = 1;
        projected = projected || here;
    }
    return projected;
}

// Bonds per thread of the sweep and the sweep CTAs an SM keeps resident: a
// thread issues the record loads of all its bonds, then all their gathers,
// then solves them. A level's bonds share no node, so the order among them is
// free. Measured on GB300 (impact 256x128x128, sweep ms per substep): one bond
// per thread with six 256-thread CTAs per SM 2.50; two bonds, four CTAs 2.66;
// one bond, eight CTAs (spilling at 32 registers) 2.76; two bonds, five CTAs
// 2.93.
#ifndef GBL_SOLVE_PER
#define GBL_SOLVE_PER 1
#endif
#ifndef GBL_SOLVE_MIN_BLOCKS
#define GBL_SOLVE_MIN_BLOCKS 6
#endif
constexpr int kSolvePer = GBL_SOLVE_PER;

// Programmatic dependent launch (sm_90+): a sweep level is launched while the
// previous one still runs; its CTAs load what no earlier kernel of the substep
// writes (records, geometry, multipliers, plastic extension, the stop flag),
// then wait for the previous grid to finish and its writes to be visible
// before they touch the nodes. A level lets the next one launch only after its
// own wait, so at most two levels overlap and everything before the previous
// level is complete when a level starts.
__device__ __forceinline__ void waitPreviousGrid() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void allowNextGrid() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// The projection of one live bond (LatticePhysics.hpp:1132-1168) from its
// record, geometry, multiplier and plastic extension and its gathered nodes;
// the multiplier is stored unless this is the last iteration. Returns whether
// the nodes moved (a degenerate bond leaves them).
template <class R, bool Direct, bool Plastic>
__device__ __forceinline__ bool projectBond(const Dev<R> &L, const Settings<R> &S, std::uint32_t d,
                                            const BondRec<R> &rec, const Q4<R> &g, R lambda, R plastic, bool last,
                                            Q4<R> &qa, Q4<R> &qb) {
    const std::uint32_t a = endA(rec), b = endB(rec);
    const V3<R> ua = xyz(qa), ub = xyz(qb), edge{g.x, g.y, g.z};
    const V3<R> delta = Direct ? (xyz(L.x0[b]) + ub) - (xyz(L.x0[a]) + ua) : edge + (ub - ua);
    const R cl = length(delta);
    if (!(cl > R(1.0e-12))) return false;
    const R original = rec.rest;
    const R rest = Plastic ? original + plastic : original;
    R constraint;
    if (Direct) {
        constraint = cl - rest;
    } else {
        const V3<R> du = ub - ua;
        const R num = rec.rsm + R(2) * dot(edge, du) + dot(du, du);
        constraint = (Plastic ? num - plastic * (rest + original) : num) / (cl + rest);
    }
    const V3<R> dir = delta / cl;
    const R wa = qa.w, wb = qb.w;
    const R alpha = g.w / (S.dt * S.dt);
    const R dl = (-constraint - alpha * lambda) / (wa + wb + alpha);
    if (!last) __stcs(L.lambda + d, lambda + dl);
    const V3<R> na = ua - (wa * dl) * dir;
    const V3<R> nb = ub + (wb * dl) * dir;
    qa = Q4<R>{na.x, na.y, na.z, wa};
    qb = Q4<R>{nb.x, nb.y, nb.z, wb};
    return true;
}

// The support projection of a node after its last bond of the sweep.
template <class R>
__device__ __forceinline__ void supportLast(const Dev<R> &L, const Settings<R> &S, std::uint32_t i, bool have,
                                            Q4<R> &q, bool &write) {
    if (!have) q = L.u[i];
    V3<R> u = xyz(q);
    if (supportProject(L, S, i, u)) {
        q = Q4<R>{u.x, u.y, u.z, q.w};
        write = true;
    }
}
// A bond's projection, then the support projection of the nodes whose last
// bond of the sweep it is, then the write-back of what moved.
template <class R, bool Direct, bool Plastic, bool Support>
__device__ __forceinline__ void finishBond(const Dev<R> &L, const Settings<R> &S, std::uint32_t d,
                                           const BondRec<R> &rec, bool live, const Q4<R> &g, R lambda, R plastic,
                                           bool last, Q4<R> qa, Q4<R> qb) {
    const std::uint32_t a = endA(rec), b = endB(rec);
    bool write_a = false, write_b = false;
    if (live) write_a = write_b = projectBond<R, Direct, Plastic>(L, S, d, rec, g, lambda, plastic, last, qa, qb);
    if (Support) {
        if (rec.a & kLastABit) supportLast(L, S, a, live, qa, write_a);
        if (rec.b & kLastBBit) supportLast(L, S, b, live, qb, write_b);
    }
    if (write_a) L.u[a] = qa;
    if (write_b) L.u[b] = qb;
}

template <class R, bool Many, bool Direct, bool First, bool Last, bool Plastic, bool Support>
__global__ void __launch_bounds__(kThreads, GBL_SOLVE_MIN_BLOCKS) kSolve(const Grid<R> launch, Settings<R> S) {
    const Work w = item<Many>(launch);
    const Dev<R> L = descriptor<R, Many>(launch, w);
    BondRec<R> rec[kSolvePer];
    Q4<R> geo[kSolvePer], qa[kSolvePer], qb[kSolvePer];
    R lam[kSolvePer], pl[kSolvePer];
    std::uint32_t at[kSolvePer];
    // Everything that no kernel since the last end sample has written.
#pragma unroll
    for (int k = 0; k < kSolvePer; ++k) {
        at[k] = w.begin + threadIdx.x + static_cast<std::uint32_t>(k) * kThreads;
        if (at[k] < w.end) {
            rec[k] = ldStream(L.rec + at[k]);
            geo[k] = ldStream(L.geo + at[k]);
            lam[k] = First ? R(0) : __ldcs(L.lambda + at[k]);
            pl[k] = Plastic ? L.plastic[at[k]].x : R(0);
        }
    }
    const unsigned stop = L.ctl->stop;
    waitPreviousGrid();
    allowNextGrid();
    if (stop) return;
    bool live[kSolvePer], ok[kSolvePer];
#pragma unroll
    for (int k = 0; k < kSolvePer; ++k) {
        ok[k] = at[k] < w.end && endsInBounds(rec[k], L.N, kSiteSolve);
        live[k] = ok[k] && !(rec[k].a & kDeadBit);
        if (live[k]) {
            qa[k] = ldShared(L.u + endA(rec[k]));
            qb[k] = ldShared(L.u + endB(rec[k]));
        }
    }
#pragma unroll
    for (int k = 0; k < kSolvePer; ++k)
        if (ok[k])
            finishBond<R, Direct, Plastic, Support>(L, S, at[k], rec[k], live[k], geo[k], lam[k], pl[k], Last, qa[k],
                                                    qb[k]);
}

// The whole sweep of one lattice in one CTA: every iteration, every level in
// order with a barrier between levels, then the isolated nodes' support. A
// lattice of a batch small enough for one CTA runs here, so its nodes stay in
// L2 (and the SM's L1) across all its levels instead of being streamed from
// HBM again at every level launch; the arithmetic and the per-node order are
// those of the level launches.
// The CTA size (256, 512 or 1024 threads) is a launch shape the batch's
// autotuner picks; two CTAs per SM below 1024 threads.
constexpr unsigned kSweepThreads = 512; // the default shape
constexpr std::uint32_t kMaxFusedLevels = 1024;
// A lattice's one-CTA sweep takes as long as its bonds over one CTA's rate, so
// only lattices small enough to finish well within the batch's level launches
// are swept whole (measured: a 48^3 trial alone in one CTA bounded the whole
// batch's sweep). The default bound; the autotuner picks its own.
constexpr std::uint32_t kMaxFusedBonds = 1U << 18;

template <class R, bool Support>
__device__ __forceinline__ void supportIsolatedInCta(const Dev<R> &L, const Settings<R> &S) {
    if (!Support || !L.isolated_count) return;
    __syncthreads();
    for (std::uint32_t t = threadIdx.x; t < L.isolated_count; t += blockDim.x) {
        const std::uint32_t i = L.isolated[t];
        if (!inBounds(i, L.N, kSiteIsolated)) continue;
        const Q4<R> uq = L.u[i];
        V3<R> u = xyz(uq);
        if (supportProject(L, S, i, u)) L.u[i] = Q4<R>{u.x, u.y, u.z, uq.w};
    }
}

// Shared-memory staging of a small lattice's nodes for its one-CTA sweep: the
// whole position array (one 16-byte record per node) comes in by one bulk
// copy (the copy engine, cp.async.bulk, completing on an mbarrier), every
// gather and write of the sweep then stays in the SM, and the array goes back
// to global memory once at the end. The waits are bounded: a copy that has
// not landed after kStageSpins polls marks the lattice's control block with
// kErrStageWait (the host reports it), waits as long again for the copy to
// drain, and the CTA leaves.
constexpr std::uint32_t kStageSpins = 1U << 26;
// Positions the staged sweep holds: 14,336 x 16 B = 224 KiB of dynamic shared
// memory, with the descriptor and the barrier inside the 227 KiB a CTA may take.
constexpr std::uint32_t kStagedMaxNodes = 14336;
constexpr std::uint32_t kStageChunk = 32768; // bytes per bulk copy

__device__ __forceinline__ std::uint32_t smemAddress(const void *p) {
    return static_cast<std::uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ bool barrierDone(std::uint64_t *bar, std::uint32_t parity) {
    std::uint32_t done;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(done)
                 : "r"(smemAddress(bar)), "r"(parity)
                 : "memory");
    return done != 0;
}
__device__ __forceinline__ bool waitBarrier(std::uint64_t *bar, std::uint32_t parity) {
    for (std::uint32_t spin = 0; spin < kStageSpins; ++spin)
        if (barrierDone(bar, parity)) return true;
    return false;
}

// The CTA's nodes [0, n) from global `src` into shared `dst` (n x 16 bytes,
// both 16-byte aligned). Returns false, after the bounded drain, when the
// copy did not land in time (every thread returns the same).
template <class R>
__device__ bool stageNodesIn(Q4<R> *dst, const Q4<R> *src, std::uint32_t n, std::uint64_t *bar, Ctl *ctl) {
    const std::uint32_t bytes = n * static_cast<std::uint32_t>(sizeof(Q4<R>));
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smemAddress(bar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smemAddress(bar)), "r"(bytes)
                     : "memory");
        for (std::uint32_t off = 0; off < bytes; off += kStageChunk) {
            const std::uint32_t len = bytes - off < kStageChunk ? bytes - off : kStageChunk;
            asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
                             "r"(smemAddress(reinterpret_cast<unsigned char *>(dst) + off)),
                         "l"(__cvta_generic_to_global(reinterpret_cast<const unsigned char *>(src) + off)), "r"(len),
                         "r"(smemAddress(bar))
                         : "memory");
        }
    }
    __syncthreads(); // the barrier is initialised before anyone waits on it
    const bool landed = waitBarrier(bar, 0);
    if (__syncthreads_and(landed ? 1 : 0)) return true;
    if (threadIdx.x == 0) atomicOr(&ctl->error, kErrStageWait);
    (void)waitBarrier(bar, 0); // the copy still writes this CTA's shared memory: let it drain
    __syncthreads();
    return false;
}

template <class R, bool Direct, bool Plastic, bool Support, unsigned T, bool Staged = false>
__global__ void __launch_bounds__(T, T >= 1024 ? 1 : 2) kSweepLattice(const Grid<R> launch, Settings<R> S) {
    // The lattice's descriptor, copied once into shared memory: its fields
    // are read throughout the sweep, and shared memory is never written by
    // the sweep's global stores, so the compiler may keep them as it likes.
    __shared__ __align__(16) unsigned char desc[sizeof(Dev<R>)];
    __shared__ std::uint64_t stage_bar;
    extern __shared__ __align__(128) unsigned char sweep_nodes[];
    {
        const Work w = item<true>(launch);
        const unsigned *src = reinterpret_cast<const unsigned *>(launch.table + w.lattice);
        unsigned *dst = reinterpret_cast<unsigned *>(desc);
        for (unsigned k = threadIdx.x; k < sizeof(Dev<R>) / sizeof(unsigned); k += blockDim.x) dst[k] = src[k];
    }
    __syncthreads();
    Q4<R> *const global_u = reinterpret_cast<const Dev<R> *>(desc)->u;
    const std::uint32_t node_count = reinterpret_cast<const Dev<R> *>(desc)->N;
    if (reinterpret_cast<const Dev<R> *>(desc)->ctl->stop) return;
    if constexpr (Staged) {
        // The sweep's node reads and writes go to the staged copy: the
        // shared-memory descriptor's position pointer is swapped for it
        // (generic loads and stores reach shared memory through it).
        Q4<R> *nodes = reinterpret_cast<Q4<R> *>(sweep_nodes);
        if (!stageNodesIn(nodes, global_u, node_count, &stage_bar, reinterpret_cast<const Dev<R> *>(desc)->ctl))
            return;
        if (threadIdx.x == 0) reinterpret_cast<Dev<R> *>(desc)->u = nodes;
        __syncthreads();
    }
    const Dev<R> &L = *reinterpret_cast<const Dev<R> *>(desc);
    const unsigned I = S.iterations;
    // One bond per thread per round; the rounds of the whole sweep in order
    // (iteration, level, base). The next round's streamed data (record,
    // geometry, multiplier, plastic extension: nothing the node updates
    // touch) is loaded before the current round's node gathers, so two
    // rounds' memory traffic is in flight. A round's multipliers are written
    // one iteration before the round reads them, except in a sweep of one
    // round per iteration, whose next round is itself: there they are loaded
    // after the write.
    struct Round {
        unsigned it;
        std::uint32_t lv, base;
    };
    struct Streamed {
        BondRec<R> rec;
        Q4<R> geo;
        R lam, pl;
    };
    auto advance = [&](Round &r) {
        r.base += T;
        if (r.base < L.level_begin[r.lv + 1]) return true;
        if (++r.lv == L.level_count) {
            r.lv = 0;
            if (++r.it == I) return false;
        }
        r.base = L.level_begin[r.lv];
        return true;
    };
    const bool self_next = L.level_count == 1 && L.level_begin[1] - L.level_begin[0] <= T;
    auto load = [&](const Round &r, Streamed &x) {
        const std::uint32_t d = r.base + threadIdx.x;
        if (d < L.level_begin[r.lv + 1]) {
            x.rec = ldStream(L.rec + d);
            x.geo = ldStream(L.geo + d);
            x.lam = (r.it == 0 || self_next) ? R(0) : __ldcs(L.lambda + d);
            x.pl = Plastic ? L.plastic[d].x : R(0);
        }
    };
    Round cur{0, 0, L.level_begin[0]};
    Streamed now{}, next{};
    load(cur, now);
    for (;;) {
        Round nxt = cur;
        const bool more = advance(nxt);
        if (more) load(nxt, next);
        const std::uint32_t end = L.level_begin[cur.lv + 1];
        const std::uint32_t d = cur.base + threadIdx.x;
        if (d < end && endsInBounds(now.rec, L.N, kSiteSolve)) {
            if (self_next && cur.it != 0) now.lam = __ldcs(L.lambda + d);
            const bool live = !(now.rec.a & kDeadBit);
            Q4<R> qa{}, qb{};
            if (live) {
                if constexpr (Staged) {
                    qa = L.u[endA(now.rec)];
                    qb = L.u[endB(now.rec)];
                } else {
                    qa = ldShared(L.u + endA(now.rec));
                    qb = ldShared(L.u + endB(now.rec));
                }
            }
            finishBond<R, Direct, Plastic, Support>(L, S, d, now.rec, live, now.geo, now.lam, now.pl,
                                                    cur.it + 1 == I, qa, qb);
        }
        if (!more) {
            supportIsolatedInCta<R, Support>(L, S);
            if constexpr (Staged) {
                // The staged positions back to global memory.
                __syncthreads();
                for (std::uint32_t i = threadIdx.x; i < node_count; i += blockDim.x) global_u[i] = L.u[i];
            }
            break;
        }
        if (nxt.lv != cur.lv || nxt.it != cur.it) {
            __syncthreads();
            if (nxt.it != cur.it) {
                supportIsolatedInCta<R, Support>(L, S);
                __syncthreads();
            }
        }
        cur = nxt;
        now = next;
    }
}

// Radial pair damping of one level (LatticePhysics.hpp:1170-1184).
template <class R, bool Many, bool Direct>
__global__ void __launch_bounds__(kThreads) kDamp(const Grid<R> launch, R fraction) {
    const Work w = item<Many>(launch);
    const Dev<R> L = descriptor<R, Many>(launch, w);
    if (L.ctl->stop) return;
    // Items are sweep levels' ranges: any length, strided over the CTA.
    for (std::uint32_t d = w.begin + threadIdx.x; d < w.end; d += blockDim.x) {
        const BondRec<R> rec = L.rec[d];
        if ((rec.a & kDeadBit) || !endsInBounds(rec, L.N, kSiteDamp)) continue;
        const std::uint32_t a = endA(rec), b = endB(rec);
        const Q4<R> va = L.v[a], vb = L.v[b];
        const R ma = va.w, mb = vb.w;
        if (ma <= R(0) || mb <= R(0)) continue;
        const Q4<R> g = L.geo[d];
        const V3<R> n = normalized(bondVector<R, Direct>(L, a, b, V3<R>{g.x, g.y, g.z}));
        const R rel = dot(xyz(vb) - xyz(va), n);
        const R im = R(1) / ma + R(1) / mb;
        const R impulse = -fraction * rel / im;
        const V3<R> na = xyz(va) - (impulse / ma) * n;
        const V3<R> nb = xyz(vb) + (impulse / mb) * n;
        L.v[a] = Q4<R>{na.x, na.y, na.z, ma};
        L.v[b] = Q4<R>{nb.x, nb.y, nb.z, mb};
    }
}

// Support projection of the nodes that have no bond to carry it (isolated
// nodes), after a sweep (LatticePhysics.hpp:1255-1261).
template <class R, bool Many>
__global__ void __launch_bounds__(kThreads) kSupportIsolated(const Grid<R> launch, Settings<R> S) {
    const Work w = item<Many>(launch);
    const Dev<R> L = descriptor<R, Many>(launch, w);
    if (L.ctl->stop) return;
    const std::uint32_t t = w.begin + threadIdx.x;
    if (t >= w.end) return;
    const std::uint32_t i = L.isolated[t];
    if (!inBounds(i, L.N, kSiteIsolated)) return;
    const Q4<R> uq = L.u[i];
    V3<R> u = xyz(uq);
    // Written back whenever a projection ran, even by a zero distance, so the
    // sign of a zero component is whatever the projection made it.
    if (supportProject(L, S, i, u)) L.u[i] = Q4<R>{u.x, u.y, u.z, uq.w};
}

// Velocity from accepted positions, then the support response of
// non-candidates when no damping sweep follows (LatticePhysics.hpp:1725-1730).
template <class R, bool Many>
__global__ void __launch_bounds__(kThreads) kVelocity(const Grid<R> launch, Settings<R> S, int respond) {
    const Work w = item<Many>(launch);
    __shared__ SharedDesc<R> desc;
    const Dev<R> &L = descriptorIn<R, Many>(launch, w, desc);
    if (L.ctl->stop) return;
    const std::uint32_t i = w.begin + threadIdx.x;
    if (i >= w.end) return;
    const Q4<R> vq = L.v[i];
    V3<R> vel = (xyz(L.u[i]) - xyz(L.up[i])) / S.dt;
    if (respond && !L.candidate[i])
        for (std::uint32_t p = 0; p < S.plane_count; ++p)
            if (L.engaged[p * L.N + i]) vel = supportVelocity(S.planes[p], vel, L.approach[p * L.N + i]);
    L.v[i] = Q4<R>{vel.x, vel.y, vel.z, vq.w};
}

// Support response of non-candidates after the damping sweep (CpuLatticeBackend.cpp:414-415).
template <class R, bool Many>
__global__ void __launch_bounds__(kThreads) kSupportVelocity(const Grid<R> launch, Settings<R> S) {
    const Work w = item<Many>(launch);
    const Dev<R> L = descriptor<R, Many>(launch, w);
    if (L.ctl->stop) return;
    const std::uint32_t i = w.begin + threadIdx.x;
    if (i >= w.end || L.candidate[i]) return;
    const Q4<R> vq = L.v[i];
    V3<R> vel = xyz(vq);
    for (std::uint32_t p = 0; p < S.plane_count; ++p)
        if (L.engaged[p * L.N + i]) vel = supportVelocity(S.planes[p], vel, L.approach[p * L.N + i]);
    L.v[i] = Q4<R>{vel.x, vel.y, vel.z, vq.w};
}

// ---------------------------------------------------------------------------
// End-of-substep sample, plastic return and failure (LatticePhysics.hpp:1018-1114).
// One thread per bond in schedule order; a CTA is one "tile" of 256 bonds.
// The reference folds its FP64 ledgers one bond at a time in bond order
// (CpuLatticeBackend.cpp:446-478). Here every reduction has a fixed order that
// depends on the bond order only, never on thread timing: plastic work is
// summed per tile by a fixed shuffle tree and the tiles in index order; broken
// bonds and damage-record candidates are flagged one bit per bond and listed
// in bond order by kTileCounts/kBlockScan/kTopScan/kEmitEvents.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned floatBits(float x) { return __float_as_uint(x); }

// Sum over a warp in a fixed order (lane 0 holds the result).
__device__ __forceinline__ double warpSumFixed(double x) {
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffU, x, o);
    return x;
}

template <class R, bool Many, bool Direct, bool Plastic>
__global__ void __launch_bounds__(kThreads) kEndSample(const Grid<R> launch, Settings<R> S, int part) {
    const Work w = item<Many>(launch);
    __shared__ SharedDesc<R> desc;
    const Dev<R> &L = descriptorIn<R, Many>(launch, w, desc);
    __shared__ double tile_work[kThreads / 32];
    __shared__ unsigned peak[4];
    if (L.ctl->stop) return;
    // part 0: every tile; 1: the tiles outside the contact halo; 2: inside it.
    if (part != 0) {
        const bool late = L.late_tile_stamp[w.begin / kThreads] == substepStamp(L);
        if (late != (part == 2)) return;
    }
    const std::uint32_t j = w.begin + threadIdx.x; // storage index; items start on multiples of 256
    // A bond can raise the run's damage maximum only if it exceeds the maximum
    // as the substep began (CpuLatticeBackend.cpp:462-465); the bound is formed
    // once per CTA.
    __shared__ double damage_floor;
    __shared__ int any_work;
    if (threadIdx.x < 4) peak[threadIdx.x] = 0;
    if (threadIdx.x == 0) {
        damage_floor = L.ctl->max_damage + 1.0e-6;
        any_work = 0;
    }
    __syncthreads();
    double plastic_work = 0.0;
    if (j < w.end) {
        // Every per-bond array is loaded at once, ahead of the liveness test
        // and of the node gathers that wait on the record: one trip to memory
        // for all of them rather than one after another (single-use data,
        // streamed past L2 so the node arrays stay there).
        const BondRec<R> rec = ldStream(L.rec + j);
        const Q4<R> g = ldStream(L.geo + j);
        Q4<R> pv = L.prev[j];
        const Q4<R> t4 = ldStream(L.thr4 + j);
        const Q2<R> t2 = L.thr2[j];
        Q2<R> pl = Plastic ? L.plastic[j] : Q2<R>{R(0), R(0)};
        if (!(rec.a & kDeadBit) && endsInBounds(rec, L.N, kSiteEndSample)) {
            const std::uint32_t a = endA(rec), b = endB(rec);
            const V3<R> edge{g.x, g.y, g.z};
            float plastic_stretch = 0.0F;
            R pext = R(0);
            // The bond's current length, used by the plastic return, the
            // sample and the stored energy of a failure alike.
            const R len = length(bondVector<R, Direct>(L, a, b, edge));
            if (Plastic) {
                pext = pl.x;
                if (S.yield_stretch > R(0)) {
                    const R elastic = len - rec.rest - pl.x;
                    const R magnitude = absR(elastic);
                    const R h = S.hardening;
                    const R yield = S.yield_stretch * rec.rest + h * pl.y;
                    if (magnitude > yield) {
                        const R inc = (magnitude - yield) / (R(1) + h);
                        pl.x = pl.x + (elastic < R(0) ? -inc : inc);
                        pl.y = pl.y + inc;
                        L.plastic[j] = pl;
                        pext = pl.x;
                        const R c = g.w;
                        if (c > R(0)) {
                            const R yield_end = yield + h * inc;
                            plastic_work = static_cast<double>(R(0.5) * (yield + yield_end) * inc / c);
                        }
                    }
                    plastic_stretch = static_cast<float>(absR(pl.x) / rec.rest);
                }
            }
            R t, c, s;
            sampleBond<R, Direct>(L, a, b, rec, edge, len, t, c, s);
            const R pt = maxR(R(0), maxR(pv.x, t));
            const R pc = maxR(R(0), maxR(pv.y, c));
            const R ps = maxR(R(0), maxR(pv.z, s));
            pv.x = maxR(R(0), t);
            pv.y = maxR(R(0), c);
            pv.z = maxR(R(0), s);
            const R dtn = damageProgress(pt, t4.x, t4.y);
            const R dcp = damageProgress(pc, t4.z, t4.w);
            const R dsh = damageProgress(ps, t2.x, t2.y);
            R damage = dtn;
            std::uint8_t mode = 1;
            if (dcp > damage) { damage = dcp; mode = 2; }
            if (dsh > damage) { damage = dsh; mode = 3; }
            if (damage > pv.w) {
                pv.w = damage;
                L.mode[j] = mode;
            }
            L.prev[j] = pv;
            const float dmg = static_cast<float>(pv.w);
            const std::uint32_t js = L.dev2sched[j];
            if (pv.w >= R(1)) {
                const R cc = g.w;
                R energy = R(0);
                if (!(cc <= R(0))) {
                    const R ext = len - rec.rest - pext;
                    energy = R(0.5) * ext * ext / cc;
                }
                L.rec[j].a = rec.a | kDeadBit;
                // Both slots keep their weight, sign-flipped: dead for the
                // strain, still there for a sheet's rest geometry.
                L.nbr[L.slot_a[j]].w = -absR(L.nbr[L.slot_a[j]].w);
                L.nbr[L.slot_b[j]].w = -absR(L.nbr[L.slot_b[j]].w);
                L.ev_removed[js] = static_cast<double>(energy);
                L.ev_ends[js] = make_uint2(a, b);
                atomicOr(L.ev_bits + (js >> 5), 1U << (js & 31U));
            }
            if (static_cast<double>(dmg) > damage_floor) {
                L.ev_damage[js] = dmg;
                atomicOr(L.dmg_bits + (js >> 5), 1U << (js & 31U));
            }
            // Peaks are non-negative, so their bit patterns order as the values do.
            atomicMax(&peak[0], floatBits(static_cast<float>(pt)));
            atomicMax(&peak[1], floatBits(static_cast<float>(pc)));
            atomicMax(&peak[2], floatBits(static_cast<float>(ps)));
            if (Plastic && S.yield_stretch > R(0)) atomicMax(&peak[3], floatBits(plastic_stretch));
        }
    }
    // Fixed-order sums of the plastic work; a sum of zeros is +0 whichever
    // way it is formed, so all-zero warps and tiles skip the FP64 adds.
    double warp_work = 0.0;
    if (Plastic && __any_sync(0xffffffffU, plastic_work != 0.0)) {
        warp_work = warpSumFixed(plastic_work);
        if ((threadIdx.x & 31) == 0) any_work = 1;
    }
    if ((threadIdx.x & 31) == 0) tile_work[threadIdx.x / 32] = warp_work;
    __syncthreads();
    if (threadIdx.x == 0) {
        double wsum = 0.0;
        if (any_work)
            for (int q = 0; q < kThreads / 32; ++q) wsum += tile_work[q];
        L.tile_plastic[w.begin / kThreads] = wsum;
        if (peak[0]) atomicMax(&L.ctl->max_t, peak[0]);
        if (peak[1]) atomicMax(&L.ctl->max_c, peak[1]);
        if (peak[2]) atomicMax(&L.ctl->max_s, peak[2]);
        if (peak[3]) atomicMax(&L.ctl->max_plastic, peak[3]);
    }
}

// ---------------------------------------------------------------------------
// The substep ledger's ordered lists and FP64 sums, fully parallel and in a
// fixed order. A "tile" is 256 bonds of schedule order (8 bit words); a scan
// block is kScanBlock tiles. Every sum below is formed in an order fixed by the
// bond order alone: sequential inside a 32-bond word, a Hillis-Steele scan
// across the words of a tile, across the tiles of a block, across the blocks.
// ---------------------------------------------------------------------------
constexpr unsigned kScanBlock = 1024;

// Hillis-Steele inclusive scan of one double per thread across a 1024-thread
// CTA (a fixed order); `buf` is 1024 doubles of shared memory.
__device__ __forceinline__ double blockInclusiveScan(double x, double *buf) {
    buf[threadIdx.x] = x;
    __syncthreads();
    for (unsigned o = 1; o < blockDim.x; o <<= 1) {
        const double y = threadIdx.x >= o ? buf[threadIdx.x - o] : 0.0;
        __syncthreads();
        if (threadIdx.x >= o) buf[threadIdx.x] += y;
        __syncthreads();
    }
    const double r = buf[threadIdx.x];
    __syncthreads();
    return r;
}

__device__ __forceinline__ unsigned blockExclusiveScanU(unsigned x, unsigned *buf, unsigned &total) {
    buf[threadIdx.x] = x;
    __syncthreads();
    for (unsigned o = 1; o < blockDim.x; o <<= 1) {
        const unsigned y = threadIdx.x >= o ? buf[threadIdx.x - o] : 0U;
        __syncthreads();
        if (threadIdx.x >= o) buf[threadIdx.x] += y;
        __syncthreads();
    }
    const unsigned inclusive = buf[threadIdx.x];
    total = buf[blockDim.x - 1];
    __syncthreads();
    return inclusive - x;
}

// Removed energy of a tile's broken bonds: per word, in bit order; across the
// tile's words by an inclusive shuffle scan. Returns this lane's inclusive sum
// (lane 7, or the last word of the tile, holds the tile's total).
__device__ __forceinline__ double tileRemovedScan(double own) {
    const unsigned lane = threadIdx.x & 31;
    double inclusive = own;
    for (int o = 1; o < 32; o <<= 1) {
        const double y = __shfl_up_sync(0xffffffffU, inclusive, o);
        if (lane >= static_cast<unsigned>(o)) inclusive += y;
    }
    return inclusive;
}

// One warp per tile: broken-bond and damage-candidate counts and the tile's
// removed energy.
template <class R, bool Many>
__global__ void __launch_bounds__(kThreads) kTileCounts(const Grid<R> launch) {
    const Work w = item<Many>(launch);
    const Dev<R> L = descriptor<R, Many>(launch, w);
    if (L.ctl->stop) return;
    const unsigned tile = w.begin + threadIdx.x / 32; // items: up to 8 tiles of one lattice
    const unsigned lane = threadIdx.x & 31;
    if (tile >= w.end) return;
    constexpr unsigned kWords = kThreads / 32;
    const unsigned wd = tile * kWords + lane;
    const bool word = lane < kWords && wd < L.words_b;
    const unsigned bits = word ? L.ev_bits[wd] : 0U;
    const unsigned dbits = word ? L.dmg_bits[wd] : 0U;
    double own = 0.0;
    for (unsigned m = bits; m; m &= m - 1) own += L.ev_removed[wd * 32 + static_cast<unsigned>(__ffs(m) - 1)];
    unsigned nb = __popc(bits), nd = __popc(dbits);
    for (int o = 16; o > 0; o >>= 1) {
        nb += __shfl_down_sync(0xffffffffU, nb, o);
        nd += __shfl_down_sync(0xffffffffU, nd, o);
    }
    const double total = __shfl_sync(0xffffffffU, tileRemovedScan(own), 31);
    if (lane == 0) {
        L.ev_tile[tile] = nb;
        L.dmg_tile[tile] = nd;
        L.tile_removed[tile] = total;
    }
}

// One CTA per scan block: exclusive offsets of the tiles inside the block (in
// place) and the block's totals; the plastic work of the end-sample tiles of
// the same index range is reduced by a fixed tree.
template <class R, bool Many>
__global__ void __launch_bounds__(kScanBlock) kBlockScan(const Grid<R> launch, int plastic) {
    const Work w = item<Many>(launch);
    const Dev<R> L = descriptor<R, Many>(launch, w);
    __shared__ double dbuf[kScanBlock];
    __shared__ unsigned ubuf[kScanBlock];
    if (L.ctl->stop) return;
    const unsigned blk = w.begin; // one item per (lattice, scan block)
    const unsigned t = blk * kScanBlock + threadIdx.x;
    const bool in = t < L.tiles_b;
    unsigned tb = 0, td = 0;
    const unsigned ob = blockExclusiveScanU(in ? L.ev_tile[t] : 0U, ubuf, tb);
    const unsigned od = blockExclusiveScanU(in ? L.dmg_tile[t] : 0U, ubuf, td);
    // The inclusive scan leaves dbuf holding every thread's inclusive sum.
    (void)blockInclusiveScan(in ? L.tile_removed[t] : 0.0, dbuf);
    const double exclusive = threadIdx.x ? dbuf[threadIdx.x - 1] : 0.0;
    const double removed_total = dbuf[kScanBlock - 1];
    __syncthreads();
    if (in) {
        L.ev_tile[t] = ob;
        L.dmg_tile[t] = od;
        L.tile_removed[t] = exclusive;
    }
    double block_work = 0.0;
    if (plastic) {
        dbuf[threadIdx.x] = in ? L.tile_plastic[t] : 0.0;
        __syncthreads();
        for (unsigned s = kScanBlock / 2; s > 0; s >>= 1) {
            if (threadIdx.x < s) dbuf[threadIdx.x] += dbuf[threadIdx.x + s];
            __syncthreads();
        }
        block_work = dbuf[0];
    }
    if (threadIdx.x == 0) {
        L.blk_ev[blk] = tb;
        L.blk_dmg[blk] = td;
        L.blk_removed[blk] = removed_total;
        L.blk_plastic[blk] = block_work;
    }
}

// One CTA: exclusive offsets of the blocks (rounds of 1024 blocks with a
// carry), and the substep's totals.
template <class R, bool Many>
__global__ void __launch_bounds__(kScanBlock) kTopScan(const Grid<R> launch) {
    const Work w = item<Many>(launch);
    const Dev<R> L = descriptor<R, Many>(launch, w);
    const unsigned blocks = L.tiles_b / kScanBlock + 1; // one item per lattice
    __shared__ double dbuf[kScanBlock];
    __shared__ unsigned ubuf[kScanBlock];
    __shared__ double plastic_carry;
    Ctl &c = *L.ctl;
    if (c.stop) return;
    unsigned carry_b = 0, carry_d = 0;
    double carry_r = 0.0;
    if (threadIdx.x == 0) plastic_carry = 0.0;
    for (unsigned base = 0; base < blocks; base += kScanBlock) {
        const unsigned k = base + threadIdx.x;
        const bool in = k < blocks;
        unsigned tb = 0, td = 0;
        const unsigned ob = blockExclusiveScanU(in ? L.blk_ev[k] : 0U, ubuf, tb);
        const unsigned od = blockExclusiveScanU(in ? L.blk_dmg[k] : 0U, ubuf, td);
        (void)blockInclusiveScan(in ? L.blk_removed[k] : 0.0, dbuf);
        const double before = threadIdx.x ? dbuf[threadIdx.x - 1] : 0.0;
        const double round_total = dbuf[kScanBlock - 1];
        __syncthreads();
        dbuf[threadIdx.x] = in ? L.blk_plastic[k] : 0.0;
        __syncthreads();
        for (unsigned s = kScanBlock / 2; s > 0; s >>= 1) {
            if (threadIdx.x < s) dbuf[threadIdx.x] += dbuf[threadIdx.x + s];
            __syncthreads();
        }
        if (in) {
            L.blk_ev[k] = carry_b + ob;
            L.blk_dmg[k] = carry_d + od;
            L.blk_removed[k] = carry_r + before;
        }
        if (threadIdx.x == 0) plastic_carry += dbuf[0];
        carry_b += tb;
        carry_d += td;
        carry_r += round_total;
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        c.event_count = carry_b;
        c.dmg_count = carry_d;
        c.removed_substep = carry_r;
        c.plastic_substep = plastic_carry;
        c.energy_gain = 0;
        c.dirty_count = 0; // the restart of this substep has consumed the list
    }
}

// One warp per tile: the tile's broken bonds in bond order with their removed
// energy and their prefix of the substep's removed energy (block offset, tile
// offset, in-tile inclusive scan: the same orders as the counts), and its
// damage candidates in order. The bit words are cleared for the next substep.
template <class R, bool Many>
__global__ void __launch_bounds__(kThreads) kEmitEvents(const Grid<R> launch) {
    const Work w = item<Many>(launch);
    const Dev<R> L = descriptor<R, Many>(launch, w);
    const Ctl &c = *L.ctl;
    if (c.stop || (c.event_count == 0 && c.dmg_count == 0)) return;
    const unsigned tile = w.begin + threadIdx.x / 32;
    const unsigned lane = threadIdx.x & 31;
    if (tile >= w.end) return;
    constexpr unsigned kWords = kThreads / 32;
    const unsigned wd = tile * kWords + lane;
    const bool word = lane < kWords && wd < L.words_b;
    const unsigned blk = tile / kScanBlock;
    unsigned bits = word ? L.ev_bits[wd] : 0U;
    if (__any_sync(0xffffffffU, bits != 0)) {
        double own = 0.0;
        for (unsigned m = bits; m; m &= m - 1) own += L.ev_removed[wd * 32 + static_cast<unsigned>(__ffs(m) - 1)];
        const double inclusive = tileRemovedScan(own);
        const double exclusive = __shfl_up_sync(0xffffffffU, inclusive, 1);
        unsigned n = __popc(bits), x = n;
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned y = __shfl_up_sync(0xffffffffU, x, o);
            if (lane >= static_cast<unsigned>(o)) x += y;
        }
        unsigned at = L.blk_ev[blk] + L.ev_tile[tile] + x - n;
        const double offset = L.blk_removed[blk] + L.tile_removed[tile];
        double run = lane == 0 ? 0.0 : exclusive;
        for (; bits; bits &= bits - 1) {
            const unsigned j = wd * 32 + static_cast<unsigned>(__ffs(bits) - 1);
            const double e = L.ev_removed[j];
            run += e;
            L.ev_list[at] = j;
            L.ev_packed[at] = e;
            L.ev_prefix[at] = offset + run;
            ++at;
        }
        if (word) L.ev_bits[wd] = 0; // the end sample sets bits with atomicOr
    }
    unsigned dbits = word ? L.dmg_bits[wd] : 0U;
    if (__any_sync(0xffffffffU, dbits != 0)) {
        unsigned n = __popc(dbits), x = n;
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned y = __shfl_up_sync(0xffffffffU, x, o);
            if (lane >= static_cast<unsigned>(o)) x += y;
        }
        unsigned at = L.blk_dmg[blk] + L.dmg_tile[tile] + x - n;
        for (; dbits; dbits &= dbits - 1) {
            const unsigned j = wd * 32 + static_cast<unsigned>(__ffs(dbits) - 1);
            L.dmg_list[at] = j;
            L.dmg_value[at] = L.ev_damage[j];
            ++at;
        }
        if (word) L.dmg_bits[wd] = 0;
    }
}

// Parallel over this substep's broken bonds, in list order: the energy-gain
// test of each bond against the running removed energy it would see
// (CpuLatticeBackend.cpp:469-474), the first-failure list, and the dirty
// marks and list of the next substep's restart (CpuLatticeBackend.cpp:476-477).
template <class R, bool Many>
__global__ void __launch_bounds__(kThreads) kLedgerBroken(const Grid<R> launch) {
    const Work w = part<Many>(launch);
    const Dev<R> L = descriptor<R, Many>(launch, w);
    Ctl &c = *L.ctl;
    if (c.stop) return;
    const unsigned n = c.event_count;
    const bool first_round = c.broken_bonds == 0;
    const double prior = c.removed_energy;
    const double fraction = c.energy_flat_fraction;
    // Items: part `begin` of `end` parts of this lattice's event list.
    for (unsigned e = w.begin * blockDim.x + threadIdx.x; e < n; e += w.end * blockDim.x) {
        const std::uint32_t j = L.ev_list[e];
        if (!inBounds(j, L.B, kSiteEvent)) continue;
        const double running = prior + L.ev_prefix[e];
        const double removed = L.ev_packed[e];
        if (removed > fraction * (running < 1.0e-12 ? 1.0e-12 : running)) atomicOr(&c.energy_gain, 1U);
        if (first_round) L.ffb[e] = j;
        const uint2 e2 = L.ev_ends[j];
        const std::uint32_t ends[2] = {e2.x, e2.y};
        for (int q = 0; q < 2; ++q) {
            const std::uint32_t node = ends[q];
            if (!inBounds(node, L.N, kSiteEventEnd)) continue;
            unsigned *word = reinterpret_cast<unsigned *>(L.dirty + (node & ~3U));
            const unsigned bit = 1U << (8 * (node & 3U));
            if (!(atomicOr(word, bit) & bit)) {
                const unsigned at = atomicAdd(&c.dirty_count, 1U);
                if (inBounds(at, L.N, kSiteDirty)) L.dirty_list[at] = node;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// The energy audit's measure (LatticePhysics.hpp:1676-1682): a lattice's
// kinetic energy, each node's term formed in backend precision and widened,
// folded serially in node order as the reference folds it, so the audit
// ledgers match the reference's bit for bit. The CTA forms the next chunk of
// terms in shared memory while thread 0 folds the current one; the fold is
// one chain of dependent FP64 adds (N of them), so the kernel is bound by FP64
// add latency. kAuditMark keeps the energy before a phase; the other modes
// charge the drop across the phase to the striker or the damping ledger.
// ---------------------------------------------------------------------------
constexpr unsigned kFoldThreads = 1024;
constexpr int kAuditMark = 0, kAuditStriker = 1, kAuditDamping = 2;

template <class R, bool Many>
__global__ void __launch_bounds__(kFoldThreads) kKineticFold(const Grid<R> launch, int mode) {
    const Work w = item<Many>(launch);
    const Dev<R> L = descriptor<R, Many>(launch, w);
    Ctl &c = *L.ctl;
    if (c.stop) return;
    __shared__ double terms[2][kFoldThreads];
    double total = 0.0;
    unsigned buf = 0;
    // Thread 0 reaches the barrier of chunk k+1 only after folding chunk k,
    // so chunk k+2 never overwrites a buffer still being read.
    for (std::uint32_t base = 0; base < L.N; base += kFoldThreads, buf ^= 1U) {
        const std::uint32_t i = base + threadIdx.x;
        if (i < L.N) {
            const Q4<R> q = L.v[i]; // w: the node's mass
            const V3<R> v = xyz(q);
            terms[buf][threadIdx.x] = static_cast<double>(R(0.5) * q.w * dot(v, v));
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            const std::uint32_t n = L.N - base < kFoldThreads ? L.N - base : kFoldThreads;
#pragma unroll 8
            for (std::uint32_t k = 0; k < n; ++k) total += terms[buf][k];
        }
    }
    if (threadIdx.x != 0) return;
    if (mode == kAuditMark) c.ke_mark = total;
    else if (mode == kAuditStriker) c.striker_dissipated += c.ke_mark - total;
    else c.damping_dissipated += c.ke_mark - total;
}

// ---------------------------------------------------------------------------
// The external-load ledger of a substep (ExternalLoads.hpp:126-140): thirteen
// independent serial folds over the loaded nodes in list order -- impulse,
// angular impulse, work, requested impulse and requested angular impulse, per
// component -- then added to the run's ledger. Lane q of warp 0 runs fold q,
// so the thirteen chains advance together and each keeps the reference's
// order; the other warps stage the next chunk of node contributions into
// shared memory meanwhile. The wrench sources' node runs tile the list in
// source order, so the same pass folds each source's own change and hands it
// to its ledger when its run ends.
//
// A fold is a chain of dependent FP64 adds, one per loaded node, so its
// length sets its time (GB300's FP64 add latency is long). Nothing in the
// substep reads the ledger before the exit rules at its end, so the kernel
// runs on a stream of its own from the kick, whose contributions it reads,
// beside the contact passes, the sweep and the end sample.
// ---------------------------------------------------------------------------
constexpr int kLedgerFolds = 13;
constexpr unsigned kLedgerThreads = 128;                   // one folding lane, three staging warps
constexpr unsigned kLedgerStagers = kLedgerThreads - 32;
constexpr unsigned kLedgerChunk = 384;                      // entries staged per round

// Adds a source's folded change (component q) to its ledger.
__device__ __forceinline__ void addLoadComponent(LoadLedger &g, int q, double x) {
    if (q < 3) g.imp[q] = g.imp[q] + x;
    else if (q < 6) g.ang[q - 3] = g.ang[q - 3] + x;
    else if (q == 6) g.work = g.work + x;
    else if (q < 10) g.req_imp[q - 7] = g.req_imp[q - 7] + x;
    else g.req_ang[q - 10] = g.req_ang[q - 10] + x;
}

// One CTA per (lattice, component): blockIdx.y is the component q. Thread 0
// folds it; the other warps stage the next chunk of its node contributions.
// Each fold is one chain of dependent FP64 adds, and GB300 has little FP64
// issue per SM, so the thirteen chains run on thirteen SMs (measured, 1,984
// loaded nodes: 246 us with the chains on thirteen warps of one CTA, 182 us
// on thirteen lanes of one warp).
template <class R, bool Many>
__global__ void __launch_bounds__(kLedgerThreads) kLoadLedger(const Grid<R> launch, Settings<R> S) {
    const Work w = item<Many>(launch);
    const Dev<R> L = descriptor<R, Many>(launch, w);
    Ctl &c = *L.ctl;
    // A lattice stopped, or whose kick failed this substep, folds nothing
    // (kLedger stops the latter).
    if (c.stop || c.error) return;
    if (!(c.ext_count && c.loads_remaining > 0)) return;
    __shared__ double stage[2][kLedgerChunk];
    const int q = static_cast<int>(blockIdx.y);
    const bool folder = threadIdx.x == 0;
    const bool stager = threadIdx.x >= 32;
    const std::uint32_t n = c.ext_count;
    const unsigned sources = c.wrench_count;
    const auto fill = [&](std::uint32_t base, unsigned buf) {
        const std::uint32_t cnt = n - base < kLedgerChunk ? n - base : kLedgerChunk;
#pragma unroll 4
        for (unsigned e = threadIdx.x - 32; e < cnt; e += kLedgerStagers) {
            const std::uint32_t node = L.ext_nodes[base + e];
            stage[buf][e] = inBounds(node, L.N, kSiteLoad)
                ? L.ext_contrib[kLedgerFolds * static_cast<std::size_t>(node) + q] : 0.0;
        }
    };
    // Flushes every source whose run ends at `at`: the component's change to
    // the source's ledger; component 0 also keeps the step count, the elapsed
    // time and the source's place in the status order.
    unsigned k = 0;
    double run = 0.0;
    const auto flush = [&](std::uint32_t at) {
        while (k < sources && L.wrench[k].end == at) {
            SourceSlot &slot = L.sources[L.wrench[k].slot];
            addLoadComponent(slot.load, q, run);
            if (q == 0) {
                if (slot.load.steps == 0) slot.order = c.source_seq++;
                slot.load.steps += 1;
                slot.load.elapsed = slot.load.elapsed + static_cast<double>(S.dt);
            }
            run = 0.0;
            ++k;
        }
    };
    if (stager) fill(0, 0);
    if (folder) flush(0);
    __syncthreads();
    double total = 0.0;
    unsigned buf = 0;
    for (std::uint32_t base = 0; base < n; base += kLedgerChunk, buf ^= 1U) {
        if (stager) {
            if (base + kLedgerChunk < n) fill(base + kLedgerChunk, buf ^ 1U);
        } else if (folder) {
            const std::uint32_t cnt = n - base < kLedgerChunk ? n - base : kLedgerChunk;
            const double *col = stage[buf];
            if (sources == 0) {
                // Unrolled so the shared-memory loads run ahead of the
                // dependent adds.
#pragma unroll 8
                for (std::uint32_t e = 0; e < cnt; ++e) total += col[e];
            } else {
                for (std::uint32_t e = 0; e < cnt; ++e) {
                    const double x = col[e];
                    total += x;
                    run += x;
                    flush(base + e + 1);
                }
            }
        }
        __syncthreads();
    }
    if (folder) {
        flush(n); // only sources with empty runs past the list's end remain
        LoadLedger &g = c.ext;
        addLoadComponent(g, q, total);
        if (q == 0) {
            g.steps += 1;
            g.elapsed += static_cast<double>(S.dt);
        }
    }
    // loads_remaining counts down in kLedger, after every component's CTA
    // has read it.
}

// ---------------------------------------------------------------------------
// The serial tail of a substep, one thread: the substep's FP64 sums into the
// run totals, the damage-record scan over its (few) candidates in bond order,
// the sphere drift and support contact, the failure-round bookkeeping and the
// exit rules (CpuLatticeBackend.cpp:279-298, 441-488), after the load ledger.
// ---------------------------------------------------------------------------
template <class R, bool Many>
__global__ void kLedger(const Grid<R> launch, Settings<R> S) {
    const Work w = item<Many>(launch);
    const Dev<R> L = descriptor<R, Many>(launch, w);
    if (threadIdx.x != 0) return;
    Ctl &c = *L.ctl;
    if (c.stop) return;
    if (c.error) {
        c.stop = 1;
        atomicSub(L.running, 1U);
        return;
    }
    const unsigned long long step = c.total_steps;
    if (c.ext_count && c.loads_remaining > 0) c.loads_remaining -= 1; // the substep's load, folded by kLoadLedger
    c.full_restart = 0;
    c.plastic_work += c.plastic_substep;
    for (unsigned e = 0; e < c.dmg_count; ++e) {
        const float dmg = L.dmg_value[e];
        if (static_cast<double>(dmg) > c.max_damage + 1.0e-6) {
            c.max_damage = dmg;
            c.last_damage_gain_step = step;
        }
    }
    const unsigned broken = c.event_count;
    c.projections += (c.live_bonds - c.broken_bonds) * S.iterations;
    if (broken) {
        c.nc_rebuild = 1; // a failure changes which pairs no live bond holds
        if (c.broken_bonds == 0) c.ffb_count = broken;
        c.removed_energy += c.removed_substep;
        if (c.energy_gain) c.last_energy_gain_step = step;
        c.broken_bonds += broken;
    }
    Sphere<R> sp = *L.sphere;
    if (!S.sphere_enabled) sp.velocity = sp.velocity + S.dt * S.gravity;
    sp.center = sp.center + S.dt * sp.velocity;
    sphereSupport(S, sp, c.contact);
    *L.sphere = sp;
    c.total_steps = step + 1;
    if (broken) {
        if (c.first_failure_step == ~0ULL) c.first_failure_step = step;
        c.last_failure_step = step;
        ++c.failure_rounds;
    }
    const double available = c.removable_energy + c.ext.work;
    c.exit_reason = c.removable_energy > 0 && available <= 0
        ? 6U
        : exitReason(c.total_steps, c.broken_bonds, c.last_failure_step, c.quiet_steps, c.min_steps, c.no_failure_steps,
                     c.energy_flat_steps, c.last_energy_gain_step, c.calm_steps, c.last_damage_gain_step, c.max_damage,
                     c.calm_damage_margin, c.removed_energy, c.removable_energy > 0 ? available : 0.0);
    if (c.exit_reason == 0 && c.step_limit != 0 && c.total_steps >= c.step_limit) c.exit_reason = 3U;
    if (c.exit_reason != 0) {
        c.stop = 1;
        atomicSub(L.running, 1U);
    }
}

// ---------------------------------------------------------------------------
// Node-to-node contact (LatticePhysics.hpp:1441-1647; stage order
// CpuLatticeBackend.cpp:424-436), after the second sphere pass and before the
// end sample. The pair list holds, for every movable owner node, the movable
// nodes of higher index within 2 r + skin that no live bond holds, in the
// order of the 27 grid cells around the owner (z, then y, then x, from -1)
// and ascending within a cell, at most kPairsPerNode per owner. It is rebuilt
// when a bond failed in the previous substep or a node drifted more than
// skin / 2 since the last build. The grid is hashed into buckets whose
// members are kept ascending; every bucket scan keeps only the nodes of the
// cell it visits, so which cells share a bucket never changes the list, and
// each lattice sizes its own table. The narrow phase is the reference's
// serial chain in list order, run by one warp.
// ---------------------------------------------------------------------------
constexpr std::uint32_t kPairsPerNode = 24;
constexpr unsigned kContactScanThreads = 1024;

// Teschner et al., "Optimized Spatial Hashing for Collision Detection of
// Deformable Objects" (2003): three primes, exclusive-or, masked.
__device__ __forceinline__ std::uint32_t cellBucket(int x, int y, int z, std::uint32_t mask) {
    return ((static_cast<std::uint32_t>(x) * 73856093U) ^ (static_cast<std::uint32_t>(y) * 19349663U) ^
            (static_cast<std::uint32_t>(z) * 83492791U)) & mask;
}

template <class R> __device__ __forceinline__ R contactCutoff(const Settings<R> &S) {
    return R(2) * S.nc_radius + S.nc_skin;
}

// The drift test (nodeContactStale): any node farther than skin / 2 from where
// the list was built asks for a rebuild.
template <class R, bool Many>
__global__ void __launch_bounds__(kThreads) kContactStale(const Grid<R> launch, Settings<R> S) {
    const Work w = item<Many>(launch);
    const Dev<R> L = descriptor<R, Many>(launch, w);
    Ctl &c = *L.ctl;
    if (c.stop || *static_cast<volatile unsigned *>(&c.nc_rebuild)) return;
    const std::uint32_t i = w.begin + threadIdx.x;
    if (i >= w.end) return;
    const R half = R(0.5) * S.nc_skin;
    const R limit = half * half;
    const V3<R> d = xyz(L.u[i]) - xyz(L.nc_built[i]);
    if (dot(d, d) > limit) c.nc_rebuild = 1U;
}

// Rebuild, step 0 (bucket items): clear the bucket counts.
template <class R, bool Many>
__global__ void __launch_bounds__(kThreads) kContactClear(const Grid<R> launch) {
    const Work w = item<Many>(launch);
    const Dev<R> L = descriptor<R, Many>(launch, w);
    Ctl &c = *L.ctl;
    if (c.stop || !c.nc_rebuild) return;
    const std::uint32_t b = w.begin + threadIdx.x;
    if (b < w.end) L.nc_count[b] = 0U;
    if (w.begin == 0 && threadIdx.x == 0) c.nc_members = 0U;
}

// Rebuild, step 1 (nodeContactStoreCell, node items): the node's cell at the
// positions of this substep, the positions kept for the drift test, and the
// bucket counts of the movable nodes.
template <class R, bool Many>
__global__ void __launch_bounds__(kThreads) kContactCells(const Grid<R> launch, Settings<R> S) {
    const Work w = item<Many>(launch);
    const Dev<R> L = descriptor<R, Many>(launch, w);
    if (L.ctl->stop || !L.ctl->nc_rebuild) return;
    const std::uint32_t i = w.begin + threadIdx.x;
    if (i >= w.end) return;
    const R inverse_cell = R(1) / contactCutoff(S);
    const V3<R> p = pos(L, i);
    const int x = static_cast<int>(floor(p.x * inverse_cell));
    const int y = static_cast<int>(floor(p.y * inverse_cell));
    const int z = static_cast<int>(floor(p.z * inverse_cell));
    const std::uint32_t b = cellBucket(x, y, z, L.nc_mask);
    L.nc_cell[i] = make_int4(x, y, z, static_cast<int>(b));
    L.nc_built[i] = L.u[i];
    if (!(L.v[i].w <= R(0))) atomicAdd(&L.nc_count[b], 1U);
}

// Rebuild, step 2 (bucket items): each bucket's first member slot. Buckets of
// one CTA are contiguous; the CTAs' runs are placed in any order, which only
// moves whole buckets. The count becomes the scatter cursor.
template <class R, bool Many>
__global__ void __launch_bounds__(kThreads) kContactBuckets(const Grid<R> launch) {
    __shared__ unsigned buf[kThreads];
    __shared__ unsigned base;
    const Work w = item<Many>(launch);
    const Dev<R> L = descriptor<R, Many>(launch, w);
    Ctl &c = *L.ctl;
    if (c.stop || !c.nc_rebuild) return;
    const std::uint32_t b = w.begin + threadIdx.x;
    const unsigned n = b < w.end ? L.nc_count[b] : 0U;
    unsigned total = 0;
    const unsigned ex = blockExclusiveScanU(n, buf, total);
    if (threadIdx.x == 0) base = atomicAdd(&c.nc_members, total);
    __syncthreads();
    if (b < w.end) {
        L.nc_start[b] = base + ex;
        L.nc_count[b] = 0U;
    }
}

// Rebuild, step 3 (node items): the movable nodes into their buckets.
template <class R, bool Many>
__global__ void __launch_bounds__(kThreads) kContactScatter(const Grid<R> launch) {
    const Work w = item<Many>(launch);
    const Dev<R> L = descriptor<R, Many>(launch, w);
    if (L.ctl->stop || !L.ctl->nc_rebuild) return;
    const std::uint32_t i = w.begin + threadIdx.x;
    if (i >= w.end || L.v[i].w <= R(0)) return;
    const std::uint32_t b = static_cast<std::uint32_t>(L.nc_cell[i].w);
    L.nc_members[L.nc_start[b] + atomicAdd(&L.nc_count[b], 1U)] = i;
}

// Rebuild, step 4 (bucket items): each bucket's members ascending (buckets
// hold half a node on average; an insertion sort in place).
template <class R, bool Many>
__global__ void __launch_bounds__(kThreads) kContactSort(const Grid<R> launch) {
    const Work w = item<Many>(launch);
    const Dev<R> L = descriptor<R, Many>(launch, w);
    if (L.ctl->stop || !L.ctl->nc_rebuild) return;
    const std::uint32_t b = w.begin + threadIdx.x;
    if (b >= w.end) return;
    const std::uint32_t n = L.nc_count[b];
    std::uint32_t *m = L.nc_members + L.nc_start[b];
    for (std::uint32_t k = 1; k < n; ++k) {
        const std::uint32_t v = m[k];
        std::uint32_t j = k;
        for (; j > 0 && m[j - 1] > v; --j) m[j] = m[j - 1];
        m[j] = v;
    }
}

// Rebuild, step 5 (nodeContactGather, node items; tile = the item's 256
// nodes). Count pass: each owner's pairs and the tile's total, and the pairs
// that did not fit. Write pass: the pairs at the owner's place in the list.
template <class R, bool Many, bool Write>
__global__ void __launch_bounds__(kThreads) kContactGather(const Grid<R> launch, Settings<R> S) {
    __shared__ unsigned buf[kThreads];
    const Work w = item<Many>(launch);
    const Dev<R> L = descriptor<R, Many>(launch, w);
    Ctl &c = *L.ctl;
    if (c.stop || !c.nc_rebuild) return;
    const std::uint32_t i = w.begin + threadIdx.x;
    const bool in = i < w.end;
    const std::uint32_t tile = w.begin / kThreads;
    std::uint32_t at = 0;
    if (Write) {
        unsigned total = 0;
        at = L.nc_tile[tile] + blockExclusiveScanU(in ? L.nc_fill[i] : 0U, buf, total);
    }
    std::uint32_t fill = 0, overflow = 0;
    if (in && !(L.v[i].w <= R(0))) {
        const std::size_t N = L.N;
        const R cutoff = contactCutoff(S);
        const R cutoff_sq = cutoff * cutoff;
        const V3<R> p = pos(L, i);
        const int4 home = L.nc_cell[i];
        for (int dz = -1; dz <= 1; ++dz)
            for (int dy = -1; dy <= 1; ++dy)
                for (int dx = -1; dx <= 1; ++dx) {
                    const int gx = home.x + dx, gy = home.y + dy, gz = home.z + dz;
                    const std::uint32_t b = cellBucket(gx, gy, gz, L.nc_mask);
                    const std::uint32_t first = L.nc_start[b], n = L.nc_count[b];
                    for (std::uint32_t k = 0; k < n; ++k) {
                        const std::uint32_t j = L.nc_members[first + k];
                        if (j <= i) continue;
                        const int4 cj = L.nc_cell[j];
                        if (cj.x != gx || cj.y != gy || cj.z != gz) continue;
                        const V3<R> r = pos(L, j) - p;
                        if (dot(r, r) > cutoff_sq) continue;
                        // The pair's bond, if the owner lists one to j; a live one holds the pair.
                        std::uint32_t bond = kNoBond;
                        bool held = false;
                        for (std::uint32_t s = 0; s < L.D; ++s) {
                            const std::size_t slot = s * N + i;
                            const std::uint32_t bs = L.nbr_bond[slot];
                            if (bs == kNoBond) break;
                            if (L.nbr_other[slot] != j) continue;
                            bond = bs;
                            held = !signbit(L.nbr[slot].w);
                            break;
                        }
                        if (held) continue;
                        if (fill == kPairsPerNode) {
                            ++overflow;
                            continue;
                        }
                        if (Write) {
                            L.nc_pa[at + fill] = i;
                            L.nc_pb[at + fill] = j;
                            L.nc_pbond[at + fill] = bond;
                        }
                        ++fill;
                    }
                }
    }
    if (!Write) {
        if (in) L.nc_fill[i] = fill;
        unsigned total = 0;
        blockExclusiveScanU(fill, buf, total);
        if (threadIdx.x == 0) L.nc_tile[tile] = total;
        if (overflow) atomicAdd(&c.node.pair_overflow, static_cast<unsigned long long>(overflow));
    }
}

// Rebuild, step 6 (one CTA per lattice): the tiles' first pairs in node order,
// and the list's length (nodeContactActiveList).
template <class R, bool Many>
__global__ void __launch_bounds__(kContactScanThreads) kContactTiles(const Grid<R> launch) {
    __shared__ unsigned buf[kContactScanThreads];
    const Work w = item<Many>(launch);
    const Dev<R> L = descriptor<R, Many>(launch, w);
    Ctl &c = *L.ctl;
    if (c.stop || !c.nc_rebuild) return;
    const std::uint32_t tiles = (L.N + kThreads - 1) / kThreads;
    unsigned carry = 0;
    for (std::uint32_t t0 = 0; t0 < tiles; t0 += kContactScanThreads) {
        const std::uint32_t t = t0 + threadIdx.x;
        unsigned total = 0;
        const unsigned ex = blockExclusiveScanU(t < tiles ? L.nc_tile[t] : 0U, buf, total);
        if (t < tiles) L.nc_tile[t] = carry + ex;
        carry += total;
    }
    if (threadIdx.x == 0) {
        c.nc_pairs = carry;
        c.node.pairs_listed += carry;
    }
}

// The narrow phase (nodeContactPass and nodeContactPair), one warp per lattice.
// The lanes evaluate the next 32 pairs of the list against the current state
// at once; the first pair whose response changes a velocity or a position is
// applied by its lane, and the window restarts after it. Pairs before it
// changed nothing, so they saw exactly the state the serial order shows them:
// their tests and overlaps are counted as they are.
template <class R, bool Many>
__global__ void __launch_bounds__(32) kContactNarrow(const Grid<R> launch, Settings<R> S) {
    const Work w = item<Many>(launch);
    const Dev<R> L = descriptor<R, Many>(launch, w);
    Ctl &c = *L.ctl;
    if (c.stop) return;
    const unsigned lane = threadIdx.x;
    constexpr unsigned kAll = 0xffffffffU;
    if (lane == 0 && c.nc_rebuild) {
        ++c.node.rebuilds;
        c.nc_rebuild = 0U;
    }
    __syncwarp();
    const std::uint32_t count = c.nc_pairs;
    NodeAcc acc = c.node;
    const bool respond = S.nc_mode == 2U;
    for (std::uint32_t at = 0; at < count;) {
        const std::uint32_t q = at + lane;
        bool tested = false, acts = false, impulse_on = false;
        std::uint32_t a = 0, b = 0;
        R gap = R(0), ma = R(0), mb = R(0), impulse = R(0), pair_inverse = R(0), ia = R(0), ib = R(0);
        V3<R> n{}, va{}, vb{};
        if (q < count) {
            a = L.nc_pa[q];
            b = L.nc_pb[q];
            const std::uint32_t bond = L.nc_pbond[q];
            const Q4<R> qa = L.v[a], qb = L.v[b];
            ma = qa.w;
            mb = qb.w;
            const bool held = bond != kNoBond && !(L.rec[bond].a & kDeadBit);
            if (!held && !(ma <= R(0) || mb <= R(0))) {
                tested = true;
                const V3<R> r = pos(L, b) - pos(L, a);
                const R distance = length(r);
                n = normalized(r);
                gap = distance - R(2) * S.nc_radius;
                if (respond) {
                    va = xyz(qa);
                    vb = xyz(qb);
                    const R vn = dot(vb - va, n);
                    if (!(gap > maxR(S.nc_margin, -vn * S.dt))) {
                        ia = R(1) / ma;
                        ib = R(1) / mb;
                        pair_inverse = ia + ib;
                        const R restitution = -vn > S.nc_threshold ? S.nc_restitution : R(0);
                        const R desired = gap > S.nc_margin ? -gap / S.dt : -restitution * minR(vn, R(0));
                        impulse = maxR(R(0), (desired - vn) / pair_inverse);
                        impulse_on = impulse > R(0);
                        acts = impulse_on || gap < -S.nc_margin;
                    }
                }
            }
        }
        const unsigned acting = __ballot_sync(kAll, acts);
        const unsigned first = acting ? static_cast<unsigned>(__ffs(acting)) - 1U : 32U;
        const bool counted = tested && lane <= first;
        acc.pair_tests += static_cast<unsigned long long>(__popc(__ballot_sync(kAll, counted)));
        // The deepest overlap among the counted pairs (a running maximum of
        // the same values, so the order of the lanes does not matter).
        R deepest = counted && gap < R(0) ? -gap : R(0);
        for (int o = 16; o > 0; o >>= 1) deepest = maxR(deepest, __shfl_xor_sync(kAll, deepest, o));
        if (deepest > static_cast<R>(acc.max_overlap)) acc.max_overlap = static_cast<double>(deepest);
        if (first == 32U) {
            at += 32;
            continue;
        }
        double dissipated = 0.0, mx = 0.0, my = 0.0, mz = 0.0;
        R correction = R(0);
        if (lane == first) {
            if (impulse_on) {
                const V3<R> va0 = va, vb0 = vb;
                const R before = R(0.5) * ma * dot(va, va) + R(0.5) * mb * dot(vb, vb);
                const V3<R> j = impulse * n;
                vb = vb + ib * j;
                va = va - ia * j;
                const V3<R> rel = vb - va;
                const V3<R> t = rel - dot(rel, n) * n;
                const R speed = length(t);
                if (speed > R(1.0e-12)) {
                    const V3<R> dir = t / speed;
                    const R stick = speed / pair_inverse;
                    const R friction = stick <= S.nc_static * impulse ? stick : minR(stick, S.nc_dynamic * impulse);
                    const V3<R> f = -friction * dir;
                    vb = vb + ib * f;
                    va = va - ia * f;
                }
                L.v[a] = Q4<R>{va.x, va.y, va.z, ma};
                L.v[b] = Q4<R>{vb.x, vb.y, vb.z, mb};
                dissipated = static_cast<double>(before - (R(0.5) * ma * dot(va, va) + R(0.5) * mb * dot(vb, vb)));
                mx = static_cast<double>(ma * (va.x - va0.x) + mb * (vb.x - vb0.x));
                my = static_cast<double>(ma * (va.y - va0.y) + mb * (vb.y - vb0.y));
                mz = static_cast<double>(ma * (va.z - va0.z) + mb * (vb.z - vb0.z));
            }
            if (gap < -S.nc_margin) {
                correction = minR(-gap - S.nc_margin, R(0.2) * S.nc_radius);
                const V3<R> shift = (correction / pair_inverse) * n;
                const Q4<R> ua = L.u[a], ub = L.u[b];
                const V3<R> na = xyz(ua) - ia * shift, nb = xyz(ub) + ib * shift;
                L.u[a] = Q4<R>{na.x, na.y, na.z, ua.w};
                L.u[b] = Q4<R>{nb.x, nb.y, nb.z, ub.w};
            }
        }
        // The applied pair's sums, folded in list order on every lane.
        if (__shfl_sync(kAll, impulse_on, first)) {
            acc.dissipated += __shfl_sync(kAll, dissipated, first);
            acc.momentum[0] += __shfl_sync(kAll, mx, first);
            acc.momentum[1] += __shfl_sync(kAll, my, first);
            acc.momentum[2] += __shfl_sync(kAll, mz, first);
            ++acc.contacts;
        }
        correction = __shfl_sync(kAll, correction, first);
        if (correction > static_cast<R>(acc.max_correction)) acc.max_correction = static_cast<double>(correction);
        __syncwarp(); // the applied pair's writes, before the next window reads
        at += first + 1U;
    }
    if (lane == 0) c.node = acc;
}

// ---------------------------------------------------------------------------
// Bond order between the state (schedule order) and the device (storage,
// level-major order), moved on the device: upload writes the per-bond arrays
// in schedule order and download reads them in schedule order, so the host
// converts element by element in sequence and never gathers.
// ---------------------------------------------------------------------------
template <class R> struct BondSet {
    std::uint32_t *slot_a, *slot_b;
    BondRec<R> *rec;
    Q4<R> *geo, *prev, *thr4;
    Q2<R> *thr2, *plastic;
    std::uint8_t *mode;
};

__device__ __forceinline__ std::size_t gridStride() { return static_cast<std::size_t>(gridDim.x) * blockDim.x; }
__device__ __forceinline__ std::size_t gridFirst() {
    return static_cast<std::size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
}

// Upload: storage entry dd takes schedule entry dev2sched[dd].
template <class R>
__global__ void __launch_bounds__(kThreads) kBondsToStorage(BondSet<R> dst, BondSet<R> src,
                                                            const std::uint32_t *dev2sched, std::uint32_t B) {
    for (std::size_t dd = gridFirst(); dd < B; dd += gridStride()) {
        const std::uint32_t j = dev2sched[dd];
        dst.slot_a[dd] = src.slot_a[j];
        dst.slot_b[dd] = src.slot_b[j];
        dst.rec[dd] = src.rec[j];
        dst.geo[dd] = src.geo[j];
        dst.prev[dd] = src.prev[j];
        dst.thr4[dd] = src.thr4[j];
        dst.thr2[dd] = src.thr2[j];
        dst.plastic[dd] = src.plastic[j];
        dst.mode[dd] = src.mode[j];
    }
}

// The inverse permutation, schedule index -> storage index.
__global__ void __launch_bounds__(kThreads) kInvertOrder(std::uint32_t *sched2dev, const std::uint32_t *dev2sched,
                                                         std::uint32_t B) {
    for (std::size_t dd = gridFirst(); dd < B; dd += gridStride()) sched2dev[dev2sched[dd]] = static_cast<std::uint32_t>(dd);
}

// Neighbour slots name their bond by schedule index on upload; the device
// keeps storage indices.
__global__ void __launch_bounds__(kThreads) kSlotsToStorage(std::uint32_t *nbr_bond, const std::uint32_t *sched2dev,
                                                            std::size_t P) {
    for (std::size_t s = gridFirst(); s < P; s += gridStride()) {
        const std::uint32_t j = nbr_bond[s];
        if (j != kNoBond) nbr_bond[s] = sched2dev[j];
    }
}

// Download straight into the state's layout: doubles (exact widenings), bonds
// in schedule order, so the host copies each array as it is.
template <class R>
__global__ void __launch_bounds__(kThreads) kNodesOut(double *u, double *up, double *v, const Q4<R> *du,
                                                      const Q4<R> *dup, const Q4<R> *dv, std::uint32_t N) {
    for (std::size_t i = gridFirst(); i < N; i += gridStride()) {
        const Q4<R> a = du[i], b = dup[i], c = dv[i];
        u[3 * i] = a.x; u[3 * i + 1] = a.y; u[3 * i + 2] = a.z;
        up[3 * i] = b.x; up[3 * i + 1] = b.y; up[3 * i + 2] = b.z;
        v[3 * i] = c.x; v[3 * i + 1] = c.y; v[3 * i + 2] = c.z;
    }
}

struct BondsOut {
    std::uint8_t *alive, *mode;
    double *damage, *tensile, *compressive, *shear, *plastic_extension, *plastic_strain;
};

template <class R>
__global__ void __launch_bounds__(kThreads) kBondsOut(BondsOut o, BondSet<R> src, const std::uint32_t *dev2sched,
                                                      std::uint32_t B) {
    for (std::size_t dd = gridFirst(); dd < B; dd += gridStride()) {
        const std::uint32_t j = dev2sched[dd];
        const Q4<R> p = src.prev[dd];
        const Q2<R> pl = src.plastic[dd];
        o.alive[j] = (src.rec[dd].a & kDeadBit) ? 0 : 1;
        o.mode[j] = src.mode[dd];
        o.damage[j] = p.w;
        o.tensile[j] = p.x;
        o.compressive[j] = p.y;
        o.shear[j] = p.z;
        o.plastic_extension[j] = pl.x;
        o.plastic_strain[j] = pl.y;
    }
}

// Upload straight from the state's layout: a chunk of the caller's arrays
// (doubles, schedule order) staged on the device as it is, converted here to
// the device layout (WorkingLattice::fromState, LatticeWorking.hpp:53-124;
// each value rounded once, to nearest, as the host cast rounds it).
struct NodesIn {
    const double *u, *up, *v, *x0, *mass, *inv_mass;
};
template <class R>
__global__ void __launch_bounds__(kThreads) kNodesIn(Q4<R> *du, Q4<R> *dv, Q4<R> *dx0, Q4<R> *dup, NodesIn in,
                                                     std::size_t first, std::size_t n) {
    for (std::size_t k = gridFirst(); k < n; k += gridStride()) {
        const std::size_t i = first + k;
        du[i] = Q4<R>{R(in.u[3 * k]), R(in.u[3 * k + 1]), R(in.u[3 * k + 2]), R(in.inv_mass[k])};
        dv[i] = Q4<R>{R(in.v[3 * k]), R(in.v[3 * k + 1]), R(in.v[3 * k + 2]), R(in.mass[k])};
        dx0[i] = Q4<R>{R(in.x0[3 * k]), R(in.x0[3 * k + 1]), R(in.x0[3 * k + 2]), R(0)};
        dup[i] = Q4<R>{R(in.up[3 * k]), R(in.up[3 * k + 1]), R(in.up[3 * k + 2]), R(0)};
    }
}

// Neighbour slots: (rest, weight if alive), the other node (itself when
// padded), the bond by schedule index (kSlotsToStorage maps it).
struct SlotsIn {
    const double *rest, *weight;
    const std::uint8_t *alive;
    const std::uint32_t *other, *bond;
};
template <class R>
__global__ void __launch_bounds__(kThreads) kSlotsIn(Q4<R> *nbr, std::uint32_t *nbr_other, std::uint32_t *nbr_bond,
                                                     SlotsIn in, std::size_t first, std::size_t n, std::uint32_t N) {
    for (std::size_t k = gridFirst(); k < n; k += gridStride()) {
        const std::size_t s = first + k;
        const std::uint32_t bond = in.bond[k];
        const bool present = bond != kNoBond;
        const R w = R(in.weight[k]);
        nbr[s] = Q4<R>{R(in.rest[3 * k]), R(in.rest[3 * k + 1]), R(in.rest[3 * k + 2]),
                       present ? (in.alive[k] ? w : -absR(w)) : R(0)};
        nbr_other[s] = present ? in.other[k] : static_cast<std::uint32_t>(s % N);
        nbr_bond[s] = bond;
    }
}

// Bonds, in schedule order; `plastic` is set when any bond has flowed.
struct BondsIn {
    const std::uint32_t *a, *b, *slot_a, *slot_b;
    const std::uint8_t *alive, *mode, *last_a, *last_b;
    const double *rsm, *rest, *edge, *compliance, *tensile, *compressive, *shear, *damage, *threshold, *extension,
        *strain;
};
template <class R>
__global__ void __launch_bounds__(kThreads) kBondsIn(BondSet<R> out, BondsIn in, std::size_t first, std::size_t n,
                                                     unsigned *plastic) {
    bool flowed = false;
    for (std::size_t k = gridFirst(); k < n; k += gridStride()) {
        const std::size_t j = first + k;
        out.rec[j] = BondRec<R>{in.a[k] | (in.alive[k] ? 0U : kDeadBit) | (in.last_a[k] ? kLastABit : 0U),
                                in.b[k] | (in.last_b[k] ? kLastBBit : 0U), R(in.rsm[k]), R(in.rest[k])};
        out.geo[j] = Q4<R>{R(in.edge[3 * k]), R(in.edge[3 * k + 1]), R(in.edge[3 * k + 2]), R(in.compliance[k])};
        out.prev[j] = Q4<R>{R(in.tensile[k]), R(in.compressive[k]), R(in.shear[k]), R(in.damage[k])};
        const double *t = in.threshold + 6 * k;
        out.thr4[j] = Q4<R>{R(t[0]), R(t[1]), R(t[2]), R(t[3])};
        out.thr2[j] = Q2<R>{R(t[4]), R(t[5])};
        const Q2<R> pl{R(in.extension[k]), R(in.strain[k])};
        out.plastic[j] = pl;
        flowed = flowed || pl.x != R(0);
        out.slot_a[j] = in.slot_a[k];
        out.slot_b[j] = in.slot_b[k];
        out.mode[j] = in.mode[k];
    }
    if (__any_sync(0xffffffffU, flowed) && (threadIdx.x & 31) == 0) atomicOr(plastic, 1U);
}

// A frame (captureFrame, LatticeWorking.hpp:290-303): positions as float,
// aliveness and damage (as float) by schedule index.
template <class R>
__global__ void __launch_bounds__(kThreads) kFrameOut(float *u, std::uint8_t *alive, float *damage, const Q4<R> *du,
                                                      BondSet<R> src, const std::uint32_t *dev2sched, std::uint32_t N,
                                                      std::uint32_t B) {
    for (std::size_t i = gridFirst(); i < N; i += gridStride()) {
        const Q4<R> a = du[i];
        u[3 * i] = static_cast<float>(a.x);
        u[3 * i + 1] = static_cast<float>(a.y);
        u[3 * i + 2] = static_cast<float>(a.z);
    }
    for (std::size_t dd = gridFirst(); dd < B; dd += gridStride()) {
        const std::uint32_t j = dev2sched[dd];
        alive[j] = (src.rec[dd].a & kDeadBit) ? 0 : 1;
        damage[j] = static_cast<float>(src.prev[dd].w);
    }
}

// Words copied by the device from any memory it can read (host memory in
// place, where the device has coherent pageable access).
__global__ void __launch_bounds__(kThreads) kCopyWords(std::uint32_t *dst, const std::uint32_t *src, std::size_t n) {
    for (std::size_t k = gridFirst(); k < n; k += gridStride()) dst[k] = src[k];
}

} // namespace gbl
