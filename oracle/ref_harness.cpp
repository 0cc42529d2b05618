// Reference harness: runs the reference's own lattice lane on a case file.
//
// Test infrastructure only. Compiled (oracle/Makefile, target `ref`) from this
// file plus the reference's sources where they lie, never copied. It builds the
// asset and matter of a case through the reference's public types
// (matter/Lattice.hpp LatticeAsset, fracture/ActiveMatter.hpp ActiveMatter),
// then calls
//   buildLatticeSchedule      src/fastlattice/LatticeSchedule.cpp:71
//   buildLatticeState         src/fastlattice/FastLattice.cpp:47
//   makeCpuLatticeBackend     src/fastlattice/CpuLatticeBackend.cpp:569
//   makeParallelCpuLatticeBackend (ParallelCpuLatticeBackend.cpp:2015)
//   LatticeBackend::upload/setExternalForces/setExternalWrenches/run/download (FastLattice.hpp:255-369)
// and writes the schedule, the final state and the RunStatus to an output case.
//
// usage: ref_harness <case> <out> [float|double] [serial|parallel] [threads] [--per-substep]
#include "fastlattice/FastLattice.hpp"
#include "fastlattice/LatticeSchedule.hpp"
#include "matter/Lattice.hpp"
#include "matter/BoxLattice.hpp"
#include "material/MaterialCompiler.hpp"

#include "case_layout.hpp"
#include "lsio.hpp"

#include <chrono>
#include <cstdio>
#include <cstring>
#include <limits>
#include <memory>
#include <string>
#include <vector>

using namespace banjo;
using namespace banjo::fastlattice;

namespace {

V3<double> v3at(const std::vector<double> &s, int at) { return {s[at], s[at + 1], s[at + 2]}; }

StepSettings<double> unpackSettings(const std::vector<double> &s) {
    if (s.size() != static_cast<std::size_t>(lsio::kSettingsWidth) &&
        s.size() != static_cast<std::size_t>(lsio::kAuditEnergy) &&
        s.size() != static_cast<std::size_t>(lsio::kNodeContact))
        throw std::runtime_error("settings width");
    StepSettings<double> out{};
    out.dt = s[lsio::kDt];
    out.gravity = v3at(s, lsio::kGravity);
    out.constraint_iterations = static_cast<std::uint32_t>(s[lsio::kIterations]);
    out.bond_integrator = kBondXpbd;
    out.damping_fraction = s[lsio::kDampingFraction];
    out.sphere_enabled = static_cast<std::uint8_t>(s[lsio::kSphereEnabled]);
    out.direct_arithmetic = static_cast<std::uint8_t>(s[lsio::kDirectArithmetic]);
    out.audit_energy = s.size() > static_cast<std::size_t>(lsio::kAuditEnergy) && s[lsio::kAuditEnergy] != 0 ? 1 : 0;
    out.plastic_yield_stretch = s[lsio::kPlasticYield];
    out.plastic_hardening = s[lsio::kPlasticHardening];
    out.plate_half_thickness = s[lsio::kPlateHalfThickness];
    const int c = lsio::kContact;
    out.contact.static_friction = s[c];
    out.contact.dynamic_friction = s[c + 1];
    out.contact.restitution = s[c + 2];
    out.contact.restitution_speed_threshold = s[c + 3];
    out.contact.node_contact_radius = s[c + 4];
    out.contact.contact_margin = s[c + 5];
    out.contact.prefilter_slack = s[c + 6];
    out.node_contact.mode = kNodeContactOff;
    if (s.size() > static_cast<std::size_t>(lsio::kNodeContact)) {
        const int n = lsio::kNodeContact;
        out.node_contact.mode = static_cast<std::uint8_t>(s[n]);
        out.node_contact.radius = s[n + 1];
        out.node_contact.skin = s[n + 2];
        out.node_contact.margin = s[n + 3];
        out.node_contact.restitution = s[n + 4];
        out.node_contact.restitution_speed_threshold = s[n + 5];
        out.node_contact.static_friction = s[n + 6];
        out.node_contact.dynamic_friction = s[n + 7];
        out.node_contact.bucket_mask = static_cast<std::uint32_t>(s[n + 8]);
    }
    out.support.plane_count = static_cast<std::uint32_t>(s[lsio::kPlaneCount]);
    for (unsigned p = 0; p < kMaxSupportPlanes; ++p) {
        const int b = lsio::kPlanes + static_cast<int>(p) * lsio::kPlaneWidth;
        SupportPlane<double> &pl = out.support.planes[p];
        pl.point = v3at(s, b + lsio::kPlanePoint);
        pl.normal = v3at(s, b + lsio::kPlaneNormal);
        pl.tangent = v3at(s, b + lsio::kPlaneTangent);
        pl.bitangent = v3at(s, b + lsio::kPlaneBitangent);
        pl.restitution = s[b + lsio::kPlaneRestitution];
        pl.static_friction = s[b + lsio::kPlaneStatic];
        pl.dynamic_friction = s[b + lsio::kPlaneDynamic];
        pl.node_radius = s[b + lsio::kPlaneNodeRadius];
        pl.reach_capped = static_cast<std::uint8_t>(s[b + lsio::kPlaneReachCapped]);
        pl.footprint_count = static_cast<std::uint32_t>(s[b + lsio::kPlaneFootprintCount]);
        for (unsigned f = 0; f < kMaxFootprints; ++f) {
            const int o = b + lsio::kPlaneFootprints + 4 * static_cast<int>(f);
            pl.footprints[f] = {s[o], s[o + 1], s[o + 2], s[o + 3]};
        }
    }
    return out;
}

SphereState<double> unpackSphere(const std::vector<double> &s) {
    SphereState<double> out{};
    out.center = v3at(s, 0);
    out.velocity = v3at(s, 3);
    out.angular_velocity = v3at(s, 6);
    out.radius = s[9];
    out.mass = s[10];
    out.inertia = s[11];
    return out;
}

std::vector<double> packSphere(const SphereState<double> &s) {
    return {s.center.x, s.center.y, s.center.z, s.velocity.x, s.velocity.y, s.velocity.z,
            s.angular_velocity.x, s.angular_velocity.y, s.angular_velocity.z, s.radius, s.mass, s.inertia};
}

void packStatus(lsio::Case &out, const RunStatus &st) {
    std::vector<std::uint64_t> u(lsio::kStatusU64Width, 0);
    u[lsio::kTotalSteps] = st.total_steps;
    u[lsio::kFirstFailureStep] = st.first_failure_step;
    u[lsio::kLastFailureStep] = st.last_failure_step;
    u[lsio::kFailureRounds] = st.failure_rounds;
    u[lsio::kBrokenBonds] = st.broken_bonds;
    u[lsio::kLastEnergyGainStep] = st.last_energy_gain_step;
    u[lsio::kLastDamageGainStep] = st.last_damage_gain_step;
    u[lsio::kExitReason] = st.exit_reason;
    u[lsio::kRankDeficientNodes] = st.rank_deficient_nodes;
    u[lsio::kImpulseContacts] = st.contact.impulse_contacts;
    u[lsio::kCandidateOverflow] = st.contact.candidate_overflow;
    u[lsio::kBallSupportEvents] = st.contact.ball_support_events;
    u[lsio::kLaunches] = st.launches;
    u[lsio::kNodeContacts] = st.node_contact.contacts;
    u[lsio::kNodePairTests] = st.node_contact.pair_tests;
    u[lsio::kNodeRebuilds] = st.node_contact.rebuilds;
    u[lsio::kNodePairsListed] = st.node_contact.pairs_listed;
    u[lsio::kNodePairOverflow] = st.node_contact.pair_overflow;
    u[lsio::kEnergyAudited] = st.energy_audited ? 1 : 0;
    std::vector<double> d(lsio::kStatusF64Width, 0.0);
    d[lsio::kRemovedEnergy] = st.removed_energy_j;
    d[lsio::kMaxDamage] = st.max_damage;
    d[lsio::kPlasticWork] = st.plastic_work_j;
    d[lsio::kMaxTensile] = st.max_tensile_stretch;
    d[lsio::kMaxCompressive] = st.max_compressive_strain;
    d[lsio::kMaxShear] = st.max_shear_strain;
    d[lsio::kMaxPlasticStretch] = st.max_plastic_stretch;
    d[lsio::kImpulseX] = st.contact.impulse_to_material_x;
    d[lsio::kImpulseY] = st.contact.impulse_to_material_y;
    d[lsio::kImpulseZ] = st.contact.impulse_to_material_z;
    d[lsio::kContactDissipated] = st.contact.dissipated_kinetic_energy_j;
    d[lsio::kMaxPenetration] = st.contact.maximum_penetration_m;
    d[lsio::kMaxCorrection] = st.contact.maximum_position_correction_m;
    d[lsio::kMaxCenterShift] = st.contact.maximum_center_shift_m;
    d[lsio::kExternalWork] = st.external_load.work_j;
    d[lsio::kExternalImpulseX] = st.external_load.impulse_n_s.x;
    d[lsio::kExternalImpulseY] = st.external_load.impulse_n_s.y;
    d[lsio::kExternalImpulseZ] = st.external_load.impulse_n_s.z;
    d[lsio::kExternalSteps] = static_cast<double>(st.external_load.steps);
    d[lsio::kWallSeconds] = st.wall_seconds;
    d[lsio::kNodeDissipated] = st.node_contact.dissipated_kinetic_energy_j;
    d[lsio::kNodeMaxOverlap] = st.node_contact.maximum_overlap_m;
    d[lsio::kNodeMaxCorrection] = st.node_contact.maximum_position_correction_m;
    d[lsio::kNodeMomentumX] = st.node_contact.momentum_residual_x;
    d[lsio::kNodeMomentumY] = st.node_contact.momentum_residual_y;
    d[lsio::kNodeMomentumZ] = st.node_contact.momentum_residual_z;
    d[lsio::kDampingDissipated] = st.damping_dissipated_j;
    d[lsio::kStrikerDissipated] = st.striker_dissipated_j;
    out.put("status_u64", u);
    out.put("status_f64", d);
    if (!st.external_sources.empty()) {
        std::vector<std::uint8_t> names;
        std::vector<double> ledgers;
        for (const ExternalWrenchLedger &sl : st.external_sources) {
            names.insert(names.end(), sl.source.begin(), sl.source.end());
            names.push_back(0);
            const ExternalLoadLedger &g = sl.load;
            const double row[lsio::kSourceLedgerWidth] = {
                static_cast<double>(g.steps), g.elapsed_s, g.requested_impulse_n_s.x, g.requested_impulse_n_s.y,
                g.requested_impulse_n_s.z, g.impulse_n_s.x, g.impulse_n_s.y, g.impulse_n_s.z,
                g.requested_angular_impulse_kg_m2_s.x, g.requested_angular_impulse_kg_m2_s.y,
                g.requested_angular_impulse_kg_m2_s.z, g.angular_impulse_kg_m2_s.x, g.angular_impulse_kg_m2_s.y,
                g.angular_impulse_kg_m2_s.z, g.work_j};
            ledgers.insert(ledgers.end(), row, row + lsio::kSourceLedgerWidth);
        }
        out.put("source_names", names);
        out.put("source_ledgers", ledgers);
    }
}

// The wrenches of a case file (case_layout.hpp).
std::vector<ExternalWrench> unpackWrenches(const lsio::Case &c) {
    const auto names = c.get<std::uint8_t>("wrench_names");
    const auto counts = c.get<std::uint32_t>("wrench_node_count");
    const auto nodes = c.get<std::uint32_t>("wrench_nodes");
    const auto vec = c.get<double>("wrench_vectors");
    std::vector<ExternalWrench> out(counts.size());
    std::size_t at = 0, node = 0;
    for (std::size_t k = 0; k < out.size(); ++k) {
        ExternalWrench &w = out[k];
        while (at < names.size() && names[at] != 0) w.source.push_back(static_cast<char>(names[at++]));
        ++at;
        w.nodes.assign(nodes.begin() + static_cast<std::ptrdiff_t>(node),
                       nodes.begin() + static_cast<std::ptrdiff_t>(node + counts[k]));
        node += counts[k];
        const double *v = vec.data() + lsio::kWrenchWidth * k;
        w.point_world_m = {v[0], v[1], v[2]};
        w.force_n = {v[3], v[4], v[5]};
        w.torque_n_m = {v[6], v[7], v[8]};
    }
    return out;
}

struct Built {
    std::unique_ptr<LatticeAsset> asset;
    ActiveMatter matter;
};

Built buildFromCase(const lsio::Case &c) {
    Built b;
    const auto N = c.scalar<std::uint32_t>("node_count");
    const auto B = c.scalar<std::uint32_t>("bond_count");
    const auto ref = c.get<double>("ref_pos");
    const auto pos = c.get<double>("pos");
    const auto vel = c.get<double>("vel");
    const auto mass = c.get<double>("mass");
    const auto ba = c.get<std::uint32_t>("bond_a");
    const auto bb = c.get<std::uint32_t>("bond_b");
    const auto rest = c.get<double>("rest_length");
    const auto comp = c.get<double>("compliance");
    const auto thr = c.get<double>("threshold");
    b.asset = std::make_unique<LatticeAsset>();
    b.asset->nodes.resize(N);
    for (std::uint32_t i = 0; i < N; ++i)
        b.asset->nodes[i].local_position_m = Vec3{ref[3 * i], ref[3 * i + 1], ref[3 * i + 2]};
    b.asset->bonds.resize(B);
    for (std::uint32_t k = 0; k < B; ++k) {
        BondRest &r = b.asset->bonds[k];
        r.node_a = ba[k];
        r.node_b = bb[k];
        r.rest_length_m = rest[k];
        r.compliance = comp[k];
        r.damage_start_stretch = thr[6 * k];
        r.damage_end_stretch = thr[6 * k + 1];
        r.compression_damage_start_strain = thr[6 * k + 2];
        r.compression_damage_end_strain = thr[6 * k + 3];
        r.shear_damage_start_strain = thr[6 * k + 4];
        r.shear_damage_end_strain = thr[6 * k + 5];
    }
    b.matter.asset = b.asset.get();
    b.matter.nodes.resize(N);
    b.matter.reference_positions_world_m.resize(N);
    for (std::uint32_t i = 0; i < N; ++i) {
        ActiveNodeState &n = b.matter.nodes[i];
        n.position_world_m = Vec3{pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
        n.previous_position_world_m = n.position_world_m;
        n.velocity_m_s = Vec3{vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]};
        n.mass_kg = mass[i];
        b.matter.reference_positions_world_m[i] = Vec3{ref[3 * i], ref[3 * i + 1], ref[3 * i + 2]};
    }
    b.matter.bonds.resize(B);
    if (c.has("alive")) {
        const auto alive = c.get<std::uint8_t>("alive");
        for (std::uint32_t k = 0; k < B; ++k) b.matter.bonds[k].alive = alive[k] != 0;
    }
    return b;
}

// The notched bar's material: the reference's own compiler, so the oracle thresholds of
// the notched bar are the reference's numbers (MaterialCompiler.cpp:44-214).
void compileMaterial(const lsio::Case &c, lsio::Case &out) {
    const auto m = c.get<double>("material"); // density, E, nu, tensile, yield, hardening, Gc, cell, horizon
    MaterialDefinition material{};
    material.model = MaterialModel::BrittleBond;
    material.density_kg_m3 = m[0];
    material.young_modulus_pa = m[1];
    material.poisson_ratio = m[2];
    material.tensile_strength_pa = m[3];
    // Undeclared compressive and shear strengths compile to disabled ramps
    // (MaterialCompiler.cpp compiledFailureStrain: a zero strain is infinity).
    material.compressive_strength_pa = 0.0;
    material.shear_strength_pa = 0.0;
    material.fracture_energy_j_m2 = m[6];
    material.yield_strength_pa = m[4];
    material.hardening_ratio = m[5];
    const double cell = m[7];
    const unsigned horizon = static_cast<unsigned>(m[8]);
    CompiledBrittleMaterial compiled =
        withEnergyScaledFailure(compileElasticLatticeReference(material, cell, horizon), material, cell, horizon);
    compiled = withPlasticFlow(compiled, material);
    out.put("compiled", std::vector<double>{compiled.bond_compliance, compiled.damage_start_stretch,
                                             compiled.damage_end_stretch, compiled.compression_damage_start_strain,
                                             compiled.compression_damage_end_strain, compiled.shear_damage_start_strain,
                                             compiled.shear_damage_end_strain, compiled.energy_scaled_stretch,
                                             compiled.strength_bound_active ? 1.0 : 0.0, compiled.yield_stretch,
                                             compiled.plastic_hardening_ratio});
}

} // namespace

int main(int argc, char **argv) {
    if (argc < 3) {
        std::fprintf(stderr, "usage: %s <case> <out> [float|double] [serial|parallel] [threads] [--per-substep]\n", argv[0]);
        return 2;
    }
    try {
        lsio::Case c;
        c.read(argv[1]);
        lsio::Case out;
        if (c.has("material")) {
            compileMaterial(c, out);
            if (!c.has("node_count")) { out.write(argv[2]); return 0; }
        }
        const Precision precision =
            (argc > 3 && std::strcmp(argv[3], "double") == 0) ? Precision::Double : Precision::Float;
        const bool parallel = argc > 4 && std::strcmp(argv[4], "parallel") == 0;
        const unsigned threads = argc > 5 ? static_cast<unsigned>(std::stoul(argv[5])) : 0U;
        bool per_substep = false;
        for (int a = 1; a < argc; ++a) per_substep = per_substep || std::strcmp(argv[a], "--per-substep") == 0;

        Built built = buildFromCase(c);
        const auto blocks = c.get<std::uint32_t>("node_block_begin");
        const LatticeSchedule schedule = buildLatticeSchedule(*built.asset, blocks);
        const auto origin_v = c.get<double>("origin");
        const Vec3 origin{origin_v[0], origin_v[1], origin_v[2]};
        LatticeState state = buildLatticeState(built.matter, schedule, origin);
        // A pinned node keeps its mass and takes no motion: the caller-owned
        // state's inverse mass is zeroed, which is how the XPBD lane holds a
        // node still (LatticePhysics.hpp bondSolve weights by inv_mass).
        if (c.has("pinned")) {
            const auto pinned = c.get<std::uint8_t>("pinned");
            for (std::uint32_t i = 0; i < state.node_count; ++i)
                if (pinned[i]) state.inv_mass[i] = 0.0;
        }
        StepSettings<double> settings = unpackSettings(c.get<double>("settings"));
        if (precision == Precision::Double) settings.direct_arithmetic = 1;
        SphereState<double> sphere = unpackSphere(c.get<double>("sphere"));

        out.put("sched_bond_order", schedule.bond_order);
        out.put("sched_color", schedule.bond_color);
        out.put("sched_range_begin", schedule.range_begin);
        out.put("sched_range_end", schedule.range_end);
        out.put("sched_bond_block_begin", schedule.bond_block_begin);
        out.putScalar<std::uint32_t>("sched_color_count", schedule.color_count);
        out.putScalar<std::uint32_t>("sched_boundary_bond_count", schedule.boundary_bond_count);
        out.put("state_adj_bonds", state.adj_bonds);
        out.put("state_nbr_other", state.nbr_other);
        out.putScalar<std::uint32_t>("state_max_degree", state.max_degree);

        std::unique_ptr<LatticeBackend> backend = parallel
            ? makeParallelCpuLatticeBackend(schedule, precision, threads == 0 ? availableCpuCount() : threads)
            : makeCpuLatticeBackend(schedule, precision);
        backend->upload(state, settings, sphere);
        const std::uint64_t steps = c.scalar<std::uint64_t>("steps");
        const std::uint64_t substeps_per_step = c.scalarOr<std::uint64_t>("substeps_per_step", 1);
        // Loads: a constant field for the whole run, or a field ramped linearly
        // in time and re-set every rigid step (span substeps_per_step).
        const bool ramp = c.has("force_ramp_steps");
        std::vector<Vec3> base;
        if (c.has("forces")) {
            const auto f = c.get<double>("forces");
            base.resize(state.node_count);
            for (std::uint32_t i = 0; i < state.node_count; ++i) base[i] = Vec3{f[3 * i], f[3 * i + 1], f[3 * i + 2]};
            if (!ramp) backend->setExternalForces(base, c.scalar<std::uint64_t>("force_substeps"));
        }
        if (c.has("wrench_names")) backend->setExternalWrenches(unpackWrenches(c), c.scalar<std::uint64_t>("wrench_substeps"));
        std::vector<std::uint32_t> break_step(state.bond_count, std::numeric_limits<std::uint32_t>::max());
        std::vector<std::uint8_t> alive_before = state.alive;
        LatticeState scratch = state;
        SphereState<double> sphere_scratch{};
        const auto start = std::chrono::steady_clock::now();
        RunStatus status{};
        const std::uint64_t chunk = per_substep ? 1 : (ramp ? substeps_per_step : steps);
        for (std::uint64_t done = 0; done < steps;) {
            if (ramp) {
                const std::uint64_t rigid_step = done / substeps_per_step;
                const double scale = c.scalar<double>("force_ramp_scale") * static_cast<double>(rigid_step) /
                                     static_cast<double>(c.scalar<std::uint64_t>("force_ramp_steps"));
                if (done % substeps_per_step == 0) {
                    std::vector<Vec3> f(base.size());
                    for (std::size_t i = 0; i < f.size(); ++i) f[i] = scale * base[i];
                    backend->setExternalForces(f, substeps_per_step);
                }
            }
            RunControl control{};
            control.max_steps = std::min(chunk, steps - done);
            if (c.has("checkpoint_at")) {
                // Checkpoint and resume: download the state, upload it into
                // a fresh backend (FastLattice.hpp:359-361), carry on.
                const std::uint64_t at = c.scalar<std::uint64_t>("checkpoint_at");
                if (done < at) control.max_steps = std::min(control.max_steps, at - done);
                if (done == at && at != 0) {
                    backend->download(state, sphere);
                    backend = parallel ? makeParallelCpuLatticeBackend(schedule, precision,
                                                                        threads == 0 ? availableCpuCount() : threads)
                                       : makeCpuLatticeBackend(schedule, precision);
                    backend->upload(state, settings, sphere);
                }
            }
            status = backend->run(control);
            done += control.max_steps;
            if (per_substep) {
                backend->download(scratch, sphere_scratch);
                for (std::uint32_t k = 0; k < state.bond_count; ++k)
                    if (alive_before[k] && !scratch.alive[k]) break_step[k] = static_cast<std::uint32_t>(done - 1);
                alive_before = scratch.alive;
            }
        }
        const double wall = std::chrono::duration<double>(std::chrono::steady_clock::now() - start).count();
        backend->download(state, sphere);
        out.put("u", state.u);
        out.put("u_prev", state.u_prev);
        out.put("v", state.v);
        out.put("alive", state.alive);
        out.put("failure_mode", state.failure_mode);
        out.put("damage", state.damage);
        out.put("plastic_extension", state.plastic_extension);
        out.put("plastic_strain", state.plastic_strain);
        out.put("prev_tensile", state.prev_tensile);
        out.put("prev_compressive", state.prev_compressive);
        out.put("prev_shear", state.prev_shear);
        out.put("sphere_out", packSphere(sphere));
        out.put("first_failure_bonds", backend->firstFailureBonds());
        if (per_substep) out.put("break_step", break_step);
        packStatus(out, status);
        out.putScalar<double>("wall_seconds", wall);
        out.putScalar<std::uint32_t>("threads", parallel ? (threads == 0 ? availableCpuCount() : threads) : 1U);
        out.write(argv[2]);
    } catch (const std::exception &e) {
        std::fprintf(stderr, "ref_harness: %s\n", e.what());
        return 1;
    }
    return 0;
}
