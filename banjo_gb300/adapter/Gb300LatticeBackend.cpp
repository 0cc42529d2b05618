// The reference-side binding of the GB300 lattice library.
//
// Added to the reference tree in place of src/fastlattice/CudaLatticeUnavailable.cpp
// (whose factory only throws), this file implements the reference's own
// LatticeBackend interface (src/fastlattice/FastLattice.hpp:255-369) and its
// CUDA factory and queries (FastLattice.hpp:400-405) over the C ABI of
// include/gbl.h. Every conversion is a member copy between a reference struct
// and its C mirror; the C ABI's result codes are rethrown as the exception
// types the reference's backends throw.
#include "fastlattice/FastLattice.hpp"

#include "gbl.h"

#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace banjo::fastlattice {
namespace {

[[noreturn]] void rethrow(gbl_result rc) {
    char message[1024] = {0};
    gbl_last_error(message, sizeof(message));
    switch (rc) {
    case GBL_INVALID_ARGUMENT: throw std::invalid_argument(message);
    case GBL_OVERFLOW_ERROR: throw std::overflow_error(message);
    case GBL_LOGIC_ERROR: throw std::logic_error(message);
    default: throw std::runtime_error(message);
    }
}

void check(gbl_result rc) {
    if (rc != GBL_OK) rethrow(rc);
}

void put3(double out[3], const V3<double> &v) {
    out[0] = v.x;
    out[1] = v.y;
    out[2] = v.z;
}

gbl_schedule_view scheduleView(const LatticeSchedule &s, std::uint32_t node_count) {
    gbl_schedule_view v{};
    v.node_count = node_count;
    v.bond_count = static_cast<std::uint32_t>(s.bond_order.size());
    v.block_count = s.block_count;
    v.color_count = s.color_count;
    v.boundary_bond_count = s.boundary_bond_count;
    v.node_block_begin = s.node_block_begin.data();
    v.bond_order = s.bond_order.data();
    v.bond_schedule_index = s.bond_schedule_index.data();
    v.bond_block_begin = s.bond_block_begin.data();
    v.range_begin = s.range_begin.data();
    v.range_end = s.range_end.data();
    v.bond_color = s.bond_color.data();
    return v;
}

// The view only reads through its pointers on upload; download writes into the
// vectors, which are sized first (the reference's toState resizes the same way).
gbl_state_view stateView(LatticeState &s) {
    gbl_state_view v{};
    v.origin[0] = s.origin.x;
    v.origin[1] = s.origin.y;
    v.origin[2] = s.origin.z;
    v.node_count = s.node_count;
    v.bond_count = s.bond_count;
    v.max_degree = s.max_degree;
    v.x0 = s.x0.data(); v.u = s.u.data(); v.u_prev = s.u_prev.data(); v.v = s.v.data();
    v.inv_mass = s.inv_mass.data(); v.mass = s.mass.data();
    v.adj_offsets = s.adj_offsets.data(); v.adj_bonds = s.adj_bonds.data();
    v.nbr_bond = s.nbr_bond.data(); v.nbr_other = s.nbr_other.data(); v.nbr_rest = s.nbr_rest.data();
    v.nbr_weight = s.nbr_weight.data(); v.nbr_alive = s.nbr_alive.data();
    v.bond_slot_a = s.bond_slot_a.data(); v.bond_slot_b = s.bond_slot_b.data();
    v.bond_a = s.bond_a.data(); v.bond_b = s.bond_b.data();
    v.rest_edge = s.rest_edge.data(); v.rest_length = s.rest_length.data();
    v.rest_length_sq_minus = s.rest_length_sq_minus.data(); v.weight = s.weight.data();
    v.compliance = s.compliance.data(); v.threshold = s.threshold.data();
    v.alive = s.alive.data(); v.failure_mode = s.failure_mode.data(); v.damage = s.damage.data();
    v.prev_tensile = s.prev_tensile.data(); v.prev_compressive = s.prev_compressive.data();
    v.prev_shear = s.prev_shear.data();
    v.plastic_extension = s.plastic_extension.data(); v.plastic_strain = s.plastic_strain.data();
    return v;
}

gbl_step_settings settingsOf(const StepSettings<double> &s) {
    gbl_step_settings o{};
    o.dt = s.dt;
    put3(o.gravity, s.gravity);
    o.constraint_iterations = s.constraint_iterations;
    o.bond_integrator = s.bond_integrator;
    o.damping_fraction = s.damping_fraction;
    o.sphere_enabled = s.sphere_enabled;
    o.direct_arithmetic = s.direct_arithmetic;
    o.audit_energy = s.audit_energy;
    o.plastic_yield_stretch = s.plastic_yield_stretch;
    o.plastic_hardening = s.plastic_hardening;
    o.plate_half_thickness = s.plate_half_thickness;
    o.contact = {s.contact.static_friction, s.contact.dynamic_friction, s.contact.restitution,
                 s.contact.restitution_speed_threshold, s.contact.node_contact_radius, s.contact.contact_margin,
                 s.contact.prefilter_slack};
    o.node_contact.mode = s.node_contact.mode;
    o.node_contact.radius = s.node_contact.radius;
    o.node_contact.skin = s.node_contact.skin;
    o.node_contact.margin = s.node_contact.margin;
    o.node_contact.restitution = s.node_contact.restitution;
    o.node_contact.restitution_speed_threshold = s.node_contact.restitution_speed_threshold;
    o.node_contact.static_friction = s.node_contact.static_friction;
    o.node_contact.dynamic_friction = s.node_contact.dynamic_friction;
    o.node_contact.bucket_mask = s.node_contact.bucket_mask;
    o.plane_count = s.support.plane_count;
    for (unsigned p = 0; p < kMaxSupportPlanes && p < GBL_MAX_SUPPORT_PLANES; ++p) {
        const SupportPlane<double> &in = s.support.planes[p];
        gbl_support_plane &pl = o.planes[p];
        put3(pl.point, in.point); put3(pl.normal, in.normal);
        put3(pl.tangent, in.tangent); put3(pl.bitangent, in.bitangent);
        pl.restitution = in.restitution;
        pl.static_friction = in.static_friction;
        pl.dynamic_friction = in.dynamic_friction;
        pl.node_radius = in.node_radius;
        pl.reach_capped = in.reach_capped;
        pl.footprint_count = in.footprint_count;
        for (unsigned f = 0; f < kMaxFootprints && f < GBL_MAX_FOOTPRINTS; ++f)
            pl.footprints[f] = {in.footprints[f].center_t, in.footprints[f].center_b, in.footprints[f].half_t,
                                in.footprints[f].half_b};
    }
    return o;
}

gbl_sphere sphereOf(const SphereState<double> &s) {
    gbl_sphere o{};
    put3(o.center, s.center);
    put3(o.velocity, s.velocity);
    put3(o.angular_velocity, s.angular_velocity);
    o.radius = s.radius;
    o.mass = s.mass;
    o.inertia = s.inertia;
    return o;
}

SphereState<double> sphereOf(const gbl_sphere &s) {
    SphereState<double> o{};
    o.center = {s.center[0], s.center[1], s.center[2]};
    o.velocity = {s.velocity[0], s.velocity[1], s.velocity[2]};
    o.angular_velocity = {s.angular_velocity[0], s.angular_velocity[1], s.angular_velocity[2]};
    o.radius = s.radius;
    o.mass = s.mass;
    o.inertia = s.inertia;
    return o;
}

void statusOf(const gbl_run_status &s, RunStatus &o) {
    o.bond_integrator = kBondXpbd;
    o.total_steps = s.total_steps;
    o.first_failure_step = s.first_failure_step;
    o.last_failure_step = s.last_failure_step;
    o.failure_rounds = s.failure_rounds;
    o.broken_bonds = s.broken_bonds;
    o.removed_energy_j = s.removed_energy_j;
    o.last_energy_gain_step = s.last_energy_gain_step;
    o.max_damage = s.max_damage;
    o.last_damage_gain_step = s.last_damage_gain_step;
    o.contact.impulse_contacts = s.contact.impulse_contacts;
    o.contact.impulse_to_material_x = s.contact.impulse_to_material_x;
    o.contact.impulse_to_material_y = s.contact.impulse_to_material_y;
    o.contact.impulse_to_material_z = s.contact.impulse_to_material_z;
    o.contact.dissipated_kinetic_energy_j = s.contact.dissipated_kinetic_energy_j;
    o.contact.maximum_penetration_m = s.contact.maximum_penetration_m;
    o.contact.maximum_position_correction_m = s.contact.maximum_position_correction_m;
    o.contact.maximum_center_shift_m = s.contact.maximum_center_shift_m;
    o.contact.candidate_overflow = s.contact.candidate_overflow;
    o.contact.ball_support_events = s.contact.ball_support_events;
    o.external_load.steps = s.external_load.steps;
    o.external_load.elapsed_s = s.external_load.elapsed_s;
    o.external_load.requested_impulse_n_s = {s.external_load.requested_impulse_n_s[0],
                                             s.external_load.requested_impulse_n_s[1],
                                             s.external_load.requested_impulse_n_s[2]};
    o.external_load.impulse_n_s = {s.external_load.impulse_n_s[0], s.external_load.impulse_n_s[1],
                                   s.external_load.impulse_n_s[2]};
    o.external_load.requested_angular_impulse_kg_m2_s = {s.external_load.requested_angular_impulse_kg_m2_s[0],
                                                         s.external_load.requested_angular_impulse_kg_m2_s[1],
                                                         s.external_load.requested_angular_impulse_kg_m2_s[2]};
    o.external_load.angular_impulse_kg_m2_s = {s.external_load.angular_impulse_kg_m2_s[0],
                                               s.external_load.angular_impulse_kg_m2_s[1],
                                               s.external_load.angular_impulse_kg_m2_s[2]};
    o.external_load.work_j = s.external_load.work_j;
    o.exit_reason = s.exit_reason;
    o.launches = s.launches;
    o.kernel_seconds = s.kernel_seconds;
    o.wall_seconds = s.wall_seconds;
    o.frames_captured = s.frames_captured;
    for (unsigned p = 0; p < kPhaseCount && p < GBL_PHASE_COUNT; ++p) o.phase_seconds[p] = s.phase_seconds[p];
    o.max_tensile_stretch = s.max_tensile_stretch;
    o.max_compressive_strain = s.max_compressive_strain;
    o.max_shear_strain = s.max_shear_strain;
    o.rank_deficient_nodes = s.rank_deficient_nodes;
    o.plastic_work_j = s.plastic_work_j;
    o.max_plastic_stretch = s.max_plastic_stretch;
    o.node_contact.contacts = s.node_contact.contacts;
    o.node_contact.pair_tests = s.node_contact.pair_tests;
    o.node_contact.rebuilds = s.node_contact.rebuilds;
    o.node_contact.pairs_listed = s.node_contact.pairs_listed;
    o.node_contact.pair_overflow = s.node_contact.pair_overflow;
    o.node_contact.dissipated_kinetic_energy_j = s.node_contact.dissipated_kinetic_energy_j;
    o.node_contact.maximum_overlap_m = s.node_contact.maximum_overlap_m;
    o.node_contact.maximum_position_correction_m = s.node_contact.maximum_position_correction_m;
    o.node_contact.momentum_residual_x = s.node_contact.momentum_residual_x;
    o.node_contact.momentum_residual_y = s.node_contact.momentum_residual_y;
    o.node_contact.momentum_residual_z = s.node_contact.momentum_residual_z;
    o.damping_dissipated_j = s.damping_dissipated_j;
    o.striker_dissipated_j = s.striker_dissipated_j;
    o.energy_audited = s.energy_audited != 0;
}

class Gb300LatticeBackend final : public LatticeBackend {
public:
    Gb300LatticeBackend(const LatticeSchedule &schedule, Precision precision, unsigned threads_per_block) {
        const std::uint32_t nodes = schedule.node_block_begin.empty() ? 0U : schedule.node_block_begin.back();
        const gbl_schedule_view view = scheduleView(schedule, nodes);
        check(gbl_create(&view, precision == Precision::Double ? GBL_PRECISION_DOUBLE : GBL_PRECISION_FLOAT,
                         threads_per_block, &backend_));
    }
    ~Gb300LatticeBackend() override { gbl_destroy(backend_); }
    Gb300LatticeBackend(const Gb300LatticeBackend &) = delete;
    Gb300LatticeBackend &operator=(const Gb300LatticeBackend &) = delete;

    [[nodiscard]] std::string name() const override {
        char buffer[64] = {0};
        check(gbl_name(backend_, buffer, sizeof(buffer)));
        return buffer;
    }

    void upload(const LatticeState &state, const StepSettings<double> &settings,
                const SphereState<double> &sphere) override {
        gbl_state_view view = stateView(const_cast<LatticeState &>(state));
        const gbl_step_settings s = settingsOf(settings);
        const gbl_sphere sp = sphereOf(sphere);
        check(gbl_upload(backend_, &view, &s, &sp));
        node_count_ = state.node_count;
        bond_count_ = state.bond_count;
        status_ = {};
    }

    void setExternalForces(const std::vector<Vec3> &forces_world_n, std::uint64_t substeps) override {
        std::vector<double> flat(3 * forces_world_n.size());
        for (std::size_t i = 0; i < forces_world_n.size(); ++i) {
            flat[3 * i] = forces_world_n[i].x;
            flat[3 * i + 1] = forces_world_n[i].y;
            flat[3 * i + 2] = forces_world_n[i].z;
        }
        check(gbl_set_external_forces(backend_, flat.empty() ? nullptr : flat.data(), forces_world_n.size(), substeps));
    }

    void setExternalWrenches(const std::vector<ExternalWrench> &wrenches, std::uint64_t substeps) override {
        std::vector<gbl_external_wrench> in(wrenches.size());
        for (std::size_t k = 0; k < wrenches.size(); ++k) {
            const ExternalWrench &w = wrenches[k];
            gbl_external_wrench &o = in[k];
            o.source = w.source.c_str();
            o.nodes = w.nodes.data();
            o.node_count = w.nodes.size();
            const Vec3 *from[3] = {&w.point_world_m, &w.force_n, &w.torque_n_m};
            double *to[3] = {o.point_world_m, o.force_n, o.torque_n_m};
            for (int q = 0; q < 3; ++q) {
                to[q][0] = from[q]->x;
                to[q][1] = from[q]->y;
                to[q][2] = from[q]->z;
            }
        }
        check(gbl_set_external_wrenches(backend_, in.empty() ? nullptr : in.data(), in.size(), substeps));
    }

    RunStatus run(const RunControl &control) override {
        gbl_run_control c{};
        c.max_steps = control.max_steps;
        c.quiet_steps = control.quiet_steps;
        c.min_steps = control.min_steps;
        c.no_failure_steps = control.no_failure_steps;
        c.energy_flat_steps = control.energy_flat_steps;
        c.energy_flat_fraction = control.energy_flat_fraction;
        c.calm_steps = control.calm_steps;
        c.calm_damage_margin = control.calm_damage_margin;
        c.removable_energy_j = control.removable_energy_j;
        c.capture_stride = control.capture_stride;
        c.max_frames = control.max_frames;
        c.steps_per_launch = control.steps_per_launch;
        // std::atomic<bool> of one byte, read between launches.
        c.abandon = reinterpret_cast<const volatile std::uint8_t *>(control.abandon);
        gbl_run_status s{};
        const gbl_result rc = gbl_run(backend_, &c, &s);
        readSources();
        check(rc);
        statusOf(s, status_);
        return status_;
    }

    void download(LatticeState &state, SphereState<double> &sphere) override {
        state.node_count = node_count_;
        state.bond_count = bond_count_;
        state.u.resize(3 * static_cast<std::size_t>(node_count_));
        state.u_prev.resize(3 * static_cast<std::size_t>(node_count_));
        state.v.resize(3 * static_cast<std::size_t>(node_count_));
        for (auto *v : {&state.damage, &state.prev_tensile, &state.prev_compressive, &state.prev_shear,
                        &state.plastic_extension, &state.plastic_strain})
            v->resize(bond_count_);
        state.alive.resize(bond_count_);
        state.failure_mode.resize(bond_count_);
        gbl_state_view view = stateView(state);
        gbl_sphere sp{};
        check(gbl_download(backend_, &view, &sp));
        sphere = sphereOf(sp);
    }

    std::vector<FrameCapture> takeFrames() override {
        std::uint64_t n = 0;
        check(gbl_frame_count(backend_, &n));
        std::vector<FrameCapture> frames(n);
        for (std::uint64_t k = 0; k < n; ++k) {
            FrameCapture &f = frames[k];
            f.u.resize(3 * static_cast<std::size_t>(node_count_));
            f.alive.resize(bond_count_);
            f.damage.resize(bond_count_);
            gbl_sphere sp{};
            check(gbl_take_frame(backend_, k, &f.step, f.u.data(), f.alive.data(), f.damage.data(), &sp));
            f.sphere = sphereOf(sp);
        }
        check(gbl_clear_frames(backend_));
        status_.frames_captured = 0;
        return frames;
    }

    [[nodiscard]] const RunStatus &status() const override { return status_; }

    [[nodiscard]] std::vector<std::uint32_t> firstFailureBonds() const override {
        std::uint64_t n = 0;
        check(gbl_first_failure_bonds(backend_, nullptr, 0, &n));
        std::vector<std::uint32_t> out(n);
        check(gbl_first_failure_bonds(backend_, out.data(), n, &n));
        return out;
    }

private:
    // RunStatus::external_sources, read back after every run.
    void readSources() {
        std::uint64_t n = 0;
        check(gbl_external_source_count(backend_, &n));
        status_.external_sources.resize(n);
        for (std::uint64_t k = 0; k < n; ++k) {
            std::size_t length = 0;
            check(gbl_external_source(backend_, k, nullptr, 0, &length, nullptr));
            std::string name(length + 1, '\0');
            gbl_load_ledger g{};
            check(gbl_external_source(backend_, k, name.data(), name.size(), &length, &g));
            name.resize(length);
            ExternalWrenchLedger &o = status_.external_sources[k];
            o.source = name;
            o.load.steps = g.steps;
            o.load.elapsed_s = g.elapsed_s;
            o.load.requested_impulse_n_s = {g.requested_impulse_n_s[0], g.requested_impulse_n_s[1],
                                            g.requested_impulse_n_s[2]};
            o.load.impulse_n_s = {g.impulse_n_s[0], g.impulse_n_s[1], g.impulse_n_s[2]};
            o.load.requested_angular_impulse_kg_m2_s = {g.requested_angular_impulse_kg_m2_s[0],
                                                        g.requested_angular_impulse_kg_m2_s[1],
                                                        g.requested_angular_impulse_kg_m2_s[2]};
            o.load.angular_impulse_kg_m2_s = {g.angular_impulse_kg_m2_s[0], g.angular_impulse_kg_m2_s[1],
                                              g.angular_impulse_kg_m2_s[2]};
            o.load.work_j = g.work_j;
        }
    }

    gbl_backend *backend_{};
    RunStatus status_{};
    std::uint32_t node_count_{}, bond_count_{};
};

} // namespace

std::unique_ptr<LatticeBackend> makeCudaLatticeBackend(const LatticeSchedule &schedule, Precision precision,
                                                       unsigned threads_per_block) {
    return std::make_unique<Gb300LatticeBackend>(schedule, precision, threads_per_block);
}

bool cudaLatticeAvailable() { return gbl_available() != 0; }

std::string cudaLatticeDescription() {
    char buffer[256] = {0};
    gbl_description(buffer, sizeof(buffer));
    return buffer;
}

unsigned cudaLatticeMultiprocessorCount() { return gbl_multiprocessor_count(); }

} // namespace banjo::fastlattice
