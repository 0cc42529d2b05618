// Every field through the reference-side binding, with no device.
//
// Linked with the reference's own objects, the binding
// (banjo_gb300/adapter/Gb300LatticeBackend.cpp) and the recording stand-in for
// the library (tests/adapter_stub.cpp), this program drives the binding as the
// reference's callers do -- makeCudaLatticeBackend, upload, setExternalForces,
// setExternalWrenches, run, download, firstFailureBonds, takeFrames -- with a
// distinct value in every field of every reference struct, and checks that
// each value arrives in its C field (FastLattice.hpp:37-55, 79-128, 182-253;
// LatticePhysics.hpp:114-158, 188-202, 248-284; LatticeSchedule.hpp:28-44),
// and that everything the library hands back arrives in its reference field.
// The field correspondence is written out here a second time, independently
// of the binding, so a dropped or swapped field fails the run.
#include "fastlattice/FastLattice.hpp"
#include "fastlattice/LatticeSchedule.hpp"

#include "adapter_stub.hpp"

#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

using namespace banjo::fastlattice;
using banjo::Vec3;

namespace {

int failures = 0;

void require(bool ok, const std::string &what) {
    if (!ok) {
        ++failures;
        std::printf("[FAIL] %s\n", what.c_str());
    }
}

template <class A, class B> void same(const A &got, const B &want, const std::string &what) {
    require(static_cast<double>(got) == static_cast<double>(want), what);
}

template <class T, class U> void sameVec(const std::vector<T> &got, const std::vector<U> &want, const std::string &what) {
    bool ok = got.size() == want.size();
    for (std::size_t i = 0; ok && i < got.size(); ++i) ok = static_cast<double>(got[i]) == static_cast<double>(want[i]);
    require(ok, what);
}

void same3(const double *got, const Vec3 &want, const std::string &what) {
    same(got[0], want.x, what + ".x");
    same(got[1], want.y, what + ".y");
    same(got[2], want.z, what + ".z");
}

void same3(const double *got, const V3<double> &want, const std::string &what) {
    same(got[0], want.x, what + ".x");
    same(got[1], want.y, what + ".y");
    same(got[2], want.z, what + ".z");
}

// A counter of distinct values for the input fields.
struct Distinct {
    double next = 1.0;
    double operator()() { return next += 1.0; }
};

template <class T> std::vector<T> ramp(std::size_t n, double base, double step = 1.0) {
    std::vector<T> v(n);
    for (std::size_t i = 0; i < n; ++i) v[i] = static_cast<T>(base + step * static_cast<double>(i));
    return v;
}

} // namespace

int main() {
    constexpr std::uint32_t N = 5, B = 7, D = 3, blocks = 2, colors = 3;
    Distinct d;

    LatticeSchedule sched;
    sched.block_count = blocks;
    sched.color_count = colors;
    sched.boundary_bond_count = 2;
    sched.node_block_begin = {0, 3, N};
    sched.bond_order = ramp<std::uint32_t>(B, 40);
    sched.bond_schedule_index = ramp<std::uint32_t>(B, 60);
    sched.bond_block_begin = {0, 4, B};
    sched.range_begin = ramp<std::uint32_t>(blocks * 2 * colors, 80);
    sched.range_end = ramp<std::uint32_t>(blocks * 2 * colors, 100);
    sched.bond_color = ramp<std::uint8_t>(B, 120);

    LatticeState st;
    st.origin = {d(), d(), d()};
    st.node_count = N;
    st.bond_count = B;
    st.max_degree = D;
    st.x0 = ramp<double>(3 * N, 1000.5);
    st.u = ramp<double>(3 * N, 1100.5);
    st.u_prev = ramp<double>(3 * N, 1200.5);
    st.v = ramp<double>(3 * N, 1300.5);
    st.inv_mass = ramp<double>(N, 1400.5);
    st.mass = ramp<double>(N, 1500.5);
    st.adj_offsets = {0, 2, 4, 6, 8, 10};
    st.adj_bonds = ramp<std::uint32_t>(10, 1600);
    st.nbr_bond = ramp<std::uint32_t>(D * N, 1700);
    st.nbr_other = ramp<std::uint32_t>(D * N, 1800);
    st.nbr_rest = ramp<double>(3 * D * N, 1900.5);
    st.nbr_weight = ramp<double>(D * N, 2000.5);
    st.nbr_alive = ramp<std::uint8_t>(D * N, 1);
    st.bond_slot_a = ramp<std::uint32_t>(B, 2100);
    st.bond_slot_b = ramp<std::uint32_t>(B, 2200);
    st.bond_a = ramp<std::uint32_t>(B, 2300);
    st.bond_b = ramp<std::uint32_t>(B, 2400);
    st.rest_edge = ramp<double>(3 * B, 2500.5);
    st.rest_length = ramp<double>(B, 2600.5);
    st.rest_length_sq_minus = ramp<double>(B, 2700.5);
    st.weight = ramp<double>(B, 2800.5);
    st.compliance = ramp<double>(B, 2900.5);
    st.threshold = ramp<double>(6 * B, 3000.5);
    st.alive = ramp<std::uint8_t>(B, 10);
    st.failure_mode = ramp<std::uint8_t>(B, 30);
    st.damage = ramp<double>(B, 3100.5);
    st.prev_tensile = ramp<double>(B, 3200.5);
    st.prev_compressive = ramp<double>(B, 3300.5);
    st.prev_shear = ramp<double>(B, 3400.5);
    st.plastic_extension = ramp<double>(B, 3500.5);
    st.plastic_strain = ramp<double>(B, 3600.5);

    StepSettings<double> s{};
    s.dt = d();
    s.gravity = {d(), d(), d()};
    s.constraint_iterations = 7;
    s.bond_integrator = 0;
    s.damping_fraction = d();
    s.sphere_enabled = 1;
    s.direct_arithmetic = 1;
    s.audit_energy = 1;
    s.plastic_yield_stretch = d();
    s.plastic_hardening = d();
    s.plate_half_thickness = d();
    s.contact = {d(), d(), d(), d(), d(), d(), d()};
    s.node_contact.mode = 2;
    s.node_contact.radius = d();
    s.node_contact.skin = d();
    s.node_contact.margin = d();
    s.node_contact.restitution = d();
    s.node_contact.restitution_speed_threshold = d();
    s.node_contact.static_friction = d();
    s.node_contact.dynamic_friction = d();
    s.node_contact.bucket_mask = 1023;
    s.support.plane_count = 2;
    for (unsigned p = 0; p < kMaxSupportPlanes; ++p) {
        SupportPlane<double> &pl = s.support.planes[p];
        pl.point = {d(), d(), d()};
        pl.normal = {d(), d(), d()};
        pl.tangent = {d(), d(), d()};
        pl.bitangent = {d(), d(), d()};
        pl.restitution = d();
        pl.static_friction = d();
        pl.dynamic_friction = d();
        pl.node_radius = d();
        pl.reach_capped = static_cast<std::uint8_t>(p + 1);
        pl.footprint_count = 3 + p;
        for (unsigned f = 0; f < kMaxFootprints; ++f) pl.footprints[f] = {d(), d(), d(), d()};
    }
    SphereState<double> sphere{{d(), d(), d()}, {d(), d(), d()}, {d(), d(), d()}, d(), d(), d()};

    std::unique_ptr<LatticeBackend> be = makeCudaLatticeBackend(sched, Precision::Double, 384);
    const stub::Record &r = stub::record();
    same(r.precision, GBL_PRECISION_DOUBLE, "create precision");
    same(r.threads_per_block, 384, "create threads_per_block");
    same(r.schedule.node_count, N, "schedule node_count");
    same(r.schedule.bond_count, B, "schedule bond_count");
    same(r.schedule.block_count, blocks, "schedule block_count");
    same(r.schedule.color_count, colors, "schedule color_count");
    same(r.schedule.boundary_bond_count, sched.boundary_bond_count, "schedule boundary_bond_count");
    sameVec(r.node_block_begin, sched.node_block_begin, "schedule node_block_begin");
    sameVec(r.bond_order, sched.bond_order, "schedule bond_order");
    sameVec(r.bond_schedule_index, sched.bond_schedule_index, "schedule bond_schedule_index");
    sameVec(r.bond_block_begin, sched.bond_block_begin, "schedule bond_block_begin");
    sameVec(r.range_begin, sched.range_begin, "schedule range_begin");
    sameVec(r.range_end, sched.range_end, "schedule range_end");
    sameVec(r.bond_color, sched.bond_color, "schedule bond_color");
    require(be->name() == stub::kName, "name");

    be->upload(st, s, sphere);
    same3(r.state.origin, st.origin, "state origin");
    same(r.state.node_count, N, "state node_count");
    same(r.state.bond_count, B, "state bond_count");
    same(r.state.max_degree, D, "state max_degree");
    sameVec(r.x0, st.x0, "state x0");
    sameVec(r.u, st.u, "state u");
    sameVec(r.u_prev, st.u_prev, "state u_prev");
    sameVec(r.v, st.v, "state v");
    sameVec(r.inv_mass, st.inv_mass, "state inv_mass");
    sameVec(r.mass, st.mass, "state mass");
    sameVec(r.adj_offsets, st.adj_offsets, "state adj_offsets");
    sameVec(r.adj_bonds, st.adj_bonds, "state adj_bonds");
    sameVec(r.nbr_bond, st.nbr_bond, "state nbr_bond");
    sameVec(r.nbr_other, st.nbr_other, "state nbr_other");
    sameVec(r.nbr_rest, st.nbr_rest, "state nbr_rest");
    sameVec(r.nbr_weight, st.nbr_weight, "state nbr_weight");
    sameVec(r.nbr_alive, st.nbr_alive, "state nbr_alive");
    sameVec(r.bond_slot_a, st.bond_slot_a, "state bond_slot_a");
    sameVec(r.bond_slot_b, st.bond_slot_b, "state bond_slot_b");
    sameVec(r.bond_a, st.bond_a, "state bond_a");
    sameVec(r.bond_b, st.bond_b, "state bond_b");
    sameVec(r.rest_edge, st.rest_edge, "state rest_edge");
    sameVec(r.rest_length, st.rest_length, "state rest_length");
    sameVec(r.rest_length_sq_minus, st.rest_length_sq_minus, "state rest_length_sq_minus");
    sameVec(r.weight, st.weight, "state weight");
    sameVec(r.compliance, st.compliance, "state compliance");
    sameVec(r.threshold, st.threshold, "state threshold");
    sameVec(r.alive, st.alive, "state alive");
    sameVec(r.failure_mode, st.failure_mode, "state failure_mode");
    sameVec(r.damage, st.damage, "state damage");
    sameVec(r.prev_tensile, st.prev_tensile, "state prev_tensile");
    sameVec(r.prev_compressive, st.prev_compressive, "state prev_compressive");
    sameVec(r.prev_shear, st.prev_shear, "state prev_shear");
    sameVec(r.plastic_extension, st.plastic_extension, "state plastic_extension");
    sameVec(r.plastic_strain, st.plastic_strain, "state plastic_strain");

    const gbl_step_settings &c = r.settings;
    same(c.dt, s.dt, "settings dt");
    same3(c.gravity, s.gravity, "settings gravity");
    same(c.constraint_iterations, s.constraint_iterations, "settings constraint_iterations");
    same(c.bond_integrator, s.bond_integrator, "settings bond_integrator");
    same(c.damping_fraction, s.damping_fraction, "settings damping_fraction");
    same(c.sphere_enabled, s.sphere_enabled, "settings sphere_enabled");
    same(c.direct_arithmetic, s.direct_arithmetic, "settings direct_arithmetic");
    same(c.audit_energy, s.audit_energy, "settings audit_energy");
    same(c.plastic_yield_stretch, s.plastic_yield_stretch, "settings plastic_yield_stretch");
    same(c.plastic_hardening, s.plastic_hardening, "settings plastic_hardening");
    same(c.plate_half_thickness, s.plate_half_thickness, "settings plate_half_thickness");
    same(c.contact.static_friction, s.contact.static_friction, "contact static_friction");
    same(c.contact.dynamic_friction, s.contact.dynamic_friction, "contact dynamic_friction");
    same(c.contact.restitution, s.contact.restitution, "contact restitution");
    same(c.contact.restitution_speed_threshold, s.contact.restitution_speed_threshold, "contact threshold");
    same(c.contact.node_contact_radius, s.contact.node_contact_radius, "contact node_contact_radius");
    same(c.contact.contact_margin, s.contact.contact_margin, "contact contact_margin");
    same(c.contact.prefilter_slack, s.contact.prefilter_slack, "contact prefilter_slack");
    same(c.node_contact.mode, s.node_contact.mode, "node_contact mode");
    same(c.node_contact.radius, s.node_contact.radius, "node_contact radius");
    same(c.node_contact.skin, s.node_contact.skin, "node_contact skin");
    same(c.node_contact.margin, s.node_contact.margin, "node_contact margin");
    same(c.node_contact.restitution, s.node_contact.restitution, "node_contact restitution");
    same(c.node_contact.restitution_speed_threshold, s.node_contact.restitution_speed_threshold,
         "node_contact restitution_speed_threshold");
    same(c.node_contact.static_friction, s.node_contact.static_friction, "node_contact static_friction");
    same(c.node_contact.dynamic_friction, s.node_contact.dynamic_friction, "node_contact dynamic_friction");
    same(c.node_contact.bucket_mask, s.node_contact.bucket_mask, "node_contact bucket_mask");
    same(c.plane_count, s.support.plane_count, "support plane_count");
    for (unsigned p = 0; p < kMaxSupportPlanes; ++p) {
        const std::string k = "plane " + std::to_string(p) + " ";
        const gbl_support_plane &g = c.planes[p];
        const SupportPlane<double> &w = s.support.planes[p];
        same3(g.point, w.point, k + "point");
        same3(g.normal, w.normal, k + "normal");
        same3(g.tangent, w.tangent, k + "tangent");
        same3(g.bitangent, w.bitangent, k + "bitangent");
        same(g.restitution, w.restitution, k + "restitution");
        same(g.static_friction, w.static_friction, k + "static_friction");
        same(g.dynamic_friction, w.dynamic_friction, k + "dynamic_friction");
        same(g.node_radius, w.node_radius, k + "node_radius");
        same(g.reach_capped, w.reach_capped, k + "reach_capped");
        same(g.footprint_count, w.footprint_count, k + "footprint_count");
        for (unsigned f = 0; f < kMaxFootprints; ++f) {
            const std::string kf = k + "footprint " + std::to_string(f) + " ";
            same(g.footprints[f].center_t, w.footprints[f].center_t, kf + "center_t");
            same(g.footprints[f].center_b, w.footprints[f].center_b, kf + "center_b");
            same(g.footprints[f].half_t, w.footprints[f].half_t, kf + "half_t");
            same(g.footprints[f].half_b, w.footprints[f].half_b, kf + "half_b");
        }
    }
    same3(r.sphere.center, sphere.center, "sphere center");
    same3(r.sphere.velocity, sphere.velocity, "sphere velocity");
    same3(r.sphere.angular_velocity, sphere.angular_velocity, "sphere angular_velocity");
    same(r.sphere.radius, sphere.radius, "sphere radius");
    same(r.sphere.mass, sphere.mass, "sphere mass");
    same(r.sphere.inertia, sphere.inertia, "sphere inertia");

    std::vector<Vec3> forces(N);
    for (auto &f : forces) f = {d(), d(), d()};
    be->setExternalForces(forces, 77);
    same(r.force_count, N, "forces count");
    same(r.force_substeps, 77, "forces substeps");
    require(r.forces.size() == 3 * N, "forces size");
    for (std::uint32_t i = 0; i < N && r.forces.size() == 3 * N; ++i) same3(&r.forces[3 * i], forces[i], "force");

    std::vector<ExternalWrench> wrenches(2);
    wrenches[0] = {"grip-left", {4, 1}, {d(), d(), d()}, {d(), d(), d()}, {d(), d(), d()}};
    wrenches[1] = {"grip-right", {2}, {d(), d(), d()}, {d(), d(), d()}, {d(), d(), d()}};
    be->setExternalWrenches(wrenches, 55);
    same(r.wrench_substeps, 55, "wrench substeps");
    require(r.wrenches.size() == 2, "wrench count");
    for (std::size_t k = 0; k < r.wrenches.size() && k < 2; ++k) {
        const std::string kk = "wrench " + std::to_string(k) + " ";
        require(r.wrenches[k].source == wrenches[k].source, kk + "source");
        sameVec(r.wrenches[k].nodes, wrenches[k].nodes, kk + "nodes");
        same3(r.wrenches[k].point, wrenches[k].point_world_m, kk + "point");
        same3(r.wrenches[k].force, wrenches[k].force_n, kk + "force");
        same3(r.wrenches[k].torque, wrenches[k].torque_n_m, kk + "torque");
    }

    std::atomic<bool> abandon{false};
    RunControl ctl;
    ctl.max_steps = 301;
    ctl.quiet_steps = 302;
    ctl.min_steps = 303;
    ctl.no_failure_steps = 304;
    ctl.energy_flat_steps = 305;
    ctl.energy_flat_fraction = 306.5;
    ctl.calm_steps = 307;
    ctl.calm_damage_margin = 308.5;
    ctl.removable_energy_j = 309.5;
    ctl.capture_stride = 310;
    ctl.max_frames = 311;
    ctl.steps_per_launch = 312;
    ctl.abandon = &abandon;
    const RunStatus got = be->run(ctl);
    same(r.control.max_steps, ctl.max_steps, "control max_steps");
    same(r.control.quiet_steps, ctl.quiet_steps, "control quiet_steps");
    same(r.control.min_steps, ctl.min_steps, "control min_steps");
    same(r.control.no_failure_steps, ctl.no_failure_steps, "control no_failure_steps");
    same(r.control.energy_flat_steps, ctl.energy_flat_steps, "control energy_flat_steps");
    same(r.control.energy_flat_fraction, ctl.energy_flat_fraction, "control energy_flat_fraction");
    same(r.control.calm_steps, ctl.calm_steps, "control calm_steps");
    same(r.control.calm_damage_margin, ctl.calm_damage_margin, "control calm_damage_margin");
    same(r.control.removable_energy_j, ctl.removable_energy_j, "control removable_energy_j");
    same(r.control.capture_stride, ctl.capture_stride, "control capture_stride");
    same(r.control.max_frames, ctl.max_frames, "control max_frames");
    same(r.control.steps_per_launch, ctl.steps_per_launch, "control steps_per_launch");
    require(static_cast<const volatile void *>(r.control.abandon) == static_cast<const void *>(&abandon),
            "control abandon flag address");

    const gbl_run_status w = stub::statusPattern();
    same(got.total_steps, w.total_steps, "status total_steps");
    same(got.first_failure_step, w.first_failure_step, "status first_failure_step");
    same(got.last_failure_step, w.last_failure_step, "status last_failure_step");
    same(got.failure_rounds, w.failure_rounds, "status failure_rounds");
    same(got.broken_bonds, w.broken_bonds, "status broken_bonds");
    same(got.removed_energy_j, w.removed_energy_j, "status removed_energy_j");
    same(got.last_energy_gain_step, w.last_energy_gain_step, "status last_energy_gain_step");
    same(got.max_damage, w.max_damage, "status max_damage");
    same(got.last_damage_gain_step, w.last_damage_gain_step, "status last_damage_gain_step");
    same(got.contact.impulse_contacts, w.contact.impulse_contacts, "contact impulse_contacts");
    same(got.contact.impulse_to_material_x, w.contact.impulse_to_material_x, "contact impulse x");
    same(got.contact.impulse_to_material_y, w.contact.impulse_to_material_y, "contact impulse y");
    same(got.contact.impulse_to_material_z, w.contact.impulse_to_material_z, "contact impulse z");
    same(got.contact.dissipated_kinetic_energy_j, w.contact.dissipated_kinetic_energy_j, "contact dissipated");
    same(got.contact.maximum_penetration_m, w.contact.maximum_penetration_m, "contact penetration");
    same(got.contact.maximum_position_correction_m, w.contact.maximum_position_correction_m, "contact correction");
    same(got.contact.maximum_center_shift_m, w.contact.maximum_center_shift_m, "contact center shift");
    same(got.contact.candidate_overflow, w.contact.candidate_overflow, "contact candidate_overflow");
    same(got.contact.ball_support_events, w.contact.ball_support_events, "contact ball_support_events");
    auto ledger = [&](const ExternalLoadLedger &g, const gbl_load_ledger &e, const std::string &k) {
        same(g.steps, e.steps, k + " steps");
        same(g.elapsed_s, e.elapsed_s, k + " elapsed_s");
        same3(e.requested_impulse_n_s, g.requested_impulse_n_s, k + " requested_impulse");
        same3(e.impulse_n_s, g.impulse_n_s, k + " impulse");
        same3(e.requested_angular_impulse_kg_m2_s, g.requested_angular_impulse_kg_m2_s, k + " requested_angular");
        same3(e.angular_impulse_kg_m2_s, g.angular_impulse_kg_m2_s, k + " angular");
        same(g.work_j, e.work_j, k + " work_j");
    };
    ledger(got.external_load, w.external_load, "external_load");
    require(got.external_sources.size() == stub::kSources, "external_sources count");
    for (unsigned k = 0; k < got.external_sources.size() && k < stub::kSources; ++k) {
        require(got.external_sources[k].source == stub::sourceName(k), "external source name");
        ledger(got.external_sources[k].load, stub::sourceLedger(k), "external source " + std::to_string(k));
    }
    same(got.exit_reason, w.exit_reason, "status exit_reason");
    same(got.launches, w.launches, "status launches");
    same(got.kernel_seconds, w.kernel_seconds, "status kernel_seconds");
    same(got.wall_seconds, w.wall_seconds, "status wall_seconds");
    same(got.frames_captured, w.frames_captured, "status frames_captured");
    for (unsigned p = 0; p < kPhaseCount; ++p) same(got.phase_seconds[p], w.phase_seconds[p], "status phase_seconds");
    same(got.max_tensile_stretch, w.max_tensile_stretch, "status max_tensile_stretch");
    same(got.max_compressive_strain, w.max_compressive_strain, "status max_compressive_strain");
    same(got.max_shear_strain, w.max_shear_strain, "status max_shear_strain");
    same(got.rank_deficient_nodes, w.rank_deficient_nodes, "status rank_deficient_nodes");
    same(got.plastic_work_j, w.plastic_work_j, "status plastic_work_j");
    same(got.max_plastic_stretch, w.max_plastic_stretch, "status max_plastic_stretch");
    same(got.node_contact.contacts, w.node_contact.contacts, "node_contact contacts");
    same(got.node_contact.pair_tests, w.node_contact.pair_tests, "node_contact pair_tests");
    same(got.node_contact.rebuilds, w.node_contact.rebuilds, "node_contact rebuilds");
    same(got.node_contact.pairs_listed, w.node_contact.pairs_listed, "node_contact pairs_listed");
    same(got.node_contact.pair_overflow, w.node_contact.pair_overflow, "node_contact pair_overflow");
    same(got.node_contact.dissipated_kinetic_energy_j, w.node_contact.dissipated_kinetic_energy_j,
         "node_contact dissipated");
    same(got.node_contact.maximum_overlap_m, w.node_contact.maximum_overlap_m, "node_contact overlap");
    same(got.node_contact.maximum_position_correction_m, w.node_contact.maximum_position_correction_m,
         "node_contact correction");
    same(got.node_contact.momentum_residual_x, w.node_contact.momentum_residual_x, "node_contact momentum x");
    same(got.node_contact.momentum_residual_y, w.node_contact.momentum_residual_y, "node_contact momentum y");
    same(got.node_contact.momentum_residual_z, w.node_contact.momentum_residual_z, "node_contact momentum z");
    same(got.damping_dissipated_j, w.damping_dissipated_j, "status damping_dissipated_j");
    same(got.striker_dissipated_j, w.striker_dissipated_j, "status striker_dissipated_j");
    require(got.energy_audited == (w.energy_audited != 0), "status energy_audited");
    require(&be->status() != nullptr && be->status().broken_bonds == w.broken_bonds, "status() after run");

    LatticeState out;
    SphereState<double> sp{};
    be->download(out, sp);
    same(out.node_count, N, "download node_count");
    same(out.bond_count, B, "download bond_count");
    auto expect = [&](unsigned a, std::size_t n) {
        std::vector<double> v(n);
        for (std::size_t i = 0; i < n; ++i) v[i] = stub::downloaded(a, i);
        return v;
    };
    sameVec(out.u, expect(0, 3 * N), "download u");
    sameVec(out.u_prev, expect(1, 3 * N), "download u_prev");
    sameVec(out.v, expect(2, 3 * N), "download v");
    sameVec(out.alive, expect(3, B), "download alive");
    sameVec(out.failure_mode, expect(4, B), "download failure_mode");
    sameVec(out.damage, expect(5, B), "download damage");
    sameVec(out.prev_tensile, expect(6, B), "download prev_tensile");
    sameVec(out.prev_compressive, expect(7, B), "download prev_compressive");
    sameVec(out.prev_shear, expect(8, B), "download prev_shear");
    sameVec(out.plastic_extension, expect(9, B), "download plastic_extension");
    sameVec(out.plastic_strain, expect(10, B), "download plastic_strain");
    const gbl_sphere ws = stub::downloadedSphere();
    same3(ws.center, sp.center, "download sphere center");
    same3(ws.velocity, sp.velocity, "download sphere velocity");
    same3(ws.angular_velocity, sp.angular_velocity, "download sphere angular_velocity");
    same(sp.radius, ws.radius, "download sphere radius");
    same(sp.mass, ws.mass, "download sphere mass");
    same(sp.inertia, ws.inertia, "download sphere inertia");

    const std::vector<std::uint32_t> ffb = be->firstFailureBonds();
    sameVec(ffb, std::vector<std::uint32_t>(std::begin(stub::kFirstFailure), std::end(stub::kFirstFailure)),
            "firstFailureBonds");

    const std::vector<FrameCapture> frames = be->takeFrames();
    require(frames.size() == stub::kFrames, "frames count");
    for (unsigned f = 0; f < frames.size() && f < stub::kFrames; ++f) {
        const std::string k = "frame " + std::to_string(f) + " ";
        same(frames[f].step, 1000 + f, k + "step");
        std::vector<double> u(3 * N), alive(B), damage(B);
        for (std::size_t i = 0; i < u.size(); ++i) u[i] = stub::frameValue(f, 0, i);
        for (std::size_t j = 0; j < B; ++j) {
            alive[j] = stub::frameValue(f, 1, j);
            damage[j] = stub::frameValue(f, 2, j);
        }
        sameVec(frames[f].u, u, k + "u");
        sameVec(frames[f].alive, alive, k + "alive");
        sameVec(frames[f].damage, damage, k + "damage");
        same(frames[f].sphere.radius, stub::frameSphere(f).radius, k + "sphere radius");
    }
    same(be->status().frames_captured, 0, "frames_captured cleared by takeFrames");

    require(cudaLatticeAvailable(), "cudaLatticeAvailable");
    require(cudaLatticeDescription() == stub::kDescription, "cudaLatticeDescription");
    same(cudaLatticeMultiprocessorCount(), stub::kMultiprocessors, "cudaLatticeMultiprocessorCount");
    be.reset();
    same(r.destroyed, 1, "destroy on release");

    if (failures == 0) std::printf("[PASS] every field through the binding\n");
    return failures == 0 ? 0 : 1;
}
