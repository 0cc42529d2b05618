// The recording stand-in for the lattice library (see tests/adapter_stub.hpp).
#include "adapter_stub.hpp"

#include <cstring>

namespace stub {

Record &record() {
    static Record r;
    return r;
}

namespace {

template <class T> std::vector<T> grab(const T *p, std::size_t n) {
    return p ? std::vector<T>(p, p + n) : std::vector<T>();
}

void putString(const char *s, char *buffer, size_t capacity) {
    if (!buffer || capacity == 0) return;
    std::strncpy(buffer, s, capacity - 1);
    buffer[capacity - 1] = '\0';
}

// A distinct value per field: field k of a struct gets base + k.
double field(double base, unsigned k) { return base + static_cast<double>(k); }

} // namespace

gbl_load_ledger sourceLedger(unsigned k) {
    gbl_load_ledger g{};
    const double b = 500.0 + 100.0 * k;
    g.steps = 40 + k;
    g.elapsed_s = field(b, 1);
    for (int q = 0; q < 3; ++q) {
        g.requested_impulse_n_s[q] = field(b, 2 + q);
        g.impulse_n_s[q] = field(b, 5 + q);
        g.requested_angular_impulse_kg_m2_s[q] = field(b, 8 + q);
        g.angular_impulse_kg_m2_s[q] = field(b, 11 + q);
    }
    g.work_j = field(b, 14);
    return g;
}

const char *sourceName(unsigned k) { return k == 0 ? "grip-left" : "grip-right"; }

gbl_run_status statusPattern() {
    gbl_run_status s{};
    s.total_steps = 101;
    s.first_failure_step = 102;
    s.last_failure_step = 103;
    s.failure_rounds = 104;
    s.broken_bonds = 105;
    s.removed_energy_j = 106.5;
    s.last_energy_gain_step = 107;
    s.max_damage = 108.5;
    s.last_damage_gain_step = 109;
    s.contact.impulse_contacts = 110;
    s.contact.impulse_to_material_x = 111.5;
    s.contact.impulse_to_material_y = 112.5;
    s.contact.impulse_to_material_z = 113.5;
    s.contact.dissipated_kinetic_energy_j = 114.5;
    s.contact.maximum_penetration_m = 115.5;
    s.contact.maximum_position_correction_m = 116.5;
    s.contact.maximum_center_shift_m = 117.5;
    s.contact.candidate_overflow = 118;
    s.contact.ball_support_events = 119;
    s.external_load = sourceLedger(7);
    s.exit_reason = 4;
    s.launches = 121;
    s.kernel_seconds = 122.5;
    s.wall_seconds = 123.5;
    s.frames_captured = 124;
    for (unsigned p = 0; p < GBL_PHASE_COUNT; ++p) s.phase_seconds[p] = 200.5 + p;
    s.max_tensile_stretch = 125.5F;
    s.max_compressive_strain = 126.5F;
    s.max_shear_strain = 127.5F;
    s.rank_deficient_nodes = 128;
    s.plastic_work_j = 129.5;
    s.max_plastic_stretch = 130.5F;
    s.node_contact.contacts = 131;
    s.node_contact.pair_tests = 132;
    s.node_contact.rebuilds = 133;
    s.node_contact.pairs_listed = 134;
    s.node_contact.pair_overflow = 135;
    s.node_contact.dissipated_kinetic_energy_j = 136.5;
    s.node_contact.maximum_overlap_m = 137.5;
    s.node_contact.maximum_position_correction_m = 138.5;
    s.node_contact.momentum_residual_x = 139.5;
    s.node_contact.momentum_residual_y = 140.5;
    s.node_contact.momentum_residual_z = 141.5;
    s.damping_dissipated_j = 142.5;
    s.striker_dissipated_j = 143.5;
    s.energy_audited = 1;
    return s;
}

gbl_sphere downloadedSphere() {
    gbl_sphere s{};
    for (int q = 0; q < 3; ++q) {
        s.center[q] = field(900.0, q);
        s.velocity[q] = field(910.0, q);
        s.angular_velocity[q] = field(920.0, q);
    }
    s.radius = 930.5;
    s.mass = 931.5;
    s.inertia = 932.5;
    return s;
}

// Download arrays: 0 u, 1 u_prev, 2 v, 3 alive, 4 failure_mode, 5 damage,
// 6 prev_tensile, 7 prev_compressive, 8 prev_shear, 9 plastic_extension,
// 10 plastic_strain.
double downloaded(unsigned array, std::size_t i) {
    if (array == 3) return static_cast<double>((i + 1) % 2);
    if (array == 4) return static_cast<double>(1 + i % 3);
    return 10000.0 * (array + 1) + 0.25 * static_cast<double>(i);
}

// Frame arrays: 0 u, 1 alive, 2 damage.
float frameValue(unsigned frame, unsigned array, std::size_t i) {
    if (array == 1) return static_cast<float>((i + frame) % 2);
    return 50.0F * static_cast<float>(frame + 1) + 10.0F * static_cast<float>(array) + 0.5F * static_cast<float>(i);
}

gbl_sphere frameSphere(unsigned frame) {
    gbl_sphere s = downloadedSphere();
    s.radius += frame;
    return s;
}

} // namespace stub

using stub::record;

extern "C" {

struct gbl_backend {
    std::uint32_t nodes, bonds;
};

int gbl_available(void) { return 1; }
gbl_result gbl_description(char *buffer, size_t capacity) {
    stub::putString(stub::kDescription, buffer, capacity);
    return GBL_OK;
}
unsigned gbl_multiprocessor_count(void) { return stub::kMultiprocessors; }
gbl_result gbl_last_error(char *buffer, size_t capacity) {
    stub::putString("stub: no error", buffer, capacity);
    return GBL_OK;
}

gbl_result gbl_create(const gbl_schedule_view *s, int precision, unsigned threads_per_block, gbl_backend **out) {
    stub::Record &r = record();
    r.schedule = *s;
    const std::size_t blocks = s->block_count, B = s->bond_count;
    const std::size_t ranges = blocks * 2 * (s->color_count ? s->color_count : 1);
    r.node_block_begin = stub::grab(s->node_block_begin, blocks + 1);
    r.bond_order = stub::grab(s->bond_order, B);
    r.bond_schedule_index = stub::grab(s->bond_schedule_index, B);
    r.bond_block_begin = stub::grab(s->bond_block_begin, blocks + 1);
    r.range_begin = stub::grab(s->range_begin, ranges);
    r.range_end = stub::grab(s->range_end, ranges);
    r.bond_color = stub::grab(s->bond_color, B);
    r.precision = precision;
    r.threads_per_block = threads_per_block;
    *out = new gbl_backend{s->node_count, s->bond_count};
    return GBL_OK;
}

void gbl_destroy(gbl_backend *b) {
    ++record().destroyed;
    delete b;
}

gbl_result gbl_name(const gbl_backend *, char *buffer, size_t capacity) {
    stub::putString(stub::kName, buffer, capacity);
    return GBL_OK;
}

gbl_result gbl_upload(gbl_backend *, const gbl_state_view *v, const gbl_step_settings *settings,
                      const gbl_sphere *sphere) {
    stub::Record &r = record();
    r.state = *v;
    const std::size_t N = v->node_count, B = v->bond_count, D = v->max_degree;
    r.x0 = stub::grab(v->x0, 3 * N);
    r.u = stub::grab<double>(v->u, 3 * N);
    r.u_prev = stub::grab<double>(v->u_prev, 3 * N);
    r.v = stub::grab<double>(v->v, 3 * N);
    r.inv_mass = stub::grab(v->inv_mass, N);
    r.mass = stub::grab(v->mass, N);
    r.adj_offsets = stub::grab(v->adj_offsets, N + 1);
    r.adj_bonds = stub::grab(v->adj_bonds, r.adj_offsets.empty() ? 0 : r.adj_offsets.back());
    r.nbr_bond = stub::grab(v->nbr_bond, D * N);
    r.nbr_other = stub::grab(v->nbr_other, D * N);
    r.nbr_rest = stub::grab(v->nbr_rest, 3 * D * N);
    r.nbr_weight = stub::grab(v->nbr_weight, D * N);
    r.nbr_alive = stub::grab(v->nbr_alive, D * N);
    r.bond_slot_a = stub::grab(v->bond_slot_a, B);
    r.bond_slot_b = stub::grab(v->bond_slot_b, B);
    r.bond_a = stub::grab(v->bond_a, B);
    r.bond_b = stub::grab(v->bond_b, B);
    r.rest_edge = stub::grab(v->rest_edge, 3 * B);
    r.rest_length = stub::grab(v->rest_length, B);
    r.rest_length_sq_minus = stub::grab(v->rest_length_sq_minus, B);
    r.weight = stub::grab(v->weight, B);
    r.compliance = stub::grab(v->compliance, B);
    r.threshold = stub::grab(v->threshold, 6 * B);
    r.alive = stub::grab<std::uint8_t>(v->alive, B);
    r.failure_mode = stub::grab<std::uint8_t>(v->failure_mode, B);
    r.damage = stub::grab<double>(v->damage, B);
    r.prev_tensile = stub::grab<double>(v->prev_tensile, B);
    r.prev_compressive = stub::grab<double>(v->prev_compressive, B);
    r.prev_shear = stub::grab<double>(v->prev_shear, B);
    r.plastic_extension = stub::grab<double>(v->plastic_extension, B);
    r.plastic_strain = stub::grab<double>(v->plastic_strain, B);
    r.settings = *settings;
    r.sphere = *sphere;
    return GBL_OK;
}

gbl_result gbl_set_external_forces(gbl_backend *, const double *f, uint64_t count, uint64_t substeps) {
    stub::Record &r = record();
    r.forces = stub::grab(f, 3 * count);
    r.force_count = count;
    r.force_substeps = substeps;
    return GBL_OK;
}

gbl_result gbl_set_external_wrenches(gbl_backend *, const gbl_external_wrench *w, uint64_t count, uint64_t substeps) {
    stub::Record &r = record();
    r.wrenches.clear();
    for (uint64_t k = 0; k < count; ++k) {
        stub::Record::Wrench o;
        o.source = w[k].source;
        o.nodes = stub::grab(w[k].nodes, w[k].node_count);
        std::memcpy(o.point, w[k].point_world_m, sizeof(o.point));
        std::memcpy(o.force, w[k].force_n, sizeof(o.force));
        std::memcpy(o.torque, w[k].torque_n_m, sizeof(o.torque));
        r.wrenches.push_back(o);
    }
    r.wrench_substeps = substeps;
    return GBL_OK;
}

gbl_result gbl_external_source_count(gbl_backend *, uint64_t *count) {
    *count = record().runs ? stub::kSources : 0;
    return GBL_OK;
}

gbl_result gbl_external_source(gbl_backend *, uint64_t index, char *name, size_t capacity, size_t *length,
                               gbl_load_ledger *ledger) {
    const char *n = stub::sourceName(static_cast<unsigned>(index));
    *length = std::strlen(n);
    stub::putString(n, name, capacity);
    if (ledger) *ledger = stub::sourceLedger(static_cast<unsigned>(index));
    return GBL_OK;
}

gbl_result gbl_run(gbl_backend *, const gbl_run_control *control, gbl_run_status *status) {
    stub::Record &r = record();
    r.control = *control;
    ++r.runs;
    *status = stub::statusPattern();
    return GBL_OK;
}

gbl_result gbl_download(gbl_backend *b, gbl_state_view *v, gbl_sphere *sphere) {
    const std::size_t N = b->nodes, B = b->bonds;
    double *d3[3] = {v->u, v->u_prev, v->v};
    for (unsigned a = 0; a < 3; ++a)
        for (std::size_t i = 0; i < 3 * N; ++i) d3[a][i] = stub::downloaded(a, i);
    for (std::size_t j = 0; j < B; ++j) {
        v->alive[j] = static_cast<std::uint8_t>(stub::downloaded(3, j));
        v->failure_mode[j] = static_cast<std::uint8_t>(stub::downloaded(4, j));
    }
    double *db[6] = {v->damage, v->prev_tensile, v->prev_compressive, v->prev_shear, v->plastic_extension,
                     v->plastic_strain};
    for (unsigned a = 0; a < 6; ++a)
        for (std::size_t j = 0; j < B; ++j) db[a][j] = stub::downloaded(5 + a, j);
    *sphere = stub::downloadedSphere();
    return GBL_OK;
}

gbl_result gbl_first_failure_bonds(const gbl_backend *, uint32_t *out, uint64_t capacity, uint64_t *count) {
    *count = 3;
    for (uint64_t k = 0; k < 3 && k < capacity && out; ++k) out[k] = stub::kFirstFailure[k];
    return GBL_OK;
}

gbl_result gbl_frame_count(const gbl_backend *, uint64_t *count) {
    *count = stub::kFrames;
    return GBL_OK;
}

gbl_result gbl_take_frame(const gbl_backend *b, uint64_t index, uint64_t *step, float *u, uint8_t *alive,
                          float *damage, gbl_sphere *sphere) {
    const unsigned f = static_cast<unsigned>(index);
    *step = 1000 + index;
    for (std::size_t i = 0; i < 3 * static_cast<std::size_t>(b->nodes); ++i) u[i] = stub::frameValue(f, 0, i);
    for (std::size_t j = 0; j < b->bonds; ++j) {
        alive[j] = static_cast<uint8_t>(stub::frameValue(f, 1, j));
        damage[j] = stub::frameValue(f, 2, j);
    }
    *sphere = stub::frameSphere(f);
    return GBL_OK;
}

gbl_result gbl_clear_frames(gbl_backend *) { return GBL_OK; }

} // extern "C"
