/*
 * gbl.h -- C ABI of the GB300 bonded-lattice XPBD fracture substep.
 *
 * This is the drop-in boundary for the reference's lattice step API
 * (src/fastlattice/FastLattice.hpp:255-405, class LatticeBackend and its
 * factories). It replaces the removed CUDA backend, whose factory survives as a
 * stub that throws (src/fastlattice/CudaLatticeUnavailable.cpp:11-25). Every
 * struct below mirrors a reference struct field for field, in plain C types, so
 * a C++ adapter (banjo_gb300/adapter/Gb300LatticeBackend.cpp) converts by member
 * copies and the library needs no reference headers. No torch or CUDA types appear in any signature.
 *
 * Errors: every entry point returns a gbl_result. A non-zero value is the C
 * image of the exception the reference throws in the same situation
 * (FastLattice.hpp:263-358): GBL_INVALID_ARGUMENT for std::invalid_argument,
 * GBL_RUNTIME_ERROR for std::runtime_error (no device, device failure),
 * GBL_OVERFLOW_ERROR for std::overflow_error, GBL_LOGIC_ERROR for
 * std::logic_error. gbl_last_error() returns the message of the last failure
 * on the calling thread.
 *
 * Threading: one host thread per backend between run calls; a backend is not
 * reentrant (FastLattice.hpp:293-295 states the same rule for the reference
 * backends). Different backends may be used from different threads.
 */
#ifndef GBL_H
#define GBL_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int gbl_result;
#define GBL_OK 0
#define GBL_INVALID_ARGUMENT 1
#define GBL_RUNTIME_ERROR 2
#define GBL_OVERFLOW_ERROR 3
#define GBL_LOGIC_ERROR 4

/* Precision (FastLattice.hpp:32). */
#define GBL_PRECISION_FLOAT 0
#define GBL_PRECISION_DOUBLE 1

#define GBL_MAX_SUPPORT_PLANES 2      /* LatticePhysics.hpp:103 */
#define GBL_MAX_FOOTPRINTS 4          /* LatticePhysics.hpp:104 */
#define GBL_MAX_CANDIDATES_PER_BLOCK 1024 /* LatticePhysics.hpp:105 */
#define GBL_PHASE_COUNT 16            /* FastLattice.hpp:130 */
#define GBL_NO_BOND 0xffffffffu       /* LatticePhysics.hpp:106 */

/* ---- Schedule: mirrors LatticeSchedule (LatticeSchedule.hpp:28-44). ---- */
typedef struct gbl_schedule_view {
    uint32_t node_count;
    uint32_t bond_count;
    uint32_t block_count;
    uint32_t color_count;
    uint32_t boundary_bond_count;
    const uint32_t *node_block_begin;    /* block_count + 1 */
    const uint32_t *bond_order;          /* bond_count: schedule index -> asset bond */
    const uint32_t *bond_schedule_index; /* bond_count: asset bond -> schedule index */
    const uint32_t *bond_block_begin;    /* block_count + 1 */
    const uint32_t *range_begin;         /* block_count * 2 * max(color_count, 1) */
    const uint32_t *range_end;
    const uint8_t *bond_color;           /* bond_count, per schedule index */
} gbl_schedule_view;

/* ---- Canonical state: mirrors LatticeState (FastLattice.hpp:37-55). ----
 * Host double arrays in schedule order, caller-owned. For gbl_upload every
 * pointer is read; for gbl_download only u, u_prev, v, alive, failure_mode,
 * damage, plastic_extension, plastic_strain and prev_* are written (the
 * reference's WorkingLattice::toState, LatticeWorking.hpp:126-142), into
 * caller buffers of the uploaded sizes. */
typedef struct gbl_state_view {
    double origin[3];
    uint32_t node_count;
    uint32_t bond_count;
    uint32_t max_degree;
    const double *x0;          /* 3N */
    double *u;                 /* 3N */
    double *u_prev;            /* 3N */
    double *v;                 /* 3N */
    const double *inv_mass;    /* N */
    const double *mass;        /* N */
    const uint32_t *adj_offsets; /* N + 1 */
    const uint32_t *adj_bonds;
    const uint32_t *nbr_bond;  /* max_degree * N, k-major */
    const uint32_t *nbr_other; /* max_degree * N */
    const double *nbr_rest;    /* 3 * max_degree * N */
    const double *nbr_weight;  /* max_degree * N */
    const uint8_t *nbr_alive;  /* max_degree * N */
    const uint32_t *bond_slot_a; /* B */
    const uint32_t *bond_slot_b; /* B */
    const uint32_t *bond_a;    /* B */
    const uint32_t *bond_b;    /* B */
    const double *rest_edge;   /* 3B */
    const double *rest_length; /* B */
    const double *rest_length_sq_minus; /* B */
    const double *weight;      /* B */
    const double *compliance;  /* B */
    const double *threshold;   /* 6B: ds, de, cs, ce, ss, se */
    uint8_t *alive;            /* B */
    uint8_t *failure_mode;     /* B */
    double *damage;            /* B */
    double *prev_tensile;      /* B */
    double *prev_compressive;  /* B */
    double *prev_shear;        /* B */
    double *plastic_extension; /* B */
    double *plastic_strain;    /* B */
} gbl_state_view;

/* ---- Step settings: mirrors StepSettings<double> (LatticePhysics.hpp:114-158, 188-202, 248-284). */
typedef struct gbl_footprint {
    double center_t, center_b, half_t, half_b;
} gbl_footprint;

typedef struct gbl_support_plane {
    double point[3], normal[3], tangent[3], bitangent[3];
    double restitution, static_friction, dynamic_friction;
    double node_radius;
    uint8_t reach_capped;
    uint32_t footprint_count;
    gbl_footprint footprints[GBL_MAX_FOOTPRINTS];
} gbl_support_plane;

typedef struct gbl_contact_settings {
    double static_friction, dynamic_friction, restitution, restitution_speed_threshold;
    double node_contact_radius, contact_margin;
    double prefilter_slack;
} gbl_contact_settings;

typedef struct gbl_node_contact_settings {
    uint8_t mode; /* 0 off, 1 measure (pairs tested, overlap recorded, no response), 2 on */
    double radius, skin, margin, restitution, restitution_speed_threshold, static_friction, dynamic_friction;
    uint32_t bucket_mask;
} gbl_node_contact_settings;

typedef struct gbl_step_settings {
    double dt;
    double gravity[3];
    uint32_t constraint_iterations;
    uint8_t bond_integrator;   /* 0 XPBD; 1 (Verlet reference) is refused */
    double damping_fraction;
    uint8_t sphere_enabled;
    uint8_t direct_arithmetic; /* must be 0 for float, 1 for double */
    uint8_t audit_energy;
    double plastic_yield_stretch;
    double plastic_hardening;
    double plate_half_thickness; /* > 0 (plate bending) is refused */
    gbl_contact_settings contact;
    gbl_node_contact_settings node_contact;
    uint32_t plane_count;
    gbl_support_plane planes[GBL_MAX_SUPPORT_PLANES];
} gbl_step_settings;

/* SphereState<double> (LatticePhysics.hpp:144-148). */
typedef struct gbl_sphere {
    double center[3], velocity[3], angular_velocity[3];
    double radius, mass, inertia;
} gbl_sphere;

/* RunControl (FastLattice.hpp:79-128). `abandon`, when not null, is read
 * between substeps; once it holds a non-zero byte the run stops, exit reason 7. */
typedef struct gbl_run_control {
    uint64_t max_steps;
    uint64_t quiet_steps;
    uint64_t min_steps;
    uint64_t no_failure_steps;
    uint64_t energy_flat_steps;
    double energy_flat_fraction; /* reference default 1e-3 */
    uint64_t calm_steps;
    double calm_damage_margin;   /* reference default 0.5 */
    double removable_energy_j;
    uint64_t capture_stride;
    uint32_t max_frames;
    uint64_t steps_per_launch;
    const volatile uint8_t *abandon;
} gbl_run_control;

/* RunStatus (FastLattice.hpp:182-245), the fields the XPBD lane fills. */
typedef struct gbl_contact_accumulators {
    unsigned long long impulse_contacts;
    double impulse_to_material_x, impulse_to_material_y, impulse_to_material_z;
    double dissipated_kinetic_energy_j;
    double maximum_penetration_m;
    double maximum_position_correction_m;
    double maximum_center_shift_m;
    unsigned long long candidate_overflow;
    unsigned long long ball_support_events;
} gbl_contact_accumulators;

typedef struct gbl_load_ledger {
    uint64_t steps;
    double elapsed_s;
    double requested_impulse_n_s[3], impulse_n_s[3];
    double requested_angular_impulse_kg_m2_s[3], angular_impulse_kg_m2_s[3];
    double work_j;
} gbl_load_ledger;

/* NodeContactAccumulators (LatticePhysics.hpp:204-221). */
typedef struct gbl_node_contact_accumulators {
    unsigned long long contacts, pair_tests, rebuilds, pairs_listed, pair_overflow;
    double dissipated_kinetic_energy_j;
    double maximum_overlap_m;
    double maximum_position_correction_m;
    double momentum_residual_x, momentum_residual_y, momentum_residual_z;
} gbl_node_contact_accumulators;

typedef struct gbl_run_status {
    uint64_t total_steps;
    uint64_t first_failure_step;
    uint64_t last_failure_step;
    uint32_t failure_rounds;
    uint32_t broken_bonds;
    double removed_energy_j;
    uint64_t last_energy_gain_step;
    double max_damage;
    uint64_t last_damage_gain_step;
    gbl_contact_accumulators contact;
    gbl_load_ledger external_load;
    unsigned exit_reason;
    unsigned launches;
    double kernel_seconds;
    double wall_seconds;
    uint32_t frames_captured;
    double phase_seconds[GBL_PHASE_COUNT];
    float max_tensile_stretch, max_compressive_strain, max_shear_strain;
    uint32_t rank_deficient_nodes;
    double plastic_work_j;
    float max_plastic_stretch;
    gbl_node_contact_accumulators node_contact;
    /* StepSettings::audit_energy only: the kinetic energy the damping sweep
     * and the striker passes took out of the lattice, each a difference of
     * the lattice's total kinetic energy across the phase, folded in node
     * order (RunStatus::damping_dissipated_j, striker_dissipated_j,
     * energy_audited; FastLattice.hpp:209-216). */
    double damping_dissipated_j;
    double striker_dissipated_j;
    uint8_t energy_audited;
    /* Not in the reference's RunStatus: the bond projections the sweeps ran
     * since upload, per substep the bonds alive when its sweep starts times
     * the solver iterations -- the throughput measure's numerator. */
    uint64_t bond_projections;
} gbl_run_status;

typedef struct gbl_backend gbl_backend;

/* ---- Device queries: cudaLatticeAvailable / Description / MultiprocessorCount
 * (FastLattice.hpp:403-405). ---- */
int gbl_available(void);
gbl_result gbl_description(char *buffer, size_t capacity);
unsigned gbl_multiprocessor_count(void);
gbl_result gbl_last_error(char *buffer, size_t capacity);

/* makeCudaLatticeBackend(schedule, precision, threads_per_block)
 * (FastLattice.hpp:401-402). The schedule is copied. threads_per_block 0
 * picks the default. Fails with GBL_RUNTIME_ERROR when there is no device. */
gbl_result gbl_create(const gbl_schedule_view *schedule, int precision, unsigned threads_per_block,
                      gbl_backend **out);
void gbl_destroy(gbl_backend *backend);
/* LatticeBackend::name (FastLattice.hpp:266). */
gbl_result gbl_name(const gbl_backend *backend, char *buffer, size_t capacity);
/* LatticeBackend::upload (FastLattice.hpp:267-268). Clears status, loads,
 * frames and the first-failure record, as the reference's upload does. */
gbl_result gbl_upload(gbl_backend *backend, const gbl_state_view *state, const gbl_step_settings *settings,
                      const gbl_sphere *sphere);
/* LatticeBackend::setExternalForces (FastLattice.hpp:274-277, the CPU rules of
 * ExternalLoads.hpp:28-50): forces_world_n holds 3 * count doubles in schedule
 * node order; count 0 with substeps 0 cancels. */
gbl_result gbl_set_external_forces(gbl_backend *backend, const double *forces_world_n, uint64_t count,
                                   uint64_t substeps);
/* ExternalWrench (FastLattice.hpp:153-157): a named node region driven by a
 * force and a torque about a world point. */
typedef struct gbl_external_wrench {
    const char *source;      /* NUL-terminated, nonempty, distinct per call */
    const uint32_t *nodes;   /* node_count schedule node indices, any order */
    uint64_t node_count;
    double point_world_m[3], force_n[3], torque_n_m[3];
} gbl_external_wrench;
/* LatticeBackend::setExternalWrenches (FastLattice.hpp:278-288, the CPU rules
 * of ExternalLoads.hpp:52-77 and 171-238): replaces any external load; each
 * wrench is spread over its nodes by mass about their mass centre from the
 * current geometry at every kick, for `substeps` substeps. count 0 with
 * substeps 0 cancels. An invalid set leaves the previous load in place
 * (GBL_INVALID_ARGUMENT). A run whose geometry a wrench can no longer carry
 * stops before that kick with GBL_INVALID_ARGUMENT, as the reference throws. */
gbl_result gbl_set_external_wrenches(gbl_backend *backend, const gbl_external_wrench *wrenches, uint64_t count,
                                     uint64_t substeps);
/* RunStatus::external_sources (FastLattice.hpp:191): the ledger of every
 * wrench source kicked since upload, in the order of their first kick.
 * gbl_external_source_count, then gbl_external_source for each index: the
 * name (its full length in *name_length; at most name_capacity - 1 bytes and
 * a NUL written) and its ledger. */
gbl_result gbl_external_source_count(gbl_backend *backend, uint64_t *count);
gbl_result gbl_external_source(gbl_backend *backend, uint64_t index, char *name, size_t name_capacity,
                               size_t *name_length, gbl_load_ledger *load);
/* LatticeBackend::run (FastLattice.hpp:360); the status accumulates across calls. */
gbl_result gbl_run(gbl_backend *backend, const gbl_run_control *control, gbl_run_status *status_out);
/* LatticeBackend::status (FastLattice.hpp:364). */
gbl_result gbl_status(const gbl_backend *backend, gbl_run_status *status_out);
/* LatticeBackend::download (FastLattice.hpp:361). */
gbl_result gbl_download(gbl_backend *backend, gbl_state_view *state, gbl_sphere *sphere);
/* LatticeBackend::firstFailureBonds (FastLattice.hpp:368): schedule indices
 * removed in the substep of the first failure since upload. `count` receives
 * the full length; at most `capacity` are written. */
gbl_result gbl_first_failure_bonds(const gbl_backend *backend, uint32_t *out, uint64_t capacity, uint64_t *count);
/* LatticeBackend::takeFrames (FastLattice.hpp:363). Frames captured since the
 * last take, oldest first: gbl_frame_count, then gbl_take_frame for each index
 * with caller buffers (u: 3N floats, alive: B bytes, damage: B floats), then
 * gbl_clear_frames. */
gbl_result gbl_frame_count(const gbl_backend *backend, uint64_t *count);
gbl_result gbl_take_frame(const gbl_backend *backend, uint64_t index, uint64_t *step, float *u, uint8_t *alive,
                          float *damage, gbl_sphere *sphere);
gbl_result gbl_clear_frames(gbl_backend *backend);

/* Issue work on this CUDA stream (a cudaStream_t passed as void*; null: the
 * backend's own stream). For callers that time or order the substep against
 * their own work. */
gbl_result gbl_set_stream(gbl_backend *backend, void *cuda_stream);

/* Kernel launches one substep makes (the nodes of the captured substep graph). */
gbl_result gbl_kernels_per_substep(gbl_backend *backend, uint64_t *count);

/* Per-phase device time (milliseconds, 16 phases named as
 * latticePhaseName, FastLattice.cpp:22-27) of `substeps` substeps run outside
 * the captured graph with an event between phases. Advances the state like
 * gbl_run with max_steps = substeps and exit rules off. */
gbl_result gbl_profile_phases(gbl_backend *backend, uint64_t substeps, double *phase_ms);

/* The phase-diff debug mode: one substep run outside the captured graph,
 * with the lattice's state downloaded after every phase whose bit is set in
 * phase_mask (bit p: the phase latticePhaseName(p) names) into states[i] and,
 * when spheres is not null, spheres[i], for the i-th set bit; a phase the
 * substep marks more than once (the sweep's, once per iteration) gives its
 * last. Each view is a caller-owned state of the lattice's counts, as for
 * gbl_download. The substep then completes like one of gbl_run. The device
 * fuses or reorders some phases (support projection inside the sweep, the
 * restart and part of the end sample beside the contact passes), so a
 * snapshot equals the reference's at the same phase only where both have
 * finished the same work: after the kick (nodes), the first contact pass,
 * the sweep with its support projection (phase 7), the velocity update, the
 * damping, the second contact pass (nodes), the end sample and the ledger. */
gbl_result gbl_debug_substep(gbl_backend *backend, uint32_t phase_mask, gbl_state_view *states, gbl_sphere *spheres);

/* ---- The batch: many independent lattices advanced together. ----
 * The reference runs a batch of trials as one backend per trial
 * (runTileImpact, src/fastlattice/TileImpactScene.cpp:777; makeBackend
 * :345-351); these calls replace that loop with one device-resident set of
 * lattices stepped by shared launches, one substep per launch sequence for
 * every lattice at once. Each lattice keeps its own state, control block,
 * ledgers and exit rules: its results are bit for bit those of the same
 * lattice run alone by gbl_run. The lattices share the step settings.
 *
 * Order: gbl_batch_create, gbl_batch_add per lattice (uploads it),
 * gbl_batch_settle (settings; resets every lattice's RunStatus), then any
 * number of gbl_batch_run; loads, status and downloads per lattice index.
 * A lattice that meets an exit rule stops; the others go on. gbl_batch_run
 * returns when every lattice has stopped or after max_steps substeps. */
typedef struct gbl_batch gbl_batch;
gbl_result gbl_batch_create(int precision, gbl_batch **out);
void gbl_batch_destroy(gbl_batch *batch);
/* Uploads one lattice (schedule and state as for gbl_create/gbl_upload);
 * `index` receives its position in the batch. */
gbl_result gbl_batch_add(gbl_batch *batch, const gbl_schedule_view *schedule, const gbl_state_view *state,
                         const gbl_sphere *sphere, uint32_t *index);
gbl_result gbl_batch_settle(gbl_batch *batch, const gbl_step_settings *settings);
gbl_result gbl_batch_set_external_forces(gbl_batch *batch, uint32_t index, const double *forces_world_n,
                                         uint64_t count, uint64_t substeps);
/* External wrenches and their source ledgers on lattice `index` of the batch,
 * as gbl_set_external_wrenches / gbl_external_source_count /
 * gbl_external_source on a backend. */
gbl_result gbl_batch_set_external_wrenches(gbl_batch *batch, uint32_t index, const gbl_external_wrench *wrenches,
                                           uint64_t count, uint64_t substeps);
gbl_result gbl_batch_external_source_count(gbl_batch *batch, uint32_t index, uint64_t *count);
gbl_result gbl_batch_external_source(gbl_batch *batch, uint32_t index, uint64_t source, char *name,
                                     size_t name_capacity, size_t *name_length, gbl_load_ledger *load);
gbl_result gbl_batch_run(gbl_batch *batch, const gbl_run_control *control);
gbl_result gbl_batch_size(const gbl_batch *batch, uint32_t *count);
gbl_result gbl_batch_status(gbl_batch *batch, uint32_t index, gbl_run_status *status_out);
gbl_result gbl_batch_download(gbl_batch *batch, uint32_t index, gbl_state_view *state, gbl_sphere *sphere);
gbl_result gbl_batch_first_failure_bonds(gbl_batch *batch, uint32_t index, uint32_t *out, uint64_t capacity,
                                         uint64_t *count);
/* The batch's launch shapes and the autotuner that picks them. Every shape
 * runs the same sweep levels in the same order, so results never depend on
 * it; only speed does. gbl_batch_tune (after gbl_batch_settle) times the
 * projection sweep of the lattices present under each candidate shape --
 * positions are saved before and restored after, so the lattices' state is
 * unchanged -- and keeps the fastest; gbl_batch_set_tuning applies a known
 * shape without timing (zero fields keep the current value). */
typedef struct gbl_tuning {
    uint32_t sweep_threads;   /* CTA size of the one-CTA sweep of a small lattice: 256, 512 or 1024 */
    uint32_t whole_max_bonds; /* the largest lattice (bonds) swept by one CTA; larger ones are level-launched */
    uint64_t group_bytes;     /* node bytes of a group of level-launched lattices swept together */
    double sweep_ms;          /* the kept shape's sweep, per substep (tune only) */
    double default_ms;        /* the default shape's sweep, per substep (tune only) */
    uint32_t candidates;      /* shapes timed (tune only) */
    uint32_t staged_max_nodes; /* one-CTA sweeps of lattices up to this many nodes stage their positions in
                                  shared memory (float lane; at most 14,336; 0 off in tune's output; in
                                  set_tuning 0 keeps the current value and 0xFFFFFFFF turns staging off) */
} gbl_tuning;
gbl_result gbl_batch_tune(gbl_batch *batch, gbl_tuning *chosen);
gbl_result gbl_batch_set_tuning(gbl_batch *batch, const gbl_tuning *shape);
/* As gbl_profile_phases, over every lattice of the batch. */
gbl_result gbl_batch_profile_phases(gbl_batch *batch, uint64_t substeps, double *phase_ms);
gbl_result gbl_batch_kernels_per_substep(gbl_batch *batch, uint64_t *count);
gbl_result gbl_batch_set_stream(gbl_batch *batch, void *cuda_stream);

/* ---- The server: continuous batching of lattice requests. ----
 * The reference serves no requests (its callers build one backend per trial,
 * TileImpactScene.cpp:345-351); this is the served form of the same step. A
 * request is one lattice and a substep count. Requests queue in arrival order
 * and are admitted while their device footprint (gbl_serve_footprint) fits
 * what is left of the budget; admitted requests advance together, a chunk of
 * substeps per gbl_serve_step, each stopping at its own count, and leave at
 * once, freeing their memory for the next in line (admission is re-checked in
 * the same call). Every request's result is the one it gets alone.
 *
 * gbl_serve_submit prepares the request's device image from the views on the
 * calling thread, outside the server's lock (so submissions from other threads
 * overlap a running gbl_serve_step); the views may be freed when it returns.
 * The result is kept on the device until gbl_serve_take. Times are seconds on
 * the server's steady clock since its creation, -1 before the event. */
typedef struct gbl_server gbl_server;
enum { GBL_REQUEST_QUEUED = 0, GBL_REQUEST_RUNNING = 1, GBL_REQUEST_DONE = 2 };
typedef struct gbl_request_info {
    int32_t phase;
    uint32_t slot;          /* while RUNNING */
    uint64_t substeps;      /* requested */
    uint64_t substeps_done;
    uint64_t device_bytes;  /* charged against the budget while RUNNING */
    double submitted_s;
    double admitted_s;
    double finished_s;
} gbl_request_info;
typedef struct gbl_server_stats {
    uint64_t queued;
    uint64_t running;
    uint64_t done;          /* finished, not yet taken */
    uint64_t bytes_in_use;
    uint64_t budget_bytes;
    uint64_t substeps_run;  /* chunks stepped, in substeps */
    double device_seconds;  /* device time of the steps */
    double clock_s;
    double admit_seconds;   /* host time admitting (device upload of prepared requests) */
    double retire_seconds;  /* host time retiring (finished requests' results written on the device) */
    double run_seconds;     /* host time of the stepping itself (graph rebuilds and launches included) */
} gbl_server_stats;
gbl_result gbl_serve_create(int precision, const gbl_step_settings *settings, uint64_t budget_bytes, gbl_server **out);
void gbl_serve_destroy(gbl_server *server);
gbl_result gbl_serve_submit(gbl_server *server, const gbl_schedule_view *schedule, const gbl_state_view *state,
                            const gbl_sphere *sphere, uint64_t substeps, uint64_t *ticket);
/* As gbl_serve_submit, but the state's arrays are borrowed until the request
 * is admitted (gbl_serve_poll reports RUNNING or DONE, or it is cancelled):
 * the caller keeps them alive and unchanged until then. Only the sweep order
 * is prepared here; at admission the arrays are copied to the device as
 * they are and converted there, so no host image of the request is written. */
gbl_result gbl_serve_submit_borrowed(gbl_server *server, const gbl_schedule_view *schedule,
                                     const gbl_state_view *state, const gbl_sphere *sphere, uint64_t substeps,
                                     uint64_t *ticket);
/* Admits what fits, advances every admitted request by up to `substeps`
 * substeps, retires the finished, admits again. */
gbl_result gbl_serve_step(gbl_server *server, uint64_t substeps, gbl_server_stats *stats);
gbl_result gbl_serve_poll(gbl_server *server, uint64_t ticket, gbl_request_info *info);
/* The finished request's state (arrays gbl_download writes), sphere and
 * RunStatus; the request is then forgotten. As a request finishes, the device
 * writes its result in the state's layout into a buffer of its own (charged
 * against the budget, about 72 bytes per node and 50 per bond, in place of
 * the lattice's footprint); the copies into `state` run here, on the calling
 * thread, and free it (state may be null). */
gbl_result gbl_serve_take(gbl_server *server, uint64_t ticket, gbl_state_view *state, gbl_sphere *sphere,
                          gbl_run_status *status);
gbl_result gbl_serve_cancel(gbl_server *server, uint64_t ticket);
gbl_result gbl_serve_stats(gbl_server *server, gbl_server_stats *stats);
/* Requests submitted from now on with at least `bonds` bonds run in the
 * server's large lane (default 4,194,304): a step advances the large lane one
 * chunk on a helper thread while the small lane advances chunk after chunk
 * beside it, so small requests do not wait on a large lattice's substeps.
 * Results do not depend on the lane. */
gbl_result gbl_serve_set_lane_threshold(gbl_server *server, uint32_t bonds);
/* Device bytes a lattice of these counts is charged on admission. */
gbl_result gbl_serve_footprint(int precision, uint32_t node_count, uint32_t bond_count, uint32_t max_degree,
                               uint32_t block_count, uint64_t *bytes);

/* The bonds that broke between two aliveness snapshots (one byte per bond,
 * schedule order, non-zero = alive), listed in schedule order -- without
 * allocating anything. This entry point has no counterpart in the reference.
 * It is for callers that must not allocate device memory while they run:
 * a real-time frame loop, where cudaMalloc/cudaFree would synchronise the
 * device and stall the frame, or a caller recording its work into a CUDA
 * graph, where allocation calls cannot be captured.
 *
 * All pointers are device pointers owned by the caller: `broken` has room for
 * bond_count indices, `broken_count` receives the count. The work is enqueued
 * on `cuda_stream` (null: the default stream) and the outputs are ready when
 * the stream reaches that point. At most 134,217,728 bonds (larger counts are
 * refused with GBL_INVALID_ARGUMENT): the scratch is a fixed 64 KiB static
 * device array, held by every GPU that loads the library until the process
 * exits. The first call in a context (the device's primary context, again
 * after a device reset) looks up that array's device address; make it before
 * any stream capture. A CUDA error already pending on the calling thread is
 * reported as GBL_RUNTIME_ERROR and left pending, and nothing is launched.
 * Calls share the array: calls whose work overlaps on the GPU race, so order
 * them on one stream. */
gbl_result gbl_broken_between_noalloc(const uint8_t *alive_before, const uint8_t *alive_after, uint64_t bond_count,
                                      uint32_t *broken, uint32_t *broken_count, void *cuda_stream);

/* The bounds-checked build (libgbl_checked.so, compiled with
 * GBL_BOUNDS_CHECK): every index the kernels read out of device data is
 * checked against its array's length before use; a violation is counted, the
 * first one's site, index and length kept, and the access skipped -- nothing
 * traps. report[0] = violations since the last clear, report[1..3] = the
 * first one's site, index and length. *checked is 0 in the normal build,
 * whose report is all zeros. */
gbl_result gbl_bounds_report(uint64_t report[4], int *checked);
gbl_result gbl_bounds_clear(void);

/* sizeof of a struct of this header by its name ("gbl_step_settings", ...),
 * 0 for an unknown name: lets a binding check its own layout. */
size_t gbl_struct_size(const char *name);

/* ---- Host builders, for callers without the reference's C++: ----
 * buildLatticeSchedule (LatticeSchedule.cpp:71-155) and buildLatticeState
 * (FastLattice.cpp:47-169) restated. Outputs live in library-owned objects
 * whose views stay valid until freed. */
typedef struct gbl_schedule gbl_schedule;
gbl_result gbl_build_schedule(uint32_t node_count, uint32_t bond_count, const uint32_t *bond_a, const uint32_t *bond_b,
                              const uint32_t *node_block_begin, uint32_t block_count, gbl_schedule **out);
gbl_result gbl_schedule_view_of(const gbl_schedule *schedule, gbl_schedule_view *view);
void gbl_schedule_free(gbl_schedule *schedule);

typedef struct gbl_state gbl_state;
/* The asset (reference positions, bonds and their rest records) and the
 * matter (node positions, velocities, masses, bond aliveness/damage/mode), in
 * asset order, as ActiveMatter holds them (fracture/ActiveMatter.hpp). */
typedef struct gbl_matter_view {
    uint32_t node_count;
    uint32_t bond_count;
    const double *reference_position; /* 3N world */
    const double *position;           /* 3N world */
    const double *velocity;           /* 3N */
    const double *mass;               /* N */
    const uint32_t *bond_a;           /* B */
    const uint32_t *bond_b;           /* B */
    const double *rest_length;        /* B */
    const double *compliance;         /* B */
    const double *threshold;          /* 6B */
    const uint8_t *alive;             /* B or null (all alive) */
    const double *damage;             /* B or null */
    const uint8_t *failure_mode;      /* B or null */
} gbl_matter_view;
gbl_result gbl_build_state(const gbl_matter_view *matter, const gbl_schedule *schedule, const double origin[3],
                           gbl_state **out);
/* A view whose arrays are owned by the state object (writable, so the same
 * object can receive a download). */
gbl_result gbl_state_view_of(gbl_state *state, gbl_state_view *view);
/* Sets inv_mass of the flagged nodes to 0 (a pinned node keeps its mass). */
gbl_result gbl_state_pin(gbl_state *state, const uint8_t *pinned);
void gbl_state_free(gbl_state *state);

/* A box lattice, the input generator of the reference's box scenes
 * (generateBoxTileLattice, src/matter/BoxLattice.cpp:49-173, and
 * boxLatticeSlabs :175-195), restated for uniform bonds: cell-centre nodes of
 * one mass, node index x + nx*(y + ny*z), bonds (node, neighbour) for every
 * integer offset of the positive half-space in the generator's walk order,
 * rest length spacing*|offset|, one compliance and one threshold record for
 * every bond. Feed its matter view to gbl_build_schedule/gbl_build_state. */
typedef struct gbl_box_spec {
    uint32_t nx, ny, nz;
    uint32_t horizon;       /* offsets within `horizon` cells on each axis (0 means 1) */
    uint32_t max_offset_sq; /* 0: the generator's rule |o| <= horizon; else |o|^2 <= max_offset_sq */
    uint32_t slabs;         /* z-slabs requested */
    double spacing;
    double center[3];
    double node_mass;
    double compliance;
    double threshold[6];    /* ds, de, cs, ce, ss, se */
} gbl_box_spec;
typedef struct gbl_box gbl_box;
gbl_result gbl_build_box(const gbl_box_spec *spec, gbl_box **out);
/* Views into the box (valid until gbl_box_free): its matter, and its
 * block_count + 1 slab node offsets. */
gbl_result gbl_box_view_of(const gbl_box *box, gbl_matter_view *matter, const uint32_t **node_block_begin,
                           uint32_t *block_count);
void gbl_box_free(gbl_box *box);

/* ---- Scene-side: the impact scene's step settings (buildSettings,
 * src/fastlattice/TileImpactScene.cpp:259-336) from the request and the
 * scene's derived quantities, for a caller that has no physics engine to
 * build the rest of the scene with. The contact pairs are the scene's
 * combined materials (ball on tile, tile on tile, tile on ground). */
typedef struct gbl_contact_pair {
    double static_friction, dynamic_friction, restitution;
} gbl_contact_pair;
typedef struct gbl_ledge {
    double center[3], dimensions[3]; /* world frame, m */
} gbl_ledge;
typedef struct gbl_impact_scene {
    double dt;                       /* substep, s */
    double gravity[3];
    uint32_t constraint_iterations;  /* at least one is used */
    double bond_damping;             /* the compiled material's damping rate, 1/s (0: none) */
    uint8_t multi_body;              /* every object is lattice: no rigid striker */
    uint8_t double_precision;
    uint8_t audit_energy;
    gbl_contact_pair ball_tile, tile_tile, tile_ground;
    double cell_size;                /* m */
    double node_contact_radius_factor, node_contact_skin_factor; /* times the cell size */
    uint8_t node_contact_mode;       /* 0 off, 1 measure, 2 on */
    double ball_radius;
    double yield_stretch, plastic_hardening_ratio; /* the compiled material's */
    uint8_t bridge;                  /* 0: ground only; 1: a ledge plane over the ground */
    double ground_y, support_y;      /* world heights of the ground and of the ledge tops */
    uint32_t ledge_count;            /* at most GBL_MAX_FOOTPRINTS */
    gbl_ledge ledges[GBL_MAX_FOOTPRINTS];
    double origin[3];                /* the lattice's origin (LatticeState::origin) */
    uint32_t node_count;             /* sizes the node-contact hash table */
} gbl_impact_scene;
gbl_result gbl_impact_settings(const gbl_impact_scene *scene, gbl_step_settings *out);

#ifdef __cplusplus
}
#endif

#endif /* GBL_H */
