// The GB300 lattice backend: device state, the captured substep graph, and the
// C ABI of include/gbl.h that mirrors LatticeBackend (FastLattice.hpp:255-405).
#include "gbl_internal.hpp"
#include "gbl_kernels.cuh"

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <type_traits>
#include <vector>

namespace gbl {

namespace {

void check(cudaError_t e, const char *what) {
    if (e != cudaSuccess) runtime(std::string(what) + ": " + cudaGetErrorString(e));
}

// One device allocation per upload, carved into aligned arrays.
class Arena {
public:
    ~Arena() { release(); }
    void release() {
        if (base_) cudaFree(base_);
        base_ = nullptr;
        bytes_ = 0;
    }
    template <class T> void reserve(T *&p, std::size_t count) {
        offsets_.push_back({reinterpret_cast<void **>(&p), bytes_});
        bytes_ += (count * sizeof(T) + 255) & ~static_cast<std::size_t>(255);
    }
    void commit() {
        check(cudaMalloc(&base_, bytes_ ? bytes_ : 256), "device allocation");
        for (auto &o : offsets_) *o.first = static_cast<char *>(base_) + o.second;
        offsets_.clear();
    }

private:
    void *base_{};
    std::size_t bytes_{};
    std::vector<std::pair<void **, std::size_t>> offsets_;
};

} // namespace

class BackendBase {
public:
    virtual ~BackendBase() = default;
    virtual std::string name() const = 0;
    virtual void upload(const gbl_state_view &, const gbl_step_settings &, const gbl_sphere &) = 0;
    virtual void setExternalForces(const double *forces, std::uint64_t count, std::uint64_t substeps) = 0;
    virtual void run(const gbl_run_control &) = 0;
    virtual void download(gbl_state_view &, gbl_sphere *) = 0;
    virtual void profile(std::uint64_t substeps, double *phase_ms) = 0;
    virtual void setStream(cudaStream_t s) = 0;
    virtual std::uint64_t kernelsPerSubstep() = 0;
    gbl_run_status status{};
    std::vector<std::uint32_t> first_failure;
    struct Frame {
        std::uint64_t step;
        std::vector<float> u, damage;
        std::vector<std::uint8_t> alive;
        gbl_sphere sphere;
    };
    std::vector<Frame> frames;
};

template <class R> class Backend final : public BackendBase {
    static constexpr bool kDirect = std::is_same<R, double>::value;
    // One slab's candidates, staged for the serial contact pass.
    static constexpr unsigned kSphereSmem = kCandidatesPerBlock * sizeof(Staged<R>);

public:
    Backend(Schedule s, unsigned threads_per_block) : sched_(std::move(s)), tpb_(threads_per_block) {
        check(cudaFuncSetAttribute(kSpherePass<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSphereSmem),
              "contact pass shared memory");
        check(cudaStreamCreateWithFlags(&own_stream_, cudaStreamNonBlocking), "stream");
        stream_ = own_stream_;
        check(cudaEventCreate(&ev0_), "event");
        check(cudaEventCreate(&ev1_), "event");
    }
    ~Backend() override {
        dropGraph();
        if (ctl_host_) cudaFreeHost(ctl_host_);
        if (ext_force_) cudaFree(ext_force_);
        if (ext_req_) cudaFree(ext_req_);
        if (ext_contrib_) cudaFree(ext_contrib_);
        if (ext_nodes_) cudaFree(ext_nodes_);
        cudaEventDestroy(ev0_);
        cudaEventDestroy(ev1_);
        cudaStreamDestroy(own_stream_);
    }

    std::string name() const override { return kDirect ? "gb300-double" : "gb300-float"; }

    std::uint64_t kernelsPerSubstep() override {
        if (!uploaded_) invalid("the substep graph needs an uploaded lattice");
        ensureGraph();
        std::size_t n = 0;
        check(cudaGraphGetNodes(graph_, nullptr, &n), "graph nodes");
        return n;
    }

    void setStream(cudaStream_t s) override {
        stream_ = s ? s : own_stream_;
        dropGraph();
    }

    // ---- upload (FastLattice.hpp:267-268; WorkingLattice::fromState, LatticeWorking.hpp:53-124)
    void upload(const gbl_state_view &st, const gbl_step_settings &set, const gbl_sphere &sphere) override {
        validate(st, set);
        const std::uint32_t N = st.node_count, B = st.bond_count, D = st.max_degree;
        dropGraph();
        arena_.release();
        buildLevels(st);
        Dev<R> d{};
        d.N = N; d.B = B; d.D = D; d.blocks = sched_.block_count;
        d.words_b = (B + 31) / 32;
        d.tiles_b = (B + kThreads - 1) / kThreads;
        const std::size_t P = static_cast<std::size_t>(D) * N;
        arena_.reserve(d.u, N); arena_.reserve(d.v, N); arena_.reserve(d.x0, N); arena_.reserve(d.up, N);
        arena_.reserve(d.strain, 2 * static_cast<std::size_t>(N));
        arena_.reserve(d.rinv, 9 * static_cast<std::size_t>(N)); arena_.reserve(d.unm, 3 * static_cast<std::size_t>(N));
        arena_.reserve(d.approach, kPlanes * static_cast<std::size_t>(N));
        arena_.reserve(d.dirty, N); arena_.reserve(d.engaged, kPlanes * static_cast<std::size_t>(N));
        arena_.reserve(d.candidate, N); arena_.reserve(d.cand_bits, (N + 31) / 32 + 1);
        arena_.reserve(d.nbr, P); arena_.reserve(d.nbr_other, P); arena_.reserve(d.nbr_bond, P);
        arena_.reserve(d.slot_a, B); arena_.reserve(d.slot_b, B);
        arena_.reserve(d.rec, B); arena_.reserve(d.geo, B); arena_.reserve(d.prev, B); arena_.reserve(d.thr4, B);
        arena_.reserve(d.thr2, B); arena_.reserve(d.plastic, B); arena_.reserve(d.lambda, B); arena_.reserve(d.mode, B);
        arena_.reserve(d.ev_bits, d.words_b + 1); arena_.reserve(d.ev_tile, d.tiles_b + 1); arena_.reserve(d.ev_list, B + 1);
        arena_.reserve(d.ev_removed, B); arena_.reserve(d.ev_packed, B + 1); arena_.reserve(d.ev_prefix, B + 1);
        arena_.reserve(d.ev_ends, B); arena_.reserve(d.dev2sched, B);
        arena_.reserve(d.isolated, isolated_.size() + 1);
        arena_.reserve(d.dmg_bits, d.words_b + 1); arena_.reserve(d.dmg_tile, d.tiles_b + 1);
        arena_.reserve(d.dmg_list, B + 1); arena_.reserve(d.ev_damage, B); arena_.reserve(d.dmg_value, B + 1);
        arena_.reserve(d.tile_plastic, d.tiles_b + 1); arena_.reserve(d.tile_removed, d.tiles_b + 1);
        const std::size_t scan_blocks = d.tiles_b / kScanBlock + 1;
        arena_.reserve(d.blk_ev, scan_blocks); arena_.reserve(d.blk_dmg, scan_blocks);
        arena_.reserve(d.blk_removed, scan_blocks); arena_.reserve(d.blk_plastic, scan_blocks);
        arena_.reserve(d.node_block_begin, sched_.block_count + 1);
        arena_.reserve(d.cand_list, static_cast<std::size_t>(sched_.block_count) * kCandidatesPerBlock);
        arena_.reserve(d.cand_count, sched_.block_count);
        arena_.reserve(d.dirty_list, N + 1); arena_.reserve(d.ffb, B + 1);
        arena_.reserve(d.sphere, 1); arena_.reserve(d.ctl, 1);
        arena_.commit();

        // Nodes.
        std::vector<Q4<R>> u(N), v(N), x0(N);
        for (std::uint32_t i = 0; i < N; ++i) {
            u[i] = {R(st.u[3 * i]), R(st.u[3 * i + 1]), R(st.u[3 * i + 2]), R(st.inv_mass[i])};
            v[i] = {R(st.v[3 * i]), R(st.v[3 * i + 1]), R(st.v[3 * i + 2]), R(st.mass[i])};
            x0[i] = {R(st.x0[3 * i]), R(st.x0[3 * i + 1]), R(st.x0[3 * i + 2]), R(0)};
        }
        std::vector<Q4<R>> up(N);
        for (std::uint32_t i = 0; i < N; ++i)
            up[i] = {R(st.u_prev[3 * i]), R(st.u_prev[3 * i + 1]), R(st.u_prev[3 * i + 2]), R(0)};
        copy(d.u, u); copy(d.v, v); copy(d.x0, x0); copy(d.up, up);
        mass_.resize(N); inv_mass_.resize(N);
        for (std::uint32_t i = 0; i < N; ++i) { mass_[i] = R(st.mass[i]); inv_mass_[i] = R(st.inv_mass[i]); }
        x0_host_ = x0;
        zero(d.strain, 2 * static_cast<std::size_t>(N)); zero(d.rinv, 9 * static_cast<std::size_t>(N));
        zero(d.unm, 3 * static_cast<std::size_t>(N)); zero(d.approach, kPlanes * static_cast<std::size_t>(N));
        zero(d.engaged, kPlanes * static_cast<std::size_t>(N)); zero(d.candidate, N);
        zero(d.cand_bits, (N + 31) / 32 + 1);
        check(cudaMemsetAsync(d.dirty, 1, N, stream_), "memset");
        // Neighbour slots: (rest, weight if alive), the other node (itself when padded).
        {
            std::vector<Q4<R>> nbr(P);
            std::vector<std::uint32_t> other(P), bond(P);
            for (std::size_t s = 0; s < P; ++s) {
                const bool present = st.nbr_bond[s] != kNoBond;
                const std::uint32_t node = static_cast<std::uint32_t>(s % N);
                nbr[s] = {R(st.nbr_rest[3 * s]), R(st.nbr_rest[3 * s + 1]), R(st.nbr_rest[3 * s + 2]),
                          (present && st.nbr_alive[s]) ? R(st.nbr_weight[s]) : R(0)};
                other[s] = present ? st.nbr_other[s] : node;
                bond[s] = present ? sched2dev_[st.nbr_bond[s]] : kNoBond;
            }
            copy(d.nbr, nbr); copy(d.nbr_other, other); copy(d.nbr_bond, bond);
        }
        // Bonds, level-major storage (storage index d holds schedule index j).
        {
            std::vector<BondRec<R>> rec(B);
            std::vector<Q4<R>> geo(B), prev(B), thr4(B);
            std::vector<Q2<R>> thr2(B), plastic(B);
            std::vector<std::uint32_t> slot_a(B), slot_b(B);
            std::vector<std::uint8_t> mode(B);
            plastic_state_ = false;
            for (std::uint32_t dd = 0; dd < B; ++dd) {
                const std::uint32_t j = dev2sched_[dd];
                rec[dd] = {st.bond_a[j] | (st.alive[j] ? 0U : kDeadBit) | (last_a_[dd] ? kLastABit : 0U),
                           st.bond_b[j] | (last_b_[dd] ? kLastBBit : 0U), R(st.rest_length_sq_minus[j]),
                           R(st.rest_length[j])};
                geo[dd] = {R(st.rest_edge[3 * j]), R(st.rest_edge[3 * j + 1]), R(st.rest_edge[3 * j + 2]),
                           R(st.compliance[j])};
                prev[dd] = {R(st.prev_tensile[j]), R(st.prev_compressive[j]), R(st.prev_shear[j]), R(st.damage[j])};
                const double *t = st.threshold + 6 * static_cast<std::size_t>(j);
                thr4[dd] = {R(t[0]), R(t[1]), R(t[2]), R(t[3])};
                thr2[dd] = {R(t[4]), R(t[5])};
                plastic[dd] = {R(st.plastic_extension[j]), R(st.plastic_strain[j])};
                plastic_state_ = plastic_state_ || plastic[dd].x != R(0);
                slot_a[dd] = st.bond_slot_a[j];
                slot_b[dd] = st.bond_slot_b[j];
                mode[dd] = st.failure_mode[j];
            }
            copy(d.rec, rec); copy(d.geo, geo); copy(d.prev, prev); copy(d.thr4, thr4); copy(d.thr2, thr2);
            copy(d.plastic, plastic); copy(d.slot_a, slot_a); copy(d.slot_b, slot_b); copy(d.mode, mode);
            copy(d.dev2sched, dev2sched_);
            if (!isolated_.empty()) copy(d.isolated, isolated_);
            d.isolated_count = static_cast<std::uint32_t>(isolated_.size());
        }
        zero(d.lambda, B);
        zero(d.ev_bits, d.words_b + 1);
        zero(d.dmg_bits, d.words_b + 1);
        zero(d.tile_plastic, d.tiles_b + 1);
        zero(d.tile_removed, d.tiles_b + 1);
        copy(d.node_block_begin, sched_.node_block_begin);
        zero(d.cand_count, sched_.block_count);
        // Settings and sphere.
        S_ = convertSettings(set);
        plastic_ = plastic_state_ || S_.yield_stretch > R(0);
        Sphere<R> sp{};
        sp.center = {R(sphere.center[0]), R(sphere.center[1]), R(sphere.center[2])};
        sp.velocity = {R(sphere.velocity[0]), R(sphere.velocity[1]), R(sphere.velocity[2])};
        sp.angular = {R(sphere.angular_velocity[0]), R(sphere.angular_velocity[1]), R(sphere.angular_velocity[2])};
        sp.radius = R(sphere.radius); sp.mass = R(sphere.mass); sp.inertia = R(sphere.inertia);
        copyRaw(d.sphere, &sp, 1);
        std::memcpy(d.origin, st.origin, sizeof(d.origin));
        if (!ctl_host_) check(cudaMallocHost(&ctl_host_, sizeof(Ctl)), "pinned allocation");
        std::memset(ctl_host_, 0, sizeof(Ctl));
        ctl_host_->first_failure_step = ctl_host_->last_failure_step = ctl_host_->last_energy_gain_step = ~0ULL;
        ctl_host_->full_restart = 1;
        ctl_host_->energy_flat_fraction = 1.0e-3;
        ctl_host_->calm_damage_margin = 0.5;
        check(cudaMemcpyAsync(d.ctl, ctl_host_, sizeof(Ctl), cudaMemcpyHostToDevice, stream_), "copy");
        // Loads do not survive an upload (ExternalLoads.hpp:26 reset): the
        // control block starts with no loaded nodes.
        d.ext_force = ext_force_; d.ext_req = ext_req_; d.ext_contrib = ext_contrib_; d.ext_nodes = ext_nodes_;
        dev_ = d;
        N_ = N; B_ = B;
        status = gbl_run_status{};
        status.first_failure_step = status.last_failure_step = status.last_energy_gain_step = ~0ULL;
        first_failure.clear();
        frames.clear();
        check(cudaStreamSynchronize(stream_), "upload");
        uploaded_ = true;
    }

    // ---- setExternalForces (ExternalLoads.hpp:28-50)
    void setExternalForces(const double *forces, std::uint64_t count, std::uint64_t substeps) override {
        if (!uploaded_) invalid("external load needs an uploaded lattice");
        if (count == 0) {
            if (substeps != 0) invalid("empty external load needs zero substeps");
            setLoads(0, 0);
            return;
        }
        if (count != N_ || substeps == 0 || !forces)
            invalid("external load needs one force per node and a finite nonzero span");
        std::vector<Q4<R>> applied(N_, Q4<R>{R(0), R(0), R(0), R(0)});
        std::vector<std::uint32_t> nodes;
        for (std::uint32_t i = 0; i < N_; ++i) {
            const double fx = forces[3 * i], fy = forces[3 * i + 1], fz = forces[3 * i + 2];
            const R cx = R(fx), cy = R(fy), cz = R(fz);
            if (!std::isfinite(fx) || !std::isfinite(fy) || !std::isfinite(fz) || !std::isfinite(std::hypot(fx, fy, fz)) ||
                !std::isfinite(cx) || !std::isfinite(cy) || !std::isfinite(cz))
                invalid("external force is not finite in backend precision");
            if (fx == 0 && fy == 0 && fz == 0) continue;
            if (!(mass_[i] > 0) || !(inv_mass_[i] > 0) || !std::isfinite(mass_[i]) || !std::isfinite(inv_mass_[i]))
                invalid("external force needs a finite positive movable node mass");
            applied[i] = {cx, cy, cz, R(1)};
            nodes.push_back(i);
        }
        if (ext_capacity_n_ < N_) {
            if (ext_force_) cudaFree(ext_force_);
            if (ext_req_) cudaFree(ext_req_);
            if (ext_contrib_) cudaFree(ext_contrib_);
            if (ext_nodes_) cudaFree(ext_nodes_);
            check(cudaMalloc(&ext_force_, sizeof(Q4<R>) * N_), "device allocation");
            check(cudaMalloc(&ext_req_, sizeof(double) * 3 * N_), "device allocation");
            check(cudaMalloc(&ext_contrib_, sizeof(double) * 13 * N_), "device allocation");
            check(cudaMalloc(&ext_nodes_, sizeof(std::uint32_t) * N_), "device allocation");
            ext_capacity_n_ = N_;
        }
        copy(ext_force_, applied);
        copyRaw(ext_req_, forces, 3 * static_cast<std::size_t>(N_));
        if (!nodes.empty()) copy(ext_nodes_, nodes);
        if (dev_.ext_force != ext_force_) {
            dev_.ext_force = ext_force_; dev_.ext_req = ext_req_; dev_.ext_contrib = ext_contrib_; dev_.ext_nodes = ext_nodes_;
            dropGraph();
        }
        setLoads(static_cast<std::uint32_t>(nodes.size()), nodes.empty() ? 0 : substeps);
    }

    // ---- run (CpuLatticeBackend.cpp:255-304)
    void run(const gbl_run_control &control) override {
        if (!uploaded_) invalid("lattice run needs an uploaded lattice");
        const auto start = std::chrono::steady_clock::now();
        check(cudaMemcpyAsync(ctl_host_, dev_.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, stream_), "copy");
        check(cudaStreamSynchronize(stream_), "status");
        Ctl &c = *ctl_host_;
        c.stop = 0;
        c.exit_reason = 0;
        c.quiet_steps = control.quiet_steps; c.min_steps = control.min_steps; c.no_failure_steps = control.no_failure_steps;
        c.energy_flat_steps = control.energy_flat_steps; c.calm_steps = control.calm_steps;
        c.energy_flat_fraction = control.energy_flat_fraction; c.calm_damage_margin = control.calm_damage_margin;
        c.removable_energy = control.removable_energy_j;
        check(cudaMemcpyAsync(dev_.ctl, ctl_host_, sizeof(Ctl), cudaMemcpyHostToDevice, stream_), "copy");
        const std::uint64_t before = c.total_steps;
        ensureGraph();
        std::uint64_t chunk = control.steps_per_launch ? control.steps_per_launch : control.max_steps;
        if (control.abandon && chunk > 64) chunk = 64;
        const bool capture = control.capture_stride != 0;
        std::uint64_t launched = 0;
        bool abandoned = false;
        check(cudaEventRecord(ev0_, stream_), "event");
        while (launched < control.max_steps) {
            if (control.abandon && *control.abandon) { abandoned = true; break; }
            const std::uint64_t n = std::min(chunk, control.max_steps - launched);
            for (std::uint64_t k = 0; k < n; ++k) {
                if (capture) {
                    const std::uint64_t step = before + launched + k;
                    if (step % control.capture_stride == 0 && status.frames_captured < control.max_frames) {
                        if (stopped()) break;
                        captureFrame(step);
                    }
                }
                check(cudaGraphLaunch(exec_, stream_), "graph launch");
            }
            launched += n;
            ++status.launches;
            if (stopped()) break;
        }
        check(cudaEventRecord(ev1_, stream_), "event");
        check(cudaMemcpyAsync(ctl_host_, dev_.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, stream_), "copy");
        check(cudaStreamSynchronize(stream_), "lattice run");
        float ms = 0;
        cudaEventElapsedTime(&ms, ev0_, ev1_);
        status.kernel_seconds += ms * 1e-3;
        if (c.error & kErrExternalOverflow) {
            c.error = 0;
            check(cudaMemcpyAsync(dev_.ctl, ctl_host_, sizeof(Ctl), cudaMemcpyHostToDevice, stream_), "copy");
            check(cudaStreamSynchronize(stream_), "status");
            overflow("external force kick exceeds backend precision");
        }
        fillStatus();
        const std::uint64_t done = c.total_steps - before;
        if (abandoned && c.exit_reason == 0) status.exit_reason = 7;
        else if (status.exit_reason == 0 && done >= control.max_steps) status.exit_reason = 3;
        if (c.ffb_count > first_failure.size()) {
            first_failure.resize(c.ffb_count);
            check(cudaMemcpy(first_failure.data(), dev_.ffb, sizeof(std::uint32_t) * c.ffb_count, cudaMemcpyDeviceToHost),
                  "copy");
        }
        status.wall_seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - start).count();
    }

    // ---- download (WorkingLattice::toState, LatticeWorking.hpp:126-142)
    void download(gbl_state_view &st, gbl_sphere *sphere) override {
        if (!uploaded_) invalid("lattice download needs an uploaded lattice");
        if (st.node_count != N_ || st.bond_count != B_) invalid("download state does not match the lattice");
        check(cudaStreamSynchronize(stream_), "download");
        const auto u = fetch(dev_.u, N_), up = fetch(dev_.up, N_), v = fetch(dev_.v, N_);
        for (std::uint32_t i = 0; i < N_; ++i) {
            st.u[3 * i] = u[i].x; st.u[3 * i + 1] = u[i].y; st.u[3 * i + 2] = u[i].z;
            st.u_prev[3 * i] = up[i].x; st.u_prev[3 * i + 1] = up[i].y; st.u_prev[3 * i + 2] = up[i].z;
            st.v[3 * i] = v[i].x; st.v[3 * i + 1] = v[i].y; st.v[3 * i + 2] = v[i].z;
        }
        const auto rec = fetch(dev_.rec, B_);
        const auto prev = fetch(dev_.prev, B_);
        const auto pl = fetch(dev_.plastic, B_);
        const auto mode = fetch(dev_.mode, B_);
        for (std::uint32_t dd = 0; dd < B_; ++dd) {
            const std::uint32_t j = dev2sched_[dd];
            st.alive[j] = (rec[dd].a & kDeadBit) ? 0 : 1;
            st.failure_mode[j] = mode[dd];
            st.damage[j] = prev[dd].w;
            st.prev_tensile[j] = prev[dd].x; st.prev_compressive[j] = prev[dd].y; st.prev_shear[j] = prev[dd].z;
            st.plastic_extension[j] = pl[dd].x; st.plastic_strain[j] = pl[dd].y;
        }
        if (sphere) *sphere = fetchSphere();
    }

    // Per-phase device time: the substep enqueued outside the graph, with an
    // event between phases (phase names of FastLattice.cpp:22-27).
    void profile(std::uint64_t substeps, double *phase_ms) override {
        if (!uploaded_) invalid("profiling needs an uploaded lattice");
        for (unsigned p = 0; p < GBL_PHASE_COUNT; ++p) phase_ms[p] = 0.0;
        std::vector<cudaEvent_t> evs;
        std::vector<unsigned> ids;
        auto mark = [&](unsigned phase) {
            cudaEvent_t e;
            check(cudaEventCreate(&e), "event");
            check(cudaEventRecord(e, stream_), "event");
            evs.push_back(e);
            ids.push_back(phase);
        };
        check(cudaMemcpyAsync(ctl_host_, dev_.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, stream_), "copy");
        check(cudaStreamSynchronize(stream_), "status");
        ctl_host_->stop = 0;
        ctl_host_->exit_reason = 0;
        ctl_host_->quiet_steps = ctl_host_->min_steps = ctl_host_->no_failure_steps = 0;
        ctl_host_->energy_flat_steps = ctl_host_->calm_steps = 0;
        ctl_host_->removable_energy = 0;
        check(cudaMemcpyAsync(dev_.ctl, ctl_host_, sizeof(Ctl), cudaMemcpyHostToDevice, stream_), "copy");
        for (std::uint64_t s = 0; s < substeps; ++s) {
            mark(0);
            enqueueSubstep(mark);
        }
        check(cudaStreamSynchronize(stream_), "profile");
        for (std::size_t k = 0; k + 1 < evs.size(); ++k) {
            float ms = 0;
            cudaEventElapsedTime(&ms, evs[k], evs[k + 1]);
            phase_ms[ids[k + 1]] += ms;
        }
        for (auto e : evs) cudaEventDestroy(e);
        check(cudaMemcpyAsync(ctl_host_, dev_.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, stream_), "copy");
        check(cudaStreamSynchronize(stream_), "status");
        fillStatus();
        for (unsigned p = 0; p < GBL_PHASE_COUNT; ++p) status.phase_seconds[p] += phase_ms[p] * 1e-3;
    }

private:
    // Levels of the projection sweep. The reference sweeps bonds in one serial
    // order: every slab's interior colours, then the boundary colours of even
    // slabs, then of odd slabs (CpuLatticeBackend.cpp:336-348, 395-407). A
    // bond's depth is one more than the deepest earlier bond at either of its
    // nodes; bonds of equal depth share no node, and along every node the
    // depths rise in the serial order, so running the levels in depth order,
    // each level in any thread order, is the serial sweep exactly. Bonds are
    // stored level-major (stable in the serial order), and each node's last
    // bond of the sweep is flagged: its support projection follows that bond.
    struct Level { std::uint32_t begin, end; };

    void buildLevels(const gbl_state_view &st) {
        const std::uint32_t N = st.node_count, B = st.bond_count, C = sched_.color_count;
        std::vector<std::uint32_t> order;
        order.reserve(B);
        auto sweep = [&](std::uint32_t blk, std::uint32_t boundary) {
            for (std::uint32_t c = 0; c < C; ++c) {
                const std::size_t key = sched_.rangeKey(blk, boundary, c);
                for (std::uint32_t j = sched_.range_begin[key]; j < sched_.range_end[key]; ++j) order.push_back(j);
            }
        };
        for (std::uint32_t blk = 0; blk < sched_.block_count; ++blk) sweep(blk, 0);
        for (std::uint32_t blk = 0; blk < sched_.block_count; blk += 2) sweep(blk, 1);
        for (std::uint32_t blk = 1; blk < sched_.block_count; blk += 2) sweep(blk, 1);
        if (order.size() != B) invalid("lattice schedule ranges do not cover every bond exactly once");
        std::vector<std::uint32_t> depth(B), reached(N, 0), last(N, kNoBond);
        std::uint32_t deepest = 0;
        for (const std::uint32_t j : order) {
            const std::uint32_t a = st.bond_a[j], b = st.bond_b[j];
            if (a >= N || b >= N || a == b) invalid("lattice bond joins invalid nodes");
            const std::uint32_t d = std::max(reached[a], reached[b]) + 1;
            depth[j] = d;
            reached[a] = reached[b] = d;
            last[a] = last[b] = j;
            deepest = std::max(deepest, d);
        }
        std::vector<std::uint32_t> first(deepest + 2, 0);
        for (std::uint32_t j = 0; j < B; ++j) ++first[depth[j] + 1];
        for (std::uint32_t d = 1; d <= deepest; ++d) first[d + 1] += first[d];
        dev2sched_.assign(B, 0);
        sched2dev_.assign(B, 0);
        {
            std::vector<std::uint32_t> fill(first.begin(), first.end());
            for (const std::uint32_t j : order) dev2sched_[fill[depth[j]]++] = j;
        }
        for (std::uint32_t d = 0; d < B; ++d) sched2dev_[dev2sched_[d]] = d;
        levels_.clear();
        for (std::uint32_t d = 1; d <= deepest; ++d)
            if (first[d + 1] > first[d]) levels_.push_back({first[d], first[d + 1]});
        last_a_.assign(B, 0);
        last_b_.assign(B, 0);
        isolated_.clear();
        for (std::uint32_t i = 0; i < N; ++i) {
            if (last[i] == kNoBond) {
                isolated_.push_back(i);
                continue;
            }
            const std::uint32_t dd = sched2dev_[last[i]];
            (st.bond_a[last[i]] == i ? last_a_ : last_b_)[dd] = 1;
        }
    }

    static void validate(const gbl_state_view &st, const gbl_step_settings &s) {
        if (s.bond_integrator != 0) invalid("this lattice backend implements the XPBD integrator only");
        if (s.node_contact.mode != 0) invalid("this lattice backend does not implement node-to-node contact");
        if (s.plate_half_thickness > 0.0) invalid("this lattice backend does not implement plate bending");
        if (s.audit_energy) invalid("this lattice backend does not implement the energy audit");
        if ((s.direct_arithmetic != 0) != kDirect)
            invalid(kDirect ? "the double backend runs the direct (absolute position) arithmetic"
                            : "the float backend runs the displacement arithmetic");
        if (s.plane_count > kPlanes) invalid("at most two support planes");
        for (std::uint32_t p = 0; p < s.plane_count; ++p)
            if (s.planes[p].footprint_count > kFootprints) invalid("at most four footprints per plane");
        if (!(s.dt > 0.0) || !std::isfinite(s.dt)) invalid("lattice step needs a finite positive timestep");
        if (st.node_count > kNodeMask) invalid("lattice exceeds 2^30 nodes");
    }

    Settings<R> convertSettings(const gbl_step_settings &s) const {
        Settings<R> o{};
        o.dt = R(s.dt);
        o.gravity = {R(s.gravity[0]), R(s.gravity[1]), R(s.gravity[2])};
        o.iterations = s.constraint_iterations;
        o.damping_fraction = R(s.damping_fraction);
        o.sphere_enabled = s.sphere_enabled;
        o.yield_stretch = R(s.plastic_yield_stretch);
        o.hardening = R(s.plastic_hardening);
        o.c_static = R(s.contact.static_friction); o.c_dynamic = R(s.contact.dynamic_friction);
        o.c_restitution = R(s.contact.restitution); o.c_threshold = R(s.contact.restitution_speed_threshold);
        o.c_node_radius = R(s.contact.node_contact_radius); o.c_margin = R(s.contact.contact_margin);
        o.c_slack = R(s.contact.prefilter_slack);
        o.plane_count = s.plane_count;
        for (unsigned p = 0; p < kPlanes; ++p) {
            const gbl_support_plane &in = s.planes[p];
            Plane<R> &pl = o.planes[p];
            pl.point = {R(in.point[0]), R(in.point[1]), R(in.point[2])};
            pl.normal = {R(in.normal[0]), R(in.normal[1]), R(in.normal[2])};
            pl.tangent = {R(in.tangent[0]), R(in.tangent[1]), R(in.tangent[2])};
            pl.bitangent = {R(in.bitangent[0]), R(in.bitangent[1]), R(in.bitangent[2])};
            pl.restitution = R(in.restitution); pl.static_friction = R(in.static_friction);
            pl.dynamic_friction = R(in.dynamic_friction); pl.node_radius = R(in.node_radius);
            pl.reach_capped = in.reach_capped; pl.footprint_count = in.footprint_count;
            for (unsigned f = 0; f < kFootprints; ++f) {
                pl.fp[f][0] = R(in.footprints[f].center_t); pl.fp[f][1] = R(in.footprints[f].center_b);
                pl.fp[f][2] = R(in.footprints[f].half_t); pl.fp[f][3] = R(in.footprints[f].half_b);
            }
        }
        return o;
    }

    template <class T> void copy(T *dst, const std::vector<T> &src) {
        if (!src.empty()) check(cudaMemcpyAsync(dst, src.data(), sizeof(T) * src.size(), cudaMemcpyHostToDevice, stream_), "copy");
        check(cudaStreamSynchronize(stream_), "copy");
    }
    template <class T> void copyRaw(T *dst, const T *src, std::size_t n) {
        if (n) check(cudaMemcpyAsync(dst, src, sizeof(T) * n, cudaMemcpyHostToDevice, stream_), "copy");
        check(cudaStreamSynchronize(stream_), "copy");
    }
    template <class T> void zero(T *dst, std::size_t n) {
        if (n) check(cudaMemsetAsync(dst, 0, sizeof(T) * n, stream_), "memset");
    }
    template <class T> std::vector<T> fetch(const T *src, std::size_t n) {
        std::vector<T> out(n);
        if (n) check(cudaMemcpy(out.data(), src, sizeof(T) * n, cudaMemcpyDeviceToHost), "copy");
        return out;
    }
    gbl_sphere fetchSphere() {
        Sphere<R> sp{};
        check(cudaMemcpy(&sp, dev_.sphere, sizeof(sp), cudaMemcpyDeviceToHost), "copy");
        gbl_sphere o{};
        o.center[0] = sp.center.x; o.center[1] = sp.center.y; o.center[2] = sp.center.z;
        o.velocity[0] = sp.velocity.x; o.velocity[1] = sp.velocity.y; o.velocity[2] = sp.velocity.z;
        o.angular_velocity[0] = sp.angular.x; o.angular_velocity[1] = sp.angular.y; o.angular_velocity[2] = sp.angular.z;
        o.radius = sp.radius; o.mass = sp.mass; o.inertia = sp.inertia;
        return o;
    }

    void setLoads(std::uint32_t count, std::uint64_t remaining) {
        check(cudaMemcpyAsync(&dev_.ctl->ext_count, &count, sizeof(count), cudaMemcpyHostToDevice, stream_), "copy");
        check(cudaMemcpyAsync(&dev_.ctl->loads_remaining, &remaining, sizeof(remaining), cudaMemcpyHostToDevice, stream_),
              "copy");
        check(cudaStreamSynchronize(stream_), "copy");
    }

    bool stopped() {
        unsigned stop = 0;
        check(cudaMemcpyAsync(&ctl_host_->stop, &dev_.ctl->stop, sizeof(unsigned), cudaMemcpyDeviceToHost, stream_), "copy");
        check(cudaStreamSynchronize(stream_), "status");
        stop = ctl_host_->stop;
        return stop != 0;
    }

    void captureFrame(std::uint64_t step) {
        check(cudaStreamSynchronize(stream_), "capture");
        Frame f;
        f.step = step;
        const auto u = fetch(dev_.u, N_);
        f.u.resize(3 * static_cast<std::size_t>(N_));
        for (std::uint32_t i = 0; i < N_; ++i) {
            f.u[3 * i] = static_cast<float>(u[i].x); f.u[3 * i + 1] = static_cast<float>(u[i].y);
            f.u[3 * i + 2] = static_cast<float>(u[i].z);
        }
        const auto rec = fetch(dev_.rec, B_);
        const auto prev = fetch(dev_.prev, B_);
        f.alive.resize(B_);
        f.damage.resize(B_);
        for (std::uint32_t dd = 0; dd < B_; ++dd) {
            const std::uint32_t j = dev2sched_[dd];
            f.alive[j] = (rec[dd].a & kDeadBit) ? 0 : 1;
            f.damage[j] = static_cast<float>(prev[dd].w);
        }
        f.sphere = fetchSphere();
        frames.push_back(std::move(f));
        ++status.frames_captured;
    }

    void fillStatus() {
        const Ctl &c = *ctl_host_;
        status.total_steps = c.total_steps;
        status.first_failure_step = c.first_failure_step;
        status.last_failure_step = c.last_failure_step;
        status.failure_rounds = c.failure_rounds;
        status.broken_bonds = c.broken_bonds;
        status.removed_energy_j = c.removed_energy;
        status.last_energy_gain_step = c.last_energy_gain_step;
        status.max_damage = c.max_damage;
        status.last_damage_gain_step = c.last_damage_gain_step;
        status.contact.impulse_contacts = c.contact.impulse_contacts;
        status.contact.impulse_to_material_x = c.contact.impulse_x;
        status.contact.impulse_to_material_y = c.contact.impulse_y;
        status.contact.impulse_to_material_z = c.contact.impulse_z;
        status.contact.dissipated_kinetic_energy_j = c.contact.dissipated;
        status.contact.maximum_penetration_m = c.contact.max_penetration;
        status.contact.maximum_position_correction_m = c.contact.max_correction;
        status.contact.maximum_center_shift_m = c.contact.max_center_shift;
        status.contact.candidate_overflow = c.contact.candidate_overflow;
        status.contact.ball_support_events = c.contact.ball_support_events;
        status.external_load.steps = c.ext.steps;
        status.external_load.elapsed_s = c.ext.elapsed;
        for (int q = 0; q < 3; ++q) {
            status.external_load.requested_impulse_n_s[q] = c.ext.req_imp[q];
            status.external_load.impulse_n_s[q] = c.ext.imp[q];
            status.external_load.requested_angular_impulse_kg_m2_s[q] = c.ext.req_ang[q];
            status.external_load.angular_impulse_kg_m2_s[q] = c.ext.ang[q];
        }
        status.external_load.work_j = c.ext.work;
        status.exit_reason = c.exit_reason;
        float f;
        std::memcpy(&f, &c.max_t, 4); status.max_tensile_stretch = f;
        std::memcpy(&f, &c.max_c, 4); status.max_compressive_strain = f;
        std::memcpy(&f, &c.max_s, 4); status.max_shear_strain = f;
        std::memcpy(&f, &c.max_plastic, 4); status.max_plastic_stretch = f;
        status.rank_deficient_nodes = c.rank_deficient;
        status.plastic_work_j = c.plastic_work;
    }

    void dropGraph() {
        if (exec_) cudaGraphExecDestroy(exec_);
        if (graph_) cudaGraphDestroy(graph_);
        exec_ = nullptr;
        graph_ = nullptr;
    }

    void ensureGraph() {
        if (exec_) return;
        check(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal), "graph capture");
        enqueueSubstep([](unsigned) {});
        check(cudaStreamEndCapture(stream_, &graph_), "graph capture");
        check(cudaGraphInstantiate(&exec_, graph_, 0), "graph instantiate");
    }

    static unsigned gridFor(std::size_t n, unsigned per = kThreads) {
        return static_cast<unsigned>(std::max<std::size_t>(1, (n + per - 1) / per));
    }

    // One substep: the reference's phase order (CpuLatticeBackend.cpp:357-488).
    template <class Mark> void enqueueSubstep(Mark &&mark) {
        const Dev<R> &L = dev_;
        const Settings<R> &S = S_;
        const unsigned nodes = gridFor(N_);
        const unsigned restart_grid = std::min(gridFor(N_), 152U * 16U);
        kRestartStrain<R, kDirect><<<restart_grid, kThreads, 0, stream_>>>(L);
        mark(1);
        kRestartBonds<R, kDirect><<<std::min(gridFor(static_cast<std::size_t>(B_)), 152U * 16U), kThreads, 0, stream_>>>(L);
        mark(2);
        kKick<R><<<nodes, kThreads, 0, stream_>>>(L, S);
        if (S.sphere_enabled) kCandidates<R><<<sched_.block_count, 1024, 0, stream_>>>(L);
        mark(3);
        if (S.sphere_enabled) kSpherePass<R><<<1, kSphereThreads, kSphereSmem, stream_>>>(L, S, 1);
        mark(4);
        const unsigned I = S.iterations;
        for (unsigned it = 0; it < I; ++it) {
            const bool first = it == 0, last = it + 1 == I;
            for (const Level &lv : levels_) launchSolve(lv, first, last);
            mark(5);
            if (S.plane_count && L.isolated_count)
                kSupportIsolated<R><<<gridFor(L.isolated_count), kThreads, 0, stream_>>>(L, S);
            mark(7);
        }
        kVelocity<R><<<nodes, kThreads, 0, stream_>>>(L, S, S.damping_fraction <= R(0) ? 1 : 0);
        mark(8);
        if (S.damping_fraction > R(0)) {
            for (const Level &lv : levels_)
                kDamp<R, kDirect><<<gridFor(lv.end - lv.begin), kThreads, 0, stream_>>>(L, lv.begin, lv.end,
                                                                                        S.damping_fraction);
            kSupportVelocity<R><<<nodes, kThreads, 0, stream_>>>(L, S);
            mark(9);
        }
        if (S.sphere_enabled) kSpherePass<R><<<1, kSphereThreads, kSphereSmem, stream_>>>(L, S, 2);
        mark(10);
        kStrainAll<R, kDirect><<<nodes, kThreads, 0, stream_>>>(L);
        mark(11);
        if (plastic_) kEndSample<R, kDirect, true><<<std::max(1U, dev_.tiles_b), kThreads, 0, stream_>>>(L, S);
        else kEndSample<R, kDirect, false><<<std::max(1U, dev_.tiles_b), kThreads, 0, stream_>>>(L, S);
        const unsigned tile_grid = gridFor(dev_.tiles_b, kThreads / 32);
        const unsigned scan_blocks = gridFor(dev_.tiles_b, kScanBlock);
        kTileCounts<R><<<tile_grid, kThreads, 0, stream_>>>(L);
        kBlockScan<R><<<scan_blocks, kScanBlock, 0, stream_>>>(L, plastic_ ? 1 : 0);
        kTopScan<R><<<1, kScanBlock, 0, stream_>>>(L, scan_blocks);
        kEmitEvents<R><<<tile_grid, kThreads, 0, stream_>>>(L);
        kLedgerBroken<R><<<152U * 4U, kThreads, 0, stream_>>>(L);
        mark(12);
        kLedger<R><<<1, 1, 0, stream_>>>(L, S);
        mark(13);
        check(cudaGetLastError(), "kernel launch");
    }

    void launchSolve(const Level &lv, bool first, bool last) {
        const unsigned grid = gridFor(lv.end - lv.begin);
        const bool support = S_.plane_count != 0;
        // One instantiation per (first, last, plastic, support) combination.
        const int key = (first ? 8 : 0) | (last ? 4 : 0) | (plastic_ ? 2 : 0) | (support ? 1 : 0);
#define GBL_SOLVE(K)                                                                                                \
    case K:                                                                                                         \
        kSolve<R, kDirect, ((K) & 8) != 0, ((K) & 4) != 0, ((K) & 2) != 0, ((K) & 1) != 0>                          \
            <<<grid, kThreads, 0, stream_>>>(dev_, S_, lv.begin, lv.end);                                          \
        break;
        switch (key) {
            GBL_SOLVE(0) GBL_SOLVE(1) GBL_SOLVE(2) GBL_SOLVE(3) GBL_SOLVE(4) GBL_SOLVE(5) GBL_SOLVE(6) GBL_SOLVE(7)
            GBL_SOLVE(8) GBL_SOLVE(9) GBL_SOLVE(10) GBL_SOLVE(11) GBL_SOLVE(12) GBL_SOLVE(13) GBL_SOLVE(14)
            GBL_SOLVE(15)
        }
#undef GBL_SOLVE
    }

    Schedule sched_;
    unsigned tpb_;
    std::vector<Level> levels_;
    std::vector<std::uint32_t> dev2sched_, sched2dev_, isolated_;
    std::vector<std::uint8_t> last_a_, last_b_;
    Arena arena_;
    Dev<R> dev_{};
    Settings<R> S_{};
    std::uint32_t N_{}, B_{};
    bool uploaded_{false}, plastic_{false}, plastic_state_{false};
    std::vector<R> mass_, inv_mass_;
    std::vector<Q4<R>> x0_host_;
    Ctl *ctl_host_{};
    Q4<R> *ext_force_{};
    double *ext_req_{}, *ext_contrib_{};
    std::uint32_t *ext_nodes_{};
    std::uint32_t ext_capacity_n_{};
    cudaStream_t own_stream_{}, stream_{};
    cudaEvent_t ev0_{}, ev1_{};
    cudaGraph_t graph_{};
    cudaGraphExec_t exec_{};
};

} // namespace gbl

struct gbl_backend {
    std::unique_ptr<gbl::BackendBase> impl;
};

extern "C" {

int gbl_available(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n > 0 ? 1 : 0;
}

gbl_result gbl_description(char *buffer, size_t capacity) {
    return gbl::guard([&] {
        if (!buffer || capacity == 0) gbl::invalid("null buffer");
        std::string d;
        int n = 0;
        if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
            cudaGetLastError();
            d = "no CUDA device";
        } else {
            cudaDeviceProp p{};
            gbl::check(cudaGetDeviceProperties(&p, 0), "device properties");
            d = std::string(p.name) + ", sm_" + std::to_string(p.major) + std::to_string(p.minor) + ", " +
                std::to_string(p.multiProcessorCount) + " SMs, " +
                std::to_string(p.totalGlobalMem / (1024 * 1024)) + " MiB";
        }
        std::snprintf(buffer, capacity, "%s", d.c_str());
    });
}

unsigned gbl_multiprocessor_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        return 0;
    }
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
    return static_cast<unsigned>(sms);
}

gbl_result gbl_create(const gbl_schedule_view *schedule, int precision, unsigned threads_per_block, gbl_backend **out) {
    return gbl::guard([&] {
        if (!schedule || !out) gbl::invalid("null argument");
        if (!gbl_available()) gbl::runtime("no CUDA device is available for the lattice backend");
        gbl::Schedule s = gbl::Schedule::fromView(*schedule);
        auto *b = new gbl_backend;
        try {
            if (precision == GBL_PRECISION_DOUBLE)
                b->impl = std::make_unique<gbl::Backend<double>>(std::move(s), threads_per_block);
            else if (precision == GBL_PRECISION_FLOAT)
                b->impl = std::make_unique<gbl::Backend<float>>(std::move(s), threads_per_block);
            else
                gbl::invalid("unknown precision");
        } catch (...) {
            delete b;
            throw;
        }
        *out = b;
    });
}

void gbl_destroy(gbl_backend *backend) { delete backend; }

gbl_result gbl_name(const gbl_backend *backend, char *buffer, size_t capacity) {
    return gbl::guard([&] {
        if (!backend || !buffer || capacity == 0) gbl::invalid("null argument");
        std::snprintf(buffer, capacity, "%s", backend->impl->name().c_str());
    });
}

gbl_result gbl_upload(gbl_backend *backend, const gbl_state_view *state, const gbl_step_settings *settings,
                      const gbl_sphere *sphere) {
    return gbl::guard([&] {
        if (!backend || !state || !settings || !sphere) gbl::invalid("null argument");
        backend->impl->upload(*state, *settings, *sphere);
    });
}

gbl_result gbl_set_external_forces(gbl_backend *backend, const double *forces, uint64_t count, uint64_t substeps) {
    return gbl::guard([&] {
        if (!backend) gbl::invalid("null backend");
        backend->impl->setExternalForces(forces, count, substeps);
    });
}

gbl_result gbl_run(gbl_backend *backend, const gbl_run_control *control, gbl_run_status *status_out) {
    return gbl::guard([&] {
        if (!backend || !control) gbl::invalid("null argument");
        backend->impl->run(*control);
        if (status_out) *status_out = backend->impl->status;
    });
}

gbl_result gbl_status(const gbl_backend *backend, gbl_run_status *status_out) {
    return gbl::guard([&] {
        if (!backend || !status_out) gbl::invalid("null argument");
        *status_out = backend->impl->status;
    });
}

gbl_result gbl_download(gbl_backend *backend, gbl_state_view *state, gbl_sphere *sphere) {
    return gbl::guard([&] {
        if (!backend || !state) gbl::invalid("null argument");
        backend->impl->download(*state, sphere);
    });
}

gbl_result gbl_first_failure_bonds(const gbl_backend *backend, uint32_t *out, uint64_t capacity, uint64_t *count) {
    return gbl::guard([&] {
        if (!backend || !count) gbl::invalid("null argument");
        const auto &f = backend->impl->first_failure;
        *count = f.size();
        if (out) std::memcpy(out, f.data(), sizeof(uint32_t) * std::min<std::uint64_t>(capacity, f.size()));
    });
}

gbl_result gbl_frame_count(const gbl_backend *backend, uint64_t *count) {
    return gbl::guard([&] {
        if (!backend || !count) gbl::invalid("null argument");
        *count = backend->impl->frames.size();
    });
}

gbl_result gbl_take_frame(const gbl_backend *backend, uint64_t index, uint64_t *step, float *u, uint8_t *alive,
                          float *damage, gbl_sphere *sphere) {
    return gbl::guard([&] {
        if (!backend) gbl::invalid("null backend");
        const auto &fr = backend->impl->frames;
        if (index >= fr.size()) gbl::invalid("frame index out of range");
        const auto &f = fr[index];
        if (step) *step = f.step;
        if (u) std::memcpy(u, f.u.data(), sizeof(float) * f.u.size());
        if (alive) std::memcpy(alive, f.alive.data(), f.alive.size());
        if (damage) std::memcpy(damage, f.damage.data(), sizeof(float) * f.damage.size());
        if (sphere) *sphere = f.sphere;
    });
}

gbl_result gbl_clear_frames(gbl_backend *backend) {
    return gbl::guard([&] {
        if (!backend) gbl::invalid("null backend");
        backend->impl->frames.clear();
        backend->impl->status.frames_captured = 0;
    });
}

gbl_result gbl_set_stream(gbl_backend *backend, void *cuda_stream) {
    return gbl::guard([&] {
        if (!backend) gbl::invalid("null backend");
        backend->impl->setStream(static_cast<cudaStream_t>(cuda_stream));
    });
}

gbl_result gbl_kernels_per_substep(gbl_backend *backend, uint64_t *count) {
    return gbl::guard([&] {
        if (!backend || !count) gbl::invalid("null argument");
        *count = backend->impl->kernelsPerSubstep();
    });
}

gbl_result gbl_profile_phases(gbl_backend *backend, uint64_t substeps, double *phase_ms) {
    return gbl::guard([&] {
        if (!backend || !phase_ms) gbl::invalid("null argument");
        backend->impl->profile(substeps, phase_ms);
    });
}

} // extern "C"
