// The GB300 lattice engine: device-resident lattices, the captured substep
// graph, and the C ABI of include/gbl.h -- the single-lattice LatticeBackend
// (FastLattice.hpp:255-405) and the batch of independent lattices.
//
// An Engine holds K lattices. Each keeps its own device arrays, control block
// and ledgers; a substep is one launch per phase (and per sweep level) over
// all of them, driven by work lists of (lattice, range) items. Lattices never
// interact, so every lattice's results are identical alone and in a batch.
#include "gbl_internal.hpp"
#include "gbl_kernels.cuh"

#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <cstdlib>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <functional>
#include <map>
#include <memory>
#include <new>
#include <mutex>
#include <set>
#include <string>
#include <exception>
#include <thread>
#include <type_traits>
#include <utility>
#include <vector>

namespace gbl {

namespace {

void check(cudaError_t e, const char *what) {
    if (e != cudaSuccess) runtime(std::string(what) + ": " + cudaGetErrorString(e));
}

// One allocation per lattice, carved into aligned arrays. The layout is
// recorded once (reserve) and bound to a base: a host image while the
// lattice is prepared, then its device allocation (stream-ordered, from the
// device's memory pool: admitting and retiring lattices does not synchronise
// the device).
class Arena {
public:
    Arena() = default;
    Arena(const Arena &) = delete;
    Arena &operator=(const Arena &) = delete;
    ~Arena() { release(); }
    void release() {
        if (base_) cudaFreeAsync(base_, stream_);
        base_ = nullptr;
    }
    template <class T> void reserve(T *&p, std::size_t count) {
        offsets_.push_back({reinterpret_cast<void **>(&p), bytes_});
        bytes_ += (count * sizeof(T) + 255) & ~static_cast<std::size_t>(255);
    }
    void bind(void *base) {
        for (auto &o : offsets_) *o.first = static_cast<char *>(base) + o.second;
    }
    void allocate(cudaStream_t stream) {
        release();
        stream_ = stream;
        check(cudaMallocAsync(&base_, bytes_ ? bytes_ : 256, stream), "device allocation");
        bind(base_);
    }
    [[nodiscard]] std::size_t bytes() const { return bytes_; }
    [[nodiscard]] void *base() const { return base_; }

private:
    void *base_{};
    cudaStream_t stream_{};
    std::size_t bytes_{};
    std::vector<std::pair<void **, std::size_t>> offsets_;
};

template <class T> void upload(T *dst, const std::vector<T> &src, cudaStream_t s) {
    if (!src.empty()) check(cudaMemcpyAsync(dst, src.data(), sizeof(T) * src.size(), cudaMemcpyHostToDevice, s), "copy");
}
template <class T> void uploadRaw(T *dst, const T *src, std::size_t n, cudaStream_t s) {
    if (n) check(cudaMemcpyAsync(dst, src, sizeof(T) * n, cudaMemcpyHostToDevice, s), "copy");
}
template <class T> void zero(T *dst, std::size_t n, cudaStream_t s) {
    if (n) check(cudaMemsetAsync(dst, 0, sizeof(T) * n, s), "memset");
}
// Helper threads of the library's parallel loops and copies, counted across
// every caller: a loop or copy borrows at most the cores not already lent,
// so concurrent callers (the submitting threads of a server, its admission)
// share the host instead of oversubscribing it. The caller's own thread
// always works.
std::atomic<long> g_helpers{0};
std::size_t borrowHelpers(std::size_t want) {
    const long cores = static_cast<long>(std::max(1U, std::thread::hardware_concurrency()));
    long lent = g_helpers.load();
    for (;;) {
        const long take = std::min<long>(static_cast<long>(want), std::max(0L, cores - 1 - lent));
        if (take <= 0) return 0;
        if (g_helpers.compare_exchange_weak(lent, lent + take)) return static_cast<std::size_t>(take);
    }
}
void returnHelpers(std::size_t n) { g_helpers -= static_cast<long>(n); }

struct Segment {
    void *dst;
    const void *src;
    std::size_t bytes;
};

// A crew of host threads that runs one job after another, each job split over
// the crew (the calling thread included) as job(t, T). The helpers are
// borrowed once for the crew's life, so a copy of many slices starts its
// threads once. A job must not throw.
class Crew {
public:
    using Job = std::function<void(std::size_t, std::size_t)>;
    explicit Crew(std::size_t want) : T_(1 + borrowHelpers(want)) {
        for (std::size_t t = 1; t < T_; ++t) threads_.emplace_back([this, t] { serve(t); });
    }
    Crew(const Crew &) = delete;
    Crew &operator=(const Crew &) = delete;
    ~Crew() {
        {
            std::lock_guard<std::mutex> g(m_);
            quit_ = true;
        }
        go_.notify_all();
        for (auto &th : threads_) th.join();
        returnHelpers(T_ - 1);
    }
    // job(t, T) on every member; returns when all have finished.
    void run(const Job &job) {
        {
            std::lock_guard<std::mutex> g(m_);
            job_ = &job;
            ++round_;
            left_ = T_ - 1;
        }
        go_.notify_all();
        job(0, T_);
        std::unique_lock<std::mutex> g(m_);
        done_.wait(g, [&] { return left_ == 0; });
        job_ = nullptr;
    }

private:
    void serve(std::size_t t) {
        std::size_t seen = 0;
        for (;;) {
            const Job *job = nullptr;
            {
                std::unique_lock<std::mutex> g(m_);
                go_.wait(g, [&] { return quit_ || round_ != seen; });
                if (quit_) return;
                seen = round_;
                job = job_;
            }
            (*job)(t, T_);
            std::lock_guard<std::mutex> g(m_);
            if (--left_ == 0) done_.notify_one();
        }
    }
    std::size_t T_;
    std::vector<std::thread> threads_;
    std::mutex m_;
    std::condition_variable go_, done_;
    const Job *job_{};
    std::size_t round_{}, left_{};
    bool quit_{};
};

// How large copies between pageable host memory and the device move
// (GBL_HOST_COPY): "pinned" (the default) -- host threads copy between the
// caller's memory and two page-locked staging buffers, whose contents the copy
// engines move while the threads fill or drain the other one; "driver" -- one
// cudaMemcpyAsync per 64 MB piece from several threads, the driver staging
// pageable memory itself.
bool pinnedCopies() {
    static const bool yes = [] {
        const char *env = std::getenv("GBL_HOST_COPY");
        return !(env && std::strcmp(env, "driver") == 0);
    }();
    return yes;
}

// The page-locked staging buffers of the pinned copies, per device: two
// slices, allocated at the device's first such copy and kept for the process
// (pinning memory costs about as much as copying it, so it is done once),
// under the ID of the context they were allocated in -- a device reset frees
// them, and the next copy allocates them again. Copies to one device take
// turns on its buffers.
constexpr std::size_t kPinnedSlice = std::size_t(64) << 20;
constexpr std::size_t kPinnedMinBytes = kPinnedSlice;
constexpr int kPinnedDevices = 64;
struct PinnedStage {
    std::mutex m;
    char *buf{};
    unsigned long long context{};
    bool refused{}; // page-locked memory was refused in this context: copies go through the driver
};
PinnedStage &pinnedStage(int device) {
    static PinnedStage *stages = new PinnedStage[kPinnedDevices]; // never destroyed: copies may run at teardown
    if (device < 0 || device >= kPinnedDevices) runtime("CUDA device ordinal out of range");
    return stages[device];
}

// One slice of a pinned copy: pieces of segments, each at its offset in a
// staging buffer.
struct SlicePiece {
    char *host;
    char *device;
    std::size_t bytes, at;
};

// The pinned copy of `segments` (host to device or device to host), slice by
// slice through the two staging buffers on a stream of its own: to the device,
// the crew fills one buffer while the copy engines empty the other; from the
// device, the engines fill one while the crew drains the other (the caller's
// crew, or one of the copy's own). Returns true when every byte has arrived,
// false (having copied nothing) when the slices cannot be allocated.
bool copySegmentsPinned(const std::vector<Segment> &segments, cudaMemcpyKind kind, Crew *crew_in) {
    const bool up = kind == cudaMemcpyHostToDevice;
    std::vector<std::vector<SlicePiece>> slices(1);
    std::size_t used = 0, total = 0;
    for (const Segment &g : segments) {
        char *host = up ? static_cast<char *>(const_cast<void *>(g.src)) : static_cast<char *>(g.dst);
        char *device = up ? static_cast<char *>(g.dst) : static_cast<char *>(const_cast<void *>(g.src));
        for (std::size_t off = 0; off < g.bytes;) {
            if (used == kPinnedSlice) {
                slices.emplace_back();
                used = 0;
            }
            const std::size_t n = std::min(g.bytes - off, kPinnedSlice - used);
            slices.back().push_back({host + off, device + off, n, used});
            used += n;
            off += n;
            total += n;
        }
    }
    if (!total) return true;
    int device = 0;
    check(cudaGetDevice(&device), "device");
    check(cudaSetDevice(device), "device"); // its context current on this thread, so its ID can be read
    PinnedStage &stage = pinnedStage(device);
    std::lock_guard<std::mutex> lock(stage.m);
    const unsigned long long context = currentContextId();
    if (context != 0 && context != stage.context) {
        // Buffers of an earlier context of this device went with it.
        stage.buf = nullptr;
        stage.refused = false;
        stage.context = context;
    }
    if (stage.refused) return false;
    if (!stage.buf) {
        const cudaError_t e = cudaHostAlloc(reinterpret_cast<void **>(&stage.buf), 2 * kPinnedSlice,
                                            cudaHostAllocDefault);
        if (e != cudaSuccess) {
            // Refused (a locked-memory limit, say): the copies are the
            // driver's. The error is this call's own; it is not left pending.
            if (cudaPeekAtLastError() == e) cudaGetLastError();
            stage.buf = nullptr;
            stage.refused = true;
            return false;
        }
    }
    cudaStream_t stream = nullptr;
    cudaEvent_t moved[2] = {nullptr, nullptr};
    struct Release {
        cudaStream_t &s;
        cudaEvent_t (&e)[2];
        ~Release() {
            if (s) {
                cudaStreamSynchronize(s);
                cudaStreamDestroy(s);
            }
            for (cudaEvent_t ev : e)
                if (ev) cudaEventDestroy(ev);
        }
    } release{stream, moved};
    check(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "stream");
    check(cudaEventCreateWithFlags(&moved[0], cudaEventDisableTiming), "event");
    check(cudaEventCreateWithFlags(&moved[1], cudaEventDisableTiming), "event");
    std::unique_ptr<Crew> own;
    if (!crew_in)
        own = std::make_unique<Crew>(std::min<std::size_t>(15, (total + (std::size_t(4) << 20) - 1) >> 22));
    Crew &crew = crew_in ? *crew_in : *own;
    // The crew's share of a slice: its bytes split evenly over the members.
    auto hostSide = [&](const std::vector<SlicePiece> &slice, char *buf) {
        std::size_t bytes = 0;
        for (const SlicePiece &p : slice) bytes += p.bytes;
        crew.run([&](std::size_t t, std::size_t T) {
            const std::size_t lo = bytes * t / T, hi = bytes * (t + 1) / T;
            for (const SlicePiece &p : slice) {
                const std::size_t a = std::max(lo, p.at), b = std::min(hi, p.at + p.bytes);
                if (a >= b) continue;
                if (up) std::memcpy(buf + a, p.host + (a - p.at), b - a);
                else std::memcpy(p.host + (a - p.at), buf + a, b - a);
            }
        });
    };
    auto engines = [&](const std::vector<SlicePiece> &slice, char *buf, int k) {
        for (const SlicePiece &p : slice)
            check(up ? cudaMemcpyAsync(p.device, buf + p.at, p.bytes, kind, stream)
                     : cudaMemcpyAsync(buf + p.at, p.device, p.bytes, kind, stream),
                  "copy");
        check(cudaEventRecord(moved[k], stream), "event");
    };
    char *buf[2] = {stage.buf, stage.buf + kPinnedSlice};
    const std::size_t S = slices.size();
    if (up) {
        for (std::size_t k = 0; k < S; ++k) {
            const int b = static_cast<int>(k & 1);
            if (k >= 2) check(cudaEventSynchronize(moved[b]), "copy"); // the engines have read this buffer
            hostSide(slices[k], buf[b]);
            engines(slices[k], buf[b], b);
        }
    } else {
        engines(slices[0], buf[0], 0);
        if (S > 1) engines(slices[1], buf[1], 1);
        for (std::size_t k = 0; k < S; ++k) {
            const int b = static_cast<int>(k & 1);
            check(cudaEventSynchronize(moved[b]), "copy");
            hostSide(slices[k], buf[b]);
            if (k + 2 < S) engines(slices[k + 2], buf[b], b);
        }
    }
    check(cudaStreamSynchronize(stream), "copy");
    return true;
}

// Copies between pageable host memory and the device. Pinned (above) when a
// crew is handed in, for every copy from the device, and for a copy to the
// device that fills at least one slice; otherwise (a small copy to the
// device, a copy the caller sends to the driver, or GBL_HOST_COPY=driver)
// split into pieces of at most 64 MB copied by several host threads at once
// (each on its own stream): the driver's staging of pageable memory is
// host-bound, one thread at a time. Measured: the 4096 downloads of a batch's
// trials 3.0 s pinned, 4.6-4.7 s through the driver; the host images of 532
// served requests arriving at 2000/s (a tenth of them 1.2 GB) admitted in
// 5.6-5.8 s pinned, 3.4 s through the driver, so a served image goes to the
// driver. Returns when every piece has arrived.
enum class Staging { kAuto, kDriver };
void copySegments(const std::vector<Segment> &segments, cudaMemcpyKind kind, Crew *crew = nullptr,
                  Staging staging = Staging::kAuto) {
    std::size_t total = 0;
    for (const Segment &g : segments) total += g.bytes;
    const bool pinned =
        crew || (staging == Staging::kAuto && pinnedCopies() &&
                 (kind == cudaMemcpyDeviceToHost || total >= kPinnedMinBytes));
    if (pinned && copySegmentsPinned(segments, kind, crew)) return;
    constexpr std::size_t kPiece = std::size_t(64) << 20;
    std::vector<Segment> pieces;
    for (const Segment &g : segments)
        for (std::size_t off = 0; off < g.bytes; off += kPiece)
            pieces.push_back({static_cast<char *>(g.dst) + off, static_cast<const char *>(g.src) + off,
                              std::min(kPiece, g.bytes - off)});
    if (pieces.empty()) return;
    if (pieces.size() == 1) {
        check(cudaMemcpy(pieces[0].dst, pieces[0].src, pieces[0].bytes, kind), "copy");
        return;
    }
    std::atomic<int> failed{static_cast<int>(cudaSuccess)};
    const std::size_t T = 1 + borrowHelpers(std::min<std::size_t>(15, pieces.size() - 1));
    std::vector<std::thread> pool;
    auto note = [&](cudaError_t e) {
        int ok = static_cast<int>(cudaSuccess);
        if (e != cudaSuccess) failed.compare_exchange_strong(ok, static_cast<int>(e));
    };
    auto work = [&](std::size_t t) {
        cudaStream_t s = nullptr;
        const cudaError_t made = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
        if (made != cudaSuccess) {
            note(made);
            return;
        }
        for (std::size_t c = t; c < pieces.size(); c += T)
            note(cudaMemcpyAsync(pieces[c].dst, pieces[c].src, pieces[c].bytes, kind, s));
        note(cudaStreamSynchronize(s));
        cudaStreamDestroy(s);
    };
    for (std::size_t t = 1; t < T; ++t) pool.emplace_back(work, t);
    work(0);
    for (auto &th : pool) th.join();
    returnHelpers(T - 1);
    check(static_cast<cudaError_t>(failed.load()), "copy");
}
void copyParallel(void *dst, const void *src, std::size_t bytes, cudaMemcpyKind kind) {
    copySegments({{dst, src, bytes}}, kind);
}

// Whether the device reads pageable host memory coherently through the host's
// page tables (as over a Grace CPU's chip-to-chip link).
bool deviceReadsPageable() {
    static const bool yes = [] {
        int dev = 0, access = 0, tables = 0;
        if (cudaGetDevice(&dev) != cudaSuccess) return false;
        if (cudaDeviceGetAttribute(&access, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess) return false;
        if (cudaDeviceGetAttribute(&tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev) != cudaSuccess)
            return false;
        return access == 1 && tables == 1;
    }();
    return yes;
}

// Whether an upload of `bytes` of caller arrays has its conversion kernels
// read them in place (where the device reads pageable memory) rather than
// staged: copied in chunks into device buffers (through the pinned slices, or
// the driver's staging for small lattices) and converted there. GBL_UPLOAD=
// in_place or staged fixes the choice; by default a lattice below 1 GiB of
// arrays is read in place (no host copy, nothing for the host to wait for: a
// batch's members upload behind one another) and a larger one is staged.
// Measured on the 9.8 GB impact lattice on a Grace host, per process: in place
// 0.43-1.35 s on first reads and 0.16-1.17 s again (it varies from process to
// process: the device's translations of the host's pages), staged through the
// pinned slices 0.21-0.30 s, staged through the driver's copies 1.36-1.45 s.
constexpr std::size_t kInPlaceMaxBytes = std::size_t(1) << 30;
bool uploadInPlace(std::size_t bytes) {
    if (!deviceReadsPageable()) return false;
    static const int choice = [] {
        const char *env = std::getenv("GBL_UPLOAD");
        if (env && std::strcmp(env, "in_place") == 0) return 1;
        if (env && std::strcmp(env, "staged") == 0) return 2;
        return 0;
    }();
    return choice == 1 || (choice == 0 && bytes < kInPlaceMaxBytes);
}

// An allocator that leaves trivial elements uninitialised when a vector is
// sized: the per-bond scratch of an upload (hundreds of MB for a large
// lattice) is written in full, or filled in parallel, before it is read, and
// a vector's own zero fill would be one thread's pass over all of it.
template <class T> struct NoInit : std::allocator<T> {
    template <class U> struct rebind { using other = NoInit<U>; };
    NoInit() = default;
    template <class U> NoInit(const NoInit<U> &) {}
    template <class U, class... A> void construct(U *p, A &&...a) {
        if constexpr (sizeof...(A) == 0) ::new (static_cast<void *>(p)) U;
        else ::new (static_cast<void *>(p)) U(std::forward<A>(a)...);
    }
};
template <class T> using Scratch = std::vector<T, NoInit<T>>;

// A static split of [0, n) over host threads, for the O(N + B) conversion
// loops of upload and download (f(begin, end) on disjoint ranges; f must not
// throw). Small ranges stay on the calling thread.
template <class F> void parallelFor(std::size_t n, F &&f, std::size_t grain = std::size_t(1) << 16) {
    const std::size_t want = std::min<std::size_t>(32, (n + grain - 1) / grain);
    const std::size_t T = want <= 1 ? 1 : 1 + borrowHelpers(want - 1);
    if (T <= 1) {
        f(std::size_t(0), n);
        return;
    }
    std::vector<std::thread> pool;
    pool.reserve(T - 1);
    for (std::size_t t = 1; t < T; ++t) pool.emplace_back([&f, n, t, T] { f(n * t / T, n * (t + 1) / T); });
    f(std::size_t(0), n / T);
    for (auto &th : pool) th.join();
    returnHelpers(T - 1);
}

} // namespace

struct Frame {
    std::uint64_t step;
    std::vector<float> u, damage;
    std::vector<std::uint8_t> alive;
    gbl_sphere sphere;
};

// The arrays a download writes, in the state's own layout (doubles, bonds in
// schedule order), in one device buffer: written by the device from a
// lattice's arrays, then copied array by array into a caller's state. A
// finished served request's result waits here for its caller, its lattice's
// own memory already freed.
struct StateOut {
    char *base{};
    std::size_t bytes{};
    std::uint32_t N{}, B{};
    double *u{}, *up{}, *v{};
    BondsOut o{};

    void copyTo(const gbl_state_view &st) const {
        if (st.node_count != N || st.bond_count != B) invalid("result state does not match the lattice");
        const std::size_t n3 = 3 * static_cast<std::size_t>(N) * sizeof(double), b = B;
        copySegments({{st.u, u, n3}, {st.u_prev, up, n3}, {st.v, v, n3}, {st.alive, o.alive, b},
                      {st.failure_mode, o.mode, b}, {st.damage, o.damage, 8 * b}, {st.prev_tensile, o.tensile, 8 * b},
                      {st.prev_compressive, o.compressive, 8 * b}, {st.prev_shear, o.shear, 8 * b},
                      {st.plastic_extension, o.plastic_extension, 8 * b},
                      {st.plastic_strain, o.plastic_strain, 8 * b}},
                     cudaMemcpyDeviceToHost);
    }
};

// One lattice resident on the device.
template <class R> struct Resident {
    static constexpr bool kDirect = std::is_same<R, double>::value;
    struct Level { std::uint32_t begin, end; };

    Schedule sched;
    std::uint32_t N{}, B{};
    std::uint64_t live_bonds{}; // bonds alive at upload
    Arena arena;
    Dev<R> dev{};
    std::vector<Level> levels;
    Scratch<std::uint32_t> dev2sched;         // storage -> schedule order
    std::vector<std::uint32_t> isolated;      // nodes without bonds
    Scratch<std::uint8_t> last_a, last_b;     // the last bond of its end a / b in the sweep, by schedule index
    bool plastic_state{};
    std::vector<R> mass, inv_mass;
    Sphere<R> sphere0{};
    // External loads (allocated on first use).
    Q4<R> *ext_force{};
    double *ext_req{}, *ext_contrib{};
    std::uint32_t *ext_nodes{};
    std::uint32_t ext_count{};
    std::uint64_t ext_remaining{};
    bool ext_dirty{};
    // External wrenches (allocated on first use): the set wrenches in name
    // order, their nodes listed in ext_nodes; every source kicked since
    // upload keeps a ledger slot, named by source_names.
    WrenchDev *wrench_dev{};
    std::uint32_t wrench_count{}, wrench_cap{};
    SourceSlot *source_dev{};
    std::size_t source_cap{};
    std::vector<std::string> source_names;
    // What a caller reads back.
    gbl_run_status status{};
    std::vector<std::uint32_t> first_failure;
    std::vector<Frame> frames;
    // The prepared host image of the filled part of the allocation.
    struct FreeImage {
        void operator()(unsigned char *p) const { std::free(p); }
    };
    std::unique_ptr<unsigned char, FreeImage> image_;
    std::size_t filled_{};

    explicit Resident(Schedule s) : sched(std::move(s)) {}
    Resident(const Resident &) = delete;
    Resident &operator=(const Resident &) = delete;
    // Node-to-node contact scratch (allocated when the settings turn it on).
    void *nc_mem{};
    // Upload in progress: the caller's state (direct upload), the sweep's
    // level boundaries, whether any bond has flowed (read back by commit).
    gbl_state_view view_{};
    std::vector<std::uint32_t> level_begin_;
    unsigned flowed_host_{};
    unsigned *flowed_dev_{};         // the in-place conversion's flag, until commitFinish reads it
    cudaEvent_t committed_{};        // commitBegin's work, until commitFinish waits for it
    cudaStream_t commit_stream_{};
    bool in_place_{};                // this upload's kernels read the caller's arrays in place

    // Bytes of the caller's arrays an upload reads: 14 doubles per node, 41
    // bytes per neighbour slot, 164 per bond.
    std::size_t hostBytes() const {
        return static_cast<std::size_t>(N) * 14 * sizeof(double) + static_cast<std::size_t>(dev.D) * N * 41 +
               static_cast<std::size_t>(B) * 164;
    }

    // The table size rule of latticeContactBucketMask (LatticePhysics.hpp:239-243),
    // applied to this lattice's own node count.
    static std::uint32_t contactBuckets(std::uint32_t n) {
        std::uint32_t size = 64U;
        while (size < 2U * n && size < (1U << 22)) size <<= 1U;
        return size;
    }
    // The scratch's parts in allocation order, each rounded to 256 bytes.
    static std::array<std::size_t, 10> contactParts(std::uint32_t n) {
        const std::size_t N = n, buckets = contactBuckets(n), tiles = (N + kThreads - 1) / kThreads;
        const std::size_t pairs = kPairsPerNode * N * 4;
        std::array<std::size_t, 10> parts{N * sizeof(Q4<R>), N * sizeof(int4), buckets * 4, buckets * 4, N * 4, N * 4,
                                         (tiles + 1) * 4, pairs, pairs, pairs};
        for (auto &b : parts) b = (b + 255) & ~std::size_t(255);
        return parts;
    }
    static std::size_t contactBytes(std::uint32_t n) {
        std::size_t total = 0;
        for (auto b : contactParts(n)) total += b;
        return total;
    }
    void ensureContact() {
        if (nc_mem) return;
        const auto parts = contactParts(N);
        check(cudaMalloc(&nc_mem, contactBytes(N)), "device allocation");
        char *p = static_cast<char *>(nc_mem);
        std::size_t k = 0;
        auto take = [&]() {
            char *at = p;
            p += parts[k++];
            return at;
        };
        dev.nc_built = reinterpret_cast<Q4<R> *>(take());
        dev.nc_cell = reinterpret_cast<int4 *>(take());
        dev.nc_count = reinterpret_cast<std::uint32_t *>(take());
        dev.nc_start = reinterpret_cast<std::uint32_t *>(take());
        dev.nc_members = reinterpret_cast<std::uint32_t *>(take());
        dev.nc_fill = reinterpret_cast<std::uint32_t *>(take());
        dev.nc_tile = reinterpret_cast<std::uint32_t *>(take());
        dev.nc_pa = reinterpret_cast<std::uint32_t *>(take());
        dev.nc_pb = reinterpret_cast<std::uint32_t *>(take());
        dev.nc_pbond = reinterpret_cast<std::uint32_t *>(take());
        dev.nc_mask = contactBuckets(N) - 1U;
    }

    ~Resident() {
        if (committed_) {
            cudaEventSynchronize(committed_);
            cudaEventDestroy(committed_);
        }
        if (flowed_dev_) cudaFree(flowed_dev_);
        if (nc_mem) cudaFree(nc_mem);
        if (ext_force) cudaFree(ext_force);
        if (ext_req) cudaFree(ext_req);
        if (ext_contrib) cudaFree(ext_contrib);
        if (ext_nodes) cudaFree(ext_nodes);
        if (wrench_dev) cudaFree(wrench_dev);
        if (source_dev) cudaFree(source_dev);
    }

    // Levels of the projection sweep. The reference sweeps bonds in one
    // serial order: every slab's interior colours, then the boundary colours
    // of even slabs, then of odd slabs (CpuLatticeBackend.cpp:336-348,
    // 395-407). A bond's depth is one more than the deepest earlier bond at
    // either of its nodes; bonds of equal depth share no node, and along every
    // node the depths rise in the serial order, so running the levels in
    // depth order, each level in any thread order, is the serial sweep
    // exactly. Bonds are stored level-major (stable in the serial order), and
    // each node's last bond of the sweep is flagged: its support projection
    // follows that bond.
    void buildLevels(const gbl_state_view &st) {
        const std::uint32_t C = sched.color_count, K = sched.block_count;
        const std::uint32_t *nbb = sched.node_block_begin.data();
        // The serial order as segments: every slab's interior colours, then
        // the boundary colours of even slabs, then of odd slabs.
        struct Seg { std::uint32_t slab, phase, begin, end; };
        std::vector<Seg> segs;
        std::uint32_t total = 0;
        auto add = [&](std::uint32_t blk, std::uint32_t boundary, std::uint32_t phase) {
            for (std::uint32_t c = 0; c < C; ++c) {
                const std::size_t key = sched.rangeKey(blk, boundary, c);
                const std::uint32_t n = sched.range_end[key] - sched.range_begin[key];
                if (n) segs.push_back({blk, phase, sched.range_begin[key], sched.range_begin[key] + n});
                total += n;
            }
        };
        for (std::uint32_t blk = 0; blk < K; ++blk) add(blk, 0, 0);
        for (std::uint32_t blk = 0; blk < K; blk += 2) add(blk, 1, 1);
        for (std::uint32_t blk = 1; blk < K; blk += 2) add(blk, 1, 2);
        if (total != B) invalid("lattice schedule ranges do not cover every bond exactly once");
        // Segments grouped by (phase, slab), in serial order.
        struct Task { std::uint32_t phase, slab, seg_begin, seg_end; };
        std::vector<Task> tasks;
        for (std::uint32_t k = 0; k < segs.size(); ++k) {
            if (tasks.empty() || tasks.back().phase != segs[k].phase || tasks.back().slab != segs[k].slab)
                tasks.push_back({segs[k].phase, segs[k].slab, k, k});
            tasks.back().seg_end = k + 1;
        }
        // Within a phase the slabs touch disjoint nodes when every interior
        // bond stays in its slab and every boundary bond in its slab and the
        // next; then the slabs of a phase run in parallel (the per-node order
        // of the serial walk is kept exactly), else the walk is serial.
        std::atomic<bool> bad{false}, local{true};
        parallelFor(tasks.size(), [&](std::size_t lo, std::size_t hi) {
            for (std::size_t t = lo; t < hi; ++t) {
                const Task &task = tasks[t];
                const std::uint32_t n0 = nbb[task.slab];
                const std::uint32_t n1 = nbb[std::min<std::uint32_t>(task.slab + (task.phase == 0 ? 1U : 2U), K)];
                for (std::uint32_t k = task.seg_begin; k < task.seg_end; ++k)
                    for (std::uint32_t j = segs[k].begin; j < segs[k].end; ++j) {
                        const std::uint32_t a = st.bond_a[j], b = st.bond_b[j];
                        if (a >= N || b >= N || a == b) bad.store(true);
                        else if (a < n0 || a >= n1 || b < n0 || b >= n1) local.store(false);
                    }
            }
        }, 1);
        if (bad.load()) invalid("lattice bond joins invalid nodes");
        Scratch<std::uint32_t> depth(B);
        parallelFor(B, [&](std::size_t lo, std::size_t hi) {
            std::memset(depth.data() + lo, 0, sizeof(std::uint32_t) * (hi - lo));
        });
        std::vector<std::uint32_t> reached(N, 0), last(N, kNoBond);
        auto walk = [&](const Task &task) {
            std::uint32_t deepest = 0;
            for (std::uint32_t k = task.seg_begin; k < task.seg_end; ++k)
                for (std::uint32_t j = segs[k].begin; j < segs[k].end; ++j) {
                    const std::uint32_t a = st.bond_a[j], b = st.bond_b[j];
                    const std::uint32_t d = std::max(reached[a], reached[b]) + 1;
                    depth[j] = d;
                    reached[a] = reached[b] = d;
                    last[a] = last[b] = j;
                    deepest = std::max(deepest, d);
                }
            return deepest;
        };
        std::uint32_t deepest = 0;
        if (local.load()) {
            std::mutex m;
            for (std::uint32_t phase = 0; phase < 3; ++phase) {
                std::vector<std::uint32_t> ids;
                for (std::uint32_t t = 0; t < tasks.size(); ++t)
                    if (tasks[t].phase == phase) ids.push_back(t);
                parallelFor(ids.size(), [&](std::size_t lo, std::size_t hi) {
                    std::uint32_t dmax = 0;
                    for (std::size_t q = lo; q < hi; ++q) dmax = std::max(dmax, walk(tasks[ids[q]]));
                    std::lock_guard<std::mutex> lock(m);
                    deepest = std::max(deepest, dmax);
                }, 1);
            }
        } else {
            for (const Task &task : tasks) deepest = std::max(deepest, walk(task));
        }
        // Storage order: by depth, stable in the serial order (a parallel
        // counting sort over chunks of the serial walk).
        Scratch<std::uint32_t> order(B);
        {
            std::vector<std::uint32_t> at(segs.size() + 1, 0);
            for (std::size_t k = 0; k < segs.size(); ++k) at[k + 1] = at[k] + (segs[k].end - segs[k].begin);
            parallelFor(segs.size(), [&](std::size_t lo, std::size_t hi) {
                for (std::size_t k = lo; k < hi; ++k)
                    for (std::uint32_t j = segs[k].begin, o = at[k]; j < segs[k].end; ++j, ++o) order[o] = j;
            }, 1);
        }
        const std::uint32_t D1 = deepest + 2;
        const std::size_t chunk = std::max<std::size_t>(std::size_t(1) << 16, (B + 63) / 64);
        const std::size_t nchunks = (B + chunk - 1) / chunk;
        std::vector<std::uint32_t> counts(nchunks * D1, 0);
        parallelFor(nchunks, [&](std::size_t lo, std::size_t hi) {
            for (std::size_t c = lo; c < hi; ++c) {
                std::uint32_t *h = counts.data() + c * D1;
                for (std::size_t o = c * chunk; o < std::min<std::size_t>(B, (c + 1) * chunk); ++o) ++h[depth[order[o]]];
            }
        }, 1);
        std::vector<std::uint32_t> first(D1 + 1, 0);
        for (std::uint32_t d = 0; d < D1; ++d) {
            std::uint32_t sum = 0;
            for (std::size_t c = 0; c < nchunks; ++c) sum += counts[c * D1 + d];
            first[d + 1] = first[d] + sum;
        }
        // counts becomes each chunk's starting offset within each depth.
        for (std::uint32_t d = 0; d < D1; ++d) {
            std::uint32_t run = first[d];
            for (std::size_t c = 0; c < nchunks; ++c) {
                const std::uint32_t n = counts[c * D1 + d];
                counts[c * D1 + d] = run;
                run += n;
            }
        }
        dev2sched.resize(B); // every entry written by the scatter below
        parallelFor(nchunks, [&](std::size_t lo, std::size_t hi) {
            for (std::size_t c = lo; c < hi; ++c) {
                std::uint32_t *fill = counts.data() + c * D1;
                for (std::size_t o = c * chunk; o < std::min<std::size_t>(B, (c + 1) * chunk); ++o) {
                    const std::uint32_t j = order[o];
                    dev2sched[fill[depth[j]]++] = j;
                }
            }
        }, 1);
        levels.clear();
        for (std::uint32_t d = 1; d <= deepest; ++d)
            if (first[d + 1] > first[d]) levels.push_back({first[d], first[d + 1]});
        last_a.resize(B);
        last_b.resize(B);
        parallelFor(B, [&](std::size_t lo, std::size_t hi) {
            std::memset(last_a.data() + lo, 0, hi - lo);
            std::memset(last_b.data() + lo, 0, hi - lo);
        });
        parallelFor(N, [&](std::size_t lo, std::size_t hi) {
            for (std::size_t i = lo; i < hi; ++i) {
                if (last[i] == kNoBond) continue;
                (st.bond_a[last[i]] == i ? last_a : last_b)[last[i]] = 1; // by schedule index
            }
        });
        isolated.clear();
        for (std::uint32_t i = 0; i < N; ++i)
            if (last[i] == kNoBond) isolated.push_back(i);
    }

    // The device arrays of one lattice, in one allocation: first the arrays an
    // upload fills from the state, then the ones that start at zero. Returns
    // the size of the first part.
    static std::size_t reserve(Arena &a, Dev<R> &d, std::uint32_t N, std::uint32_t B, std::uint32_t D,
                               std::uint32_t blocks, std::size_t isolated) {
        const std::size_t P = static_cast<std::size_t>(D) * N;
        a.reserve(d.u, N); a.reserve(d.v, N); a.reserve(d.x0, N); a.reserve(d.up, N);
        a.reserve(d.nbr, P); a.reserve(d.nbr_other, P); a.reserve(d.nbr_bond, P);
        a.reserve(d.slot_a, B); a.reserve(d.slot_b, B);
        a.reserve(d.rec, B); a.reserve(d.geo, B); a.reserve(d.prev, B); a.reserve(d.thr4, B);
        a.reserve(d.thr2, B); a.reserve(d.plastic, B); a.reserve(d.mode, B);
        a.reserve(d.dev2sched, B); a.reserve(d.isolated, isolated + 1);
        a.reserve(d.node_block_begin, blocks + 1);
        a.reserve(d.level_begin, kMaxFusedLevels + 1);
        a.reserve(d.sphere, 1);
        a.reserve(d.dirty, N + 4);
        const std::size_t filled = a.bytes();
        a.reserve(d.strain, 2 * static_cast<std::size_t>(N));
        a.reserve(d.rinv, 9 * static_cast<std::size_t>(N)); a.reserve(d.unm, 3 * static_cast<std::size_t>(N));
        a.reserve(d.approach, kPlanes * static_cast<std::size_t>(N));
        a.reserve(d.engaged, kPlanes * static_cast<std::size_t>(N));
        a.reserve(d.candidate, N); a.reserve(d.cand_bits, (N + 31) / 32 + 1);
        a.reserve(d.lambda, B);
        a.reserve(d.ev_bits, d.words_b + 1); a.reserve(d.ev_tile, d.tiles_b + 1); a.reserve(d.ev_list, B + 1);
        a.reserve(d.ev_removed, B); a.reserve(d.ev_packed, B + 1); a.reserve(d.ev_prefix, B + 1);
        a.reserve(d.ev_ends, B);
        a.reserve(d.dmg_bits, d.words_b + 1); a.reserve(d.dmg_tile, d.tiles_b + 1);
        a.reserve(d.dmg_list, B + 1); a.reserve(d.ev_damage, B); a.reserve(d.dmg_value, B + 1);
        a.reserve(d.tile_plastic, d.tiles_b + 1); a.reserve(d.tile_removed, d.tiles_b + 1);
        const std::size_t scan_blocks = d.tiles_b / kScanBlock + 1;
        a.reserve(d.blk_ev, scan_blocks); a.reserve(d.blk_dmg, scan_blocks);
        a.reserve(d.blk_removed, scan_blocks); a.reserve(d.blk_plastic, scan_blocks);
        a.reserve(d.cand_list, static_cast<std::size_t>(blocks) * kCandidatesPerBlock);
        a.reserve(d.cand_count, blocks);
        a.reserve(d.dirty_list, N + 1); a.reserve(d.ffb, B + 1);
        a.reserve(d.halo_stamp, N); a.reserve(d.late_tile_stamp, d.tiles_b + 1);
        return filled;
    }

    // Device bytes a lattice of these counts takes (its isolated nodes at
    // most N; external load buffers included): what admission charges.
    static std::size_t footprint(std::uint32_t N, std::uint32_t B, std::uint32_t D, std::uint32_t blocks) {
        Arena a;
        Dev<R> d{};
        d.words_b = (B + 31) / 32;
        d.tiles_b = (B + kThreads - 1) / kThreads;
        reserve(a, d, N, B, D, blocks, N);
        return a.bytes() + static_cast<std::size_t>(N) * (sizeof(Q4<R>) + 16 * sizeof(double) + sizeof(std::uint32_t));
    }

    // upload, host half (FastLattice.hpp:267-268; WorkingLattice::fromState,
    // LatticeWorking.hpp:53-124): the device layout of the state, written into
    // a host image of the allocation. No CUDA call: lattices can be prepared
    // on several threads at once.
    void prepare(const gbl_state_view &st, const gbl_sphere &sphere, bool image = true) {
        N = st.node_count;
        B = st.bond_count;
        if (N > kNodeMask) invalid("lattice exceeds 2^30 nodes");
        if (sched.bond_count != B || sched.node_count != N) invalid("lattice schedule does not match the lattice");
        const std::uint32_t D = st.max_degree;
        buildLevels(st);
        Dev<R> &d = dev;
        d = Dev<R>{};
        d.N = N; d.B = B; d.D = D; d.blocks = sched.block_count;
        d.words_b = (B + 31) / 32;
        d.tiles_b = (B + kThreads - 1) / kThreads;
        filled_ = reserve(arena, d, N, B, D, sched.block_count, isolated.size());
        mass.resize(N);
        inv_mass.resize(N);
        parallelFor(N, [&](std::size_t lo, std::size_t hi) {
            for (std::size_t i = lo; i < hi; ++i) {
                mass[i] = R(st.mass[i]);
                inv_mass[i] = R(st.inv_mass[i]);
            }
        });
        std::atomic<std::uint64_t> live{0};
        parallelFor(B, [&](std::size_t lo, std::size_t hi) {
            std::uint64_t n = 0;
            for (std::size_t j = lo; j < hi; ++j) n += st.alive[j] != 0;
            live += n;
        });
        live_bonds = live;
        d.isolated_count = static_cast<std::uint32_t>(isolated.size());
        // Level boundaries for the one-CTA sweep, when the levels fit its table.
        d.level_count = levels.size() <= kMaxFusedLevels ? static_cast<std::uint32_t>(levels.size()) : 0U;
        level_begin_.assign(d.level_count + 1, 0U);
        for (std::uint32_t k = 0; k < d.level_count; ++k) level_begin_[k] = levels[k].begin;
        level_begin_[d.level_count] = d.level_count ? levels[d.level_count - 1].end : 0U;
        sphere0.center = {R(sphere.center[0]), R(sphere.center[1]), R(sphere.center[2])};
        sphere0.velocity = {R(sphere.velocity[0]), R(sphere.velocity[1]), R(sphere.velocity[2])};
        sphere0.angular = {R(sphere.angular_velocity[0]), R(sphere.angular_velocity[1]), R(sphere.angular_velocity[2])};
        sphere0.radius = R(sphere.radius);
        sphere0.mass = R(sphere.mass);
        sphere0.inertia = R(sphere.inertia);
        std::memcpy(d.origin, st.origin, sizeof(d.origin));
        // Loads do not survive an upload (ExternalLoads.hpp:26 reset).
        ext_count = 0;
        ext_remaining = 0;
        clearSources();
        status = gbl_run_status{};
        status.first_failure_step = status.last_failure_step = status.last_energy_gain_step = ~0ULL;
        first_failure.clear();
        frames.clear();
        if (image) writeImage(st);
        else view_ = st; // commit reads the caller's arrays, which stay valid until it returns
    }

    // The device layout written into a host image of the allocation (the
    // served form: a request's state need not outlive its submission).
    void writeImage(const gbl_state_view &st) {
        Dev<R> &d = dev;
        const std::uint32_t D = d.D;
        image_.reset(static_cast<unsigned char *>(std::aligned_alloc(256, filled_ ? filled_ : 256)));
        if (!image_) throw std::bad_alloc();
        arena.bind(image_.get());
        parallelFor(N, [&](std::size_t lo, std::size_t hi) {
            for (std::size_t i = lo; i < hi; ++i) {
                d.u[i] = {R(st.u[3 * i]), R(st.u[3 * i + 1]), R(st.u[3 * i + 2]), R(st.inv_mass[i])};
                d.v[i] = {R(st.v[3 * i]), R(st.v[3 * i + 1]), R(st.v[3 * i + 2]), R(st.mass[i])};
                d.x0[i] = {R(st.x0[3 * i]), R(st.x0[3 * i + 1]), R(st.x0[3 * i + 2]), R(0)};
                d.up[i] = {R(st.u_prev[3 * i]), R(st.u_prev[3 * i + 1]), R(st.u_prev[3 * i + 2]), R(0)};
            }
        });
        // Every node starts dirty: the first substep restarts in full.
        std::memset(d.dirty, 1, N);
        std::memset(d.dirty + N, 0, 4);
        // Neighbour slots: (rest, weight if alive), the other node (itself when padded).
        const std::size_t P = static_cast<std::size_t>(D) * N;
        parallelFor(P, [&](std::size_t lo, std::size_t hi) {
            for (std::size_t s = lo; s < hi; ++s) {
                const bool present = st.nbr_bond[s] != kNoBond;
                const std::uint32_t node = static_cast<std::uint32_t>(s % N);
                const R w = R(st.nbr_weight[s]);
                d.nbr[s] = {R(st.nbr_rest[3 * s]), R(st.nbr_rest[3 * s + 1]), R(st.nbr_rest[3 * s + 2]),
                            present ? (st.nbr_alive[s] ? w : -absR(w)) : R(0)};
                d.nbr_other[s] = present ? st.nbr_other[s] : node;
                d.nbr_bond[s] = present ? st.nbr_bond[s] : kNoBond; // schedule index; storage index on the device
            }
        });
        // Bonds in schedule order, read and written in sequence; commit moves
        // them to storage (level-major) order on the device.
        std::atomic<bool> plastic_any{false};
        parallelFor(B, [&](std::size_t lo, std::size_t hi) {
            bool any = false;
            for (std::size_t j = lo; j < hi; ++j) {
                d.rec[j] = {st.bond_a[j] | (st.alive[j] ? 0U : kDeadBit) | (last_a[j] ? kLastABit : 0U),
                            st.bond_b[j] | (last_b[j] ? kLastBBit : 0U), R(st.rest_length_sq_minus[j]),
                            R(st.rest_length[j])};
                d.geo[j] = {R(st.rest_edge[3 * j]), R(st.rest_edge[3 * j + 1]), R(st.rest_edge[3 * j + 2]),
                            R(st.compliance[j])};
                d.prev[j] = {R(st.prev_tensile[j]), R(st.prev_compressive[j]), R(st.prev_shear[j]), R(st.damage[j])};
                const double *t = st.threshold + 6 * j;
                d.thr4[j] = {R(t[0]), R(t[1]), R(t[2]), R(t[3])};
                d.thr2[j] = {R(t[4]), R(t[5])};
                d.plastic[j] = {R(st.plastic_extension[j]), R(st.plastic_strain[j])};
                any = any || d.plastic[j].x != R(0);
                d.slot_a[j] = st.bond_slot_a[j];
                d.slot_b[j] = st.bond_slot_b[j];
                d.mode[j] = st.failure_mode[j];
            }
            if (any) plastic_any.store(true);
        });
        plastic_state = plastic_any.load();
        std::memcpy(d.dev2sched, dev2sched.data(), sizeof(std::uint32_t) * B);
        if (!isolated.empty()) std::memcpy(d.isolated, isolated.data(), sizeof(std::uint32_t) * isolated.size());
        std::memcpy(d.node_block_begin, sched.node_block_begin.data(), sizeof(std::uint32_t) * (sched.block_count + 1));
        std::memcpy(d.level_begin, level_begin_.data(), sizeof(std::uint32_t) * level_begin_.size());
        *d.sphere = sphere0;
    }

    // The per-bond arrays of the device layout, and the same arrays in a
    // buffer laid out as the allocation's [slot_a, dev2sched) range.
    BondSet<R> bonds() const {
        return {dev.slot_a, dev.slot_b, dev.rec, dev.geo, dev.prev, dev.thr4, dev.thr2, dev.plastic, dev.mode};
    }
    BondSet<R> bondsAt(char *region) const {
        const char *lo = reinterpret_cast<const char *>(dev.slot_a);
        auto at = [&](auto *p) {
            return reinterpret_cast<decltype(p)>(region + (reinterpret_cast<const char *>(p) - lo));
        };
        return {at(dev.slot_a), at(dev.slot_b), at(dev.rec), at(dev.geo), at(dev.prev),
                at(dev.thr4), at(dev.thr2), at(dev.plastic), at(dev.mode)};
    }
    static unsigned reorderGrid(std::size_t n) {
        return static_cast<unsigned>(std::min<std::size_t>((n + kThreads - 1) / kThreads, 152 * 16));
    }

    // upload, device half: one allocation, the prepared image copied in, the
    // rest cleared. The host image is released.
    void commit(cudaStream_t stream) {
        commitBegin(stream);
        commitFinish();
    }

    // commit's first half: the allocation, the copies and the conversion and
    // reordering kernels, enqueued on `stream`; the host waits only for the
    // allocation (and, on the staged and image paths, for its own copies).
    void commitBegin(cudaStream_t stream) {
        if (!image_ && !view_.u && N) logic("lattice committed before it was prepared");
        commit_stream_ = stream;
        arena.allocate(stream);
        char *base = static_cast<char *>(arena.base());
        // The per-bond arrays, [slot_a, dev2sched) of the allocation, arrive in
        // schedule order in a staging copy and are moved to storage order.
        const std::size_t lo = static_cast<std::size_t>(reinterpret_cast<char *>(dev.slot_a) - base);
        const std::size_t hi = static_cast<std::size_t>(reinterpret_cast<char *>(dev.dev2sched) - base);
        char *staged = nullptr;
        if (B) check(cudaMallocAsync(&staged, hi - lo, stream), "device allocation");
        // Host-side copies on other streams need the allocation made; the
        // in-place path keeps all its work on `stream`.
        in_place_ = !image_ && uploadInPlace(hostBytes());
        if (!in_place_) check(cudaStreamSynchronize(stream), "device allocation");
        if (image_) {
            const unsigned char *img = image_.get();
            copySegments({{base, img, lo}, {staged, img + lo, B ? hi - lo : 0}, {base + hi, img + hi, filled_ - hi}},
                         cudaMemcpyHostToDevice, nullptr, Staging::kDriver);
        } else {
            convertOnDevice(staged, stream);
        }
        if (B) {
            const unsigned grid = reorderGrid(B);
            std::uint32_t *sched2dev_dev = dev.ev_list; // scratch of the cleared part, cleared below
            kInvertOrder<<<grid, kThreads, 0, stream>>>(sched2dev_dev, dev.dev2sched, B);
            const std::size_t P = static_cast<std::size_t>(dev.D) * N;
            if (P) kSlotsToStorage<<<reorderGrid(P), kThreads, 0, stream>>>(dev.nbr_bond, sched2dev_dev, P);
            kBondsToStorage<R><<<grid, kThreads, 0, stream>>>(bonds(), bondsAt(staged), dev.dev2sched, B);
            check(cudaGetLastError(), "kernel launch");
            check(cudaFreeAsync(staged, stream), "device free");
        }
        if (arena.bytes() > filled_)
            check(cudaMemsetAsync(base + filled_, 0, arena.bytes() - filled_, stream), "memset");
        dev.ext_force = ext_force; dev.ext_req = ext_req; dev.ext_contrib = ext_contrib; dev.ext_nodes = ext_nodes;
        check(cudaEventCreateWithFlags(&committed_, cudaEventDisableTiming), "event");
        check(cudaEventRecord(committed_, stream), "event");
    }

    // commit's second half: waits for the work commitBegin enqueued, then
    // reads whether any bond has flowed; the caller's state is not read again.
    void commitFinish() {
        if (committed_) {
            check(cudaEventSynchronize(committed_), "upload");
            cudaEventDestroy(committed_);
            committed_ = nullptr;
        }
        if (flowed_dev_) {
            check(cudaMemcpy(&flowed_host_, flowed_dev_, sizeof(unsigned), cudaMemcpyDeviceToHost), "copy");
            check(cudaFreeAsync(flowed_dev_, commit_stream_), "device free");
            flowed_dev_ = nullptr;
            plastic_state = flowed_host_ != 0;
        }
        image_.reset();
        view_ = gbl_state_view{};
    }

    // The direct upload where the device reads pageable host memory: the
    // conversion kernels read the caller's arrays in place, in sequence.
    void convertFromHost(char *staged, cudaStream_t stream) {
        const gbl_state_view &st = view_;
        unsigned *flowed = nullptr;
        check(cudaMallocAsync(&flowed, 256, stream), "device allocation");
        check(cudaMemsetAsync(flowed, 0, sizeof(unsigned), stream), "memset");
        if (N)
            kNodesIn<R><<<reorderGrid(N), kThreads, 0, stream>>>(
                dev.u, dev.v, dev.x0, dev.up, NodesIn{st.u, st.u_prev, st.v, st.x0, st.mass, st.inv_mass}, 0, N);
        const std::size_t P = static_cast<std::size_t>(dev.D) * N;
        if (P)
            kSlotsIn<R><<<reorderGrid(P), kThreads, 0, stream>>>(
                dev.nbr, dev.nbr_other, dev.nbr_bond,
                SlotsIn{st.nbr_rest, st.nbr_weight, st.nbr_alive, st.nbr_other, st.nbr_bond}, 0, P, N);
        if (B) {
            const BondsIn in{st.bond_a, st.bond_b, st.bond_slot_a, st.bond_slot_b, st.alive, st.failure_mode,
                             last_a.data(), last_b.data(), st.rest_length_sq_minus, st.rest_length, st.rest_edge,
                             st.compliance, st.prev_tensile, st.prev_compressive, st.prev_shear, st.damage,
                             st.threshold, st.plastic_extension, st.plastic_strain};
            kBondsIn<R><<<reorderGrid(B), kThreads, 0, stream>>>(bondsAt(staged), in, 0, B, flowed);
        }
        // The small arrays, read in place too (this lattice keeps them until
        // commitFinish), and every node dirty: the first substep restarts in full.
        auto words = [&](void *dst, const void *src, std::size_t bytes) {
            if (!bytes) return;
            const std::size_t n = bytes / sizeof(std::uint32_t);
            kCopyWords<<<reorderGrid(n), kThreads, 0, stream>>>(static_cast<std::uint32_t *>(dst),
                                                              static_cast<const std::uint32_t *>(src), n);
        };
        static_assert(sizeof(Sphere<R>) % sizeof(std::uint32_t) == 0, "sphere record copied as words");
        words(dev.dev2sched, dev2sched.data(), sizeof(std::uint32_t) * B);
        words(dev.isolated, isolated.data(), sizeof(std::uint32_t) * isolated.size());
        words(dev.node_block_begin, sched.node_block_begin.data(), sizeof(std::uint32_t) * (sched.block_count + 1));
        words(dev.level_begin, level_begin_.data(), sizeof(std::uint32_t) * level_begin_.size());
        words(dev.sphere, &sphere0, sizeof(sphere0));
        check(cudaGetLastError(), "kernel launch");
        check(cudaMemsetAsync(dev.dirty, 1, N, stream), "memset");
        check(cudaMemsetAsync(dev.dirty + N, 0, 4, stream), "memset");
        flowed_dev_ = flowed; // read by commitFinish
    }

    // The direct upload: the caller's arrays, chunk by chunk, copied as they
    // are into one of two device staging buffers (the next chunk's copy runs
    // while the previous chunk converts) and converted there, the bonds into
    // `staged` in schedule order; then the small arrays.
    void convertOnDevice(char *staged, cudaStream_t stream) {
        const gbl_state_view &st = view_;
        if (in_place_) {
            convertFromHost(staged, stream);
            return;
        }
        // Each staging buffer holds up to 256 MB of the caller's arrays (less
        // when the whole lattice needs less).
        const std::size_t P = static_cast<std::size_t>(dev.D) * N;
        const std::size_t whole = std::max({N * 14 * sizeof(double), P * 41, static_cast<std::size_t>(B) * 164});
        auto round = [](std::size_t x) { return (x + 255) & ~std::size_t(255); };
        // A multiple of 256 bytes: the second buffer and every part start aligned.
        const std::size_t kStage = round(std::min(std::size_t(256) << 20, whole + 32 * 256));
        // Pinned copies for a lattice of at least one slice: one crew of host
        // threads copies every chunk, a thread per 4 MB of the arrays, at
        // most 16. A smaller lattice's chunks go through the driver's staging.
        std::unique_ptr<Crew> crew;
        if (pinnedCopies() && hostBytes() >= kPinnedMinBytes)
            crew = std::make_unique<Crew>(std::min<std::size_t>(15, hostBytes() >> 22));
        char *stage = nullptr;
        check(cudaMallocAsync(&stage, 2 * kStage + 256, stream), "device allocation");
        unsigned *flowed = reinterpret_cast<unsigned *>(stage + 2 * kStage);
        check(cudaMemsetAsync(flowed, 0, sizeof(unsigned), stream), "memset");
        check(cudaStreamSynchronize(stream), "device allocation");
        cudaEvent_t used[2] = {nullptr, nullptr};
        check(cudaEventCreateWithFlags(&used[0], cudaEventDisableTiming), "event");
        check(cudaEventCreateWithFlags(&used[1], cudaEventDisableTiming), "event");
        bool pending[2] = {false, false};
        int turn = 0;
        struct Part { const void *src; std::size_t bytes; };
        // One chunk: its parts staged into the free buffer, then converted.
        auto chunk = [&](std::initializer_list<Part> parts, auto &&convert) {
            if (pending[turn]) check(cudaEventSynchronize(used[turn]), "upload");
            char *buf = stage + static_cast<std::size_t>(turn) * kStage;
            std::vector<Segment> segments;
            std::vector<const char *> at;
            std::size_t off = 0;
            for (const Part &q : parts) {
                at.push_back(buf + off);
                segments.push_back({buf + off, q.src, q.bytes});
                off += round(q.bytes);
            }
            copySegments(segments, cudaMemcpyHostToDevice, crew.get());
            convert(at);
            check(cudaGetLastError(), "kernel launch");
            check(cudaEventRecord(used[turn], stream), "event");
            pending[turn] = true;
            turn ^= 1;
        };
        auto f64 = [](const char *p) { return reinterpret_cast<const double *>(p); };
        auto u32 = [](const char *p) { return reinterpret_cast<const std::uint32_t *>(p); };
        auto u8 = [](const char *p) { return reinterpret_cast<const std::uint8_t *>(p); };
        const std::size_t per_node = (kStage - 6 * 256) / (14 * sizeof(double));
        for (std::size_t i0 = 0; i0 < N; i0 += per_node) {
            const std::size_t n = std::min<std::size_t>(per_node, N - i0);
            chunk({{st.u + 3 * i0, 24 * n}, {st.u_prev + 3 * i0, 24 * n}, {st.v + 3 * i0, 24 * n},
                   {st.x0 + 3 * i0, 24 * n}, {st.mass + i0, 8 * n}, {st.inv_mass + i0, 8 * n}},
                  [&](const std::vector<const char *> &at) {
                      const NodesIn in{f64(at[0]), f64(at[1]), f64(at[2]), f64(at[3]), f64(at[4]), f64(at[5])};
                      kNodesIn<R><<<reorderGrid(n), kThreads, 0, stream>>>(dev.u, dev.v, dev.x0, dev.up, in, i0, n);
                  });
        }
        const std::size_t per_slot = (kStage - 5 * 256) / 41;
        for (std::size_t s0 = 0; s0 < P; s0 += per_slot) {
            const std::size_t n = std::min(per_slot, P - s0);
            chunk({{st.nbr_rest + 3 * s0, 24 * n}, {st.nbr_weight + s0, 8 * n}, {st.nbr_alive + s0, n},
                   {st.nbr_other + s0, 4 * n}, {st.nbr_bond + s0, 4 * n}},
                  [&](const std::vector<const char *> &at) {
                      const SlotsIn in{f64(at[0]), f64(at[1]), u8(at[2]), u32(at[3]), u32(at[4])};
                      kSlotsIn<R><<<reorderGrid(n), kThreads, 0, stream>>>(dev.nbr, dev.nbr_other, dev.nbr_bond, in,
                                                                           s0, n, N);
                  });
        }
        const BondSet<R> out = B ? bondsAt(staged) : BondSet<R>{};
        const std::size_t per_bond = (kStage - 19 * 256) / 164;
        for (std::size_t j0 = 0; j0 < B; j0 += per_bond) {
            const std::size_t n = std::min<std::size_t>(per_bond, B - j0);
            chunk({{st.bond_a + j0, 4 * n}, {st.bond_b + j0, 4 * n}, {st.bond_slot_a + j0, 4 * n},
                   {st.bond_slot_b + j0, 4 * n}, {st.alive + j0, n}, {st.failure_mode + j0, n},
                   {last_a.data() + j0, n}, {last_b.data() + j0, n}, {st.rest_length_sq_minus + j0, 8 * n},
                   {st.rest_length + j0, 8 * n}, {st.rest_edge + 3 * j0, 24 * n}, {st.compliance + j0, 8 * n},
                   {st.prev_tensile + j0, 8 * n}, {st.prev_compressive + j0, 8 * n}, {st.prev_shear + j0, 8 * n},
                   {st.damage + j0, 8 * n}, {st.threshold + 6 * j0, 48 * n}, {st.plastic_extension + j0, 8 * n},
                   {st.plastic_strain + j0, 8 * n}},
                  [&](const std::vector<const char *> &at) {
                      const BondsIn in{u32(at[0]), u32(at[1]), u32(at[2]), u32(at[3]), u8(at[4]), u8(at[5]),
                                       u8(at[6]), u8(at[7]), f64(at[8]), f64(at[9]), f64(at[10]), f64(at[11]),
                                       f64(at[12]), f64(at[13]), f64(at[14]), f64(at[15]), f64(at[16]),
                                       f64(at[17]), f64(at[18])};
                      kBondsIn<R><<<reorderGrid(n), kThreads, 0, stream>>>(out, in, j0, n, flowed);
                  });
        }
        // The small arrays, and every node dirty: the first substep restarts in full.
        copySegments({{dev.dev2sched, dev2sched.data(), sizeof(std::uint32_t) * B},
                      {dev.isolated, isolated.data(), sizeof(std::uint32_t) * isolated.size()},
                      {dev.node_block_begin, sched.node_block_begin.data(),
                       sizeof(std::uint32_t) * (sched.block_count + 1)},
                      {dev.level_begin, level_begin_.data(), sizeof(std::uint32_t) * level_begin_.size()},
                      {dev.sphere, &sphere0, sizeof(sphere0)}},
                     cudaMemcpyHostToDevice, crew.get());
        check(cudaMemsetAsync(dev.dirty, 1, N, stream), "memset");
        check(cudaMemsetAsync(dev.dirty + N, 0, 4, stream), "memset");
        check(cudaMemcpyAsync(&flowed_host_, flowed, sizeof(unsigned), cudaMemcpyDeviceToHost, stream), "copy");
        check(cudaFreeAsync(stage, stream), "device free");
        check(cudaStreamSynchronize(stream), "upload");
        plastic_state = flowed_host_ != 0;
        cudaEventDestroy(used[0]);
        cudaEventDestroy(used[1]);
    }

    // setExternalForces (ExternalLoads.hpp:28-50): validated in full before
    // anything changes, so an invalid replacement leaves the old load intact.
    void setExternalForces(const double *forces, std::uint64_t count, std::uint64_t substeps, cudaStream_t stream) {
        if (count == 0) {
            if (substeps != 0) invalid("empty external load needs zero substeps");
            ext_count = 0;
            ext_remaining = 0;
            wrench_count = 0;
            ext_dirty = true;
            return;
        }
        if (count != N || substeps == 0 || !forces)
            invalid("external load needs one force per node and a finite nonzero span");
        std::vector<Q4<R>> applied(N, Q4<R>{R(0), R(0), R(0), R(0)});
        std::vector<std::uint32_t> nodes;
        for (std::uint32_t i = 0; i < N; ++i) {
            const double fx = forces[3 * i], fy = forces[3 * i + 1], fz = forces[3 * i + 2];
            const R cx = R(fx), cy = R(fy), cz = R(fz);
            if (!std::isfinite(fx) || !std::isfinite(fy) || !std::isfinite(fz) || !std::isfinite(std::hypot(fx, fy, fz)) ||
                !std::isfinite(cx) || !std::isfinite(cy) || !std::isfinite(cz))
                invalid("external force is not finite in backend precision");
            if (fx == 0 && fy == 0 && fz == 0) continue;
            if (!(mass[i] > 0) || !(inv_mass[i] > 0) || !std::isfinite(mass[i]) || !std::isfinite(inv_mass[i]))
                invalid("external force needs a finite positive movable node mass");
            applied[i] = {cx, cy, cz, R(1)};
            nodes.push_back(i);
        }
        ensureLoadBuffers();
        gbl::upload(ext_force, applied, stream);
        uploadRaw(ext_req, forces, 3 * static_cast<std::size_t>(N), stream);
        gbl::upload(ext_nodes, nodes, stream);
        check(cudaStreamSynchronize(stream), "external load");
        ext_count = static_cast<std::uint32_t>(nodes.size());
        ext_remaining = nodes.empty() ? 0 : substeps;
        wrench_count = 0; // forces replace any wrenches
        ext_dirty = true;
    }

    // Loads and source ledgers cleared (an upload; a new control block).
    void clearSources() {
        wrench_count = 0;
        source_names.clear();
        if (source_dev) check(cudaMemset(source_dev, 0, sizeof(SourceSlot) * source_cap), "clear");
    }

    void ensureLoadBuffers() {
        if (ext_force) return;
        check(cudaMalloc(&ext_force, sizeof(Q4<R>) * N), "device allocation");
        check(cudaMalloc(&ext_req, sizeof(double) * 3 * N), "device allocation");
        check(cudaMalloc(&ext_contrib, sizeof(double) * 13 * N), "device allocation");
        check(cudaMalloc(&ext_nodes, sizeof(std::uint32_t) * N), "device allocation");
        dev.ext_force = ext_force; dev.ext_req = ext_req; dev.ext_contrib = ext_contrib; dev.ext_nodes = ext_nodes;
    }

    // setExternalWrenches (ExternalLoads.hpp:52-77): validated in full (the
    // spread from the current geometry included, on the device) before
    // anything changes, so an invalid replacement leaves the old load intact.
    void setExternalWrenches(const gbl_external_wrench *ws, std::uint64_t count, std::uint64_t substeps,
                             cudaStream_t stream) {
        if (count == 0) {
            if (substeps != 0) invalid("empty external load needs zero substeps");
            ext_count = 0;
            ext_remaining = 0;
            wrench_count = 0;
            ext_dirty = true;
            return;
        }
        if (!ws) invalid("external wrench needs its wrenches");
        if (substeps == 0) invalid("external wrench needs a finite nonzero span");
        struct Staged {
            std::string source;
            std::vector<std::uint32_t> nodes;
            double point[3], force[3], torque[3];
        };
        auto finite3 = [](const double *v) { return std::isfinite(v[0]) && std::isfinite(v[1]) && std::isfinite(v[2]); };
        std::vector<Staged> staged(count);
        std::set<std::string> names;
        std::vector<std::uint8_t> used(N, 0);
        for (std::uint64_t k = 0; k < count; ++k) {
            const gbl_external_wrench &in = ws[k];
            Staged &w = staged[k];
            if (in.source) w.source = in.source;
            if (w.source.empty() || !names.insert(w.source).second || in.node_count == 0 || !in.nodes)
                invalid("external wrench needs distinct named nonempty regions");
            if (!finite3(in.point_world_m) || !finite3(in.force_n) || !finite3(in.torque_n_m) ||
                !std::isfinite(std::hypot(in.force_n[0], in.force_n[1], in.force_n[2])) ||
                !std::isfinite(std::hypot(in.torque_n_m[0], in.torque_n_m[1], in.torque_n_m[2])))
                invalid("external wrench must be finite");
            w.nodes.assign(in.nodes, in.nodes + in.node_count);
            std::sort(w.nodes.begin(), w.nodes.end());
            for (const std::uint32_t i : w.nodes) {
                if (i >= N || used[i]) invalid("external wrench nodes repeat, overlap or exceed the lattice");
                used[i] = 1;
            }
            std::memcpy(w.point, in.point_world_m, sizeof(w.point));
            std::memcpy(w.force, in.force_n, sizeof(w.force));
            std::memcpy(w.torque, in.torque_n_m, sizeof(w.torque));
        }
        std::sort(staged.begin(), staged.end(), [](const Staged &a, const Staged &b) { return a.source < b.source; });
        staged.erase(std::remove_if(staged.begin(), staged.end(), [](const Staged &w) {
            return w.force[0] == 0 && w.force[1] == 0 && w.force[2] == 0 && w.torque[0] == 0 && w.torque[1] == 0 &&
                   w.torque[2] == 0;
        }), staged.end());
        std::vector<std::uint32_t> list;
        std::vector<WrenchDev> descs;
        std::vector<std::string> names_after = source_names;
        for (const Staged &w : staged) {
            for (const std::uint32_t i : w.nodes)
                if (!(mass[i] > 0) || !(inv_mass[i] > 0) || !std::isfinite(mass[i]) || !std::isfinite(inv_mass[i]))
                    invalid("external wrench needs finite movable node masses");
            WrenchDev d{};
            d.begin = static_cast<std::uint32_t>(list.size());
            list.insert(list.end(), w.nodes.begin(), w.nodes.end());
            d.end = static_cast<std::uint32_t>(list.size());
            const auto at = std::find(names_after.begin(), names_after.end(), w.source);
            d.slot = static_cast<std::uint32_t>(at - names_after.begin());
            if (at == names_after.end()) names_after.push_back(w.source);
            std::memcpy(d.point, w.point, sizeof(d.point));
            std::memcpy(d.force, w.force, sizeof(d.force));
            std::memcpy(d.torque, w.torque, sizeof(d.torque));
            descs.push_back(d);
        }
        if (!descs.empty()) {
            // The spread at the current geometry, checked on the device (in
            // buffers of its own: the load in place stays untouched).
            struct Temp {
                void *p = nullptr;
                ~Temp() { if (p) cudaFree(p); }
            } wd, ld, verdict;
            check(cudaMalloc(&wd.p, sizeof(WrenchDev) * descs.size()), "device allocation");
            check(cudaMalloc(&ld.p, sizeof(std::uint32_t) * list.size()), "device allocation");
            check(cudaMalloc(&verdict.p, sizeof(unsigned)), "device allocation");
            gbl::upload(static_cast<WrenchDev *>(wd.p), descs, stream);
            gbl::upload(static_cast<std::uint32_t *>(ld.p), list, stream);
            check(cudaMemsetAsync(verdict.p, 0, sizeof(unsigned), stream), "clear");
            kWrench<R><<<static_cast<unsigned>(descs.size()), kWrenchThreads, 0, stream>>>(
                dev, static_cast<const WrenchDev *>(wd.p), static_cast<const std::uint32_t *>(ld.p),
                static_cast<unsigned *>(verdict.p), 0);
            check(cudaGetLastError(), "kernel launch");
            unsigned bad = 0;
            check(cudaMemcpyAsync(&bad, verdict.p, sizeof(unsigned), cudaMemcpyDeviceToHost, stream), "copy");
            check(cudaStreamSynchronize(stream), "external wrench");
            if (bad)
                invalid("external wrench cannot be spread over its nodes at the current geometry (torque, "
                        "resultant or node force not representable)");
        }
        ensureLoadBuffers();
        if (descs.size() > wrench_cap) {
            if (wrench_dev) cudaFree(wrench_dev);
            wrench_cap = static_cast<std::uint32_t>(descs.size());
            check(cudaMalloc(&wrench_dev, sizeof(WrenchDev) * wrench_cap), "device allocation");
            dev.wrench = wrench_dev;
        }
        if (names_after.size() > source_cap) {
            const std::size_t cap = std::max<std::size_t>(names_after.size(), 2 * source_cap);
            SourceSlot *grown = nullptr;
            check(cudaMalloc(&grown, sizeof(SourceSlot) * cap), "device allocation");
            check(cudaMemsetAsync(grown, 0, sizeof(SourceSlot) * cap, stream), "clear");
            if (source_dev) {
                check(cudaMemcpyAsync(grown, source_dev, sizeof(SourceSlot) * source_cap, cudaMemcpyDeviceToDevice,
                                      stream), "copy");
                check(cudaStreamSynchronize(stream), "copy");
                cudaFree(source_dev);
            }
            source_dev = grown;
            source_cap = cap;
            dev.sources = source_dev;
        }
        check(cudaMemsetAsync(ext_force, 0, sizeof(Q4<R>) * N, stream), "clear"); // the kick writes the wrench nodes
        if (!descs.empty()) {
            gbl::upload(wrench_dev, descs, stream);
            gbl::upload(ext_nodes, list, stream);
        }
        check(cudaStreamSynchronize(stream), "external wrench");
        source_names = std::move(names_after);
        wrench_count = static_cast<std::uint32_t>(descs.size());
        ext_count = static_cast<std::uint32_t>(list.size());
        ext_remaining = list.empty() ? 0 : substeps;
        ext_dirty = true;
    }

    // RunStatus::external_sources: every source kicked since upload, in the
    // order of its first kick (ExternalLoads.hpp:131-140).
    std::vector<std::pair<std::string, LoadLedger>> sources() const {
        std::vector<std::pair<std::string, LoadLedger>> out;
        if (source_names.empty()) return out;
        std::vector<SourceSlot> slots(source_names.size());
        check(cudaMemcpy(slots.data(), source_dev, sizeof(SourceSlot) * slots.size(), cudaMemcpyDeviceToHost), "copy");
        std::vector<std::size_t> kicked;
        for (std::size_t k = 0; k < slots.size(); ++k)
            if (slots[k].load.steps) kicked.push_back(k);
        std::sort(kicked.begin(), kicked.end(),
                  [&](std::size_t a, std::size_t b) { return slots[a].order < slots[b].order; });
        for (const std::size_t k : kicked) out.emplace_back(source_names[k], slots[k].load);
        return out;
    }

    // The device arrays a download needs, raw, into `raw` (its buffers reused
    // when large enough).
    // The state's layout of this lattice's arrays, written by the device into
    // a new buffer on `stream` (the caller synchronises and frees it).
    StateOut stateOut(cudaStream_t stream) const {
        StateOut out;
        out.N = N;
        out.B = B;
        const std::size_t n3 = 3 * static_cast<std::size_t>(N) * sizeof(double), b = B;
        auto round = [](std::size_t x) { return (x + 255) & ~std::size_t(255); };
        const std::size_t parts[11] = {round(n3), round(n3), round(n3), round(b), round(b), round(8 * b), round(8 * b),
                                       round(8 * b), round(8 * b), round(8 * b), round(8 * b)};
        for (std::size_t q : parts) out.bytes += q;
        check(cudaMallocAsync(&out.base, out.bytes ? out.bytes : 256, stream), "device allocation");
        char *at[11];
        for (std::size_t q = 0, off = 0; q < 11; off += parts[q], ++q) at[q] = out.base + off;
        out.u = reinterpret_cast<double *>(at[0]);
        out.up = reinterpret_cast<double *>(at[1]);
        out.v = reinterpret_cast<double *>(at[2]);
        out.o = BondsOut{reinterpret_cast<std::uint8_t *>(at[3]), reinterpret_cast<std::uint8_t *>(at[4]),
                         reinterpret_cast<double *>(at[5]), reinterpret_cast<double *>(at[6]),
                         reinterpret_cast<double *>(at[7]), reinterpret_cast<double *>(at[8]),
                         reinterpret_cast<double *>(at[9]), reinterpret_cast<double *>(at[10])};
        if (N) kNodesOut<R><<<reorderGrid(N), kThreads, 0, stream>>>(out.u, out.up, out.v, dev.u, dev.up, dev.v, N);
        if (B) kBondsOut<R><<<reorderGrid(B), kThreads, 0, stream>>>(out.o, bonds(), dev.dev2sched, B);
        check(cudaGetLastError(), "kernel launch");
        return out;
    }

    // download (WorkingLattice::toState, LatticeWorking.hpp:126-142): the
    // device writes the state's layout, copied straight into the caller's
    // arrays (which the caller has already touched).
    void download(gbl_state_view &st, gbl_sphere *sphere, cudaStream_t stream) {
        if (st.node_count != N || st.bond_count != B) invalid("download state does not match the lattice");
        const StateOut out = stateOut(stream);
        check(cudaStreamSynchronize(stream), "download");
        out.copyTo(st);
        check(cudaFreeAsync(out.base, stream), "device free");
        check(cudaStreamSynchronize(stream), "download");
        if (sphere) *sphere = fetchSphere();
    }

    gbl_sphere fetchSphere() const {
        Sphere<R> sp{};
        check(cudaMemcpy(&sp, dev.sphere, sizeof(sp), cudaMemcpyDeviceToHost), "copy");
        gbl_sphere o{};
        o.center[0] = sp.center.x; o.center[1] = sp.center.y; o.center[2] = sp.center.z;
        o.velocity[0] = sp.velocity.x; o.velocity[1] = sp.velocity.y; o.velocity[2] = sp.velocity.z;
        o.angular_velocity[0] = sp.angular.x; o.angular_velocity[1] = sp.angular.y; o.angular_velocity[2] = sp.angular.z;
        o.radius = sp.radius; o.mass = sp.mass; o.inertia = sp.inertia;
        return o;
    }

    void captureFrame(std::uint64_t step, cudaStream_t stream) {
        Frame f;
        f.step = step;
        f.u.resize(3 * static_cast<std::size_t>(N));
        f.alive.resize(B);
        f.damage.resize(B);
        // Written on the device in the frame's layout, then copied straight in.
        auto round = [](std::size_t x) { return (x + 255) & ~std::size_t(255); };
        const std::size_t nu = 3 * static_cast<std::size_t>(N) * sizeof(float), b = B;
        char *buf = nullptr;
        check(cudaMallocAsync(&buf, round(nu) + round(b) + round(4 * b) + 256, stream), "device allocation");
        float *u = reinterpret_cast<float *>(buf);
        std::uint8_t *alive = reinterpret_cast<std::uint8_t *>(buf + round(nu));
        float *damage = reinterpret_cast<float *>(buf + round(nu) + round(b));
        if (N || B)
            kFrameOut<R><<<reorderGrid(std::max<std::size_t>(N, B)), kThreads, 0, stream>>>(u, alive, damage, dev.u,
                                                                                         bonds(), dev.dev2sched, N, B);
        check(cudaGetLastError(), "kernel launch");
        check(cudaStreamSynchronize(stream), "frame");
        copySegments({{f.u.data(), u, nu}, {f.alive.data(), alive, b}, {f.damage.data(), damage, 4 * b}},
                     cudaMemcpyDeviceToHost);
        check(cudaFreeAsync(buf, stream), "device free");
        f.sphere = fetchSphere();
        frames.push_back(std::move(f));
        ++status.frames_captured;
    }

    void fillStatus(const Ctl &c) {
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
        status.node_contact.contacts = c.node.contacts;
        status.node_contact.pair_tests = c.node.pair_tests;
        status.node_contact.rebuilds = c.node.rebuilds;
        status.node_contact.pairs_listed = c.node.pairs_listed;
        status.node_contact.pair_overflow = c.node.pair_overflow;
        status.node_contact.dissipated_kinetic_energy_j = c.node.dissipated;
        status.node_contact.maximum_overlap_m = c.node.max_overlap;
        status.node_contact.maximum_position_correction_m = c.node.max_correction;
        status.node_contact.momentum_residual_x = c.node.momentum[0];
        status.node_contact.momentum_residual_y = c.node.momentum[1];
        status.node_contact.momentum_residual_z = c.node.momentum[2];
        status.exit_reason = c.exit_reason;
        float f;
        std::memcpy(&f, &c.max_t, 4); status.max_tensile_stretch = f;
        std::memcpy(&f, &c.max_c, 4); status.max_compressive_strain = f;
        std::memcpy(&f, &c.max_s, 4); status.max_shear_strain = f;
        std::memcpy(&f, &c.max_plastic, 4); status.max_plastic_stretch = f;
        status.rank_deficient_nodes = c.rank_deficient;
        status.plastic_work_j = c.plastic_work;
        status.damping_dissipated_j = c.damping_dissipated;
        status.striker_dissipated_j = c.striker_dissipated;
        status.bond_projections = c.projections;
    }
};

// Lattices advanced together, one launch per phase and per sweep level.
//
// Lattices live in slots: a slot's control block, descriptor and work items
// are its own, and lattices enter (admit) and leave (retire) between substeps
// without touching the others, which is what continuous batching needs. The
// work lists and the captured substep graph are rebuilt when the set changes.
template <class R> class Engine {
    static constexpr bool kDirect = std::is_same<R, double>::value;
    static constexpr unsigned kSphereSlab = sphereSlabBytes<R>();

public:
    Engine() {
        // Two staging buffers for the contact pass where the device's shared
        // memory per block holds them, else one.
        int device = 0, optin = 0;
        check(cudaGetDevice(&device), "device");
        // Lattices are allocated from the device's pool, stream-ordered. Up to
        // 16 GiB that lattices free stays in the pool for the next upload or
        // admission instead of going back to the driver at the next
        // synchronisation (re-mapping gigabytes costs a large share of an
        // upload otherwise); beyond that it is released, so allocations
        // outside the pool still find the device's memory. A property of
        // this process's pool only.
        {
            cudaMemPool_t pool = nullptr;
            check(cudaDeviceGetDefaultMemPool(&pool, device), "memory pool");
            std::uint64_t keep = std::uint64_t(16) << 30;
            check(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep), "memory pool");
        }
        check(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device), "device attribute");
        sphere_buffers_ = 2U * kSphereSlab + 1024U <= static_cast<unsigned>(optin) ? 2U : 1U;
        const int smem = static_cast<int>(sphere_buffers_ * kSphereSlab);
        check(cudaFuncSetAttribute(kSpherePass<R, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem),
              "contact pass shared memory");
        check(cudaFuncSetAttribute(kSpherePass<R, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem),
              "contact pass shared memory");
        allowStagedSharedMemory();
        check(cudaStreamCreateWithFlags(&own_stream_, cudaStreamNonBlocking), "stream");
        check(cudaStreamCreateWithFlags(&side_, cudaStreamNonBlocking), "stream");
        check(cudaStreamCreateWithFlags(&loads_, cudaStreamNonBlocking), "stream");
        check(cudaEventCreateWithFlags(&fork_, cudaEventDisableTiming), "event");
        check(cudaEventCreateWithFlags(&join_, cudaEventDisableTiming), "event");
        check(cudaEventCreateWithFlags(&load_fork_, cudaEventDisableTiming), "event");
        check(cudaEventCreateWithFlags(&load_join_, cudaEventDisableTiming), "event");
        stream_ = own_stream_;
        check(cudaEventCreate(&ev0_), "event");
        check(cudaEventCreate(&ev1_), "event");
        check(cudaMallocHost(&running_host_, sizeof(unsigned)), "pinned allocation");
        check(cudaMalloc(&running_, sizeof(unsigned)), "device allocation");
    }
    Engine(const Engine &) = delete;
    Engine &operator=(const Engine &) = delete;
    ~Engine() {
        dropGraph();
        slots_.clear();
        if (ctl_) cudaFree(ctl_);
        if (table_) cudaFree(table_);
        if (work_) cudaFree(work_);
        if (running_) cudaFree(running_);
        if (running_host_) cudaFreeHost(running_host_);
        cudaEventDestroy(ev0_);
        cudaEventDestroy(ev1_);
        cudaEventDestroy(fork_);
        cudaEventDestroy(join_);
        cudaEventDestroy(load_fork_);
        cudaEventDestroy(load_join_);
        cudaStreamDestroy(side_);
        cudaStreamDestroy(loads_);
        cudaStreamDestroy(own_stream_);
    }

    // Slots in use, and the largest slot index + 1.
    [[nodiscard]] std::size_t size() const { return active_.size(); }
    [[nodiscard]] std::size_t slots() const { return slots_.size(); }
    [[nodiscard]] bool occupied(std::size_t k) const { return k < slots_.size() && slots_[k] != nullptr; }
    Resident<R> &lattice(std::size_t k) {
        if (!occupied(k)) invalid("lattice index out of range");
        return *slots_[k];
    }
    [[nodiscard]] const Ctl &control(std::size_t k) const { return ctl_host_.at(k); }
    [[nodiscard]] cudaStream_t stream() const { return stream_; }
    [[nodiscard]] bool settled() const { return ready_; }
    void setStream(cudaStream_t s) {
        stream_ = s ? s : own_stream_;
        dropGraph();
    }

    void clear() {
        dropGraph();
        slots_.clear();
        active_.clear();
        ready_ = false;
        dirty_ = true;
    }

    // Upload one lattice into the first free slot. Before settle() this only
    // uploads; after it the lattice is admitted: a fresh control block (a new
    // RunStatus) with `step_limit` substeps to run (0: no limit).
    std::size_t add(const Schedule &sched, const gbl_state_view &st, const gbl_sphere &sphere,
                    std::uint64_t step_limit = 0) {
        return place(prepare(sched, st, sphere, false), step_limit);
    }

    // The host half of add: no CUDA call and no engine state, so any number
    // of threads may prepare lattices while the engine runs. With `image`
    // the device layout is written to a host image and the caller's state is
    // not read again; without, the lattice converts on the device from the
    // caller's arrays when it is placed.
    static std::unique_ptr<Resident<R>> prepare(const Schedule &sched, const gbl_state_view &st,
                                                const gbl_sphere &sphere, bool image = true) {
        auto r = std::make_unique<Resident<R>>(sched);
        r->prepare(st, sphere, image);
        return r;
    }

    // The device half of add: a prepared lattice takes the first free slot.
    std::size_t place(std::unique_ptr<Resident<R>> r, std::uint64_t step_limit = 0) {
        std::lock_guard<std::mutex> lock(place_mutex_);
        r->commit(stream_);
        std::size_t k = 0;
        while (k < slots_.size() && slots_[k]) ++k;
        if (k == slots_.size()) slots_.emplace_back();
        slots_[k] = std::move(r);
        listActive();
        dirty_ = true;
        if (ready_) {
            growControl(slots_.size());
            if (slots_[k]->plastic_state && !plastic_) {
                plastic_ = true;
                dropGraph();
            }
            if (S_.nc_mode != 0) slots_[k]->ensureContact();
            initControl(k, step_limit);
            pushDescriptor(k);
            check(cudaStreamSynchronize(stream_), "admit");
        }
        return k;
    }

    // Take a lattice out (its device memory is freed); the others go on.
    void retire(std::size_t k) {
        if (!occupied(k)) invalid("lattice index out of range");
        check(cudaStreamSynchronize(stream_), "retire");
        slots_[k].reset();
        while (!slots_.empty() && !slots_.back()) slots_.pop_back();
        listActive();
        dirty_ = true;
    }

    // The settings every lattice shares, and a fresh control block (reset:
    // a new RunStatus) for every lattice present.
    void settle(const gbl_step_settings &set) {
        validate(set);
        if (active_.empty()) invalid("the batch holds no lattice");
        dropGraph();
        S_ = convertSettings(set);
        plastic_ = S_.yield_stretch > R(0);
        for (auto k : active_) plastic_ = plastic_ || slots_[k]->plastic_state;
        if (S_.nc_mode != 0)
            for (auto k : active_) slots_[k]->ensureContact();
        growControl(slots_.size());
        for (auto k : active_) initControl(k, 0);
        for (auto k : active_) pushDescriptor(k);
        check(cudaStreamSynchronize(stream_), "settle");
        ready_ = true;
        dirty_ = true;
    }

    // A settle() without lattices: the settings of a server that admits later.
    void configure(const gbl_step_settings &set) {
        validate(set);
        dropGraph();
        S_ = convertSettings(set);
        plastic_ = S_.yield_stretch > R(0);
        for (auto k : active_) plastic_ = plastic_ || slots_[k]->plastic_state;
        if (S_.nc_mode != 0) {
            for (auto k : active_) {
                slots_[k]->ensureContact();
                pushDescriptor(k);
            }
            check(cudaStreamSynchronize(stream_), "descriptors");
        }
        ready_ = true;
        dirty_ = true;
    }

    void setExternalForces(std::size_t k, const double *forces, std::uint64_t count, std::uint64_t substeps) {
        requireReady();
        Resident<R> &l = lattice(k);
        const bool had = l.ext_force != nullptr;
        l.setExternalForces(forces, count, substeps, stream_);
        if (!had && l.ext_force) {
            pushDescriptor(k); // the descriptor now points at the load buffers
            check(cudaStreamSynchronize(stream_), "descriptor");
            dropGraph();       // a single lattice's launches carry the descriptor itself
        }
    }

    // External wrenches on lattice k (its spread is launched for it alone,
    // before the shared kick).
    void setExternalWrenches(std::size_t k, const gbl_external_wrench *ws, std::uint64_t count,
                             std::uint64_t substeps) {
        requireReady();
        Resident<R> &l = lattice(k);
        const void *before[3] = {l.ext_force, l.wrench_dev, l.source_dev};
        l.setExternalWrenches(ws, count, substeps, stream_);
        if (before[0] != l.ext_force || before[1] != l.wrench_dev || before[2] != l.source_dev) {
            pushDescriptor(k);
            check(cudaStreamSynchronize(stream_), "descriptor");
            dirty_ = true; // the wrench slots' work items and the graph
        }
    }

    // run (CpuLatticeBackend.cpp:255-304) for every lattice with one control;
    // a lattice whose step limit is spent stays stopped.
    void run(const gbl_run_control &control) {
        requireReady();
        const auto start = std::chrono::steady_clock::now();
        if (active_.empty()) return;
        pullControl();
        unsigned running = 0;
        for (auto k : active_) {
            Ctl &c = ctl_host_[k];
            Resident<R> &l = *slots_[k];
            const bool spent = c.step_limit != 0 && c.total_steps >= c.step_limit;
            c.stop = spent ? 1U : 0U;
            if (spent) c.exit_reason = 3;
            else c.exit_reason = 0;
            running += spent ? 0U : 1U;
            c.quiet_steps = control.quiet_steps; c.min_steps = control.min_steps;
            c.no_failure_steps = control.no_failure_steps; c.energy_flat_steps = control.energy_flat_steps;
            c.calm_steps = control.calm_steps; c.energy_flat_fraction = control.energy_flat_fraction;
            c.calm_damage_margin = control.calm_damage_margin; c.removable_energy = control.removable_energy_j;
            if (l.ext_dirty) {
                c.ext_count = l.ext_count;
                c.wrench_count = l.wrench_count;
                c.loads_remaining = l.ext_remaining;
                l.ext_dirty = false;
            }
        }
        pushControl();
        *running_host_ = running;
        check(cudaMemcpyAsync(running_, running_host_, sizeof(unsigned), cudaMemcpyHostToDevice, stream_), "copy");
        std::vector<std::uint64_t> before(slots_.size(), 0);
        for (auto k : active_) before[k] = ctl_host_[k].total_steps;
        prepare();
        std::uint64_t chunk = control.steps_per_launch ? control.steps_per_launch : control.max_steps;
        if (control.abandon && chunk > 64) chunk = 64;
        const bool capture = control.capture_stride != 0;
        std::uint64_t launched = 0;
        bool abandoned = false;
        check(cudaEventRecord(ev0_, stream_), "event");
        while (running && launched < control.max_steps) {
            if (control.abandon && *control.abandon) { abandoned = true; break; }
            const std::uint64_t n = std::min(chunk, control.max_steps - launched);
            bool halted = false;
            for (std::uint64_t s = 0; s < n; ++s) {
                if (capture) {
                    bool synced = false;
                    for (auto k : active_) {
                        const std::uint64_t step = before[k] + launched + s;
                        Resident<R> &l = *slots_[k];
                        if (step % control.capture_stride != 0 || l.status.frames_captured >= control.max_frames) continue;
                        if (!synced) {
                            if (allStopped()) { halted = true; break; }
                            synced = true;
                        }
                        l.captureFrame(step, stream_);
                    }
                    if (halted) break;
                }
                check(cudaGraphLaunch(exec_, stream_), "graph launch");
            }
            launched += n;
            for (auto k : active_) ++slots_[k]->status.launches;
            if (halted || allStopped()) break;
        }
        check(cudaEventRecord(ev1_, stream_), "event");
        check(cudaStreamSynchronize(stream_), "lattice run");
        float ms = 0;
        cudaEventElapsedTime(&ms, ev0_, ev1_);
        pullControl();
        bool overflowed = false, wrenched = false, stage_timeout = false;
        for (auto k : active_) {
            Ctl &c = ctl_host_[k];
            Resident<R> &l = *slots_[k];
            l.status.kernel_seconds += ms * 1e-3;
            if (c.error & kErrExternalOverflow) {
                c.error = 0;
                overflowed = true;
            }
            if (c.error & kErrWrench) {
                c.error = 0;
                wrenched = true;
            }
            if (c.error & kErrStageWait) {
                c.error = 0;
                stage_timeout = true;
            }
            l.ext_remaining = c.loads_remaining;
            l.fillStatus(c);
            const std::uint64_t done = c.total_steps - before[k];
            if (abandoned && c.exit_reason == 0) l.status.exit_reason = 7;
            else if (l.status.exit_reason == 0 && done >= control.max_steps) l.status.exit_reason = 3;
            if (c.ffb_count > l.first_failure.size()) {
                l.first_failure.resize(c.ffb_count);
                check(cudaMemcpy(l.first_failure.data(), l.dev.ffb, sizeof(std::uint32_t) * c.ffb_count,
                                 cudaMemcpyDeviceToHost), "copy");
            }
        }
        if (overflowed) {
            pushControl();
            check(cudaStreamSynchronize(stream_), "status");
            overflow("external force kick exceeds backend precision");
        }
        if (wrenched) {
            pushControl();
            check(cudaStreamSynchronize(stream_), "status");
            invalid("external wrench cannot be spread over its nodes at the current geometry (torque, resultant "
                    "or node force not representable)");
        }
        if (stage_timeout) {
            pushControl();
            check(cudaStreamSynchronize(stream_), "status");
            runtime("the staged sweep's bulk copy into shared memory did not complete within its bounded wait");
        }
        const double wall = std::chrono::duration<double>(std::chrono::steady_clock::now() - start).count();
        for (auto k : active_) slots_[k]->status.wall_seconds += wall;
    }

    // Per-phase device time: the substep enqueued outside the graph, with an
    // event between phases (phase names of FastLattice.cpp:22-27).
    void profile(std::uint64_t substeps, double *phase_ms) {
        requireReady();
        for (unsigned p = 0; p < GBL_PHASE_COUNT; ++p) phase_ms[p] = 0.0;
        if (active_.empty()) return;
        armUncaptured();
        std::vector<cudaEvent_t> evs;
        std::vector<unsigned> ids;
        auto mark = [&](unsigned phase) {
            cudaEvent_t e;
            check(cudaEventCreate(&e), "event");
            check(cudaEventRecord(e, stream_), "event");
            evs.push_back(e);
            ids.push_back(phase);
        };
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
        settleUncaptured(phase_ms);
    }

    // The phase-diff debug mode: one substep of every lattice, enqueued phase
    // by phase outside the graph, with lattice `k`'s state downloaded after
    // each phase whose bit is set in `mask` -- into views[i] for the i-th set
    // bit, the last occurrence of a phase that repeats (the sweep marks its
    // phases once per iteration). The state arrays and the sphere are those a
    // download returns; the run then carries on as a normal substep.
    void debugSubstep(std::size_t k, std::uint32_t mask, gbl_state_view *views, gbl_sphere *spheres) {
        requireReady();
        if (!occupied(k)) invalid("unknown lattice");
        armUncaptured();
        auto mark = [&](unsigned phase) {
            if (phase >= 32 || !((mask >> phase) & 1U)) return;
            const unsigned i = static_cast<unsigned>(__builtin_popcount(mask & ((1U << phase) - 1U)));
            check(cudaDeviceSynchronize(), "phase snapshot");
            lattice(k).download(views[i], spheres ? &spheres[i] : nullptr, stream_);
        };
        enqueueSubstep(mark);
        check(cudaDeviceSynchronize(), "phase snapshot");
        std::vector<double> none(GBL_PHASE_COUNT, 0.0);
        settleUncaptured(none.data());
    }

private:
    // Before substeps enqueued outside the graph: the control blocks as a run
    // sets them (exit rules off, spent lattices stopped, loads armed).
    void armUncaptured() {
        pullControl();
        unsigned running = 0;
        for (auto k : active_) {
            Ctl &c = ctl_host_[k];
            const bool spent = c.step_limit != 0 && c.total_steps >= c.step_limit;
            c.stop = spent ? 1U : 0U;
            c.exit_reason = spent ? 3U : 0U;
            running += spent ? 0U : 1U;
            c.quiet_steps = c.min_steps = c.no_failure_steps = c.energy_flat_steps = c.calm_steps = 0;
            c.removable_energy = 0;
            Resident<R> &l = *slots_[k];
            if (l.ext_dirty) {
                c.ext_count = l.ext_count;
                c.wrench_count = l.wrench_count;
                c.loads_remaining = l.ext_remaining;
                l.ext_dirty = false;
            }
        }
        pushControl();
        *running_host_ = running;
        check(cudaMemcpyAsync(running_, running_host_, sizeof(unsigned), cudaMemcpyHostToDevice, stream_), "copy");
        prepare();
    }

    // After them: the statuses read back, the phase times added.
    void settleUncaptured(const double *phase_ms) {
        pullControl();
        for (auto k : active_) {
            slots_[k]->ext_remaining = ctl_host_[k].loads_remaining;
            slots_[k]->fillStatus(ctl_host_[k]);
            for (unsigned p = 0; p < GBL_PHASE_COUNT; ++p) slots_[k]->status.phase_seconds[p] += phase_ms[p] * 1e-3;
        }
    }

public:

    // The batch autotuner: times the projection sweep of the lattices present
    // under candidate launch shapes and keeps the fastest. The sweep writes
    // positions (saved here and restored after), multipliers (rewritten by
    // the first iteration of every sweep) and support contact flags (cleared
    // by every kick), so the lattices' state is unchanged.
    gbl_tuning tune() {
        requireReady();
        if (active_.empty()) invalid("the batch holds no lattice");
        dropGraph();
        std::size_t total = 0;
        for (auto k : active_) total += sizeof(Q4<R>) * slots_[k]->N;
        void *saved = nullptr;
        check(cudaMallocAsync(&saved, total ? total : 256, stream_), "device allocation");
        auto positions = [&](bool save) {
            std::size_t off = 0;
            for (auto k : active_) {
                const std::size_t n = sizeof(Q4<R>) * slots_[k]->N;
                char *keep = static_cast<char *>(saved) + off;
                void *u = slots_[k]->dev.u;
                if (n) check(cudaMemcpyAsync(save ? keep : u, save ? u : keep, n, cudaMemcpyDeviceToDevice, stream_), "copy");
                off += n;
            }
        };
        positions(true);
        cudaEvent_t t0 = nullptr, t1 = nullptr;
        check(cudaEventCreate(&t0), "event");
        check(cudaEventCreate(&t1), "event");
        auto timeShape = [&](const Shape &sh) {
            shape_ = sh;
            buildWork();
            cudaGraph_t g = nullptr;
            cudaGraphExec_t e = nullptr;
            check(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal), "graph capture");
            if (many_) enqueueSweep<true>([](unsigned) {});
            else enqueueSweep<false>([](unsigned) {});
            check(cudaStreamEndCapture(stream_, &g), "graph capture");
            check(cudaGraphInstantiate(&e, g, 0), "graph instantiate");
            check(cudaGraphLaunch(e, stream_), "graph launch");
            float best = 0.0F;
            for (int rep = 0; rep < 3; ++rep) {
                check(cudaEventRecord(t0, stream_), "event");
                check(cudaGraphLaunch(e, stream_), "graph launch");
                check(cudaEventRecord(t1, stream_), "event");
                check(cudaEventSynchronize(t1), "tune");
                float ms = 0.0F;
                check(cudaEventElapsedTime(&ms, t0, t1), "event");
                best = rep == 0 ? ms : std::min(best, ms);
            }
            cudaGraphExecDestroy(e);
            cudaGraphDestroy(g);
            return static_cast<double>(best);
        };
        const Shape fallback{};
        gbl_tuning out{};
        Shape best = fallback;
        double best_ms = timeShape(fallback);
        out.default_ms = best_ms;
        out.candidates = 1;
        if (many_) {
            // The one-CTA sweep's CTA size and reach together, then the group size.
            for (unsigned threads : {256U, 512U, 1024U})
                for (std::uint32_t reach : {1U << 16, 1U << 17, 1U << 18, 1U << 19}) {
                    Shape sh = best;
                    sh.sweep_threads = threads;
                    sh.whole_max_bonds = reach;
                    if (sh.sweep_threads == fallback.sweep_threads && sh.whole_max_bonds == fallback.whole_max_bonds)
                        continue;
                    const double ms = timeShape(sh);
                    ++out.candidates;
                    if (ms < best_ms) { best_ms = ms; best = sh; }
                }
            const Shape base = best;
            for (std::size_t mb : {16U, 32U, 96U, 192U}) {
                Shape sh = base;
                sh.group_bytes = mb << 20;
                const double ms = timeShape(sh);
                ++out.candidates;
                if (ms < best_ms) { best_ms = ms; best = sh; }
            }
            // The shared-memory staged sweep for the small whole lattices.
            if (!kDirect) {
                const Shape kept = best;
                for (std::uint32_t nodes : {kStagedMaxNodes / 2, kStagedMaxNodes}) {
                    Shape sh = kept;
                    sh.staged_max_nodes = nodes;
                    const double ms = timeShape(sh);
                    ++out.candidates;
                    if (ms < best_ms) { best_ms = ms; best = sh; }
                }
            }
        }
        positions(false);
        check(cudaFreeAsync(saved, stream_), "device free");
        check(cudaStreamSynchronize(stream_), "tune");
        cudaEventDestroy(t0);
        cudaEventDestroy(t1);
        shape_ = best;
        dirty_ = true;
        out.sweep_threads = best.sweep_threads;
        out.whole_max_bonds = best.whole_max_bonds;
        out.group_bytes = best.group_bytes;
        out.staged_max_nodes = best.staged_max_nodes;
        out.sweep_ms = best_ms;
        return out;
    }

    void setShape(const gbl_tuning &t) {
        if (t.sweep_threads && t.sweep_threads != 256 && t.sweep_threads != 512 && t.sweep_threads != 1024)
            invalid("the one-CTA sweep takes 256, 512 or 1024 threads");
        if (t.whole_max_bonds > (1U << 24)) invalid("the one-CTA sweep takes lattices of at most 2^24 bonds");
        if (t.sweep_threads) shape_.sweep_threads = t.sweep_threads;
        if (t.whole_max_bonds) shape_.whole_max_bonds = t.whole_max_bonds;
        if (t.group_bytes) shape_.group_bytes = t.group_bytes;
        // staged_max_nodes: 0 keeps the current value, ~0 turns staging off.
        if (t.staged_max_nodes != ~0U && t.staged_max_nodes > kStagedMaxNodes)
            invalid("the staged sweep holds at most 14,336 nodes in shared memory");
        if (t.staged_max_nodes == ~0U) shape_.staged_max_nodes = 0;
        else if (t.staged_max_nodes) shape_.staged_max_nodes = t.staged_max_nodes;
        dirty_ = true;
    }

    std::uint64_t kernelsPerSubstep() {
        requireReady();
        if (active_.empty()) return 0;
        prepare();
        std::size_t n = 0;
        check(cudaGraphGetNodes(graph_, nullptr, &n), "graph nodes");
        return n;
    }

    void download(std::size_t k, gbl_state_view &st, gbl_sphere *sphere) {
        requireReady();
        check(cudaStreamSynchronize(stream_), "download");
        lattice(k).download(st, sphere, stream_);
    }

    static void validate(const gbl_step_settings &s) {
        // The Verlet reference integrator is serial-double only: the reference's
        // parallel lane refuses it the same way (ParallelCpuLatticeBackend.cpp:1380-1381).
        if (s.bond_integrator != 0) invalid("this lattice backend implements the XPBD integrator only");
        if (s.node_contact.mode != 0 &&
            !(2.0 * s.node_contact.radius + s.node_contact.skin > 0.0 &&
              std::isfinite(2.0 * s.node_contact.radius + s.node_contact.skin)))
            invalid("node-to-node contact needs a finite positive cutoff (2 radius + skin)");
        if ((s.direct_arithmetic != 0) != kDirect)
            invalid(kDirect ? "the double backend runs the direct (absolute position) arithmetic"
                            : "the float backend runs the displacement arithmetic");
        if (s.plane_count > kPlanes) invalid("at most two support planes");
        for (std::uint32_t p = 0; p < s.plane_count; ++p)
            if (s.planes[p].footprint_count > kFootprints) invalid("at most four footprints per plane");
        if (!(s.dt > 0.0) || !std::isfinite(s.dt)) invalid("lattice step needs a finite positive timestep");
    }

private:
    void requireReady() const {
        if (!ready_) invalid("the lattice backend needs an upload before this call");
    }

    static Settings<R> convertSettings(const gbl_step_settings &s) {
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
        o.nc_mode = s.node_contact.mode;
        o.nc_radius = R(s.node_contact.radius); o.nc_skin = R(s.node_contact.skin);
        o.nc_margin = R(s.node_contact.margin); o.nc_restitution = R(s.node_contact.restitution);
        o.nc_threshold = R(s.node_contact.restitution_speed_threshold);
        o.nc_static = R(s.node_contact.static_friction); o.nc_dynamic = R(s.node_contact.dynamic_friction);
        o.plate_half_thickness = R(s.plate_half_thickness);
        o.audit = s.audit_energy ? 1U : 0U;
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

    void listActive() {
        active_.clear();
        for (std::size_t k = 0; k < slots_.size(); ++k)
            if (slots_[k]) active_.push_back(static_cast<std::uint32_t>(k));
    }

    // Control blocks and descriptors for `need` slots, kept across growth.
    void growControl(std::size_t need) {
        if (need <= cap_) return;
        std::size_t cap = std::max<std::size_t>(cap_ ? cap_ * 2 : 1, need);
        Ctl *ctl = nullptr;
        Dev<R> *table = nullptr;
        check(cudaMalloc(&ctl, sizeof(Ctl) * cap), "device allocation");
        check(cudaMalloc(&table, sizeof(Dev<R>) * cap), "device allocation");
        if (ctl_) {
            check(cudaMemcpyAsync(ctl, ctl_, sizeof(Ctl) * cap_, cudaMemcpyDeviceToDevice, stream_), "copy");
            check(cudaStreamSynchronize(stream_), "copy");
            cudaFree(ctl_);
            cudaFree(table_);
        }
        ctl_ = ctl;
        table_ = table;
        cap_ = cap;
        ctl_host_.resize(cap);
        // Every descriptor points at its control block: all move.
        for (auto k : active_)
            if (k < cap_) {
                slots_[k]->dev.ctl = ctl_ + k;
                pushDescriptor(k);
            }
        check(cudaStreamSynchronize(stream_), "descriptors");
        dropGraph();
        dirty_ = true;
    }

    void initControl(std::size_t k, std::uint64_t step_limit) {
        Ctl c{};
        c.first_failure_step = c.last_failure_step = c.last_energy_gain_step = ~0ULL;
        c.full_restart = 1;
        c.nc_rebuild = 1; // the pair list is built before its first use
        c.energy_flat_fraction = 1.0e-3;
        c.calm_damage_margin = 0.5;
        c.step_limit = step_limit;
        c.live_bonds = slots_[k]->live_bonds;
        ctl_host_[k] = c;
        Resident<R> &l = *slots_[k];
        l.dev.ctl = ctl_ + k;
        l.dev.running = running_;
        l.ext_count = 0;
        l.ext_remaining = 0;
        l.ext_dirty = false;
        l.clearSources();
        l.status = gbl_run_status{};
        l.status.first_failure_step = l.status.last_failure_step = l.status.last_energy_gain_step = ~0ULL;
        l.status.energy_audited = S_.audit ? 1 : 0; // CpuLatticeBackend.cpp:114
        l.first_failure.clear();
        l.frames.clear();
        check(cudaMemcpyAsync(ctl_ + k, &ctl_host_[k], sizeof(Ctl), cudaMemcpyHostToDevice, stream_), "copy");
        check(cudaStreamSynchronize(stream_), "copy");
    }

    void pushDescriptor(std::size_t k) {
        check(cudaMemcpyAsync(table_ + k, &slots_[k]->dev, sizeof(Dev<R>), cudaMemcpyHostToDevice, stream_), "copy");
    }

    // Control blocks of the slots, between the host mirror and the device, in
    // one copy (a free slot's block is read by no kernel).
    void pullControl() {
        if (slots_.empty()) return;
        check(cudaMemcpyAsync(ctl_host_.data(), ctl_, sizeof(Ctl) * slots_.size(), cudaMemcpyDeviceToHost, stream_),
              "copy");
        check(cudaStreamSynchronize(stream_), "status");
    }
    void pushControl() {
        if (slots_.empty()) return;
        check(cudaMemcpyAsync(ctl_, ctl_host_.data(), sizeof(Ctl) * slots_.size(), cudaMemcpyHostToDevice, stream_),
              "copy");
        check(cudaStreamSynchronize(stream_), "status");
    }

    bool allStopped() {
        check(cudaMemcpyAsync(running_host_, running_, sizeof(unsigned), cudaMemcpyDeviceToHost, stream_), "copy");
        check(cudaStreamSynchronize(stream_), "status");
        return *running_host_ == 0;
    }

    // Work lists and graph for the lattices present.
    void prepare() {
        if (dirty_) {
            buildWork();
            dropGraph();
            dirty_ = false;
        }
        if (!exec_) {
            check(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal), "graph capture");
            enqueueSubstep([](unsigned) {});
            check(cudaStreamEndCapture(stream_, &graph_), "graph capture");
            check(cudaGraphInstantiate(&exec_, graph_, 0), "graph instantiate");
        }
    }

    // A launch's items: [first, first + count) of the work array; for a
    // single lattice, the same items as (base, end, per).
    struct Span { std::uint32_t first, count, base, end, per; };

    // A lattice of a batch swept by one CTA (kSweepLattice): small enough to
    // keep its nodes in L2 across its levels, with levels that fit the table.
    bool sweptWhole(const Resident<R> &l) const {
        return l.B > 0 && l.B <= shape_.whole_max_bonds && l.dev.level_count == l.levels.size();
    }

    // Work lists of every phase, one item per CTA, lattices in slot order.
    void buildWork() {
        many_ = active_.size() > 1;
        std::vector<Work> all;
        auto ranges = [&](std::uint32_t k, std::uint32_t begin, std::uint32_t end, std::uint32_t per) {
            for (std::uint32_t b = begin; b < end; b += per) all.push_back({k, b, std::min(end, b + per)});
        };
        // Items of [begin_k, end_k) per lattice in chunks of `per`.
        auto span = [&](auto &&bounds, std::uint32_t per) {
            const std::uint32_t first = static_cast<std::uint32_t>(all.size());
            std::uint32_t b0 = 0, e0 = 0;
            bool lead = true;
            for (auto k : active_) {
                std::uint32_t b = 0, e = 0;
                bounds(*slots_[k], b, e);
                if (lead) { b0 = b; e0 = e; lead = false; }
                ranges(k, b, e, per);
            }
            return Span{first, static_cast<std::uint32_t>(all.size()) - first, b0, e0, per};
        };
        using Res = Resident<R>;
        using U = std::uint32_t;
        nodes_ = span([](const Res &l, U &b, U &e) { b = 0; e = l.N; }, kThreads);
        bonds_ = span([](const Res &l, U &b, U &e) { b = 0; e = l.B; }, kThreads);
        tiles_ = span([](const Res &l, U &b, U &e) { b = 0; e = l.dev.tiles_b; }, kThreads / 32);
        blocks_ = span([](const Res &l, U &b, U &e) { b = 0; e = l.dev.tiles_b / kScanBlock + 1; }, 1);
        each_ = span([](const Res &, U &b, U &e) { b = 0; e = 1; }, 1);
        slabs_ = span([](const Res &l, U &b, U &e) { b = 0; e = l.sched.block_count; }, 1);
        buckets_ = span([](const Res &l, U &b, U &e) { b = 0; e = l.nc_mem ? l.dev.nc_mask + 1U : 0U; }, kThreads);
        // With many lattices, the small ones sweep in one CTA each (largest first);
        // the level launches and the isolated-node launch cover the others.
        auto leveled = [this](const Res &l) { return !many_ || !sweptWhole(l); };
        {
            // Those whose positions fit the staged sweep's shared memory take
            // it when the shape asks for it.
            std::vector<std::uint32_t> whole, staged;
            staged_nodes_ = 0;
            if (many_)
                for (auto k : active_) {
                    const Res &l = *slots_[k];
                    if (!sweptWhole(l)) continue;
                    if (!kDirect && l.N <= shape_.staged_max_nodes) {
                        staged.push_back(k);
                        staged_nodes_ = std::max(staged_nodes_, l.N);
                    } else {
                        whole.push_back(k);
                    }
                }
            const auto larger = [this](std::uint32_t x, std::uint32_t y) { return slots_[x]->B > slots_[y]->B; };
            std::stable_sort(whole.begin(), whole.end(), larger);
            std::stable_sort(staged.begin(), staged.end(), larger);
            U first = static_cast<U>(all.size());
            for (auto k : whole) all.push_back({k, 0, 1});
            whole_ = Span{first, static_cast<U>(whole.size()), 0, 1, 1};
            first = static_cast<U>(all.size());
            for (auto k : staged) all.push_back({k, 0, 1});
            staged_ = Span{first, static_cast<U>(staged.size()), 0, 1, 1};
        }
        {
            const U first = static_cast<U>(all.size());
            for (auto k : active_) {
                const U parts = std::max(1U, std::min(608U, slots_[k]->B / 65536U));
                for (U q = 0; q < parts; ++q) all.push_back({k, q, parts});
            }
            const U count = static_cast<U>(all.size()) - first;
            broken_ = Span{first, count, 0, count, 1};
        }
        {
            // One item per (lattice, wrench slot): the batch's spreads in one launch.
            const U first = static_cast<U>(all.size());
            for (auto k : active_)
                for (U q = 0; q < slots_[k]->wrench_cap; ++q) all.push_back({k, q, slots_[k]->wrench_cap});
            wrench_ = Span{first, static_cast<U>(all.size()) - first, 0, 0, 1};
        }
        // The level-launched lattices in groups whose node arrays fit in L2
        // together: a group runs its whole sweep (every iteration, every
        // level) before the next, so its nodes stay resident across levels.
        groups_.clear();
        {
            std::vector<std::vector<U>> members(1);
            std::size_t bytes = 0;
            for (auto k : active_) {
                const Res &l = *slots_[k];
                if (!leveled(l)) continue;
                const std::size_t need = static_cast<std::size_t>(l.N) * sizeof(Q4<R>);
                if (!members.back().empty() && bytes + need > shape_.group_bytes) {
                    members.emplace_back();
                    bytes = 0;
                }
                members.back().push_back(k);
                bytes += need;
            }
            for (const auto &ids : members) {
                if (ids.empty()) continue;
                auto over = [&](auto &&bounds, U per) {
                    const U first = static_cast<U>(all.size());
                    U b0 = 0, e0 = 0;
                    bool lead = true;
                    for (auto k : ids) {
                        U b = 0, e = 0;
                        bounds(*slots_[k], b, e);
                        if (lead) { b0 = b; e0 = e; lead = false; }
                        ranges(k, b, e, per);
                    }
                    return Span{first, static_cast<U>(all.size()) - first, b0, e0, per};
                };
                Group g;
                std::size_t deepest = 0;
                for (auto k : ids) deepest = std::max(deepest, slots_[k]->levels.size());
                for (std::size_t d = 0; d < deepest; ++d)
                    g.levels.push_back(over([&](const Res &l, U &b, U &e) {
                        b = d < l.levels.size() ? l.levels[d].begin : 0;
                        e = d < l.levels.size() ? l.levels[d].end : 0;
                    }, kThreads * kSolvePer));
                g.isolated = over([](const Res &l, U &b, U &e) { b = 0; e = static_cast<U>(l.isolated.size()); },
                                  kThreads);
                groups_.push_back(std::move(g));
            }
        }
        // The radial damping sweep runs level by level over every lattice, the
        // ones swept whole included: it has no whole-lattice form.
        damp_.clear();
        if (S_.damping_fraction > R(0)) {
            std::size_t deepest = 0;
            for (auto k : active_) deepest = std::max(deepest, slots_[k]->levels.size());
            for (std::size_t d = 0; d < deepest; ++d) {
                const U first = static_cast<U>(all.size());
                U b0 = 0, e0 = 0;
                bool lead = true;
                for (auto k : active_) {
                    const Res &l = *slots_[k];
                    const U b = d < l.levels.size() ? l.levels[d].begin : 0;
                    const U e = d < l.levels.size() ? l.levels[d].end : 0;
                    if (lead) { b0 = b; e0 = e; lead = false; }
                    ranges(k, b, e, kThreads * kSolvePer);
                }
                damp_.push_back(Span{first, static_cast<U>(all.size()) - first, b0, e0, kThreads * kSolvePer});
            }
        }
        if (all.size() > work_cap_) {
            if (work_) cudaFree(work_);
            work_cap_ = std::max<std::size_t>(all.size(), 2 * work_cap_);
            check(cudaMalloc(&work_, sizeof(Work) * work_cap_), "device allocation");
        }
        upload(work_, all, stream_);
        check(cudaStreamSynchronize(stream_), "work lists");
        one_ = active_.empty() ? 0 : active_.front();
    }

    void dropGraph() {
        if (exec_) cudaGraphExecDestroy(exec_);
        if (graph_) cudaGraphDestroy(graph_);
        exec_ = nullptr;
        graph_ = nullptr;
    }

    // The launch form of a span: the work list and descriptor table for many
    // lattices, the descriptor itself and the item arithmetic for one.
    Grid<R> grid(const Span &s) const {
        Grid<R> g{};
        if (many_) {
            g.table = table_;
            g.list = work_ + s.first;
        } else {
            g.base = s.base;
            g.end = s.end;
            g.per = s.per;
            g.one = slots_[one_]->dev;
        }
        return g;
    }

    template <class Mark> void enqueueSubstep(Mark &&mark) {
        if (many_) enqueueSubstepAs<true>(mark);
        else enqueueSubstepAs<false>(mark);
    }

    // One substep for every lattice: the reference's phase order
    // (CpuLatticeBackend.cpp:357-488).
    template <bool M, class Mark> void enqueueSubstepAs(Mark &&mark) {
        const Settings<R> &S = S_;
        cudaStream_t st = stream_;
        // With a sphere, the restart runs beside the first contact pass (on
        // the second stream, from the starting positions the kick keeps);
        // without, before the kick.
        const bool side_restart = S.sphere_enabled != 0;
        if (!side_restart) restartPhase<M>(st, 0, mark);
        if (M) {
            if (wrench_.count) kWrenchMany<R><<<wrench_.count, kWrenchThreads, 0, st>>>(grid(wrench_));
        } else {
            for (auto k : active_) {
                const Resident<R> &l = *slots_[k];
                if (l.wrench_cap)
                    kWrench<R><<<l.wrench_cap, kWrenchThreads, 0, st>>>(l.dev, l.dev.wrench, l.dev.ext_nodes, nullptr,
                                                                       1);
            }
        }
        if (nodes_.count) kKick<R, M><<<nodes_.count, kThreads, 0, st>>>(grid(nodes_), S);
        // The load ledger, on its own stream until the serial tail.
        check(cudaEventRecord(load_fork_, st), "event");
        check(cudaStreamWaitEvent(loads_, load_fork_, 0), "stream wait");
        kLoadLedger<R, M><<<dim3(each_.count, kLedgerFolds), kLedgerThreads, 0, loads_>>>(grid(each_), S);
        check(cudaEventRecord(load_join_, loads_), "event");
        if (S.sphere_enabled && slabs_.count) {
            kCandidates<R, M><<<slabs_.count, 1024, 0, st>>>(grid(slabs_));
            kMarkHalo<R, M><<<slabs_.count, 1024, 0, st>>>(grid(slabs_));
        }
        mark(3);
        if (side_restart) {
            check(cudaEventRecord(fork_, st), "event");
            check(cudaStreamWaitEvent(side_, fork_, 0), "stream wait");
            restartPhase<M>(side_, 1);
            check(cudaEventRecord(join_, side_), "event");
            if (S.audit) audit<M>(st, kAuditMark);
            kSpherePass<R, M><<<each_.count, kSphereThreads, sphere_buffers_ * kSphereSlab, st>>>(grid(each_), S, 1,
                                                                                               sphere_buffers_);
            if (S.audit) audit<M>(st, kAuditStriker);
            check(cudaStreamWaitEvent(st, join_, 0), "stream wait");
        }
        mark(4);
        enqueueSweep<M>(mark);
        if (nodes_.count)
            kVelocity<R, M><<<nodes_.count, kThreads, 0, st>>>(grid(nodes_), S, S.damping_fraction <= R(0) ? 1 : 0);
        mark(8);
        if (S.damping_fraction > R(0)) {
            if (S.audit) audit<M>(st, kAuditMark);
            for (const Span &lv : damp_)
                if (lv.count) kDamp<R, M, kDirect><<<lv.count, kThreads, 0, st>>>(grid(lv), S.damping_fraction);
            if (S.audit) audit<M>(st, kAuditDamping);
            if (nodes_.count) kSupportVelocity<R, M><<<nodes_.count, kThreads, 0, st>>>(grid(nodes_), S);
            mark(9);
        }
        // With a sphere, the strain and end sample outside the contact halo
        // run on a second stream beside the second contact pass; the halo's
        // follow it. Node-to-node contact moves nodes anywhere after that
        // pass, so with it on the end phase waits for it whole.
        const bool contact = S.nc_mode != 0;
        const bool split = S.sphere_enabled != 0 && !contact;
        if (split) {
            check(cudaEventRecord(fork_, st), "event");
            check(cudaStreamWaitEvent(side_, fork_, 0), "stream wait");
            endPhase<M>(side_, 1);
            check(cudaEventRecord(join_, side_), "event");
        }
        if (S.sphere_enabled) {
            if (S.audit) audit<M>(st, kAuditMark);
            kSpherePass<R, M><<<each_.count, kSphereThreads, sphere_buffers_ * kSphereSlab, st>>>(grid(each_), S, 2,
                                                                                               sphere_buffers_);
            if (S.audit) audit<M>(st, kAuditStriker);
        }
        mark(10);
        if (split) check(cudaStreamWaitEvent(st, join_, 0), "stream wait");
        if (contact) contactPhase<M>(st, mark);
        endPhase<M>(st, split ? 2 : 0, mark);
        if (tiles_.count) kTileCounts<R, M><<<tiles_.count, kThreads, 0, st>>>(grid(tiles_));
        kBlockScan<R, M><<<blocks_.count, kScanBlock, 0, st>>>(grid(blocks_), plastic_ ? 1 : 0);
        kTopScan<R, M><<<each_.count, kScanBlock, 0, st>>>(grid(each_));
        if (tiles_.count) kEmitEvents<R, M><<<tiles_.count, kThreads, 0, st>>>(grid(tiles_));
        kLedgerBroken<R, M><<<broken_.count, kThreads, 0, st>>>(grid(broken_));
        mark(12);
        check(cudaStreamWaitEvent(st, load_join_, 0), "stream wait");
        kLedger<R, M><<<each_.count, 32, 0, st>>>(grid(each_), S);
        mark(13);
        check(cudaGetLastError(), "kernel launch");
    }

    // The energy audit (CpuLatticeBackend.cpp:388-422): every lattice's
    // kinetic energy folded in node order, before a phase or after it.
    template <bool M> void audit(cudaStream_t st, int mode) {
        kKineticFold<R, M><<<each_.count, kFoldThreads, 0, st>>>(grid(each_), mode);
    }

    // The projection sweep: the small lattices of a batch sweep whole, one
    // CTA each, on the second stream beside the level launches of the others.
    template <bool M, class Mark> void enqueueSweep(Mark &&mark) {
        const Settings<R> &S = S_;
        cudaStream_t st = stream_;
        const bool whole = M && (whole_.count || staged_.count);
        if (whole) {
            check(cudaEventRecord(fork_, st), "event");
            check(cudaStreamWaitEvent(side_, fork_, 0), "stream wait");
            if (whole_.count) launchSweepWhole(whole_, side_);
            if (staged_.count) launchSweepStaged(staged_, side_);
            check(cudaEventRecord(join_, side_), "event");
        }
        const unsigned I = S.iterations;
        for (const Group &g : groups_)
            for (unsigned it = 0; it < I; ++it) {
                const bool first = it == 0, last = it + 1 == I;
                for (const Span &lv : g.levels) launchSolve<M>(lv, first, last, g.levels.size() >= 2);
                mark(5);
                if (S.plane_count && g.isolated.count)
                    kSupportIsolated<R, M><<<g.isolated.count, kThreads, 0, st>>>(grid(g.isolated), S);
                mark(7);
            }
        if (whole) {
            check(cudaStreamWaitEvent(st, join_, 0), "stream wait");
            mark(5);
        }
    }

    // A launch that may start while the previous kernel of the stream still
    // runs (programmatic dependent launch); the kernel waits for it itself.
    // Only between sweep levels of two or more levels per iteration: a level
    // reads the multipliers its own range wrote one iteration earlier, which
    // must be complete -- with a single level that writer would be the very
    // kernel it overlaps.
    template <class... P, class... A>
    void launchOverlapped(bool overlap, void (*kernel)(P...), unsigned blocks, unsigned threads, A &&...args) {
        if (!overlap) {
            kernel<<<blocks, threads, 0, stream_>>>(std::forward<A>(args)...);
            return;
        }
        cudaLaunchConfig_t cfg{};
        cfg.gridDim = dim3(blocks);
        cfg.blockDim = dim3(threads);
        cfg.dynamicSmemBytes = 0;
        cfg.stream = stream_;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        check(cudaLaunchKernelEx(&cfg, kernel, std::forward<A>(args)...), "kernel launch");
    }

    void launchSweepWhole(const Span &span, cudaStream_t st) {
        switch (shape_.sweep_threads) {
        case 256: launchSweepWholeAs<256>(span, st); break;
        case 1024: launchSweepWholeAs<1024>(span, st); break;
        default: launchSweepWholeAs<512>(span, st); break;
        }
    }
    template <unsigned T> void launchSweepWholeAs(const Span &span, cudaStream_t st) {
        const bool support = S_.plane_count != 0;
        const int key = (plastic_ ? 2 : 0) | (support ? 1 : 0);
        const Grid<R> g = grid(span);
        switch (key) {
        case 0: kSweepLattice<R, kDirect, false, false, T><<<span.count, T, 0, st>>>(g, S_); break;
        case 1: kSweepLattice<R, kDirect, false, true, T><<<span.count, T, 0, st>>>(g, S_); break;
        case 2: kSweepLattice<R, kDirect, true, false, T><<<span.count, T, 0, st>>>(g, S_); break;
        default: kSweepLattice<R, kDirect, true, true, T><<<span.count, T, 0, st>>>(g, S_); break;
        }
    }

    // The whole sweeps of the lattices whose positions fit in shared memory
    // (float lane): staged in by one bulk copy, swept in the SM, written back.
    void launchSweepStaged(const Span &span, cudaStream_t st) {
        if constexpr (!kDirect) {
            switch (shape_.sweep_threads) {
            case 256: launchSweepStagedAs<256>(span, st); break;
            case 1024: launchSweepStagedAs<1024>(span, st); break;
            default: launchSweepStagedAs<512>(span, st); break;
            }
        }
    }
    template <unsigned T> void launchSweepStagedAs(const Span &span, cudaStream_t st) {
        const bool support = S_.plane_count != 0;
        const int key = (plastic_ ? 2 : 0) | (support ? 1 : 0);
        const Grid<R> g = grid(span);
        const std::size_t smem = static_cast<std::size_t>(staged_nodes_) * sizeof(Q4<R>);
        switch (key) {
        case 0: kSweepLattice<R, kDirect, false, false, T, true><<<span.count, T, smem, st>>>(g, S_); break;
        case 1: kSweepLattice<R, kDirect, false, true, T, true><<<span.count, T, smem, st>>>(g, S_); break;
        case 2: kSweepLattice<R, kDirect, true, false, T, true><<<span.count, T, smem, st>>>(g, S_); break;
        default: kSweepLattice<R, kDirect, true, true, T, true><<<span.count, T, smem, st>>>(g, S_); break;
        }
    }
    // The shared memory every staged instance may take: set once.
    void allowStagedSharedMemory() {
        if constexpr (!kDirect) {
            const int bytes = static_cast<int>(kStagedMaxNodes * sizeof(Q4<R>));
            auto allow = [&](auto kernel) {
                check(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes),
                      "staged sweep shared memory");
            };
            allow(kSweepLattice<R, kDirect, false, false, 256, true>);
            allow(kSweepLattice<R, kDirect, false, true, 256, true>);
            allow(kSweepLattice<R, kDirect, true, false, 256, true>);
            allow(kSweepLattice<R, kDirect, true, true, 256, true>);
            allow(kSweepLattice<R, kDirect, false, false, 512, true>);
            allow(kSweepLattice<R, kDirect, false, true, 512, true>);
            allow(kSweepLattice<R, kDirect, true, false, 512, true>);
            allow(kSweepLattice<R, kDirect, true, true, 512, true>);
            allow(kSweepLattice<R, kDirect, false, false, 1024, true>);
            allow(kSweepLattice<R, kDirect, false, true, 1024, true>);
            allow(kSweepLattice<R, kDirect, true, false, 1024, true>);
            allow(kSweepLattice<R, kDirect, true, true, 1024, true>);
        }
    }

    // Node-to-node contact: the drift test, the pair-list rebuild (every
    // kernel of it returns at once when no rebuild is due), the narrow phase.
    template <bool M, class Mark> void contactPhase(cudaStream_t st, Mark &&mark) {
        const Settings<R> &S = S_;
        if (nodes_.count) kContactStale<R, M><<<nodes_.count, kThreads, 0, st>>>(grid(nodes_), S);
        if (buckets_.count) kContactClear<R, M><<<buckets_.count, kThreads, 0, st>>>(grid(buckets_));
        if (nodes_.count) kContactCells<R, M><<<nodes_.count, kThreads, 0, st>>>(grid(nodes_), S);
        if (buckets_.count) kContactBuckets<R, M><<<buckets_.count, kThreads, 0, st>>>(grid(buckets_));
        if (nodes_.count) kContactScatter<R, M><<<nodes_.count, kThreads, 0, st>>>(grid(nodes_));
        if (buckets_.count) kContactSort<R, M><<<buckets_.count, kThreads, 0, st>>>(grid(buckets_));
        if (nodes_.count) kContactGather<R, M, false><<<nodes_.count, kThreads, 0, st>>>(grid(nodes_), S);
        kContactTiles<R, M><<<each_.count, kContactScanThreads, 0, st>>>(grid(each_));
        if (nodes_.count) kContactGather<R, M, true><<<nodes_.count, kThreads, 0, st>>>(grid(nodes_), S);
        mark(14);
        kContactNarrow<R, M><<<each_.count, 32, 0, st>>>(grid(each_), S);
        mark(15);
    }

    // The start-of-substep restart: strain of the dirty (or all) nodes, then
    // the start samples of their bonds.
    template <bool M, class Mark = void (*)(unsigned)>
    void restartPhase(cudaStream_t st, int after_kick, Mark &&mark = [](unsigned) {}) {
        if (nodes_.count) {
            const R plate = S_.plate_half_thickness, yield = S_.yield_stretch;
            if (plate > R(0))
                kRestartStrain<R, M, kDirect, true><<<nodes_.count, kThreads, 0, st>>>(grid(nodes_), after_kick, plate,
                                                                                       yield);
            else
                kRestartStrain<R, M, kDirect, false><<<nodes_.count, kThreads, 0, st>>>(grid(nodes_), after_kick,
                                                                                        plate, yield);
        }
        mark(1);
        if (bonds_.count)
            kRestartBondsAll<R, M, kDirect><<<bonds_.count, kThreads, 0, st>>>(grid(bonds_), after_kick);
        if (nodes_.count)
            kRestartBondsDirty<R, M, kDirect><<<nodes_.count, kThreads, 0, st>>>(grid(nodes_), after_kick);
        mark(2);
    }

    // Strain of the nodes, then the end sample of the bonds, of one part
    // (0 all, 1 outside the contact halo, 2 inside it).
    template <bool M, class Mark = void (*)(unsigned)>
    void endPhase(cudaStream_t st, int part, Mark &&mark = [](unsigned) {}) {
        if (nodes_.count) {
            const R plate = S_.plate_half_thickness, yield = S_.yield_stretch;
            if (plate > R(0))
                kStrainAll<R, M, kDirect, true><<<nodes_.count, kThreads, 0, st>>>(grid(nodes_), part, plate, yield);
            else
                kStrainAll<R, M, kDirect, false><<<nodes_.count, kThreads, 0, st>>>(grid(nodes_), part, plate, yield);
        }
        mark(11);
        if (bonds_.count) {
            if (plastic_) kEndSample<R, M, kDirect, true><<<bonds_.count, kThreads, 0, st>>>(grid(bonds_), S_, part);
            else kEndSample<R, M, kDirect, false><<<bonds_.count, kThreads, 0, st>>>(grid(bonds_), S_, part);
        }
    }

    template <bool M> void launchSolve(const Span &lv, bool first, bool last, bool overlap) {
        if (!lv.count) return;
        const bool support = S_.plane_count != 0;
        const int key = (first ? 8 : 0) | (last ? 4 : 0) | (plastic_ ? 2 : 0) | (support ? 1 : 0);
#define GBL_SOLVE(K)                                                                                                \
    case K:                                                                                                         \
        launchOverlapped(overlap,                                                                                   \
                         kSolve<R, M, kDirect, ((K) & 8) != 0, ((K) & 4) != 0, ((K) & 2) != 0, ((K) & 1) != 0>,     \
                         lv.count, kThreads, grid(lv), S_);                                                         \
        break;
        switch (key) {
            GBL_SOLVE(0) GBL_SOLVE(1) GBL_SOLVE(2) GBL_SOLVE(3) GBL_SOLVE(4) GBL_SOLVE(5) GBL_SOLVE(6) GBL_SOLVE(7)
            GBL_SOLVE(8) GBL_SOLVE(9) GBL_SOLVE(10) GBL_SOLVE(11) GBL_SOLVE(12) GBL_SOLVE(13) GBL_SOLVE(14)
            GBL_SOLVE(15)
        }
#undef GBL_SOLVE
    }

    std::vector<std::unique_ptr<Resident<R>>> slots_;
    std::vector<std::uint32_t> active_;
    std::mutex place_mutex_;
    Settings<R> S_{};
    bool plastic_{false}, ready_{false}, many_{false}, dirty_{true};
    unsigned sphere_buffers_{1};
    std::uint32_t one_{0};
    Ctl *ctl_{};
    std::size_t cap_{0}, work_cap_{0};
    std::vector<Ctl> ctl_host_;
    unsigned *running_{}, *running_host_{};
    Dev<R> *table_{};
    Work *work_{};
    Span nodes_{}, bonds_{}, tiles_{}, blocks_{}, each_{}, slabs_{}, broken_{}, whole_{}, staged_{}, buckets_{},
        wrench_{};
    std::uint32_t staged_nodes_{0}; // the staged sweep's shared memory, in nodes
    // Level-launched lattices, in groups swept one after another.
    struct Group {
        std::vector<Span> levels;
        Span isolated{};
    };
    std::vector<Group> groups_;
    std::vector<Span> damp_; // the damping sweep's levels, every lattice
    // Node bytes a group may hold: its node arrays stay in the 129 MB L2
    // beside the streamed bond records of a level.
    // Launch shapes of a batch's sweep (results do not depend on them): the
    // one-CTA sweep's CTA size, the largest lattice it takes, and the node
    // bytes of a level-launched group. Defaults measured on the trial
    // workload; tune() times candidates on the lattices present.
    struct Shape {
        unsigned sweep_threads = kSweepThreads;
        std::uint32_t whole_max_bonds = kMaxFusedBonds;
        std::size_t group_bytes = std::size_t(48) << 20;
        std::uint32_t staged_max_nodes = 0; // whole sweeps staged in shared memory up to this many nodes
    };
    Shape shape_;
    cudaStream_t own_stream_{}, stream_{}, side_{}, loads_{};
    cudaEvent_t ev0_{}, ev1_{}, fork_{}, join_{}, load_fork_{}, load_join_{};
    cudaGraph_t graph_{};
    cudaGraphExec_t exec_{};
};

// The single-lattice LatticeBackend: an engine of one lattice.
class BackendBase {
public:
    virtual ~BackendBase() = default;
    virtual std::string name() const = 0;
    virtual void upload(const gbl_state_view &, const gbl_step_settings &, const gbl_sphere &) = 0;
    virtual void setExternalForces(const double *forces, std::uint64_t count, std::uint64_t substeps) = 0;
    virtual void setExternalWrenches(const gbl_external_wrench *ws, std::uint64_t count, std::uint64_t substeps) = 0;
    virtual std::vector<std::pair<std::string, LoadLedger>> sources() = 0;
    virtual void run(const gbl_run_control &) = 0;
    virtual void download(gbl_state_view &, gbl_sphere *) = 0;
    virtual void debugSubstep(std::uint32_t mask, gbl_state_view *views, gbl_sphere *spheres) = 0;
    virtual void profile(std::uint64_t substeps, double *phase_ms) = 0;
    virtual void setStream(cudaStream_t s) = 0;
    virtual std::uint64_t kernelsPerSubstep() = 0;
    virtual const gbl_run_status &status() const = 0;
    virtual gbl_run_status &mutableStatus() = 0;
    virtual const std::vector<std::uint32_t> &firstFailure() const = 0;
    virtual std::vector<Frame> &frames() = 0;
};

template <class R> class Backend final : public BackendBase {
public:
    explicit Backend(Schedule s) : sched_(std::move(s)) {}
    std::string name() const override { return std::is_same<R, double>::value ? "gb300-double" : "gb300-float"; }
    void upload(const gbl_state_view &st, const gbl_step_settings &set, const gbl_sphere &sphere) override {
        Engine<R>::validate(set);
        engine_.clear();
        engine_.add(sched_, st, sphere);
        engine_.settle(set);
    }
    void setExternalForces(const double *forces, std::uint64_t count, std::uint64_t substeps) override {
        if (engine_.size() == 0) invalid("external load needs an uploaded lattice");
        engine_.setExternalForces(0, forces, count, substeps);
    }
    void setExternalWrenches(const gbl_external_wrench *ws, std::uint64_t count, std::uint64_t substeps) override {
        if (engine_.size() == 0) invalid("external wrench needs an uploaded lattice");
        engine_.setExternalWrenches(0, ws, count, substeps);
    }
    std::vector<std::pair<std::string, LoadLedger>> sources() override {
        if (engine_.size() == 0) return {};
        return engine_.lattice(0).sources();
    }
    void run(const gbl_run_control &control) override {
        if (engine_.size() == 0) invalid("lattice run needs an uploaded lattice");
        engine_.run(control);
    }
    void download(gbl_state_view &st, gbl_sphere *sphere) override {
        if (engine_.size() == 0) invalid("lattice download needs an uploaded lattice");
        engine_.download(0, st, sphere);
    }
    void profile(std::uint64_t substeps, double *phase_ms) override {
        if (engine_.size() == 0) invalid("profiling needs an uploaded lattice");
        engine_.profile(substeps, phase_ms);
    }
    void debugSubstep(std::uint32_t mask, gbl_state_view *views, gbl_sphere *spheres) override {
        if (engine_.size() == 0) invalid("the phase-diff substep needs an uploaded lattice");
        engine_.debugSubstep(0, mask, views, spheres);
    }
    void setStream(cudaStream_t s) override { engine_.setStream(s); }
    std::uint64_t kernelsPerSubstep() override {
        if (engine_.size() == 0) invalid("the substep graph needs an uploaded lattice");
        return engine_.kernelsPerSubstep();
    }
    const gbl_run_status &status() const override { return engine_.size() ? lat().status : empty_; }
    gbl_run_status &mutableStatus() override { return engine_.size() ? engine_.lattice(0).status : empty_; }
    const std::vector<std::uint32_t> &firstFailure() const override { return engine_.size() ? lat().first_failure : none_; }
    std::vector<Frame> &frames() override { return engine_.size() ? engine_.lattice(0).frames : no_frames_; }

private:
    const Resident<R> &lat() const { return const_cast<Engine<R> &>(engine_).lattice(0); }
    Schedule sched_;
    Engine<R> engine_;
    gbl_run_status empty_{};
    std::vector<std::uint32_t> none_;
    std::vector<Frame> no_frames_;
};

// The batch: K independent lattices sharing step settings.
class BatchBase {
public:
    virtual ~BatchBase() = default;
    virtual std::size_t add(const Schedule &s, const gbl_state_view &st, const gbl_sphere &sp) = 0;
    virtual void settle(const gbl_step_settings &set) = 0;
    virtual void setExternalForces(std::size_t k, const double *f, std::uint64_t n, std::uint64_t substeps) = 0;
    virtual void setExternalWrenches(std::size_t k, const gbl_external_wrench *ws, std::uint64_t count,
                                     std::uint64_t substeps) = 0;
    virtual std::vector<std::pair<std::string, LoadLedger>> sources(std::size_t k) = 0;
    virtual void run(const gbl_run_control &c) = 0;
    virtual void download(std::size_t k, gbl_state_view &st, gbl_sphere *sp) = 0;
    virtual const gbl_run_status &status(std::size_t k) = 0;
    virtual std::vector<std::uint32_t> firstFailure(std::size_t k) = 0;
    virtual std::size_t size() const = 0;
    virtual void profile(std::uint64_t substeps, double *phase_ms) = 0;
    virtual std::uint64_t kernelsPerSubstep() = 0;
    virtual void setStream(cudaStream_t s) = 0;
    virtual gbl_tuning tune() = 0;
    virtual void setShape(const gbl_tuning &t) = 0;
};

template <class R> class Batch final : public BatchBase {
public:
    std::size_t add(const Schedule &s, const gbl_state_view &st, const gbl_sphere &sp) override {
        return engine_.add(s, st, sp);
    }
    void settle(const gbl_step_settings &set) override { engine_.settle(set); }
    void setExternalForces(std::size_t k, const double *f, std::uint64_t n, std::uint64_t substeps) override {
        engine_.setExternalForces(k, f, n, substeps);
    }
    void setExternalWrenches(std::size_t k, const gbl_external_wrench *ws, std::uint64_t count,
                             std::uint64_t substeps) override {
        engine_.setExternalWrenches(k, ws, count, substeps);
    }
    std::vector<std::pair<std::string, LoadLedger>> sources(std::size_t k) override {
        return engine_.lattice(k).sources();
    }
    void run(const gbl_run_control &c) override { engine_.run(c); }
    void download(std::size_t k, gbl_state_view &st, gbl_sphere *sp) override { engine_.download(k, st, sp); }
    const gbl_run_status &status(std::size_t k) override { return engine_.lattice(k).status; }
    std::vector<std::uint32_t> firstFailure(std::size_t k) override { return engine_.lattice(k).first_failure; }
    std::size_t size() const override { return engine_.size(); }
    void profile(std::uint64_t substeps, double *phase_ms) override { engine_.profile(substeps, phase_ms); }
    std::uint64_t kernelsPerSubstep() override { return engine_.kernelsPerSubstep(); }
    void setStream(cudaStream_t s) override { engine_.setStream(s); }
    gbl_tuning tune() override { return engine_.tune(); }
    void setShape(const gbl_tuning &t) override { engine_.setShape(t); }

private:
    Engine<R> engine_;
};

// The served form: requests (one lattice each, with a substep count) arrive at
// any time; they are admitted in arrival order while their device footprint
// fits the HBM budget, run together one chunk of substeps at a time with every
// other admitted request, and leave as soon as their own count is done, which
// frees their memory for the next in line. Each request's result is the one it
// would get alone: lattices never interact, and each keeps its own control
// block and ledgers.
//
// Two lanes, each an engine with its own streams and substep graph: requests
// of at least kLargeBonds bonds in one, the rest in the other. A step runs the
// large lane's chunk on a helper thread while the calling thread keeps
// stepping the small lane chunk after chunk (retiring and admitting small
// requests between chunks) until the large chunk is done, so a small request
// advances at its own lane's pace instead of a large lattice's, and the two
// lanes' kernels share the GPU.
class ServerBase {
public:
    virtual ~ServerBase() = default;
    virtual std::uint64_t submit(const gbl_schedule_view &s, const gbl_state_view &st, const gbl_sphere &sp,
                                 std::uint64_t substeps, bool borrowed) = 0;
    virtual void step(std::uint64_t substeps, gbl_server_stats *stats) = 0;
    virtual void poll(std::uint64_t ticket, gbl_request_info &info) = 0;
    virtual void take(std::uint64_t ticket, gbl_state_view *st, gbl_sphere *sp, gbl_run_status *status) = 0;
    virtual void cancel(std::uint64_t ticket) = 0;
    virtual void stats(gbl_server_stats &out) = 0;
    virtual void setLaneThreshold(std::uint32_t bonds) = 0;
};

template <class R> class Server final : public ServerBase {
public:
    static constexpr std::uint32_t kLargeBonds = 1U << 22;
    static constexpr std::uint32_t kServedWholeBonds = 1U << 14;
    static constexpr unsigned kSmall = 0, kLarge = 1;

    Server(const gbl_step_settings &settings, std::uint64_t budget)
        : budget_(budget), contact_(settings.node_contact.mode != 0), t0_(clock()) {
        for (auto &lane : lanes_) lane.configure(settings);
        // A server holds few lattices at a time: a lattice swept whole by one
        // CTA takes that CTA's serial time per substep (about 3.5 ms for
        // 2^18 bonds), where level launches spread it over the GPU. Only
        // tiny lattices sweep whole here.
        gbl_tuning shape{};
        shape.whole_max_bonds = kServedWholeBonds;
        for (auto &lane : lanes_) lane.setShape(shape);
    }
    ~Server() override {
        for (auto &kv : requests_)
            if (kv.second.phase == GBL_REQUEST_DONE && kv.second.out.base)
                cudaFreeAsync(kv.second.out.base, lanes_[kv.second.lane].stream());
        for (auto &lane : lanes_) cudaStreamSynchronize(lane.stream());
    }

    std::uint64_t submit(const gbl_schedule_view &sv, const gbl_state_view &st, const gbl_sphere &sp,
                         std::uint64_t substeps, bool borrowed) override {
        if (substeps == 0) invalid("a served request needs at least one substep");
        if (sv.node_count != st.node_count || sv.bond_count != st.bond_count)
            invalid("lattice schedule does not match the lattice");
        const std::uint64_t bytes =
            Resident<R>::footprint(st.node_count, st.bond_count, st.max_degree, sv.block_count) +
            (contact_ ? Resident<R>::contactBytes(st.node_count) : 0);
        if (bytes > budget_) invalid("request exceeds the device memory budget on its own");
        Request q;
        q.submitted = clock() - t0_;
        // Prepared here, on the caller's thread, outside the lock (a step may
        // be running meanwhile): the device image, or for a borrowed state
        // only the sweep order -- the device converts the caller's arrays at
        // admission.
        q.prepared = Engine<R>::prepare(Schedule::fromView(sv), st, sp, !borrowed);
        q.nodes = st.node_count;
        q.bonds = st.bond_count;
        q.lane = st.bond_count >= large_bonds_.load(std::memory_order_relaxed) ? kLarge : kSmall;
        q.sphere = sp;
        q.substeps = substeps;
        q.bytes = bytes;
        std::lock_guard<std::mutex> lock(mutex_);
        q.ticket = ++last_ticket_;
        const std::uint64_t t = q.ticket;
        requests_.emplace(t, std::move(q));
        queue_.push_back(t);
        ++queued_;
        return t;
    }

    void step(std::uint64_t substeps, gbl_server_stats *out) override {
        std::lock_guard<std::mutex> lock(mutex_);
        admit(true);
        if (substeps > 0 && (lanes_[kSmall].size() > 0 || lanes_[kLarge].size() > 0)) {
            gbl_run_control c{}; // RunControl's defaults (FastLattice.hpp:79-128), exit rules off
            c.energy_flat_fraction = 1.0e-3;
            c.calm_damage_margin = 0.5;
            c.max_steps = substeps;
            const double t0 = clock();
            double large_device = 0.0, small_device = 0.0;
            if (lanes_[kLarge].size() > 0) {
                // The large lane's chunk on a helper thread; that thread
                // touches nothing but its lane until it is joined.
                std::atomic<bool> large_done{false};
                std::exception_ptr failure;
                std::thread large([&] {
                    try {
                        const double before = kernelSeconds(kLarge);
                        lanes_[kLarge].run(c);
                        large_device = kernelSeconds(kLarge) - before;
                    } catch (...) {
                        failure = std::current_exception();
                    }
                    large_done.store(true, std::memory_order_release);
                });
                try {
                    bool first = true;
                    while (lanes_[kSmall].size() > 0 && (first || !large_done.load(std::memory_order_acquire))) {
                        small_device += runLane(kSmall, c);
                        admit(false);
                        first = false;
                    }
                } catch (...) {
                    large.join();
                    throw;
                }
                large.join();
                if (failure) std::rethrow_exception(failure);
                substeps_run_ += substeps;
                retireFinished(kLarge);
            } else {
                small_device += runLane(kSmall, c);
            }
            run_seconds_ += clock() - t0;
            device_seconds_ += std::max(large_device, small_device);
            admit(true); // memory freed this step goes to the next in line now
        }
        if (out) fillStats(*out);
    }

    void poll(std::uint64_t ticket, gbl_request_info &info) override {
        std::lock_guard<std::mutex> lock(mutex_);
        const Request &q = find(ticket);
        info = gbl_request_info{};
        info.phase = q.phase;
        info.slot = q.phase == GBL_REQUEST_RUNNING ? static_cast<std::uint32_t>(q.slot) : ~0U;
        info.substeps = q.substeps;
        info.substeps_done =
            q.phase == GBL_REQUEST_RUNNING ? lanes_[q.lane].control(q.slot).total_steps : q.done_steps;
        info.device_bytes = q.bytes;
        info.submitted_s = q.submitted;
        info.admitted_s = q.admitted;
        info.finished_s = q.finished;
    }

    void take(std::uint64_t ticket, gbl_state_view *st, gbl_sphere *sp, gbl_run_status *status) override {
        StateOut out;
        unsigned lane = kSmall;
        {
            std::lock_guard<std::mutex> lock(mutex_);
            Request &q = find(ticket);
            if (q.phase != GBL_REQUEST_DONE) invalid("the request has not finished");
            if (st && (st->node_count != q.nodes || st->bond_count != q.bonds))
                invalid("result state does not match the request's lattice");
            if (sp) *sp = q.sphere;
            if (status) *status = q.status;
            out = q.out;
            lane = q.lane;
            requests_.erase(ticket);
            --done_;
        }
        // The copies into the caller's arrays run on the caller's thread,
        // outside the lock (they use their own streams); the result's device
        // memory is then freed, stream-ordered, under the lock (a step may be
        // capturing on the lane's stream).
        if (st) out.copyTo(*st);
        std::lock_guard<std::mutex> lock(mutex_);
        check(cudaFreeAsync(out.base, lanes_[lane].stream()), "device free");
        used_ -= out.bytes;
    }

    void cancel(std::uint64_t ticket) override {
        std::lock_guard<std::mutex> lock(mutex_);
        Request &q = find(ticket);
        if (q.phase == GBL_REQUEST_QUEUED) {
            queue_.erase(std::find(queue_.begin(), queue_.end(), ticket));
            --queued_;
        } else if (q.phase == GBL_REQUEST_RUNNING) {
            lanes_[q.lane].retire(q.slot);
            used_ -= q.bytes;
            --running_;
        } else if (q.phase == GBL_REQUEST_DONE) {
            --done_;
            check(cudaFreeAsync(q.out.base, lanes_[q.lane].stream()), "device free");
            used_ -= q.out.bytes;
        }
        requests_.erase(ticket);
    }

    void stats(gbl_server_stats &o) override {
        std::lock_guard<std::mutex> lock(mutex_);
        fillStats(o);
    }

    // Requests submitted from now on with at least `bonds` bonds take the
    // large lane.
    void setLaneThreshold(std::uint32_t bonds) override { large_bonds_.store(bonds, std::memory_order_relaxed); }

private:
    void fillStats(gbl_server_stats &o) {
        o = gbl_server_stats{};
        o.queued = queued_;
        o.running = running_;
        o.done = done_;
        o.bytes_in_use = used_;
        o.budget_bytes = budget_;
        o.substeps_run = substeps_run_;
        o.device_seconds = device_seconds_;
        o.clock_s = clock() - t0_;
        o.admit_seconds = admit_seconds_;
        o.retire_seconds = retire_seconds_;
        o.run_seconds = run_seconds_;
    }

    struct Request {
        std::uint64_t ticket{}, substeps{}, bytes{}, done_steps{};
        std::uint32_t nodes{}, bonds{};
        unsigned lane{kSmall};
        std::unique_ptr<Resident<R>> prepared;
        gbl_sphere sphere{};
        int phase{GBL_REQUEST_QUEUED};
        std::size_t slot{};
        double submitted{-1}, admitted{-1}, finished{-1};
        gbl_run_status status{};
        StateOut out; // a finished request's result, on the device until taken
    };

    static double clock() {
        return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
    }

    Request &find(std::uint64_t ticket) {
        auto it = requests_.find(ticket);
        if (it == requests_.end()) invalid("unknown request ticket");
        return it->second;
    }

    double kernelSeconds(unsigned lane) {
        double s = 0;
        Engine<R> &e = lanes_[lane];
        for (std::size_t k = 0; k < e.slots(); ++k)
            if (e.occupied(k)) s = std::max(s, e.lattice(k).status.kernel_seconds);
        return s;
    }

    // One chunk of the small lane, then its finished requests retired.
    double runLane(unsigned lane, const gbl_run_control &c) {
        const double before = kernelSeconds(lane);
        lanes_[lane].run(c);
        const double device = kernelSeconds(lane) - before;
        if (lane == kSmall && lanes_[kLarge].size() == 0) substeps_run_ += c.max_steps;
        retireFinished(lane);
        return device;
    }

    // Arrival order, while the next request fits what is left of the budget.
    // With `any_lane` false (the large lane is running on its helper thread)
    // admission stops at the first large request in line.
    // (Converting admitted requests on a second stream beside the running
    // ones was measured slower: the conversion's reads of host memory slowed
    // the running kernels by more than they overlapped.)
    void admit(bool any_lane) {
        const double t0 = clock();
        while (!queue_.empty()) {
            Request &q = requests_.at(queue_.front());
            if (used_ + q.bytes > budget_) break;
            if (!any_lane && q.lane != kSmall) break;
            q.slot = lanes_[q.lane].place(std::move(q.prepared), q.substeps);
            q.phase = GBL_REQUEST_RUNNING;
            q.admitted = clock() - t0_;
            used_ += q.bytes;
            auto &tickets = slot_ticket_[q.lane];
            tickets.resize(std::max(tickets.size(), q.slot + 1));
            tickets[q.slot] = q.ticket;
            queue_.pop_front();
            --queued_;
            ++running_;
        }
        admit_seconds_ += clock() - t0;
    }

    void retireFinished(unsigned lane) {
        const double t0 = clock();
        Engine<R> &e = lanes_[lane];
        for (std::size_t k = 0; k < e.slots(); ++k) {
            if (!e.occupied(k)) continue;
            const Ctl &c = e.control(k);
            if (!(c.step_limit != 0 && c.total_steps >= c.step_limit) && c.exit_reason == 0) continue;
            Request &q = requests_.at(slot_ticket_[lane][k]);
            Resident<R> &l = e.lattice(k);
            // The result, in the state's layout, stays on the device until
            // take() copies it out; the lattice's own memory is freed now.
            q.out = l.stateOut(e.stream());
            check(cudaStreamSynchronize(e.stream()), "retire");
            q.sphere = l.fetchSphere();
            q.status = l.status;
            q.status.exit_reason = c.exit_reason;
            q.done_steps = c.total_steps;
            e.retire(k); // synchronises the stream: the result is written
            used_ -= q.bytes;
            used_ += q.out.bytes;
            q.phase = GBL_REQUEST_DONE;
            q.finished = clock() - t0_;
            --running_;
            ++done_;
        }
        retire_seconds_ += clock() - t0;
    }

    Engine<R> lanes_[2];
    std::atomic<std::uint32_t> large_bonds_{kLargeBonds};
    std::uint64_t budget_, used_{0}, last_ticket_{0};
    bool contact_; // node-to-node contact on: every request also holds its pair-list scratch
    std::uint64_t queued_{0}, running_{0}, done_{0}, substeps_run_{0};
    double device_seconds_{0}, admit_seconds_{0}, retire_seconds_{0}, run_seconds_{0};
    double t0_;
    std::map<std::uint64_t, Request> requests_;
    std::deque<std::uint64_t> queue_;
    std::vector<std::uint64_t> slot_ticket_[2];
    std::mutex mutex_;
};

} // namespace gbl

struct gbl_backend {
    std::unique_ptr<gbl::BackendBase> impl;
};
struct gbl_batch {
    std::unique_ptr<gbl::BatchBase> impl;
};
struct gbl_server {
    std::unique_ptr<gbl::ServerBase> impl;
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
        (void)threads_per_block; // the launch shapes are the engine's own
        if (!schedule || !out) gbl::invalid("null argument");
        if (!gbl_available()) gbl::runtime("no CUDA device is available for the lattice backend");
        gbl::Schedule s = gbl::Schedule::fromView(*schedule);
        auto b = std::make_unique<gbl_backend>();
        if (precision == GBL_PRECISION_DOUBLE) b->impl = std::make_unique<gbl::Backend<double>>(std::move(s));
        else if (precision == GBL_PRECISION_FLOAT) b->impl = std::make_unique<gbl::Backend<float>>(std::move(s));
        else gbl::invalid("unknown precision");
        *out = b.release();
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

gbl_result gbl_set_external_wrenches(gbl_backend *backend, const gbl_external_wrench *wrenches, uint64_t count,
                                     uint64_t substeps) {
    return gbl::guard([&] {
        if (!backend) gbl::invalid("null backend");
        backend->impl->setExternalWrenches(wrenches, count, substeps);
    });
}

gbl_result gbl_external_source_count(gbl_backend *backend, uint64_t *count) {
    return gbl::guard([&] {
        if (!backend || !count) gbl::invalid("null argument");
        *count = backend->impl->sources().size();
    });
}

namespace gbl {
// One entry of RunStatus::external_sources, out through the C ABI.
void sourceOut(const std::vector<std::pair<std::string, LoadLedger>> &all, uint64_t index, char *name,
               size_t name_capacity, size_t *name_length, gbl_load_ledger *load) {
    if (index >= all.size()) invalid("no external source at that index");
    const auto &[source, g] = all[index];
    if (name_length) *name_length = source.size();
    if (name && name_capacity) {
        const std::size_t n = std::min(source.size(), name_capacity - 1);
        std::memcpy(name, source.data(), n);
        name[n] = 0;
    }
    if (load) {
        load->steps = g.steps;
        load->elapsed_s = g.elapsed;
        for (int q = 0; q < 3; ++q) {
            load->requested_impulse_n_s[q] = g.req_imp[q];
            load->impulse_n_s[q] = g.imp[q];
            load->requested_angular_impulse_kg_m2_s[q] = g.req_ang[q];
            load->angular_impulse_kg_m2_s[q] = g.ang[q];
        }
        load->work_j = g.work;
    }
}
} // namespace gbl

gbl_result gbl_external_source(gbl_backend *backend, uint64_t index, char *name, size_t name_capacity,
                               size_t *name_length, gbl_load_ledger *load) {
    return gbl::guard([&] {
        if (!backend) gbl::invalid("null backend");
        gbl::sourceOut(backend->impl->sources(), index, name, name_capacity, name_length, load);
    });
}

gbl_result gbl_run(gbl_backend *backend, const gbl_run_control *control, gbl_run_status *status_out) {
    return gbl::guard([&] {
        if (!backend || !control) gbl::invalid("null argument");
        backend->impl->run(*control);
        if (status_out) *status_out = backend->impl->status();
    });
}

gbl_result gbl_status(const gbl_backend *backend, gbl_run_status *status_out) {
    return gbl::guard([&] {
        if (!backend || !status_out) gbl::invalid("null argument");
        *status_out = backend->impl->status();
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
        const auto &f = backend->impl->firstFailure();
        *count = f.size();
        if (out) std::memcpy(out, f.data(), sizeof(uint32_t) * std::min<std::uint64_t>(capacity, f.size()));
    });
}

gbl_result gbl_frame_count(const gbl_backend *backend, uint64_t *count) {
    return gbl::guard([&] {
        if (!backend || !count) gbl::invalid("null argument");
        *count = const_cast<gbl_backend *>(backend)->impl->frames().size();
    });
}

gbl_result gbl_take_frame(const gbl_backend *backend, uint64_t index, uint64_t *step, float *u, uint8_t *alive,
                          float *damage, gbl_sphere *sphere) {
    return gbl::guard([&] {
        if (!backend) gbl::invalid("null backend");
        const auto &fr = const_cast<gbl_backend *>(backend)->impl->frames();
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
        backend->impl->frames().clear();
        backend->impl->mutableStatus().frames_captured = 0;
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

gbl_result gbl_debug_substep(gbl_backend *backend, uint32_t phase_mask, gbl_state_view *states, gbl_sphere *spheres) {
    return gbl::guard([&] {
        if (!backend || (phase_mask && !states)) gbl::invalid("null argument");
        if (phase_mask >> GBL_PHASE_COUNT) gbl::invalid("phase mask names no such phase");
        backend->impl->debugSubstep(phase_mask, states, spheres);
    });
}

gbl_result gbl_batch_create(int precision, gbl_batch **out) {
    return gbl::guard([&] {
        if (!out) gbl::invalid("null argument");
        if (!gbl_available()) gbl::runtime("no CUDA device is available for the lattice backend");
        auto b = std::make_unique<gbl_batch>();
        if (precision == GBL_PRECISION_DOUBLE) b->impl = std::make_unique<gbl::Batch<double>>();
        else if (precision == GBL_PRECISION_FLOAT) b->impl = std::make_unique<gbl::Batch<float>>();
        else gbl::invalid("unknown precision");
        *out = b.release();
    });
}

void gbl_batch_destroy(gbl_batch *batch) { delete batch; }

gbl_result gbl_batch_add(gbl_batch *batch, const gbl_schedule_view *schedule, const gbl_state_view *state,
                         const gbl_sphere *sphere, uint32_t *index) {
    return gbl::guard([&] {
        if (!batch || !schedule || !state || !sphere) gbl::invalid("null argument");
        const std::size_t k = batch->impl->add(gbl::Schedule::fromView(*schedule), *state, *sphere);
        if (index) *index = static_cast<uint32_t>(k);
    });
}

gbl_result gbl_batch_settle(gbl_batch *batch, const gbl_step_settings *settings) {
    return gbl::guard([&] {
        if (!batch || !settings) gbl::invalid("null argument");
        batch->impl->settle(*settings);
    });
}

gbl_result gbl_batch_set_external_forces(gbl_batch *batch, uint32_t index, const double *forces, uint64_t count,
                                         uint64_t substeps) {
    return gbl::guard([&] {
        if (!batch) gbl::invalid("null batch");
        batch->impl->setExternalForces(index, forces, count, substeps);
    });
}

gbl_result gbl_batch_set_external_wrenches(gbl_batch *batch, uint32_t index, const gbl_external_wrench *wrenches,
                                           uint64_t count, uint64_t substeps) {
    return gbl::guard([&] {
        if (!batch) gbl::invalid("null batch");
        batch->impl->setExternalWrenches(index, wrenches, count, substeps);
    });
}

gbl_result gbl_batch_external_source_count(gbl_batch *batch, uint32_t index, uint64_t *count) {
    return gbl::guard([&] {
        if (!batch || !count) gbl::invalid("null argument");
        *count = batch->impl->sources(index).size();
    });
}

gbl_result gbl_batch_external_source(gbl_batch *batch, uint32_t index, uint64_t source, char *name,
                                     size_t name_capacity, size_t *name_length, gbl_load_ledger *load) {
    return gbl::guard([&] {
        if (!batch) gbl::invalid("null batch");
        gbl::sourceOut(batch->impl->sources(index), source, name, name_capacity, name_length, load);
    });
}

gbl_result gbl_batch_tune(gbl_batch *batch, gbl_tuning *chosen) {
    return gbl::guard([&] {
        if (!batch) gbl::invalid("null batch");
        const gbl_tuning t = batch->impl->tune();
        if (chosen) *chosen = t;
    });
}

gbl_result gbl_batch_set_tuning(gbl_batch *batch, const gbl_tuning *shape) {
    return gbl::guard([&] {
        if (!batch || !shape) gbl::invalid("null argument");
        batch->impl->setShape(*shape);
    });
}

gbl_result gbl_batch_run(gbl_batch *batch, const gbl_run_control *control) {
    return gbl::guard([&] {
        if (!batch || !control) gbl::invalid("null argument");
        batch->impl->run(*control);
    });
}

gbl_result gbl_batch_size(const gbl_batch *batch, uint32_t *count) {
    return gbl::guard([&] {
        if (!batch || !count) gbl::invalid("null argument");
        *count = static_cast<uint32_t>(batch->impl->size());
    });
}

gbl_result gbl_batch_status(gbl_batch *batch, uint32_t index, gbl_run_status *status_out) {
    return gbl::guard([&] {
        if (!batch || !status_out) gbl::invalid("null argument");
        *status_out = batch->impl->status(index);
    });
}

gbl_result gbl_batch_download(gbl_batch *batch, uint32_t index, gbl_state_view *state, gbl_sphere *sphere) {
    return gbl::guard([&] {
        if (!batch || !state) gbl::invalid("null argument");
        batch->impl->download(index, *state, sphere);
    });
}

gbl_result gbl_batch_first_failure_bonds(gbl_batch *batch, uint32_t index, uint32_t *out, uint64_t capacity,
                                         uint64_t *count) {
    return gbl::guard([&] {
        if (!batch || !count) gbl::invalid("null argument");
        const auto f = batch->impl->firstFailure(index);
        *count = f.size();
        if (out) std::memcpy(out, f.data(), sizeof(uint32_t) * std::min<std::uint64_t>(capacity, f.size()));
    });
}

gbl_result gbl_batch_profile_phases(gbl_batch *batch, uint64_t substeps, double *phase_ms) {
    return gbl::guard([&] {
        if (!batch || !phase_ms) gbl::invalid("null argument");
        batch->impl->profile(substeps, phase_ms);
    });
}

gbl_result gbl_batch_kernels_per_substep(gbl_batch *batch, uint64_t *count) {
    return gbl::guard([&] {
        if (!batch || !count) gbl::invalid("null argument");
        *count = batch->impl->kernelsPerSubstep();
    });
}

gbl_result gbl_batch_set_stream(gbl_batch *batch, void *cuda_stream) {
    return gbl::guard([&] {
        if (!batch) gbl::invalid("null batch");
        batch->impl->setStream(static_cast<cudaStream_t>(cuda_stream));
    });
}

gbl_result gbl_serve_create(int precision, const gbl_step_settings *settings, uint64_t budget_bytes, gbl_server **out) {
    return gbl::guard([&] {
        if (!settings || !out) gbl::invalid("null argument");
        if (!gbl_available()) gbl::runtime("no CUDA device is available for the lattice backend");
        auto s = std::make_unique<gbl_server>();
        if (precision == GBL_PRECISION_DOUBLE) s->impl = std::make_unique<gbl::Server<double>>(*settings, budget_bytes);
        else if (precision == GBL_PRECISION_FLOAT) s->impl = std::make_unique<gbl::Server<float>>(*settings, budget_bytes);
        else gbl::invalid("unknown precision");
        *out = s.release();
    });
}

void gbl_serve_destroy(gbl_server *server) { delete server; }

gbl_result gbl_serve_submit(gbl_server *server, const gbl_schedule_view *schedule, const gbl_state_view *state,
                            const gbl_sphere *sphere, uint64_t substeps, uint64_t *ticket) {
    return gbl::guard([&] {
        if (!server || !schedule || !state || !sphere || !ticket) gbl::invalid("null argument");
        *ticket = server->impl->submit(*schedule, *state, *sphere, substeps, false);
    });
}

gbl_result gbl_serve_submit_borrowed(gbl_server *server, const gbl_schedule_view *schedule,
                                     const gbl_state_view *state, const gbl_sphere *sphere, uint64_t substeps,
                                     uint64_t *ticket) {
    return gbl::guard([&] {
        if (!server || !schedule || !state || !sphere || !ticket) gbl::invalid("null argument");
        *ticket = server->impl->submit(*schedule, *state, *sphere, substeps, true);
    });
}

gbl_result gbl_serve_step(gbl_server *server, uint64_t substeps, gbl_server_stats *stats) {
    return gbl::guard([&] {
        if (!server) gbl::invalid("null server");
        server->impl->step(substeps, stats);
    });
}

gbl_result gbl_serve_poll(gbl_server *server, uint64_t ticket, gbl_request_info *info) {
    return gbl::guard([&] {
        if (!server || !info) gbl::invalid("null argument");
        server->impl->poll(ticket, *info);
    });
}

gbl_result gbl_serve_take(gbl_server *server, uint64_t ticket, gbl_state_view *state, gbl_sphere *sphere,
                          gbl_run_status *status) {
    return gbl::guard([&] {
        if (!server) gbl::invalid("null server");
        server->impl->take(ticket, state, sphere, status);
    });
}

gbl_result gbl_serve_cancel(gbl_server *server, uint64_t ticket) {
    return gbl::guard([&] {
        if (!server) gbl::invalid("null server");
        server->impl->cancel(ticket);
    });
}

gbl_result gbl_serve_stats(gbl_server *server, gbl_server_stats *stats) {
    return gbl::guard([&] {
        if (!server || !stats) gbl::invalid("null argument");
        server->impl->stats(*stats);
    });
}

gbl_result gbl_serve_set_lane_threshold(gbl_server *server, uint32_t bonds) {
    return gbl::guard([&] {
        if (!server) gbl::invalid("null argument");
        if (bonds == 0) gbl::invalid("the large lane's threshold must be at least one bond");
        server->impl->setLaneThreshold(bonds);
    });
}

gbl_result gbl_serve_footprint(int precision, uint32_t node_count, uint32_t bond_count, uint32_t max_degree,
                               uint32_t block_count, uint64_t *bytes) {
    return gbl::guard([&] {
        if (!bytes) gbl::invalid("null argument");
        if (precision == GBL_PRECISION_DOUBLE)
            *bytes = gbl::Resident<double>::footprint(node_count, bond_count, max_degree, block_count);
        else if (precision == GBL_PRECISION_FLOAT)
            *bytes = gbl::Resident<float>::footprint(node_count, bond_count, max_degree, block_count);
        else gbl::invalid("unknown precision");
    });
}

gbl_result gbl_bounds_report(uint64_t report[4], int *checked) {
    return gbl::guard([&] {
        if (!report || !checked) gbl::invalid("null argument");
#ifdef GBL_BOUNDS_CHECK
        *checked = 1;
        unsigned long long v[4] = {};
        gbl::check(cudaMemcpyFromSymbol(v, gbl::g_bounds_violation, sizeof(v)), "bounds record");
        for (int k = 0; k < 4; ++k) report[k] = v[k];
#else
        *checked = 0;
        for (int k = 0; k < 4; ++k) report[k] = 0;
#endif
    });
}

gbl_result gbl_bounds_clear(void) {
    return gbl::guard([&] {
#ifdef GBL_BOUNDS_CHECK
        const unsigned long long zero[4] = {};
        gbl::check(cudaMemcpyToSymbol(gbl::g_bounds_violation, zero, sizeof(zero)), "bounds record");
#endif
    });
}

} // extern "C"
