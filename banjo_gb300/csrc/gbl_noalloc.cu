// Broken-bond listing that allocates nothing.
//
// Some callers of this library must not allocate device memory while they
// run: a game or tool's real-time frame loop, where cudaMalloc/cudaFree
// synchronise the device and stall the frame, or a caller that records its
// frame's work into a CUDA graph, where allocation calls cannot be captured.
// Such a caller still wants the set of bonds a fracture round removed, in
// schedule order, from aliveness snapshots it already holds on the device.
//
// This file is the variant of the library's ordered event compaction (the
// per-tile counts, their exclusive scan and the in-order emission) whose
// per-tile scratch lives in a file-scope static device array instead of an
// allocation. Its size is fixed: kMaxBonds bonds (64 KiB of tile counts).
// Every GPU that loads the library holds the array until the process exits.
//
// Every call shares that one array and it keeps the last call's contents;
// each call overwrites every tile count it reads before reading it, so nothing
// needs clearing between calls. Two calls whose work overlaps on the GPU (on
// different streams, or from different host threads without ordering) race on
// the array and may return wrong lists: order them on one stream.
#include "gbl_internal.hpp"

#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <string>

namespace gbl {

// The current context's unique ID, or 0 when none is current or the driver
// cannot say. The two driver calls are reached through the runtime's entry
// point table, so the library does not link the driver library itself.
unsigned long long currentContextId() {
    using GetCurrent = int (*)(void **);
    using GetId = int (*)(void *, unsigned long long *);
    struct Calls {
        GetCurrent get_current{};
        GetId get_id{};
    };
    static const Calls calls = [] {
        Calls c;
        void *a = nullptr, *b = nullptr;
        cudaDriverEntryPointQueryResult qa{}, qb{};
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000, cudaEnableDefault, &qa) == cudaSuccess &&
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &qb) == cudaSuccess &&
            qa == cudaDriverEntryPointSuccess && qb == cudaDriverEntryPointSuccess) {
            c.get_current = reinterpret_cast<GetCurrent>(a);
            c.get_id = reinterpret_cast<GetId>(b);
        }
        return c;
    }();
    if (!calls.get_current || !calls.get_id) return 0;
    void *ctx = nullptr;
    unsigned long long id = 0;
    if (calls.get_current(&ctx) != 0 || !ctx || calls.get_id(ctx, &id) != 0) return 0;
    return id;
}

namespace {

constexpr unsigned kNoAllocThreads = 256;
constexpr unsigned kNoAllocRounds = 32;                           // bonds per thread per tile
constexpr unsigned kNoAllocTile = kNoAllocThreads * kNoAllocRounds; // 8192 bonds per CTA
constexpr std::uint64_t kNoAllocMaxBonds = 1ULL << 27;            // 134,217,728 bonds
constexpr unsigned kNoAllocMaxTiles = static_cast<unsigned>(kNoAllocMaxBonds / kNoAllocTile); // 16384

// The scratch: one count, then one offset, per tile of 8192 bonds.
static __device__ __align__(256) std::uint32_t g_noalloc_tiles[kNoAllocMaxTiles];

__device__ __forceinline__ bool brokeBetween(const std::uint8_t *before, const std::uint8_t *after, std::uint64_t j,
                                             std::uint64_t n) {
    return j < n && before[j] != 0 && after[j] == 0;
}

// Pass 1: broken bonds per tile.
__global__ void __launch_bounds__(kNoAllocThreads)
kNoAllocCount(const std::uint8_t *before, const std::uint8_t *after, std::uint64_t n, std::uint32_t *tiles) {
    __shared__ unsigned warp_sum[kNoAllocThreads / 32];
    const std::uint64_t base = static_cast<std::uint64_t>(blockIdx.x) * kNoAllocTile;
    unsigned count = 0;
    for (unsigned r = 0; r < kNoAllocRounds; ++r)
        count += __popc(__ballot_sync(0xffffffffU, brokeBetween(before, after, base + r * kNoAllocThreads + threadIdx.x, n)));
    if ((threadIdx.x & 31) == 0) warp_sum[threadIdx.x / 32] = count;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned total = 0;
        for (unsigned w = 0; w < kNoAllocThreads / 32; ++w) total += warp_sum[w];
        tiles[blockIdx.x] = total;
    }
}

// Pass 2: exclusive scan of the tile counts in place, one CTA; the total is
// the caller's count.
__global__ void __launch_bounds__(1024) kNoAllocScan(std::uint32_t *tiles, unsigned tile_count, std::uint32_t *total) {
    __shared__ unsigned warp_sum[32];
    const unsigned per = (tile_count + blockDim.x - 1) / blockDim.x;
    const unsigned first = threadIdx.x * per;
    unsigned local = 0;
    for (unsigned t = first; t < first + per && t < tile_count; ++t) local += tiles[t];
    unsigned x = local;
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned y = __shfl_up_sync(0xffffffffU, x, o);
        if ((threadIdx.x & 31) >= static_cast<unsigned>(o)) x += y;
    }
    if ((threadIdx.x & 31) == 31) warp_sum[threadIdx.x / 32] = x;
    __syncthreads();
    if (threadIdx.x < 32) {
        unsigned s = warp_sum[threadIdx.x];
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned y = __shfl_up_sync(0xffffffffU, s, o);
            if (threadIdx.x >= static_cast<unsigned>(o)) s += y;
        }
        warp_sum[threadIdx.x] = s;
    }
    __syncthreads();
    unsigned run = x - local + (threadIdx.x >= 32 ? warp_sum[threadIdx.x / 32 - 1] : 0U);
    for (unsigned t = first; t < first + per && t < tile_count; ++t) {
        const unsigned c = tiles[t];
        tiles[t] = run;
        run += c;
    }
    if (threadIdx.x == blockDim.x - 1) *total = run;
}

// Pass 3: each tile writes its broken bonds, in bond order, from its offset.
__global__ void __launch_bounds__(kNoAllocThreads)
kNoAllocEmit(const std::uint8_t *before, const std::uint8_t *after, std::uint64_t n, const std::uint32_t *tiles,
             std::uint32_t *out) {
    __shared__ unsigned warp_sum[kNoAllocThreads / 32];
    __shared__ unsigned carry;
    const std::uint64_t base = static_cast<std::uint64_t>(blockIdx.x) * kNoAllocTile;
    if (threadIdx.x == 0) carry = tiles[blockIdx.x];
    __syncthreads();
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x / 32;
    for (unsigned r = 0; r < kNoAllocRounds; ++r) {
        const std::uint64_t j = base + r * kNoAllocThreads + threadIdx.x;
        const bool hit = brokeBetween(before, after, j, n);
        const unsigned bits = __ballot_sync(0xffffffffU, hit);
        if (lane == 0) warp_sum[warp] = __popc(bits);
        __syncthreads();
        unsigned before_warp = 0, round_total = 0;
        for (unsigned w = 0; w < kNoAllocThreads / 32; ++w) {
            if (w < warp) before_warp += warp_sum[w];
            round_total += warp_sum[w];
        }
        if (hit) out[carry + before_warp + __popc(bits & ((1U << lane) - 1U))] = static_cast<std::uint32_t>(j);
        __syncthreads();
        if (threadIdx.x == 0) carry += round_total;
        __syncthreads();
    }
}

// Device address of the scratch array: in host code the array's name is only
// a host-side stand-in. The address belongs to the context the module was
// loaded into, so it is kept per device together with that context's unique
// ID (cuCtxGetId, which a context created after a device reset does not
// share) and looked up again when the current context is another one.
std::mutex g_setup_mutex;
constexpr int kMaxDevices = 64;
struct ScratchAddress {
    unsigned long long context{};
    std::uint32_t *address{};
};
ScratchAddress g_scratch[kMaxDevices];

std::uint32_t *scratchForCurrentDevice() {
    int device = 0;
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess) runtime(std::string("no current CUDA device: ") + cudaGetErrorString(e));
    if (device < 0 || device >= kMaxDevices) runtime("CUDA device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    ScratchAddress &slot = g_scratch[device];
    const unsigned long long context = currentContextId();
    if (slot.address && context != 0 && context == slot.context) return slot.address;
    void *ptr = nullptr;
    e = cudaGetSymbolAddress(&ptr, g_noalloc_tiles); // makes the device's context current if none was
    if (e != cudaSuccess || !ptr)
        runtime(std::string("cannot resolve the static scratch array: ") + cudaGetErrorString(e));
    slot.address = static_cast<std::uint32_t *>(ptr);
    slot.context = currentContextId();
    return slot.address;
}

} // namespace
} // namespace gbl

extern "C" gbl_result gbl_broken_between_noalloc(const uint8_t *alive_before, const uint8_t *alive_after,
                                                 uint64_t bond_count, uint32_t *broken, uint32_t *broken_count,
                                                 void *cuda_stream) {
    return gbl::guard([&] {
        if (bond_count > gbl::kNoAllocMaxBonds)
            gbl::invalid("gbl_broken_between_noalloc handles at most 134217728 bonds (its static scratch holds "
                         "16384 tiles of 8192); got " + std::to_string(bond_count));
        if (!broken_count || (bond_count && (!alive_before || !alive_after || !broken)))
            gbl::invalid("gbl_broken_between_noalloc needs device pointers for both snapshots and both outputs");
        cudaStream_t stream = static_cast<cudaStream_t>(cuda_stream);
        // An error already pending belongs to earlier work: report it without
        // clearing it, and launch nothing.
        const cudaError_t pending = cudaPeekAtLastError();
        if (pending != cudaSuccess)
            gbl::runtime(std::string("an earlier CUDA error is pending, nothing was listed: ") +
                         cudaGetErrorString(pending));
        std::uint32_t *tiles = gbl::scratchForCurrentDevice();
        if (bond_count == 0) {
            const cudaError_t e = cudaMemsetAsync(broken_count, 0, sizeof(std::uint32_t), stream);
            if (e != cudaSuccess) gbl::runtime(std::string("count reset: ") + cudaGetErrorString(e));
            return;
        }
        const unsigned tile_count = static_cast<unsigned>((bond_count + gbl::kNoAllocTile - 1) / gbl::kNoAllocTile);
        gbl::kNoAllocCount<<<tile_count, gbl::kNoAllocThreads, 0, stream>>>(alive_before, alive_after, bond_count, tiles);
        gbl::kNoAllocScan<<<1, 1024, 0, stream>>>(tiles, tile_count, broken_count);
        gbl::kNoAllocEmit<<<tile_count, gbl::kNoAllocThreads, 0, stream>>>(alive_before, alive_after, bond_count, tiles,
                                                                            broken);
        // Nothing was pending before the launches, so an error now is theirs.
        const cudaError_t e = cudaPeekAtLastError();
        if (e != cudaSuccess) {
            (void)cudaGetLastError();
            gbl::runtime(std::string("broken-bond listing launch: ") + cudaGetErrorString(e));
        }
    });
}
