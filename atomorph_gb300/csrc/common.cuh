// Shared device/host helpers of the atomorph_gb300 CUDA library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <string>
#include <vector>

namespace amg {

// ------------------------------------------------------------- errors -----
void set_error(const std::string &msg);       // per-thread last error text
extern std::atomic<uint64_t> g_launches;      // kernels launched by the library

#define AMG_CUDA(call)                                                              \
    do {                                                                            \
        cudaError_t e_ = (call);                                                    \
        if (e_ != cudaSuccess) {                                                    \
            ::amg::set_error(std::string(#call) + ": " + cudaGetErrorString(e_));   \
            return AM_ERR_CUDA;                                                     \
        }                                                                           \
    } while (0)

// Device allocation inside a function returning an AM_* status.  A failed
// cudaMalloc also leaves its error pending in the runtime (what the next
// cudaGetLastError reports); it is taken off here, so the caller's next call
// (which retries the allocation) is not failed by this one's error.
#define AMG_ALLOC(ptr, bytes)                                                       \
    do {                                                                            \
        cudaError_t e_ = cudaMalloc((ptr), (bytes));                                \
        if (e_ != cudaSuccess) {                                                    \
            cudaGetLastError();                                                     \
            *(ptr) = nullptr;                                                       \
            ::amg::set_error(std::string("cudaMalloc(" #ptr "): ") + cudaGetErrorString(e_)); \
            return AM_ERR_NOMEM;                                                    \
        }                                                                           \
    } while (0)

// Launch bookkeeping: every kernel launch goes through this so the process-wide
// launch counter (am_launch_count) is exact.
#define AMG_LAUNCH(kernel, grid, block, smem, stream, ...)                          \
    do {                                                                            \
        kernel<<<(grid), (block), (smem), (stream)>>>(__VA_ARGS__);                 \
        ::amg::g_launches.fetch_add(1, std::memory_order_relaxed);                  \
    } while (0)

constexpr int kSMs = 152;  // GB300: 2 dies x 76 SMs

// Opt-in per-kernel timing with CUDA events recorded on the launching stream
// around each launch; read back (and waited for) by collect().
enum ProfId {
    PROF_SPLAT, PROF_SCAN, PROF_SCATTER, PROF_RESOLVE, PROF_PAIR, PROF_SWEEP_RANDOM, PROF_SWEEP_LOCAL,
    PROF_MLP, PROF_FLUID, PROF_BIN, PROF_FLUID_MANAGE, PROF_FLUID_DRAW, PROF_COUNT
};
struct Prof {
    bool on = false;
    struct Span { int id; cudaEvent_t a, b; };
    std::vector<Span> pending;
    std::vector<cudaEvent_t> pool;
    double ms[PROF_COUNT] = {};
    uint64_t launches[PROF_COUNT] = {};
    cudaEvent_t open_ev = nullptr;
    cudaEvent_t take() {
        cudaEvent_t e = nullptr;
        if (pool.empty()) cudaEventCreate(&e);
        else { e = pool.back(); pool.pop_back(); }
        return e;
    }
    void open(cudaStream_t s) {
        if (!on) return;
        open_ev = take();
        cudaEventRecord(open_ev, s);
    }
    void close(int id, cudaStream_t s) {
        if (!on || !open_ev) return;
        cudaEvent_t b = take();
        cudaEventRecord(b, s);
        pending.push_back({id, open_ev, b});
        open_ev = nullptr;
    }
    void collect() {
        for (auto &sp : pending) {
            float t = 0.f;
            cudaEventSynchronize(sp.b);
            cudaEventElapsedTime(&t, sp.a, sp.b);
            ms[sp.id] += t;
            launches[sp.id] += 1;
            pool.push_back(sp.a);
            pool.push_back(sp.b);
        }
        pending.clear();
    }
    void reset() {
        collect();
        for (int i = 0; i < PROF_COUNT; ++i) { ms[i] = 0; launches[i] = 0; }
    }
    ~Prof() {
        for (auto &sp : pending) { cudaEventDestroy(sp.a); cudaEventDestroy(sp.b); }
        for (auto e : pool) cudaEventDestroy(e);
    }
};
extern const char *const kProfNames[PROF_COUNT];

// ------------------------------------------------------------- points -----
// The reference's 8-byte point word (atomorph.h:275-284), little-endian:
// bits 0-15 x, 16-31 y, 32-39 x_fract, 40-47 y_fract, 48-55 flags.
constexpr uint8_t kHasPixel = 1;
constexpr uint8_t kHasFluid = 2;

__host__ __device__ __forceinline__ int32_t pt_X(uint64_t w) {  // x in 1/256 px
    return (int32_t)(((w & 0xFFFFu) << 8) | ((w >> 32) & 0xFFu));
}
__host__ __device__ __forceinline__ int32_t pt_Y(uint64_t w) {
    return (int32_t)((((w >> 16) & 0xFFFFu) << 8) | ((w >> 40) & 0xFFu));
}
__host__ __device__ __forceinline__ uint32_t pt_x(uint64_t w) { return (uint32_t)(w & 0xFFFFu); }
__host__ __device__ __forceinline__ uint32_t pt_y(uint64_t w) { return (uint32_t)((w >> 16) & 0xFFFFu); }
__host__ __device__ __forceinline__ uint32_t pt_xf(uint64_t w) { return (uint32_t)((w >> 32) & 0xFFu); }
__host__ __device__ __forceinline__ uint32_t pt_yf(uint64_t w) { return (uint32_t)((w >> 40) & 0xFFu); }
__host__ __device__ __forceinline__ uint32_t pt_flags(uint64_t w) { return (uint32_t)((w >> 48) & 0xFFu); }
__host__ __device__ __forceinline__ uint64_t pt_make(uint32_t x, uint32_t y, uint32_t xf, uint32_t yf,
                                                     uint32_t flags) {
    return (uint64_t)(x & 0xFFFFu) | ((uint64_t)(y & 0xFFFFu) << 16) | ((uint64_t)(xf & 0xFFu) << 32) |
           ((uint64_t)(yf & 0xFFu) << 40) | ((uint64_t)(flags & 0xFFu) << 48);
}
// point_distance (atomorph.h:334-339): squared distance in 1/256 px, exact.
// Coordinates are below 2^24, so differences fit in 32 bits and every
// product is a 32 x 32 -> 64-bit multiply (64 x 64-bit integer multiplies
// are slow on GB300).
__host__ __device__ __forceinline__ uint64_t pt_dist(uint64_t a, uint64_t b) {
    const int32_t dx = pt_X(a) - pt_X(b);
    const int32_t dy = pt_Y(a) - pt_Y(b);
    return (uint64_t)((int64_t)dx * dx + (int64_t)dy * dy);
}

// Target sum s = p + n of a column (its points at the two neighbouring key
// frames), 1/256 px, x in the low word and y in the high word.
__host__ __device__ __forceinline__ uint64_t sums_pack(int32_t sx, int32_t sy) {
    return (uint64_t)(uint32_t)sx | ((uint64_t)(uint32_t)sy << 32);
}
__host__ __device__ __forceinline__ int32_t sums_x(uint64_t s) { return (int32_t)(uint32_t)s; }
__host__ __device__ __forceinline__ int32_t sums_y(uint64_t s) { return (int32_t)(uint32_t)(s >> 32); }

// Gain of exchanging the points a1, a2 of two columns at one key frame, in
// the reference's six-point criterion (thread.cpp:1014-1022):
//   c1 - c2 = d(p1,a1)+d(a1,n1)+d(p2,a2)+d(a2,n2) - d(p2,a1)-d(a1,n2)-d(p1,a2)-d(a2,n1)
//           = 2 (a1 - a2) . (s2 - s1),   s = p + n,
// since every squared norm appears once on each side.  Exact in int64:
// |a1 - a2| < 2^24 and |s2 - s1| < 2^25 per axis.
__host__ __device__ __forceinline__ int64_t pair_gain(uint64_t a1, uint64_t S1, uint64_t a2, uint64_t S2) {
    const int32_t dx = pt_X(a1) - pt_X(a2), dy = pt_Y(a1) - pt_Y(a2);
    const int32_t ex = sums_x(S2) - sums_x(S1), ey = sums_y(S2) - sums_y(S1);
    return 2 * ((int64_t)dx * ex + (int64_t)dy * ey);
}

// ------------------------------------------------------------ hashing -----
// Counter-based randomness: every random choice is a pure function of
// (seed, sweep, chain, frame, index), so a run is reproducible and a resumed
// run continues the same stream.
__host__ __device__ __forceinline__ uint32_t mix32(uint32_t x) {
    x ^= x >> 16; x *= 0x7feb352dU;
    x ^= x >> 15; x *= 0x846ca68bU;
    x ^= x >> 16;
    return x;
}
__host__ __device__ __forceinline__ uint64_t mix64(uint64_t x) {
    x ^= x >> 30; x *= 0xbf58476d1ce4e5b9ULL;
    x ^= x >> 27; x *= 0x94d049bb133111ebULL;
    x ^= x >> 31;
    return x;
}

// Bijection of [0, n) (n <= 2^31) keyed by `key`: a 4-round balanced Feistel
// network on the smallest even bit width covering n, with cycle walking.
__device__ __forceinline__ uint32_t permute_index(uint32_t x, uint32_t n, uint32_t half_bits, uint64_t key) {
    const uint32_t mask = (1u << half_bits) - 1u;
    const uint32_t k0 = (uint32_t)key, k1 = (uint32_t)(key >> 32);
    do {
        uint32_t L = x >> half_bits, R = x & mask;
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            uint32_t F = mix32(R ^ (r & 1 ? k1 : k0) ^ (0x9e3779b9u * (uint32_t)(r + 1))) & mask;
            uint32_t nL = R;
            R = L ^ F;
            L = nL;
        }
        x = (L << half_bits) | R;
    } while (x >= n);
    return x;
}
// Key of one (sweep, phase) of a job's plain refinement: a pure function of
// the job's seed and sweep counter, so batched and per-job sweeps draw the
// same pairs.
__host__ __device__ __forceinline__ uint64_t sweep_key(unsigned seed, uint64_t sweep, uint32_t phase) {
    return mix64(((uint64_t)seed << 40) ^ (sweep << 4) ^ phase);
}

__host__ __device__ __forceinline__ uint32_t half_bits_for(uint32_t n) {
    uint32_t b = 1;
    while ((1ull << b) < n) ++b;
    return (b + 1) / 2;
}

// ------------------------------------------------------------ reductions --
__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

}  // namespace amg
