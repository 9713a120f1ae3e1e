// Allocation-free exact atom cost (am_get_cost_noalloc; the reference has no
// counterpart — its cost, thread::get_energy, thread.cpp:1109-1125, is a host
// loop over its own chains).
//
// Who needs it: a caller that polls the refinement's cost while other work
// runs on the device.  cudaMalloc and cudaFree may synchronise the whole
// device, so a first-use allocation would stall every stream in flight
// (frames being rendered and presented, another handle's refinement), and a
// caller that sized its device memory up front has no room for new buffers.
// am_get_cost may allocate its accumulator on first use; this variant keeps
// its scratch in one file-scope device array and allocates nothing.
//
// Scratch: kCostPartials partial sums, one per chunk of kCostChunk columns
// (a column = one atom at one key frame), and one result word.  The largest
// chains it accepts therefore hold kCostPartials * kCostChunk = 2^27 columns
// (134,217,728 — e.g. 16.7 M atoms over 8 key frames); larger ones are
// rejected with AM_ERR_ARG.  Every call overwrites all partials it reads and
// the result word, so nothing in the array has to start at zero.  All calls
// in the process share the array: two calls that overlap in time (two host
// threads, or two handles on different streams) race on it, and their
// callers must serialise them.
//
// Setup: the first call on each device, with that device current, looks up
// the array's device address once (cudaGetSymbolAddress) and caches it; make
// that first call before any stream capture begins.  Each call makes the
// handle's device current while it runs and restores the calling thread's
// current device before it returns.
#include <mutex>

#include "engine.h"

namespace amg {
namespace {

constexpr uint32_t kCostChunk = 2048;            // columns per partial sum (256 threads x 8)
constexpr uint32_t kCostPartials = 1u << 16;     // partial sums the array holds
constexpr uint64_t kCostMaxColumns = (uint64_t)kCostChunk * kCostPartials;
constexpr int kMaxDevices = 64;

// 512 KB + 8 B of device memory, part of the module image.
__device__ __align__(256) unsigned long long g_cost_scratch[kCostPartials + 1];

// partial[c] = sum of d(P[j][i], P[(j+1)%K][i]) over columns t = j*N + i of
// chunk c (thread.cpp:1117-1121); written, never accumulated.
__global__ void __launch_bounds__(256) k_cost_chunks(const uint64_t *__restrict__ P, uint64_t N, uint32_t K,
                                                     uint64_t nchunks, unsigned long long *partial) {
    __shared__ unsigned long long part[8];
    const uint64_t total = N * K;
    for (uint64_t c = blockIdx.x; c < nchunks; c += gridDim.x) {
        unsigned long long acc = 0;
        const uint64_t base = c * kCostChunk;
#pragma unroll
        for (uint32_t k = 0; k < kCostChunk / 256; ++k) {
            uint64_t t = base + (uint64_t)k * 256 + threadIdx.x;
            if (t < total) {
                uint32_t j = (uint32_t)(t / N);
                uint64_t i = t - (uint64_t)j * N;
                uint32_t jn = j + 1 == K ? 0 : j + 1;
                acc += pt_dist(__ldg(P + t), __ldg(P + (uint64_t)jn * N + i));
            }
        }
        acc = warp_sum_u64(acc);
        if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
        __syncthreads();
        if (threadIdx.x < 32) {
            unsigned long long v = threadIdx.x < 8 ? part[threadIdx.x] : 0ull;
            v = warp_sum_u64(v);
            if (threadIdx.x == 0) partial[c] = v;
        }
        __syncthreads();
    }
}

// result = sum of the partials minus the columns of width-1 chains, which
// cost nothing in the reference (thread.cpp:1113).  One CTA.
__global__ void __launch_bounds__(1024) k_cost_total(const unsigned long long *__restrict__ partial, uint64_t nchunks,
                                                     const uint64_t *__restrict__ P, uint64_t N, uint32_t K,
                                                     const uint64_t *__restrict__ single, uint32_t nsingle,
                                                     unsigned long long *result) {
    __shared__ unsigned long long part[32];
    unsigned long long acc = 0;
    for (uint64_t c = threadIdx.x; c < nchunks; c += blockDim.x) acc += partial[c];
    for (uint32_t s = threadIdx.x; s < nsingle; s += blockDim.x) {
        uint64_t i = single[s];
        for (uint32_t j = 0; j < K; ++j) acc -= pt_dist(P[(uint64_t)j * N + i], P[(uint64_t)((j + 1) % K) * N + i]);
    }
    acc = warp_sum_u64(acc);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        unsigned long long v = threadIdx.x < (blockDim.x >> 5) ? part[threadIdx.x] : 0ull;
        v = warp_sum_u64(v);
        if (threadIdx.x == 0) *result = v;
    }
}

std::mutex g_scratch_mu;
unsigned long long *g_scratch_ptr[kMaxDevices] = {};

// Device address of g_cost_scratch on the current device (looked up once).
int cost_scratch(unsigned long long **out) {
    int dev = 0;
    AMG_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) {
        set_error("am_get_cost_noalloc: device ordinal out of range");
        return AM_ERR_ARG;
    }
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_ptr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_cost_scratch);
        if (e != cudaSuccess || !p) {
            set_error(std::string("am_get_cost_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            return AM_ERR_CUDA;
        }
        g_scratch_ptr[dev] = (unsigned long long *)p;
    }
    *out = g_scratch_ptr[dev];
    return AM_OK;
}

}  // namespace

int Engine::compute_cost_noalloc(uint64_t *exact) {
    if (N == 0 || K == 0) { *exact = 0; return AM_OK; }
    const uint64_t total = N * K;
    if (total > kCostMaxColumns) {
        set_error("am_get_cost_noalloc: the chains hold " + std::to_string(total) +
                  " columns (atoms x key frames); the static scratch covers at most " +
                  std::to_string(kCostMaxColumns));
        return AM_ERR_ARG;
    }
    // The handle's device is made current for the call and the caller's
    // current device is put back on every return path.
    struct DeviceGuard {
        int prev = -1;
        ~DeviceGuard() {
            if (prev >= 0) cudaSetDevice(prev);
        }
    } guard;
    AMG_CUDA(cudaGetDevice(&guard.prev));
    if (guard.prev != device) AMG_CUDA(cudaSetDevice(device));
    unsigned long long *scratch = nullptr;
    int rc = cost_scratch(&scratch);
    if (rc) return rc;
    const uint64_t nchunks = (total + kCostChunk - 1) / kCostChunk;
    unsigned grid = (unsigned)std::min<uint64_t>(nchunks, (uint64_t)kSMs * 8);
    AMG_LAUNCH(k_cost_chunks, grid, 256, 0, stream, d_P.p, N, K, nchunks, scratch);
    AMG_LAUNCH(k_cost_total, 1, 1024, 0, stream, scratch, nchunks, d_P.p, N, K, d_singles.p,
               (uint32_t)singles.size(), scratch + kCostPartials);
    AMG_CUDA(cudaGetLastError());
    unsigned long long v = 0;
    AMG_CUDA(cudaMemcpyAsync(&v, scratch + kCostPartials, 8, cudaMemcpyDeviceToHost, stream));
    AMG_CUDA(cudaStreamSynchronize(stream));
    *exact = v;
    return AM_OK;
}

}  // namespace amg
