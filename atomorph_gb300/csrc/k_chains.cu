// Chain kernels: exact cost reduction, the plain refinement sweep, chain
// construction, and the stable radix sort the construction uses.
//
// Chains live in HBM frame-major: P[k * N + off_c + x] is point x of chain c
// at key frame k, the reference's 8-byte point word.  A refinement phase only
// writes frames that are not neighbours of each other, so the six points a
// swap reads (frames y-1, y, y+1) are stable while the phase runs and every
// pair is disjoint by construction: no locks, no atomics on points.
#include "common.cuh"
#include "kernels.h"
#include "sweep.cuh"

namespace amg {
namespace {

// ---------------------------------------------------------------- cost ----
__global__ void k_cost(const uint64_t *__restrict__ P, uint64_t N, uint32_t K, unsigned long long *out) {
    unsigned long long acc = 0;
    for (uint32_t j = 0; j < K; ++j) {
        const uint32_t jn = j + 1 == K ? 0 : j + 1;
        for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < N; i += (uint64_t)gridDim.x * blockDim.x)
            acc += pt_dist(__ldg(P + (uint64_t)j * N + i), __ldg(P + (uint64_t)jn * N + i));
    }
    acc = warp_sum_u64(acc);
    __shared__ unsigned long long part[32];
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        unsigned long long v = threadIdx.x < (blockDim.x >> 5) ? part[threadIdx.x] : 0ull;
        v = warp_sum_u64(v);
        if (threadIdx.x == 0 && v) atomicAdd(out, v);
    }
}

// Width-1 chains cost nothing in the reference (thread.cpp:1113).
__global__ void k_cost_sub(const uint64_t *__restrict__ P, uint64_t N, uint32_t K, const uint64_t *single,
                           uint32_t nsingle, unsigned long long *out) {
    uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nsingle) return;
    uint64_t i = single[s];
    unsigned long long acc = 0;
    for (uint32_t j = 0; j < K; ++j) acc += pt_dist(P[(uint64_t)j * N + i], P[(uint64_t)((j + 1) % K) * N + i]);
    if (acc) atomicAdd(out, (unsigned long long)(0ull - acc));
}

// ------------------------------------------------------- random sweep ----
__global__ void __launch_bounds__(256) k_sweep_random(SweepArgs a) {
    const uint64_t pairs = __ldg(a.pair_off + a.C);
    unsigned long long gain = 0, acc = 0;
    for (uint32_t fi = 0; fi < a.nframes; ++fi)
        for (uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r < pairs;
             r += (uint64_t)gridDim.x * blockDim.x)
            sweep_pair(a, fi, r, gain, acc);
    gain = warp_sum_u64(gain);
    acc = warp_sum_u64(acc);
    if ((threadIdx.x & 31) == 0) {
        if (gain) atomicAdd(a.gain, gain);
        if (acc) atomicAdd(a.accepted, acc);
    }
}

// --------------------------------------------------------- radix sort ----
constexpr int kRsThreads = 256;
constexpr int kRsTile = 2048;

__global__ void __launch_bounds__(kRsThreads) k_rs_hist(const uint32_t *__restrict__ keys, size_t n, int shift,
                                                         uint32_t *hist, uint32_t ntiles) {
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    size_t base = (size_t)blockIdx.x * kRsTile;
    for (int i = threadIdx.x; i < kRsTile; i += kRsThreads) {
        size_t g = base + i;
        if (g < n) atomicAdd(&h[(keys[g] >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[(size_t)threadIdx.x * ntiles + blockIdx.x] = h[threadIdx.x];
}

__global__ void __launch_bounds__(kRsThreads) k_rs_scatter(const uint32_t *__restrict__ kin,
                                                            const uint32_t *__restrict__ vin, uint32_t *kout,
                                                            uint32_t *vout, size_t n, int shift,
                                                            const uint32_t *__restrict__ hist, uint32_t ntiles) {
    __shared__ uint32_t base[256];
    __shared__ uint32_t wcnt[kRsThreads / 32][257];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    base[threadIdx.x] = hist[(size_t)threadIdx.x * ntiles + blockIdx.x];
    size_t tile = (size_t)blockIdx.x * kRsTile;
    for (int c = 0; c < kRsTile; c += kRsThreads) {
        for (int k = threadIdx.x; k < (kRsThreads / 32) * 257; k += kRsThreads) (&wcnt[0][0])[k] = 0;
        __syncthreads();
        size_t g = tile + c + threadIdx.x;
        bool valid = g < n;
        uint32_t key = valid ? kin[g] : 0u;
        uint32_t d = valid ? ((key >> shift) & 255u) : 256u;
        unsigned mask = __match_any_sync(0xffffffffu, d);
        int rank = __popc(mask & ((1u << lane) - 1u));
        if (rank == 0) wcnt[warp][d] = __popc(mask);
        __syncthreads();
        if (valid) {
            uint32_t pos = base[d] + rank;
            for (int w = 0; w < warp; ++w) pos += wcnt[w][d];
            kout[pos] = key;
            vout[pos] = vin[g];
        }
        __syncthreads();
        {
            uint32_t s = 0;
            for (int w = 0; w < kRsThreads / 32; ++w) s += wcnt[w][threadIdx.x];
            base[threadIdx.x] += s;
        }
        __syncthreads();
    }
}

// Single-CTA exclusive scan (setup-sized arrays).
__global__ void __launch_bounds__(1024) k_scan_u32(uint32_t *a, size_t n, uint32_t *total) {
    __shared__ uint32_t warp_tot[32];
    __shared__ uint32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (size_t base = 0; base < n; base += 1024) {
        size_t i = base + threadIdx.x;
        uint32_t v = i < n ? a[i] : 0u;
        uint32_t x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warp_tot[warp] = x;
        __syncthreads();
        if (warp == 0) {
            uint32_t t = warp_tot[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
                if (lane >= o) t += y;
            }
            warp_tot[lane] = t;
        }
        __syncthreads();
        uint32_t excl = carry + (warp ? warp_tot[warp - 1] : 0u) + x - v;
        if (i < n) a[i] = excl;
        __syncthreads();
        if (threadIdx.x == 1023) carry = excl + v;
        __syncthreads();
    }
    if (threadIdx.x == 0 && total) *total = carry;
}

// ------------------------------------------------------- chain build -----
__global__ void k_chain_build(ChainBuildArgs a) {
    const uint64_t total = a.N * a.K;
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < total;
         t += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t k = (uint32_t)(t / a.N);
        uint64_t gi = t - (uint64_t)k * a.N;
        uint32_t c = find_chain(a.chain_off, a.C, gi);
        uint32_t x = (uint32_t)(gi - a.chain_off[c]);
        int32_t b = a.blob_of[(size_t)k * a.C + c];
        uint32_t sz = b >= 0 ? a.blob_size[(size_t)k * a.maxb + b] : 0u;
        uint64_t key = mix64(a.seed ^ mix64(((uint64_t)c << 24) ^ (uint64_t)k));
        uint64_t word;
        if (sz == 0) {
            // Empty blob: one volatile point at the interpolated centre,
            // HAS_FLUID only; its duplicates carry no flags (thread.cpp:824-848).
            uint32_t xy = a.vol_xy[(size_t)k * a.C + c];
            if (x == 0) {
                word = pt_make(xy & 0xFFFF, xy >> 16, 0, 0, kHasFluid);
            } else {
                uint32_t r = mix32((uint32_t)key ^ mix32(x * 2654435761u));
                word = pt_make(xy & 0xFFFF, xy >> 16, r & 255u, (r >> 8) & 255u, 0);
            }
        } else {
            const uint32_t *surf = a.sorted + (size_t)k * a.npx + a.blob_start[(size_t)k * a.maxb + b];
            if (x < sz) {
                uint32_t p = surf[x];
                word = pt_make(p % a.CW, p / a.CW, 0, 0, kHasPixel | kHasFluid);
            } else {
                // Duplicates: the shuffled surface list taken cyclically,
                // random fractions, HAS_FLUID cleared.
                uint32_t j = permute_index(x % sz, sz, half_bits_for(sz), key);
                uint32_t p = surf[j];
                uint32_t r = mix32((uint32_t)(key >> 32) ^ mix32(x * 2246822519u + 7u));
                word = pt_make(p % a.CW, p / a.CW, r & 255u, (r >> 8) & 255u, kHasPixel);
            }
        }
        a.P[(uint64_t)k * a.N + gi] = word;
    }
}

__global__ void k_labels_to_keys(const int32_t *__restrict__ L, uint32_t *keys, size_t n, uint32_t nb) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        keys[i] = L[i] >= 0 ? (uint32_t)L[i] : nb;
}

}  // namespace

int labels_to_keys(const int32_t *labels, uint32_t *keys, size_t n, uint32_t nb, cudaStream_t s) {
    if (!n) return AM_OK;
    unsigned grid = (unsigned)std::min<size_t>((n + 255) / 256, (size_t)kSMs * 16);
    AMG_LAUNCH(k_labels_to_keys, grid, 256, 0, s, labels, keys, n, nb);
    AMG_CUDA(cudaGetLastError());
    return AM_OK;
}

int launch_cost(const uint64_t *P, uint64_t N, uint32_t K, const uint64_t *single, uint32_t nsingle,
                unsigned long long *out, cudaStream_t s) {
    AMG_CUDA(cudaMemsetAsync(out, 0, sizeof(unsigned long long), s));
    if (N == 0 || K == 0) return AM_OK;
    uint64_t total = N * K;
    unsigned grid = (unsigned)std::min<uint64_t>((total + 255) / 256, (uint64_t)kSMs * 8);
    AMG_LAUNCH(k_cost, grid, 256, 0, s, P, N, K, out);
    if (nsingle) AMG_LAUNCH(k_cost_sub, (nsingle + 127) / 128, 128, 0, s, P, N, K, single, nsingle, out);
    AMG_CUDA(cudaGetLastError());
    return AM_OK;
}

int launch_sweep_random(const SweepArgs &a, cudaStream_t s) {
    AMG_LAUNCH(k_sweep_random, (unsigned)(kSMs * 8), 256, 0, s, a);
    AMG_CUDA(cudaGetLastError());
    return AM_OK;
}

size_t radix_hist_words(size_t n) { return 256 * ((n + kRsTile - 1) / kRsTile) + 1; }

// Multi-CTA exclusive scan for large arrays: block sums of kScanBlock
// elements, a single-CTA scan of the sums, then each block's scan with its
// offset.
constexpr uint32_t kScanBlock = 4096;  // 1024 threads x 4

__device__ __forceinline__ uint32_t block_excl_scan_1024(uint32_t v, uint32_t *warp_tot, uint32_t *block_total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t t = warp_tot[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        warp_tot[lane] = t;
    }
    __syncthreads();
    const uint32_t excl = (warp ? warp_tot[warp - 1] : 0u) + x - v;
    if (block_total) *block_total = warp_tot[31];
    __syncthreads();
    return excl;
}

__global__ void __launch_bounds__(1024) k_scan_sums(const uint32_t *__restrict__ a, size_t n, uint32_t *sums) {
    __shared__ uint32_t warp_tot[32];
    const size_t base = (size_t)blockIdx.x * kScanBlock + (size_t)threadIdx.x * 4;
    uint32_t v = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k)
        if (base + k < n) v += a[base + k];
    uint32_t tot = 0;
    block_excl_scan_1024(v, warp_tot, &tot);
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(1024) k_scan_apply(uint32_t *a, size_t n, const uint32_t *__restrict__ offs) {
    __shared__ uint32_t warp_tot[32];
    const size_t base = (size_t)blockIdx.x * kScanBlock + (size_t)threadIdx.x * 4;
    uint32_t v[4], sum = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        v[k] = base + k < n ? a[base + k] : 0u;
        sum += v[k];
    }
    uint32_t run = block_excl_scan_1024(sum, warp_tot, nullptr) + offs[blockIdx.x];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (base + k < n) a[base + k] = run;
        run += v[k];
    }
}

int launch_scan_u32(uint32_t *a, size_t n, uint32_t *total, cudaStream_t s) {
    if (n <= 8 * (size_t)kScanBlock) {
        AMG_LAUNCH(k_scan_u32, 1, 1024, 0, s, a, n, total);
        AMG_CUDA(cudaGetLastError());
        return AM_OK;
    }
    static thread_local uint32_t *sums = nullptr;
    static thread_local size_t sums_cap = 0;
    const size_t nb = (n + kScanBlock - 1) / kScanBlock;
    if (nb + 1 > sums_cap) {
        if (sums) cudaFree(sums);
        sums = nullptr;
        sums_cap = 0;
        AMG_ALLOC(&sums, (nb + 1) * sizeof(uint32_t));
        sums_cap = nb + 1;
    }
    AMG_LAUNCH(k_scan_sums, (unsigned)nb, 1024, 0, s, a, n, sums);
    AMG_LAUNCH(k_scan_u32, 1, 1024, 0, s, sums, nb, total);
    AMG_LAUNCH(k_scan_apply, (unsigned)nb, 1024, 0, s, a, n, sums);
    AMG_CUDA(cudaGetLastError());
    return AM_OK;
}

int radix_sort_pairs(uint32_t *keys, uint32_t *vals, uint32_t *tk, uint32_t *tv, uint32_t *hist, size_t n,
                     int bits, cudaStream_t s) {
    if (n == 0) return AM_OK;
    uint32_t ntiles = (uint32_t)((n + kRsTile - 1) / kRsTile);
    uint32_t *ki = keys, *vi = vals, *ko = tk, *vo = tv;
    int passes = std::max(1, (bits + 7) / 8);
    for (int p = 0; p < passes; ++p) {
        int shift = 8 * p;
        AMG_LAUNCH(k_rs_hist, ntiles, kRsThreads, 0, s, ki, n, shift, hist, ntiles);
        int rc = launch_scan_u32(hist, (size_t)256 * ntiles, nullptr, s);
        if (rc) return rc;
        AMG_LAUNCH(k_rs_scatter, ntiles, kRsThreads, 0, s, ki, vi, ko, vo, n, shift, hist, ntiles);
        std::swap(ki, ko);
        std::swap(vi, vo);
    }
    if (ki != keys) {
        AMG_CUDA(cudaMemcpyAsync(keys, ki, n * 4, cudaMemcpyDeviceToDevice, s));
        AMG_CUDA(cudaMemcpyAsync(vals, vi, n * 4, cudaMemcpyDeviceToDevice, s));
    }
    AMG_CUDA(cudaGetLastError());
    return AM_OK;
}

int launch_chain_build(const ChainBuildArgs &a, cudaStream_t s) {
    uint64_t total = a.N * a.K;
    if (!total) return AM_OK;
    unsigned grid = (unsigned)std::min<uint64_t>((total + 255) / 256, (uint64_t)kSMs * 16);
    AMG_LAUNCH(k_chain_build, grid, 256, 0, s, a);
    AMG_CUDA(cudaGetLastError());
    return AM_OK;
}

}  // namespace amg
