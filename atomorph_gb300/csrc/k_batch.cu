// Batched plain refinement: many morph jobs of uneven size refined by ONE
// persistent cooperative launch that runs every sweep and every phase.
//
// The reference refines one morph at a time, one chain per call
// (thread.cpp:1043-1068); C3-style workloads (dozens of jobs of 2k-200k
// atoms) leave a GB300 mostly idle when each job's small sweeps are launched
// separately.  Here the phases' work of all jobs is cut into chunks of
// `chunk` pairs (a chunk never spans two jobs), CTAs take chunks
// round-robin, and a grid barrier separates the phases (frames of one phase
// are never adjacent, so the pairs of one phase are independent).  Every
// pair runs sweep_pair with the job's own key, so the result is bit-identical
// to refining each job on its own, whatever the launch shape.
//
// The grid barrier (gridbar.cuh) is bounded, and the launch cooperative.
#include "common.cuh"
#include "kernels.h"
#include "gridbar.cuh"
#include "sweep.cuh"

namespace amg {
namespace {

__global__ void k_batch_sweeps(BatchArgs b) {
    __shared__ unsigned long long red[32];
    const int nphase = (int)b.nphase;
    for (uint32_t s = 0; s < b.sweeps; ++s) {
        for (int p = 0; p < nphase; ++p) {
            // (constant indices: a dynamic index into the parameter array would copy it to local memory)
            const uint32_t lo = p == 0 ? b.ch_off[0] : (p == 1 ? b.ch_off[1] : b.ch_off[2]);
            const uint32_t hi = p == 0 ? b.ch_off[1] : (p == 1 ? b.ch_off[2] : b.ch_off[3]);
            for (uint32_t ch = lo + blockIdx.x; ch < hi; ch += gridDim.x) {
                const uint32_t j = b.ch_job[ch];
                const BatchJob &J = b.jobs[j];
                SweepArgs a;
                a.P = J.P; a.N = J.N; a.K = J.K; a.C = J.C;
                a.chain_off = J.chain_off; a.pair_off = J.pair_off;
                a.frames = J.frames + J.ph_off[p]; a.nframes = J.ph_n[p];
                a.key = sweep_key(J.seed, J.sweep0 + s, (uint32_t)p);
                const uint64_t start = b.ch_start[ch], end = start + b.ch_count[ch];
                const uint32_t fi = b.ch_fi[ch];
                unsigned long long gain = 0, acc = 0;
                for (uint64_t r = start + threadIdx.x; r < end; r += blockDim.x) sweep_pair(a, fi, r, gain, acc);
                gain = warp_sum_u64(gain);
                if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = gain;
                __syncthreads();
                if (threadIdx.x < 32) {
                    unsigned long long v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0ull;
                    v = warp_sum_u64(v);
                    if (threadIdx.x == 0 && v) atomicAdd(b.gains + (uint64_t)j * b.sweeps + s, v);
                }
                __syncthreads();
            }
            const bool last = s + 1 == b.sweeps && p + 1 == nphase;
            if (!last && !grid_barrier(b.bar, b.err)) return;
        }
    }
}

}  // namespace

int batch_max_ctas_per_sm(uint32_t threads, int *out) {
    int n = 0;
    AMG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_batch_sweeps, (int)threads, 0));
    *out = n;
    return AM_OK;
}

int launch_batch_sweeps(const BatchArgs &b, uint32_t grid, uint32_t threads, cudaStream_t s) {
    if (b.sweeps == 0 || b.nphase == 0) return AM_OK;
    BatchArgs arg = b;
    void *params[] = {&arg};
    AMG_CUDA(cudaLaunchCooperativeKernel((const void *)k_batch_sweeps, dim3(grid), dim3(threads), params, 0, s));
    g_launches.fetch_add(1, std::memory_order_relaxed);
    return AM_OK;
}

}  // namespace amg
