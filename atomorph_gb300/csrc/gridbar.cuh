// Grid-wide barrier of the persistent cooperative launches (k_batch.cu,
// k_local.cu).  Words: bar[0] arrivals, bar[1] generation, bar[2] abort, all
// zeroed before the launch.  The wait is bounded: a CTA that polls longer than
// kBarrierTries times (about a second) sets err and the abort flag, and every
// CTA leaves at its next barrier; the host reports AM_ERR_TIMEOUT.  The
// launches are cooperative, so all CTAs are co-resident and a barrier never
// waits on a CTA that has not started.
#pragma once

#include "common.cuh"

namespace amg {

constexpr uint32_t kBarrierTries = 1u << 24;  // x ~64 ns sleep: about a second

__device__ __forceinline__ bool grid_barrier(unsigned *bar, int *err) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        ok = 1;
        volatile unsigned *gen = bar + 1;
        volatile int *abort_flag = (volatile int *)(bar + 2);
        unsigned g = *gen;
        __threadfence();
        if (atomicAdd(bar, 1u) == gridDim.x - 1) {
            atomicExch(bar, 0u);
            __threadfence();
            atomicAdd(bar + 1, 1u);
        } else {
            uint32_t tries = 0;
            while (*gen == g) {
                if (*abort_flag) { ok = 0; break; }
                if (++tries > kBarrierTries) {
                    atomicExch(err, AM_ERR_TIMEOUT);
                    atomicExch((int *)(bar + 2), 1);
                    ok = 0;
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
    }
    __syncthreads();
    return ok;
}

}  // namespace amg
