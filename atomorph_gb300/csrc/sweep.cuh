// One proposal of the plain refinement, shared by the per-job sweep
// (k_chains.cu) and the batched persistent sweep (k_batch.cu) so the two are
// bit-identical.
#pragma once

#include "common.cuh"
#include "kernels.h"

namespace amg {

__device__ __forceinline__ uint32_t find_chain(const uint64_t *__restrict__ off, uint32_t C, uint64_t r) {
    // largest c with off[c] <= r (off[0] = 0, off[C] = total > r)
    uint32_t lo = 0, hi = C;
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) >> 1;
        if (__ldg(off + mid) <= r) lo = mid; else hi = mid;
    }
    return lo;
}

// Pair r of phase frame fi: frame y = frames[fi], pair r of the chains'
// disjoint random pairs (a keyed Feistel permutation of each chain's
// columns, consecutive positions paired).  The reference's criterion
// (thread.cpp:1014-1022), exact in integers: swap when c1 >= c2.
__device__ __forceinline__ void sweep_pair(const SweepArgs &a, uint32_t fi, uint64_t r, unsigned long long &gain,
                                           unsigned long long &acc) {
    uint32_t y = __ldg(a.frames + fi);
    uint32_t yn = y + 1 == a.K ? 0 : y + 1;
    uint32_t yp = y == 0 ? a.K - 1 : y - 1;
    uint32_t c = find_chain(a.pair_off, a.C, r);
    uint32_t i = (uint32_t)(r - __ldg(a.pair_off + c));
    uint64_t off = __ldg(a.chain_off + c);
    uint32_t w = (uint32_t)(__ldg(a.chain_off + c + 1) - off);
    uint64_t key = mix64(a.key ^ mix64(((uint64_t)c << 20) ^ y));
    uint32_t hb = half_bits_for(w);
    uint32_t x1 = permute_index(2 * i, w, hb, key);
    uint32_t x2 = permute_index(2 * i + 1, w, hb, key);
    uint64_t *Py = a.P + (uint64_t)y * a.N + off;
    const uint64_t *Pp = a.P + (uint64_t)yp * a.N + off;
    const uint64_t *Pn = a.P + (uint64_t)yn * a.N + off;
    uint64_t a1 = Py[x1], a2 = Py[x2];
    uint64_t p1 = Pp[x1], p2 = Pp[x2], n1 = Pn[x1], n2 = Pn[x2];
    uint64_t c1 = pt_dist(p1, a1) + pt_dist(a1, n1) + pt_dist(p2, a2) + pt_dist(a2, n2);
    uint64_t c2 = pt_dist(p2, a1) + pt_dist(a1, n2) + pt_dist(p1, a2) + pt_dist(a2, n1);
    if (c1 >= c2) {
        Py[x1] = a2;
        Py[x2] = a1;
        gain += c1 - c2;
        acc += 1;
    }
}

}  // namespace amg
