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

// Features of a candidate swap of columns 1 and 2 at frame y for the learned
// pair proposal, from the two atoms a1, a2 and their neighbours at frames
// y - 1 (p) and y + 1 (n): position difference (x, y) and distance in units
// of 16 px, colour difference (r, g, b, a) of the atoms' key-frame pixels,
// each column's current cost log1p(d(p, a) + d(a, n)) / (16 px)^2, and the
// parity of the two atoms' HAS_PIXEL flags.  What the swap would cost (the
// label's other half) is not among them.
__device__ __forceinline__ void pair_features(uint64_t a1, uint64_t a2, uint64_t p1, uint64_t n1, uint64_t p2,
                                              uint64_t n2, uint32_t col1, uint32_t col2, float *f) {
    constexpr float inv_s = 1.f / 4096.f, inv_s2 = 1.f / (4096.f * 4096.f);
    const float dx = (float)(pt_X(a1) - pt_X(a2)), dy = (float)(pt_Y(a1) - pt_Y(a2));
    f[0] = dx * inv_s;
    f[1] = dy * inv_s;
#pragma unroll
    for (int ch = 0; ch < 4; ++ch)
        f[2 + ch] = ((float)((col1 >> (8 * ch)) & 255u) - (float)((col2 >> (8 * ch)) & 255u)) * (1.f / 255.f);
    f[6] = log1pf((float)(pt_dist(p1, a1) + pt_dist(a1, n1)) * inv_s2);
    f[7] = log1pf((float)(pt_dist(p2, a2) + pt_dist(a2, n2)) * inv_s2);
    f[8] = (float)(((pt_flags(a1) ^ pt_flags(a2)) & kHasPixel) ? 1 : 0);
    f[9] = sqrtf(dx * dx + dy * dy) * inv_s;
}
// Key-frame colour under atom w at frame y (0 outside the canvas).
__device__ __forceinline__ uint32_t atom_colour(const uint32_t *display, uint32_t CW, uint32_t CH, uint32_t y,
                                                uint64_t w) {
    const uint32_t x = pt_x(w), yy = pt_y(w);
    return (x < CW && yy < CH) ? __ldg(display + ((size_t)y * CH + yy) * CW + x) : 0u;
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
    if (a.log_feat && mix64(a.key ^ (r * 0x9E3779B97F4A7C15ull) ^ y) % a.log_every == 0) {
        const unsigned long long at = atomicAdd(a.log_count, 1ull);
        if (at < a.log_cap) {
            float f[kMlpIn];
            pair_features(a1, a2, p1, n1, p2, n2, atom_colour(a.display, a.CW, a.CH, y, a1),
                          atom_colour(a.display, a.CW, a.CH, y, a2), f);
#pragma unroll
            for (int k = 0; k < kMlpIn; ++k) a.log_feat[at * kMlpIn + k] = f[k];
            // the reference's criterion also accepts ties (c1 == c2), which gain
            // nothing; the label marks the swaps that lower the cost
            a.log_label[at] = c1 > c2 ? 1.f : 0.f;
        }
    }
    if (c1 >= c2) {
        Py[x1] = a2;
        Py[x2] = a1;
        gain += c1 - c2;
        acc += 1;
    }
}

}  // namespace amg
