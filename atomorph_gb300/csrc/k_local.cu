// Guided refinement: spatially local swap candidates, exact gains, and a
// disjoint set of swaps chosen by locally dominant claims.
//
// A swap at key frame y only exchanges which columns hold two of frame y's
// points (thread.cpp:1035-1037); the set of points of frame y never changes.
// So a spatial index of frame y's points, built once, stays valid while the
// refinement runs — only its column labels move, and the apply kernel moves
// them with the points:
//   slot_pt[y][s]   point of slot s (slots sorted by 2x2-pixel cell, static)
//   cell_start[y][] first slot of each cell
//   col[y][s]       column currently holding slot s
//   slot_of[y][x]   slot currently held by column x
// A column x1 at frame y costs d(p1,a1)+d(a1,n1) with p1/n1 its points at the
// neighbouring frames; it is cheapest where its point sits at m1 = (p1+n1)/2.
// Candidates come from the column's own neighbourhood, the cell of m1 and a
// few uniform random columns (k_local_propose); every
// candidate's gain is the reference's exact six-point criterion
// (thread.cpp:1014-1022) in integers.  Each column proposes its best strictly
// improving partner and claims both columns with atomicMax on
// (gain, proposer); a proposal is applied when it holds the claim of both
// columns, so applied swaps are disjoint and every applied gain is exact.
#include "common.cuh"
#include "kernels.h"

namespace amg {
namespace {

__device__ __forceinline__ uint32_t cell_of(uint64_t w, uint32_t ncx, uint32_t ncy) {
    uint32_t cx = min((uint32_t)pt_X(w) >> 9, ncx - 1), cy = min((uint32_t)pt_Y(w) >> 9, ncy - 1);
    return cy * ncx + cx;
}

__global__ void k_cell_keys(const uint64_t *__restrict__ Py, uint64_t N, uint32_t ncx, uint32_t ncy, uint32_t *keys,
                            uint32_t *vals) {
    for (uint64_t x = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; x < N; x += (uint64_t)gridDim.x * blockDim.x) {
        keys[x] = cell_of(Py[x], ncx, ncy);
        vals[x] = (uint32_t)x;
    }
}

// After sorting (keys, vals) by cell: slots, inverse map and cell counts.
__global__ void k_slots(const uint64_t *__restrict__ Py, const uint32_t *__restrict__ keys,
                        const uint32_t *__restrict__ vals, uint64_t N, uint64_t *slot_pt, uint32_t *col,
                        uint32_t *slot_of, uint32_t *cell_cnt) {
    for (uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; s < N; s += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t x = vals[s];
        slot_pt[s] = Py[x];
        col[s] = x;
        slot_of[x] = (uint32_t)s;
        atomicAdd(&cell_cnt[keys[s]], 1u);
    }
}

__global__ void k_chain_ids(const uint64_t *__restrict__ off, uint32_t C, uint64_t N, uint32_t *chain_id) {
    for (uint64_t x = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; x < N; x += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t lo = 0, hi = C;
        while (hi - lo > 1) {
            uint32_t mid = (lo + hi) >> 1;
            if (off[mid] <= x) lo = mid; else hi = mid;
        }
        chain_id[x] = lo;
    }
}

__device__ __forceinline__ int64_t swap_gain(uint64_t p1, uint64_t a1, uint64_t n1, uint64_t p2, uint64_t a2,
                                             uint64_t n2) {
    uint64_t c1 = pt_dist(p1, a1) + pt_dist(a1, n1) + pt_dist(p2, a2) + pt_dist(a2, n2);
    uint64_t c2 = pt_dist(p2, a1) + pt_dist(a1, n2) + pt_dist(p1, a2) + pt_dist(a2, n1);
    return (int64_t)c1 - (int64_t)c2;
}

// Monotone key: positive gains order like their float value; ties broken by
// the proposer's index.
__device__ __forceinline__ unsigned long long claim_key(int64_t gain, uint32_t x1) {
    float g = (float)gain;
    return ((unsigned long long)__float_as_uint(g) << 32) | x1;
}

// Scans up to `cap` slots of cell (qx, qy) starting at a hashed offset and
// keeps the best strictly improving partner.
__device__ __forceinline__ void scan_cell(const LocalArgs &a, const uint32_t *cs, const uint64_t *spt,
                                          const uint32_t *col, const uint64_t *Pp, const uint64_t *Pn, int qx, int qy,
                                          uint32_t cap, uint32_t h, uint32_t x1, uint32_t c, uint64_t p1,
                                          uint64_t a1, uint64_t n1, int64_t &best, uint32_t &bx) {
    if (qx < 0 || qy < 0 || qx >= (int)a.ncx || qy >= (int)a.ncy || cap == 0) return;
    uint32_t cell = (uint32_t)qy * a.ncx + (uint32_t)qx;
    uint32_t beg = cs[cell], n = cs[cell + 1] - beg;
    if (n == 0) return;
    uint32_t take = min(n, cap), start = n > cap ? h % n : 0;
    for (uint32_t j = 0; j < take; ++j) {
        uint32_t s = beg + (start + j) % n;
        uint32_t x2 = col[s];
        if (x2 == x1 || a.chain_id[x2] != c) continue;
        int64_t g = swap_gain(p1, a1, n1, Pp[x2], spt[s], Pn[x2]);
        if (g > best) { best = g; bx = x2; }
    }
}

// Candidates of column x1 at frame y, all checked with the exact criterion:
//   * the column's own neighbourhood (the cell of its point a1 and the four
//     cells around it): resolves the local crossings left after the coarse
//     transport is right, which uniform pairs almost never sample at large N;
//   * the cell of its target m1: moves a column straight to where its
//     neighbours in the other key frames pull it;
//   * a few uniform random columns of the same chain: the reference's own
//     proposal, for the coarse, long-range part.
__global__ void __launch_bounds__(256) k_local_propose(LocalArgs a) {
    const uint64_t N = a.N;
    const uint64_t total = N * a.nframes;
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < total; t += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t fi = (uint32_t)(t / N);
        uint32_t x1 = (uint32_t)(t - (uint64_t)fi * N);
        uint32_t y = a.frames[fi];
        uint32_t yn = y + 1 == a.K ? 0 : y + 1, yp = y == 0 ? a.K - 1 : y - 1;
        const uint64_t *Py = a.P + (uint64_t)y * N, *Pp = a.P + (uint64_t)yp * N, *Pn = a.P + (uint64_t)yn * N;
        a.prop[t] = 0xFFFFFFFFu;
        uint32_t c = a.chain_id[x1];
        if (a.chain_w1[c]) continue;  // width-1 chains do not refine (thread.cpp:1045)
        uint64_t a1 = Py[x1], p1 = Pp[x1], n1 = Pn[x1];
        const uint32_t *cs = a.cell_start + (uint64_t)y * (a.ncells + 1);
        const uint64_t *spt = a.slot_pt + (uint64_t)y * N;
        const uint32_t *col = a.col + (uint64_t)y * N;
        int64_t best = 0;
        uint32_t bx = 0xFFFFFFFFu;
        uint32_t h = mix32((uint32_t)a.key ^ mix32(x1 * 0x9E3779B1u + y));
        // own neighbourhood: centre cell, then the 4-neighbour cells
        int ax = (int)min((uint32_t)pt_X(a1) >> 9, a.ncx - 1), ay = (int)min((uint32_t)pt_Y(a1) >> 9, a.ncy - 1);
        if (a.self_cap) {
            uint32_t per = max(1u, a.self_cap / 3u);
            scan_cell(a, cs, spt, col, Pp, Pn, ax, ay, per, h, x1, c, p1, a1, n1, best, bx);
            const int dx4[4] = {1, -1, 0, 0}, dy4[4] = {0, 0, 1, -1};
            uint32_t r0 = h >> 28;
            for (int k = 0; k < 2; ++k) {
                int d = (int)((r0 + 2u * k) & 3u);
                scan_cell(a, cs, spt, col, Pp, Pn, ax + dx4[d], ay + dy4[d], per, h >> 3, x1, c, p1, a1, n1, best, bx);
            }
        }
        // target cell
        if (a.cap) {
            int32_t mx = (pt_X(p1) + pt_X(n1)) >> 1, my = (pt_Y(p1) + pt_Y(n1)) >> 1;
            int cx = (int)min((uint32_t)max(mx, 0) >> 9, a.ncx - 1), cy = (int)min((uint32_t)max(my, 0) >> 9, a.ncy - 1);
            scan_cell(a, cs, spt, col, Pp, Pn, cx, cy, a.cap, h >> 5, x1, c, p1, a1, n1, best, bx);
        }
        // uniform random partners in the same chain
        if (a.nrandom) {
            uint64_t off = a.chain_off[c];
            uint32_t w = (uint32_t)(a.chain_off[c + 1] - off);
            uint32_t r = h;
            for (uint32_t k = 0; k < a.nrandom; ++k) {
                r = mix32(r + 0x68E31DA4u);
                uint32_t x2 = (uint32_t)off + r % w;
                if (x2 == x1) continue;
                int64_t g = swap_gain(p1, a1, n1, Pp[x2], Py[x2], Pn[x2]);
                if (g > best) { best = g; bx = x2; }
            }
        }
        if (bx != 0xFFFFFFFFu) {
            unsigned long long k = claim_key(best, x1);
            a.prop[t] = bx;
            a.pgain[t] = (unsigned long long)best;
            atomicMax(a.claim + (uint64_t)fi * N + x1, k);
            atomicMax(a.claim + (uint64_t)fi * N + bx, k);
        }
    }
}

__global__ void __launch_bounds__(256) k_local_apply(LocalArgs a) {
    const uint64_t N = a.N;
    const uint64_t total = N * a.nframes;
    unsigned long long gain = 0, acc = 0;
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < total; t += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t x2 = a.prop[t];
        if (x2 == 0xFFFFFFFFu) continue;
        uint32_t fi = (uint32_t)(t / N);
        uint32_t x1 = (uint32_t)(t - (uint64_t)fi * N);
        unsigned long long k1 = a.claim[(uint64_t)fi * N + x1], k2 = a.claim[(uint64_t)fi * N + x2];
        if (k1 != k2 || (uint32_t)k1 != x1) continue;
        uint32_t y = a.frames[fi];
        uint64_t *Py = a.P + (uint64_t)y * N;
        uint32_t *slot_of = a.slot_of + (uint64_t)y * N, *col = a.col + (uint64_t)y * N;
        uint64_t w1 = Py[x1], w2 = Py[x2];
        Py[x1] = w2;
        Py[x2] = w1;
        uint32_t s1 = slot_of[x1], s2 = slot_of[x2];
        slot_of[x1] = s2;
        slot_of[x2] = s1;
        col[s1] = x2;
        col[s2] = x1;
        gain += a.pgain[t];
        acc += 1;
    }
    gain = warp_sum_u64(gain);
    acc = warp_sum_u64(acc);
    if ((threadIdx.x & 31) == 0) {
        if (gain) atomicAdd(a.gain, gain);
        if (acc) atomicAdd(a.accepted, acc);
    }
}

}  // namespace

int local_index_build(LocalIndex &ix, const uint64_t *P, uint64_t N, uint32_t K, uint32_t CW, uint32_t CH,
                      const uint64_t *chain_off, uint32_t C, uint32_t *keys, uint32_t *vals, uint32_t *tk,
                      uint32_t *tv, uint32_t *hist, cudaStream_t s) {
    ix.ncx = (CW + 1) / 2;
    ix.ncy = (CH + 1) / 2;
    ix.ncells = ix.ncx * ix.ncy;
    unsigned grid = (unsigned)std::min<uint64_t>((N + 255) / 256, (uint64_t)kSMs * 8);
    int bits = 1;
    while ((1ull << bits) < (uint64_t)ix.ncells) ++bits;
    AMG_CUDA(cudaMemsetAsync(ix.cell_start, 0, (size_t)K * (ix.ncells + 1) * 4, s));
    for (uint32_t y = 0; y < K; ++y) {
        const uint64_t *Py = P + (uint64_t)y * N;
        AMG_LAUNCH(k_cell_keys, grid, 256, 0, s, Py, N, ix.ncx, ix.ncy, keys, vals);
        int rc = radix_sort_pairs(keys, vals, tk, tv, hist, N, bits, s);
        if (rc) return rc;
        uint32_t *cs = ix.cell_start + (uint64_t)y * (ix.ncells + 1);
        AMG_LAUNCH(k_slots, grid, 256, 0, s, Py, keys, vals, N, ix.slot_pt + (uint64_t)y * N, ix.col + (uint64_t)y * N,
                   ix.slot_of + (uint64_t)y * N, cs);
        rc = launch_scan_u32(cs, (size_t)ix.ncells + 1, nullptr, s);
        if (rc) return rc;
    }
    AMG_LAUNCH(k_chain_ids, grid, 256, 0, s, chain_off, C, N, ix.chain_id);
    AMG_CUDA(cudaGetLastError());
    return AM_OK;
}

int launch_local_apply(const LocalArgs &a, cudaStream_t s) {
    uint64_t total = a.N * a.nframes;
    if (!total) return AM_OK;
    unsigned grid = (unsigned)std::min<uint64_t>((total + 255) / 256, (uint64_t)kSMs * 8);
    AMG_LAUNCH(k_local_apply, grid, 256, 0, s, a);
    AMG_CUDA(cudaGetLastError());
    return AM_OK;
}

int launch_local_phase(const LocalArgs &a, cudaStream_t s) {
    uint64_t total = a.N * a.nframes;
    if (!total) return AM_OK;
    AMG_CUDA(cudaMemsetAsync(a.claim, 0, total * sizeof(unsigned long long), s));
    unsigned grid = (unsigned)std::min<uint64_t>((total + 255) / 256, (uint64_t)kSMs * 8);
    AMG_LAUNCH(k_local_propose, grid, 256, 0, s, a);
    AMG_LAUNCH(k_local_apply, grid, 256, 0, s, a);
    AMG_CUDA(cudaGetLastError());
    return AM_OK;
}

}  // namespace amg
