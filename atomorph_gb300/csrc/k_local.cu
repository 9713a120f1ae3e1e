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
// The index also holds s = p + n of the column at every slot, in slot order
// (k_slot_sums once, then kept current by the apply kernel); the six-point
// criterion (thread.cpp:1014-1022) of a swap is exactly
// 2 (a1 - a2) . (s2 - s1) (pair_gain), so a candidate costs two reads from
// the same slot-ordered arrays its cell window lives in.
// Candidates come from the column's own neighbourhood, the cell of m1 and a
// few uniform random columns (k_local_propose).  Each slot proposes its best
// strictly improving partner slot and claims both with atomicMax on
// (gain, proposer slot); a proposal is applied when it holds the claim of
// both slots, so applied swaps are disjoint and every applied gain is exact.
#include "common.cuh"
#include "kernels.h"
#include "gridbar.cuh"

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

// Target sums of the columns holding the slots: sv[y][s] = p + n for the
// column x at slot s of frame y, with p, n its points at frames y-1 and y+1
// (1/256 px; x in the low word, y in the high word).  Built once with the
// index; afterwards k_local_apply keeps it current: a swap at frame y moves
// the two columns' sums at frame y to their new slots and changes the two
// columns' sums at frames y-1 and y+1 by the exchanged points' difference.
// The same pass records each slot's chain (slot_ch), which no swap changes.
__global__ void __launch_bounds__(256) k_slot_sums(const uint64_t *__restrict__ P, const uint32_t *__restrict__ col,
                                                   const uint32_t *__restrict__ chain_id,
                                                   const uint8_t *__restrict__ chain_w1, uint64_t N, uint32_t K,
                                                   uint64_t *sv, uint32_t *slot_ch) {
    const uint64_t total = N * K;
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < total; t += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t y = (uint32_t)(t / N);
        uint32_t yn = y + 1 == K ? 0 : y + 1, yp = y == 0 ? K - 1 : y - 1;
        uint32_t x = col[t];
        uint64_t p = P[(uint64_t)yp * N + x], n = P[(uint64_t)yn * N + x];
        sv[t] = sums_pack(pt_X(p) + pt_X(n), pt_Y(p) + pt_Y(n));
        const uint32_t ch = chain_id[x];
        slot_ch[t] = chain_w1[ch] ? kNoChain : ch;
    }
}

// sv[i] += (dx, dy) with one 32-bit atomic per half: two frames of one phase
// (y-1 and y+1 around a frame y) may update the same entry concurrently.
__device__ __forceinline__ void sums_add(uint64_t *sv, uint64_t i, int32_t dx, int32_t dy) {
    unsigned *w = reinterpret_cast<unsigned *>(sv + i);
    if (dx) atomicAdd(w, (unsigned)dx);
    if (dy) atomicAdd(w + 1, (unsigned)dy);
}

// Monotone key: positive gains order like their float value; ties broken by
// the proposer's slot.
__device__ __forceinline__ unsigned long long claim_key(int64_t gain, uint32_t s1) {
    float g = (float)gain;
    return ((unsigned long long)__float_as_uint(g) << 32) | s1;
}

struct Col {        // the proposing column
    uint32_t s1;    // its slot
    uint64_t a1;    // its point
    uint64_t S1;    // its target sum
    uint64_t lo, hi;// its chain's column range
};

// Scans up to `cap` slots of cell (qx, qy) starting at a hashed offset and
// keeps the best strictly improving partner slot.
__device__ __forceinline__ void scan_cell(const LocalArgs &a, const uint32_t *cs, const uint64_t *spt,
                                          const uint32_t *col, const uint64_t *sv, int qx, int qy, uint32_t cap,
                                          uint32_t h, const Col &c, int64_t &best, uint32_t &bs) {
    if (qx < 0 || qy < 0 || qx >= (int)a.ncx || qy >= (int)a.ncy || cap == 0) return;
    uint32_t cell = (uint32_t)qy * a.ncx + (uint32_t)qx;
    uint32_t beg = cs[cell], n = cs[cell + 1] - beg;
    if (n == 0) return;
    uint32_t take = min(n, cap), start = n > cap ? h % n : 0;
    for (uint32_t j = 0; j < take; ++j) {
        uint32_t s = beg + (start + j) % n;
        if (s == c.s1) continue;
        uint32_t x2 = col[s];
        if (x2 < c.lo || x2 >= c.hi) continue;
        int64_t g = pair_gain(c.a1, c.S1, spt[s], sv[s]);
        if (g > best) { best = g; bs = s; }
    }
}

// Candidates of the column at slot s1 of frame y, all checked with the exact
// criterion:
//   * the column's own neighbourhood (the cell of its point a1 and two of the
//     four cells around it): resolves the local crossings left after the
//     coarse transport is right, which uniform pairs almost never sample at
//     large N;
//   * the cell of its target m1 = S1/2: moves a column straight to where its
//     neighbours in the other key frames pull it;
//   * a few uniform random columns of the same chain: the reference's own
//     proposal, for the coarse, long-range part.
// Slot-major: a column reads its own point and target sum, and those of its
// cell-window candidates, from slot-ordered arrays (coalesced, L2-resident
// windows); only the random candidates are scattered loads.  With `sel` set
// only the listed slots propose (the learned gate's choice).
// Returns the best gain found (0 when no improving partner).
__device__ __forceinline__ int64_t propose_one(const LocalArgs &a, uint32_t fi, uint32_t s1) {
    const uint64_t N = a.N;
    const uint64_t t = (uint64_t)fi * N + s1;
    {
        Col c;
        c.s1 = s1;
        uint32_t y = a.frames[fi];
        const uint64_t *spt = a.slot_pt + (uint64_t)y * N;
        const uint32_t *col = a.col + (uint64_t)y * N;
        const uint64_t *sv = a.sv + (uint64_t)y * N;
        a.prop[t] = 0xFFFFFFFFu;
        // independent loads: the slot's chain, point, target sum and column
        const uint32_t ch = a.slot_ch[(uint64_t)y * N + c.s1];
        c.a1 = spt[c.s1];
        c.S1 = sv[c.s1];
        const uint32_t x1 = col[c.s1];
        if (ch == kNoChain) return 0;  // width-1 chains do not refine (thread.cpp:1045)
        c.lo = a.single_chain ? 0ull : a.chain_off[ch];
        c.hi = a.single_chain ? N : a.chain_off[ch + 1];
        const uint32_t *cs = a.cell_start + (uint64_t)y * (a.ncells + 1);
        int64_t best = 0;
        uint32_t bs = 0xFFFFFFFFu;
        uint32_t h = mix32((uint32_t)a.key ^ mix32(c.s1 * 0x9E3779B1u + y));
        // own neighbourhood: centre cell, then two of the 4-neighbour cells
        int ax = (int)min((uint32_t)pt_X(c.a1) >> 9, a.ncx - 1), ay = (int)min((uint32_t)pt_Y(c.a1) >> 9, a.ncy - 1);
        if (a.self_cap) {
            uint32_t per = max(1u, a.self_cap / 3u);
            scan_cell(a, cs, spt, col, sv, ax, ay, per, h, c, best, bs);
            uint32_t r0 = h >> 28;
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                int d = (int)((r0 + 2u * k) & 3u);  // 0..3: +x, -x, +y, -y
                int dx = d == 0 ? 1 : (d == 1 ? -1 : 0), dy = d == 2 ? 1 : (d == 3 ? -1 : 0);
                scan_cell(a, cs, spt, col, sv, ax + dx, ay + dy, per, h >> 3, c, best, bs);
            }
        }
        // target cell
        if (a.cap) {
            int32_t mx = sums_x(c.S1) >> 1, my = sums_y(c.S1) >> 1;
            int cx = (int)min((uint32_t)max(mx, 0) >> 9, a.ncx - 1), cy = (int)min((uint32_t)max(my, 0) >> 9, a.ncy - 1);
            scan_cell(a, cs, spt, col, sv, cx, cy, a.cap, h >> 5, c, best, bs);
        }
        // uniform random partners in the same chain
        if (a.nrandom) {
            uint32_t w = (uint32_t)(c.hi - c.lo);
            const uint32_t *slot_of = a.slot_of + (uint64_t)y * N;
            uint32_t r = h;
            for (uint32_t k = 0; k < a.nrandom; ++k) {
                r = mix32(r + 0x68E31DA4u);
                uint32_t x2 = (uint32_t)c.lo + r % w;
                if (x2 == x1) continue;
                uint32_t s = slot_of[x2];
                int64_t g = pair_gain(c.a1, c.S1, spt[s], sv[s]);
                if (g > best) { best = g; bs = s; }
            }
        }
        if (a.hot) a.hot[(uint64_t)y * N + c.s1] = gain_bucket(best);
        if (bs != 0xFFFFFFFFu) {
            unsigned long long k = claim_key(best, c.s1);
            a.prop[t] = bs;
            a.pgain[t] = (unsigned long long)best;
            atomicMax(a.claim + (uint64_t)fi * N + c.s1, k);
            atomicMax(a.claim + (uint64_t)fi * N + bs, k);
        }
        return best;
    }
}

// Slot t of a gated list: t = fi * N + s < 2^32 (the host checks), so a
// 32-bit division splits it.
__device__ __forceinline__ void split_slot(uint32_t t, uint32_t n32, uint32_t &fi, uint32_t &s) {
    fi = t / n32;
    s = t - fi * n32;
}

__global__ void __launch_bounds__(256) k_local_propose(LocalArgs a) {
    if (a.sel && a.sel_groups) {
        // listed 32-slot regions, one warp each; while recording, the region's
        // summed best gain is its training target
        const uint64_t total = a.N * a.nframes, nsel = *a.nsel;
        const int lane = threadIdx.x & 31;
        const uint64_t w0 = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
        const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
        for (uint64_t i = w0; i < nsel; i += nw) {
            const uint32_t g = a.sel[i];
            const uint64_t t = (uint64_t)g * 32 + lane;
            int64_t best = 0;
            if (t < total) {
                uint32_t fi, s1;
                split_slot((uint32_t)t, (uint32_t)a.N, fi, s1);
                best = propose_one(a, fi, s1);
            }
            if (a.rec_idx) {
                float sum = (float)best;
#pragma unroll
                for (int o = 16; o; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
                const uint32_t j = a.rec_idx[g];
                if (lane == 0 && j != 0xFFFFFFFFu) a.rec_gain[j] = log1pf(sum / kGainScale);
            }
        }
    } else if (a.sel) {
        const uint64_t total = *a.nsel;
        for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total;
             i += (uint64_t)gridDim.x * blockDim.x) {
            uint32_t fi, s1;
            split_slot(a.sel[i], (uint32_t)a.N, fi, s1);
            propose_one(a, fi, s1);
        }
    } else {
        for (uint32_t fi = 0; fi < a.nframes; ++fi)
            for (uint64_t s1 = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; s1 < a.N;
                 s1 += (uint64_t)gridDim.x * blockDim.x)
                propose_one(a, fi, (uint32_t)s1);
    }
}

// A proposal (s1 -> s2) is applied when it holds the claim of both slots:
// applied swaps are then disjoint, so the columns at s1 and s2 are read and
// written by this thread alone.
__device__ __forceinline__ void apply_one(const LocalArgs &a, uint32_t fi, uint32_t s1, unsigned long long &gain,
                                          unsigned long long &acc) {
    const uint64_t N = a.N;
    const uint64_t t = (uint64_t)fi * N + s1;
    {
        uint32_t s2 = a.prop[t];
        if (s2 == 0xFFFFFFFFu) return;
        unsigned long long k1 = a.claim[(uint64_t)fi * N + s1], k2 = a.claim[(uint64_t)fi * N + s2];
        if (k1 != k2 || (uint32_t)k1 != s1) return;
        uint32_t y = a.frames[fi];
        uint64_t *Py = a.P + (uint64_t)y * N;
        uint32_t *slot_of = a.slot_of + (uint64_t)y * N, *col = a.col + (uint64_t)y * N;
        uint32_t x1 = col[s1], x2 = col[s2];
        uint64_t w1 = Py[x1], w2 = Py[x2];
        Py[x1] = w2;
        Py[x2] = w1;
        slot_of[x1] = s2;
        slot_of[x2] = s1;
        col[s1] = x2;
        col[s2] = x1;
        // The sums at frame y follow their columns to the other slot (no
        // other thread touches slots s1, s2 of frame y in this phase).
        uint64_t *svy = a.sv + (uint64_t)y * N;
        const uint64_t t1 = svy[s1];
        svy[s1] = svy[s2];
        svy[s2] = t1;
        // x1 now holds w2 and x2 holds w1 at frame y: their target sums at the
        // neighbouring frames move by the difference (twice for K = 2, where
        // y-1 and y+1 are the same frame and s = 2 p).
        if (a.K > 1) {
            const int32_t dx = pt_X(w2) - pt_X(w1), dy = pt_Y(w2) - pt_Y(w1);
            const uint32_t yn = y + 1 == a.K ? 0 : y + 1, yp = y == 0 ? a.K - 1 : y - 1;
            for (int side = 0; side < 2; ++side) {
                const uint64_t yy = side ? yn : yp;
                const uint32_t *so = a.slot_of + yy * N;
                sums_add(a.sv, yy * N + so[x1], dx, dy);
                sums_add(a.sv, yy * N + so[x2], -dx, -dy);
            }
        }
        gain += a.pgain[t];
        acc += 1;
    }
}

__global__ void __launch_bounds__(256) k_local_apply(LocalArgs a) {
    unsigned long long gain = 0, acc = 0;
    if (a.sel && a.sel_groups) {
        const uint64_t total = a.N * a.nframes, nsel = *a.nsel;
        const int lane = threadIdx.x & 31;
        const uint64_t w0 = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
        const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
        for (uint64_t i = w0; i < nsel; i += nw) {
            const uint64_t t = (uint64_t)a.sel[i] * 32 + lane;
            if (t < total) {
                uint32_t fi, s1;
                split_slot((uint32_t)t, (uint32_t)a.N, fi, s1);
                apply_one(a, fi, s1, gain, acc);
            }
        }
    } else if (a.sel) {
        const uint64_t total = *a.nsel;
        for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total;
             i += (uint64_t)gridDim.x * blockDim.x) {
            uint32_t fi, s1;
            split_slot(a.sel[i], (uint32_t)a.N, fi, s1);
            apply_one(a, fi, s1, gain, acc);
        }
    } else {
        for (uint32_t fi = 0; fi < a.nframes; ++fi)
            for (uint64_t s1 = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; s1 < a.N;
                 s1 += (uint64_t)gridDim.x * blockDim.x)
                apply_one(a, fi, (uint32_t)s1, gain, acc);
    }
    gain = warp_sum_u64(gain);
    acc = warp_sum_u64(acc);
    if ((threadIdx.x & 31) == 0) {
        if (gain) atomicAdd(a.gain, gain);
        if (acc) atomicAdd(a.accepted, acc);
    }
}

// Every job's guided sweeps in one persistent cooperative launch.  Per sweep
// and phase, three stages over chunks of (job, frame, slot range) separated
// by grid barriers: clear the claims, propose (propose_one), apply
// (apply_one).  The job's LocalArgs are those its own guided sweeps use, with
// the same keys, so every job ends bit-identical to refining it alone.
__global__ void __launch_bounds__(256, 4) k_batch_local(BatchLocalArgs b) {
    __shared__ unsigned long long red[8];
    const int nphase = (int)b.nphase;
    for (uint32_t s = 0; s < b.sweeps; ++s) {
        for (int p = 0; p < nphase; ++p) {
            const uint32_t lo = p == 0 ? b.ch_off[0] : (p == 1 ? b.ch_off[1] : b.ch_off[2]);
            const uint32_t hi = p == 0 ? b.ch_off[1] : (p == 1 ? b.ch_off[2] : b.ch_off[3]);
            for (int stage = 0; stage < 3; ++stage) {
                for (uint32_t ch = lo + blockIdx.x; ch < hi; ch += gridDim.x) {
                    const uint32_t j = b.ch_job[ch], fi = b.ch_fi[ch];
                    const BatchLocalJob &J = b.jobs[j];
                    const uint64_t start = b.ch_start[ch], end = start + b.ch_count[ch];
                    if (stage == 0) {
                        for (uint64_t r = start + threadIdx.x; r < end; r += blockDim.x)
                            J.a.claim[(uint64_t)fi * J.a.N + r] = 0ull;
                        continue;
                    }
                    LocalArgs a = J.a;
                    a.frames = J.frames + (p == 0 ? J.ph_off[0] : (p == 1 ? J.ph_off[1] : J.ph_off[2]));
                    a.nframes = p == 0 ? J.ph_n[0] : (p == 1 ? J.ph_n[1] : J.ph_n[2]);
                    a.key = mix64(((uint64_t)J.seed << 40) ^ ((J.sweep0 + s) << 4) ^ (uint64_t)p ^ 0x5bd1e995ULL);
                    if (stage == 1) {
                        for (uint64_t r = start + threadIdx.x; r < end; r += blockDim.x) propose_one(a, fi, (uint32_t)r);
                        continue;
                    }
                    unsigned long long gain = 0, acc = 0;
                    for (uint64_t r = start + threadIdx.x; r < end; r += blockDim.x) apply_one(a, fi, (uint32_t)r, gain, acc);
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
                const bool last = stage == 2 && s + 1 == b.sweeps && p + 1 == nphase;
                if (!last && !grid_barrier(b.bar, b.err)) return;
            }
        }
    }
}

}  // namespace

int batch_local_max_ctas_per_sm(uint32_t threads, int *out) {
    int n = 0;
    AMG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_batch_local, (int)threads, 0));
    *out = n;
    return AM_OK;
}

int launch_batch_local(const BatchLocalArgs &b, uint32_t grid, uint32_t threads, cudaStream_t s) {
    if (b.sweeps == 0 || b.nphase == 0) return AM_OK;
    if (threads > 256) {
        set_error("am_batch: the batched guided kernel runs at most 256 threads per CTA");
        return AM_ERR_ARG;
    }
    BatchLocalArgs arg = b;
    void *params[] = {&arg};
    AMG_CUDA(cudaLaunchCooperativeKernel((const void *)k_batch_local, dim3(grid), dim3(threads), params, 0, s));
    g_launches.fetch_add(1, std::memory_order_relaxed);
    return AM_OK;
}

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
    unsigned g2 = (unsigned)std::min<uint64_t>((N * K + 255) / 256, (uint64_t)kSMs * 8);
    AMG_LAUNCH(k_slot_sums, g2, 256, 0, s, P, ix.col, ix.chain_id, ix.chain_w1, N, K, ix.sv, ix.slot_ch);
    AMG_CUDA(cudaGetLastError());
    return AM_OK;
}

int launch_chain_ids(const uint64_t *chain_off, uint32_t C, uint64_t N, uint32_t *out, cudaStream_t s) {
    if (!N) return AM_OK;
    unsigned grid = (unsigned)std::min<uint64_t>((N + 255) / 256, (uint64_t)kSMs * 8);
    AMG_LAUNCH(k_chain_ids, grid, 256, 0, s, chain_off, C, N, out);
    AMG_CUDA(cudaGetLastError());
    return AM_OK;
}

int launch_local_propose(const LocalArgs &a, cudaStream_t s) {
    uint64_t total = a.N * a.nframes;
    if (!total) return AM_OK;
    unsigned grid = (unsigned)std::min<uint64_t>((total + 255) / 256, (uint64_t)kSMs * 8);
    AMG_LAUNCH(k_local_propose, grid, 256, 0, s, a);
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
    int rc = launch_local_propose(a, s);
    if (!rc) rc = launch_local_apply(a, s);
    return rc;
}

}  // namespace amg
