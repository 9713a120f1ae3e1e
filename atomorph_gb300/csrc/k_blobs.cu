// Blob stage: 4-connected component labelling of each key frame, exact blob
// statistics, and the blob matching sweep.
//
// With blob_threshold >= 1 (every colour distance is <= 1, color.h:17-24),
// blob_min_size <= 1, blob_max_size >= every component and blob_number <= the
// component count, the greedy merging of blobify_frame (thread.cpp:225-412)
// ends with exactly the 4-connected components of the opaque pixels and
// unify_frame (thread.cpp:426-585) leaves them unchanged; that regime is what
// label_components computes.  Components are numbered by their first pixel in
// row-major order.
//
// Outside that regime merge_blobs restates blobify / unify's rules as rounds
// of parallel agglomeration (Boruvka style) from single-pixel blobs: every
// blob below blob_max_size picks its neighbour blob of least colour distance
// (color_distance of the rounded mean colours, color.h:17-24) within
// blob_threshold, or its nearest one at any distance while it is below
// blob_min_size; the picks are merged, at most down to blob_number blobs.
// Then "dust" (blobs still below blob_min_size, which have no neighbours
// left) merges with the nearest dust whose rounded centroid lies within
// blob_box_grip on both axes, again down to blob_number.  The reference
// merges one pair at a time in a random order (its result depends on that
// order); these rounds merge all picks at once with seeded tie-breaks, so
// the same rules give a different but equally valid partition.
#include "common.cuh"
#include "kernels.h"

#include <vector>

namespace amg {

constexpr int kScanTile = 2048;

struct BlobWork {
    uint32_t *tile_cnt = nullptr;
    size_t tile_cap = 0;
    int32_t *root_rank = nullptr;
    size_t px_cap = 0;
    int *err = nullptr;
    // merge_blobs scratch, n pixels each
    void *merge = nullptr;
    size_t merge_cap = 0;
};

BlobWork *blob_work_create() { return new BlobWork(); }
void blob_work_destroy(BlobWork *w) {
    if (!w) return;
    if (w->tile_cnt) cudaFree(w->tile_cnt);
    if (w->root_rank) cudaFree(w->root_rank);
    if (w->err) cudaFree(w->err);
    if (w->merge) cudaFree(w->merge);
    delete w;
}

namespace {

__global__ void k_cc_init(const uint8_t *__restrict__ present, int32_t *L, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        L[i] = present[i] ? (int32_t)i : -1;
}

__device__ __forceinline__ int32_t cc_find(int32_t *L, int32_t x) {
    // Path halving; labels only ever point to smaller indices of the same set.
    for (int it = 0; it < (1 << 24); ++it) {
        int32_t p = L[x];
        if (p == x) return x;
        int32_t gp = L[p];
        if (gp != p) L[x] = gp;
        x = p;
    }
    return x;
}

__device__ __forceinline__ void cc_union(int32_t *L, int32_t a, int32_t b, int *err) {
    // Lock-free union: hook the larger root under the smaller one by CAS; a
    // failed CAS means that root was just hooked, so retry from its parent.
    for (int it = 0; it < (1 << 20); ++it) {
        a = cc_find(L, a);
        b = cc_find(L, b);
        if (a == b) return;
        if (a < b) { int32_t t = a; a = b; b = t; }
        int32_t old = atomicCAS(&L[a], a, b);
        if (old == a) return;
    }
    atomicExch(err, 1);  // iteration bound reached: reported, never spins
}

__global__ void k_cc_merge(const uint8_t *__restrict__ present, int32_t *L, uint32_t W, uint32_t H, int *err) {
    size_t n = (size_t)W * H;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        if (!present[i]) continue;
        uint32_t x = (uint32_t)(i % W), y = (uint32_t)(i / W);
        if (x + 1 < W && present[i + 1]) cc_union(L, (int32_t)i, (int32_t)(i + 1), err);
        if (y + 1 < H && present[i + W]) cc_union(L, (int32_t)i, (int32_t)(i + W), err);
    }
}

// Every label becomes its root.  No path compression here: with merging
// finished, the only values written are roots, so a thread walking through a
// pixel another thread just rewrote still reaches the same root (with
// compression, a stale halving write could replace a root by an ancestor).
__global__ void k_cc_flatten(int32_t *L, size_t n, int *err) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        int32_t x = L[i];
        if (x < 0) continue;
        int it = 0;
        for (int32_t p = L[x]; p != x && it < (1 << 24); p = L[x], ++it) x = p;
        if (L[x] != x) atomicExch(err, 1);
        L[i] = x;
    }
}

// Roots per scan tile.
__global__ void __launch_bounds__(256) k_root_count(const int32_t *__restrict__ L, size_t n, uint32_t *cnt) {
    __shared__ uint32_t s;
    if (threadIdx.x == 0) s = 0;
    __syncthreads();
    size_t base = (size_t)blockIdx.x * kScanTile;
    uint32_t c = 0;
    for (int k = threadIdx.x; k < kScanTile; k += 256) {
        size_t i = base + k;
        if (i < n && L[i] == (int32_t)i) ++c;
    }
    atomicAdd(&s, c);
    __syncthreads();
    if (threadIdx.x == 0) cnt[blockIdx.x] = s;
}

// Rank of each root in row-major order (= component index).
__global__ void __launch_bounds__(256) k_root_rank(const int32_t *__restrict__ L, size_t n,
                                                    const uint32_t *__restrict__ off, int32_t *rank) {
    __shared__ uint32_t warp_tot[8];
    __shared__ uint32_t base;
    if (threadIdx.x == 0) base = off[blockIdx.x];
    __syncthreads();
    size_t tile = (size_t)blockIdx.x * kScanTile;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int c = 0; c < kScanTile; c += 256) {
        size_t i = tile + c + threadIdx.x;
        bool root = i < n && L[i] == (int32_t)i;
        unsigned b = __ballot_sync(0xffffffffu, root);
        if (lane == 0) warp_tot[warp] = __popc(b);
        __syncthreads();
        uint32_t pre = 0;
        for (int w = 0; w < warp; ++w) pre += warp_tot[w];
        if (root) rank[i] = (int32_t)(base + pre + __popc(b & ((1u << lane) - 1u)));
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t t = 0;
            for (int w = 0; w < 8; ++w) t += warp_tot[w];
            base += t;
        }
        __syncthreads();
    }
}

// Roots were ranked by k_root_rank and every present pixel's label is a root
// after k_cc_flatten; when flattening flagged a failure the host discards the
// labels, and k_blob_stats ignores any label outside [0, nblobs).
__global__ void k_relabel(int32_t *L, const int32_t *__restrict__ rank, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        int32_t r = L[i];
        if (r >= 0) L[i] = rank[r];
    }
}

// Exact per-blob sums; lanes with the same label reduce together first.
__global__ void k_blob_stats(const int32_t *__restrict__ L, const uint32_t *__restrict__ stored, uint32_t W,
                             size_t n, unsigned long long *stats, uint32_t nblobs) {
    const int lane = threadIdx.x & 31;
    for (size_t base = blockIdx.x * (size_t)blockDim.x; base < n; base += (size_t)gridDim.x * blockDim.x) {
        size_t i = base + threadIdx.x;
        int32_t l = i < n ? L[i] : -1;
        if (l >= (int32_t)nblobs) l = -1;  // never written out of range
        unsigned peers = __match_any_sync(0xffffffffu, l);
        uint32_t c = i < n ? stored[i] : 0u;
        uint32_t v[7] = {1u, (uint32_t)(i % W), (uint32_t)(i / W), c & 255u, (c >> 8) & 255u, (c >> 16) & 255u,
                         c >> 24};
        uint32_t sum[7];
#pragma unroll
        for (int k = 0; k < 7; ++k) sum[k] = __reduce_add_sync(peers, v[k]);
        if (l >= 0 && lane == __ffs(peers) - 1) {
#pragma unroll
            for (int k = 0; k < 7; ++k) atomicAdd(stats + (size_t)7 * l + k, (unsigned long long)sum[k]);
        }
    }
}

// ------------------------------------------------------ blob merging -----
struct MergeArgs {
    int32_t *L;                  // [n] union-find over pixels, -1 where absent
    const uint8_t *present;
    const uint32_t *stored;
    uint32_t W, H;
    size_t n;
    uint32_t *size, *sr, *sg, *sb, *sa;   // per root (indexed by its pixel)
    unsigned long long *sx, *sy;          // per root centroid sums
    uint32_t *rc;                // per root rounded mean colour (stored space)
    unsigned long long *best;    // per root best pick key
    unsigned long long *acc;     // per root best proposal received (distance key | proposer)
    int32_t *pick;               // per root picked partner root
    uint8_t *dust;               // per root: below min size with no neighbour left
    uint8_t *retired;            // per root: found no pick once, never initiates again
                                 // (thread.cpp:383-399; it may still be absorbed)
    double threshold;
    unsigned long long min_size, max_size;
    uint32_t key;                // round key of the tie-breaks
    long long *budget;           // merges still allowed (count - blob_number)
    unsigned long long *merged;  // merges made this round
    unsigned long long *picks;   // roots with a pick this round
    int *err;
};

__device__ __forceinline__ uint32_t tie31(uint32_t a, uint32_t b, uint32_t key) {
    const uint32_t lo = min(a, b), hi = max(a, b);
    return mix32(lo * 0x9E3779B1u ^ mix32(hi ^ key)) & 0x7FFFFFFFu;
}

// Exact per-root sums of size, colour and position (lanes with the same root
// reduce together first).
__global__ void k_bm_stats(MergeArgs a) {
    const int lane = threadIdx.x & 31;
    for (size_t base = blockIdx.x * (size_t)blockDim.x; base < a.n; base += (size_t)gridDim.x * blockDim.x) {
        const size_t i = base + threadIdx.x;
        const int32_t r = i < a.n ? a.L[i] : -1;
        const unsigned peers = __match_any_sync(0xffffffffu, r);
        const uint32_t c = i < a.n ? a.stored[i] : 0u;
        const uint32_t v[7] = {1u, c & 255u, (c >> 8) & 255u, (c >> 16) & 255u, c >> 24, (uint32_t)(i % a.W),
                               (uint32_t)(i / a.W)};
        uint32_t sum[7];
#pragma unroll
        for (int k = 0; k < 7; ++k) sum[k] = __reduce_add_sync(peers, v[k]);
        if (r >= 0 && lane == __ffs(peers) - 1) {
            atomicAdd(a.size + r, sum[0]);
            atomicAdd(a.sr + r, sum[1]); atomicAdd(a.sg + r, sum[2]);
            atomicAdd(a.sb + r, sum[3]); atomicAdd(a.sa + r, sum[4]);
            atomicAdd(a.sx + r, (unsigned long long)sum[5]); atomicAdd(a.sy + r, (unsigned long long)sum[6]);
        }
    }
}

__device__ __forceinline__ uint32_t rmean(uint32_t sum, uint32_t cnt) { return (2u * sum + cnt) / (2u * cnt); }

// Rounded mean colour of each root (create_color of the mean, as the
// reference's create_color(bl->r, ...) rounds).
__global__ void k_bm_mean(MergeArgs a) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < a.n; i += (size_t)gridDim.x * blockDim.x) {
        if (a.L[i] != (int32_t)i) continue;
        const uint32_t c = a.size[i];
        a.rc[i] = rmean(a.sr[i], c) | (rmean(a.sg[i], c) << 8) | (rmean(a.sb[i], c) << 16) | (rmean(a.sa[i], c) << 24);
        a.best[i] = ~0ull;
        a.acc[i] = ~0ull;
        a.pick[i] = -1;
    }
}

__device__ __forceinline__ double cdist(uint32_t c1, uint32_t c2) {
    int d = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int e = (int)((c1 >> (8 * k)) & 255u) - (int)((c2 >> (8 * k)) & 255u);
        d += e * e;
    }
    return sqrt((double)d) / 510.0;
}

// The pick key of root r for neighbour root s (0 when r may not pick s):
// within-threshold picks first, then the distance, then a seeded tie-break.
__device__ __forceinline__ unsigned long long pick_key(const MergeArgs &a, int32_t r, int32_t s) {
    const double d = cdist(a.rc[r], a.rc[s]);
    const bool over = !(d <= a.threshold);
    if (over && a.size[r] >= a.min_size) return 0ull;
    return ((unsigned long long)over << 63) | ((unsigned long long)__float_as_uint((float)d) << 31) |
           tie31((uint32_t)r, (uint32_t)s, a.key);
}

// Best pick of every root below the maximum size over its 4-neighbour blobs.
__global__ void k_bm_best(MergeArgs a, int write_pick) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < a.n; i += (size_t)gridDim.x * blockDim.x) {
        const int32_t r = a.L[i];
        if (r < 0 || a.size[r] >= a.max_size || a.retired[r]) continue;
        const uint32_t x = (uint32_t)(i % a.W), y = (uint32_t)(i / a.W);
        const size_t nb[4] = {x + 1 < a.W ? i + 1 : i, x > 0 ? i - 1 : i, y + 1 < a.H ? i + a.W : i, y > 0 ? i - a.W : i};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            if (nb[k] == i) continue;
            const int32_t s2 = a.L[nb[k]];
            if (s2 < 0 || s2 == r) continue;
            const unsigned long long key = pick_key(a, r, s2);
            if (!key) continue;
            if (!write_pick) atomicMin(a.best + r, key);
            else if (key == a.best[r]) a.pick[r] = s2;
        }
    }
}

__device__ __forceinline__ int32_t bm_find(int32_t *L, int32_t x) {
    for (int it = 0; it < (1 << 24); ++it) {
        const int32_t p = L[x];
        if (p == x) return x;
        x = p;
    }
    return x;
}

// Hooks root r to its pick when the merge budget allows: the larger root goes
// under the smaller by CAS; a pick already in the same set refunds the merge.
__device__ void bm_merge(const MergeArgs &a, int32_t r, int32_t s) {
    // reserve one merge of the budget (budget -= 1); none left: give it back
    const long long old = (long long)atomicAdd((unsigned long long *)a.budget, ~0ull);
    if (old <= 0) {
        atomicAdd((unsigned long long *)a.budget, 1ull);
        return;
    }
    for (int it = 0; it < (1 << 20); ++it) {
        int32_t u = bm_find(a.L, r), v = bm_find(a.L, s);
        if (u == v) {
            atomicAdd((unsigned long long *)a.budget, 1ull);
            return;
        }
        if (u < v) { const int32_t t = u; u = v; v = t; }
        if (atomicCAS(&a.L[u], u, v) == u) {
            atomicAdd(a.merged, 1ull);
            if (a.retired) a.retired[v] = 0;  // the merged blob keeps expanding
            return;
        }
    }
    atomicAdd((unsigned long long *)a.budget, 1ull);
    atomicExch(a.err, 1);
}

// Pairwise merges per round, each blob in at most one (the reference merges
// one pair at a time and re-reads the means after each): mutual picks merge;
// otherwise a seeded coin makes each blob a proposer or an acceptor, a
// proposer proposes to its pick when that is an acceptor without a mutual
// pick, and an acceptor takes its best proposal.
__device__ __forceinline__ bool proposer(const MergeArgs &a, uint32_t r) { return mix32(r ^ a.key) & 1u; }
__device__ __forceinline__ bool mutual(const MergeArgs &a, int32_t r) {
    const int32_t s2 = a.pick[r];
    return s2 >= 0 && a.pick[s2] == r;
}

__global__ void k_bm_propose(MergeArgs a) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < a.n; i += (size_t)gridDim.x * blockDim.x) {
        if (a.L[i] != (int32_t)i) continue;
        const int32_t r = (int32_t)i, s2 = a.pick[r];
        if (s2 < 0 || mutual(a, r) || !proposer(a, (uint32_t)r)) continue;
        if (proposer(a, (uint32_t)s2) || mutual(a, s2)) continue;
        atomicMin(a.acc + s2, (a.best[r] & ~0x7FFFFFFFull) | (unsigned long long)r);
    }
}

__global__ void k_bm_union(MergeArgs a) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < a.n; i += (size_t)gridDim.x * blockDim.x) {
        if (a.L[i] != (int32_t)i) continue;
        const int32_t r = (int32_t)i, s2 = a.pick[r];
        if (s2 >= 0) atomicAdd(a.picks, 1ull);
        else a.retired[r] = 1;
        if (s2 >= 0 && mutual(a, r)) {
            if (r < s2) bm_merge(a, r, s2);
        } else if (a.acc[r] != ~0ull) {
            bm_merge(a, r, (int32_t)(a.acc[r] & 0x7FFFFFFFull));
        }
    }
}

// Dust roots (below min size after the agglomeration) into a list with their
// rounded centroids.
__global__ void k_bm_dust_list(MergeArgs a, uint32_t *list, uint32_t *cnt, uint32_t cap) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < a.n; i += (size_t)gridDim.x * blockDim.x) {
        if (a.L[i] != (int32_t)i || !a.dust[i]) continue;
        const uint32_t k = atomicAdd(cnt, 1u);
        if (k < cap) list[k] = (uint32_t)i;
    }
}

__device__ __forceinline__ uint32_t centroid(const MergeArgs &a, uint32_t r, int axis) {
    const unsigned long long s = axis ? a.sy[r] : a.sx[r], c = a.size[r];
    return (uint32_t)((2ull * s + c) / (2ull * c));  // round(mean)
}

// Nearest other dust root within the box grip on both axes (unify_frame,
// thread.cpp:541-557: least dx^2 + dy^2 of the rounded centroids).
__global__ void k_bm_dust_pick(MergeArgs a, const uint32_t *__restrict__ list, uint32_t nd, uint32_t grip) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nd; i += gridDim.x * blockDim.x) {
        const uint32_t r = list[i];
        const int64_t rx = centroid(a, r, 0), ry = centroid(a, r, 1);
        unsigned long long best = ~0ull;
        uint32_t pick = r;
        for (uint32_t j = 0; j < nd; ++j) {
            const uint32_t s2 = list[j];
            if (s2 == r) continue;
            const int64_t dx = (int64_t)centroid(a, s2, 0) - rx, dy = (int64_t)centroid(a, s2, 1) - ry;
            if (dx > grip || -dx > grip || dy > grip || -dy > grip) continue;
            const unsigned long long key =
                ((unsigned long long)(dx * dx + dy * dy) << 31) | tie31(r, s2, a.key);
            if (key < best) { best = key; pick = s2; }
        }
        a.best[r] = best;
        a.pick[r] = (int32_t)pick;
    }
}

__global__ void k_bm_dust_union(MergeArgs a, const uint32_t *__restrict__ list, uint32_t nd) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nd; i += gridDim.x * blockDim.x) {
        const uint32_t r = list[i];
        if (a.best[r] != ~0ull) bm_merge(a, (int32_t)r, a.pick[r]);
    }
}

// Roots after a round: full paths (no compression while roots change).
__global__ void k_bm_flatten(int32_t *L, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const int32_t x = L[i];
        if (x >= 0) L[i] = bm_find(L, x);
    }
}

// Dust marks after the agglomeration: roots still below the minimum size.
__global__ void k_bm_mark_dust(MergeArgs a) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < a.n; i += (size_t)gridDim.x * blockDim.x)
        a.dust[i] = a.L[i] == (int32_t)i && a.size[i] < a.min_size;
}

// ---------------------------------------------------------- matching -----
struct BlobDesc {
    double size, x, y, r, g, b, a;
};

__device__ __forceinline__ uint32_t cbyte(double v) { return (uint32_t)(int)round(v * 255.0) & 255u; }

// blob_distance (thread.cpp:1151-1174).
__device__ double blob_dist(const double *b1, const double *b2, double bbox_d, double wr, double ws, double wx) {
    double sz1 = b1[0], sz2 = b2[0], szs = sz1 + sz2;
    double pix = 0.0, col = 0.0, siz = 0.0;
    if (szs > 0) siz = fabs(sz1 - sz2) / szs;
    if (sz1 > 0 && sz2 > 0) {
        int32_t x1 = (int32_t)(uint16_t)b1[1], y1 = (int32_t)(uint16_t)b1[2];
        int32_t x2 = (int32_t)(uint16_t)b2[1], y2 = (int32_t)(uint16_t)b2[2];
        int32_t xd = x1 - x2, yd = y1 - y2;
        pix = sqrt(double((uint32_t)(xd * xd + yd * yd)) / bbox_d);
        int rd = (int)cbyte(b1[3]) - (int)cbyte(b2[3]), gd = (int)cbyte(b1[4]) - (int)cbyte(b2[4]);
        int bd = (int)cbyte(b1[5]) - (int)cbyte(b2[5]), ad = (int)cbyte(b1[6]) - (int)cbyte(b2[6]);
        col = sqrt((double)(rd * rd + gd * gd + bd * bd + ad * ad)) / 510.0;
    }
    return wx * pix + wr * col + ws * siz;
}

__global__ void __launch_bounds__(512) k_blob_match(MatchArgs a) {
    extern __shared__ int32_t sperm[];  // [K][Wb]
    const uint32_t Wb = a.Wb, K = a.K;
    for (uint32_t i = threadIdx.x; i < Wb * K; i += blockDim.x) sperm[i] = a.perm[i];
    __syncthreads();
    auto D = [&](uint32_t g, uint32_t k) { return a.desc + ((size_t)k * Wb + sperm[k * Wb + g]) * 7; };
    const uint32_t hb = half_bits_for(Wb);
    const uint32_t npairs = Wb / 2;
    // Phases of frames that are not neighbours: even / odd (+ last when K odd).
    for (uint32_t s = 0; s < a.sweeps; ++s) {
        for (uint32_t ph = 0; ph < 3; ++ph) {
            for (uint32_t y = 0; y < K; ++y) {
                uint32_t p = (K == 1) ? 0 : ((K % 2 == 1 && y == K - 1 && K > 1) ? 2 : (y & 1));
                if (p != ph) continue;
                uint32_t yn = (y + 1) % K, yp = (y + K - 1) % K;
                uint64_t key = mix64(a.key ^ mix64(((uint64_t)s << 32) ^ ((uint64_t)y << 8) ^ ph));
                bool force = a.degenerate && ((s + 1) % a.degenerate == 0) && y == 0;
                for (uint32_t i = threadIdx.x; i < npairs; i += blockDim.x) {
                    uint32_t x1 = permute_index(2 * i, Wb, hb, key), x2 = permute_index(2 * i + 1, Wb, hb, key);
                    const double *b1 = D(x1, y), *b2 = D(x2, y);
                    if (b1[0] == 0 && b2[0] == 0) continue;  // both volatile (thread.cpp:689-694)
                    const double *b1p = D(x1, yp), *b2p = D(x2, yp), *b1n = D(x1, yn), *b2n = D(x2, yn);
                    double c1 = blob_dist(b1p, b1, a.bbox_d, a.w_rgba, a.w_size, a.w_xy) +
                                blob_dist(b1, b1n, a.bbox_d, a.w_rgba, a.w_size, a.w_xy);
                    c1 += blob_dist(b2p, b2, a.bbox_d, a.w_rgba, a.w_size, a.w_xy) +
                          blob_dist(b2, b2n, a.bbox_d, a.w_rgba, a.w_size, a.w_xy);
                    double c2 = blob_dist(b2p, b1, a.bbox_d, a.w_rgba, a.w_size, a.w_xy) +
                                blob_dist(b1, b2n, a.bbox_d, a.w_rgba, a.w_size, a.w_xy);
                    c2 += blob_dist(b1p, b2, a.bbox_d, a.w_rgba, a.w_size, a.w_xy) +
                          blob_dist(b2, b1n, a.bbox_d, a.w_rgba, a.w_size, a.w_xy);
                    if (c1 >= c2 || force) {
                        int32_t t = sperm[y * Wb + x1];
                        sperm[y * Wb + x1] = sperm[y * Wb + x2];
                        sperm[y * Wb + x2] = t;
                    }
                }
            }
            __syncthreads();
        }
    }
    // Energy of the final map (thread.cpp:1087-1107), reduced in FP64.
    __shared__ double red[512];
    double e = 0.0;
    for (uint32_t i = threadIdx.x; i < Wb; i += blockDim.x) {
        const double *prev = D(i, K - 1);
        for (uint32_t j = 0; j < K; ++j) {
            const double *cur = D(i, j);
            e += blob_dist(prev, cur, a.bbox_d, a.w_rgba, a.w_size, a.w_xy);
            prev = cur;
        }
    }
    red[threadIdx.x] = e;
    __syncthreads();
    for (uint32_t o = blockDim.x / 2; o; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0 && a.energy_out) *a.energy_out = red[0];
    for (uint32_t i = threadIdx.x; i < Wb * K; i += blockDim.x) a.perm[i] = sperm[i];
}

}  // namespace

int label_components(BlobWork *w, const uint8_t *present, const uint32_t *stored, uint32_t CW, uint32_t CH,
                     int32_t *labels, uint32_t *nblobs, cudaStream_t s) {
    (void)stored;
    size_t n = (size_t)CW * CH;
    if (n == 0) { *nblobs = 0; return AM_OK; }
    size_t ntiles = (n + kScanTile - 1) / kScanTile;
    if (ntiles + 1 > w->tile_cap) {
        if (w->tile_cnt) cudaFree(w->tile_cnt);
        w->tile_cnt = nullptr;
        w->tile_cap = 0;  // recorded once the buffer exists
        AMG_ALLOC(&w->tile_cnt, (ntiles + 1) * 4);
        w->tile_cap = ntiles + 1;
    }
    if (n > w->px_cap) {
        if (w->root_rank) cudaFree(w->root_rank);
        w->root_rank = nullptr;
        w->px_cap = 0;
        AMG_ALLOC(&w->root_rank, n * 4);
        w->px_cap = n;
    }
    if (!w->err) AMG_ALLOC(&w->err, sizeof(int));
    AMG_CUDA(cudaMemsetAsync(w->err, 0, sizeof(int), s));
    unsigned grid = (unsigned)std::min<size_t>((n + 255) / 256, (size_t)kSMs * 16);
    AMG_LAUNCH(k_cc_init, grid, 256, 0, s, present, labels, n);
    AMG_LAUNCH(k_cc_merge, grid, 256, 0, s, present, labels, CW, CH, w->err);
    AMG_LAUNCH(k_cc_flatten, grid, 256, 0, s, labels, n, w->err);
    AMG_LAUNCH(k_root_count, (unsigned)ntiles, 256, 0, s, labels, n, w->tile_cnt);
    AMG_CUDA(cudaMemsetAsync(w->tile_cnt + ntiles, 0, 4, s));
    int rc = launch_scan_u32(w->tile_cnt, ntiles + 1, nullptr, s);
    if (rc) return rc;
    AMG_LAUNCH(k_root_rank, (unsigned)ntiles, 256, 0, s, labels, n, w->tile_cnt, w->root_rank);
    AMG_LAUNCH(k_relabel, grid, 256, 0, s, labels, w->root_rank, n);
    uint32_t total = 0;
    int err = 0;
    AMG_CUDA(cudaMemcpyAsync(&total, w->tile_cnt + ntiles, 4, cudaMemcpyDeviceToHost, s));
    AMG_CUDA(cudaMemcpyAsync(&err, w->err, sizeof(int), cudaMemcpyDeviceToHost, s));
    AMG_CUDA(cudaStreamSynchronize(s));
    if (err) {
        set_error("connected-component labelling exceeded its iteration bound");
        return AM_ERR_TIMEOUT;
    }
    *nblobs = total;
    return AM_OK;
}

// Largest dust list the brute-force nearest-dust search takes.
constexpr uint32_t kMaxDust = 1u << 16;

// Ranks the roots of L (row-major) and relabels every pixel with its root's
// rank; *nblobs = the number of roots.
static int relabel_roots(BlobWork *w, int32_t *L, size_t n, uint32_t *nblobs, cudaStream_t s) {
    const size_t ntiles = (n + kScanTile - 1) / kScanTile;
    const unsigned grid = (unsigned)std::min<size_t>((n + 255) / 256, (size_t)kSMs * 16);
    AMG_LAUNCH(k_root_count, (unsigned)ntiles, 256, 0, s, L, n, w->tile_cnt);
    AMG_CUDA(cudaMemsetAsync(w->tile_cnt + ntiles, 0, 4, s));
    int rc = launch_scan_u32(w->tile_cnt, ntiles + 1, nullptr, s);
    if (rc) return rc;
    AMG_LAUNCH(k_root_rank, (unsigned)ntiles, 256, 0, s, L, n, w->tile_cnt, w->root_rank);
    AMG_LAUNCH(k_relabel, grid, 256, 0, s, L, w->root_rank, n);
    uint32_t total = 0;
    AMG_CUDA(cudaMemcpyAsync(&total, w->tile_cnt + ntiles, 4, cudaMemcpyDeviceToHost, s));
    AMG_CUDA(cudaStreamSynchronize(s));
    *nblobs = total;
    return AM_OK;
}

int merge_blobs(BlobWork *w, const uint8_t *present, const uint32_t *stored, uint32_t CW, uint32_t CH,
                const BlobRules &p, int32_t *labels, uint32_t *nblobs, cudaStream_t s) {
    const size_t n = (size_t)CW * CH;
    if (n == 0) { *nblobs = 0; return AM_OK; }
    const size_t ntiles = (n + kScanTile - 1) / kScanTile;
    if (ntiles + 1 > w->tile_cap) {
        if (w->tile_cnt) cudaFree(w->tile_cnt);
        w->tile_cnt = nullptr;
        w->tile_cap = 0;  // recorded once the buffer exists
        AMG_ALLOC(&w->tile_cnt, (ntiles + 1) * 4);
        w->tile_cap = ntiles + 1;
    }
    if (n > w->px_cap) {
        if (w->root_rank) cudaFree(w->root_rank);
        w->root_rank = nullptr;
        w->px_cap = 0;
        AMG_ALLOC(&w->root_rank, n * 4);
        w->px_cap = n;
    }
    if (!w->err) AMG_ALLOC(&w->err, sizeof(int));
    // scratch: 7 x u32 + 4 x u64 + 2 x u8 per pixel, then the counters
    const size_t per = 7 * 4 + 4 * 8 + 2;
    const size_t bytes = n * per + 64;
    if (bytes > w->merge_cap) {
        if (w->merge) cudaFree(w->merge);
        w->merge = nullptr;
        w->merge_cap = 0;
        AMG_ALLOC(&w->merge, bytes);
        w->merge_cap = bytes;
    }
    unsigned char *b = (unsigned char *)w->merge;
    MergeArgs a;
    a.L = labels; a.present = present; a.stored = stored; a.W = CW; a.H = CH; a.n = n;
    a.sx = (unsigned long long *)b; a.sy = a.sx + n; a.best = a.sy + n; a.acc = a.best + n;
    uint32_t *u = (uint32_t *)(a.acc + n);
    a.size = u; a.sr = u + n; a.sg = u + 2 * n; a.sb = u + 3 * n; a.sa = u + 4 * n; a.rc = u + 5 * n;
    a.pick = (int32_t *)(u + 6 * n);
    a.dust = (uint8_t *)(u + 7 * n);
    a.retired = a.dust + n;
    uint32_t *list = (uint32_t *)w->root_rank;  // the dust list borrows the rank buffer (relabelled at the end)
    long long *cnt = (long long *)(((uintptr_t)(a.retired + n) + 15) & ~(uintptr_t)15);
    a.budget = cnt; a.merged = (unsigned long long *)(cnt + 1); a.picks = (unsigned long long *)(cnt + 3);
    uint32_t *dcnt = (uint32_t *)(cnt + 2);
    a.err = w->err;
    a.threshold = p.threshold;
    a.min_size = p.min_size; a.max_size = p.max_size;
    const unsigned grid = (unsigned)std::min<size_t>((n + 255) / 256, (size_t)kSMs * 16);
    AMG_CUDA(cudaMemsetAsync(w->err, 0, sizeof(int), s));
    AMG_LAUNCH(k_cc_init, grid, 256, 0, s, present, labels, n);
    uint32_t count = 0;
    int rc = relabel_roots(w, labels, n, &count, s);  // counts the present pixels (labels rewritten below)
    if (rc) return rc;
    AMG_LAUNCH(k_cc_init, grid, 256, 0, s, present, labels, n);
    long long budget = count > p.blob_number ? (long long)(count - p.blob_number) : 0;
    AMG_CUDA(cudaMemsetAsync(a.retired, 0, n, s));
    auto stats = [&]() -> int {
        AMG_CUDA(cudaMemsetAsync(a.sx, 0, 2 * n * 8, s));
        AMG_CUDA(cudaMemsetAsync(a.size, 0, 5 * n * 4, s));
        AMG_LAUNCH(k_bm_stats, grid, 256, 0, s, a);
        AMG_LAUNCH(k_bm_mean, grid, 256, 0, s, a);
        return AM_OK;
    };
    auto finish_round = [&](unsigned long long *merged) -> int {
        AMG_LAUNCH(k_bm_flatten, grid, 256, 0, s, labels, n);
        int err = 0;
        AMG_CUDA(cudaMemcpyAsync(merged, a.merged, 8, cudaMemcpyDeviceToHost, s));
        AMG_CUDA(cudaMemcpyAsync(&budget, a.budget, 8, cudaMemcpyDeviceToHost, s));
        AMG_CUDA(cudaMemcpyAsync(&err, w->err, sizeof(int), cudaMemcpyDeviceToHost, s));
        AMG_CUDA(cudaStreamSynchronize(s));
        if (err) {
            set_error("blob merging exceeded its iteration bound");
            return AM_ERR_TIMEOUT;
        }
        return AM_OK;
    };
    // blobify_frame (thread.cpp:225-412): agglomerate until blob_number or no picks
    if (budget > 0 && p.max_size > 1) {
        AMG_CUDA(cudaMemcpyAsync(a.budget, &budget, 8, cudaMemcpyHostToDevice, s));
        for (uint32_t round = 0; round < 4096 && budget > 0; ++round) {
            a.key = mix32((uint32_t)p.seed * 0x9E3779B1u ^ round);
            if ((rc = stats())) return rc;
            AMG_LAUNCH(k_bm_best, grid, 256, 0, s, a, 0);
            AMG_LAUNCH(k_bm_best, grid, 256, 0, s, a, 1);
            AMG_LAUNCH(k_bm_propose, grid, 256, 0, s, a);
            AMG_CUDA(cudaMemsetAsync(a.merged, 0, 8, s));
            AMG_CUDA(cudaMemsetAsync(a.picks, 0, 8, s));
            AMG_LAUNCH(k_bm_union, grid, 256, 0, s, a);
            unsigned long long merged = 0, picks = 0;
            AMG_CUDA(cudaMemcpyAsync(&picks, a.picks, 8, cudaMemcpyDeviceToHost, s));
            if ((rc = finish_round(&merged))) return rc;
            if (!picks) break;  // no blob can grow (a round with picks may merge none by its coins)
        }
    }
    // unify_frame (thread.cpp:426-585): dust merges with the nearest dust
    if (budget > 0 && p.box_samples > 0 && p.min_size > 1) {
        if ((rc = stats())) return rc;
        AMG_LAUNCH(k_bm_mark_dust, grid, 256, 0, s, a);
        for (uint32_t round = 0; round < 256 && budget > 0; ++round) {
            a.key = mix32((uint32_t)p.seed * 0x85EBCA6Bu ^ round);
            AMG_CUDA(cudaMemsetAsync(dcnt, 0, 4, s));
            AMG_LAUNCH(k_bm_dust_list, grid, 256, 0, s, a, list, dcnt, kMaxDust);
            uint32_t nd = 0;
            AMG_CUDA(cudaMemcpyAsync(&nd, dcnt, 4, cudaMemcpyDeviceToHost, s));
            AMG_CUDA(cudaStreamSynchronize(s));
            if (nd > kMaxDust) {
                set_error("more than 65536 dust blobs below blob_min_size: not supported");
                return AM_ERR_UNSUPPORTED;
            }
            if (nd < 2) break;
            const unsigned gd = (unsigned)std::min<size_t>((nd + 255) / 256, (size_t)kSMs * 16);
            AMG_LAUNCH(k_bm_dust_pick, gd, 256, 0, s, a, list, nd, (uint32_t)p.box_grip);
            AMG_CUDA(cudaMemsetAsync(a.merged, 0, 8, s));
            AMG_LAUNCH(k_bm_dust_union, gd, 256, 0, s, a, list, nd);
            unsigned long long merged = 0;
            if ((rc = finish_round(&merged))) return rc;
            if (!merged) break;
            // sizes and centroids of the merged clouds for the next round
            AMG_CUDA(cudaMemsetAsync(a.sx, 0, 2 * n * 8, s));
            AMG_CUDA(cudaMemsetAsync(a.size, 0, 5 * n * 4, s));
            AMG_LAUNCH(k_bm_stats, grid, 256, 0, s, a);
        }
    }
    AMG_CUDA(cudaGetLastError());
    return relabel_roots(w, labels, n, nblobs, s);
}

int blob_stats(BlobWork *w, const int32_t *labels, const uint32_t *stored, uint32_t CW, uint32_t CH,
               uint32_t nblobs, unsigned long long *stats, cudaStream_t s) {
    (void)w;
    size_t n = (size_t)CW * CH;
    AMG_CUDA(cudaMemsetAsync(stats, 0, (size_t)nblobs * 7 * sizeof(unsigned long long), s));
    if (!n || !nblobs) return AM_OK;
    unsigned grid = (unsigned)std::min<size_t>((n + 255) / 256, (size_t)kSMs * 16);
    AMG_LAUNCH(k_blob_stats, grid, 256, 0, s, labels, stored, CW, n, stats, nblobs);
    AMG_CUDA(cudaGetLastError());
    return AM_OK;
}

int launch_blob_match(const MatchArgs &a, cudaStream_t s) {
    if (a.Wb == 0 || a.K == 0) return AM_OK;
    size_t smem = (size_t)a.Wb * a.K * sizeof(int32_t);
    if (smem > 200 * 1024) {
        set_error("blob map too large for the matching kernel");
        return AM_ERR_UNSUPPORTED;
    }
    if (smem > 48 * 1024) AMG_CUDA(cudaFuncSetAttribute(k_blob_match, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    AMG_LAUNCH(k_blob_match, 1, 512, smem, s, a);
    AMG_CUDA(cudaGetLastError());
    return AM_OK;
}

}  // namespace amg
