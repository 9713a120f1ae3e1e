// Blob stage: 4-connected component labelling of each key frame, exact blob
// statistics, and the blob matching sweep.
//
// With blob_threshold >= 1 (every colour distance is <= 1, color.h:17-24),
// blob_min_size <= 1, blob_max_size >= every component and blob_number <= the
// component count, the greedy merging of blobify_frame (thread.cpp:225-412)
// ends with exactly the 4-connected components of the opaque pixels and
// unify_frame (thread.cpp:426-585) leaves them unchanged; that regime is what
// these kernels compute.  Components are numbered by their first pixel in
// row-major order.
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
};

BlobWork *blob_work_create() { return new BlobWork(); }
void blob_work_destroy(BlobWork *w) {
    if (!w) return;
    if (w->tile_cnt) cudaFree(w->tile_cnt);
    if (w->root_rank) cudaFree(w->root_rank);
    if (w->err) cudaFree(w->err);
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
        AMG_CUDA(cudaMalloc(&w->tile_cnt, (ntiles + 1) * 4));
        w->tile_cap = ntiles + 1;
    }
    if (n > w->px_cap) {
        if (w->root_rank) cudaFree(w->root_rank);
        AMG_CUDA(cudaMalloc(&w->root_rank, n * 4));
        w->px_cap = n;
    }
    if (!w->err) AMG_CUDA(cudaMalloc(&w->err, sizeof(int)));
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
