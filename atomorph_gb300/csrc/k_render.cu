// Frame render (the atom path of morph::get_pixels(t), morph.cpp:452-678 and
// 1302-1421) as tile-binned CUDA kernels.
//
// Per key-frame pair (prepared once, reused by every output frame of the
// transition):
//   k_pair_prep    per atom: endpoints in 1/256 px, both colours with the
//                  alpha-0 substitution for a missing side (morph.cpp:500-522),
//                  Perlin lag/slope (morph.cpp:537-545, FP32), composite rank
//                  of its chain; keyed by the tile of the path midpoint.
//   radix sort + k_pair_gather   records reordered by that tile, so a warp's
//                  atoms land in few output tiles at any time of the pair.
// Per output frame:
//   k_frame_splat  exact position (LINEAR: the reference's double formula
//                  morph.cpp:1501-1515; SPLINE: the cyclic Catmull-Rom
//                  morph.cpp:526-531, spline.cpp:29-57, both evaluated with
//                  round-to-nearest FP64 operations and no fused multiply-add),
//                  colour fade, the four bilinear corners with the reference's
//                  bbox/size rules (morph.cpp:552-588), per-tile histogram.
//   scan           tile offsets.
//   k_frame_scatter  16-byte records into their tiles (a corner in a
//                  neighbouring tile duplicates the record there).
//   k_frame_resolve  one CTA per 32x32 tile: for each chain present, in the
//                  key frame's blob order, exact integer weighted means of the
//                  corners (weights (255-xf)(255-yf) etc. are integers, so the
//                  reference's per-pixel mean morph.cpp:593-623 is computed as
//                  an exactly rounded rational), then the ordered "over"
//                  composite morph.cpp:1348-1402 in FP64; 16-byte RGBA8 stores.
#include "common.cuh"
#include "kernels.h"
#include "render_math.cuh"

#include <cmath>
#include <cstring>
#include <new>
#include <vector>

namespace amg {

constexpr int kTile = 32;
constexpr uint32_t kInactive = 0xFFFFFFFFu;

// Prepared records of one key-frame pair (sorted by the tile of the path
// midpoint); kept per pair while the chains do not change, so a cycle of
// frames prepares each pair once.
struct PairData {
    int f = -1;                          // key frame of the pair held (-1: none)
    uint32_t motion = 0, fading = 0, width = 0, height = 0;
    bool noise = false;                  // mn holds the motion perturbation's noise values
    uint64_t cap = 0;
    int4 *pa = nullptr, *pb = nullptr;   // endpoints / spline control points
    uint2 *col = nullptr;
    float2 *ls = nullptr;
    float2 *mn = nullptr;                // motion noise (x, y) at the atom's first point
    uint32_t *rank = nullptr, *idx = nullptr;
    uint32_t *d_active = nullptr;        // active (sorted first) atoms, on the device
};

struct RenderWork {
    uint64_t cap = 0;       // atom capacity of the prep scratch below
    int4 *pa = nullptr, *pb = nullptr;   // unsorted prep output (scratch)
    uint2 *col = nullptr;
    float2 *ls = nullptr, *mn = nullptr;
    uint32_t *rank = nullptr;
    uint32_t *keys = nullptr, *vals = nullptr, *tkeys = nullptr, *tvals = nullptr, *hist = nullptr;
    uint4 *spl = nullptr;
    std::vector<PairData> pairs;         // cache slots
    uint4 *rec = nullptr;
    uint64_t rec_cap = 0;
    uint32_t *tile_cnt = nullptr, *tile_off = nullptr, *tile_cur = nullptr;
    uint32_t ntiles_cap = 0;
    uint32_t *zero = nullptr;   // a zero overflow count for the separate-kernel path
    // Fused frames are pipelined over two record slots: the pair preparation,
    // binning and planning of a frame run on `bs` while the previous frame
    // resolves on the render stream.  Each slot holds its tile regions
    // (planned from the previous frame's counts), their records and the
    // overflow list.
    struct Slot {
        uint4 *rec = nullptr, *ovf = nullptr;
        uint32_t *off = nullptr, *cap = nullptr, *cnt = nullptr, *ovf_cnt = nullptr;
        uint32_t tiles = 0;              // tiles the plan in off / cap is for (0: none)
        uint64_t atoms = 0;              // atom count it was planned for
        cudaEvent_t resolved = nullptr;  // after the last resolve that read the slot
    } slot[2];
    int cur = 0;                         // slot of the next fused frame
    uint64_t slot_rec_cap = 0, slot_ovf_cap = 0;
    uint32_t slot_tiles_cap = 0;
    cudaStream_t bs = nullptr;
    cudaEvent_t binned = nullptr, mark = nullptr;
    bool bs_after_s = false;             // bs must wait for the render stream before its next work
    bool s_after_bs = false;             // the render stream must wait for bs before touching slots or pairs
    int *perm = nullptr;    // [4][512] Perlin permutations on the device (lag, slope, motion x, motion y)
    bool perm_set = false;
    Prof *prof = nullptr;   // optional per-kernel timing
    // A frame binned before its call (render_frame's `ahead`): its records
    // are in slot[cur] and w->binned marks their end on bs.  The next fused
    // frame uses them when it is exactly that time and scene, and plans the
    // slot afresh otherwise.
    struct Ahead {
        bool valid = false;
        double time = 0.0;
        uint64_t key = 0;
        RenderScene sc;
    } ahead;
    // Heavy tiles: the resolves' count of this morph's frames and the note
    // its heavy tiles leave (host-mapped: frame number << 32 | heavy tiles).
    uint32_t frame_no = 0, last_helpers = 0;
    unsigned long long *note_host = nullptr, *note_dev = nullptr;
    bool note_tried = false;
};

// Drops a frame binned ahead: the slot it filled is planned afresh by the
// next fused frame (stream order puts that plan after the binning).
static void drop_ahead(RenderWork *w) {
    if (!w->ahead.valid) return;
    w->slot[w->cur].tiles = 0;
    w->ahead.valid = false;
}

// Every scene field a fused frame's binning and resolve read.
static bool same_scene(const RenderScene &a, const RenderScene &b) {
    return a.K == b.K && a.C == b.C && a.N == b.N && a.CW == b.CW && a.CH == b.CH && a.width == b.width &&
           a.height == b.height && a.bbox[0] == b.bbox[0] && a.bbox[1] == b.bbox[1] && a.bbox[2] == b.bbox[2] &&
           a.bbox[3] == b.bbox[3] && a.motion == b.motion && a.fading == b.fading && a.density == b.density &&
           a.P == b.P && a.chain_off == b.chain_off && a.display == b.display && a.rank == b.rank &&
           a.pipeline == b.pipeline && a.feather == b.feather && a.keep_background == b.keep_background &&
           a.show_blobs == b.show_blobs && a.present == b.present && a.blob_col == b.blob_col && a.perm == b.perm &&
           a.motion_noise == b.motion_noise && a.only_rank == b.only_rank && a.aux == b.aux &&
           a.bin_ctas == b.bin_ctas && a.resolve_ctas == b.resolve_ctas;
}

// Device memory the pair cache may hold (beyond one pair, which is always
// kept): all K pairs of a 1M-atom, 8-key-frame morph take 450 MB.
constexpr uint64_t kPairCacheBytes = 8ull << 30;
constexpr uint64_t kPairBytesPerAtom = 16 + 16 + 8 + 8 + 8 + 4 + 4;

void render_set_prof(RenderWork *w, Prof *p) { w->prof = p; }
Prof *render_prof(RenderWork *w) { return w ? w->prof : nullptr; }

RenderWork *render_work_create() { return new RenderWork(); }

static void pair_free(PairData &d) {
    void *ps[] = {d.pa, d.pb, d.col, d.ls, d.mn, d.rank, d.idx, d.d_active};
    for (void *p : ps)
        if (p) cudaFree(p);
    d = PairData();
}

static void rw_free(RenderWork *w) {
    void *ps[] = {w->pa, w->pb, w->col, w->ls, w->mn, w->rank, w->keys, w->vals, w->tkeys, w->tvals, w->hist, w->spl};
    for (void *p : ps)
        if (p) cudaFree(p);
    w->pa = w->pb = nullptr;
    w->col = nullptr;
    w->ls = w->mn = nullptr;
    w->rank = w->keys = w->vals = w->tkeys = w->tvals = w->hist = nullptr;
    w->spl = nullptr;
    w->cap = 0;
    for (auto &d : w->pairs) pair_free(d);
    w->pairs.clear();
}

static void slot_free(RenderWork::Slot &sl) {
    void *pl[] = {sl.rec, sl.ovf, sl.off, sl.cap, sl.cnt, sl.ovf_cnt};
    for (void *q : pl)
        if (q) cudaFree(q);
    sl.rec = sl.ovf = nullptr;
    sl.off = sl.cap = sl.cnt = sl.ovf_cnt = nullptr;
    sl.tiles = 0;
    sl.atoms = 0;
}

void render_quiesce(RenderWork *w) {
    if (w && w->bs) cudaStreamSynchronize(w->bs);
}

void render_work_destroy(RenderWork *w) {
    if (!w) return;
    render_quiesce(w);
    rw_free(w);
    if (w->rec) cudaFree(w->rec);
    if (w->tile_cnt) cudaFree(w->tile_cnt);
    if (w->tile_off) cudaFree(w->tile_off);
    if (w->tile_cur) cudaFree(w->tile_cur);
    if (w->perm) cudaFree(w->perm);
    if (w->zero) cudaFree(w->zero);
    for (auto &sl : w->slot) {
        slot_free(sl);
        if (sl.resolved) cudaEventDestroy(sl.resolved);
    }
    if (w->binned) cudaEventDestroy(w->binned);
    if (w->mark) cudaEventDestroy(w->mark);
    if (w->bs) cudaStreamDestroy(w->bs);
    if (w->note_host) cudaFreeHost(w->note_host);
    delete w;
}

const int *render_perm(RenderWork *w) { return w->perm_set ? w->perm : nullptr; }

void render_invalidate(RenderWork *w) {
    for (auto &d : w->pairs) d.f = -1;
    drop_ahead(w);
}

int render_set_perlin(RenderWork *w, const int *perm_lag, const int *perm_slope, const int *perm_mx,
                      const int *perm_my) {
    // frames in flight may still read the permutations (a seed change is rare)
    AMG_CUDA(cudaDeviceSynchronize());
    if (!w->perm) AMG_ALLOC(&w->perm, 2048 * sizeof(int));
    std::vector<int> h(2048);
    std::memcpy(h.data(), perm_lag, 512 * sizeof(int));
    std::memcpy(h.data() + 512, perm_slope, 512 * sizeof(int));
    std::memcpy(h.data() + 1024, perm_mx, 512 * sizeof(int));
    std::memcpy(h.data() + 1536, perm_my, 512 * sizeof(int));
    AMG_CUDA(cudaMemcpy(w->perm, h.data(), 2048 * sizeof(int), cudaMemcpyHostToDevice));
    w->perm_set = true;
    render_invalidate(w);
    return AM_OK;
}

static int rw_reserve(RenderWork *w, uint64_t n) {
    if (n <= w->cap) return AM_OK;
    rw_free(w);
    uint64_t c = n + n / 8 + 1024;
    AMG_ALLOC(&w->pa, c * sizeof(int4));
    AMG_ALLOC(&w->pb, c * sizeof(int4));
    AMG_ALLOC(&w->col, c * sizeof(uint2));
    AMG_ALLOC(&w->ls, c * sizeof(float2));
    AMG_ALLOC(&w->mn, c * sizeof(float2));
    AMG_ALLOC(&w->rank, c * 4);
    AMG_ALLOC(&w->keys, c * 4);
    AMG_ALLOC(&w->vals, c * 4);
    AMG_ALLOC(&w->tkeys, c * 4);
    AMG_ALLOC(&w->tvals, c * 4);
    AMG_ALLOC(&w->hist, radix_hist_words(c) * 4);
    AMG_ALLOC(&w->spl, c * sizeof(uint4));
    w->cap = c;
    return AM_OK;
}

static int pair_reserve(PairData &d, uint64_t c) {
    if (d.cap >= c) return AM_OK;
    pair_free(d);
    AMG_ALLOC(&d.pa, c * sizeof(int4));
    AMG_ALLOC(&d.pb, c * sizeof(int4));
    AMG_ALLOC(&d.col, c * sizeof(uint2));
    AMG_ALLOC(&d.ls, c * sizeof(float2));
    AMG_ALLOC(&d.mn, c * sizeof(float2));
    AMG_ALLOC(&d.rank, c * 4);
    AMG_ALLOC(&d.idx, c * 4);
    AMG_ALLOC(&d.d_active, 4);
    d.cap = c;
    return AM_OK;
}

namespace {

__device__ __forceinline__ uint32_t find_chain_r(const uint64_t *__restrict__ off, uint32_t C, uint64_t r) {
    uint32_t lo = 0, hi = C;
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) >> 1;
        if (__ldg(off + mid) <= r) lo = mid; else hi = mid;
    }
    return lo;
}

__global__ void __launch_bounds__(256) k_pair_prep(RenderScene sc, uint32_t f, const int *__restrict__ perm,
                                                    int4 *pa, int4 *pb, uint2 *col, float2 *ls, float2 *mn,
                                                    uint32_t *rank, uint32_t *keys, uint32_t *vals, uint32_t tiles_x,
                                                    uint32_t inactive_key, uint32_t key_shift) {
    __shared__ int sp[2048];  // lag, slope, motion x, motion y permutations
    for (int i = threadIdx.x; i < 2048; i += blockDim.x) sp[i] = perm ? perm[i] : 0;
    __syncthreads();
    const int bwi = (int)(sc.bbox[2] - sc.bbox[0] + 1), bhi = (int)(sc.bbox[3] - sc.bbox[1] + 1);
    const uint32_t y = f, yn = (f + 1) % sc.K;
    const float bw = (float)(sc.bbox[2] - sc.bbox[0] + 1), bh = (float)(sc.bbox[3] - sc.bbox[1] + 1);
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < sc.N; i += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t w1 = sc.P[(uint64_t)y * sc.N + i], w2 = sc.P[(uint64_t)yn * sc.N + i];
        bool h1 = pt_flags(w1) & kHasPixel, h2 = pt_flags(w2) & kHasPixel;
        vals[i] = (uint32_t)i;
        if (!h1 && !h2) {
            rank[i] = kInactive;
            keys[i] = inactive_key;
            continue;
        }
        uint32_t c = find_chain_r(sc.chain_off, sc.C, i);
        uint32_t c1 = 0, c2 = 0;
        const size_t fr = (size_t)sc.CH * sc.CW;
        if (h1) c1 = sc.display[(size_t)y * fr + (size_t)pt_y(w1) * sc.CW + pt_x(w1)];
        if (h2) c2 = sc.display[(size_t)yn * fr + (size_t)pt_y(w2) * sc.CW + pt_x(w2)];
        if (h1 && !h2) c2 = c1 & 0x00FFFFFFu;
        if (h2 && !h1) c1 = c2 & 0x00FFFFFFu;
        int32_t X1 = pt_X(w1), Y1 = pt_Y(w1), X2 = pt_X(w2), Y2 = pt_Y(w2);
        if (sc.motion == AM_SPLINE) {
            uint32_t K = sc.K;
            uint32_t s0 = (f + K - 1) % K, s2 = (f + 1) % K, s3 = (f + 2) % K;
            uint64_t q0 = sc.P[(uint64_t)s0 * sc.N + i], q2 = sc.P[(uint64_t)s2 * sc.N + i],
                     q3 = sc.P[(uint64_t)s3 * sc.N + i];
            pa[i] = make_int4(pt_X(q0), pt_Y(q0), X1, Y1);
            pb[i] = make_int4(pt_X(q2), pt_Y(q2), pt_X(q3), pt_Y(q3));
        } else {
            pa[i] = make_int4(X1, Y1, X2, Y2);
        }
        col[i] = make_uint2(c1, c2);
        float lag = 0.5f, slope = 0.5f;
        if (sc.fading == AM_PERLIN) {
            // morph.cpp:540-545: pt1 normalised by the bbox, frequency 8.
            float px = ((float)((int)pt_x(w1) - (int)sc.bbox[0]) * 256.f + (float)pt_xf(w1)) / (bw * 256.f) * 8.f;
            float py = ((float)((int)pt_y(w1) - (int)sc.bbox[1]) * 256.f + (float)pt_yf(w1)) / (bh * 256.f) * 8.f;
            lag = poctave(sp, px, py) * 0.5f + 0.5f;
            slope = poctave(sp + 512, px, py) * 0.5f + 0.5f;
        }
        ls[i] = fade_params(lag, slope);
        if (mn) {
            // the motion perturbation's noise at pt1 (x map seed + 2, y map seed + 3)
            const float u = noise_coord_rn((int)pt_x(w1), (int)pt_xf(w1), (int)sc.bbox[0], bwi);
            const float v = noise_coord_rn((int)pt_y(w1), (int)pt_yf(w1), (int)sc.bbox[1], bhi);
            mn[i] = make_float2(poctave_rn(sp + 1024, u, v), poctave_rn(sp + 1536, u, v));
        }
        rank[i] = (uint32_t)sc.rank[(size_t)f * sc.C + c];
        int mx = ((X1 + X2) >> 9), my = ((Y1 + Y2) >> 9);
        mx = min(max(mx, 0), (int)sc.width - 1);
        my = min(max(my, 0), (int)sc.height - 1);
        // tile-major, row-major inside the tile (below 2^21 tiles): where the
        // motion is coherent a warp's atoms sit in a row of distinct columns,
        // so the resolve's shared accumulators (banked by column) see few
        // conflicts
        const uint32_t tile = (uint32_t)((my / kTile) * tiles_x + (mx / kTile));
        keys[i] = key_shift ? (tile << key_shift) | ((uint32_t)(my % kTile) << 5) | (uint32_t)(mx % kTile) : tile;
    }
}

__global__ void k_pair_gather(const uint32_t *__restrict__ keys, const uint32_t *__restrict__ order, uint64_t n,
                              const int4 *pa, const int4 *pb, const uint2 *col, const float2 *ls, const float2 *mn,
                              const uint32_t *rank, int4 *pa2, int4 *pb2, uint2 *col2, float2 *ls2, float2 *mn2,
                              uint32_t *rank2, uint32_t *idx2, int spline, uint32_t *active) {
    for (uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; j < n; j += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t i = order[j];
        uint32_t r = rank[i];
        rank2[j] = r;
        idx2[j] = i;
        if (r == kInactive) {
            if (j == 0 || rank[order[j - 1]] != kInactive) *active = (uint32_t)j;
            continue;
        }
        pa2[j] = pa[i];
        if (spline) pb2[j] = pb[i];
        col2[j] = col[i];
        ls2[j] = ls[i];
        if (mn) mn2[j] = mn[i];
        if (j + 1 == n) *active = (uint32_t)n;
    }
}

// Up to four distinct tiles touched by the valid corners of base pixel
// (px, py); returns the count.
__device__ __forceinline__ int corner_tiles(uint32_t px, uint32_t py, uint32_t valid, uint32_t tiles_x,
                                            uint32_t *t) {
    int n = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (!(valid & (1u << k))) continue;
        uint32_t cx = px + (k & 1), cy = py + (k >> 1);
        uint32_t tt = (cy / kTile) * tiles_x + cx / kTile;
        bool dup = false;
        for (int j = 0; j < n; ++j) dup |= t[j] == tt;
        if (!dup) t[n++] = tt;
    }
    return n;
}

struct SplatIn {
    const int4 *pa, *pb;
    const uint2 *col;
    const float2 *ls;
    const uint32_t *rank, *idx;
    const float2 *mn;  // motion noise per atom (read when the frame's noise scale is not 0)
};

// One atom at the frame's time: exact position, faded colour and the valid
// bilinear corners (morph.cpp:523-588), packed as the 16-byte splat record
// {px | py << 16, xf | yf << 8 | valid << 16, colour, rank}.
// Control coordinates of atom i for the frame: LINEAR/none use a = pa[i]
// (x1, y1, x2, y2); SPLINE uses a = (q0.x, q0.y, q1.x, q1.y) and
// b = (q2.x, q2.y, q3.x, q3.y).
__device__ __forceinline__ void atom_controls(const RenderScene &sc, const FrameArgs &fa, const SplatIn &in,
                                              uint64_t i, int4 &a, int4 &b) {
    a = in.pa[i];
    b = make_int4(0, 0, 0, 0);
    if (sc.motion == AM_SPLINE) {
        if (fa.seg_ok) {
            b = in.pb[i];
        } else {
            uint64_t o = in.idx[i];
            uint64_t q0 = sc.P[(uint64_t)fa.seg[0] * sc.N + o], q1 = sc.P[(uint64_t)fa.seg[1] * sc.N + o];
            uint64_t q2 = sc.P[(uint64_t)fa.seg[2] * sc.N + o], q3 = sc.P[(uint64_t)fa.seg[3] * sc.N + o];
            a = make_int4(pt_X(q0), pt_Y(q0), pt_X(q1), pt_Y(q1));
            b = make_int4(pt_X(q2), pt_Y(q2), pt_X(q3), pt_Y(q3));
        }
    }
}

// Position of one axis by the exact integer paths; false when the value sits
// too close to a rounding boundary and the reference's double formula must
// decide (axis_fixed).
__device__ __forceinline__ bool axis_fast(const RenderScene &sc, const FrameArgs &fa, int axis, const int4 &a,
                                          const int4 &b, uint32_t *out) {
    const int32_t c0 = axis ? a.y : a.x, c1 = axis ? a.w : a.z, c2 = axis ? b.y : b.x, c3 = axis ? b.w : b.z;
    if (sc.motion == AM_LINEAR) {
        int32_t v;
        if (!lin_fast(fa, c0, c1, &v)) return false;
        *out = (uint32_t)v;
        return true;
    }
    if (sc.motion == AM_SPLINE) return spl_fast(fa, c0, c1, c2, c3, out);
    *out = (uint32_t)c0;
    return true;
}
__device__ __forceinline__ uint32_t axis_fixed(const RenderScene &sc, const FrameArgs &fa, int axis, const int4 &a,
                                               const int4 &b) {
    const int32_t c0 = axis ? a.y : a.x, c1 = axis ? a.w : a.z, c2 = axis ? b.y : b.x, c3 = axis ? b.w : b.z;
    if (sc.motion == AM_LINEAR) return (uint32_t)lin_fixed(fa.w1, fa.w2, c0, c1);
    return spl_fixed(fa.b0, fa.b1, fa.b2, fa.b3, c0, c1, c2, c3);
}

// The splat record of an atom at 1/256-px position (X, Y): base pixel,
// fractions and the valid bilinear corners with the reference's bbox/size
// rules (morph.cpp:552-588), packed as
// {px | py << 16, xf | yf << 8 | valid << 16, colour, rank}.
__device__ __forceinline__ uint4 finish_record(const RenderScene &sc, uint32_t X, uint32_t Y, uint32_t colour,
                                               uint32_t rr) {
    uint32_t px = X >> 8, py = Y >> 8, xf = X & 255u, yf = Y & 255u;
    if (px + 1 < sc.width && py + 1 < sc.height) {
        // every corner inside the output: the rules reduce to positive weights
        const uint32_t l = xf < 255u, r = xf > 0u, t = yf < 255u, d = yf > 0u;
        const uint32_t valid = (l & t) | ((r & t) << 1) | ((l & d) << 2) | ((r & d) << 3);
        return make_uint4(px | (py << 16), xf | (yf << 8) | (valid << 16), colour, rr);
    }
    uint32_t valid = 0;
    const uint32_t bx1 = sc.bbox[0], by1 = sc.bbox[1], bx2 = sc.bbox[2], by2 = sc.bbox[3];
    bool skip = (px >= sc.width || py >= sc.height) && (px > bx2 || px < bx1 || py > by2 || py < by1);
    if (!skip) {
        if (xf < 255u && yf < 255u) valid |= 1u;
        if ((px < bx2 || px + 1 < sc.width) && xf > 0u && yf < 255u) valid |= 2u;
        if ((py < by2 || py + 1 < sc.height) && xf < 255u && yf > 0u) valid |= 4u;
        if (xf > 0u && yf > 0u && ((py < by2 && px < bx2) || (py + 1 < sc.height && px + 1 < sc.width)))
            valid |= 8u;
        // Corners outside the output are dropped (they only arise when the
        // resolution is smaller than the key frames' bounding box).
        if (px >= sc.width || py >= sc.height) valid &= ~1u;
        if (px + 1 >= sc.width || py >= sc.height) valid &= ~2u;
        if (px >= sc.width || py + 1 >= sc.height) valid &= ~4u;
        if (px + 1 >= sc.width || py + 1 >= sc.height) valid &= ~8u;
    }
    return make_uint4(px | (py << 16), xf | (yf << 8) | (valid << 16), colour, rr);
}

// One atom at the frame's time: exact position, faded colour (morph.cpp:
// 523-588) and its splat record, FP64 fallback inline.
__device__ __forceinline__ uint4 splat_atom(const RenderScene &sc, const FrameArgs &fa, const SplatIn &in,
                                            uint64_t i) {
    int4 a, b;
    atom_controls(sc, fa, in, i, a, b);
    uint32_t X, Y;
    if (!axis_fast(sc, fa, 0, a, b, &X)) X = axis_fixed(sc, fa, 0, a, b);
    if (!axis_fast(sc, fa, 1, a, b, &Y)) Y = axis_fixed(sc, fa, 1, a, b);
    if (fa.noise_s != 0.f) {
        const float2 nz = in.mn[i];
        X = displace_rn(X, fa.noise_s, nz.x);
        Y = displace_rn(Y, fa.noise_s, nz.y);
    }
    uint2 c = in.col[i];
    float2 q = in.ls[i];
    return finish_record(sc, X, Y, fade_colour(sc.fading, c.x, c.y, q, fa.str), in.rank[i]);
}

// Tiles of the valid corners of a splat record, each distinct tile once:
// bit k of the returned mask marks corner k as the first valid corner in its
// tile; tk[k] is that corner's tile.  The four corners span at most 2 x 2
// tiles: corner k is in the base pixel's tile moved one tile right when k is
// a right corner and the base pixel is the last column of its tile, one down
// likewise.  Registers only.
__device__ __forceinline__ uint32_t record_tiles(uint4 s, uint32_t tiles_x, uint32_t *tk) {
    const uint32_t px = s.x & 0xFFFFu, py = s.x >> 16, valid = (s.y >> 16) & 15u;
    const uint32_t t00 = (py / kTile) * tiles_x + px / kTile;
    const bool cx = (px % kTile) == kTile - 1, cy = (py % kTile) == kTile - 1;
    const uint32_t dx = cx ? 1u : 0u, dy = cy ? tiles_x : 0u;
    tk[0] = t00;
    tk[1] = t00 + dx;
    tk[2] = t00 + dy;
    tk[3] = t00 + dx + dy;
    uint32_t m = valid;
    if (!cx && !cy) return m & (0u - m);                                 // one tile: its lowest valid corner
    if (!cx) return (m & 0x5u) | (m & 0xAu & ~((m & 0x5u) << 1));        // corners 0,1 and 2,3 share tiles
    if (!cy) return (m & 0x3u) | (m & 0xCu & ~((m & 0x3u) << 2));        // corners 0,2 and 1,3 share tiles
    return m;                                                            // four tiles
}

__global__ void __launch_bounds__(256) k_frame_splat(RenderScene sc, FrameArgs fa, const uint32_t *n_dev,
                                                      SplatIn in, uint4 *spl, uint32_t *tile_cnt) {
    const uint64_t n = *n_dev;
    extern __shared__ uint32_t hist[];
    const bool smem_hist = fa.ntiles <= 8192;
    if (smem_hist) {
        for (uint32_t i = threadIdx.x; i < fa.ntiles; i += blockDim.x) hist[i] = 0;
        __syncthreads();
    }
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        uint4 rec = splat_atom(sc, fa, in, i);
        spl[i] = rec;
        uint32_t tk[4];
        uint32_t m = record_tiles(rec, fa.tiles_x, tk);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            if (!(m & (1u << k))) continue;
            if (smem_hist) atomicAdd(&hist[tk[k]], 1u);
            else atomicAdd(&tile_cnt[tk[k]], 1u);
        }
    }
    if (smem_hist) {
        __syncthreads();
        for (uint32_t i = threadIdx.x; i < fa.ntiles; i += blockDim.x)
            if (hist[i]) atomicAdd(&tile_cnt[i], hist[i]);
    }
}

// Every active atom's position words at the frame's time (the readout of the
// positions the splat uses): xy[2 idx], xy[2 idx + 1], idx the atom's column.
__global__ void __launch_bounds__(256) k_atom_positions(RenderScene sc, FrameArgs fa, const uint32_t *n_dev,
                                                         SplatIn in, int32_t *xy) {
    const uint64_t n = *n_dev;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        int4 a, b;
        atom_controls(sc, fa, in, i, a, b);
        uint32_t X, Y;
        if (!axis_fast(sc, fa, 0, a, b, &X)) X = axis_fixed(sc, fa, 0, a, b);
        if (!axis_fast(sc, fa, 1, a, b, &Y)) Y = axis_fixed(sc, fa, 1, a, b);
        if (fa.noise_s != 0.f) {
            const float2 nz = in.mn[i];
            X = displace_rn(X, fa.noise_s, nz.x);
            Y = displace_rn(Y, fa.noise_s, nz.y);
        }
        const uint64_t o = in.idx[i];
        xy[2 * o] = (int32_t)X;
        xy[2 * o + 1] = (int32_t)Y;
    }
}

// ---------------------------------------------------------------------------
// Fused splat + binning without waiting for other CTAs.  Each tile owns a
// region of the record buffer planned from the previous frame's tile counts
// (atoms move continuously from frame to frame, so the counts change little;
// k_tile_plan sizes the regions with slack).  A CTA splats a contiguous chunk
// of atoms into shared memory, counts its records per tile, reserves its
// share of every tile it touches with one global atomic per tile and writes
// the records straight into the tiles' regions; records past a region's
// capacity go to the overflow list, tile in bits 20-31 of .y, which the
// resolve also reads.  No grid barrier, no scan in the frame's path.
constexpr int kBinThreads = 256;
// Dynamic shared memory that lets at most n CTAs share an SM (227 KB per SM
// for CTAs, 1 KB of it reserved per CTA, a little static shared memory each).
inline size_t occupancy_smem(uint32_t n) { return (size_t)(227 * 1024) / std::max<uint32_t>(n, 1) - 2048; }
constexpr uint32_t kBinMaxTiles = 2048;
constexpr uint32_t kBinPer = 2;        // records per thread held in shared memory

struct BinArgs {
    RenderScene sc;
    FrameArgs fa;
    const uint32_t *n;      // atoms of the pair (device; the grid covers an upper bound)
    SplatIn in;
    uint4 *rec;             // tile regions
    const uint32_t *off, *cap;  // [ntiles] region start and capacity
    uint32_t *cnt;          // [ntiles] records reserved; zero on entry
    uint4 *ovf;             // overflow records
    uint32_t *ovf_cnt;      // zero on entry
    uint32_t ovf_cap;
};

// Dynamic shared memory of k_frame_bin: records [per][256] uint4, tile
// histogram and CTA bases [ntiles] u32 each, fallback list [per][512] u16.
inline size_t bin_smem(uint32_t per, uint32_t ntiles) {
    return (size_t)per * kBinThreads * 16 + (size_t)ntiles * 8 + (size_t)per * kBinThreads * 2 * 2;
}

constexpr uint32_t kNoAtom = 0xFFFFFFFFu;  // X of a record slot past the last atom

// One atom's inputs for a frame: its control coordinates, colours, fade
// ramp, composite rank and (with the motion perturbation) noise pair.
struct AtomIn {
    int4 a, c;
    uint2 col;
    float2 q;
    uint32_t rank;
    float2 nz;
};
__device__ __forceinline__ void load_atom(const BinArgs &b, uint64_t i, bool noise, AtomIn &x) {
    atom_controls(b.sc, b.fa, b.in, i, x.a, x.c);
    x.col = b.in.col[i];
    x.q = b.in.ls[i];
    x.rank = b.in.rank[i];
    x.nz = noise ? b.in.mn[i] : make_float2(0.f, 0.f);
}

// The binning of one frame's atom chunk `cta` (kBinPer * kBinThreads atoms).
__device__ __forceinline__ void frame_bin(const BinArgs &b, uint32_t cta) {
    extern __shared__ __align__(16) unsigned char bsm[];
    const uint32_t ntiles = b.fa.ntiles, tid = threadIdx.x, per = kBinPer;
    uint4 *srec = reinterpret_cast<uint4 *>(bsm);
    uint32_t *hist = reinterpret_cast<uint32_t *>(bsm + (size_t)per * kBinThreads * 16);
    uint32_t *base = hist + ntiles;
    uint16_t *fix = reinterpret_cast<uint16_t *>(base + ntiles);
    __shared__ uint32_t nfix;
    const uint64_t chunk0 = (uint64_t)cta * per * kBinThreads;
    const uint64_t n_atoms = *b.n;
    if (chunk0 >= n_atoms) return;  // past the pair's active atoms
    for (uint32_t t = tid; t < ntiles; t += kBinThreads) hist[t] = 0;
    if (tid == 0) nfix = 0;
    __syncthreads();
    // ---- positions by the integer paths.  Axes that need the reference's
    // double formula are listed and evaluated together afterwards, so the
    // slow FP64 work runs in full warps instead of holding up every warp
    // that contains one such atom.
    const bool noise = b.fa.noise_s != 0.f;
    for (uint32_t r = 0; r < kBinPer; ++r) {
        const uint32_t slot = r * kBinThreads + tid;
        const uint64_t i = chunk0 + slot;
        uint4 v = make_uint4(kNoAtom, 0, 0, 0);
        uint32_t need = 0;
        if (i < n_atoms) {
            AtomIn x;
            load_atom(b, i, noise, x);
            if (axis_fast(b.sc, b.fa, 0, x.a, x.c, &v.x)) {
                if (noise) v.x = displace_rn(v.x, b.fa.noise_s, x.nz.x);
            } else {
                need |= 1u;
            }
            if (axis_fast(b.sc, b.fa, 1, x.a, x.c, &v.y)) {
                if (noise) v.y = displace_rn(v.y, b.fa.noise_s, x.nz.y);
            } else {
                need |= 2u;
            }
            v.z = fade_colour(b.sc.fading, x.col.x, x.col.y, x.q, b.fa.str);
            v.w = x.rank;
        }
        srec[slot] = v;
        const uint32_t k = __popc(need);
        if (k) {
            const uint32_t at = atomicAdd(&nfix, k);
            uint32_t e = 0;
            if (need & 1u) fix[at + e++] = (uint16_t)(slot * 2);
            if (need & 2u) fix[at + e] = (uint16_t)(slot * 2 + 1);
        }
    }
    __syncthreads();
    for (uint32_t j = tid; j < nfix; j += kBinThreads) {
        const uint32_t e = fix[j], slot = e >> 1, axis = e & 1u;
        int4 a, c;
        atom_controls(b.sc, b.fa, b.in, chunk0 + slot, a, c);
        uint32_t v = axis_fixed(b.sc, b.fa, (int)axis, a, c);
        if (noise) {
            const float2 nz = b.in.mn[chunk0 + slot];
            v = displace_rn(v, b.fa.noise_s, axis ? nz.y : nz.x);
        }
        if (axis) srec[slot].y = v;
        else srec[slot].x = v;
    }
    __syncthreads();
    for (uint32_t r = 0; r < per; ++r) {
        const uint32_t slot = r * kBinThreads + tid;
        const uint4 v = srec[slot];
        const uint4 rec = v.x == kNoAtom ? make_uint4(0, 0, 0, 0) : finish_record(b.sc, v.x, v.y, v.z, v.w);
        srec[slot] = rec;
        uint32_t tk[4];
        uint32_t m = record_tiles(rec, b.fa.tiles_x, tk);
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (m & (1u << k)) atomicAdd(&hist[tk[k]], 1u);
    }
    __syncthreads();
    // ---- this CTA's share of every tile it touches: hist becomes the CTA's
    // write cursor in the record buffer, base the end of the tile's region
    for (uint32_t t = tid; t < ntiles; t += kBinThreads) {
        const uint32_t h = hist[t];
        if (h) {
            const uint32_t o = b.off[t];
            hist[t] = o + atomicAdd(&b.cnt[t], h);
            base[t] = o + b.cap[t];
        }
    }
    __syncthreads();
    // ---- records into the tiles' regions (the overflow list past capacity)
    for (uint32_t r = 0; r < per; ++r) {
        const uint4 rec = srec[r * kBinThreads + tid];
        uint32_t tk[4];
        uint32_t m = record_tiles(rec, b.fa.tiles_x, tk);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            if (!(m & (1u << k))) continue;
            const uint32_t t = tk[k], pos = atomicAdd(&hist[t], 1u);
            if (pos < base[t]) {
                b.rec[pos] = rec;
            } else {
                const uint32_t o = atomicAdd(b.ovf_cnt, 1u);
                if (o < b.ovf_cap) b.ovf[o] = make_uint4(rec.x, rec.y | (t << 20), rec.z, rec.w);
            }
        }
    }
}

__global__ void __launch_bounds__(kBinThreads, 8) k_frame_bin(const __grid_constant__ BinArgs b) {
    frame_bin(b, blockIdx.x);
}

// Frames of several morphs rendered by one launch per kernel (am_batch_render):
// the jobs' CTAs (atom chunks, tiles, plans) follow one another in the grid,
// job j's from start[j]; every CTA runs the single-frame code on its own
// job's arguments, so each job's frame is the one its own launches give.
// The arguments travel as kernel parameters (constant bank, read uniformly).
constexpr uint32_t kBatchFrames = 32;
__device__ __forceinline__ uint32_t batch_job(const uint32_t *start, uint32_t n, uint32_t cta) {
    uint32_t lo = 0, hi = n;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (start[mid] <= cta) lo = mid;
        else hi = mid;
    }
    return lo;
}
struct BinBatch {
    uint32_t n;
    uint32_t start[kBatchFrames + 1];
    BinArgs job[kBatchFrames];
};
__global__ void __launch_bounds__(kBinThreads) k_frame_bin_batch(const __grid_constant__ BinBatch bb) {
    const uint32_t j = batch_job(bb.start, bb.n, blockIdx.x);
    frame_bin(bb.job[j], blockIdx.x - bb.start[j]);
}

// Heavy tiles: a tile with more than kHeavyRec binned records (atoms crowded
// or stacked by a chain much wider than a key frame's blob) would keep one
// CTA busy for milliseconds while the rest of the frame is done, its warps
// waiting on shared-memory atomics with nothing else to run.  The tile plan
// after a frame's binning counts the frame's heavy tiles and notes the frame
// and the count in host-mapped memory; from that note the host launches the
// morph's next frames (for kHeavyMemory frames after the last heavy one)
// with the heavy resolve: its grid ends with `helpers` extra CTAs, and the
// first helpers / (kBands - 1) heavy tiles in tile order are resolved by
// kBands CTAs each, the tile's own CTA taking row band 0 and the helpers
// bands 1 .. kBands - 1.  Every CTA of a tile reads all its records and
// accumulates, composites and writes only the rows of its band, so no CTA
// waits for another and the pixels are the ones a single CTA gives.  Frames
// of morphs without heavy tiles use the plain resolve.
constexpr uint32_t kHeavyRec = 8192;
constexpr uint32_t kBands = 32;       // one row each
constexpr uint32_t kHeavyMaxTiles = 64;
__device__ __forceinline__ uint32_t band_rows(uint32_t b) {
    constexpr uint32_t rpb = 32 / kBands;
    return (rpb >= 32 ? 0xFFFFFFFFu : ((1u << rpb) - 1u)) << (b * rpb);
}

// A frame's tile regions from the previous frame's counts src_cnt (one CTA):
// capacity count + count / 4 + 32 (or, with init, the atoms spread evenly),
// regions in tile order, clipped to the buffer; the destination slot's
// counters (cnt, ovf_cnt) are cleared.  Source and destination are the two
// record slots, so the source's counts stay intact for its resolve.  With a
// note (host-mapped), a source frame with heavy tiles is noted as
// frame_no << 32 | heavy tiles.
struct PlanArgs {
    const uint32_t *src_cnt;
    uint32_t *off, *cap, *cnt;
    uint32_t ntiles;
    uint64_t init_atoms, rec_cap;
    uint32_t *ovf_cnt;
    unsigned long long *note;
    uint32_t frame_no;
};
__device__ __forceinline__ void tile_plan(const uint32_t *src_cnt, uint32_t *off, uint32_t *cap, uint32_t *cnt,
                                          uint32_t ntiles, uint64_t init_atoms, uint64_t rec_cap,
                                          uint32_t *ovf_cnt, unsigned long long *note, uint32_t frame_no) {
    uint32_t nheavy = 0;
    __shared__ uint32_t wsum[32];
    __shared__ unsigned long long carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (uint32_t t0 = 0; t0 < ntiles; t0 += 1024) {
        const uint32_t t = t0 + threadIdx.x;
        uint32_t c = 0;
        bool heavy = false;
        if (t < ntiles) {
            const uint64_t seen = init_atoms ? (init_atoms * 5 / 4) / ntiles : src_cnt[t];
            heavy = !init_atoms && seen > kHeavyRec;
            const uint64_t want = seen + seen / 4 + 32;
            c = want < (1ull << 30) ? (uint32_t)want : (1u << 30);
        }
        uint32_t x = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if ((threadIdx.x & 31) >= (uint32_t)o) x += y;
        }
        if ((threadIdx.x & 31) == 31) wsum[threadIdx.x >> 5] = x;
        __syncthreads();
        unsigned long long run = carry + x - c;
        for (uint32_t w = 0; w < (threadIdx.x >> 5); ++w) run += wsum[w];
        if (t < ntiles) {
            const unsigned long long end = run + c < rec_cap ? run + c : rec_cap;
            const unsigned long long st = run < rec_cap ? run : rec_cap;
            off[t] = (uint32_t)st;
            cap[t] = (uint32_t)(end - st);
            cnt[t] = 0u;
        }
        nheavy += (uint32_t)__syncthreads_count(heavy);
        if (threadIdx.x == 1023) {
            unsigned long long tot = 0;
            for (int w = 0; w < 32; ++w) tot += wsum[w];
            carry += tot;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        *ovf_cnt = 0u;
        if (note && nheavy)
            *reinterpret_cast<volatile unsigned long long *>(note) = ((unsigned long long)frame_no << 32) | nheavy;
    }
}
__global__ void __launch_bounds__(1024) k_tile_plan(const uint32_t *src_cnt, uint32_t *off, uint32_t *cap,
                                                    uint32_t *cnt, uint32_t ntiles, uint64_t init_atoms,
                                                    uint64_t rec_cap, uint32_t *ovf_cnt, unsigned long long *note,
                                                    uint32_t frame_no) {
    tile_plan(src_cnt, off, cap, cnt, ntiles, init_atoms, rec_cap, ovf_cnt, note, frame_no);
}
struct PlanBatch {
    uint32_t n;
    PlanArgs job[kBatchFrames];
};
// Kernel parameters may take up to 32,764 bytes (sm_70 and later, CUDA 12.1 and later).
static_assert(sizeof(BinBatch) < 32000, "batched binning arguments exceed the kernel parameter space");
static_assert(sizeof(PlanBatch) < 32000, "batched plan arguments exceed the kernel parameter space");
__global__ void __launch_bounds__(1024) k_tile_plan_batch(const __grid_constant__ PlanBatch pb) {
    const PlanArgs &a = pb.job[blockIdx.x];
    tile_plan(a.src_cnt, a.off, a.cap, a.cnt, a.ntiles, a.init_atoms, a.rec_cap, a.ovf_cnt, a.note, a.frame_no);
}

__global__ void __launch_bounds__(256) k_frame_scatter(const uint4 *__restrict__ spl, const uint32_t *n_dev,
                                                        uint32_t tiles_x, uint32_t *tile_cur, uint4 *rec) {
    const uint64_t n = *n_dev;
    const int lane = threadIdx.x & 31;
    for (uint64_t base = blockIdx.x * (uint64_t)blockDim.x; base < n; base += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t i = base + threadIdx.x;
        uint4 s = i < n ? spl[i] : make_uint4(0, 0, 0, 0);
        uint32_t valid = i < n ? (s.y >> 16) & 15u : 0u;
        uint32_t t[4] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu};
        int nt = valid ? corner_tiles(s.x & 0xFFFFu, s.x >> 16, valid, tiles_x, t) : 0;
        // Warp-aggregated slot reservation per distinct tile.
        for (int k = 0; k < 4; ++k) {
            uint32_t tt = k < nt ? t[k] : 0xFFFFFFFFu;
            unsigned act = __ballot_sync(0xffffffffu, k < nt);
            if (!act) break;
            unsigned peers = __match_any_sync(0xffffffffu, tt);
            if (k < nt) {
                int leader = __ffs(peers) - 1;
                uint32_t slot = 0;
                if (lane == leader) slot = atomicAdd(&tile_cur[tt], (uint32_t)__popc(peers));
                slot = __shfl_sync(peers, slot, leader);
                slot += __popc(peers & ((1u << lane) - 1u));
                rec[slot] = s;
            }
        }
    }
}

// Exactly rounded (half away from zero) quotient num/den, both >= 0, den > 0,
// for quotients below 2^24: a float estimate corrected in exact integers.
__device__ __forceinline__ uint32_t round_div(unsigned long long num, unsigned long long den) {
    unsigned long long a = 2ull * num + den, b = 2ull * den;
    long long q = (long long)__fdividef((float)a, (float)b);
    long long r = (long long)a - q * (long long)b;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        if (r < 0) { --q; r += (long long)b; }
        else if (r >= (long long)b) { ++q; r -= (long long)b; }
    }
    return (uint32_t)q;
}

// Exactly rounded (half away from zero) quotients of several 32-bit
// numerators over one denominator (a pixel's four channel sums over its
// weight, packed path): one IEEE reciprocal, then per numerator a
// float estimate of num / den + 1/2 — within 1 of the exact quotient for
// den < 2^24 and quotients below 256 — and one correction on the exact
// 32-bit remainder (|remainder| < 1.5 den).
struct RoundDiv {
    float rcp;
    uint32_t den;
};
__device__ __forceinline__ RoundDiv round_div_by(uint32_t den) { return RoundDiv{__frcp_rn(__uint2float_rn(den)), den}; }
__device__ __forceinline__ uint32_t round_div(const RoundDiv &d, uint32_t num) {
    uint32_t q = __float2uint_rz(__fmaf_rn(__uint2float_rn(num), d.rcp, 0.5f));
    const int r2 = 2 * (int)(num - q * d.den);
    if (r2 < -(int)d.den) --q;
    else if (r2 >= (int)d.den) ++q;
    return q;
}

constexpr int kRecCache = 1920;   // records of a tile kept in shared memory (30 KB; 4 CTAs per SM fit)
constexpr uint32_t kPackMax = 258; // contributions per pixel for which packed 32-bit sums cannot overflow
// Without per-pixel counts (density 1) the packed sums are checked through
// the weight sum W: every channel sum is at most 255 W, so W <= kPackW keeps
// them below 2^32; W itself cannot wrap while the tile holds fewer than
// kPackRec records (each contributes at most 65025 to a pixel).
constexpr uint32_t kPackW = 0xFFFFFFFFu / 255u;
constexpr uint32_t kPackRec = 0xFFFFFFFFu / 65025u;

// Shared memory of the resolve kernel, two layouts over one buffer:
//  packed: W, N, R, G, B, A as 32-bit sums [1024] each (exact while a pixel
//          has at most kPackMax contributions), then the record cache;
//  exact:  W, R, G, B, A as 64-bit sums and N as 32-bit counts.
constexpr size_t kResolveSmem = 6 * 4 * 1024 + kRecCache * 16;

// Ordered "over" of one more blob's colour onto a pixel (morph.cpp:1357-1380)
// in FP64 with round-to-nearest operations; `first` seeds the state from the
// pixel's first blob colour c0.  Out of line and on local memory: only pixels
// covered by two or more blobs get here.
__device__ __noinline__ void over_blob(double *st, bool first, uint32_t c0, uint32_t cc) {
    if (first) {
        st[0] = (c0 & 255u) / 255.0; st[1] = ((c0 >> 8) & 255u) / 255.0;
        st[2] = ((c0 >> 16) & 255u) / 255.0; st[3] = (c0 >> 24) / 255.0;
    }
    const double sr = (cc & 255u) / 255.0, sg = ((cc >> 8) & 255u) / 255.0, sb = ((cc >> 16) & 255u) / 255.0,
                 sa = (cc >> 24) / 255.0;
    const double om = __dsub_rn(1.0, sa);
    st[0] = __dadd_rn(__dmul_rn(sa, sr), __dmul_rn(om, st[0]));
    st[1] = __dadd_rn(__dmul_rn(sa, sg), __dmul_rn(om, st[1]));
    st[2] = __dadd_rn(__dmul_rn(sa, sb), __dmul_rn(om, st[2]));
    st[3] = __dadd_rn(st[3], __dmul_rn(__dsub_rn(1.0, st[3]), sa));
}
// create_color's round(x * 255) of the composite (atomorph.h color rules).
__device__ __noinline__ uint32_t over_bytes(const double *st) {
    uint32_t o = 0;
    for (int k = 0; k < 4; ++k) o |= ((uint32_t)(int)round(__dmul_rn(st[k], 255.0)) & 255u) << (8 * k);
    return o;
}

// Render options the resolve applies (morph.cpp:1313-1399, 625-674).
struct ResolveOpts {
    uint32_t show_blobs;           // AM_TEXTURE, or AM_AVERAGE / AM_DISTINCT with rank_col
    uint32_t feather;              // TEXTURE blobs: outer layers faded
    uint32_t keep_bg;
    const uint32_t *rank_col;      // [C] colour of the rank-b blob of the pair's first key frame
    uint32_t tiles_y;
    BgArgs bg;                     // the background under the composite
    uint32_t only_rank;            // one blob alone (0xFFFFFFFF: the composite of all)
    uint8_t *aux;                  //   and its per-pixel coverage / feather layer code
    uint32_t helpers;              // heavy resolve: CTAs after the tiles' own, row-band helpers of heavy tiles
};

// Where a frame's binned records are: tile t's region starts at off[t] and
// holds min(cnt[t], cap[t]) records; records past a region's capacity went
// to the overflow list with the tile in bits 20-31 of .y.
struct TileRecs {
    const uint4 *rec;
    const uint32_t *off, *cnt, *cap;
    const uint4 *ovf;
    const uint32_t *ovf_cnt;
    uint32_t ovf_cap;
};
__device__ __forceinline__ uint32_t ovf_tile(const uint4 &s) { return s.y >> 20; }
__device__ __forceinline__ uint32_t ovf_total(const TileRecs &r) { return min(*r.ovf_cnt, r.ovf_cap); }

// Calls f(record) for every record of tile t from global memory (its region,
// then its overflow records), threads striding over them.
template <class F>
__device__ __forceinline__ void visit_tile(const TileRecs &r, uint32_t t, F &&f) {
    const uint32_t beg = r.off[t], n = min(r.cnt[t], r.cap[t]);
    for (uint32_t j = threadIdx.x; j < n; j += 256) f(r.rec[beg + j]);
    const uint32_t no = ovf_total(r);
    for (uint32_t j = threadIdx.x; j < no; j += 256) {
        const uint4 v = r.ovf[j];
        if (ovf_tile(v) == t) f(v);
    }
}

// Feather layers of the tile's pixels in the rank-`cur` blob (morph.cpp:
// 625-674): layer[li] = min(feather, d - 1), d the city-block distance to
// the nearest pixel outside the blob (iterated 4-neighbour erosion peels one
// layer per step).  Membership (any valid corner of a rank-`cur` record) is
// gathered from the tiles within R = ceil(feather / 32) rings into a bitmap
// of the (2R + 1) x 32 px square window; erosion runs on the bitmap.  Pixels
// outside the window count as outside the blob: every tile pixel is more
// than 32 R >= feather pixels from them, so no layer below feather changes.
// The rows of the tile (bit r: row ty0 + r) that a record's valid corners reach.
__device__ __forceinline__ uint32_t record_rows(const uint4 &s, uint32_t ty0) {
    const uint32_t r0 = (s.x >> 16) - ty0, valid = (s.y >> 16) & 15u;
    uint32_t m = 0;
    if (r0 < 32u && (valid & 3u)) m |= 1u << r0;
    if (r0 + 1u < 32u && (valid & 12u)) m |= 1u << (r0 + 1u);
    return m;
}
// Which tile and rows CTA `cta` of a heavy resolve grid takes when it is a
// helper (cta >= ntiles) or the own CTA of a heavy tile; false for a helper
// without a heavy tile.  Block-wide (every thread calls it); heavy tiles
// counted in tile order from cnt.  Out of line.
__device__ __noinline__ bool heavy_assign(const TileRecs &tr, uint32_t ntiles, const ResolveOpts &o, uint32_t cta,
                                          uint32_t *tile, uint32_t *rows) {
    __shared__ uint32_t wsum[8], s_kth;
    const uint32_t per = kBands - 1, served = min(o.helpers / per, kHeavyMaxTiles);
    const bool helper = cta >= ntiles;
    const uint32_t k = helper ? (cta - ntiles) / per : 0u, lim = helper ? 0u : cta;
    // thread t counts the heavy tiles of its chunk of the tile range
    const uint32_t chunk = (ntiles + 255u) / 256u, t0 = threadIdx.x * chunk, t1 = min(t0 + chunk, ntiles);
    uint32_t c = 0, before = 0;
    for (uint32_t t = t0; t < t1; ++t)
        if (tr.cnt[t] > kHeavyRec) {
            ++c;
            before += t < lim;
        }
    // exclusive prefix of c over the block, the total and the count before lim
    const uint32_t lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
    uint32_t x = c;
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, d);
        if (lane >= (uint32_t)d) x += y;
    }
    if (threadIdx.x == 0) s_kth = 0xFFFFFFFFu;
    if (lane == 31) wsum[wid] = x;
    __syncthreads();
    uint32_t pre = x - c, total = 0;
    for (uint32_t w = 0; w < 8; ++w) {
        if (w < wid) pre += wsum[w];
        total += wsum[w];
    }
    for (int d = 16; d; d >>= 1) before += __shfl_xor_sync(0xffffffffu, before, d);
    __syncthreads();
    if (lane == 0) wsum[wid] = before;
    __syncthreads();
    before = 0;
    for (uint32_t w = 0; w < 8; ++w) before += wsum[w];
    if (helper && k >= pre && k < pre + c) {
        uint32_t left = k - pre;
        for (uint32_t t = t0; t < t1; ++t)
            if (tr.cnt[t] > kHeavyRec && left-- == 0) {
                s_kth = t;
                break;
            }
    }
    __syncthreads();
    if (!helper) {
        *tile = cta;
        *rows = before < served ? band_rows(0) : 0xFFFFFFFFu;
        return true;
    }
    if (k >= min(total, served) || s_kth == 0xFFFFFFFFu) return false;
    *tile = s_kth;
    *rows = band_rows(1u + (cta - ntiles) % per);
    return true;
}

// The composite rank a record takes part in: its own, or none when one other
// blob is drawn alone.
__device__ __forceinline__ uint32_t rank_of(const ResolveOpts &o, const uint4 &s) {
    return (o.only_rank == 0xFFFFFFFFu || s.w == o.only_rank) ? s.w : 0xFFFFFFFFu;
}

__device__ __noinline__ void feather_layers(const TileRecs &tr, uint32_t tiles_x, uint32_t tiles_y, uint32_t tile,
                                            uint32_t cur, uint32_t F, uint32_t *bm, uint8_t *layer) {
    const int R = (int)((F + 31) / 32), WW = 2 * R + 1, WH = 32 * WW, nw = WW * WH;
    uint32_t *A = bm, *B = bm + nw;
    for (int i = threadIdx.x; i < nw; i += 256) A[i] = 0u;
    for (int i = threadIdx.x; i < 1024; i += 256) layer[i] = (uint8_t)F;
    __syncthreads();
    const int tx = (int)(tile % tiles_x), ty = (int)(tile / tiles_x);
    const int x0 = (tx - R) * 32, y0 = (ty - R) * 32;
    for (int dy = -R; dy <= R; ++dy)
        for (int dx = -R; dx <= R; ++dx) {
            const int ux = tx + dx, uy = ty + dy;
            if (ux < 0 || uy < 0 || ux >= (int)tiles_x || uy >= (int)tiles_y) continue;
            const uint32_t t2 = (uint32_t)uy * tiles_x + (uint32_t)ux;
            visit_tile(tr, t2, [&](const uint4 &s) {
                if (s.w != cur) return;
                const int px = (int)(s.x & 0xFFFFu), py = (int)(s.x >> 16);
                const uint32_t valid = (s.y >> 16) & 15u;
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    if (!(valid & (1u << k))) continue;
                    const int wx = px + (k & 1) - x0, wy = py + (k >> 1) - y0;
                    if (wx < 0 || wy < 0 || wx >= 32 * WW || wy >= WH) continue;
                    atomicOr(&A[wy * WW + (wx >> 5)], 1u << (wx & 31));
                }
            });
        }
    __syncthreads();
    for (uint32_t step = 0; step < F; ++step) {
        for (int i = threadIdx.x; i < nw; i += 256) {
            const int row = i / WW, w = i % WW;
            const uint32_t a = A[i];
            const uint32_t left = (a << 1) | (w > 0 ? A[i - 1] >> 31 : 0u);
            const uint32_t right = (a >> 1) | (w + 1 < WW ? A[i + 1] << 31 : 0u);
            const uint32_t up = row > 0 ? A[i - WW] : 0u, down = row + 1 < WH ? A[i + WW] : 0u;
            const uint32_t e = a & left & right & up & down;
            B[i] = e;
            uint32_t removed = a & ~e;
            if (removed && w == R && row >= 32 * R && row < 32 * R + 32)
                while (removed) {
                    const int bit = __ffs(removed) - 1;
                    removed &= removed - 1u;
                    layer[(row - 32 * R) * 32 + bit] = (uint8_t)step;
                }
        }
        __syncthreads();
        uint32_t *t = A; A = B; B = t;
    }
}

// Extra dynamic shared memory of the resolve for a feather: two window
// bitmaps and the tile's layers.
__host__ __device__ inline size_t feather_smem(uint32_t F) {
    if (!F) return 0;
    const size_t R = (F + 31) / 32, WW = 2 * R + 1;
    return 2 * WW * (32 * WW) * 4 + 1024;
}


// Stacked records of an uncached tile are reduced in the warp when at least
// kStackMin of a warp's 32 share a base pixel (the accumulation in
// frame_resolve).
constexpr uint32_t kStackMin = 4;

// The resolve of one 32 x 32 tile of a frame; Banded: only the tile's rows
// in `rows` (bit r: row r), the rest left to the tile's other CTAs.
template <bool Banded>
__device__ __forceinline__ void resolve_tile(const TileRecs &tr, uint32_t tiles_x, uint32_t width, uint32_t height,
                                             uint32_t density, uint8_t *out, const ResolveOpts &o, uint32_t tile,
                                             uint32_t rows) {
    extern __shared__ __align__(16) unsigned char sm[];
    constexpr bool banded = Banded;
    __shared__ uint32_t red[2][8];  // per-warp rank minima, alternating between blob ranks
    __shared__ int s_over;
    // packed mode: six 32-bit accumulators per pixel (a warp's 32-bit
    // atomics spread over 32 banks); exact mode: 64-bit sums and a count
    uint32_t *pW = reinterpret_cast<uint32_t *>(sm), *pN = pW + 1024, *pR = pW + 2048, *pG = pW + 3072,
             *pB = pW + 4096, *pA = pW + 5120;
    uint4 *cache = reinterpret_cast<uint4 *>(sm + 6 * 4 * 1024);
    unsigned long long *xW = reinterpret_cast<unsigned long long *>(sm), *xR = xW + 1024, *xG = xW + 2048,
                       *xB = xW + 3072, *xA = xW + 4096;
    uint32_t *xN = reinterpret_cast<uint32_t *>(xW + 5120);
    const uint32_t tx0 = (tile % tiles_x) * kTile, ty0 = (tile / tiles_x) * kTile;
    const uint4 *__restrict__ rec = tr.rec;
    const uint32_t beg = tr.off[tile], nmain = min(tr.cnt[tile], tr.cap[tile]);
    // overflow records of this tile (normally none)
    // s_nov: this tile's overflow records (read by every thread below);
    // s_app: the cache cursor they are appended at (a separate word, so the
    // append never overwrites the count while a warp may still read it)
    __shared__ uint32_t s_nov, s_app;
    const uint32_t novf = ovf_total(tr);
    if (novf) {
        if (threadIdx.x == 0) s_nov = 0;
        __syncthreads();
        uint32_t c = 0;
        for (uint32_t j = threadIdx.x; j < novf; j += 256) c += ovf_tile(tr.ovf[j]) == tile;
        if (c) atomicAdd(&s_nov, c);
        __syncthreads();
    }
    const uint32_t nrec = nmain + (novf ? s_nov : 0u);
    const bool feathered = o.feather > 0 && o.show_blobs == AM_TEXTURE;
    uint8_t *flayer = sm + kResolveSmem + (o.feather ? feather_smem(o.feather) - 1024 : 0);
    // thread t owns pixels t, t + 256, t + 512, t + 768 of the tile (rows
    // t/32 + 8q): a warp reads 32 consecutive accumulators and stores 32
    // consecutive output pixels
    int n[4];
    uint32_t c0[4];
    uint8_t lay[4] = {0, 0, 0, 0};  // one blob alone: 1 + feather layer of each pixel it reaches
    double st[4][4];  // FP64 "over" state (R, G, B, A) of pixels with 2+ blobs; local memory, rarely touched
    // density 1: a pixel's alpha needs no count, so the packed mode keeps
    // five sums per pixel and checks the weight sum instead of the count
    const bool counted = density > 1;
    for (int mode = (!counted && nrec >= kPackRec) ? 1 : 0; mode < 2; ++mode) {
        const bool packed = mode == 0;
        const bool cached = packed && nrec <= (uint32_t)kRecCache && !banded;
        uint32_t mn = 0xFFFFFFFFu;
        if (packed) {
            for (int i = threadIdx.x; i < 6 * 1024; i += 256) pW[i] = 0u;
            if (cached) {
                for (uint32_t j = threadIdx.x; j < nmain; j += 256) {
                    const uint4 v = rec[beg + j];
                    cache[j] = v;
                    mn = min(mn, rank_of(o, v));
                }
                if (novf) {
                    if (threadIdx.x == 0) s_app = nmain;
                    __syncthreads();
                    for (uint32_t j = threadIdx.x; j < novf; j += 256) {
                        const uint4 v = tr.ovf[j];
                        if (ovf_tile(v) != tile) continue;
                        cache[atomicAdd(&s_app, 1u)] = v;
                        mn = min(mn, rank_of(o, v));
                    }
                }
            }
        } else {
            for (int i = threadIdx.x; i < 5 * 1024; i += 256) xW[i] = 0ull;
            for (int i = threadIdx.x; i < 1024; i += 256) xN[i] = 0u;
        }
        if (threadIdx.x == 0) s_over = 0;
#pragma unroll
        for (int q = 0; q < 4; ++q) { n[q] = 0; c0[q] = 0; lay[q] = 0; }
        if (!cached)
            visit_tile(tr, tile, [&](const uint4 &v) {
                if (!banded || (record_rows(v, ty0) & rows)) mn = min(mn, rank_of(o, v));
            });
        for (int w = 16; w; w >>= 1) mn = min(mn, __shfl_xor_sync(0xffffffffu, mn, w));
        if ((threadIdx.x & 31) == 0) red[0][threadIdx.x >> 5] = mn;
        __syncthreads();
        uint32_t cur = red[0][0];
        for (int k = 1; k < 8; ++k) cur = min(cur, red[0][k]);
        bool over = false;
        uint32_t par = 0;
        // Two barriers per blob rank: after the accumulation (its sums and the
        // next rank's per-warp minima complete) and after the pixel pass (the
        // sums read and cleared).  The minima alternate between two arrays, so
        // a rank's writes never meet the previous rank's reads.
        while (cur != 0xFFFFFFFFu) {
            par ^= 1u;
            uint32_t nxt = 0xFFFFFFFFu;
            // cached: the tile's records in shared memory; else its region
            // and then the overflow list (other tiles' entries skipped)
            const uint32_t iter = cached ? nrec : nmain + novf;
            // one record's valid corners into the accumulators
            // (rows of the tile this call may add to: band, constant on the cached path)
            auto add_corners = [&](const uint4 &s, uint32_t band) {
                const uint32_t px = s.x & 0xFFFFu, py = s.x >> 16;
                const uint32_t xf = s.y & 255u, yf = (s.y >> 8) & 255u, valid = (s.y >> 16) & 15u;
                const uint32_t wx[2] = {255u - xf, xf}, wy[2] = {255u - yf, yf};
                const uint32_t cr = s.z & 255u, cg = (s.z >> 8) & 255u, cb = (s.z >> 16) & 255u, ca = s.z >> 24;
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    if (!(valid & (1u << k))) continue;
                    uint32_t cx = px + (k & 1) - tx0, cy = py + (k >> 1) - ty0;
                    if (cx >= (uint32_t)kTile || cy >= (uint32_t)kTile || !((band >> cy) & 1u)) continue;
                    uint32_t li = cy * kTile + cx;
                    uint32_t W = wx[k & 1] * wy[k >> 1];
                    if (packed) {
                        atomicAdd(&pW[li], W);
                        if (counted) atomicAdd(&pN[li], 1u);
                        atomicAdd(&pR[li], W * cr);
                        atomicAdd(&pG[li], W * cg);
                        atomicAdd(&pB[li], W * cb);
                        atomicAdd(&pA[li], W * ca);
                    } else {
                        atomicAdd(&xW[li], (unsigned long long)W);
                        atomicAdd(&xR[li], (unsigned long long)(W * cr));
                        atomicAdd(&xG[li], (unsigned long long)(W * cg));
                        atomicAdd(&xB[li], (unsigned long long)(W * cb));
                        atomicAdd(&xA[li], (unsigned long long)(W * ca));
                        atomicAdd(&xN[li], 1u);
                    }
                }
            };
            if (!cached) {
                // A tile too full for the record cache usually holds atoms
                // stacked on one pixel (a chain much wider than a key frame's
                // blob collapses onto that blob's pixels).  The records of a
                // warp that share the first used record's base pixel are summed
                // in the warp per corner, and each corner takes one atomic per
                // sum instead of one per record on the same address.  The trip
                // count is uniform per warp, so every lane reaches the votes.
                const uint32_t lane = threadIdx.x & 31u;
                for (uint32_t jb = threadIdx.x & ~31u; jb < iter; jb += 256) {
                    const uint32_t j = jb + lane;
                    uint4 s = make_uint4(0u, 0u, 0u, 0u);
                    bool use = false;
                    if (j < iter) {
                        bool mine = true;
                        if (j < nmain) {
                            s = rec[beg + j];
                        } else {
                            s = tr.ovf[j - nmain];
                            mine = ovf_tile(s) == tile;
                        }
                        if (banded && mine) mine = (record_rows(s, ty0) & rows) != 0;
                        if (mine) {
                            if (s.w == cur) use = true;
                            else if (s.w > cur) nxt = min(nxt, rank_of(o, s));
                        }
                    }
                    const unsigned um = __ballot_sync(0xffffffffu, use);
                    if (um) {
                        const int L = __ffs(um) - 1;
                        const uint32_t x0 = __shfl_sync(0xffffffffu, s.x, L);
                        const bool same = use && s.x == x0;
                        if ((uint32_t)__popc(__ballot_sync(0xffffffffu, same)) >= kStackMin) {
                            const uint32_t xf = s.y & 255u, yf = (s.y >> 8) & 255u, valid = (s.y >> 16) & 15u;
                            const uint32_t cr = s.z & 255u, cg = (s.z >> 8) & 255u, cb = (s.z >> 16) & 255u,
                                           ca = s.z >> 24;
#pragma unroll
                            for (int k = 0; k < 4; ++k) {
                                const uint32_t cx = (x0 & 0xFFFFu) + (k & 1) - tx0, cy = (x0 >> 16) + (k >> 1) - ty0;
                                if (cx >= (uint32_t)kTile || cy >= (uint32_t)kTile) continue;  // uniform
                                if (banded && !((rows >> cy) & 1u)) continue;                  // uniform
                                const bool a = same && ((valid >> k) & 1u);
                                // at most 32 records: 32 W and 32 W c stay below 2^32
                                const uint32_t W = a ? ((k & 1) ? xf : 255u - xf) * ((k >> 1) ? yf : 255u - yf) : 0u;
                                const uint32_t n = (uint32_t)__popc(__ballot_sync(0xffffffffu, a));
                                if (n == 0) continue;  // uniform
                                const uint32_t sW = __reduce_add_sync(0xffffffffu, W);
                                const uint32_t sR = __reduce_add_sync(0xffffffffu, W * cr);
                                const uint32_t sG = __reduce_add_sync(0xffffffffu, W * cg);
                                const uint32_t sB = __reduce_add_sync(0xffffffffu, W * cb);
                                const uint32_t sA = __reduce_add_sync(0xffffffffu, W * ca);
                                if ((int)lane == L) {
                                    const uint32_t li = cy * kTile + cx;
                                    if (packed) {
                                        atomicAdd(&pW[li], sW);
                                        if (counted) atomicAdd(&pN[li], n);
                                        atomicAdd(&pR[li], sR);
                                        atomicAdd(&pG[li], sG);
                                        atomicAdd(&pB[li], sB);
                                        atomicAdd(&pA[li], sA);
                                    } else {
                                        atomicAdd(&xW[li], (unsigned long long)sW);
                                        atomicAdd(&xR[li], (unsigned long long)sR);
                                        atomicAdd(&xG[li], (unsigned long long)sG);
                                        atomicAdd(&xB[li], (unsigned long long)sB);
                                        atomicAdd(&xA[li], (unsigned long long)sA);
                                        atomicAdd(&xN[li], n);
                                    }
                                }
                            }
                            if (same) use = false;
                        }
                    }
                    if (use) add_corners(s, banded ? rows : 0xFFFFFFFFu);
                }
            } else {
                for (uint32_t j = threadIdx.x; j < iter; j += 256) {
                    uint4 s;
                    if (cached) {
                        s = cache[j];
                    } else if (j < nmain) {
                        s = rec[beg + j];
                    } else {
                        s = tr.ovf[j - nmain];
                        if (ovf_tile(s) != tile) continue;
                    }
                    if (s.w != cur) {
                        if (s.w > cur) nxt = min(nxt, rank_of(o, s));
                        continue;
                    }
                    add_corners(s, 0xFFFFFFFFu);
                }
            }
            for (int w = 16; w; w >>= 1) nxt = min(nxt, __shfl_xor_sync(0xffffffffu, nxt, w));
            if ((threadIdx.x & 31) == 0) red[par][threadIdx.x >> 5] = nxt;
            __syncthreads();
            if (feathered)
                feather_layers(tr, tiles_x, o.tiles_y, tile, cur, o.feather,
                               reinterpret_cast<uint32_t *>(sm + kResolveSmem), flayer);
            uint32_t nx = red[par][0];
            for (int k = 1; k < 8; ++k) nx = min(nx, red[par][k]);
            // after the last blob rank the accumulators are not read again
            const bool more = !packed || nx != 0xFFFFFFFFu;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const uint32_t li = threadIdx.x + 256 * q;
                if (banded && !((rows >> (li >> 5)) & 1u)) continue;  // another CTA's band
                unsigned long long W, sr, sg, sb, sa;
                uint32_t cnt;
                if (packed) {
                    W = pW[li]; sr = pR[li]; sg = pG[li]; sb = pB[li]; sa = pA[li];
                    cnt = counted ? pN[li] : (W ? 1u : 0u);  // valid corners have positive weights
                    // more than kPackMax contributions (a weight sum above kPackW
                    // without counts) could have wrapped a 32-bit sum: this rank's
                    // pixels are drawn anyway and the tile starts over with 64-bit
                    // sums after the barrier below
                    if (counted ? cnt > kPackMax : W > kPackW) s_over = 1;
                    if (more) { pW[li] = 0u; pN[li] = 0u; pR[li] = 0u; pG[li] = 0u; pB[li] = 0u; pA[li] = 0u; }
                } else {
                    cnt = xN[li];
                    W = xW[li]; sr = xR[li]; sg = xG[li]; sb = xB[li]; sa = xA[li];
                    xW[li] = 0; xR[li] = 0; xG[li] = 0; xB[li] = 0; xA[li] = 0; xN[li] = 0;
                }
                if (!cnt) continue;
                uint32_t r, g, b, a;
                if (packed) {
                    const RoundDiv d = round_div_by((uint32_t)W);
                    r = round_div(d, (uint32_t)sr); g = round_div(d, (uint32_t)sg); b = round_div(d, (uint32_t)sb);
                    a = cnt >= density ? round_div(d, (uint32_t)sa)
                                       : round_div((unsigned long long)cnt * sa, (unsigned long long)density * W);
                } else {
                    r = round_div(sr, W); g = round_div(sg, W); b = round_div(sb, W);
                    a = cnt >= density ? round_div(sa, W)
                                       : round_div((unsigned long long)cnt * sa, (unsigned long long)density * W);
                }
                if (feathered && flayer[li] < o.feather)
                    a = (uint32_t)(int)round(__dmul_rn((double)a, __ddiv_rn((double)(flayer[li] + 1),
                                                                             (double)(o.feather + 1))));
                uint32_t cc = r | (g << 8) | (b << 16) | (a << 24);
                if (o.only_rank != 0xFFFFFFFFu) {
                    // one blob alone: every pixel it reaches, transparent ones too
                    n[q] = 1;
                    c0[q] = cc;
                    lay[q] = feathered ? (uint8_t)(flayer[li] + 1) : (uint8_t)1;
                    continue;
                }
                if (o.show_blobs != AM_TEXTURE) cc = o.rank_col[cur];
                if ((cc >> 24) == 0) continue;  // draw_atoms skips transparent blob pixels
                if (n[q] == 0) c0[q] = cc;
                else over_blob(st[q], n[q] == 1, c0[q], cc);
                n[q]++;
            }
            __syncthreads();
            if (packed && s_over) { over = true; break; }
            cur = nx;
        }
        if (!over) break;
        __syncthreads();
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const uint32_t li = threadIdx.x + 256 * q;
        const uint32_t gy = ty0 + (li >> 5), gx = tx0 + (li & 31u);
        if (gy >= height || gx >= width || (banded && !((rows >> (li >> 5)) & 1u))) continue;
        uint32_t px;
        if (o.keep_bg) px = over_background(n[q], c0[q], st[q], bg_colour(o.bg, gx, gy));
        else px = n[q] == 0 ? 0u : (n[q] == 1 ? c0[q] : over_bytes(st[q]));
        reinterpret_cast<uint32_t *>(out)[(size_t)gy * width + gx] = px;
        if (o.aux) o.aux[(size_t)gy * width + gx] = lay[q];
    }
}

// A row band of a heavy tile (out of line: the common path keeps its registers).
__device__ __noinline__ void resolve_band(const TileRecs &tr, uint32_t tiles_x, uint32_t width, uint32_t height,
                                          uint32_t density, uint8_t *out, const ResolveOpts &o, uint32_t tile,
                                          uint32_t rows) {
    resolve_tile<true>(tr, tiles_x, width, height, density, out, o, tile, rows);
}
// CTA `cta` of a frame's resolve grid: its own tile, or (Heavy) a row band
// of a heavy tile (helpers past the tiles' own CTAs).
template <bool Heavy>
__device__ __forceinline__ void frame_resolve(const TileRecs &tr, uint32_t tiles_x, uint32_t width, uint32_t height,
                                              uint32_t density, uint8_t *out, const ResolveOpts &o, uint32_t cta) {
    if (Heavy) {
        const uint32_t ntiles = tiles_x * o.tiles_y;
        if (cta >= ntiles || tr.cnt[cta] > kHeavyRec) {  // uniform
            uint32_t tile = cta, rows = 0xFFFFFFFFu;
            if (!heavy_assign(tr, ntiles, o, cta, &tile, &rows)) return;
            if (rows != 0xFFFFFFFFu) {
                resolve_band(tr, tiles_x, width, height, density, out, o, tile, rows);
                return;
            }
        }
    }
    resolve_tile<false>(tr, tiles_x, width, height, density, out, o, cta, 0xFFFFFFFFu);
}

__global__ void __launch_bounds__(256, 4) k_frame_resolve(const __grid_constant__ TileRecs tr, uint32_t tiles_x,
                                                        uint32_t width, uint32_t height, uint32_t density,
                                                        uint8_t *out, const __grid_constant__ ResolveOpts o) {
    frame_resolve<false>(tr, tiles_x, width, height, density, out, o, blockIdx.x);
}
// The resolve of a frame whose morph has had heavy tiles (o.helpers CTAs
// after the tiles' own).
__global__ void __launch_bounds__(256, 4) k_frame_resolve_heavy(const __grid_constant__ TileRecs tr,
                                                              uint32_t tiles_x, uint32_t width, uint32_t height,
                                                              uint32_t density, uint8_t *out,
                                                              const __grid_constant__ ResolveOpts o) {
    frame_resolve<true>(tr, tiles_x, width, height, density, out, o, blockIdx.x);
}
struct ResolveJob {
    TileRecs tr;
    ResolveOpts o;
    uint8_t *out;
    uint32_t tiles_x, width, height, density;
};
struct ResolveBatch {
    uint32_t n;
    uint32_t start[kBatchFrames + 1];
    ResolveJob job[kBatchFrames];
};
static_assert(sizeof(ResolveBatch) < 32000, "batched resolve arguments exceed the kernel parameter space");
__global__ void __launch_bounds__(256, 4) k_frame_resolve_batch(const __grid_constant__ ResolveBatch rb) {
    const uint32_t j = batch_job(rb.start, rb.n, blockIdx.x);
    const ResolveJob &a = rb.job[j];
    frame_resolve<false>(a.tr, a.tiles_x, a.width, a.height, a.density, a.out, a.o, blockIdx.x - rb.start[j]);
}
// The same when a job of the launch has had heavy tiles.
__global__ void __launch_bounds__(256, 4) k_frame_resolve_batch_heavy(const __grid_constant__ ResolveBatch rb) {
    const uint32_t j = batch_job(rb.start, rb.n, blockIdx.x);
    const ResolveJob &a = rb.job[j];
    frame_resolve<true>(a.tr, a.tiles_x, a.width, a.height, a.density, a.out, a.o, blockIdx.x - rb.start[j]);
}

__global__ void k_keyframe_copy(const uint32_t *__restrict__ display, const uint8_t *__restrict__ present,
                                uint32_t CW, uint32_t CH, uint32_t width, uint32_t height, uint32_t *out) {
    size_t n = (size_t)width * height;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        uint32_t x = (uint32_t)(i % width), y = (uint32_t)(i / width);
        uint32_t c = 0;
        if (x < CW && y < CH) {
            size_t j = (size_t)y * CW + x;
            if (present[j] && (display[j] >> 24)) c = display[j];
        }
        out[i] = c;
    }
}

}  // namespace

int launch_keyframe_copy(const uint32_t *display, const uint8_t *present, uint32_t CW, uint32_t CH, uint32_t width,
                         uint32_t height, uint8_t *out, cudaStream_t s) {
    size_t n = (size_t)width * height;
    if (!n) return AM_OK;
    unsigned grid = (unsigned)std::min<size_t>((n + 255) / 256, (size_t)kSMs * 16);
    AMG_LAUNCH(k_keyframe_copy, grid, 256, 0, s, display, present, CW, CH, width, height, (uint32_t *)out);
    AMG_CUDA(cudaGetLastError());
    return AM_OK;
}

// The cache slot holding pair f (prepared now when it is not there yet).
static int prep_pair(RenderWork *w, const RenderScene &sc, uint32_t f, cudaStream_t s, PairData **out) {
    int rc = rw_reserve(w, sc.N);
    if (rc) return rc;
    uint64_t per_pair = w->cap * kPairBytesPerAtom;
    size_t slots = (size_t)std::max<uint64_t>(1, std::min<uint64_t>(sc.K, kPairCacheBytes / std::max<uint64_t>(per_pair, 1)));
    if (w->pairs.size() != slots) {
        for (auto &d : w->pairs) pair_free(d);
        w->pairs.assign(slots, PairData());
    }
    PairData &d = w->pairs[f % slots];
    *out = &d;
    const bool noise = sc.motion_noise > 0.0;
    if (d.f == (int)f && d.motion == sc.motion && d.fading == sc.fading && d.width == sc.width &&
        d.height == sc.height && (d.noise || !noise))
        return AM_OK;
    if ((rc = pair_reserve(d, w->cap))) return rc;
    if (w->prof) w->prof->open(s);
    uint32_t tiles_x = (sc.width + kTile - 1) / kTile, tiles_y = (sc.height + kTile - 1) / kTile;
    unsigned grid = (unsigned)std::min<uint64_t>((sc.N + 255) / 256, (uint64_t)kSMs * 8);
    // Keys: the midpoint's tile, then its row-major place inside the tile;
    // inactive atoms carry the largest key and sort last.
    const uint64_t ntiles = (uint64_t)tiles_x * tiles_y;
    const uint32_t key_shift = ntiles < (1ull << 21) ? 10u : 0u;
    AMG_LAUNCH(k_pair_prep, grid, 256, 0, s, sc, f, w->perm_set ? w->perm : nullptr, w->pa, w->pb, w->col, w->ls,
               noise ? w->mn : nullptr, w->rank, w->keys, w->vals, tiles_x, (uint32_t)(ntiles << key_shift),
               key_shift);
    int bits = 1;
    while ((1ull << bits) < (ntiles << key_shift) + 1) ++bits;
    rc = radix_sort_pairs(w->keys, w->vals, w->tkeys, w->tvals, w->hist, sc.N, bits, s);
    if (rc) return rc;
    AMG_CUDA(cudaMemsetAsync(d.d_active, 0, 4, s));
    AMG_LAUNCH(k_pair_gather, grid, 256, 0, s, w->keys, w->vals, sc.N, w->pa, w->pb, w->col, w->ls,
               noise ? w->mn : nullptr, w->rank, d.pa, d.pb, d.col, d.ls, d.mn, d.rank, d.idx,
               (int)(sc.motion == AM_SPLINE), d.d_active);
    AMG_CUDA(cudaGetLastError());
    if (w->prof) w->prof->close(PROF_PAIR, s);
    d.f = (int)f;
    d.motion = sc.motion;
    d.fading = sc.fading;
    d.width = sc.width;
    d.height = sc.height;
    d.noise = noise;
    return AM_OK;
}

// Record slots large enough for a fused frame of n atoms over ntiles tiles:
// the planned tile regions (about 1.25 x the records of a frame plus slack;
// at most 4 records per atom) and an overflow list of 4 per atom, per slot.
static bool slots_fit(const RenderWork *w, uint64_t n, uint32_t ntiles) {
    const uint64_t need = n * 5 + (uint64_t)ntiles * 64 + 16, need_ovf = n * 4 + 16;
    return need <= w->slot_rec_cap && need_ovf <= w->slot_ovf_cap && ntiles <= w->slot_tiles_cap;
}
static int ensure_slots(RenderWork *w, uint64_t n, uint32_t ntiles, cudaStream_t s) {
    const uint64_t need = n * 5 + (uint64_t)ntiles * 64 + 16, need_ovf = n * 4 + 16;
    if (!slots_fit(w, n, ntiles)) {
        // frames in flight read the old buffers
        if (w->bs) AMG_CUDA(cudaStreamSynchronize(w->bs));
        AMG_CUDA(cudaStreamSynchronize(s));
        const uint64_t rc_new = std::max(w->slot_rec_cap, need + need / 4);
        const uint64_t oc_new = std::max(w->slot_ovf_cap, need_ovf);
        const uint32_t tc_new = std::max(w->slot_tiles_cap, ntiles);
        // capacities are recorded only once every buffer exists: after a
        // failed allocation the slots are empty and the next frame retries
        w->slot_rec_cap = w->slot_ovf_cap = 0;
        w->slot_tiles_cap = 0;
        cudaError_t e = cudaSuccess;
        for (auto &sl : w->slot) {
            slot_free(sl);
            if (e == cudaSuccess) e = cudaMalloc(&sl.rec, rc_new * sizeof(uint4));
            if (e == cudaSuccess) e = cudaMalloc(&sl.ovf, oc_new * sizeof(uint4));
            if (e == cudaSuccess) e = cudaMalloc(&sl.off, (size_t)tc_new * 4);
            if (e == cudaSuccess) e = cudaMalloc(&sl.cap, (size_t)tc_new * 4);
            if (e == cudaSuccess) e = cudaMalloc(&sl.cnt, (size_t)tc_new * 4);
            if (e == cudaSuccess) e = cudaMalloc(&sl.ovf_cnt, 4);
        }
        if (e != cudaSuccess) {
            for (auto &sl : w->slot) slot_free(sl);
            cudaGetLastError();
            set_error(std::string("render record slots: ") + cudaGetErrorString(e));
            return AM_ERR_NOMEM;
        }
        w->slot_rec_cap = rc_new;
        w->slot_ovf_cap = oc_new;
        w->slot_tiles_cap = tc_new;
    }
    return AM_OK;
}

// Row-band helper CTAs for the next frame's heavy tiles, sized from the note
// the morph's recent frames left: none while they have had no heavy tiles
// (or when the note could not be allocated), so such frames launch exactly
// their tiles.  The note is read without waiting; the frames in flight may
// not have written theirs yet.
constexpr uint32_t kHeavyMemory = 240;  // frames a heavy-tile note stays in force
static uint32_t heavy_helpers(RenderWork *w) {
    if (!w->note_tried) {
        w->note_tried = true;
        void *h = nullptr, *d = nullptr;
        if (cudaHostAlloc(&h, sizeof(unsigned long long), cudaHostAllocMapped) == cudaSuccess) {
            *static_cast<unsigned long long *>(h) = 0;
            if (cudaHostGetDevicePointer(&d, h, 0) == cudaSuccess) {
                w->note_host = static_cast<unsigned long long *>(h);
                w->note_dev = static_cast<unsigned long long *>(d);
            } else {
                cudaFreeHost(h);
            }
        }
        cudaGetLastError();  // a failed allocation only leaves the helpers off
    }
    if (!w->note_host) return 0;
    const unsigned long long v = *reinterpret_cast<volatile unsigned long long *>(w->note_host);
    const uint32_t seen = (uint32_t)(v >> 32), count = (uint32_t)v;
    if (count == 0 || w->frame_no - seen > kHeavyMemory) return 0;
    return std::min(count, kHeavyMaxTiles) * (kBands - 1);
}
// The heavy-tile field of a frame's resolve options; counts the frame (its
// plan notes heavy tiles under this number).
static void resolve_heavy(RenderWork *w, ResolveOpts &o) {
    o.helpers = heavy_helpers(w);
    ++w->frame_no;
    w->last_helpers = o.helpers;
}

void render_heavy_tiles(RenderWork *w, uint32_t *tiles, uint32_t *helpers) {
    // (no render work yet: the morph has used no GPU, so no frame either)
    render_quiesce(w);  // the plans that note heavy tiles run on the binning stream
    const unsigned long long v =
        (w && w->note_host) ? *reinterpret_cast<volatile unsigned long long *>(w->note_host) : 0ull;
    if (tiles) *tiles = (uint32_t)v;
    if (helpers) *helpers = w ? w->last_helpers : 0u;
}

// The resolve's render options for a frame of pair f at local time t.
static ResolveOpts resolve_opts(const RenderScene &sc, uint32_t f, double t, uint32_t tiles_y) {
    ResolveOpts o;
    std::memset(&o, 0, sizeof(o));
    o.show_blobs = sc.blob_col ? sc.show_blobs : AM_TEXTURE;
    o.rank_col = sc.blob_col ? sc.blob_col + (size_t)f * sc.C : nullptr;
    o.feather = std::min<uint32_t>(sc.feather, kMaxFeather);
    o.keep_bg = sc.keep_background && sc.present;
    o.tiles_y = tiles_y;
    o.bg = bg_args(sc, f, t);
    o.only_rank = sc.only_rank;
    o.aux = sc.aux;
    if (sc.only_rank != 0xFFFFFFFFu) {
        o.show_blobs = AM_TEXTURE;
        o.keep_bg = 0;
    }
    return o;
}

// Position / colour arithmetic of the frame at global time `time` (local
// time t in pair f): linear weights, the spline basis of
// GetInterpolatedSplinePoint (spline.cpp:45-57) and its fixed-point split,
// and the per-frame table of static spline coordinates.
int frame_args(RenderWork *w, const RenderScene &sc, double time, uint32_t f, double t, FrameArgs *out,
               cudaStream_t s) {
    FrameArgs &fa = *out;
    std::memset(&fa, 0, sizeof(fa));
    fa.w1 = 1.0 - t;
    fa.w2 = 1.0 - fa.w1;
    fa.w1q = (int32_t)llround(std::ldexp(fa.w1, 30));
    fa.lin_mode = fa.w1 == 1.0 ? 1u : (fa.w1 == 0.0 ? 2u : 0u);
    fa.str = (float)(1.0 - t);
    fa.noise_s = sc.motion_noise > 0.0 ? (float)(sc.motion_noise * 256.0 * std::sin(3.141592653589793 * t)) : 0.f;
    fa.seg_ok = 1;
    if (sc.motion == AM_SPLINE) {
        // GetInterpolatedSplinePoint(time) (spline.cpp:45-57) basis.
        int n = (int)sc.K;
        double delta_t = 1.0 / n;
        int p = (int)(time / delta_t);
        // cyclic indices: the reference's single wrap (spline.cpp:49-52) for n >= 2; with one
        // key frame it reads past its control points, here every index is that frame
        auto wrap = [n](int i) { return ((i % n) + n) % n; };
        double lt = (time - delta_t * (double)p) / delta_t;
        double t2 = lt * lt, t3 = t2 * lt;
        fa.b0 = 0.5 * (-t3 + 2.0 * t2 - lt);
        fa.b1 = 0.5 * (3.0 * t3 - 5.0 * t2 + 2.0);
        fa.b2 = 0.5 * (-3.0 * t3 + 4.0 * t2 + lt);
        fa.b3 = 0.5 * (t3 - t2);
        fa.seg[0] = wrap(p - 1); fa.seg[1] = wrap(p); fa.seg[2] = wrap(p + 1); fa.seg[3] = wrap(p + 2);
        fa.seg_ok = (p == (int)f) ? 1u : 0u;
        fa.bq0 = (int32_t)llround(std::ldexp(fa.b0, 30));
        fa.bq2 = (int32_t)llround(std::ldexp(fa.b2, 30));
        fa.bq3 = (int32_t)llround(std::ldexp(fa.b3, 30));
        fa.key_mode = (fa.b0 == 0.0 && fa.b1 == 1.0 && fa.b2 == 0.0 && fa.b3 == 0.0) ? 1u : 0u;
    }
    return AM_OK;
}

int render_positions(RenderWork *w, const RenderScene &sc, double time, uint64_t frame_key, int32_t *xy,
                     cudaStream_t s) {
    AMG_CUDA(cudaMemsetAsync(xy, 0xFF, (size_t)sc.N * 8, s));
    if (sc.K == 0 || sc.C == 0 || sc.N == 0) return AM_OK;
    const size_t f = (size_t)(time * sc.K);
    if (f >= sc.K) return AM_OK;
    const double dt = 1.0 / double(sc.K);
    const double t = std::max(0.0, (time - (double)(frame_key * dt)) / dt);
    // the pair cache is shared with the frames, which may run on the binning stream
    render_quiesce(w);
    w->bs_after_s = true;
    PairData *pd = nullptr;
    int rc = prep_pair(w, sc, (uint32_t)f, s, &pd);
    if (rc) return rc;
    FrameArgs fa;
    if ((rc = frame_args(w, sc, time, (uint32_t)f, t, &fa, s))) return rc;
    SplatIn in{pd->pa, pd->pb, pd->col, pd->ls, pd->rank, pd->idx, pd->mn};
    const unsigned grid = (unsigned)std::min<uint64_t>((sc.N + 255) / 256, (uint64_t)kSMs * 8);
    AMG_LAUNCH(k_atom_positions, grid, 256, 0, s, sc, fa, pd->d_active, in, xy);
    AMG_CUDA(cudaGetLastError());
    return AM_OK;
}

// The binning of a fused frame into slot[cur] on stream ps: a plan from the
// atom count when the slot has none for this frame's shape, then k_frame_bin;
// when piped, w->binned marks its end on bs.
static int fused_bin(RenderWork *w, const RenderScene &sc, const FrameArgs &fa, PairData *pd, uint32_t ntiles,
                     bool piped, cudaStream_t ps, cudaStream_t s) {
    int rc = ensure_slots(w, sc.N, ntiles, s);
    if (rc) return rc;
    RenderWork::Slot *A = &w->slot[w->cur];
    if (A->tiles != ntiles || A->atoms != sc.N) {
        // plan from the atom count; the slot's last resolve must be done
        if (piped) AMG_CUDA(cudaStreamWaitEvent(w->bs, A->resolved, 0));
        AMG_LAUNCH(k_tile_plan, 1, 1024, 0, ps, A->cnt, A->off, A->cap, A->cnt, ntiles, std::max<uint64_t>(sc.N, 1),
                   w->slot_rec_cap, A->ovf_cnt, (unsigned long long *)nullptr, 0u);
        A->tiles = ntiles;
        A->atoms = sc.N;
    }
    // atoms of the pair: at most N; the active count stays on the device
    const uint64_t n = sc.N;
    BinArgs b;
    b.sc = sc; b.fa = fa; b.n = pd->d_active;
    b.in = SplatIn{pd->pa, pd->pb, pd->col, pd->ls, pd->rank, pd->idx, pd->mn};
    b.rec = A->rec;
    b.off = A->off; b.cap = A->cap; b.cnt = A->cnt;
    b.ovf = A->ovf; b.ovf_cnt = A->ovf_cnt; b.ovf_cap = (uint32_t)std::min<uint64_t>(w->slot_ovf_cap, UINT32_MAX);
    const unsigned grid = (unsigned)((n + (uint64_t)kBinPer * kBinThreads - 1) / ((uint64_t)kBinPer * kBinThreads));
    // once per process (thread-safe static initialisation)
    static const cudaError_t battr = cudaFuncSetAttribute(k_frame_bin, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                          (int)occupancy_smem(1));
    AMG_CUDA(battr);
    if (w->prof) w->prof->open(ps);
    const size_t bsm = std::max(bin_smem(kBinPer, ntiles), sc.bin_ctas ? occupancy_smem(sc.bin_ctas) : (size_t)0);
    if (n) AMG_LAUNCH(k_frame_bin, grid, kBinThreads, bsm, ps, b);
    if (w->prof) w->prof->close(PROF_BIN, ps);
    if (piped) AMG_CUDA(cudaEventRecord(w->binned, w->bs));
    return AM_OK;
}

// Bins the frame `nx` ahead of its call, on bs into the slot its tile plan
// was just made for, when it is a pipelined fused frame of the same tile
// grid; remembered in w->ahead.
static int bin_ahead(RenderWork *w, const FrameAhead &nx, uint32_t ntiles_now, cudaStream_t s) {
    const RenderScene &sc = nx.sc;
    if (sc.K == 0 || sc.C == 0 || sc.N == 0 || !sc.pipeline || sc.only_rank != 0xFFFFFFFFu) return AM_OK;
    const size_t f = (size_t)(nx.time * sc.K);
    if (f >= sc.K) return AM_OK;
    const uint32_t tiles_x = (sc.width + kTile - 1) / kTile, tiles_y = (sc.height + kTile - 1) / kTile;
    const uint32_t ntiles = tiles_x * tiles_y;
    if (ntiles != ntiles_now || ntiles > kBinMaxTiles) return AM_OK;
    const double dt = 1.0 / double(sc.K);
    const double t = std::max(0.0, (nx.time - (double)(nx.frame_key * dt)) / dt);
    PairData *pd = nullptr;
    int rc = prep_pair(w, sc, (uint32_t)f, w->bs, &pd);
    if (rc) return rc;
    FrameArgs fa;
    if ((rc = frame_args(w, sc, nx.time, (uint32_t)f, t, &fa, w->bs))) return rc;
    fa.tiles_x = tiles_x;
    fa.ntiles = ntiles;
    if ((rc = fused_bin(w, sc, fa, pd, ntiles, true, w->bs, s))) return rc;
    w->ahead.valid = true;
    w->ahead.time = nx.time;
    w->ahead.key = nx.frame_key;
    w->ahead.sc = sc;
    return AM_OK;
}

int render_frame(RenderWork *w, const RenderScene &sc, double time, uint64_t frame_key, uint8_t *out,
                 cudaStream_t s, const FrameAhead *ahead) {
    const size_t bytes = (size_t)sc.width * sc.height * 4;
    if (sc.K == 0 || sc.C == 0 || sc.N == 0) {
        AMG_CUDA(cudaMemsetAsync(out, 0, bytes, s));
        return AM_OK;
    }
    size_t f = (size_t)(time * sc.K);
    if (f >= sc.K) {
        AMG_CUDA(cudaMemsetAsync(out, 0, bytes, s));
        return AM_OK;
    }
    double dt = 1.0 / double(sc.K);
    double t = std::max(0.0, (time - (double)(frame_key * dt)) / dt);
    uint32_t tiles_x = (sc.width + kTile - 1) / kTile, tiles_y = (sc.height + kTile - 1) / kTile;
    uint32_t ntiles = tiles_x * tiles_y;
    const bool fused = ntiles <= kBinMaxTiles;
    if (!w->bs) {
        AMG_CUDA(cudaStreamCreateWithFlags(&w->bs, cudaStreamNonBlocking));
        AMG_CUDA(cudaEventCreateWithFlags(&w->binned, cudaEventDisableTiming));
        AMG_CUDA(cudaEventCreateWithFlags(&w->mark, cudaEventDisableTiming));
        for (auto &sl : w->slot) AMG_CUDA(cudaEventCreateWithFlags(&sl.resolved, cudaEventDisableTiming));
    }
    // The pre-resolve work of a pipelined fused frame runs on bs; everything
    // else (a frame whose caller waits for it, the separate-kernel path) runs
    // on the render stream alone, with no cross-stream events.  Switching
    // between the two orders one stream after the other, once.
    const bool piped = fused && sc.pipeline;
    const cudaStream_t ps = piped ? w->bs : s;
    if (piped && w->bs_after_s) {
        AMG_CUDA(cudaEventRecord(w->mark, s));
        AMG_CUDA(cudaStreamWaitEvent(w->bs, w->mark, 0));
        w->bs_after_s = false;
    } else if (!piped && w->s_after_bs) {
        AMG_CUDA(cudaEventRecord(w->mark, w->bs));
        AMG_CUDA(cudaStreamWaitEvent(s, w->mark, 0));
        w->s_after_bs = false;
    }
    if (piped) w->s_after_bs = true;
    else w->bs_after_s = true;
    // a frame binned ahead of this call: its records, when it is this frame
    bool binned_ahead = false;
    if (w->ahead.valid) {
        binned_ahead = piped && time == w->ahead.time && frame_key == w->ahead.key && same_scene(sc, w->ahead.sc);
        if (binned_ahead) w->ahead.valid = false;
        else drop_ahead(w);
    }
    PairData *pd = nullptr;
    FrameArgs fa;
    if (!binned_ahead) {
        int rc = prep_pair(w, sc, (uint32_t)f, ps, &pd);
        if (rc) return rc;
        if ((rc = frame_args(w, sc, time, (uint32_t)f, t, &fa, ps))) return rc;
        fa.tiles_x = tiles_x;
        fa.ntiles = ntiles;
    }
    // atoms of the pair: at most N; the active count stays on the device
    uint64_t n = sc.N;
    TileRecs tr;
    RenderWork::Slot *A = nullptr, *B = nullptr;
    if (fused) {
        if (!binned_ahead) {
            int rc = fused_bin(w, sc, fa, pd, ntiles, piped, ps, s);
            if (rc) return rc;
        }
        if (piped) AMG_CUDA(cudaStreamWaitEvent(s, w->binned, 0));
        A = &w->slot[w->cur];
        B = &w->slot[w->cur ^ 1];
        tr = TileRecs{A->rec, A->off, A->cnt, A->cap, A->ovf, A->ovf_cnt,
                      (uint32_t)std::min<uint64_t>(w->slot_ovf_cap, UINT32_MAX)};
    } else {
        SplatIn in{pd->pa, pd->pb, pd->col, pd->ls, pd->rank, pd->idx, pd->mn};
        if (ntiles + 1 > w->ntiles_cap) {
            uint32_t **arrs[] = {&w->tile_cnt, &w->tile_off, &w->tile_cur};
            for (uint32_t **q : arrs) {
                if (*q) cudaFree(*q);
                *q = nullptr;
            }
            w->ntiles_cap = 0;  // recorded once all three exist
            for (uint32_t **q : arrs) AMG_ALLOC(q, (size_t)(ntiles + 1) * 4);
            w->ntiles_cap = ntiles + 1;
        }
        // records of the separate kernels: 4 per atom
        const uint64_t need = sc.N * 4 + 16;
        if (need > w->rec_cap) {
            if (w->rec) cudaFree(w->rec);
            w->rec = nullptr;
            w->rec_cap = 0;  // recorded once the buffer exists
            AMG_ALLOC(&w->rec, (need + need / 4) * sizeof(uint4));
            w->rec_cap = need + need / 4;
        }
        if (!w->zero) {
            AMG_ALLOC(&w->zero, 4);
            AMG_CUDA(cudaMemsetAsync(w->zero, 0, 4, s));
        }
        AMG_CUDA(cudaMemsetAsync(w->tile_cnt, 0, (ntiles + 1) * 4, s));
        if (n) {
            unsigned grid = (unsigned)std::min<uint64_t>((n + 255) / 256, (uint64_t)kSMs * 8);
            size_t smem = ntiles <= 8192 ? ntiles * 4 : 0;
            if (w->prof) w->prof->open(s);
            AMG_LAUNCH(k_frame_splat, grid, 256, smem, s, sc, fa, pd->d_active, in, w->spl, w->tile_cnt);
            if (w->prof) w->prof->close(PROF_SPLAT, s);
        }
        AMG_CUDA(cudaMemcpyAsync(w->tile_off, w->tile_cnt, (ntiles + 1) * 4, cudaMemcpyDeviceToDevice, s));
        {
            if (w->prof) w->prof->open(s);
            int rc = launch_scan_u32(w->tile_off, (size_t)ntiles + 1, nullptr, s);
            if (rc) return rc;
            if (w->prof) w->prof->close(PROF_SCAN, s);
        }
        AMG_CUDA(cudaMemcpyAsync(w->tile_cur, w->tile_off, (ntiles + 1) * 4, cudaMemcpyDeviceToDevice, s));
        if (n) {
            unsigned grid = (unsigned)std::min<uint64_t>((n + 255) / 256, (uint64_t)kSMs * 8);
            if (w->prof) w->prof->open(s);
            AMG_LAUNCH(k_frame_scatter, grid, 256, 0, s, w->spl, pd->d_active, tiles_x, w->tile_cur, w->rec);
            if (w->prof) w->prof->close(PROF_SCATTER, s);
        }
        tr = TileRecs{w->rec, w->tile_off, w->tile_cnt, w->tile_cnt, w->rec, w->zero, 0u};
    }
    ResolveOpts o = resolve_opts(sc, (uint32_t)f, t, tiles_y);
    resolve_heavy(w, o);
    if (w->prof) w->prof->open(s);
    {
        static const cudaError_t attr = cudaFuncSetAttribute(
            k_frame_resolve, cudaFuncAttributeMaxDynamicSharedMemorySize,
            (int)std::max(kResolveSmem + feather_smem(kMaxFeather), occupancy_smem(1)));
        static const cudaError_t hattr = cudaFuncSetAttribute(
            k_frame_resolve_heavy, cudaFuncAttributeMaxDynamicSharedMemorySize,
            (int)std::max(kResolveSmem + feather_smem(kMaxFeather), occupancy_smem(1)));
        AMG_CUDA(attr);
        AMG_CUDA(hattr);
    }
    const size_t rsm = std::max(kResolveSmem + feather_smem(o.feather),
                                sc.resolve_ctas ? occupancy_smem(sc.resolve_ctas) : (size_t)0);
    if (o.helpers)
        AMG_LAUNCH(k_frame_resolve_heavy, ntiles + o.helpers, 256, rsm, s, tr, tiles_x, sc.width, sc.height,
                   sc.density ? sc.density : 1u, out, o);
    else
        AMG_LAUNCH(k_frame_resolve, ntiles, 256, rsm, s, tr, tiles_x, sc.width, sc.height,
                   sc.density ? sc.density : 1u, out, o);
    if (w->prof) w->prof->close(PROF_RESOLVE, s);
    if (fused) {
        // the next frame's tile regions (the other slot) from this frame's
        // counts, once the other slot's last resolve is done
        if (piped) {
            AMG_CUDA(cudaEventRecord(A->resolved, s));
            AMG_CUDA(cudaStreamWaitEvent(w->bs, B->resolved, 0));
        }
        AMG_LAUNCH(k_tile_plan, 1, 1024, 0, ps, A->cnt, B->off, B->cap, B->cnt, ntiles, (uint64_t)0,
                   w->slot_rec_cap, B->ovf_cnt, w->note_dev, w->frame_no);
        B->tiles = ntiles;
        B->atoms = sc.N;
        w->cur ^= 1;
        // the frame expected next, binned beside this frame's resolve
        if (piped && ahead) {
            int rc = bin_ahead(w, *ahead, ntiles, s);
            if (rc) return rc;
        }
    }
    AMG_CUDA(cudaGetLastError());
    return AM_OK;
}


int render_frames_batch(const RenderJob *jobs, size_t n, cudaStream_t s, const BatchPipe *pipe) {
    static const cudaError_t battr = cudaFuncSetAttribute(
        k_frame_bin_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)occupancy_smem(1));
    static const cudaError_t rattr = cudaFuncSetAttribute(
        k_frame_resolve_batch, cudaFuncAttributeMaxDynamicSharedMemorySize,
        (int)std::max(kResolveSmem + feather_smem(kMaxFeather), occupancy_smem(1)));
    static const cudaError_t hattr = cudaFuncSetAttribute(
        k_frame_resolve_batch_heavy, cudaFuncAttributeMaxDynamicSharedMemorySize,
        (int)std::max(kResolveSmem + feather_smem(kMaxFeather), occupancy_smem(1)));
    AMG_CUDA(battr);
    AMG_CUDA(rattr);
    AMG_CUDA(hattr);
    // about 20 KB of launch arguments: on the heap
    std::vector<unsigned char> store(sizeof(BinBatch) + sizeof(ResolveBatch) + sizeof(PlanBatch) + 64);
    BinBatch &bb = *new (store.data()) BinBatch();
    ResolveBatch &rb = *new (store.data() + sizeof(BinBatch)) ResolveBatch();
    PlanBatch &pb = *new (store.data() + sizeof(BinBatch) + sizeof(ResolveBatch)) PlanBatch();
    struct Flip {
        RenderWork *w;
        RenderWork::Slot *B;
        uint32_t ntiles;
        uint64_t atoms;
    };
    std::vector<Flip> flips;
    uint32_t bin_ctas = 0, tiles = 0;
    bool heavy = false;  // a job of the launch gets row-band helpers
    size_t bsm = 0, rsm = 0;
    // Pipelined (pipe given): pair preparation, binning and the next tile
    // plans run on pipe->bs, the resolves on s; the plans wait for the
    // previous time's resolves, which last read the slots they fill, so a
    // time's binning runs beside the previous time's resolve.
    const cudaStream_t ps = pipe ? pipe->bs : s;
    uint32_t group = 0;
    auto flush = [&]() -> int {
        if (pb.n == 0) return AM_OK;
        bb.n = rb.n = pb.n;
        bb.start[bb.n] = bin_ctas;
        rb.start[rb.n] = tiles;
        if (pipe && group >= pipe->groups) {
            set_error("render_frames_batch: more launch groups than events");
            return AM_ERR_ARG;
        }
        if (bin_ctas) AMG_LAUNCH(k_frame_bin_batch, bin_ctas, kBinThreads, bsm, ps, bb);
        if (pipe) {
            AMG_CUDA(cudaEventRecord(pipe->binned[group], ps));
            AMG_CUDA(cudaStreamWaitEvent(s, pipe->binned[group], 0));
        }
        if (heavy) AMG_LAUNCH(k_frame_resolve_batch_heavy, tiles, 256, rsm, s, rb);
        else AMG_LAUNCH(k_frame_resolve_batch, tiles, 256, rsm, s, rb);
        if (pipe && pipe->prev_resolved && group == 0) AMG_CUDA(cudaStreamWaitEvent(ps, pipe->prev_resolved, 0));
        AMG_LAUNCH(k_tile_plan_batch, pb.n, 1024, 0, ps, pb);
        AMG_CUDA(cudaGetLastError());
        ++group;
        for (const Flip &fl : flips) {
            fl.B->tiles = fl.ntiles;
            fl.B->atoms = fl.atoms;
            fl.w->cur ^= 1;
        }
        flips.clear();
        pb.n = 0;
        bin_ctas = tiles = 0;
        heavy = false;
        bsm = rsm = 0;
        return AM_OK;
    };
    for (size_t i = 0; i < n; ++i) {
        const RenderJob &J = jobs[i];
        const RenderScene &sc = J.sc;
        RenderWork *w = J.w;
        drop_ahead(w);  // the caller has waited for the job's own streams
        const size_t bytes = (size_t)sc.width * sc.height * 4;
        const size_t f = (sc.K && sc.C && sc.N) ? (size_t)(J.time * sc.K) : 0;
        if (sc.K == 0 || sc.C == 0 || sc.N == 0 || f >= sc.K) {
            AMG_CUDA(cudaMemsetAsync(J.out, 0, bytes, s));
            continue;
        }
        const uint32_t tiles_x = (sc.width + kTile - 1) / kTile, tiles_y = (sc.height + kTile - 1) / kTile;
        const uint32_t ntiles = tiles_x * tiles_y;
        // a second frame of a job already in this launch would plan the slot
        // the first one bins into: launch what is gathered first
        bool again = false;
        for (const Flip &fl : flips) again |= fl.w == w;
        if (again || ntiles > kBinMaxTiles || sc.only_rank != 0xFFFFFFFFu) {
            int rc = flush();
            if (rc) return rc;
        }
        if (ntiles > kBinMaxTiles || sc.only_rank != 0xFFFFFFFFu) {
            RenderScene one = sc;
            one.pipeline = 0;  // everything on s
            int rc = render_frame(w, one, J.time, J.frame_key, J.out, s);
            if (rc) return rc;
            continue;
        }
        const double dt = 1.0 / double(sc.K);
        const double t = std::max(0.0, (J.time - (double)(J.frame_key * dt)) / dt);
        PairData *pd = nullptr;
        int rc = prep_pair(w, sc, (uint32_t)f, ps, &pd);
        if (rc) return rc;
        const uint32_t k = pb.n;
        BinArgs &b = bb.job[k];
        if ((rc = frame_args(w, sc, J.time, (uint32_t)f, t, &b.fa, ps))) return rc;
        b.fa.tiles_x = tiles_x;
        b.fa.ntiles = ntiles;
        // slots too small are reallocated: nothing in flight may still use them
        if (pipe && !slots_fit(w, sc.N, ntiles)) AMG_CUDA(cudaStreamSynchronize(pipe->bs));
        if ((rc = ensure_slots(w, sc.N, ntiles, s))) return rc;
        RenderWork::Slot *A = &w->slot[w->cur], *B = &w->slot[w->cur ^ 1];
        if (A->tiles != ntiles || A->atoms != sc.N) {
            AMG_LAUNCH(k_tile_plan, 1, 1024, 0, ps, A->cnt, A->off, A->cap, A->cnt, ntiles,
                       std::max<uint64_t>(sc.N, 1), w->slot_rec_cap, A->ovf_cnt, (unsigned long long *)nullptr, 0u);
            A->tiles = ntiles;
            A->atoms = sc.N;
        }
        b.sc = sc;
        b.n = pd->d_active;
        b.in = SplatIn{pd->pa, pd->pb, pd->col, pd->ls, pd->rank, pd->idx, pd->mn};
        b.rec = A->rec;
        b.off = A->off; b.cap = A->cap; b.cnt = A->cnt;
        b.ovf = A->ovf; b.ovf_cnt = A->ovf_cnt; b.ovf_cap = (uint32_t)std::min<uint64_t>(w->slot_ovf_cap, UINT32_MAX);
        bb.start[k] = bin_ctas;
        bin_ctas += (uint32_t)((sc.N + (uint64_t)kBinPer * kBinThreads - 1) / ((uint64_t)kBinPer * kBinThreads));
        bsm = std::max({bsm, bin_smem(kBinPer, ntiles), sc.bin_ctas ? occupancy_smem(sc.bin_ctas) : (size_t)0});
        ResolveJob &r = rb.job[k];
        r.tr = TileRecs{A->rec, A->off, A->cnt, A->cap, A->ovf, A->ovf_cnt, b.ovf_cap};
        r.o = resolve_opts(sc, (uint32_t)f, t, tiles_y);
        resolve_heavy(w, r.o);
        r.out = J.out;
        r.tiles_x = tiles_x;
        r.width = sc.width;
        r.height = sc.height;
        r.density = sc.density ? sc.density : 1u;
        rb.start[k] = tiles;
        tiles += ntiles + r.o.helpers;
        heavy |= r.o.helpers != 0;
        rsm = std::max({rsm, kResolveSmem + feather_smem(r.o.feather),
                        sc.resolve_ctas ? occupancy_smem(sc.resolve_ctas) : (size_t)0});
        pb.job[k] = PlanArgs{A->cnt, B->off, B->cap, B->cnt, ntiles, 0, w->slot_rec_cap, B->ovf_cnt, w->note_dev,
                             w->frame_no};
        flips.push_back(Flip{w, B, ntiles, sc.N});
        pb.n = k + 1;
        if (pb.n == kBatchFrames && (rc = flush())) return rc;
    }
    return flush();
}

}  // namespace amg
