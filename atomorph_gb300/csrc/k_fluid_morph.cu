// The morph's fluid path: particle management per key-frame pair
// (morph::step_fluid / update_particle, morph.cpp:680-1055) and the fluid
// frame render (morph::draw_fluid, morph.cpp:1057-1300), on the GPU fluid
// solver's particles (k_fluid.cu).
//
// Particle slot i belongs to column i of the chains (the reference walks the
// chains' columns and particles with one counter, morph.cpp:843-876).  Per
// frame of pair f (key frames y = f and y+1):
//   k_fm_classify  source / destination maps of the pair on the canvas
//                  (positions of the columns' points that carry fluid; the
//                  largest column wins a shared position, like the
//                  reference's map assignment), particles of another pair
//                  retire, active particles are counted per chain and mark
//                  the sources / destinations they hold.
//   host           active limit of each chain = round((1-t) S_y + t S_y+1)
//                  from its blobs' surfaces; chains create or delete the
//                  difference.
//   deletion       a uniformly random subset of the chain's active
//                  particles (the reference shuffles and pops): the active
//                  particles in a keyed Feistel permutation of the chain's
//                  columns, the first `to_delete` of them.
//   creation       free slots are taken from the end of the chain (the
//                  reference pops the last free particle).  Phase 1: the
//                  chain's free sources, in a keyed random order (the
//                  reference draws uniformly among the free sources each
//                  time), each with its column's destination.  Phase 2, when
//                  the sources run out: the chain's free destinations in
//                  ascending position (the reference's map order), each with
//                  its column's source; a particle whose source another
//                  particle already holds starts as a copy of it plus a
//                  uniform [0, 1) fuzz, otherwise at its attractor.
//   k_fm_update    update_particle: ideal colour from the two key frames
//                  with the alpha-0 rule and the fade of the atom path,
//                  attractor = the source column's trajectory point,
//                  colour blending, first-frame setup.
//   solver         FluidModel::step x fluidsteps (k_fluid.cu).
//   draw           colour correction, bilinear splat with continuous
//                  weights (quantised to 2^-32, so sums are exact integers
//                  and order-free) and per-pixel rounded means.
// The reference's RNG stream (std::default_random_engine) is replaced by
// counter-based hashes: which particles are created or deleted is
// statistically, not bitwise, the reference's.  Counts, pairings and the
// draw arithmetic are exact.
#include "common.cuh"
#include "fluid.cuh"
#include "kernels.h"
#include "render_math.cuh"

#include <cmath>
#include <cstring>
#include <vector>

namespace amg {

struct FluidMorph {
    uint32_t n = 0, cw = 0, ch = 0, out_w = 0, out_h = 0, C = 0;
    uint32_t *frame_key = nullptr;   // [n] pair the particle belongs to
    uint32_t *src_pos = nullptr, *dst_pos = nullptr;  // [n] canvas positions
    uint8_t *owner = nullptr;        // [n] first to occupy its source
    int32_t *src_map = nullptr, *dst_map = nullptr;   // [cw*ch] column or -1
    uint32_t *src_cnt = nullptr, *dst_cnt = nullptr;  // [cw*ch] particles holding the position
    unsigned long long *src_any = nullptr;            // [cw*ch] (hash << 32 | slot + 1) of a holder
    uint32_t *flags_a = nullptr, *flags_b = nullptr, *slot_by_rank = nullptr;  // [n]
    uint32_t *ckeys = nullptr, *cvals = nullptr, *tk = nullptr, *tv = nullptr, *hist = nullptr;  // phase 2 sort
    uint32_t *chain_cnt = nullptr;   // [C] active particles
    uint32_t *to_create = nullptr, *to_delete = nullptr, *phase1 = nullptr;  // [C]
    uint32_t *ncand = nullptr;       // phase 2 candidates
    unsigned long long *acc = nullptr;  // [5][out_w*out_h] W, R, G, B, A sums
    uint32_t *col[2] = {nullptr, nullptr};  // [out_w*out_h] fluid colours (feather / background passes)
    uint8_t *mem[2] = {nullptr, nullptr};   // [out_w*out_h] 1 where the fluid image has the pixel
    uint64_t frames = 0;             // frames stepped (random key)
    uint32_t *link = nullptr;        // [2][n] source and destination column of each particle's last update
    // Per column: the Perlin lag, slope and motion-noise pair at its point
    // of the pair's first key frame (a particle's values are its source
    // column's), built once per pair and chain state (k_fm_noise).
    float4 *ntab = nullptr;
    uint64_t ntab_n = 0;
    struct {
        bool valid = false;
        uint64_t version = 0, seed_key = 0;
        uint32_t y = 0, fading = 0;
        bool noise = false;
        const uint64_t *P = nullptr;
    } ntab_key;
};

// draw_fluid options: feather layers, keep_background (the background from
// the key frames, or a given image), scratch for the passes.
struct FluidDrawOpts {
    uint32_t feather = 0, keep_bg = 0;
    BgArgs bg{};
    const uint32_t *bg_img = nullptr;
    uint32_t *col[2] = {nullptr, nullptr};
    uint8_t *mem[2] = {nullptr, nullptr};
};

namespace {

__device__ __forceinline__ uint32_t pt_pos(uint64_t w, uint32_t cw) { return pt_y(w) * cw + pt_x(w); }
__device__ __forceinline__ bool pt_fluid(uint64_t w) { return pt_flags(w) & kHasFluid; }
__device__ __forceinline__ bool pt_pixel(uint64_t w) { return pt_flags(w) & kHasPixel; }
__device__ __forceinline__ float u01(uint64_t h) { return (float)(h >> 40) * (1.0f / 16777216.0f); }

struct FmArgs {
    const uint64_t *P;          // [K][N] published chains
    uint64_t N;
    uint32_t K, C, y, yn, f, cw, ch, width, height;
    const uint64_t *chain_off;  // [C+1]
    const uint32_t *chain_id;   // [N]
    const uint32_t *surf;       // [K][C] surface of the chain's blob in each key frame
    const uint32_t *display;    // [K][CH][CW]
    const int *perm;            // Perlin lag / slope permutations
    uint32_t motion, fading;
    uint32_t bbox[4];
    FrameArgs fa;               // position arithmetic of the frame
    float t;                    // local time in the pair
    float sp;                   // sparseness (grid units per pixel)
    uint64_t key;               // random key of this frame
    const float4 *ntab;         // [N] lag, slope, motion noise x, y per column (k_fm_noise)
    float *PF;                  // particle fields [kFlFields][N]
    uint8_t *flags;             // bit0 active, bit1 mature
    FluidMorph m;
};

#define PF_(k, i) a.PF[(size_t)(k) * a.N + (i)]

// Adds 1 to cnt[key] for the calling lane and returns its previous value as
// if the lanes had added one at a time; the converged lanes naming the same
// counter make one atomic (every particle of a one-chain morph names the
// same per-chain counter).
__device__ __forceinline__ uint32_t agg_add1(uint32_t *cnt, uint32_t key) {
    const unsigned act = __activemask();
    const unsigned peers = __match_any_sync(act, key);
    const int lane = threadIdx.x & 31, leader = __ffs(peers) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(&cnt[key], (uint32_t)__popc(peers));
    base = __shfl_sync(peers, base, leader);
    return base + __popc(peers & ((1u << lane) - 1u));
}

__global__ void k_fm_classify(FmArgs a) {
    for (uint64_t x = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; x < a.N; x += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t p1 = a.P[(uint64_t)a.y * a.N + x], p2 = a.P[(uint64_t)a.yn * a.N + x];
        if (pt_fluid(p1)) atomicMax(&a.m.src_map[pt_pos(p1, a.cw)], (int32_t)x);
        if (pt_fluid(p2)) atomicMax(&a.m.dst_map[pt_pos(p2, a.cw)], (int32_t)x);
        uint8_t fl = a.flags[x];
        if ((fl & 1u) && a.m.frame_key[x] == a.f) {
            agg_add1(a.m.chain_cnt, a.chain_id[x]);
            const uint32_t sp = a.m.src_pos[x], dp = a.m.dst_pos[x];
            if (sp < a.cw * a.ch) {
                atomicAdd(&a.m.src_cnt[sp], 1u);
                atomicMax(&a.m.src_any[sp], ((unsigned long long)mix32((uint32_t)x ^ (uint32_t)a.key) << 32) | (x + 1));
            }
            if (dp < a.cw * a.ch) atomicAdd(&a.m.dst_cnt[dp], 1u);
        } else if (fl & 1u) {
            a.flags[x] = fl & ~1u;
        }
    }
}

// Column of the chain's j-th position in a keyed random order.
__device__ __forceinline__ uint64_t perm_col(const FmArgs &a, uint32_t c, uint64_t off, uint32_t w, uint32_t j,
                                             uint64_t salt) {
    const uint64_t key = mix64(a.key ^ salt ^ ((uint64_t)c << 20));
    return off + permute_index(j, w, half_bits_for(w), key);
}

// flags_a[i] = 1 for the active particles of chains that delete, in each
// chain's random order.
__global__ void k_fm_del_flags(FmArgs a) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < a.N; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t c = a.chain_id[i];
        const uint64_t off = a.chain_off[c];
        const uint32_t w = (uint32_t)(a.chain_off[c + 1] - off);
        uint32_t v = 0;
        if (a.m.to_delete[c]) {
            const uint64_t x = perm_col(a, c, off, w, (uint32_t)(i - off), 0x64656cull);
            v = a.flags[x] & 1u;
        }
        a.m.flags_a[i] = v;
    }
}

// After the scan: the first to_delete active particles of each chain retire.
__global__ void k_fm_delete(FmArgs a, const uint32_t *__restrict__ raw) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < a.N; i += (uint64_t)gridDim.x * blockDim.x) {
        if (!raw[i]) continue;
        const uint32_t c = a.chain_id[i];
        const uint64_t off = a.chain_off[c];
        const uint32_t w = (uint32_t)(a.chain_off[c + 1] - off);
        if (a.m.flags_a[i] - a.m.flags_a[off] < a.m.to_delete[c]) {
            const uint64_t x = perm_col(a, c, off, w, (uint32_t)(i - off), 0x64656cull);
            a.flags[x] &= ~1u;
        }
    }
}

// Free slots from the end of each creating chain: flags_b[off + j] = 1 when
// column off + w - 1 - j is free.
__global__ void k_fm_free_flags(FmArgs a) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < a.N; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t c = a.chain_id[i];
        const uint64_t off = a.chain_off[c], end = a.chain_off[c + 1];
        const uint64_t x = end - 1 - (i - off);
        a.m.flags_b[i] = a.m.to_create[c] && !(a.flags[x] & 1u);
    }
}
__global__ void k_fm_free_rank(FmArgs a, const uint32_t *__restrict__ raw) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < a.N; i += (uint64_t)gridDim.x * blockDim.x) {
        if (!raw[i]) continue;
        const uint32_t c = a.chain_id[i];
        const uint64_t off = a.chain_off[c], end = a.chain_off[c + 1];
        const uint32_t r = a.m.flags_b[i] - a.m.flags_b[off];
        a.m.slot_by_rank[off + r] = (uint32_t)(end - 1 - (i - off));
    }
}

// A new particle in slot s: cleared dynamics, this pair, its positions.
__device__ __forceinline__ void fm_new(const FmArgs &a, uint32_t s, uint32_t sp, uint32_t dp) {
    PF_(PU, s) = 0.f;
    PF_(PV, s) = 0.f;
    PF_(PSTR, s) = 1.f;
    a.m.frame_key[s] = a.f;
    a.m.src_pos[s] = sp;
    a.m.dst_pos[s] = dp;
}

// Phase 1 candidates: the chain's free sources in random order.
__device__ __forceinline__ bool free_source(const FmArgs &a, uint64_t x, uint32_t *pos) {
    const uint64_t p1 = a.P[(uint64_t)a.y * a.N + x];
    if (!pt_fluid(p1)) return false;
    const uint32_t q = pt_pos(p1, a.cw);
    if (a.m.src_map[q] != (int32_t)x || a.m.src_cnt[q] != 0) return false;
    *pos = q;
    return true;
}
__global__ void k_fm_src_flags(FmArgs a) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < a.N; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t c = a.chain_id[i];
        uint32_t v = 0, q;
        if (a.m.to_create[c]) {
            const uint64_t off = a.chain_off[c];
            const uint32_t w = (uint32_t)(a.chain_off[c + 1] - off);
            v = free_source(a, perm_col(a, c, off, w, (uint32_t)(i - off), 0x737263ull), &q);
        }
        a.m.flags_a[i] = v;
    }
}
__global__ void k_fm_assign1(FmArgs a, const uint32_t *__restrict__ raw) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < a.N; i += (uint64_t)gridDim.x * blockDim.x) {
        if (!raw[i]) continue;
        const uint32_t c = a.chain_id[i];
        const uint64_t off = a.chain_off[c];
        const uint32_t r = a.m.flags_a[i] - a.m.flags_a[off];
        if (r >= a.m.to_create[c]) continue;
        const uint32_t w = (uint32_t)(a.chain_off[c + 1] - off);
        const uint64_t x = perm_col(a, c, off, w, (uint32_t)(i - off), 0x737263ull);
        uint32_t q = 0;
        free_source(a, x, &q);
        const uint64_t p2 = a.P[(uint64_t)a.yn * a.N + x];
        const uint32_t dq = pt_pos(p2, a.cw);
        const uint32_t s = a.m.slot_by_rank[off + r];
        fm_new(a, s, q, dq);
        a.m.owner[s] = 1;
        a.flags[s] = 1u;  // active, not mature: starts at its attractor (k_fm_update)
        atomicAdd(&a.m.dst_cnt[dq], 1u);
        atomicAdd(&a.m.src_cnt[q], 1u);
        agg_add1(a.m.phase1, c);
    }
}

// Phase 2 candidates: free destinations of chains whose sources ran out.
__global__ void k_fm_dst_cands(FmArgs a) {
    for (uint64_t x = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; x < a.N; x += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t c = a.chain_id[x];
        if (a.m.to_create[c] <= a.m.phase1[c]) continue;
        const uint64_t p2 = a.P[(uint64_t)a.yn * a.N + x];
        if (!pt_fluid(p2)) continue;
        const uint32_t q = pt_pos(p2, a.cw);
        if (a.m.dst_map[q] != (int32_t)x || a.m.dst_cnt[q] != 0) continue;
        const uint32_t k = agg_add1(a.m.ncand, 0u);
        a.m.ckeys[k] = q;
        a.m.cvals[k] = (uint32_t)x;
    }
}
__global__ void k_fm_rekey(FmArgs a, uint32_t n) {
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
        a.m.ckeys[k] = a.chain_id[a.m.cvals[k]];
}
// Sorted by chain, ascending position within a chain: the r-th entry of
// chain c takes the (phase1 + r)-th free slot of the chain.
__global__ void k_fm_assign2(FmArgs a, uint32_t n) {
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const uint32_t c = a.m.ckeys[k];
        uint32_t lo = 0, hi = k;  // first entry of chain c
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (a.m.ckeys[mid] < c) lo = mid + 1; else hi = mid;
        }
        const uint32_t r = k - lo, p1n = a.m.phase1[c];
        if (p1n + r >= a.m.to_create[c]) continue;
        const uint64_t x = a.m.cvals[k];
        const uint64_t off = a.chain_off[c];
        const uint64_t pt1 = a.P[(uint64_t)a.y * a.N + x], pt2 = a.P[(uint64_t)a.yn * a.N + x];
        const uint32_t sq = pt_pos(pt1, a.cw), dq = pt_pos(pt2, a.cw);
        const uint32_t s = a.m.slot_by_rank[off + p1n + r];
        fm_new(a, s, sq, dq);
        const unsigned long long par = a.m.src_any[sq];
        if (par) {
            // copy_from(parent) (fluidmodel.cpp:97-105), its maturity and
            // strength, plus a uniform [0, 1) fuzz (morph.cpp:982-1002)
            const uint32_t pi = (uint32_t)(par & 0xFFFFFFFFull) - 1;
            const int fields[] = {PX, PY, PGX, PGY, PFR, PR_, PG_, PB_, PA_, Pr, Pg, Pb, Pa, PSTR};
#pragma unroll
            for (int k2 = 0; k2 < 14; ++k2) PF_(fields[k2], s) = PF_(fields[k2], pi);
            const uint64_t h = mix64(a.key ^ ((uint64_t)s << 8) ^ 0x66757aull);
            PF_(PX, s) = fminf(PF_(PX, s) + u01(h), (float)a.width * a.sp - 10.f);
            PF_(PY, s) = fminf(PF_(PY, s) + u01(mix64(h)), (float)a.height * a.sp - 10.f);
            a.m.owner[s] = 0;
            a.flags[s] = 1u | (a.flags[pi] & 2u);
        } else {
            a.m.owner[s] = 1;
            a.flags[s] = 1u;
        }
    }
}

// The per-column table k_fm_update reads: Perlin lag and slope at the
// column's point of key frame y (morph.cpp:537-545; 0.5 without PERLIN
// fading) and the motion perturbation's noise pair there (the atom path's).
__global__ void k_fm_noise(FmArgs a, float4 *tab, int noise) {
    __shared__ int sp[2048];  // lag, slope, motion x, motion y permutations
    for (int i = threadIdx.x; i < 2048; i += blockDim.x) sp[i] = a.perm ? a.perm[i] : 0;
    __syncthreads();
    const float bw = (float)(a.bbox[2] - a.bbox[0] + 1), bh = (float)(a.bbox[3] - a.bbox[1] + 1);
    for (uint64_t x = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; x < a.N; x += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t pt1 = a.P[(uint64_t)a.y * a.N + x];
        float lag = 0.5f, slope = 0.5f, nx = 0.f, ny = 0.f;
        if (a.fading == AM_PERLIN) {
            float px = ((float)((int)pt_x(pt1) - (int)a.bbox[0]) * 256.f + (float)pt_xf(pt1)) / (bw * 256.f) * 8.f;
            float py = ((float)((int)pt_y(pt1) - (int)a.bbox[1]) * 256.f + (float)pt_yf(pt1)) / (bh * 256.f) * 8.f;
            lag = poctave(sp, px, py) * 0.5f + 0.5f;
            slope = poctave(sp + 512, px, py) * 0.5f + 0.5f;
        }
        if (noise) {
            const int bwi = (int)(a.bbox[2] - a.bbox[0] + 1), bhi = (int)(a.bbox[3] - a.bbox[1] + 1);
            const float u = noise_coord_rn((int)pt_x(pt1), (int)pt_xf(pt1), (int)a.bbox[0], bwi);
            const float v = noise_coord_rn((int)pt_y(pt1), (int)pt_yf(pt1), (int)a.bbox[1], bhi);
            nx = poctave_rn(sp + 1024, u, v);
            ny = poctave_rn(sp + 1536, u, v);
        }
        tab[x] = make_float4(lag, slope, nx, ny);
    }
}

// update_particle (morph.cpp:680-805) for every active particle.
__global__ void k_fm_update(FmArgs a) {
    for (uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; s < a.N; s += (uint64_t)gridDim.x * blockDim.x) {
        const uint8_t fl = a.flags[s];
        if (!(fl & 1u)) continue;
        const uint32_t c = a.chain_id[s];
        const uint64_t off = a.chain_off[c], end = a.chain_off[c + 1];
        const float S0 = (float)a.surf[(size_t)a.y * a.C + c], S1 = (float)a.surf[(size_t)a.yn * a.C + c];
        auto lookup = [&](const int32_t *map, uint32_t q) -> uint64_t {
            // the reference's map lookup inserts column 0 for a missing key
            const int32_t v = q < a.cw * a.ch ? map[q] : -1;
            return (v >= 0 && (uint64_t)v >= off && (uint64_t)v < end) ? (uint64_t)v : off;
        };
        uint64_t src_x = lookup(a.m.src_map, a.m.src_pos[s]);
        const uint64_t dst_x = lookup(a.m.dst_map, a.m.dst_pos[s]);
        if (S1 > S0) src_x = dst_x;
        const uint64_t pt1 = a.P[(uint64_t)a.y * a.N + src_x], pt2 = a.P[(uint64_t)a.yn * a.N + dst_x];
        const size_t fr = (size_t)a.cw * a.ch;
        const bool h1 = pt_pixel(pt1), h2 = pt_pixel(pt2);
        uint32_t c1 = a.display[(size_t)a.y * fr + pt_pos(pt1, a.cw)];
        uint32_t c2 = a.display[(size_t)a.yn * fr + pt_pos(pt2, a.cw)];
        if (h1 && !h2) {
            c2 = c1;
            if (S1 > 0.f) c2 &= 0x00FFFFFFu;
        } else if (h2 && !h1) {
            c1 = c2;
            if (S0 > 0.f) c1 &= 0x00FFFFFFu;
        }
        const float4 nt = a.ntab[src_x];  // lag, slope, motion noise at the source column's point
        const uint32_t col = fade_colour(a.fading, c1, c2, fade_params(nt.x, nt.y), 1.f - a.t);
        // attractor: the source column's trajectory point at this time
        uint32_t X = (uint32_t)pt_X(pt1), Y = (uint32_t)pt_Y(pt1);
        if (a.motion == AM_LINEAR) {
            int32_t v;
            X = lin_fast(a.fa, pt_X(pt1), pt_X(pt2), &v) ? (uint32_t)v : (uint32_t)lin_fixed(a.fa.w1, a.fa.w2, pt_X(pt1), pt_X(pt2));
            Y = lin_fast(a.fa, pt_Y(pt1), pt_Y(pt2), &v) ? (uint32_t)v : (uint32_t)lin_fixed(a.fa.w1, a.fa.w2, pt_Y(pt1), pt_Y(pt2));
        } else if (a.motion == AM_SPLINE) {
            const uint64_t q0 = a.P[(uint64_t)a.fa.seg[0] * a.N + src_x], q1 = a.P[(uint64_t)a.fa.seg[1] * a.N + src_x];
            const uint64_t q2 = a.P[(uint64_t)a.fa.seg[2] * a.N + src_x], q3 = a.P[(uint64_t)a.fa.seg[3] * a.N + src_x];
            if (!spl_fast(a.fa, pt_X(q0), pt_X(q1), pt_X(q2), pt_X(q3), &X))
                X = spl_fixed(a.fa.b0, a.fa.b1, a.fa.b2, a.fa.b3, pt_X(q0), pt_X(q1), pt_X(q2), pt_X(q3));
            if (!spl_fast(a.fa, pt_Y(q0), pt_Y(q1), pt_Y(q2), pt_Y(q3), &Y))
                Y = spl_fixed(a.fa.b0, a.fa.b1, a.fa.b2, a.fa.b3, pt_Y(q0), pt_Y(q1), pt_Y(q2), pt_Y(q3));
        }
        if (a.fa.noise_s != 0.f) {
            // the Perlin motion perturbation of the atom render, at the source point
            X = displace_rn(X, a.fa.noise_s, nt.z);
            Y = displace_rn(Y, a.fa.noise_s, nt.w);
        }
        const float ptx = (float)(X >> 8) + (float)(X & 255u) / 256.f;
        const float pty = (float)(Y >> 8) + (float)(Y & 255u) / 256.f;
        const float gx = fminf(fmaxf(ptx * a.sp + 10.f, 1.f), (float)a.width * a.sp + 10.f);
        const float gy = fminf(fmaxf(pty * a.sp + 10.f, 1.f), (float)a.height * a.sp + 10.f);
        PF_(PGX, s) = gx;
        PF_(PGY, s) = gy;
        a.m.link[s] = (uint32_t)src_x;
        a.m.link[a.N + s] = (uint32_t)dst_x;
        const float R = (float)(col & 255u) / 255.f, G = (float)((col >> 8) & 255u) / 255.f,
                    B = (float)((col >> 16) & 255u) / 255.f, A = (float)(col >> 24) / 255.f;
        PF_(PR_, s) = R; PF_(PG_, s) = G; PF_(PB_, s) = B; PF_(PA_, s) = A;
        const float t = a.t;
        float r = t * R + (1.f - t) * PF_(Pr, s), g = t * G + (1.f - t) * PF_(Pg, s);
        float b = t * B + (1.f - t) * PF_(Pb, s), al = t * A + (1.f - t) * PF_(Pa, s);
        if (!(fl & 2u)) {
            if (a.m.owner[s]) {
                PF_(PX, s) = gx;
                PF_(PY, s) = gy;
                r = R; g = G; b = B; al = A;
            }
            PF_(PSTR, s) = S0 == 0.f ? 0.1f : 1.f;
            PF_(PFR, s) = 1.f;
        }
        PF_(Pr, s) = r; PF_(Pg, s) = g; PF_(Pb, s) = b; PF_(Pa, s) = al;
    }
}

// draw_fluid's splat (morph.cpp:1081-1160) of one particle.
struct DrawArgs {
    float *PF;
    uint8_t *flags;
    uint64_t n;
    uint32_t width, height;
    uint32_t bbox[4];
    float sp, t;
    unsigned long long *acc;  // [5][width*height]
};
#define DF_(k, i) a.PF[(size_t)(k) * a.n + (i)]

__device__ __forceinline__ uint32_t create_byte(float v) {
    return (uint32_t)min(max((int)rintf(v * 255.f), 0), 255);
}

__global__ void k_fm_splat(DrawArgs a) {
    const size_t npx = (size_t)a.width * a.height;
    for (uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; s < a.n; s += (uint64_t)gridDim.x * blockDim.x) {
        const uint8_t fl = a.flags[s];
        if (!(fl & 1u)) continue;
        // colour correction (morph.cpp:1085-1096)
        const float st = DF_(PSTR, s), d = a.t - (1.f - st);
        const float w = (1.f / (100.f * d * d + 1.f)) * st * st;
        const float r = w * DF_(PR_, s) + (1.f - w) * DF_(Pr, s), g = w * DF_(PG_, s) + (1.f - w) * DF_(Pg, s);
        const float b = w * DF_(PB_, s) + (1.f - w) * DF_(Pb, s), al = w * DF_(PA_, s) + (1.f - w) * DF_(Pa, s);
        DF_(Pr, s) = r; DF_(Pg, s) = g; DF_(Pb, s) = b; DF_(Pa, s) = al;
        a.flags[s] = fl | 2u;  // mature from its first frame on
        const float x = DF_(PX, s), y = DF_(PY, s);
        float px, py;
        if (x <= 10.f) px = 0.f;
        else if (x >= (float)a.width * a.sp + 10.f) px = (float)(a.width - 1);
        else px = (x - 10.f) / a.sp;
        if (y <= 10.f) py = 0.f;
        else if (y >= (float)a.height * a.sp + 10.f) py = (float)(a.height - 1);
        else py = (y - 10.f) / a.sp;
        const uint32_t ix = (uint32_t)min((int)px, (int)a.width - 1), iy = (uint32_t)min((int)py, (int)a.height - 1);
        const float fx = floorf(px), fy = floorf(py), xf = px - fx, yf = py - fy;
        if (fx >= (float)a.width || fy >= (float)a.height) {
            if (fx > (float)a.bbox[2] || fx < (float)a.bbox[0] || fy > (float)a.bbox[3] || fy < (float)a.bbox[1]) continue;
        }
        const float wt[4] = {(1.f - xf) * (1.f - yf), xf * (1.f - yf), (1.f - xf) * yf, xf * yf};
        bool ok[4];
        ok[0] = wt[0] > 0.f;
        ok[1] = (ix < a.bbox[2] || ix + 1 < a.width) && wt[1] > 0.f;
        ok[2] = (iy < a.bbox[3] || iy + 1 < a.height) && wt[2] > 0.f;
        ok[3] = wt[3] > 0.f && ((iy < a.bbox[3] && ix < a.bbox[2]) || (iy + 1 < a.height && ix + 1 < a.width));
        const uint32_t cr = create_byte(r), cg = create_byte(g), cb = create_byte(b), ca = create_byte(al);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            if (!ok[k]) continue;
            const uint32_t cx = ix + (k & 1), cy = iy + (k >> 1);
            if (cx >= a.width || cy >= a.height) continue;  // outside the output (see the atom path)
            const size_t q = (size_t)cy * a.width + cx;
            const unsigned long long W = __float2ull_rn(wt[k] * 4294967296.f);  // weight in units of 2^-32
            if (!W) continue;
            atomicAdd(&a.acc[q], W);
            atomicAdd(&a.acc[npx + q], W * cr);
            atomicAdd(&a.acc[2 * npx + q], W * cg);
            atomicAdd(&a.acc[3 * npx + q], W * cb);
            atomicAdd(&a.acc[4 * npx + q], W * ca);
        }
    }
}

__device__ __forceinline__ uint32_t rdiv64(unsigned long long num, unsigned long long den) {
    return (uint32_t)((2ull * num + den) / (2ull * den));
}

__global__ void k_fm_resolve(const unsigned long long *__restrict__ acc, size_t npx, uint32_t *out) {
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < npx; q += (size_t)gridDim.x * blockDim.x) {
        const unsigned long long W = acc[q];
        uint32_t o = 0;
        if (W) {
            o = rdiv64(acc[npx + q], W) | (rdiv64(acc[2 * npx + q], W) << 8) | (rdiv64(acc[3 * npx + q], W) << 16) |
                (rdiv64(acc[4 * npx + q], W) << 24);
        }
        out[q] = o;
    }
}

// draw_fluid's per-pixel colour (morph.cpp:1160-1201) with membership; with
// keep_background the alpha fades by afade = 1 - t^24 and truncates, as
// create_pixel converts the faded double.
__global__ void k_fm_means(const unsigned long long *__restrict__ acc, size_t npx, double afade, uint32_t *col,
                           uint8_t *mem) {
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < npx; q += (size_t)gridDim.x * blockDim.x) {
        const unsigned long long W = acc[q];
        uint32_t o = 0;
        if (W) {
            uint32_t a = rdiv64(acc[4 * npx + q], W);
            if (afade != 1.0) a = (uint32_t)(int)__dmul_rn((double)a, afade);
            o = rdiv64(acc[npx + q], W) | (rdiv64(acc[2 * npx + q], W) << 8) | (rdiv64(acc[3 * npx + q], W) << 16) |
                (a << 24);
        }
        col[q] = o;
        mem[q] = W ? 1 : 0;
    }
}

// One outward feather layer of the fluid image (morph.cpp:1204-1251): a
// pixel outside the image with members among its 4 neighbours joins it with
// their mean colour (summed in the reference's position order: up, left,
// right, down), alpha scaled by `alpha`, create_color rounding.
__global__ void k_fm_dilate(const uint32_t *__restrict__ col, const uint8_t *__restrict__ mem, uint32_t width,
                            uint32_t height, double alpha, uint32_t *col2, uint8_t *mem2) {
    const size_t npx = (size_t)width * height;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < npx; q += (size_t)gridDim.x * blockDim.x) {
        if (mem[q]) {
            col2[q] = col[q];
            mem2[q] = 1;
            continue;
        }
        const uint32_t x = (uint32_t)(q % width), y = (uint32_t)(q / width);
        size_t nb[4];
        int w = 0;
        if (y > 0 && mem[q - width]) nb[w++] = q - width;
        if (x > 0 && mem[q - 1]) nb[w++] = q - 1;
        if (x + 1 < width && mem[q + 1]) nb[w++] = q + 1;
        if (y + 1 < height && mem[q + width]) nb[w++] = q + width;
        if (!w) {
            col2[q] = 0u;
            mem2[q] = 0;
            continue;
        }
        double v[4] = {0.0, 0.0, 0.0, 0.0};
        for (int k = 0; k < w; ++k) {
            const uint32_t c = col[nb[k]];
            for (int ch = 0; ch < 4; ++ch)
                v[ch] = __dadd_rn(v[ch], __ddiv_rn(__ddiv_rn((double)((c >> (8 * ch)) & 255u), 255.0), (double)w));
        }
        v[3] = __dmul_rn(v[3], alpha);
        uint32_t o = 0;
        for (int ch = 0; ch < 4; ++ch) o |= ((uint32_t)(int)round(__dmul_rn(v[ch], 255.0)) & 255u) << (8 * ch);
        col2[q] = o;
        mem2[q] = 1;
    }
}

// The fluid image into the frame (morph.cpp:1268-1299): over the background
// with keep_background (bg_img, or the key frames' cross-fade), else as is
// with transparent black elsewhere.
__global__ void k_fm_final(const uint32_t *__restrict__ col, const uint8_t *__restrict__ mem, uint32_t width,
                           uint32_t height, uint32_t keep_bg, BgArgs bg, const uint32_t *__restrict__ bg_img,
                           uint32_t *out) {
    const size_t npx = (size_t)width * height;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < npx; q += (size_t)gridDim.x * blockDim.x) {
        if (!keep_bg) {
            out[q] = mem[q] ? col[q] : 0u;
            continue;
        }
        const uint32_t b = bg_img ? bg_img[q] : bg_colour(bg, (uint32_t)(q % width), (uint32_t)(q / width));
        out[q] = over_background(mem[q] ? 1 : 0, col[q], nullptr, b);
    }
}

int grow(void **p, size_t bytes, size_t *cap) {
    if (bytes <= *cap) return AM_OK;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    AMG_ALLOC(p, bytes);
    *cap = bytes;
    return AM_OK;
}

}  // namespace

FluidMorph *fluid_morph_create() { return new FluidMorph(); }

void fluid_morph_destroy(FluidMorph *m) {
    if (!m) return;
    void *ps[] = {m->frame_key, m->src_pos, m->dst_pos, m->owner, m->src_map, m->dst_map, m->src_cnt, m->dst_cnt,
                  m->src_any, m->flags_a, m->flags_b, m->slot_by_rank, m->ckeys, m->cvals, m->tk, m->tv, m->hist,
                  m->chain_cnt, m->to_create, m->to_delete, m->phase1, m->ncand, m->acc, m->col[0], m->col[1],
                  m->mem[0], m->mem[1], m->link, m->ntab};
    for (void *p : ps)
        if (p) cudaFree(p);
    delete m;
}

// The source and destination column each particle's last update read
// (update_particle's src_x after the growing-area rule and dst_x,
// morph.cpp:687-695), n particles: out[0..n) sources, out[n..2n) destinations.
int fluid_morph_links(FluidMorph *m, uint32_t *out, size_t n, cudaStream_t s) {
    if (!m || !m->link || n != m->n) return AM_ERR_STATE;
    AMG_CUDA(cudaMemcpyAsync(out, m->link, 2 * n * 4, cudaMemcpyDeviceToHost, s));
    AMG_CUDA(cudaStreamSynchronize(s));
    return AM_OK;
}

int fluid_draw(FluidDev *fl, unsigned long long *acc, uint32_t width, uint32_t height, double sparseness,
               const uint32_t *bbox, double t, uint8_t *out, cudaStream_t s, const FluidDrawOpts &o) {
    const size_t npx = (size_t)width * height;
    if (!npx) return AM_OK;
    AMG_CUDA(cudaMemsetAsync(acc, 0, 5 * npx * sizeof(unsigned long long), s));
    DrawArgs a;
    a.PF = fl->P; a.flags = fl->flags; a.n = fl->n; a.width = width; a.height = height;
    for (int k = 0; k < 4; ++k) a.bbox[k] = bbox[k];
    a.sp = (float)sparseness; a.t = (float)t; a.acc = acc;
    if (fl->n) {
        unsigned g = (unsigned)std::min<uint64_t>((fl->n + 255) / 256, (uint64_t)kSMs * 8);
        AMG_LAUNCH(k_fm_splat, g, 256, 0, s, a);
    }
    unsigned g2 = (unsigned)std::min<size_t>((npx + 255) / 256, (size_t)kSMs * 8);
    if (!o.feather && !o.keep_bg) {
        AMG_LAUNCH(k_fm_resolve, g2, 256, 0, s, acc, npx, (uint32_t *)out);
    } else {
        const double afade = o.keep_bg ? 1.0 - std::pow(t, 24.0) : 1.0;
        AMG_LAUNCH(k_fm_means, g2, 256, 0, s, acc, npx, afade, o.col[0], o.mem[0]);
        int cur = 0;
        for (uint32_t layer = 0; layer < o.feather; ++layer) {
            const double alpha = 1.0 - (double(layer + 1) / double(o.feather + 1));
            AMG_LAUNCH(k_fm_dilate, g2, 256, 0, s, o.col[cur], o.mem[cur], width, height, alpha, o.col[cur ^ 1],
                       o.mem[cur ^ 1]);
            cur ^= 1;
        }
        AMG_LAUNCH(k_fm_final, g2, 256, 0, s, o.col[cur], o.mem[cur], width, height, o.keep_bg, o.bg, o.bg_img,
                   (uint32_t *)out);
    }
    AMG_CUDA(cudaGetLastError());
    return AM_OK;
}

int fluid_render_only(FluidDev *fl, uint32_t width, uint32_t height, double sparseness, const uint32_t *bbox,
                      double t, uint32_t feather, const uint32_t *bg_img, uint8_t *out, cudaStream_t s) {
    const size_t npx = std::max<size_t>((size_t)width * height, 1);
    unsigned long long *acc = nullptr;
    uint32_t *col = nullptr;
    uint8_t *mem = nullptr;
    if (cudaMalloc(&acc, 5 * npx * sizeof(unsigned long long)) != cudaSuccess ||
        cudaMalloc(&col, 2 * npx * 4) != cudaSuccess || cudaMalloc(&mem, 2 * npx) != cudaSuccess) {
        cudaGetLastError();  // the failed allocation's pending error
        cudaFree(acc); cudaFree(col); cudaFree(mem);
        set_error("fluid draw: out of device memory");
        return AM_ERR_NOMEM;
    }
    FluidDrawOpts o;
    o.feather = feather;
    o.keep_bg = bg_img ? 1u : 0u;
    o.bg_img = bg_img;
    o.col[0] = col; o.col[1] = col + npx; o.mem[0] = mem; o.mem[1] = mem + npx;
    int rc = fluid_draw(fl, acc, width, height, sparseness, bbox, t, out, s, o);
    cudaError_t e = cudaStreamSynchronize(s);
    cudaFree(acc); cudaFree(col); cudaFree(mem);
    if (rc) return rc;
    AMG_CUDA(e);
    return AM_OK;
}

void fluid_init_particles(FluidDev *fl, FluidMorph *m, uint32_t width, uint32_t height, double sparseness,
                          cudaStream_t s) {
    // morph.cpp:244-258: cleared particles parked at the middle of the grid,
    // green so a stray one would show.
    const uint32_t n = fl->n;
    std::vector<float> P((size_t)kFlFields * n, 0.f);
    const float x = (float)(width * sparseness / 2.0 - 10.0), y = (float)(height * sparseness / 2.0 - 10.0);
    for (uint32_t i = 0; i < n; ++i) {
        P[(size_t)PX * n + i] = x; P[(size_t)PY * n + i] = y;
        P[(size_t)PGX * n + i] = x; P[(size_t)PGY * n + i] = y;
        P[(size_t)PFR * n + i] = 1.f; P[(size_t)PSTR * n + i] = 1.f;
        P[(size_t)PG_ * n + i] = 1.f; P[(size_t)PA_ * n + i] = 1.f;
        P[(size_t)Pg * n + i] = 1.f; P[(size_t)Pa * n + i] = 1.f;
    }
    cudaMemcpyAsync(fl->P, P.data(), P.size() * 4, cudaMemcpyHostToDevice, s);
    cudaMemsetAsync(fl->flags, 0, n, s);
    cudaMemsetAsync(m->frame_key, 0xFF, (size_t)n * 4, s);
    cudaStreamSynchronize(s);
}

int fluid_morph_frame(FluidMorph *m, FluidDev *fl, const FluidFrame &fr_in, uint8_t *out, cudaStream_t s) {
    const RenderScene &sc = fr_in.sc;
    const uint64_t N = sc.N;
    struct {
        uint32_t f;
        double t;
        FrameArgs fa;
    } fr;
    {
        // get_frame_key / the local time of draw_fluid (morph.cpp:1060-1069)
        size_t f = (size_t)(fr_in.time * sc.K);
        if (f >= sc.K) f = sc.K - 1;
        const double dt = 1.0 / double(sc.K);
        fr.f = (uint32_t)f;
        fr.t = std::max(0.0, (fr_in.time - (double)(fr_in.frame_key * dt)) / dt);
        int rc0 = frame_args(fr_in.rw, sc, fr_in.time, fr.f, fr.t, &fr.fa, s);
        if (rc0) return rc0;
    }
    if (N != fl->n) {
        set_error("fluid: particle count does not match the chains");
        return AM_ERR_STATE;
    }
    const size_t canvas = (size_t)sc.CW * sc.CH, npx = (size_t)sc.width * sc.height;
    int rc;
    // buffers (grow only)
    {
        struct B { void **p; size_t bytes; };
        B bs[] = {{(void **)&m->frame_key, N * 4}, {(void **)&m->src_pos, N * 4}, {(void **)&m->dst_pos, N * 4},
                  {(void **)&m->owner, N}, {(void **)&m->src_map, canvas * 4}, {(void **)&m->dst_map, canvas * 4},
                  {(void **)&m->src_cnt, canvas * 4}, {(void **)&m->dst_cnt, canvas * 4},
                  {(void **)&m->src_any, canvas * 8}, {(void **)&m->flags_a, N * 4}, {(void **)&m->flags_b, N * 4},
                  {(void **)&m->slot_by_rank, N * 4}, {(void **)&m->ckeys, N * 4}, {(void **)&m->cvals, N * 4},
                  {(void **)&m->tk, N * 4}, {(void **)&m->tv, N * 4}, {(void **)&m->hist, radix_hist_words(N) * 4},
                  {(void **)&m->chain_cnt, (size_t)sc.C * 4}, {(void **)&m->to_create, (size_t)sc.C * 4},
                  {(void **)&m->to_delete, (size_t)sc.C * 4}, {(void **)&m->phase1, (size_t)sc.C * 4},
                  {(void **)&m->ncand, 4}, {(void **)&m->acc, npx * 40}, {(void **)&m->col[0], npx * 4},
                  {(void **)&m->col[1], npx * 4}, {(void **)&m->mem[0], npx}, {(void **)&m->mem[1], npx},
                  {(void **)&m->link, N * 8}};
        bool fresh = m->n != N || m->C != sc.C || m->cw != sc.CW || m->ch != sc.CH || m->out_w != sc.width ||
                     m->out_h != sc.height;
        if (fresh) {
            for (auto &b : bs) {
                if (*b.p) cudaFree(*b.p);
                *b.p = nullptr;
            }
            m->n = 0;  // the buffers are sized for (n, C, ...) only once all exist
            for (auto &b : bs) AMG_ALLOC(b.p, std::max<size_t>(b.bytes, 8));
            m->n = (uint32_t)N; m->C = sc.C; m->cw = sc.CW; m->ch = sc.CH; m->out_w = sc.width; m->out_h = sc.height;
            fluid_init_particles(fl, m, sc.width, sc.height, fr_in.sparseness, s);
        }
    }
    FmArgs a;
    std::memset(&a, 0, sizeof(a));
    a.P = sc.P; a.N = N; a.K = sc.K; a.C = sc.C; a.y = fr.f; a.yn = (fr.f + 1) % sc.K; a.f = fr.f;
    a.cw = sc.CW; a.ch = sc.CH; a.width = sc.width; a.height = sc.height;
    a.chain_off = sc.chain_off; a.chain_id = fr_in.chain_id; a.surf = fr_in.surf; a.display = sc.display;
    a.perm = fr_in.perm;
    a.motion = sc.motion; a.fading = sc.fading;
    for (int k = 0; k < 4; ++k) a.bbox[k] = sc.bbox[k];
    a.fa = fr.fa;
    a.t = (float)fr.t; a.sp = (float)fr_in.sparseness;
    a.key = mix64(fr_in.seed_key ^ (++m->frames * 0x9E3779B97F4A7C15ull));
    a.PF = fl->P; a.flags = fl->flags; a.m = *m;
    const unsigned g = (unsigned)std::min<uint64_t>((N + 255) / 256, (uint64_t)kSMs * 8);
    AMG_CUDA(cudaMemsetAsync(m->src_map, 0xFF, canvas * 4, s));
    AMG_CUDA(cudaMemsetAsync(m->dst_map, 0xFF, canvas * 4, s));
    AMG_CUDA(cudaMemsetAsync(m->src_cnt, 0, canvas * 4, s));
    AMG_CUDA(cudaMemsetAsync(m->dst_cnt, 0, canvas * 4, s));
    AMG_CUDA(cudaMemsetAsync(m->src_any, 0, canvas * 8, s));
    AMG_CUDA(cudaMemsetAsync(m->chain_cnt, 0, (size_t)sc.C * 4, s));
    AMG_CUDA(cudaMemsetAsync(m->phase1, 0, (size_t)sc.C * 4, s));
    Prof *prof = render_prof(fr_in.rw);
    if (prof) prof->open(s);
    AMG_LAUNCH(k_fm_classify, g, 256, 0, s, a);
    // active limits (morph.cpp:830-835)
    std::vector<uint32_t> cnt(sc.C), create(sc.C, 0), del(sc.C, 0);
    AMG_CUDA(cudaMemcpyAsync(cnt.data(), m->chain_cnt, (size_t)sc.C * 4, cudaMemcpyDeviceToHost, s));
    AMG_CUDA(cudaStreamSynchronize(s));
    bool any_create = false, any_delete = false;
    for (uint32_t c = 0; c < sc.C; ++c) {
        const double s0 = fr_in.surf_host[(size_t)fr.f * sc.C + c], s1 = fr_in.surf_host[(size_t)a.yn * sc.C + c];
        const uint64_t w = fr_in.chain_off_host[c + 1] - fr_in.chain_off_host[c];
        const uint64_t limit = std::min<uint64_t>((uint64_t)std::llround((1.0 - fr.t) * s0 + fr.t * s1), w);
        if (cnt[c] < limit) { create[c] = (uint32_t)(limit - cnt[c]); any_create = true; }
        else if (cnt[c] > limit) { del[c] = (uint32_t)(cnt[c] - limit); any_delete = true; }
    }
    AMG_CUDA(cudaMemcpyAsync(m->to_create, create.data(), (size_t)sc.C * 4, cudaMemcpyHostToDevice, s));
    AMG_CUDA(cudaMemcpyAsync(m->to_delete, del.data(), (size_t)sc.C * 4, cudaMemcpyHostToDevice, s));
    if (any_delete) {
        AMG_LAUNCH(k_fm_del_flags, g, 256, 0, s, a);
        AMG_CUDA(cudaMemcpyAsync(m->flags_b, m->flags_a, N * 4, cudaMemcpyDeviceToDevice, s));
        if ((rc = launch_scan_u32(m->flags_a, N, nullptr, s))) return rc;
        AMG_LAUNCH(k_fm_delete, g, 256, 0, s, a, m->flags_b);
    }
    if (any_create) {
        AMG_LAUNCH(k_fm_free_flags, g, 256, 0, s, a);
        AMG_CUDA(cudaMemcpyAsync(m->tk, m->flags_b, N * 4, cudaMemcpyDeviceToDevice, s));
        if ((rc = launch_scan_u32(m->flags_b, N, nullptr, s))) return rc;
        AMG_LAUNCH(k_fm_free_rank, g, 256, 0, s, a, m->tk);
        AMG_LAUNCH(k_fm_src_flags, g, 256, 0, s, a);
        AMG_CUDA(cudaMemcpyAsync(m->tk, m->flags_a, N * 4, cudaMemcpyDeviceToDevice, s));
        if ((rc = launch_scan_u32(m->flags_a, N, nullptr, s))) return rc;
        AMG_LAUNCH(k_fm_assign1, g, 256, 0, s, a, m->tk);
        AMG_CUDA(cudaMemsetAsync(m->ncand, 0, 4, s));
        AMG_LAUNCH(k_fm_dst_cands, g, 256, 0, s, a);
        uint32_t nc = 0;
        AMG_CUDA(cudaMemcpyAsync(&nc, m->ncand, 4, cudaMemcpyDeviceToHost, s));
        AMG_CUDA(cudaStreamSynchronize(s));
        if (nc) {
            int bits = 1;
            while ((1ull << bits) < canvas) ++bits;
            if ((rc = radix_sort_pairs(m->ckeys, m->cvals, m->tk, m->tv, m->hist, nc, bits, s))) return rc;
            const unsigned g2 = (unsigned)std::min<uint64_t>((nc + 255) / 256, (uint64_t)kSMs * 8);
            AMG_LAUNCH(k_fm_rekey, g2, 256, 0, s, a, nc);
            int cbits = 1;
            while ((1ull << cbits) < (uint64_t)sc.C + 1) ++cbits;
            if ((rc = radix_sort_pairs(m->ckeys, m->cvals, m->tk, m->tv, m->hist, nc, cbits, s))) return rc;
            AMG_LAUNCH(k_fm_assign2, g2, 256, 0, s, a, nc);
        }
    }
    {
        // the per-column noise table of this pair and chain state
        const bool noise = sc.motion_noise > 0.0;
        auto &k = m->ntab_key;
        if (!k.valid || k.version != fr_in.version || k.seed_key != fr_in.seed_key || k.y != a.y ||
            k.fading != sc.fading || k.noise != noise || k.P != sc.P || m->ntab_n < N) {
            if (m->ntab_n < N) {
                if (m->ntab) cudaFree(m->ntab);
                m->ntab = nullptr;
                m->ntab_n = 0;
                k.valid = false;
                AMG_ALLOC(&m->ntab, std::max<uint64_t>(N, 1) * sizeof(float4));
                m->ntab_n = N;
            }
            AMG_LAUNCH(k_fm_noise, g, 256, 0, s, a, m->ntab, noise ? 1 : 0);
            k.valid = true;
            k.version = fr_in.version;
            k.seed_key = fr_in.seed_key;
            k.y = a.y;
            k.fading = sc.fading;
            k.noise = noise;
            k.P = sc.P;
        }
        a.ntab = m->ntab;
    }
    AMG_LAUNCH(k_fm_update, g, 256, 0, s, a);
    if (prof) prof->close(PROF_FLUID_MANAGE, s);
    // solver steps (morph.cpp:1052-1054)
    const double freedom = std::sqrt((double)sc.width * sc.width + (double)sc.height * sc.height) *
                           fr_in.sparseness / 4.0;
    if ((rc = fluid_run(fl, fr_in.fluidsteps, 0, freedom * (1.0 - fr.t), s, prof))) return rc;
    if (prof) prof->open(s);
    FluidDrawOpts dopt;
    dopt.feather = std::min<uint32_t>(sc.feather, kMaxFeather);
    dopt.keep_bg = sc.keep_background && sc.present ? 1u : 0u;
    dopt.bg = bg_args(sc, fr.f, fr.t);
    dopt.col[0] = m->col[0]; dopt.col[1] = m->col[1]; dopt.mem[0] = m->mem[0]; dopt.mem[1] = m->mem[1];
    rc = fluid_draw(fl, m->acc, sc.width, sc.height, fr_in.sparseness, sc.bbox, fr.t, out, s, dopt);
    if (prof) prof->close(PROF_FLUID_DRAW, s);
    return rc;
}

}  // namespace amg
