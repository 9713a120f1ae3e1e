// Per-atom arithmetic of the frame render shared by the atom path
// (k_render.cu) and the fluid path (k_fluid_morph.cu): Perlin noise, the
// exact position paths of LINEAR and SPLINE motion, the colour fade.
#pragma once

#include "common.cuh"
#include "kernels.h"

namespace amg {

// ----------------------------------------------------------- Perlin FP32 --
// Improved Perlin noise at z = 0 (perlin.cpp:19-43; the z terms vanish since
// fade(0) = 0), 8 octaves (perlin.cpp:57-69), on a permutation in smem.
__device__ __forceinline__ float pgrad(int hash, float x, float y) {
    int h = hash & 15;
    float u = h < 8 ? x : y, v = h < 4 ? y : (h == 12 || h == 14 ? x : 0.f);
    return ((h & 1) == 0 ? u : -u) + ((h & 2) == 0 ? v : -v);
}
__device__ __forceinline__ float pfade(float t) { return t * t * t * (t * (t * 6.f - 15.f) + 10.f); }
static __device__ float pnoise(const int *p, float x, float y) {
    float fx = floorf(x), fy = floorf(y);
    int X = (int)fx & 255, Y = (int)fy & 255;
    x -= fx; y -= fy;
    float u = pfade(x), v = pfade(y);
    int A = p[X] + Y, AA = p[A], AB = p[A + 1];
    int B = p[X + 1] + Y, BA = p[B], BB = p[B + 1];
    float l1 = pgrad(p[AA], x, y) + u * (pgrad(p[BA], x - 1.f, y) - pgrad(p[AA], x, y));
    float l2 = pgrad(p[AB], x, y - 1.f) + u * (pgrad(p[BB], x - 1.f, y - 1.f) - pgrad(p[AB], x, y - 1.f));
    return l1 + v * (l2 - l1);
}
static __device__ float poctave(const int *p, float x, float y) {
    float r = 0.f, amp = 1.f;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        r += pnoise(p, x, y) * amp;
        x *= 2.f; y *= 2.f; amp *= 0.5f;
    }
    return r;
}

// Perlin motion perturbation (no counterpart in the reference, whose atoms
// move along their LINEAR / SPLINE paths only): 8-octave noise at the atom's
// first point of the pair, normalised by the key frames' bounding box at
// frequency 8, one map per axis (PerlinNoise(seed + 2) for x, seed + 3 for
// y), evaluated in FP32 with every operation rounded to nearest separately
// and in a fixed order (the _rn intrinsics keep the compiler from fusing
// them), so a host restatement of the same operations gives the same bits.
// A frame displaces the atom's position word (integer part * 256 + fraction
// byte) by rint(s * n) in 1/256 px, s = A * 256 * sin(pi t) for amplitude A
// px and local time t in the pair, clamped to the 24-bit word.
__device__ __forceinline__ float pfade_rn(float t) {
    const float a = __fadd_rn(__fmul_rn(t, __fsub_rn(__fmul_rn(t, 6.f), 15.f)), 10.f);
    return __fmul_rn(__fmul_rn(__fmul_rn(t, t), t), a);
}
__device__ __forceinline__ float pgrad_rn(int hash, float x, float y) {
    const int h = hash & 15;
    const float u = h < 8 ? x : y, v = h < 4 ? y : (h == 12 || h == 14 ? x : 0.f);
    return __fadd_rn((h & 1) == 0 ? u : -u, (h & 2) == 0 ? v : -v);
}
__device__ __forceinline__ float plerp_rn(float t, float a, float b) { return __fadd_rn(a, __fmul_rn(t, __fsub_rn(b, a))); }
static __device__ float pnoise_rn(const int *p, float x, float y) {
    const float fx = floorf(x), fy = floorf(y);
    const int X = (int)fx & 255, Y = (int)fy & 255;
    x = __fsub_rn(x, fx);
    y = __fsub_rn(y, fy);
    const float u = pfade_rn(x), v = pfade_rn(y);
    const int A = p[X] + Y, AA = p[A], AB = p[A + 1];
    const int B = p[X + 1] + Y, BA = p[B], BB = p[B + 1];
    const float x1 = __fsub_rn(x, 1.f), y1 = __fsub_rn(y, 1.f);
    const float l1 = plerp_rn(u, pgrad_rn(p[AA], x, y), pgrad_rn(p[BA], x1, y));
    const float l2 = plerp_rn(u, pgrad_rn(p[AB], x, y1), pgrad_rn(p[BB], x1, y1));
    return plerp_rn(v, l1, l2);
}
static __device__ float poctave_rn(const int *p, float x, float y) {
    float r = 0.f, amp = 1.f;
#pragma unroll 1
    for (int i = 0; i < 8; ++i) {
        r = __fadd_rn(r, __fmul_rn(pnoise_rn(p, x, y), amp));
        x = __fmul_rn(x, 2.f);
        y = __fmul_rn(y, 2.f);
        amp = __fmul_rn(amp, 0.5f);
    }
    return r;
}
// ((v - b1) * 256 + vf) / (bw * 256) * 8 of one axis of point (v, vf).
__device__ __forceinline__ float noise_coord_rn(int v, int vf, int b1, int bw) {
    return __fmul_rn(__fdiv_rn((float)((v - b1) * 256 + vf), (float)(bw * 256)), 8.f);
}
// Position word w displaced by rint(s * n), clamped to [0, 2^24 - 1].
__device__ __forceinline__ uint32_t displace_rn(uint32_t w, float s, float n) {
    const int d = __float2int_rn(__fmul_rn(s, n));
    return (uint32_t)min(max((int)w + d, 0), 0xFFFFFF);
}

struct FrameArgs {
    double w1, w2;          // LINEAR: weight of pt1 and 1 - that weight
    double b0, b1, b2, b3;  // SPLINE basis at the frame's local time
    // The weights as round(w * 2^30) in 32 bits (every one lies in
    // (-0.08, 1], so it fits), so each product with a 32-bit coordinate
    // difference is one 32 x 32 -> 64-bit multiply-add; b1 enters through
    // the q1 term.
    int32_t w1q, bq0, bq2, bq3;
    uint32_t lin_mode;      // 0 general, 1 w1 == 1 (X = X1), 2 w1 == 0 (X = X2)
    uint32_t key_mode;      // 1 when the spline basis is exactly (0, 1, 0, 0)
    uint32_t seg_ok;        // 1 when the spline segment is the prepared one
    int32_t seg[4];         // control frames when seg_ok == 0
    float str;              // colour weight of the earlier key frame, 1 - t
    float noise_s;          // motion perturbation scale A * 256 * sin(pi t) (0: none this frame)
    uint32_t tiles_x, ntiles;
};

// Fills the frame's position arithmetic for global time `time`, local time
// t of pair f (k_render.cu).
int frame_args(RenderWork *w, const RenderScene &sc, double time, uint32_t f, double t, FrameArgs *out,
               cudaStream_t s);

// Fast exact positions.  The reference evaluates its interpolation in
// double.  The kernels evaluate the same formula's real value in 64-bit fixed
// point (weights quantised to 2^-30) and take its floor / rounded fraction,
// which equals the reference's unless the value lies within the combined
// error bound of a rounding boundary; those rare atoms (and the rarer ones
// with a negative value or a coordinate difference of 2^22 units or more)
// re-run the reference's own double formula (lin_fixed / spl_fixed below).
// The bound is per atom: quantising a weight moves the value by at most half
// a fixed-point unit per unit of the coordinate difference it multiplies,
// i.e. sum |d| / 2 units, and the reference's double rounding (a handful of
// operations on values below 2^16 px, plus its weights summing to 1 only
// within a few ulps) stays below 2^-33 px.  Returns false when the fallback
// is needed.
//
// LINEAR: X = floor(w1 a + (1 - w1) b) in 1/256 px (morph.cpp:1501-1515).
// V = b 2^30 + round(w1 2^30) (a - b), units of 2^-30 / 256 px.
__device__ __forceinline__ bool lin_fast(const FrameArgs &fa, int32_t a, int32_t b, int32_t *out) {
    if (fa.lin_mode == 1) { *out = a; return true; }
    if (fa.lin_mode == 2) { *out = b; return true; }
    const int32_t d = a - b;
    const long long V = (long long)fa.w1q * d + ((long long)b << 30);
    const uint32_t r = (uint32_t)V & ((1u << 30) - 1u);
    const uint32_t tol = ((uint32_t)abs(d) >> 1) + 64u;  // 64 units = 2^-32 px, above the reference's error
    if (r < tol || (1u << 30) - r < tol) return false;
    *out = (int32_t)(V >> 30);
    return true;
}
// SPLINE: the Catmull-Rom value v of the prepared basis (morph.cpp:526-531,
// spline.cpp:45-57), then the reference's split into integer pixel trunc(v)
// and fraction byte round(frac * 255), packed (integer << 8) | byte.
// V = q1 2^30 + sum_i round(b_i 2^30) (q_i - q1), units of 2^-38 px; its top
// 32 fraction bits f (units of 2^-32 px) give both roundings in 32-bit
// arithmetic: the integer boundary is f near 0 or 2^32, the byte is the high
// word of f * 255 + 2^31 and its boundary the low word near 0 or 2^32.
__device__ __forceinline__ bool spl_fast(const FrameArgs &fa, int32_t q0, int32_t q1, int32_t q2, int32_t q3,
                                         uint32_t *out) {
    const int32_t d0 = q0 - q1, d2 = q2 - q1, d3 = q3 - q1;
    const uint32_t a0 = (uint32_t)abs(d0), a2 = (uint32_t)abs(d2), a3 = (uint32_t)abs(d3);
    if ((a0 | a2 | a3) >= (1u << 22)) return false;  // keeps V in 63 bits and the bounds in 32
    long long V = (long long)q1 << 30;
    V += (long long)fa.bq0 * d0;
    V += (long long)fa.bq2 * d2;
    V += (long long)fa.bq3 * d3;
    if (V < 0) return false;  // left of the canvas origin: the reference's signed split decides
    const uint32_t I = (uint32_t)(V >> 38), f = (uint32_t)(V >> 6);
    const unsigned long long p = (unsigned long long)f * 255ull + 0x80000000ull;
    if (!fa.key_mode) {
        // sum |d| / 2 units of 2^-38 px quantisation + 2^-33 px reference error
        // + the 2^-32 px truncation of f, in units of 2^-32 px
        const uint32_t tol = ((a0 + a2 + a3) >> 7) + 4u;
        if (f < tol || f > ~tol) return false;
        const uint32_t lo = (uint32_t)p, t255 = tol * 255u + 255u;
        if (lo < t255 || lo > ~t255) return false;
    }
    *out = ((I & 0xFFFFu) << 8) | ((uint32_t)(p >> 32) & 0xFFu);
    return true;
}

// The FP64 fallbacks are out of line on purpose: inlined, the compiler may
// evaluate them under a predicate for every atom, and FP64 throughput is low.
static __device__ __noinline__ int32_t lin_fixed(double w1, double w2, int32_t a, int32_t b) {
    double v = __dadd_rn(__dmul_rn(w1, (double)a), __dmul_rn(w2, (double)b));
    return (int32_t)v;  // v >= 0: truncation is floor
}
// Catmull-Rom value at the prepared basis, then the reference's modf /
// round(fract * 255) split (morph.cpp:528-530).  Returns the 1/256 grid
// position as (integer part << 8) | fract byte with the integer part taken
// modulo 2^16 like the x86 build's double -> uint16 conversion.
static __device__ __noinline__ uint32_t spl_fixed(double b0, double b1, double b2, double b3, int32_t q0, int32_t q1,
                                           int32_t q2, int32_t q3) {
    double v0 = (double)(q0 >> 8) + (double)(q0 & 255) / 256.0;
    double v1 = (double)(q1 >> 8) + (double)(q1 & 255) / 256.0;
    double v2 = (double)(q2 >> 8) + (double)(q2 & 255) / 256.0;
    double v3 = (double)(q3 >> 8) + (double)(q3 & 255) / 256.0;
    double v = __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(v0, b0), __dmul_rn(v1, b1)), __dmul_rn(v2, b2)),
                         __dmul_rn(v3, b3));
    double ip = trunc(v);
    double fr = __dsub_rn(v, ip);
    uint32_t xi = (uint32_t)(int)ip & 0xFFFFu;
    uint32_t xf = (uint32_t)(int)round(__dmul_rn(fr, 255.0)) & 0xFFu;
    return (xi << 8) | xf;
}

// Colour fade of one atom (morph.cpp:537-550, 1467-1488) in FP32.  The
// PERLIN / COSINE ramp of an atom depends on its lag and slope only, so its
// parameters are prepared once per key-frame pair: fade_params gives
// (l, pi / s) with s = (slope + 0.1) / 1.1 and l = (1 - s) lag, and the
// frame's weight of the earlier colour is 0 up to l, 1 from l + s and the
// cosine ramp between.  Octave noise below -1.2 makes s <= 0: the reference's
// tests then give 0 up to l and 1 after it, a step, which pi / s = +inf
// reproduces (x is +inf past l, NaN at l, -inf before).
__device__ __forceinline__ float2 fade_params(float lag, float slope) {
    const float s = (slope + 0.1f) / 1.1f;
    return make_float2((1.f - s) * lag, s > 0.f ? 3.14159265358f / s : __int_as_float(0x7f800000));
}
__device__ __forceinline__ uint32_t fade_colour(uint32_t fading, uint32_t c1, uint32_t c2, float2 fp, float str) {
    if (fading == AM_PERLIN || fading == AM_COSINE) {
        const float x = (str - fp.x) * fp.y;
        if (!(x > 0.f)) str = 0.f;
        else if (x >= 3.14159265358f) str = 1.f;
        else str = (1.f - __cosf(x)) * 0.5f;  // x in (0, pi): the intrinsic's error is far below 1/255
    }
    uint32_t o = 0;
#pragma unroll
    for (int ch = 0; ch < 4; ++ch) {
        float a = (float)((c1 >> (8 * ch)) & 255u), b = (float)((c2 >> (8 * ch)) & 255u);
        float v = str * a + (1.f - str) * b;
        o |= ((uint32_t)(int)roundf(v) & 255u) << (8 * ch);
    }
    return o;
}

// get_background (morph.cpp:1431-1465) inputs for one frame: key frames f
// and f + 1 ([CH][CW] RGB and presence), the fading, the Perlin maps and the
// bbox the noise coordinates are normalised by; str = 1 - t.
struct BgArgs {
    uint32_t fading;
    const uint32_t *disp1, *disp2;
    const uint8_t *pres1, *pres2;
    uint32_t CW, CH;
    const int *perm;  // [2][512] (lag, slope)
    float bx1, by1, bw, bh;
    float str;
};
inline BgArgs bg_args(const RenderScene &sc, uint32_t f, double t) {
    BgArgs o;
    const size_t fr = (size_t)sc.CW * sc.CH, fn = (f + 1) % sc.K;
    o.fading = sc.fading;
    o.disp1 = sc.display + f * fr;
    o.disp2 = sc.display + fn * fr;
    o.pres1 = sc.present ? sc.present + f * fr : nullptr;
    o.pres2 = sc.present ? sc.present + fn * fr : nullptr;
    o.CW = sc.CW;
    o.CH = sc.CH;
    o.perm = sc.perm;
    o.bx1 = (float)sc.bbox[0];
    o.by1 = (float)sc.bbox[1];
    o.bw = (float)(sc.bbox[2] - sc.bbox[0] + 1);
    o.bh = (float)(sc.bbox[3] - sc.bbox[1] + 1);
    o.str = (float)(1.0 - t);
    return o;
}

// The background colour at pixel (x, y): the key frames' colours (a pixel a
// key frame lacks reads as transparent black) cross-faded, PERLIN at the
// pixel itself in FP32.
static __device__ __noinline__ uint32_t bg_colour(const BgArgs &o, uint32_t x, uint32_t y) {
    uint32_t c1 = 0, c2 = 0;
    if (x < o.CW && y < o.CH && o.pres1) {
        const size_t i = (size_t)y * o.CW + x;
        if (o.pres1[i]) c1 = o.disp1[i];
        if (o.pres2[i]) c2 = o.disp2[i];
    }
    float2 fp = fade_params(0.5f, 0.5f);
    if (o.fading == AM_PERLIN && o.perm) {
        const float px = ((float)((int)x - (int)o.bx1) / o.bw) * 8.f, py = ((float)((int)y - (int)o.by1) / o.bh) * 8.f;
        fp = fade_params(poctave(o.perm, px, py) * 0.5f + 0.5f, poctave(o.perm + 512, px, py) * 0.5f + 0.5f);
    }
    return fade_colour(o.fading, c1, c2, fp, o.str);
}

// The composite drawn over the background (morph.cpp:1387-1399, 1270-1296):
// n colours (the first c0; the FP64 "over" state st for two or more), bg the
// background colour; create_color of the result.
static __device__ __noinline__ uint32_t over_background(int n, uint32_t c0, const double *st, uint32_t bg) {
    if (n == 0) return bg;
    double r, g, b, a;
    if (n == 1) {
        r = (c0 & 255u) / 255.0; g = ((c0 >> 8) & 255u) / 255.0; b = ((c0 >> 16) & 255u) / 255.0; a = (c0 >> 24) / 255.0;
    } else {
        r = st[0]; g = st[1]; b = st[2]; a = st[3];
    }
    const double br = (bg & 255u) / 255.0, bgg = ((bg >> 8) & 255u) / 255.0, bb = ((bg >> 16) & 255u) / 255.0,
                 ba = (bg >> 24) / 255.0;
    const double om = __dsub_rn(1.0, a);
    r = __dadd_rn(__dmul_rn(a, r), __dmul_rn(om, br));
    g = __dadd_rn(__dmul_rn(a, g), __dmul_rn(om, bgg));
    b = __dadd_rn(__dmul_rn(a, b), __dmul_rn(om, bb));
    a = __dadd_rn(ba, __dmul_rn(__dsub_rn(1.0, ba), a));
    const double v[4] = {r, g, b, a};
    uint32_t o = 0;
    for (int k = 0; k < 4; ++k) o |= ((uint32_t)(int)round(__dmul_rn(v[k], 255.0)) & 255u) << (8 * k);
    return o;
}

}  // namespace amg
