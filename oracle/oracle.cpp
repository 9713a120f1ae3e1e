// ORACLE — test infrastructure only.
//
// A CPU restatement, in plain C++17, of the atomorph reference algorithms on
// the morph hot path.  It is the checker for the CUDA library: only tests/,
// __graft_entry__.smoke() and bench.py's CPU-baseline legs load it, and never
// as the thing measured or shipped.
//
// Parity is pinned against the unmodified reference library compiled from its
// own sources (oracle/Makefile -> oracle/_ref/libamref.so): the pin tests in
// tests/test_oracle_pin.py require bit-identical results for the colour
// conversions, Perlin noise, splines, the atom cost, the refinement sweeps,
// frame rendering and the fluid step, and tests/golden/ holds fixtures made by
// the reference itself (tests/golden/make_golden.py) so the pin also holds on
// machines without the reference sources.
//
// All arithmetic follows the reference's operation order in IEEE double; the
// Makefile builds with -ffp-contract=off so no fused multiply-add changes a
// bit between x86 and Arm.  Random streams use the same <random> engines and
// distributions as the reference (libstdc++), which is what makes the
// refinement sweeps bit-exact.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <map>
#include <numeric>
#include <random>
#include <set>
#include <thread>
#include <vector>

namespace {

constexpr uint8_t HAS_PIXEL = 1;
constexpr uint8_t HAS_FLUID = 2;
constexpr unsigned RGB = 0, HSP = 1, NONE = 2, LINEAR = 3, SPLINE = 4, COSINE = 5, PERLIN = 6;

// ---------------------------------------------------------------- points ---
// atomorph.h:275-284: x u16 | y u16 | x_fract u8 | y_fract u8 | flags u8.
struct Pt {
    uint16_t x, y;
    uint8_t xf, yf, flags;
};
inline Pt unpack(uint64_t w) {
    Pt p;
    p.x = (uint16_t)(w & 0xFFFF);
    p.y = (uint16_t)((w >> 16) & 0xFFFF);
    p.xf = (uint8_t)((w >> 32) & 0xFF);
    p.yf = (uint8_t)((w >> 40) & 0xFF);
    p.flags = (uint8_t)((w >> 48) & 0xFF);
    return p;
}
inline uint64_t pack(const Pt &p) {
    return (uint64_t)p.x | ((uint64_t)p.y << 16) | ((uint64_t)p.xf << 32) | ((uint64_t)p.yf << 40) |
           ((uint64_t)p.flags << 48);
}
// point_distance, atomorph.h:334-339: squared distance in 1/256 px.
inline uint64_t pdist(uint64_t a, uint64_t b) {
    Pt p = unpack(a), q = unpack(b);
    int64_t xd = std::llabs((int64_t)(256 * p.x + p.xf) - (int64_t)(256 * q.x + q.xf));
    int64_t yd = std::llabs((int64_t)(256 * p.y + p.yf) - (int64_t)(256 * q.y + q.yf));
    return (uint64_t)(xd * xd + yd * yd);
}

// ---------------------------------------------------------------- colour ---
struct Col {
    uint8_t r, g, b, a;
};
inline Col col_of(uint32_t c) { return Col{(uint8_t)c, (uint8_t)(c >> 8), (uint8_t)(c >> 16), (uint8_t)(c >> 24)}; }
inline uint32_t u32_of(Col c) { return c.r | (c.g << 8) | (c.b << 16) | ((uint32_t)c.a << 24); }

const double Pr = 0.299, Pg = 0.587, Pb = 0.114;

// HSP colour model (color.cpp:104-142), restated.
void rgb2hsp(double R, double G, double B, double *H, double *S, double *P) {
    *P = std::sqrt(R * R * Pr + G * G * Pg + B * B * Pb);
    if (R == G && R == B) { *H = 0.; *S = 0.; return; }
    if (R >= G && R >= B) {
        if (B >= G) { *H = 6. / 6. - 1. / 6. * (B - G) / (R - G); *S = 1. - G / R; }
        else        { *H = 0. / 6. + 1. / 6. * (G - B) / (R - B); *S = 1. - B / R; }
    } else if (G >= R && G >= B) {
        if (R >= B) { *H = 2. / 6. - 1. / 6. * (R - B) / (G - B); *S = 1. - B / G; }
        else        { *H = 2. / 6. + 1. / 6. * (B - R) / (G - R); *S = 1. - R / G; }
    } else {
        if (G >= R) { *H = 4. / 6. - 1. / 6. * (G - R) / (B - R); *S = 1. - R / B; }
        else        { *H = 4. / 6. + 1. / 6. * (R - G) / (B - G); *S = 1. - G / B; }
    }
}

// color.cpp:157-211, restated.
void hsp2rgb(double H, double S, double P, double *R, double *G, double *B) {
    double part, mom = 1. - S;
    if (mom > 0.) {
        if (H < 1. / 6.) {
            H = 6. * (H - 0. / 6.); part = 1. + H * (1. / mom - 1.);
            *B = P / std::sqrt(Pr / mom / mom + Pg * part * part + Pb); *R = (*B) / mom; *G = (*B) + H * ((*R) - (*B));
        } else if (H < 2. / 6.) {
            H = 6. * (-H + 2. / 6.); part = 1. + H * (1. / mom - 1.);
            *B = P / std::sqrt(Pg / mom / mom + Pr * part * part + Pb); *G = (*B) / mom; *R = (*B) + H * ((*G) - (*B));
        } else if (H < 3. / 6.) {
            H = 6. * (H - 2. / 6.); part = 1. + H * (1. / mom - 1.);
            *R = P / std::sqrt(Pg / mom / mom + Pb * part * part + Pr); *G = (*R) / mom; *B = (*R) + H * ((*G) - (*R));
        } else if (H < 4. / 6.) {
            H = 6. * (-H + 4. / 6.); part = 1. + H * (1. / mom - 1.);
            *R = P / std::sqrt(Pb / mom / mom + Pg * part * part + Pr); *B = (*R) / mom; *G = (*R) + H * ((*B) - (*R));
        } else if (H < 5. / 6.) {
            H = 6. * (H - 4. / 6.); part = 1. + H * (1. / mom - 1.);
            *G = P / std::sqrt(Pb / mom / mom + Pr * part * part + Pg); *B = (*G) / mom; *R = (*G) + H * ((*B) - (*G));
        } else {
            H = 6. * (-H + 6. / 6.); part = 1. + H * (1. / mom - 1.);
            *G = P / std::sqrt(Pr / mom / mom + Pb * part * part + Pg); *R = (*G) / mom; *B = (*G) + H * ((*R) - (*G));
        }
    } else {
        if (H < 1. / 6.)      { H = 6. * (H - 0. / 6.);  *R = std::sqrt(P * P / (Pr + Pg * H * H)); *G = (*R) * H; *B = 0.; }
        else if (H < 2. / 6.) { H = 6. * (-H + 2. / 6.); *G = std::sqrt(P * P / (Pg + Pr * H * H)); *R = (*G) * H; *B = 0.; }
        else if (H < 3. / 6.) { H = 6. * (H - 2. / 6.);  *G = std::sqrt(P * P / (Pg + Pb * H * H)); *B = (*G) * H; *R = 0.; }
        else if (H < 4. / 6.) { H = 6. * (-H + 4. / 6.); *B = std::sqrt(P * P / (Pb + Pg * H * H)); *G = (*B) * H; *R = 0.; }
        else if (H < 5. / 6.) { H = 6. * (H - 4. / 6.);  *B = std::sqrt(P * P / (Pb + Pr * H * H)); *R = (*B) * H; *G = 0.; }
        else                  { H = 6. * (-H + 6. / 6.); *R = std::sqrt(P * P / (Pr + Pb * H * H)); *B = (*R) * H; *G = 0.; }
    }
}

// color.cpp:64-92: byte-level conversions (alpha passes through).
Col to_hsp(Col c) {
    double h, s, p;
    rgb2hsp(c.r / 255.0, c.g / 255.0, c.b / 255.0, &h, &s, &p);
    Col o = c;
    o.r = (uint8_t)std::round(h * 255.0);
    o.g = (uint8_t)std::round(s * 255.0);
    o.b = (uint8_t)std::round(p * 255.0);
    return o;
}
Col to_rgb(Col c) {
    double r, g, b;
    hsp2rgb(c.r / 255.0, c.g / 255.0, c.b / 255.0, &r, &g, &b);
    Col o = c;
    o.r = (uint8_t)std::min(std::round(r * 255.0), 255.0);
    o.g = (uint8_t)std::min(std::round(g * 255.0), 255.0);
    o.b = (uint8_t)std::min(std::round(b * 255.0), 255.0);
    return o;
}
// create_color(double...), color.cpp:55-62.
inline Col make_col(double r, double g, double b, double a) {
    return Col{(uint8_t)std::round(r * 255.0), (uint8_t)std::round(g * 255.0), (uint8_t)std::round(b * 255.0),
               (uint8_t)std::round(a * 255.0)};
}
// color_distance, color.h:17-24.
inline double cdist(Col a, Col b) {
    int rd = a.r - b.r, gd = a.g - b.g, bd = a.b - b.b, ad = a.a - b.a;
    return std::sqrt((double)(rd * rd + gd * gd + bd * bd + ad * ad)) / 510.0;
}

// ---------------------------------------------------------------- Perlin ---
// Improved Perlin noise (K. Perlin 2002) with a permutation shuffled by
// std::mt19937(seed), as perlin.cpp:11-89 sets it up.
struct Perlin {
    int p[512];
    explicit Perlin(unsigned seed = 1) {
        if (seed == 0) seed = std::mt19937::default_seed;
        std::iota(p, p + 256, 0);
        std::shuffle(p, p + 256, std::mt19937(seed));
        for (int i = 0; i < 256; ++i) p[256 + i] = p[i];
    }
    static double fade(double t) { return t * t * t * (t * (t * 6 - 15) + 10); }
    static double lerp(double t, double a, double b) { return a + t * (b - a); }
    static double grad(int hash, double x, double y, double z) {
        int h = hash & 15;
        double u = h < 8 ? x : y, v = h < 4 ? y : (h == 12 || h == 14 ? x : z);
        return ((h & 1) == 0 ? u : -u) + ((h & 2) == 0 ? v : -v);
    }
    double noise(double x, double y, double z) const {
        int X = (int)std::floor(x) & 255, Y = (int)std::floor(y) & 255, Z = (int)std::floor(z) & 255;
        x -= std::floor(x); y -= std::floor(y); z -= std::floor(z);
        double u = fade(x), v = fade(y), w = fade(z);
        int A = p[X] + Y, AA = p[A] + Z, AB = p[A + 1] + Z;
        int B = p[X + 1] + Y, BA = p[B] + Z, BB = p[B + 1] + Z;
        return lerp(w,
                    lerp(v, lerp(u, grad(p[AA], x, y, z), grad(p[BA], x - 1, y, z)),
                         lerp(u, grad(p[AB], x, y - 1, z), grad(p[BB], x - 1, y - 1, z))),
                    lerp(v, lerp(u, grad(p[AA + 1], x, y, z - 1), grad(p[BA + 1], x - 1, y, z - 1)),
                         lerp(u, grad(p[AB + 1], x, y - 1, z - 1), grad(p[BB + 1], x - 1, y - 1, z - 1))));
    }
    double octave(double x, double y, int oct) const {
        double r = 0.0, amp = 1.0;
        for (int i = 0; i < oct; ++i) {
            r += noise(x, y, 0.0) * amp;
            x *= 2.0; y *= 2.0; amp *= 0.5;
        }
        return r;
    }
};

// ---------------------------------------------------------------- spline ---
// Cyclic Catmull-Rom through n points at global t in [0,1) (spline.cpp:29-57).
void spline_eval(const double *xs, const double *ys, int n, double t, double *ox, double *oy) {
    double delta_t = 1.0 / n;
    int p = (int)(t / delta_t);
    // cyclic indices: the reference's single wrap (spline.cpp:49-52) for n >= 2; with one
    // key frame it reads past its control points, here every index is that frame
    auto wrap = [n](int i) { return ((i % n) + n) % n; };
    int p0 = wrap(p - 1), p1 = wrap(p), p2 = wrap(p + 1), p3 = wrap(p + 2);
    double lt = (t - delta_t * (double)p) / delta_t;
    double t2 = lt * lt, t3 = t2 * lt;
    double b1 = 0.5 * (-t3 + 2.0 * t2 - lt);
    double b2 = 0.5 * (3.0 * t3 - 5.0 * t2 + 2.0);
    double b3 = 0.5 * (-3.0 * t3 + 4.0 * t2 + lt);
    double b4 = 0.5 * (t3 - t2);
    // Vec3D arithmetic order: ((p1*b1 + p2*b2) + p3*b3) + p4*b4.
    *ox = xs[p0] * b1 + xs[p1] * b2 + xs[p2] * b3 + xs[p3] * b4;
    *oy = ys[p0] * b1 + ys[p1] * b2 + ys[p2] * b3 + ys[p3] * b4;
}

}  // namespace

// ====================================================================== ABI ==
extern "C" {

uint32_t orc_rgb_to_hsp(uint32_t c) { return u32_of(to_hsp(col_of(c))); }
uint32_t orc_hsp_to_rgb(uint32_t c) { return u32_of(to_rgb(col_of(c))); }
double orc_octave_noise(unsigned seed, double x, double y, int oct) { return Perlin(seed).octave(x, y, oct); }
void orc_spline_eval(const double *xy, int n, double t, double *out) {
    std::vector<double> xs(n), ys(n);
    for (int i = 0; i < n; ++i) { xs[i] = xy[2 * i]; ys[i] = xy[2 * i + 1]; }
    spline_eval(xs.data(), ys.data(), n, t, out, out + 1);
}

// Atom cost, thread.cpp:1109-1125, summed over chains: exact integer total
// (returned through *exact) and the reference's double accumulation order.
double orc_energy(const uint64_t *pts, const uint64_t *widths, uint32_t C, uint32_t K, uint64_t *exact) {
    uint64_t N = 0;
    for (uint32_t c = 0; c < C; ++c) N += widths[c];
    double total = 0.0;
    unsigned __int128 ex = 0;
    uint64_t off = 0;
    for (uint32_t c = 0; c < C; ++c) {
        uint64_t w = widths[c];
        double e = 0.0;
        if (w > 1 && K > 0) {
            for (uint64_t i = 0; i < w; ++i)
                for (uint32_t j = 0; j < K; ++j) {
                    uint64_t d = pdist(pts[(uint64_t)j * N + off + i], pts[(uint64_t)((j + 1) % K) * N + off + i]);
                    e += (double)d;
                    ex += d;
                }
        }
        total += e;
        off += w;
    }
    if (exact) *exact = (uint64_t)ex;
    return total;
}

// Refinement sweeps, restating morph_asynch (thread.cpp:990-1041) on the
// frame-major layout pts[y*N + off + x].  One sweep = for every chain in
// order, K calls with repeat = width and a seed drawn from std::mt19937(seed)
// -- the same definition the harness applies to the reference, so the two
// produce identical points.
void orc_sweeps(uint64_t *pts, const uint64_t *widths, uint32_t C, uint32_t K, uint64_t nsweeps, unsigned seed) {
    uint64_t N = 0;
    for (uint32_t c = 0; c < C; ++c) N += widths[c];
    std::mt19937 seeds(seed);
    for (uint64_t s = 0; s < nsweeps; ++s) {
        uint64_t off = 0;
        for (uint32_t c = 0; c < C; ++c) {
            uint64_t w = widths[c];
            if (w <= 1) { off += w; continue; }
            for (uint32_t k = 0; k < K; ++k) {
                std::mt19937 gen((unsigned)seeds());
                std::uniform_int_distribution<size_t> ux(0, w - 1);
                std::uniform_int_distribution<size_t> uy(0, K - 1);
                size_t y = uy(gen), yn = (y + 1) % K, yp = (y > 0 ? y - 1 : K - 1);
                uint64_t *P = pts + off;
                for (uint64_t i = 0; i < w; ++i) {
                    size_t x1 = ux(gen), x2;
                    do { x2 = ux(gen); } while (x1 == x2);
                    uint64_t a1p = P[yp * N + x1], a2p = P[yp * N + x2];
                    uint64_t a1 = P[y * N + x1], a2 = P[y * N + x2];
                    uint64_t a1n = P[yn * N + x1], a2n = P[yn * N + x2];
                    double e1b = (double)(pdist(a1p, a1) + pdist(a1, a1n));
                    double e2b = (double)(pdist(a2p, a2) + pdist(a2, a2n));
                    double e1a = (double)(pdist(a2p, a1) + pdist(a1, a2n));
                    double e2a = (double)(pdist(a1p, a2) + pdist(a2, a1n));
                    double c1 = e1b + e2b, c2 = e1a + e2a;
                    if (c1 >= c2) { P[y * N + x1] = a2; P[y * N + x2] = a1; }
                }
            }
            off += w;
        }
    }
}

// ---------------------------------------------------------- motion noise ---
// Perlin motion perturbation (no counterpart in the reference, which moves
// atoms along their LINEAR / SPLINE paths only).  Definition:
//   * two noise maps, PerlinNoise(seed + 2) for x and PerlinNoise(seed + 3)
//     for y (the morph's seed; the colour fade's lag and slope maps use seed
//     and seed + 1, morph.h:136-137, morph.cpp:436-444);
//   * sampled at the atom's point pt1 at the pair's first key frame,
//     normalised by the key frames' bounding box at frequency 8, as the lag
//     map is (morph.cpp:540-545);
//   * 8-octave noise (perlin.cpp:57-69) evaluated in IEEE single precision,
//     every operation separately rounded to nearest in the order written
//     below (the GPU evaluates the same operations, so both give the same
//     bits); its FP64 form is the accuracy reference;
//   * displacement D = rint(s * n) in 1/256 px, s = (float)(A * 256 *
//     sin(pi * t)), A the amplitude in px, t the local time in the key-frame
//     pair (zero at key frames, so paths stay continuous);
//   * added to the position word the motion gives (integer part * 256 +
//     fraction byte, morph.cpp:523-531), clamped to [0, 2^24 - 1].
struct Perm {
    int p[512];
    explicit Perm(unsigned seed) {
        if (seed == 0) seed = std::mt19937::default_seed;
        std::iota(p, p + 256, 0);
        std::shuffle(p, p + 256, std::mt19937(seed));
        for (int i = 0; i < 256; ++i) p[256 + i] = p[i];
    }
};
inline float fade_f(float t) {
    const float a = t * (t * 6.0f - 15.0f) + 10.0f;
    return t * t * t * a;
}
inline float grad_f(int hash, float x, float y) {
    const int h = hash & 15;
    const float u = h < 8 ? x : y, v = h < 4 ? y : (h == 12 || h == 14 ? x : 0.0f);
    return ((h & 1) == 0 ? u : -u) + ((h & 2) == 0 ? v : -v);
}
inline float lerp_f(float t, float a, float b) { return a + t * (b - a); }
float noise_f(const int *p, float x, float y) {
    const float fx = std::floor(x), fy = std::floor(y);
    const int X = (int)fx & 255, Y = (int)fy & 255;
    x = x - fx;
    y = y - fy;
    const float u = fade_f(x), v = fade_f(y);
    const int A = p[X] + Y, AA = p[A], AB = p[A + 1];
    const int B = p[X + 1] + Y, BA = p[B], BB = p[B + 1];
    const float l1 = lerp_f(u, grad_f(p[AA], x, y), grad_f(p[BA], x - 1.0f, y));
    const float l2 = lerp_f(u, grad_f(p[AB], x, y - 1.0f), grad_f(p[BB], x - 1.0f, y - 1.0f));
    return lerp_f(v, l1, l2);
}
float octave_f(const int *p, float x, float y) {
    float r = 0.0f, amp = 1.0f;
    for (int i = 0; i < 8; ++i) {
        r = r + noise_f(p, x, y) * amp;
        x = x * 2.0f;
        y = y * 2.0f;
        amp = amp * 0.5f;
    }
    return r;
}
// The noise coordinates of point (x, xf) on one axis: the bbox-normalised
// position at frequency 8, (((x - b1) * 256 + xf) / (bw * 256)) * 8.
inline float noise_coord_f(int x, int xf, int b1, int bw) {
    return ((float)((x - b1) * 256 + xf) / (float)(bw * 256)) * 8.0f;
}
inline double noise_coord_d(int x, int xf, int b1, int bw) {
    return (((double)(x - b1) * 256 + xf) / double(bw * 256.0)) * 8.0;
}
// Displacement (dx, dy) in 1/256 px of an atom whose pair's first point is
// pt1; fp64 selects the FP64 accuracy reference instead of the definition.
void motion_offset(const Perm &mx, const Perm &my, const Perlin &nx64, const Perlin &ny64, const uint32_t *bbox,
                   double amplitude, double t, Pt pt1, bool fp64, int32_t *dx, int32_t *dy) {
    const int bw = (int)bbox[2] - (int)bbox[0] + 1, bh = (int)bbox[3] - (int)bbox[1] + 1;
    const double sd = amplitude * 256.0 * std::sin(3.141592653589793 * t);
    if (fp64) {
        const double u = noise_coord_d(pt1.x, pt1.xf, (int)bbox[0], bw), v = noise_coord_d(pt1.y, pt1.yf, (int)bbox[1], bh);
        *dx = (int32_t)std::nearbyint(sd * nx64.octave(u, v, 8));
        *dy = (int32_t)std::nearbyint(sd * ny64.octave(u, v, 8));
        return;
    }
    const float sf = (float)sd;
    const float u = noise_coord_f(pt1.x, pt1.xf, (int)bbox[0], bw), v = noise_coord_f(pt1.y, pt1.yf, (int)bbox[1], bh);
    *dx = (int32_t)std::nearbyint(sf * octave_f(mx.p, u, v));
    *dy = (int32_t)std::nearbyint(sf * octave_f(my.p, u, v));
}
// Position word plus displacement, clamped to the 24-bit word.
inline int32_t displaced(int32_t w, int32_t d) {
    const int64_t v = (int64_t)w + d;
    return (int32_t)std::min<int64_t>(std::max<int64_t>(v, 0), 0xFFFFFF);
}
// The four maps of a scene's seed.
struct NoiseMaps {
    Perm mx, my;
    Perlin mx64, my64;
    explicit NoiseMaps(unsigned seed) : mx(seed + 2), my(seed + 3), mx64(seed + 2), my64(seed + 3) {}
};

// ------------------------------------------------------------ rendering ---
// Scene handed to the renderer: what morph::get_pixels(t) reads.
struct orc_scene {
    uint32_t K, C;              // key frames (index order), chains (groups)
    uint32_t CW, CH;            // canvas of the stored key-frame colours
    uint32_t width, height;     // morph resolution (set_resolution)
    uint32_t bbox[4];           // x1 y1 x2 y2 over all key-frame pixels
    uint32_t seed;              // set_seed: Perlin lag map seed, slope map seed+1
    uint32_t motion, fading, delimiter, density;
    const uint32_t *colors;     // [K][CH][CW] stored colour (HSP or RGB)
    const uint8_t *present;     // [K][CH][CW] 1 where the key frame has a pixel
    const uint64_t *widths;     // [C]
    const uint64_t *pts;        // [K][N]
    const int32_t *blob_order;  // [K][C] group of the b-th blob of key frame k
    const uint64_t *frame_keys; // [K] map keys of the key frames
    uint32_t feather;           // set_feather: outer layers of each blob faded
    uint32_t keep_background;   // set_keep_background
    uint32_t show_blobs;        // set_show_blobs: TEXTURE 0, AVERAGE 1, DISTINCT 2
    const uint32_t *blob_avg;   // [K][C] create_color of the b-th blob's mean colour (stored space), for AVERAGE
    double motion_noise;        // Perlin motion perturbation amplitude in px (0: off); not in the reference
};

}  // extern "C"

namespace {

struct Px {
    uint16_t x, y;
    Col c;
};

// morph::get_pixel (morph.cpp:378-392): stored colour, HSP -> RGB on read;
// a missing pixel reads as (0,0,0,0).
inline Col read_pixel(const orc_scene &s, uint32_t k, uint32_t x, uint32_t y) {
    if (x >= s.CW || y >= s.CH) return Col{0, 0, 0, 0};
    size_t i = ((size_t)k * s.CH + y) * s.CW + x;
    if (!s.present[i]) return Col{0, 0, 0, 0};
    Col c = col_of(s.colors[i]);
    if (s.delimiter == HSP) c = to_rgb(c);
    return c;
}

// morph::interpolate(color, color, w), morph.cpp:1481-1488.
inline Col lerp_col(Col c1, Col c2, double w) {
    Col c;
    c.r = (uint8_t)std::round(w * double(c1.r) + (1.0 - w) * double(c2.r));
    c.g = (uint8_t)std::round(w * double(c1.g) + (1.0 - w) * double(c2.g));
    c.b = (uint8_t)std::round(w * double(c1.b) + (1.0 - w) * double(c2.b));
    c.a = (uint8_t)std::round(w * double(c1.a) + (1.0 - w) * double(c2.a));
    return c;
}
// morph.cpp:1467-1479: lag/slope cosine ramp.
inline Col ramp_col(Col c1, Col c2, double lag, double slope, double str) {
    const double pi = 3.14159265358;
    double s = (slope + 0.1) / 1.1;
    double l = (1.0 - s) * lag;
    if (str <= l) str = 0.0;
    else if (str >= (l + s)) str = 1.0;
    else str = ((-std::cos((str - l) * (pi / s)) + 1.0) / 2.0);
    return lerp_col(c1, c2, str);
}

// The atom's point at local time t of pair y (global time `time`): the
// motion's position (LINEAR morph.cpp:1501-1515, SPLINE morph.cpp:526-531,
// NONE the first point) plus the motion perturbation when it is on (FP64
// noise when fp64, for the accuracy comparison).  col = the atom's column in
// the frame-major point array.
// morph::interpolate(point, point, w) (morph.cpp:1501-1515) at w = 1 - t.
Pt lin_point(Pt pt1, Pt pt2, double t) {
    Pt pt = pt1;
    double w1 = 1.0 - t;
    double x1 = (double(256) * pt1.x + pt1.xf), y1 = (double(256) * pt1.y + pt1.yf);
    double x2 = (double(256) * pt2.x + pt2.xf), y2 = (double(256) * pt2.y + pt2.yf);
    double xx = (w1 * x1 + (1.0 - w1) * x2), yy = (w1 * y1 + (1.0 - w1) * y2);
    pt.x = (uint16_t)(xx / double(256)); pt.xf = (uint8_t)(xx - (pt.x * 256));
    pt.y = (uint16_t)(yy / double(256)); pt.yf = (uint8_t)(yy - (pt.y * 256));
    return pt;
}
// The cyclic spline of column col through every key frame at global time
// (morph.cpp:526-531, spline.cpp:45-57), split as the reference splits it.
Pt spline_point(const orc_scene &s, uint64_t N, uint64_t col, double time, Pt pt, std::vector<double> &sx,
                std::vector<double> &sy) {
    const uint32_t h = s.K;
    for (uint32_t j = 0; j < h; ++j) {
        Pt q = unpack(s.pts[(uint64_t)j * N + col]);
        sx[j] = q.x + q.xf / double(256);
        sy[j] = q.y + q.yf / double(256);
    }
    double vx, vy, ix, iy;
    spline_eval(sx.data(), sy.data(), (int)h, time, &vx, &vy);
    double fx = std::modf(vx, &ix), fy = std::modf(vy, &iy);
    // double -> uint16/uint8 as the x86 build converts: via int.
    pt.x = (uint16_t)(int)ix; pt.xf = (uint8_t)(int)std::round(fx * 255);
    pt.y = (uint16_t)(int)iy; pt.yf = (uint8_t)(int)std::round(fy * 255);
    return pt;
}
// pt displaced by the motion perturbation of an atom whose pair's first
// point is pt1 (FP64 noise when fp64).
Pt perturbed(const orc_scene &s, const NoiseMaps &nm, Pt pt, Pt pt1, double t, bool fp64) {
    if (!(s.motion_noise > 0.0)) return pt;
    int32_t dx, dy;
    motion_offset(nm.mx, nm.my, nm.mx64, nm.my64, s.bbox, s.motion_noise, t, pt1, fp64, &dx, &dy);
    const int32_t X = displaced((int32_t)pt.x * 256 + pt.xf, dx), Y = displaced((int32_t)pt.y * 256 + pt.yf, dy);
    pt.x = (uint16_t)(X >> 8); pt.xf = (uint8_t)(X & 255);
    pt.y = (uint16_t)(Y >> 8); pt.yf = (uint8_t)(Y & 255);
    return pt;
}

// The atom's point at local time t of pair y (global time `time`): the
// motion's position (LINEAR morph.cpp:1501-1515, SPLINE morph.cpp:526-531,
// NONE the first point) plus the motion perturbation when it is on (FP64
// noise when fp64, for the accuracy comparison).  col = the atom's column in
// the frame-major point array.
Pt atom_point(const orc_scene &s, const NoiseMaps &nm, uint32_t y, uint64_t N, uint64_t col, double t, double time,
              bool fp64, std::vector<double> &sx, std::vector<double> &sy) {
    const uint32_t yn = (y + 1) % s.K;
    const Pt pt1 = unpack(s.pts[(uint64_t)y * N + col]);
    const Pt pt2 = unpack(s.pts[(uint64_t)yn * N + col]);
    Pt pt = pt1;
    if (s.motion == LINEAR) pt = lin_point(pt1, pt2, t);
    else if (s.motion == SPLINE) pt = spline_point(s, N, col, time, pt1, sx, sy);
    return perturbed(s, nm, pt, pt1, t, fp64);
}

// Per-blob pixel list at local time t (morph.cpp:452-623, feather 0).
void blob_pixels(const orc_scene &s, const Perlin &lag_map, const Perlin &slope_map, const NoiseMaps &nm,
                 uint32_t group, uint32_t y, double t, double time, std::vector<Px> &out) {
    uint64_t N = 0, off = 0;
    for (uint32_t c = 0; c < s.C; ++c) {
        if (c == group) off = N;
        N += s.widths[c];
    }
    uint64_t w = s.widths[group];
    uint32_t h = s.K;
    uint32_t yn = (y + 1) % h;
    uint32_t bx1 = s.bbox[0], by1 = s.bbox[1], bx2 = s.bbox[2], by2 = s.bbox[3];
    std::map<size_t, std::vector<Col>> colors;
    std::map<size_t, std::vector<double>> weights;
    std::vector<double> sx(h), sy(h);
    for (uint64_t x = 0; x < w; ++x) {
        Pt pt1 = unpack(s.pts[(uint64_t)y * N + off + x]);
        Pt pt2 = unpack(s.pts[(uint64_t)yn * N + off + x]);
        bool h1 = pt1.flags & HAS_PIXEL, h2 = pt2.flags & HAS_PIXEL;
        if (!h1 && !h2) continue;
        Col c1, c2;
        if (h1 && !h2) { c1 = read_pixel(s, y, pt1.x, pt1.y); c2 = c1; c2.a = 0; }
        else if (h2 && !h1) { c2 = read_pixel(s, yn, pt2.x, pt2.y); c1 = c2; c1.a = 0; }
        else { c1 = read_pixel(s, y, pt1.x, pt1.y); c2 = read_pixel(s, yn, pt2.x, pt2.y); }

        Pt pt = atom_point(s, nm, y, N, off + x, t, time, false, sx, sy);
        Px px;
        px.x = pt.x;
        px.y = pt.y;
        if (s.fading == PERLIN) {
            double f = 8.0;
            double bw = bx2 - bx1 + 1.0, bh = by2 - by1 + 1.0;
            double perlin_x = (((pt1.x - (int)bx1) * 256 + pt1.xf) / double(bw * 256)) * f;
            double perlin_y = (((pt1.y - (int)by1) * 256 + pt1.yf) / double(bh * 256)) * f;
            double lag = lag_map.octave(perlin_x, perlin_y, 8) * 0.5 + 0.5;
            double slope = slope_map.octave(perlin_x, perlin_y, 8) * 0.5 + 0.5;
            px.c = ramp_col(c1, c2, lag, slope, 1.0 - t);
        } else if (s.fading == COSINE) {
            px.c = ramp_col(c1, c2, 0.5, 0.5, 1.0 - t);
        } else {
            px.c = lerp_col(c1, c2, 1.0 - t);
        }
        if (px.x >= s.width || px.y >= s.height) {
            if (px.x > bx2 || px.x < bx1 || px.y > by2 || px.y < by1) continue;
        }
        double tw = 255 * 255;
        double w11 = ((255 - pt.xf) * (255 - pt.yf)) / tw;
        double w21 = (pt.xf * (255 - pt.yf)) / tw;
        double w12 = ((255 - pt.xf) * pt.yf) / tw;
        double w22 = (pt.xf * pt.yf) / tw;
        auto pos = [](uint32_t xx, uint32_t yy) { return (size_t)yy * 65536 + xx; };
        if (w11 > 0.0) { colors[pos(px.x, px.y)].push_back(px.c); weights[pos(px.x, px.y)].push_back(w11); }
        if ((px.x < bx2 || px.x + 1 < (int)s.width) && w21 > 0.0) {
            size_t q = pos((uint16_t)(px.x + 1), px.y);
            colors[q].push_back(px.c); weights[q].push_back(w21);
        }
        if ((px.y < by2 || px.y + 1 < (int)s.height) && w12 > 0.0) {
            size_t q = pos(px.x, (uint16_t)(px.y + 1));
            colors[q].push_back(px.c); weights[q].push_back(w12);
        }
        if (w22 > 0.0) {
            if ((px.y < by2 && px.x < bx2) || (px.y + 1 < (int)s.height && px.x + 1 < (int)s.width)) {
                size_t q = pos((uint16_t)(px.x + 1), (uint16_t)(px.y + 1));
                colors[q].push_back(px.c); weights[q].push_back(w22);
            }
        }
    }
    for (auto &kv : colors) {
        std::vector<Col> &cs = kv.second;
        std::vector<double> &ws = weights[kv.first];
        double r = 0, g = 0, b = 0, a = 0, wsum = 0;
        for (size_t i = 0; i < cs.size(); ++i) {
            wsum += ws[i];
            r += cs[i].r * ws[i]; g += cs[i].g * ws[i]; b += cs[i].b * ws[i]; a += cs[i].a * ws[i];
        }
        double dw = s.density > 0 ? double(cs.size()) / double(s.density) : 0.0;
        if (dw > 1.0) dw = 1.0;
        r = std::round(r / wsum); g = std::round(g / wsum); b = std::round(b / wsum); a = std::round(dw * (a / wsum));
        Px px;
        px.x = (uint16_t)(kv.first % 65536);
        px.y = (uint16_t)(kv.first / 65536);
        px.c = Col{(uint8_t)r, (uint8_t)g, (uint8_t)b, (uint8_t)a};
        out.push_back(px);
    }
    if (s.feather == 0) return;
    // Feather (morph.cpp:625-674): peel the blob's 4-neighbour border up to
    // `feather` times; layer l's alpha scales by (l + 1) / (feather + 1).
    std::map<size_t, Col> blob;
    for (const Px &p : out) blob[(size_t)p.y * 65536 + p.x] = p.c;
    std::map<size_t, Col> peeled = blob;
    std::vector<std::set<size_t>> layers;
    while (!peeled.empty() && layers.size() < s.feather) {
        std::set<size_t> border;
        for (auto &kv : peeled) {
            const size_t pos = kv.first;
            const uint32_t x = (uint32_t)(pos % 65536), y = (uint32_t)(pos / 65536);
            if (x == 0 || x == 65535 || y == 0 || y == 65535) { border.insert(pos); continue; }
            if (!peeled.count(pos + 1) || !peeled.count(pos - 1) || !peeled.count(pos + 65536) ||
                !peeled.count(pos - 65536))
                border.insert(pos);
        }
        for (size_t pos : border) peeled.erase(pos);
        layers.push_back(border);
    }
    out.clear();
    for (size_t l = 0; l < layers.size(); ++l)
        for (size_t pos : layers[l]) {
            Px px;
            px.x = (uint16_t)(pos % 65536);
            px.y = (uint16_t)(pos / 65536);
            px.c = blob[pos];
            px.c.a = (uint8_t)std::round(double(px.c.a) * (double(l + 1) / double(s.feather + 1)));
            out.push_back(px);
        }
    for (auto &kv : peeled) {
        Px px;
        px.x = (uint16_t)(kv.first % 65536);
        px.y = (uint16_t)(kv.first / 65536);
        px.c = kv.second;
        out.push_back(px);
    }
}

// morph::get_background (morph.cpp:1431-1465): the key frames' colours at
// (x, y) cross-faded with the frame's fading (Perlin at the pixel itself).
Col background(const orc_scene &s, const Perlin &lag_map, const Perlin &slope_map, uint32_t x, uint32_t y, size_t f,
               double t) {
    const size_t fn = (f + 1) % s.K;
    const Col c1 = read_pixel(s, (uint32_t)f, x, y), c2 = read_pixel(s, (uint32_t)fn, x, y);
    if (s.fading == PERLIN) {
        const double bw = s.bbox[2] - s.bbox[0] + 1.0, bh = s.bbox[3] - s.bbox[1] + 1.0;
        const double px = ((int)x - (int)s.bbox[0]) / bw * 8.0, py = ((int)y - (int)s.bbox[1]) / bh * 8.0;
        const double lag = lag_map.octave(px, py, 8) * 0.5 + 0.5, slope = slope_map.octave(px, py, 8) * 0.5 + 0.5;
        return ramp_col(c1, c2, lag, slope, 1.0 - t);
    }
    if (s.fading == COSINE) return ramp_col(c1, c2, 0.5, 0.5, 1.0 - t);
    return lerp_col(c1, c2, 1.0 - t);
}

// show_blobs == DISTINCT colour of a group (morph.cpp:1322-1328).
Col distinct_colour(size_t group) {
    std::mt19937 gen((unsigned)group);
    std::uniform_int_distribution<unsigned char> d(0, 255);
    Col c;
    c.r = d(gen);
    c.g = d(gen);
    c.b = d(gen);
    c.a = 255;
    return c;
}

void render_one(const orc_scene &s, const Perlin &lag_map, const Perlin &slope_map, const NoiseMaps &nm,
                double time_in, uint8_t *out) {
    size_t npx = (size_t)s.width * s.height;
    std::memset(out, 0, npx * 4);
    if (s.K == 0 || s.C == 0) return;
    // normalize_time + get_frame_key (morph.cpp:404-450).
    double integ;
    double time = std::modf(time_in, &integ);
    if (time < 0.0) time += 1.0;
    size_t f = (size_t)(time * s.K);
    if (f >= s.K) return;
    double dt = 1.0 / double(s.K);
    double t = std::max(0.0, (time - (double)(s.frame_keys[f] * dt)) / dt);
    if (s.keep_background)
        for (uint32_t y = 0; y < s.height; ++y)
            for (uint32_t x = 0; x < s.width; ++x) {
                const Col c = background(s, lag_map, slope_map, x, y, f, t);
                uint8_t *d = out + ((size_t)y * s.width + x) * 4;
                d[0] = c.r; d[1] = c.g; d[2] = c.b; d[3] = c.a;
            }
    std::map<size_t, std::vector<Col>> comp;
    std::vector<Px> pix;
    for (uint32_t b = 0; b < s.C; ++b) {
        pix.clear();
        const uint32_t group = (uint32_t)s.blob_order[(size_t)f * s.C + b];
        blob_pixels(s, lag_map, slope_map, nm, group, (uint32_t)f, t, time, pix);
        // draw_atoms (morph.cpp:1313-1345): TEXTURE, AVERAGE (blob2pixel,
        // morph.cpp:1423-1429) or DISTINCT colours.
        Col ave{0, 0, 0, 0};
        if (s.show_blobs == 1 && s.blob_avg) {
            ave = col_of(s.blob_avg[(size_t)f * s.C + b]);
            if (s.delimiter == HSP) ave = to_rgb(ave);
        }
        const Col dis = distinct_colour(group);
        for (size_t i = pix.size(); i-- > 0;) {
            Px px = pix[i];
            size_t pos = (size_t)px.y * s.width + px.x;
            if (pos >= npx) continue;
            const Col c = s.show_blobs == 2 ? dis : (s.show_blobs == 1 ? ave : px.c);
            if (c.a == 0) continue;
            comp[pos].push_back(c);
        }
    }
    // Ordered "over" composite (morph.cpp:1348-1402), no blend/background.
    for (auto &kv : comp) {
        double r = 0, g = 0, b = 0, a = 0;
        for (size_t c = 0; c < kv.second.size(); ++c) {
            Col q = kv.second[c];
            double sr = q.r / 255.0, sg = q.g / 255.0, sb = q.b / 255.0, sa = q.a / 255.0;
            if (c == 0) { r = sr; g = sg; b = sb; a = sa; }
            else {
                r = sa * sr + (1.0 - sa) * r;
                g = sa * sg + (1.0 - sa) * g;
                b = sa * sb + (1.0 - sa) * b;
                a = a + (1.0 - a) * (q.a / 255.0);
            }
        }
        uint8_t *d = out + kv.first * 4;
        if (s.keep_background) {
            // morph.cpp:1387-1399
            const double bgr = d[0] / 255.0, bgg = d[1] / 255.0, bgb = d[2] / 255.0, bga = d[3] / 255.0;
            r = a * r + (1.0 - a) * bgr;
            g = a * g + (1.0 - a) * bgg;
            b = a * b + (1.0 - a) * bgb;
            a = bga + (1.0 - bga) * a;
        }
        Col o = make_col(r, g, b, a);
        d[0] = o.r; d[1] = o.g; d[2] = o.b; d[3] = o.a;
    }
}

}  // namespace

extern "C" {

// Renders one frame at time t into width*height*4 bytes (morph.cpp:1405-1421,
// fluid off).  Supports motion NONE/LINEAR/SPLINE, fading
// NONE/LINEAR/COSINE/PERLIN, TEXTURE/AVERAGE/DISTINCT blobs, feather and
// keep_background (blend_blobs has no setter in the reference and stays off).
void orc_render(const orc_scene *s, double t, uint8_t *out) {
    Perlin lag(s->seed), slope(s->seed + 1);
    const NoiseMaps nm(s->seed);
    render_one(*s, lag, slope, nm, t, out);
}

// Renders n frames with up to `threads` host threads (frames are
// independent); out holds n consecutive frames.
void orc_render_many(const orc_scene *s, const double *ts, uint32_t n, uint8_t *out, uint32_t threads) {
    Perlin lag(s->seed), slope(s->seed + 1);
    const NoiseMaps nm(s->seed);
    size_t fsz = (size_t)s->width * s->height * 4;
    if (threads <= 1) {
        for (uint32_t i = 0; i < n; ++i) render_one(*s, lag, slope, nm, ts[i], out + i * fsz);
        return;
    }
    std::vector<std::thread> pool;
    for (uint32_t w = 0; w < threads; ++w)
        pool.emplace_back([&, w]() {
            for (uint32_t i = w; i < n; i += threads) render_one(*s, lag, slope, nm, ts[i], out + i * fsz);
        });
    for (auto &th : pool) th.join();
}

// Every atom's point at time t (global time, as orc_render takes it) as two
// position words (integer part * 256 + fraction byte) per column of the
// frame-major point array; -1, -1 where the atom is drawn at neither key
// frame of its pair.  fp64 selects the FP64 noise (the accuracy reference of
// the motion perturbation) instead of its FP32 definition.
void orc_positions(const orc_scene *sp, double time_in, int fp64, int32_t *xy) {
    const orc_scene &s = *sp;
    uint64_t N = 0;
    for (uint32_t c = 0; c < s.C; ++c) N += s.widths[c];
    if (s.K == 0 || N == 0) return;
    double integ;
    double time = std::modf(time_in, &integ);
    if (time < 0.0) time += 1.0;
    const size_t f = std::min<size_t>((size_t)(time * s.K), s.K - 1);
    const double dt = 1.0 / double(s.K);
    const double t = std::max(0.0, (time - (double)(s.frame_keys[f] * dt)) / dt);
    const NoiseMaps nm(s.seed);
    std::vector<double> sx(s.K), sy(s.K);
    const uint32_t y = (uint32_t)f, yn = (y + 1) % s.K;
    for (uint64_t col = 0; col < N; ++col) {
        const Pt p1 = unpack(s.pts[(uint64_t)y * N + col]), p2 = unpack(s.pts[(uint64_t)yn * N + col]);
        if (!(p1.flags & HAS_PIXEL) && !(p2.flags & HAS_PIXEL)) {
            xy[2 * col] = xy[2 * col + 1] = -1;
            continue;
        }
        const Pt pt = atom_point(s, nm, y, N, col, t, time, fp64 != 0, sx, sy);
        xy[2 * col] = (int32_t)pt.x * 256 + pt.xf;
        xy[2 * col + 1] = (int32_t)pt.y * 256 + pt.yf;
    }
}

// morph::get_pixels(blob, t, to) (morph.cpp:452-678) of the blob-th blob of
// the key frame at time t (global time, as orc_render takes it): up to cap
// pixels into xy / rgba in the reference's order; returns the list's length
// (SIZE_MAX when the blob does not exist).
size_t orc_blob_pixels(const orc_scene *sp, size_t blob, double time_in, uint16_t *xy, uint8_t *rgba, size_t cap) {
    const orc_scene &s = *sp;
    if (s.K == 0 || s.C == 0 || blob >= s.C) return SIZE_MAX;
    double integ;
    double time = std::modf(time_in, &integ);
    if (time < 0.0) time += 1.0;
    const size_t f = std::min<size_t>((size_t)(time * s.K), s.K - 1);
    const double dt = 1.0 / double(s.K);
    const double t = std::max(0.0, (time - (double)(s.frame_keys[f] * dt)) / dt);
    Perlin lag(s.seed), slope(s.seed + 1);
    const NoiseMaps nm(s.seed);
    std::vector<Px> pix;
    blob_pixels(s, lag, slope, nm, (uint32_t)s.blob_order[f * s.C + blob], (uint32_t)f, t, time, pix);
    for (size_t i = 0; i < pix.size() && i < cap; ++i) {
        xy[2 * i] = pix[i].x;
        xy[2 * i + 1] = pix[i].y;
        rgba[4 * i] = pix[i].c.r; rgba[4 * i + 1] = pix[i].c.g; rgba[4 * i + 2] = pix[i].c.b; rgba[4 * i + 3] = pix[i].c.a;
    }
    return pix.size();
}

// update_particle's gravity target and ideal colour (morph.cpp:697-767,
// TEXTURE blobs) of n particles of the fluid frame at time `time` (global),
// given the source and destination column each one read (src_x after the
// growing-area rule, dst_x) and the surfaces s0, s1 of its chain's blobs at
// the pair's two key frames: out[6 i ..] = gravity x, y in grid units
// (sparseness grid units per pixel, 10 of margin), R, G, B, A in 0..1.
void orc_fluid_targets(const orc_scene *sp, double time_in, double sparseness, uint32_t n, const uint32_t *src,
                       const uint32_t *dst, const double *s0, const double *s1, double *out) {
    const orc_scene &s = *sp;
    uint64_t N = 0;
    for (uint32_t c = 0; c < s.C; ++c) N += s.widths[c];
    double integ;
    double time = std::modf(time_in, &integ);
    if (time < 0.0) time += 1.0;
    const size_t f = std::min<size_t>((size_t)(time * s.K), s.K - 1);
    const double dt = 1.0 / double(s.K);
    const double t = std::max(0.0, (time - (double)(s.frame_keys[f] * dt)) / dt);
    const uint32_t y = (uint32_t)f, yn = (y + 1) % s.K;
    Perlin lag_map(s.seed), slope_map(s.seed + 1);
    const NoiseMaps nm(s.seed);
    std::vector<double> sx(s.K), sy(s.K);
    const double bx1 = s.bbox[0], by1 = s.bbox[1], bw = s.bbox[2] - s.bbox[0] + 1.0, bh = s.bbox[3] - s.bbox[1] + 1.0;
    for (uint32_t i = 0; i < n; ++i) {
        const Pt pt1 = unpack(s.pts[(uint64_t)y * N + src[i]]), pt2 = unpack(s.pts[(uint64_t)yn * N + dst[i]]);
        const bool h1 = pt1.flags & HAS_PIXEL, h2 = pt2.flags & HAS_PIXEL;
        Col c1, c2;
        if (h1 && !h2) {
            c1 = read_pixel(s, y, pt1.x, pt1.y);
            c2 = c1;
            if (s1[i] > 0.0) c2.a = 0;
        } else if (h2 && !h1) {
            c2 = read_pixel(s, yn, pt2.x, pt2.y);
            c1 = c2;
            if (s0[i] > 0.0) c1.a = 0;
        } else {
            c1 = read_pixel(s, y, pt1.x, pt1.y);
            c2 = read_pixel(s, yn, pt2.x, pt2.y);
        }
        Col c;
        if (s.fading == PERLIN) {
            const double px = (((pt1.x - bx1) * 256 + pt1.xf) / double(bw * 256)) * 8.0;
            const double py = (((pt1.y - by1) * 256 + pt1.yf) / double(bh * 256)) * 8.0;
            c = ramp_col(c1, c2, lag_map.octave(px, py, 8) * 0.5 + 0.5, slope_map.octave(px, py, 8) * 0.5 + 0.5, 1.0 - t);
        } else if (s.fading == COSINE) {
            c = ramp_col(c1, c2, 0.5, 0.5, 1.0 - t);
        } else {
            c = lerp_col(c1, c2, 1.0 - t);
        }
        Pt pt = pt1;
        if (s.motion == LINEAR) pt = lin_point(pt1, pt2, t);
        else if (s.motion == SPLINE) pt = spline_point(s, N, src[i], time, pt1, sx, sy);
        pt = perturbed(s, nm, pt, pt1, t, false);
        // point2xy (atomorph.h:315-318) in float
        const float ptx = pt.x + pt.xf / float(256), pty = pt.y + pt.yf / float(256);
        double *o = out + 6 * (size_t)i;
        o[0] = std::min(std::max((ptx * sparseness) + 10.0, 1.0), double(s.width * sparseness + 10.0));
        o[1] = std::min(std::max((pty * sparseness) + 10.0, 1.0), double(s.height * sparseness + 10.0));
        o[2] = c.r / 255.0;
        o[3] = c.g / 255.0;
        o[4] = c.b / 255.0;
        o[5] = c.a / 255.0;
    }
}

// ------------------------------------------------------------ fluid step ---
// FluidModel::step (fluidmodel.cpp:165-580) restated on structure-of-arrays
// particles.  Particle fields per index i: x y u v gravity_x gravity_y
// freedom_r active mature strength R G B A r g b a (18 arrays of doubles in
// `P`, P[f*n + i]).  The grid has gx*gy nodes; the caller keeps one
// orc_fluid_grid buffer of 13*gx*gy doubles plus one byte per node alive
// across steps (nodes touched in one step are cleared at the start of the
// next, as the reference's active list does).  Wall jitter uses rand(), as the
// reference does.
enum { FX, FY, FU, FV, FGX, FGY, FFR, FACT, FMAT, FSTR, FR_, FG_, FB_, FA_, Fr, Fg, Fb, Fa, NFIELD };
enum { NM, ND, NGX, NGY, NU, NV, NAX, NAY, NR, NG, NB, NA, NW, NNODE };

void orc_fluid_step(double *P, uint32_t n, uint32_t gsx, uint32_t gsy, double *grid, uint8_t *touched,
                    uint64_t steps_left, double freedom_radius) {
    size_t G = (size_t)gsx * gsy;
    auto F = [&](int f, uint32_t i) -> double & { return P[(size_t)f * n + i]; };
    auto NDf = [&](int f, size_t node) -> double & { return grid[(size_t)f * G + node]; };
    for (size_t q = 0; q < G; ++q)
        if (touched[q]) {
            for (int f = 0; f < NNODE; ++f) NDf(f, q) = 0.0;
            touched[q] = 0;
        }
    std::vector<unsigned> pcx(n), pcy(n);
    std::vector<double> ppx(3 * (size_t)n), ppy(3 * (size_t)n), pgx(3 * (size_t)n), pgy(3 * (size_t)n);
    const double mass = 1.0;
    for (uint32_t i = 0; i < n; ++i) {
        if (F(FACT, i) == 0.0) continue;
        double px = F(FX, i), py = F(FY, i);
        pcx[i] = (unsigned)(int)(px - 0.5);
        pcy[i] = (unsigned)(int)(py - 0.5);
        double x = pcx[i] - px;
        double *ax = &ppx[3 * i], *gx = &pgx[3 * i], *ay = &ppy[3 * i], *gy = &pgy[3 * i];
        ax[0] = (0.5 * x * x + 1.5 * x + 1.125); gx[0] = (x + 1.5); x += 1.0;
        ax[1] = (-x * x + 0.75); gx[1] = (-2.0 * x); x += 1.0;
        ax[2] = (0.5 * x * x - 1.5 * x + 1.125); gx[2] = (x - 1.5);
        double y = pcy[i] - py;
        ay[0] = (0.5 * y * y + 1.5 * y + 1.125); gy[0] = (y + 1.5); y += 1.0;
        ay[1] = (-y * y + 0.75); gy[1] = (-2.0 * y); y += 1.0;
        ay[2] = (0.5 * y * y - 1.5 * y + 1.125); gy[2] = (y - 1.5);
        bool mature = F(FMAT, i) != 0.0;
        double str = F(FSTR, i);
        for (unsigned a = 0; a < 3; ++a)
            for (unsigned b = 0; b < 3; ++b) {
                size_t q = (size_t)(pcx[i] + a) * gsy + pcy[i] + b;
                touched[q] = 1;
                double phi = ax[a] * ay[b];
                NDf(NM, q) += phi * mass;
                NDf(ND, q) += phi;
                NDf(NGX, q) += gx[a] * ay[b];
                NDf(NGY, q) += ax[a] * gy[b];
                if (mature && str > 0.0) {
                    double nw = str, ow = NDf(NW, q), sw = nw + ow;
                    NDf(NR, q) = (ow * NDf(NR, q) + nw * F(Fr, i)) / sw;
                    NDf(NG, q) = (ow * NDf(NG, q) + nw * F(Fg, i)) / sw;
                    NDf(NB, q) = (ow * NDf(NB, q) + nw * F(Fb, i)) / sw;
                    NDf(NA, q) = (ow * NDf(NA, q) + nw * F(Fa, i)) / sw;
                    NDf(NW, q) = sw;
                }
            }
    }
    for (uint32_t i = 0; i < n; ++i) {
        if (F(FACT, i) == 0.0) continue;
        double px = F(FX, i), py = F(FY, i);
        unsigned cx = (unsigned)(int)px, cy = (unsigned)(int)py, cxi = cx + 1, cyi = cy + 1;
        size_t n01 = (size_t)cx * gsy + cy, n02 = (size_t)cx * gsy + cyi, n11 = (size_t)cxi * gsy + cy,
               n12 = (size_t)cxi * gsy + cyi;
        double pdx = NDf(ND, n11) - NDf(ND, n01);
        double pdy = NDf(ND, n02) - NDf(ND, n01);
        double C20 = 3.0 * pdx - NDf(NGX, n11) - 2.0 * NDf(NGX, n01);
        double C02 = 3.0 * pdy - NDf(NGY, n02) - 2.0 * NDf(NGY, n01);
        double C30 = -2.0 * pdx + NDf(NGX, n11) + NDf(NGX, n01);
        double C03 = -2.0 * pdy + NDf(NGY, n02) + NDf(NGY, n01);
        double csum1 = NDf(ND, n01) + NDf(NGY, n01) + C02 + C03;
        double csum2 = NDf(ND, n01) + NDf(NGX, n01) + C20 + C30;
        double C21 = 3.0 * NDf(ND, n12) - 2.0 * NDf(NGX, n02) - NDf(NGX, n12) - 3.0 * csum1 - C20;
        double C31 = -2.0 * NDf(ND, n12) + NDf(NGX, n02) + NDf(NGX, n12) + 2.0 * csum1 - C30;
        double C12 = 3.0 * NDf(ND, n12) - 2.0 * NDf(NGY, n11) - NDf(NGY, n12) - 3.0 * csum2 - C02;
        double C13 = -2.0 * NDf(ND, n12) + NDf(NGY, n11) + NDf(NGY, n12) + 2.0 * csum2 - C03;
        double C11 = NDf(NGX, n02) - C13 - C12 - NDf(NGX, n01);
        double u = px - cx, u2 = u * u, u3 = u * u2;
        double v = py - cy, v2 = v * v, v3 = v * v2;
        double density = NDf(ND, n01) + NDf(NGX, n01) * u + NDf(NGY, n01) * v + C20 * u2 + C02 * v2 + C30 * u3 +
                         C03 * v3 + C21 * u2 * v + C31 * u3 * v + C12 * u * v2 + C13 * u * v3 + C11 * u * v;
        double pressure = density - 1.0;
        if (pressure > 2.0) pressure = 2.0;
        double fx = 0.0, fy = 0.0;
        if (px < 4.0) fx += mass * (4.0 - px);
        else if (px > gsx - 5) fx += mass * (gsx - 5 - px);
        if (py < 4.0) fy += mass * (4.0 - py);
        else if (py > gsy - 5) fy += mass * (gsy - 5 - py);
        double *ax = &ppx[3 * i], *gx = &pgx[3 * i], *ay = &ppy[3 * i], *gy = &pgy[3 * i];
        for (unsigned a = 0; a < 3; ++a)
            for (unsigned b = 0; b < 3; ++b) {
                size_t q = (size_t)(pcx[i] + a) * gsy + pcy[i] + b;
                double phi = ax[a] * ay[b];
                NDf(NAX, q) += -((gx[a] * ay[b]) * pressure) + fx * phi;
                NDf(NAY, q) += -((ax[a] * gy[b]) * pressure) + fy * phi;
            }
    }
    for (size_t q = 0; q < G; ++q)
        if (touched[q] && NDf(NM, q) > 0.0) { NDf(NAX, q) /= NDf(NM, q); NDf(NAY, q) /= NDf(NM, q); }
    for (uint32_t i = 0; i < n; ++i) {
        if (F(FACT, i) == 0.0) continue;
        double *ax = &ppx[3 * i], *ay = &ppy[3 * i];
        for (unsigned a = 0; a < 3; ++a)
            for (unsigned b = 0; b < 3; ++b) {
                size_t q = (size_t)(pcx[i] + a) * gsy + pcy[i] + b;
                double phi = ax[a] * ay[b];
                double cax = 0.0, cay = 0.0;
                {
                    double x1 = F(FX, i), y1 = F(FY, i), x2 = F(FGX, i), y2 = F(FGY, i), acc = 0.03;
                    double A = std::abs(y1 - y2), B = std::abs(x1 - x2), Cc = std::sqrt(A * A + B * B);
                    if (acc >= Cc) acc = Cc;
                    if (B <= 0.0) { if (y2 <= y1) cay -= acc; else cay += acc; }
                    else if (Cc > 0.0) {
                        double dx = (acc * B) / Cc, dy = (A * dx) / B;
                        if (x1 <= x2) cax += dx; else cax -= dx;
                        if (y1 <= y2) cay += dy; else cay -= dy;
                    }
                }
                F(FU, i) += phi * (NDf(NAX, q) + cax);
                F(FV, i) += phi * (NDf(NAY, q) + cay);
            }
        double mu = mass * F(FU, i), mv = mass * F(FV, i);
        if (F(FMAT, i) == 0.0) { mu *= 0.0; mv *= 0.0; }
        for (unsigned a = 0; a < 3; ++a)
            for (unsigned b = 0; b < 3; ++b) {
                size_t q = (size_t)(pcx[i] + a) * gsy + pcy[i] + b;
                double phi = ax[a] * ay[b];
                NDf(NU, q) += phi * mu;
                NDf(NV, q) += phi * mv;
            }
    }
    for (size_t q = 0; q < G; ++q)
        if (touched[q] && NDf(NM, q) > 0.0) { NDf(NU, q) /= NDf(NM, q); NDf(NV, q) /= NDf(NM, q); }
    for (uint32_t i = 0; i < n; ++i) {
        if (F(FACT, i) == 0.0) continue;
        double nR = 0, nG = 0, nB = 0, nA = 0, wsum = 0, gu = 0, gv = 0;
        double *ax = &ppx[3 * i], *ay = &ppy[3 * i];
        for (unsigned a = 0; a < 3; ++a)
            for (unsigned b = 0; b < 3; ++b) {
                size_t q = (size_t)(pcx[i] + a) * gsy + pcy[i] + b;
                double phi = ax[a] * ay[b];
                gu += phi * NDf(NU, q);
                gv += phi * NDf(NV, q);
                double nw = NDf(NW, q);
                if (nw > 0.0) {
                    wsum += nw;
                    nR += NDf(NR, q) * nw; nG += NDf(NG, q) * nw; nB += NDf(NB, q) * nw; nA += NDf(NA, q) * nw;
                }
            }
        if (wsum > 0.0) {
            nR /= wsum; double wr = std::abs(nR - F(FR_, i));
            nG /= wsum; double wg = std::abs(nG - F(FG_, i));
            nB /= wsum; double wb = std::abs(nB - F(FB_, i));
            nA /= wsum; double wa = std::abs(nA - F(FA_, i));
            if (F(FMAT, i) == 0.0) { F(Fr, i) = nR; F(Fg, i) = nG; F(Fb, i) = nB; F(Fa, i) = nA; }
            else {
                F(Fr, i) = (1.0 - wr) * F(Fr, i) + wr * nR;
                F(Fg, i) = (1.0 - wg) * F(Fg, i) + wg * nG;
                F(Fb, i) = (1.0 - wb) * F(Fb, i) + wb * nB;
                F(Fa, i) = (1.0 - wa) * F(Fa, i) + wa * nA;
            }
        }
        F(FX, i) += gu;
        F(FY, i) += gv;
        {
            double x1 = F(FX, i), y1 = F(FY, i), x2 = F(FGX, i), y2 = F(FGY, i);
            double A = std::abs(y1 - y2), B = std::abs(x1 - x2), Cc = std::sqrt(A * A + B * B);
            double r = freedom_radius * F(FFR, i);
            if (Cc > r) {
                double mx = 0.0, my = 0.0, acc = Cc - r;
                if (acc >= Cc) acc = Cc;
                if (B <= 0.0) { if (y2 <= y1) my -= acc; else my += acc; }
                else if (Cc > 0.0) {
                    double dx = (acc * B) / Cc, dy = (A * dx) / B;
                    if (x1 <= x2) mx += dx; else mx -= dx;
                    if (y1 <= y2) my += dy; else my -= dy;
                }
                double w = 1.0 / (steps_left + 1);
                mx *= w; my *= w;
                F(FX, i) += mx; F(FY, i) += my;
            }
        }
        F(FU, i) += gu - F(FU, i);
        F(FV, i) += gv - F(FV, i);
        if (F(FX, i) < 1.0) { F(FX, i) = 1.0 + static_cast<double>(rand()) / RAND_MAX * 0.01; F(FU, i) = 0.0; }
        else if (F(FX, i) > gsx - 2) { F(FX, i) = gsx - 2 - static_cast<double>(rand()) / RAND_MAX * 0.01; F(FU, i) = 0.0; }
        if (F(FY, i) < 1.0) { F(FY, i) = 1.0 + static_cast<double>(rand()) / RAND_MAX * 0.01; F(FV, i) = 0.0; }
        else if (F(FY, i) > gsy - 2) { F(FY, i) = gsy - 2 - static_cast<double>(rand()) / RAND_MAX * 0.01; F(FV, i) = 0.0; }
    }
}
void orc_srand(unsigned s) { srand(s); }

// draw_fluid's colour correction and splat (morph.cpp:1081-1204) of the
// particles P[18][n] (fields as orc_fluid_step) into out (RGBA8 width x
// height, zero where no particle lands).  feather = 0, keep_background off.
// Corners outside the output are dropped like the GPU path (the reference
// would wrap them into the next row).
void orc_draw_fluid_ex(double *P, uint32_t n, uint32_t width, uint32_t height, double sparseness,
                       const uint32_t *bbox, double t, uint32_t feather, const uint8_t *background, uint8_t *out);
void orc_draw_fluid(double *P, uint32_t n, uint32_t width, uint32_t height, double sparseness, const uint32_t *bbox,
                    double t, uint8_t *out) {
    orc_draw_fluid_ex(P, n, width, height, sparseness, bbox, t, 0, nullptr, out);
}

// draw_fluid with feather and keep_background (morph.cpp:1187-1300):
// `background` (RGBA8 width x height, or null for keep_background off) is
// the image get_background prefilled; the fluid's alpha fades by 1 - t^24,
// `feather` layers grow outward (each new pixel the mean of its member
// 4-neighbours, alpha scaled by 1 - (layer + 1) / (feather + 1)), and the
// result is drawn over the background.
void orc_draw_fluid_ex(double *P, uint32_t n, uint32_t width, uint32_t height, double sparseness,
                       const uint32_t *bbox, double t, uint32_t feather, const uint8_t *background, uint8_t *out) {
    auto F = [&](int f, uint32_t i) -> double & { return P[(size_t)f * n + i]; };
    const size_t npx = (size_t)width * height;
    std::vector<double> W(npx, 0.0), R(npx, 0.0), G(npx, 0.0), B(npx, 0.0), A(npx, 0.0);
    std::vector<uint8_t> any(npx, 0);
    auto cc = [](double v) { return (uint32_t)(int)std::round(v * 255.0) & 255u; };  // create_color
    for (uint32_t i = 0; i < n; ++i) {
        if (F(FACT, i) == 0.0) continue;
        const double st = F(FSTR, i), d = t - (1.0 * (1.0 - st));
        const double w = (1.0 / (100.0 * std::pow(d, 2.0) + 1.0)) * std::pow(st, 2.0);
        F(Fr, i) = (w * F(FR_, i)) + (1.0 - w) * F(Fr, i);
        F(Fg, i) = (w * F(FG_, i)) + (1.0 - w) * F(Fg, i);
        F(Fb, i) = (w * F(FB_, i)) + (1.0 - w) * F(Fb, i);
        F(Fa, i) = (w * F(FA_, i)) + (1.0 - w) * F(Fa, i);
        double px, py;
        if (F(FX, i) <= 10.0) px = 0.0;
        else if (F(FX, i) >= width * sparseness + 10.0) px = (double)(width - 1);
        else px = (F(FX, i) - 10.0) / sparseness;
        if (F(FY, i) <= 10.0) py = 0.0;
        else if (F(FY, i) >= height * sparseness + 10.0) py = (double)(height - 1);
        else py = (F(FY, i) - 10.0) / sparseness;
        const uint32_t x = (uint32_t)std::min((int)px, (int)width - 1), y = (uint32_t)std::min((int)py, (int)height - 1);
        F(FMAT, i) = 1.0;
        double ipx, ipy;
        const double xf = std::modf(px, &ipx), yf = std::modf(py, &ipy);
        if (ipx >= width || ipy >= height) {
            if (ipx > bbox[2] || ipx < bbox[0] || ipy > bbox[3] || ipy < bbox[1]) continue;
        }
        const double w11 = (1.0 - xf) * (1.0 - yf), w21 = xf * (1.0 - yf), w12 = (1.0 - xf) * yf, w22 = xf * yf;
        const uint32_t r = cc(F(Fr, i)), g = cc(F(Fg, i)), b = cc(F(Fb, i)), a = cc(F(Fa, i));
        auto put = [&](uint32_t cx, uint32_t cy, double wt) {
            if (cx >= width || cy >= height) return;
            const size_t q = (size_t)cy * width + cx;
            W[q] += wt; R[q] += r * wt; G[q] += g * wt; B[q] += b * wt; A[q] += a * wt;
            any[q] = 1;
        };
        if (w11 > 0.0) put(x, y, w11);
        if ((x < bbox[2] || x + 1 < width) && w21 > 0.0) put(x + 1, y, w21);
        if ((y < bbox[3] || y + 1 < height) && w12 > 0.0) put(x, y + 1, w12);
        if (w22 > 0.0 && ((y < bbox[3] && x < bbox[2]) || (y + 1 < height && x + 1 < width))) put(x + 1, y + 1, w22);
    }
    std::map<size_t, Col> blob;  // fluid pixels by y * 65536 + x
    for (size_t q = 0; q < npx; ++q) {
        if (!any[q]) continue;
        double a = std::round(A[q] / W[q]);
        if (background) a *= 1.0 - std::pow(t, 24.0);
        blob[(q / width) * 65536 + q % width] =
            Col{(uint8_t)std::round(R[q] / W[q]), (uint8_t)std::round(G[q] / W[q]), (uint8_t)std::round(B[q] / W[q]),
                (uint8_t)a};
    }
    for (uint32_t layer = 0; layer < feather; ++layer) {
        const double alpha = 1.0 - (double(layer + 1) / double(feather + 1));
        std::set<size_t> border;
        for (auto &kv : blob) {
            const uint32_t x = (uint32_t)(kv.first % 65536), y = (uint32_t)(kv.first / 65536);
            if (x + 1 < width && !blob.count(kv.first + 1)) border.insert(kv.first + 1);
            if (y + 1 < height && !blob.count(kv.first + 65536)) border.insert(kv.first + 65536);
            if (x > 0 && !blob.count(kv.first - 1)) border.insert(kv.first - 1);
            if (y > 0 && !blob.count(kv.first - 65536)) border.insert(kv.first - 65536);
        }
        if (border.empty()) break;
        std::map<size_t, Col> add;
        for (size_t pos : border) {
            const uint32_t x = (uint32_t)(pos % 65536), y = (uint32_t)(pos / 65536);
            std::set<size_t> comps;
            if (x + 1 < width && blob.count(pos + 1)) comps.insert(pos + 1);
            if (y + 1 < height && blob.count(pos + 65536)) comps.insert(pos + 65536);
            if (x > 0 && blob.count(pos - 1)) comps.insert(pos - 1);
            if (y > 0 && blob.count(pos - 65536)) comps.insert(pos - 65536);
            double r = 0, g = 0, b = 0, a = 0;
            const double w = (double)comps.size();
            for (size_t c : comps) {
                const Col q = blob[c];
                r += (q.r / 255.0) / w; g += (q.g / 255.0) / w; b += (q.b / 255.0) / w; a += (q.a / 255.0) / w;
            }
            a *= alpha;
            add[pos] = make_col(r, g, b, a);
        }
        for (auto &kv : add) blob[kv.first] = kv.second;
    }
    for (size_t q = 0; q < npx; ++q) {
        uint8_t *o = out + 4 * q;
        if (background) std::memcpy(o, background + 4 * q, 4);
        else o[0] = o[1] = o[2] = o[3] = 0;
    }
    for (auto &kv : blob) {
        const size_t q = (kv.first / 65536) * width + kv.first % 65536;
        uint8_t *o = out + 4 * q;
        Col c = kv.second;
        if (background) {
            const double bgr = o[0] / 255.0, bgg = o[1] / 255.0, bgb = o[2] / 255.0, bga = o[3] / 255.0;
            double r = c.r / 255.0, g = c.g / 255.0, b = c.b / 255.0, a = c.a / 255.0;
            r = a * r + (1.0 - a) * bgr;
            g = a * g + (1.0 - a) * bgg;
            b = a * b + (1.0 - a) * bgb;
            a = bga + (1.0 - bga) * a;
            c = Col{(uint8_t)std::round(r * 255.0), (uint8_t)std::round(g * 255.0), (uint8_t)std::round(b * 255.0),
                    (uint8_t)std::round(a * 255.0)};
        }
        o[0] = c.r; o[1] = c.g; o[2] = c.b; o[3] = c.a;
    }
}

// The image get_background fills (morph.cpp:1405-1413) for time t.
void orc_background(const orc_scene *s, double time_in, uint8_t *out) {
    Perlin lag(s->seed), slope(s->seed + 1);
    double integ;
    double time = std::modf(time_in, &integ);
    if (time < 0.0) time += 1.0;
    size_t f = (size_t)(time * s->K);
    const size_t npx = (size_t)s->width * s->height;
    if (s->K == 0 || f >= s->K) { std::memset(out, 0, npx * 4); return; }
    const double dt = 1.0 / double(s->K);
    const double t = std::max(0.0, (time - (double)(s->frame_keys[f] * dt)) / dt);
    for (uint32_t y = 0; y < s->height; ++y)
        for (uint32_t x = 0; x < s->width; ++x) {
            const Col c = background(*s, lag, slope, x, y, f, t);
            uint8_t *d = out + ((size_t)y * s->width + x) * 4;
            d[0] = c.r; d[1] = c.g; d[2] = c.b; d[3] = c.a;
        }
}

// --------------------------------------------------------------- blobs -----
// 4-connected components of the present pixels of one key frame: the blobs
// blobify_frame (thread.cpp:225-412) converges to when blob_threshold >= 1,
// blob_min_size <= 1, blob_max_size >= every component and blob_number <=
// the component count.  Labels are numbered by first pixel in row-major
// order; stats[6*b..] = count, sum x, sum y, sum r, sum g, sum b, sum a of
// the stored colour.  Returns the component count.
uint32_t orc_components(const uint8_t *present, const uint32_t *colors, uint32_t W, uint32_t H, int32_t *labels,
                        double *stats, uint32_t max_blobs) {
    size_t n = (size_t)W * H;
    std::vector<int64_t> parent(n, -1);
    auto find = [&](int64_t a) {
        while (parent[a] != a) { parent[a] = parent[parent[a]]; a = parent[a]; }
        return a;
    };
    for (size_t i = 0; i < n; ++i)
        if (present[i]) parent[i] = (int64_t)i;
    for (uint32_t y = 0; y < H; ++y)
        for (uint32_t x = 0; x < W; ++x) {
            size_t i = (size_t)y * W + x;
            if (!present[i]) continue;
            if (x + 1 < W && present[i + 1]) {
                int64_t a = find(i), b = find(i + 1);
                if (a != b) parent[std::max(a, b)] = std::min(a, b);
            }
            if (y + 1 < H && present[i + W]) {
                int64_t a = find(i), b = find(i + W);
                if (a != b) parent[std::max(a, b)] = std::min(a, b);
            }
        }
    std::vector<int32_t> root_label(n, -1);
    uint32_t count = 0;
    for (size_t i = 0; i < n; ++i) {
        if (!present[i]) { labels[i] = -1; continue; }
        int64_t r = find(i);
        if (root_label[r] < 0) root_label[r] = (int32_t)count++;
        int32_t l = root_label[r];
        labels[i] = l;
        if ((uint32_t)l < max_blobs) {
            double *s = stats + 7 * (size_t)l;
            Col c = col_of(colors[i]);
            s[0] += 1; s[1] += (double)(i % W); s[2] += (double)(i / W);
            s[3] += c.r; s[4] += c.g; s[5] += c.b; s[6] += c.a;
        }
    }
    return count;
}

// blob_distance (thread.cpp:1151-1174) on blob descriptors
// {size, x, y, r, g, b, a} (means; colours 0..1 in the stored space).
double orc_blob_distance(const double *b1, const double *b2, double bbox_d, double w_rgba, double w_size,
                         double w_xy) {
    double sz1 = b1[0], sz2 = b2[0], szs = sz1 + sz2;
    double pix = 0.0, col = 0.0, siz = 0.0;
    if (szs > 0) siz = std::fabs(sz1 - sz2) / szs;
    if (sz1 > 0 && sz2 > 0) {
        // create_pixel truncates x,y to uint16; create_color rounds colours.
        uint16_t x1 = (uint16_t)b1[1], y1 = (uint16_t)b1[2], x2 = (uint16_t)b2[1], y2 = (uint16_t)b2[2];
        int32_t xd = x1 - x2, yd = y1 - y2;
        pix = std::sqrt(double((uint32_t)(xd * xd + yd * yd)) / bbox_d);
        Col c1 = make_col(b1[3], b1[4], b1[5], b1[6]), c2 = make_col(b2[3], b2[4], b2[5], b2[6]);
        col = cdist(c1, c2);
    }
    return w_xy * pix + w_rgba * col + w_size * siz;
}

// Blob-map energy (thread.cpp:1087-1107): blobs[(g*K + k)*7] is the
// descriptor of group g in key frame k; cyclic over key frames.
double orc_blob_energy(const double *blobs, uint32_t Wb, uint32_t K, double bbox_d, double w_rgba, double w_size,
                       double w_xy) {
    double e = 0.0;
    for (uint32_t i = 0; i < Wb; ++i) {
        const double *prev = blobs + ((size_t)i * K + (K - 1)) * 7;
        for (uint32_t j = 0; j < K; ++j) {
            const double *cur = blobs + ((size_t)i * K + j) * 7;
            e += orc_blob_distance(prev, cur, bbox_d, w_rgba, w_size, w_xy);
            prev = cur;
        }
    }
    return e;
}

// Blob matching by random pair swaps (thread.cpp:669-737), restated.
// perm[k*Wb + g] = index of the blob (within key frame k's descriptor list)
// assigned to group g; updated in place.  Runs `steps` proposals with
// std::default_random_engine(seed); returns the final energy.
double orc_blob_match(const double *desc, int32_t *perm, uint32_t Wb, uint32_t K, uint64_t steps, unsigned seed,
                      double bbox_d, double w_rgba, double w_size, double w_xy) {
    std::default_random_engine e1(seed);
    auto D = [&](uint32_t g, uint32_t k) { return desc + ((size_t)k * Wb + perm[(size_t)k * Wb + g]) * 7; };
    auto bd = [&](const double *a, const double *b) { return orc_blob_distance(a, b, bbox_d, w_rgba, w_size, w_xy); };
    if (K > 0 && Wb > 1) {
        std::uniform_int_distribution<size_t> ux(0, Wb - 1), uy(0, K - 1);
        for (uint64_t s = 0; s < steps; ++s) {
            size_t y = uy(e1), yn = (y + 1) % K, yp = (y > 0 ? y - 1 : K - 1);
            size_t x1 = ux(e1), x2;
            do { x2 = ux(e1); } while (x1 == x2);
            if (D(x1, y)[0] == 0 && D(x2, y)[0] == 0) continue;
            double c1 = bd(D(x1, yp), D(x1, y)) + bd(D(x1, y), D(x1, yn)) + bd(D(x2, yp), D(x2, y)) + bd(D(x2, y), D(x2, yn));
            double c2 = bd(D(x2, yp), D(x1, y)) + bd(D(x1, y), D(x2, yn)) + bd(D(x1, yp), D(x2, y)) + bd(D(x2, y), D(x1, yn));
            if (c1 >= c2) std::swap(perm[y * Wb + x1], perm[y * Wb + x2]);
        }
    }
    std::vector<double> flat((size_t)Wb * K * 7);
    for (uint32_t g = 0; g < Wb; ++g)
        for (uint32_t k = 0; k < K; ++k) std::memcpy(&flat[((size_t)g * K + k) * 7], D(g, k), 7 * sizeof(double));
    return orc_blob_energy(flat.data(), Wb, K, bbox_d, w_rgba, w_size, w_xy);
}

// Chain construction (thread.cpp:740-891, fix_volatiles 1187-1233), restated
// for one group: surf[k] lists the sorted surface positions (y*65536+x) of
// the group's blob in key frame k (count cnt[k]); cx/cy hold the blob centres
// (already interpolated for empty blobs).  Writes width*K points frame-major
// into out (out[k*width + x]).  Duplicates draw from
// std::default_random_engine(seed).  Returns width.
uint64_t orc_chain_build(const uint64_t *const *surf, const uint64_t *cnt, const double *cx, const double *cy,
                         uint32_t K, uint32_t density, unsigned seed, uint64_t *out, uint64_t out_cap) {
    uint64_t mx = 0;
    for (uint32_t k = 0; k < K; ++k) mx = std::max(mx, cnt[k]);
    uint64_t width = mx * density;
    if (!out) return width;
    if (width > out_cap) return 0;
    std::default_random_engine e1(seed);
    std::uniform_int_distribution<unsigned> ub(0, 255);
    for (uint32_t k = 0; k < K; ++k) {
        std::vector<Pt> pts;
        uint64_t p = 0;
        for (uint64_t i = 0; i < cnt[k]; ++i) {
            Pt q;
            q.x = (uint16_t)(surf[k][i] % 65536);
            q.y = (uint16_t)(surf[k][i] / 65536);
            q.xf = q.yf = 0;
            q.flags = HAS_PIXEL | HAS_FLUID;
            out[(size_t)k * width + p++] = pack(q);
            pts.push_back(q);
        }
        if (pts.empty()) {
            Pt q;
            q.x = (uint16_t)std::round(cx[k]);
            q.y = (uint16_t)std::round(cy[k]);
            q.xf = q.yf = 0;
            q.flags = HAS_FLUID;
            if (p < width) out[(size_t)k * width + p] = pack(q);
            ++p;
            pts.push_back(q);
        }
        std::shuffle(pts.begin(), pts.end(), e1);
        size_t psz = pts.size();
        for (; p < width; ++p) {
            Pt q = pts[p % psz];
            q.flags &= (uint8_t)~HAS_FLUID;
            q.xf = (uint8_t)ub(e1);
            q.yf = (uint8_t)ub(e1);
            out[(size_t)k * width + p] = pack(q);
        }
    }
    return width;
}

// fix_volatiles (thread.cpp:1187-1233): x/y of empty blobs in a cyclic list
// of K blob descriptors (7 doubles each) interpolated between the
// surrounding non-empty ones.
void orc_fix_volatiles(double *desc, uint32_t K) {
    if (K <= 1) return;
    uint32_t i = 0;
    bool started = false;
    std::vector<uint32_t> vol;
    int64_t first = -1, prev = -1;
    while (true) {
        i = (i + 1) % K;
        bool empty = desc[7 * (size_t)i] == 0;
        if (!started) {
            if (empty) {
                if (i == 0) break;
                continue;
            }
            started = true;
            first = prev = i;
            continue;
        }
        if (empty) { vol.push_back(i); continue; }
        if (!vol.empty()) {
            size_t vsz = vol.size();
            for (size_t v = 0; v < vsz; ++v) {
                double t = (v + 1.0) / double(vsz + 1.0);
                desc[7 * (size_t)vol[v] + 1] = t * desc[7 * (size_t)i + 1] + (1.0 - t) * desc[7 * (size_t)prev + 1];
                desc[7 * (size_t)vol[v] + 2] = t * desc[7 * (size_t)i + 2] + (1.0 - t) * desc[7 * (size_t)prev + 2];
            }
            vol.clear();
        }
        prev = i;
        if (prev == first) break;
    }
}

}  // extern "C"
