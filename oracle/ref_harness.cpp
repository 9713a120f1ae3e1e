// Test infrastructure only: a C-ABI harness around the UNMODIFIED atomorph
// reference library, compiled from the reference's own sources by
// oracle/Makefile into oracle/_ref/.  It is used to pin the C++ restatement
// (oracle/oracle.cpp) and to generate the golden fixtures under tests/golden/.
// Nothing in the product links or loads it.
//
// The reference is driven deterministically: the worker thread is never
// started; thread::step() is called directly from the caller's thread
// (thread.cpp:139-171), atom refinement uses the free function morph_asynch
// (thread.cpp:990-1041) with seeds drawn from a caller-seeded std::mt19937,
// and the atom cost is recomputed with thread::get_energy(chain*)
// (thread.cpp:1109-1125) because the worker's running energy is not usable.

#include <cstdint>
#include <cmath>
#include <cstring>
#include <thread>
#include <mutex>
#include <atomic>
#include <chrono>
#include <stdlib.h>
#include <algorithm>
#include <vector>
#include <future>
#include <random>
#include <map>
#include <set>
#include <limits>
#include <assert.h>
#include <iostream>

#define private public
#include "atomorph.h"
#undef private

namespace am {
void morph_asynch(point **map, size_t width, size_t height, size_t repeat,
                  unsigned rng_seed, double *gain);
}

extern "C" {

void *ref_new(void) { return new (std::nothrow) am::morph(); }
void ref_free(void *h) { delete (am::morph *)h; }

// Parameter setters mirror am::morph's (morph.h:39-76, morph.cpp:436,1553-1570).
void ref_set_seed(void *h, unsigned s) { ((am::morph *)h)->set_seed(s); }
void ref_set_delimiter(void *h, unsigned d) { ((am::morph *)h)->set_blob_delimiter((unsigned char)d); }
void ref_set_threshold(void *h, double t) { ((am::morph *)h)->set_blob_threshold(t); }
void ref_set_blob_number(void *h, size_t n) { ((am::morph *)h)->set_blob_number(n); }
void ref_set_blob_min_size(void *h, size_t n) { ((am::morph *)h)->set_blob_min_size(n); }
void ref_set_blob_max_size(void *h, size_t n) { ((am::morph *)h)->set_blob_max_size(n); }
void ref_set_box_samples(void *h, size_t n) { ((am::morph *)h)->set_blob_box_samples(n); }
void ref_set_density(void *h, unsigned d) { ((am::morph *)h)->set_density((uint16_t)d); }
void ref_set_motion(void *h, unsigned m) { ((am::morph *)h)->set_motion((unsigned char)m); }
void ref_set_fading(void *h, unsigned f) { ((am::morph *)h)->set_fading((unsigned char)f); }
void ref_set_fluid(void *h, unsigned f) { ((am::morph *)h)->set_fluid(f); }
void ref_set_degeneration(void *h, size_t d) { ((am::morph *)h)->set_degeneration(d); }
void ref_set_finite(void *h, int f) { ((am::morph *)h)->set_finite(f != 0); }
void ref_set_resolution(void *h, unsigned w, unsigned hh) {
    ((am::morph *)h)->set_resolution((uint16_t)w, (uint16_t)hh);
}
void ref_set_cycle_length(void *h, size_t c) { ((am::morph *)h)->set_cycle_length(c); }
void ref_set_feather(void *h, size_t f) { ((am::morph *)h)->set_feather(f); }
void ref_set_keep_background(void *h, int k) { ((am::morph *)h)->set_keep_background(k != 0); }
void ref_set_show_blobs(void *h, unsigned b) { ((am::morph *)h)->set_show_blobs(b); }
void ref_set_threads(void *h, size_t t) { ((am::morph *)h)->set_threads(t); }

// Same ingestion as the demo's fill_morph (demo/main.cpp:96-127): every pixel
// with alpha > 0 becomes an atom; an all-transparent image adds an empty frame.
int ref_add_image(void *h, size_t frame, const uint8_t *rgba, unsigned w, unsigned hh) {
    am::morph *m = (am::morph *)h;
    bool empty = true;
    for (size_t i = 0; i < (size_t)w * hh; ++i) {
        const uint8_t *p = rgba + 4 * i;
        if (p[3] == 0) continue;
        m->add_pixel(frame, am::create_pixel((uint16_t)(i % w), (uint16_t)(i / w), p[0], p[1], p[2], p[3]));
        empty = false;
    }
    if (empty) m->add_frame(frame);
    return 0;
}

int ref_add_pixel(void *h, size_t frame, unsigned x, unsigned y, unsigned r, unsigned g, unsigned b, unsigned a) {
    return ((am::morph *)h)->add_pixel(frame, am::create_pixel((uint16_t)x, (uint16_t)y, r, g, b, a)) ? 1 : 0;
}

unsigned ref_state(void *h) { return ((am::morph *)h)->worker.state; }
int ref_synchronize(void *h) { return ((am::morph *)h)->synchronize() ? 1 : 0; }

// Runs worker steps until the atom-morphing state is reached.  Blob matching
// is given at most max_match_steps steps (thread.cpp:598-738 runs one swap
// proposal per step); after that next_state() ends it, like the demo's
// wall-clock driver does (demo/main.cpp:257-268).  Returns the worker state.
unsigned ref_prepare(void *h, size_t max_detect_steps, size_t max_match_steps) {
    am::morph *m = (am::morph *)h;
    m->synchronize();
    am::thread &w = m->worker;
    size_t guard = 0;
    while (w.state == am::STATE_BLOB_DETECTION || w.state == am::STATE_BLOB_UNIFICATION) {
        w.step();
        if (++guard > max_detect_steps) break;
    }
    size_t n = 0;
    while (w.state == am::STATE_BLOB_MATCHING) {
        if (n >= max_match_steps) w.next_state();
        w.step();
        ++n;
    }
    m->synchronize();
    return w.state;
}

// Blob matching steps taken so far is not tracked by the reference; expose its
// current best blob-map energy (thread.cpp:713-716).
double ref_blob_energy(void *h) { return ((am::morph *)h)->worker.best_blob_map_e; }

size_t ref_frame_count(void *h) { return ((am::morph *)h)->frames.size(); }
size_t ref_blob_count(void *h, size_t frame_index) {
    am::morph *m = (am::morph *)h;
    auto it = m->frames.begin();
    std::advance(it, frame_index);
    return it->second.blobs.size();
}
size_t ref_pixel_count(void *h, size_t frame_index) {
    am::morph *m = (am::morph *)h;
    auto it = m->frames.begin();
    std::advance(it, frame_index);
    return it->second.pixels.size();
}
// Blob b of frame f (worker's frame, blob-vector order): group, surface size,
// and the running means x,y,r,g,b,a (stored colour space, 0..1).
int ref_blob_info(void *h, size_t frame_index, size_t b, size_t *group, size_t *surface, double *xyrgba) {
    am::morph *m = (am::morph *)h;
    auto it = m->worker.frames.begin();
    std::advance(it, frame_index);
    if (b >= it->second.blobs.size() || !it->second.blobs[b]) return -1;
    am::blob *bl = it->second.blobs[b];
    *group = bl->group;
    *surface = bl->surface.size();
    xyrgba[0] = bl->x; xyrgba[1] = bl->y; xyrgba[2] = bl->r;
    xyrgba[3] = bl->g; xyrgba[4] = bl->b; xyrgba[5] = bl->a;
    return 0;
}
// Writes the sorted surface positions (y*65536+x) of blob b of frame f.
size_t ref_blob_surface(void *h, size_t frame_index, size_t b, uint64_t *out) {
    am::morph *m = (am::morph *)h;
    auto it = m->worker.frames.begin();
    std::advance(it, frame_index);
    am::blob *bl = it->second.blobs[b];
    size_t i = 0;
    for (size_t p : bl->surface) out[i++] = p;
    return i;
}

size_t ref_chain_count(void *h) { return ((am::morph *)h)->worker.chains.size(); }
// Chain widths in key (group) order; returns the key-frame count (height).
size_t ref_chain_widths(void *h, uint64_t *widths) {
    am::morph *m = (am::morph *)h;
    size_t i = 0, height = 0;
    for (auto &kv : m->worker.chains) {
        widths[i++] = kv.second.width;
        height = kv.second.height;
    }
    return height;
}
// Points of all chains, frame-major: out[y * N + off_c + x] = points[x][y].word
// with the padding byte cleared.
void ref_export_points(void *h, uint64_t *out, size_t total) {
    am::morph *m = (am::morph *)h;
    size_t off = 0;
    for (auto &kv : m->worker.chains) {
        am::chain &c = kv.second;
        for (size_t y = 0; y < c.height; ++y)
            for (size_t x = 0; x < c.width; ++x)
                out[y * total + off + x] = c.points[x][y].word & 0x00FFFFFFFFFFFFFFull;
        off += c.width;
    }
}
void ref_import_points(void *h, const uint64_t *in, size_t total) {
    am::morph *m = (am::morph *)h;
    size_t off = 0;
    for (auto &kv : m->worker.chains) {
        am::chain &c = kv.second;
        for (size_t y = 0; y < c.height; ++y)
            for (size_t x = 0; x < c.width; ++x)
                c.points[x][y].word = in[y * total + off + x];
        off += c.width;
    }
    m->synchronize();
}

// True atom cost: sum over chains of thread::get_energy(chain*).
double ref_energy(void *h) {
    am::morph *m = (am::morph *)h;
    double e = 0.0;
    for (auto &kv : m->worker.chains) e += m->worker.get_energy(&kv.second);
    return e;
}

// n sweeps of the reference's own refinement.  One sweep = for every chain in
// key order, `height` calls of morph_asynch(map, w, h, repeat = w, seed), the
// seeds drawn in order from std::mt19937(seed).  Chains of width <= 1 are
// skipped as thread::morph does (thread.cpp:1045).
void ref_sweeps(void *h, size_t n, unsigned seed) {
    am::morph *m = (am::morph *)h;
    std::mt19937 seeds(seed);
    for (size_t s = 0; s < n; ++s) {
        for (auto &kv : m->worker.chains) {
            am::chain &c = kv.second;
            if (c.width <= 1) continue;
            for (size_t k = 0; k < c.height; ++k) {
                double gain = 0.0;
                am::morph_asynch(c.points, c.width, c.height, c.width, (unsigned)seeds(), &gain);
            }
        }
    }
    m->synchronize();
}

// The reference's multithreaded refinement as thread::morph runs it
// (thread.cpp:1043-1068): `calls` calls, round-robin over chains, each with
// `threads` std::threads doing cycle_length proposals (threads==0: inline).
void ref_morph_calls(void *h, size_t calls) {
    am::morph *m = (am::morph *)h;
    m->synchronize();
    am::thread &w = m->worker;
    for (size_t i = 0; i < calls; ++i) {
        w.morph();
        w.counter++;
    }
    m->synchronize();
}

// Renders one output frame at time t exactly as morph::get_pixels(t)
// (morph.cpp:1405-1421) into a width*height*4 RGBA buffer.
void ref_render(void *h, double t, uint8_t *out) {
    am::morph *m = (am::morph *)h;
    std::vector<am::pixel> img;
    m->get_pixels(t, &img);
    for (size_t i = 0; i < img.size(); ++i) {
        out[4 * i + 0] = img[i].c.r;
        out[4 * i + 1] = img[i].c.g;
        out[4 * i + 2] = img[i].c.b;
        out[4 * i + 3] = img[i].c.a;
    }
}

double ref_get_time(void *h, size_t i, size_t n) { return ((am::morph *)h)->get_time(i, n); }
// morph::get_pixels(blob, t, to) (morph.cpp:452-678): the pixel list of the
// blob-th blob of the key frame at t; up to cap pixels into xy / rgba.
// Returns the list's length, or SIZE_MAX when the reference returns nullptr.
size_t ref_blob_pixels(void *h, size_t blob, double t, uint16_t *xy, uint8_t *rgba, size_t cap) {
    std::vector<am::pixel> v;
    if (!((am::morph *)h)->get_pixels(blob, t, &v)) return SIZE_MAX;
    for (size_t i = 0; i < v.size() && i < cap; ++i) {
        xy[2 * i] = v[i].x;
        xy[2 * i + 1] = v[i].y;
        rgba[4 * i] = v[i].c.r;
        rgba[4 * i + 1] = v[i].c.g;
        rgba[4 * i + 2] = v[i].c.b;
        rgba[4 * i + 3] = v[i].c.a;
    }
    return v.size();
}
void ref_bbox(void *h, unsigned *b4) {
    am::morph *m = (am::morph *)h;
    b4[0] = m->bbox_x1; b4[1] = m->bbox_y1; b4[2] = m->bbox_x2; b4[3] = m->bbox_y2;
}
// Stored (possibly HSP) colour and presence of a pixel of frame f.
int ref_stored_pixel(void *h, size_t frame_index, unsigned x, unsigned y, uint8_t *rgba) {
    am::morph *m = (am::morph *)h;
    auto it = m->frames.begin();
    std::advance(it, frame_index);
    auto pit = it->second.pixels.find(am::xy2pos((uint16_t)x, (uint16_t)y));
    if (pit == it->second.pixels.end()) return 0;
    rgba[0] = pit->second.c.r; rgba[1] = pit->second.c.g;
    rgba[2] = pit->second.c.b; rgba[3] = pit->second.c.a;
    return 1;
}

// Colour helpers (color.cpp:64-92) and Perlin noise (perlin.cpp:11-89).
uint32_t ref_rgb_to_hsp(uint32_t c) {
    am::color x; memcpy(&x, &c, 4);
    x = am::rgb_to_hsp(x);
    uint32_t o; memcpy(&o, &x, 4); return o;
}
uint32_t ref_hsp_to_rgb(uint32_t c) {
    am::color x; memcpy(&x, &c, 4);
    x = am::hsp_to_rgb(x);
    uint32_t o; memcpy(&o, &x, 4); return o;
}
double ref_octave_noise(unsigned seed, double x, double y, int octaves) {
    PerlinNoise p(seed);
    return p.octaveNoise(x, y, octaves);
}
void ref_spline_eval(const double *xy, size_t n, double t, double *out) {
    glnemo::CRSpline s;
    for (size_t i = 0; i < n; ++i) s.AddSplinePoint(glnemo::Vec3D(xy[2 * i], xy[2 * i + 1], 0.0));
    glnemo::Vec3D v = s.GetInterpolatedSplinePoint(t);
    out[0] = v.x; out[1] = v.y;
}

// ---- Fluid solver (fluidmodel.cpp:107-580), driven directly. ----
// Particle state exchanged as 20 doubles per particle:
// x y u v gravity_x gravity_y freedom_r active mature strength R G B A r g b a dudx(unused) pad
// Node() (fluidmodel.cpp:57-68) leaves r,g,b,a,weight uninitialised and the
// first P2G colour deposit into a node reads them; the harness clears every
// node once after construction so the reference is run on zeroed state (what
// a fresh page-backed allocation holds) instead of heap garbage.
void *ref_fluid_new(unsigned gx, unsigned gy, unsigned n) {
    FluidModel *f = new FluidModel(gx, gy, n);
    for (unsigned i = 0; i < gx; ++i)
        for (unsigned j = 0; j < gy; ++j) f->grid[i][j].clear();
    return f;
}
void ref_fluid_free(void *f) { delete (FluidModel *)f; }
void ref_fluid_set(void *f, const double *s, unsigned n) {
    Particle *P = ((FluidModel *)f)->getParticles();
    for (unsigned i = 0; i < n; ++i) {
        const double *q = s + 20 * i;
        Particle *p = P + i;
        p->clear();
        p->x = q[0]; p->y = q[1]; p->u = q[2]; p->v = q[3];
        p->gravity_x = q[4]; p->gravity_y = q[5]; p->freedom_r = q[6];
        p->active = q[7] != 0.0; p->mature = q[8] != 0.0; p->strength = q[9];
        p->R = q[10]; p->G = q[11]; p->B = q[12]; p->A = q[13];
        p->r = q[14]; p->g = q[15]; p->b = q[16]; p->a = q[17];
    }
}
void ref_fluid_get(void *f, double *s, unsigned n) {
    Particle *P = ((FluidModel *)f)->getParticles();
    for (unsigned i = 0; i < n; ++i) {
        double *q = s + 20 * i;
        Particle *p = P + i;
        q[0] = p->x; q[1] = p->y; q[2] = p->u; q[3] = p->v;
        q[4] = p->gravity_x; q[5] = p->gravity_y; q[6] = p->freedom_r;
        q[7] = p->active; q[8] = p->mature; q[9] = p->strength;
        q[10] = p->R; q[11] = p->G; q[12] = p->B; q[13] = p->A;
        q[14] = p->r; q[15] = p->g; q[16] = p->b; q[17] = p->a;
        q[18] = 0.0; q[19] = 0.0;
    }
}
void ref_fluid_step(void *f, size_t steps_left, double freedom_radius, double t) {
    ((FluidModel *)f)->step(steps_left, freedom_radius, t);
}

}  // extern "C"
