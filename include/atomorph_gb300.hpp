// am::morph on the GB300 C ABI — the reference's public C++ class
// (morph.h:9-145) with its own member signatures, so code written against the
// reference (for example its demo, demo/main.cpp) compiles against this header
// unchanged and runs the morph pipeline on the GPU.
//
// Conventions of the reference kept here: setters return nothing, compute()/
// iterate() silently do nothing while the worker is busy (morph.cpp:53-66),
// synchronize() returns false while busy (morph.cpp:103), getters return 0 or
// an all-zero pixel for missing frames/blobs.  get_energy() returns the true
// atom cost (the reference's running value for atoms is not maintained
// correctly, thread.cpp:869-870).  get_blob returns a blob the class builds
// from the GPU's blob labels and descriptors (surface positions, 4-connected
// border, group, means); like the reference's pointer it stays valid until
// the next synchronize() or clear().  Blob means are exact means (the
// reference keeps running means, which can differ in the last bits).
#ifndef ATOMORPH_GB300_HPP
#define ATOMORPH_GB300_HPP

#include <cstddef>
#include <cstdint>
#include <iostream>  // callers of the reference rely on its header pulling in the iostreams
#include <map>
#include <set>
#include <stdexcept>
#include <utility>
#include <vector>

#include "atomorph_gb300.h"

namespace am {

const unsigned RGB = AM_RGB, HSP = AM_HSP, NONE = AM_NONE, LINEAR = AM_LINEAR, SPLINE = AM_SPLINE,
               COSINE = AM_COSINE, PERLIN = AM_PERLIN;
const unsigned STATE_BLOB_DETECTION = AM_STATE_BLOB_DETECTION, STATE_BLOB_UNIFICATION = AM_STATE_BLOB_UNIFICATION,
               STATE_BLOB_MATCHING = AM_STATE_BLOB_MATCHING, STATE_ATOM_MORPHING = AM_STATE_ATOM_MORPHING,
               STATE_DONE = AM_STATE_DONE;
const unsigned char HAS_PIXEL = AM_HAS_PIXEL, HAS_FLUID = AM_HAS_FLUID;
const unsigned TEXTURE = AM_TEXTURE, AVERAGE = AM_AVERAGE, DISTINCT = AM_DISTINCT;

// color.h:7-12 and atomorph.h:249-254
typedef struct color {
    uint8_t r, g, b, a;
} color;
typedef struct pixel {
    uint16_t x, y;
    color c;
} pixel;

inline color create_color(unsigned char r, unsigned char g, unsigned char b, unsigned char a) {
    color c = {r, g, b, a};
    return c;
}
inline pixel create_pixel(uint16_t x, uint16_t y, unsigned char r, unsigned char g, unsigned char b,
                          unsigned char a) {
    pixel p;
    p.x = x;
    p.y = y;
    p.c = create_color(r, g, b, a);
    return p;
}
inline pixel create_pixel(uint16_t x, uint16_t y, color c) { return create_pixel(x, y, c.r, c.g, c.b, c.a); }
inline size_t xy2pos(uint16_t x, uint16_t y) { return (size_t)y * (UINT16_MAX + 1) + x; }
inline const char *get_version() { return "1.0"; }
// atomorph.h:300-302, 355-357: build warnings and the OpenCV variant flag.
const size_t WARN_POINTER_SIZE = 1, WARN_PIXEL_SIZE = 2, WARN_POINT_SIZE = 3;
// The 8-byte atom word (atomorph.h:275-284): the layout the chains use on
// the GPU and in am_export_chains / am_import_chains.
typedef union key_point {
    struct {
        uint16_t x;
        uint16_t y;
        uint8_t x_fract;
        uint8_t y_fract;
        uint8_t flags;
    } s;
    uint64_t word;
} point;

// atomorph.h:256-263
typedef struct blob {
    size_t index;              // position in the key frame's blob vector
    std::set<size_t> surface;  // pixel positions y * 65536 + x of the blob
    std::set<size_t> border;   // 4-neighbours of the surface outside it
    size_t group = 0;          // the chain (blob group) the blob belongs to
    bool unified = false;      // a volatile (empty) blob added by matching
    double x, y, r, g, b, a;   // means; colours in the stored colour space, 0..1
} blob;

inline size_t get_warning() {
    size_t flags = 0;
    if (sizeof(void *) < 8) flags |= WARN_POINTER_SIZE;
    if (sizeof(pixel) > 8) flags |= WARN_PIXEL_SIZE;
    if (sizeof(point) > 8) flags |= WARN_POINT_SIZE;
    return flags;
}
inline bool uses_opencv() { return false; }

class morph {
  public:
    morph() {
        if (am_create(&h_) != AM_OK) throw std::bad_alloc();
    }
    ~morph() { am_destroy(h_); }
    morph(const morph &) = delete;
    morph &operator=(const morph &) = delete;

    void clear() {
        blobs_.clear();
        am_clear(h_);
    }
    bool add_pixel(size_t frame, pixel px) {
        return am_add_pixel(h_, frame, px.x, px.y, px.c.r, px.c.g, px.c.b, px.c.a) == AM_OK;
    }
    bool add_frame(size_t frame) { return am_add_frame(h_, frame) == AM_OK; }
    // Bulk form of add_pixel for a whole RGBA8 image (pixels with alpha 0 skipped).
    bool add_image(size_t frame, const uint8_t *rgba, uint32_t w, uint32_t h) {
        return am_add_pixels(h_, frame, rgba, w, h) == AM_OK;
    }
    size_t get_pixel_count(size_t frame) { return am_get_pixel_count(h_, frame); }
    size_t get_frame_key(double t) { return am_get_frame_key(h_, t); }
    size_t get_blob_count(size_t frame) { return am_get_blob_count(h_, frame); }
    size_t get_blob_count() { return am_get_blob_count_total(h_); }
    pixel get_average_pixel(size_t frame) {
        uint16_t xy[2] = {0, 0};
        uint8_t c[4] = {0, 0, 0, 0};
        am_get_average_pixel(h_, frame, xy, c);
        return create_pixel(xy[0], xy[1], c[0], c[1], c[2], c[3]);
    }
    pixel get_average_pixel(size_t frame, size_t blob) {
        uint16_t xy[2] = {0, 0};
        uint8_t c[4] = {0, 0, 0, 0};
        am_get_blob_average(h_, frame, blob, xy, c);
        return create_pixel(xy[0], xy[1], c[0], c[1], c[2], c[3]);
    }
    // morph::get_pixels(t, to) (morph.cpp:1405-1421): the full frame, row-major.
    void get_pixels(double t, std::vector<pixel> *to) {
        size_t w = get_width(), h = get_height();
        std::vector<uint8_t> rgba(w * h * 4);
        to->clear();
        if (w * h == 0) return;
        if (am_render(h_, t, rgba.data(), 0) != AM_OK) throw std::runtime_error(am_last_error());
        to->reserve(w * h);
        for (size_t i = 0; i < w * h; ++i)
            to->push_back(create_pixel((uint16_t)(i % w), (uint16_t)(i / w), rgba[4 * i], rgba[4 * i + 1],
                                       rgba[4 * i + 2], rgba[4 * i + 3]));
    }
    // morph::get_pixels(blob, t, to) (morph.cpp:452-678): the blob-th blob of
    // the key frame at t drawn alone, appended to *to in the reference's
    // order; returns the blob, or nullptr when it does not exist.
    const blob *get_pixels(size_t blob_index, double t, std::vector<pixel> *to) {
        size_t n = 0;
        if (am_get_blob_pixels(h_, blob_index, t, nullptr, nullptr, 0, &n) != AM_OK) return nullptr;
        std::vector<uint16_t> xy(2 * n + 2);
        std::vector<uint8_t> c(4 * n + 4);
        if (am_get_blob_pixels(h_, blob_index, t, xy.data(), c.data(), n, &n) != AM_OK) return nullptr;
        for (size_t i = 0; i < n; ++i)
            to->push_back(create_pixel(xy[2 * i], xy[2 * i + 1], c[4 * i], c[4 * i + 1], c[4 * i + 2], c[4 * i + 3]));
        return get_blob(get_frame_key(t), blob_index);
    }
    // morph::get_blob(f, b) (morph.h:40): nullptr when it does not exist.
    const blob *get_blob(size_t f, size_t b) {
        auto key = std::make_pair(f, b);
        auto it = blobs_.find(key);
        if (it != blobs_.end()) return &it->second;
        size_t group = 0, surface = 0;
        double v[6];
        if (am_get_blob_info(h_, f, b, &group, &surface, v) != AM_OK) return nullptr;
        am::blob bl;
        bl.index = b;
        bl.group = group;
        bl.unified = surface == 0;
        bl.x = v[0]; bl.y = v[1]; bl.r = v[2]; bl.g = v[3]; bl.b = v[4]; bl.a = v[5];
        uint32_t w = 0, h = 0;
        if (surface && am_get_blob_labels(h_, f, nullptr, &w, &h) == AM_OK && w && h) {
            std::vector<int32_t> lab((size_t)w * h);
            if (am_get_blob_labels(h_, f, lab.data(), nullptr, nullptr) == AM_OK) {
                for (size_t q = 0; q < lab.size(); ++q)
                    if (lab[q] == (int32_t)b) bl.surface.insert(xy2pos((uint16_t)(q % w), (uint16_t)(q / w)));
                for (size_t p : bl.surface) {
                    const uint16_t x = (uint16_t)(p % (UINT16_MAX + 1)), y = (uint16_t)(p / (UINT16_MAX + 1));
                    const size_t nb[4] = {x > 0 ? xy2pos(x - 1, y) : SIZE_MAX, x < UINT16_MAX ? xy2pos(x + 1, y) : SIZE_MAX,
                                          y > 0 ? xy2pos(x, y - 1) : SIZE_MAX, y < UINT16_MAX ? xy2pos(x, y + 1) : SIZE_MAX};
                    for (size_t q : nb)
                        if (q != SIZE_MAX && !bl.surface.count(q)) bl.border.insert(q);
                }
            }
        }
        return &blobs_.emplace(key, std::move(bl)).first->second;
    }
    // The same frame straight into an RGBA8 buffer (host, or device when on_device).
    bool get_frame(double t, uint8_t *rgba, bool on_device = false) {
        return am_render(h_, t, rgba, on_device ? 1 : 0) == AM_OK;
    }
    void set_seed(unsigned seed) { am_set_seed(h_, seed); }
    double get_time(size_t current_frame, size_t total_frames) { return am_get_time(h_, current_frame, total_frames); }

    uint16_t get_width() { return am_get_width(h_); }
    uint16_t get_height() { return am_get_height(h_); }
    size_t get_frame_count() { return am_get_frame_count(h_); }
    unsigned get_state() { return am_get_state(h_); }
    void next_state() { am_next_state(h_); }
    double get_energy() { return am_get_energy(h_); }
    void compute() { am_compute(h_); }
    void iterate(size_t iterations) { am_iterate(h_, iterations); }
    void compute(double seconds) { am_compute_seconds(h_, seconds); }
    void suspend() { am_suspend(h_); }
    bool suspend(double timeout) { return am_suspend_timeout(h_, timeout) == AM_OK; }
    bool is_busy() const { return am_is_busy(h_) != 0; }
    bool synchronize() {
        if (am_synchronize(h_) != AM_OK) return false;
        blobs_.clear();  // blobs returned by get_blob are valid until here
        return true;
    }

    void set_blob_delimiter(unsigned char d) { am_set_blob_delimiter(h_, d); }
    void set_blob_threshold(double t) { am_set_blob_threshold(h_, t); }
    void set_blob_max_size(size_t s) { am_set_blob_max_size(h_, s); }
    void set_blob_min_size(size_t s) { am_set_blob_min_size(h_, s); }
    void set_blob_box_grip(uint16_t g) { am_set_blob_box_grip(h_, g); }
    void set_blob_box_samples(size_t s) { am_set_blob_box_samples(h_, s); }
    void set_blob_number(size_t n) { am_set_blob_number(h_, n); }
    void set_blob_rgba_weight(unsigned char w) { am_set_blob_rgba_weight(h_, w); }
    void set_blob_size_weight(unsigned char w) { am_set_blob_size_weight(h_, w); }
    void set_blob_xy_weight(unsigned char w) { am_set_blob_xy_weight(h_, w); }
    void set_degeneration(size_t d) { am_set_degeneration(h_, d); }
    void set_motion(unsigned char m) { am_set_motion(h_, m); }
    void set_fading(unsigned char f) { am_set_fading(h_, f); }
    void set_threads(size_t t) { am_set_threads(h_, t); }
    void set_cycle_length(size_t c) { am_set_cycle_length(h_, c); }
    void set_feather(size_t f) { am_set_feather(h_, f); }
    void set_keep_background(bool k) { am_set_keep_background(h_, k ? 1 : 0); }
    void set_finite(bool f) { am_set_finite(h_, f ? 1 : 0); }
    void set_show_blobs(unsigned b) { am_set_show_blobs(h_, b); }
    void set_fluid(unsigned f) { am_set_fluid(h_, f); }
    void set_density(uint16_t d) { am_set_density(h_, d); }
    void set_resolution(uint16_t w, uint16_t h) { am_set_resolution(h_, w, h); }

    // GB300 additions
    void set_proposal(unsigned kind) { am_set_proposal(h_, kind); }
    void set_sweeps(size_t sweeps_per_step) { am_set_sweeps(h_, sweeps_per_step); }
    am_morph *handle() { return h_; }

  private:
    am_morph *h_ = nullptr;
    std::map<std::pair<size_t, size_t>, am::blob> blobs_;
};

}  // namespace am

#endif
