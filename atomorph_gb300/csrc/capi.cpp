// extern "C" entry points declared in include/atomorph_gb300.h.  Each one is
// a thin wrapper over amg::Engine; the header names the reference member each
// replaces.
#include <cmath>
#include <cstring>
#include <new>

#include "fluid.cuh"
#include "handle.h"

namespace amg {
const char *last_error();
}

using amg::Engine;

#define H(m) (m)->e
#define CHECK(m) \
    if (!(m)) return AM_ERR_ARG

extern "C" {

const char *am_last_error(void) { return amg::last_error(); }
const char *am_version(void) { return "atomorph_gb300 1.0 (reference API 1.0)"; }

int am_create(am_morph **out) {
    if (!out) return AM_ERR_ARG;
    *out = new (std::nothrow) am_morph();
    return *out ? AM_OK : AM_ERR_NOMEM;
}
void am_destroy(am_morph *m) { delete m; }
int am_clear(am_morph *m) { CHECK(m); return H(m).clear(); }

int am_add_pixel(am_morph *m, size_t frame, uint16_t x, uint16_t y, uint8_t r, uint8_t g, uint8_t b, uint8_t a) {
    CHECK(m);
    uint32_t c = r | (g << 8) | (b << 16) | ((uint32_t)a << 24);
    return H(m).add_pixel(frame, x, y, c);
}
int am_add_pixels(am_morph *m, size_t frame, const uint8_t *rgba, uint32_t w, uint32_t h) {
    CHECK(m);
    return H(m).add_pixels(frame, rgba, w, h);
}
int am_add_frame(am_morph *m, size_t frame) { CHECK(m); return H(m).add_frame(frame); }

// ---- parameters
int am_set_seed(am_morph *m, unsigned s) { CHECK(m); H(m).set_seed(s); return AM_OK; }
int am_set_blob_delimiter(am_morph *m, unsigned d) {
    CHECK(m);
    if (d != AM_RGB && d != AM_HSP) return AM_ERR_ARG;
    H(m).front.delimiter = d;
    return AM_OK;
}
int am_set_blob_threshold(am_morph *m, double t) { CHECK(m); H(m).front.threshold = t; return AM_OK; }
int am_set_blob_max_size(am_morph *m, size_t s) { CHECK(m); H(m).front.max_size = s; return AM_OK; }
int am_set_blob_min_size(am_morph *m, size_t s) { CHECK(m); H(m).front.min_size = s; return AM_OK; }
int am_set_blob_box_grip(am_morph *m, uint16_t g) { CHECK(m); H(m).front.box_grip = g; return AM_OK; }
int am_set_blob_box_samples(am_morph *m, size_t s) { CHECK(m); H(m).front.box_samples = s; return AM_OK; }
int am_set_blob_number(am_morph *m, size_t n) { CHECK(m); H(m).front.blob_number = n; return AM_OK; }
int am_set_blob_rgba_weight(am_morph *m, unsigned w) { CHECK(m); H(m).front.rgba_w = w & 255u; return AM_OK; }
int am_set_blob_size_weight(am_morph *m, unsigned w) { CHECK(m); H(m).front.size_w = w & 255u; return AM_OK; }
int am_set_blob_xy_weight(am_morph *m, unsigned w) { CHECK(m); H(m).front.xy_w = w & 255u; return AM_OK; }
int am_set_degeneration(am_morph *m, size_t d) { CHECK(m); H(m).front.degeneration = d; return AM_OK; }
int am_set_motion(am_morph *m, unsigned v) {
    CHECK(m);
    if (v != AM_NONE && v != AM_LINEAR && v != AM_SPLINE) return AM_ERR_ARG;
    H(m).front.motion = v;
    return AM_OK;
}
int am_set_fading(am_morph *m, unsigned v) {
    CHECK(m);
    if (v != AM_NONE && v != AM_LINEAR && v != AM_COSINE && v != AM_PERLIN) return AM_ERR_ARG;
    H(m).front.fading = v;
    return AM_OK;
}
int am_set_threads(am_morph *m, size_t t) { CHECK(m); H(m).front.threads = t; return AM_OK; }
int am_set_cycle_length(am_morph *m, size_t c) { CHECK(m); H(m).front.cycle_length = c; return AM_OK; }
int am_set_feather(am_morph *m, size_t f) {
    CHECK(m);
    if (f > amg::kMaxFeather) { amg::set_error("feather above 96 pixels is not supported"); return AM_ERR_UNSUPPORTED; }
    H(m).front.feather = f;
    return AM_OK;
}
int am_set_keep_background(am_morph *m, int k) {
    CHECK(m);
    H(m).front.keep_background = k != 0;
    return AM_OK;
}
int am_set_finite(am_morph *m, int f) { CHECK(m); H(m).front.finite = f != 0; return AM_OK; }
int am_set_show_blobs(am_morph *m, unsigned b) {
    CHECK(m);
    H(m).front.show_blobs = b;  // values other than AVERAGE / DISTINCT draw TEXTURE, as in the reference
    return AM_OK;
}
// morph::set_fluid / set_density (morph.cpp:1553-1570): fluid forces density 1
// and density > 1 turns the fluid off; density changes restart the morph.
int am_set_fluid(am_morph *m, unsigned f) {
    CHECK(m);
    Engine &e = H(m);
    if (e.front.fluidsteps != f) {
        e.front.fluidsteps = f;
        if (f > 0 && e.front.density > 1) { e.front.density = 1; e.identifier++; }
    }
    return AM_OK;
}
int am_set_density(am_morph *m, uint16_t d) {
    CHECK(m);
    Engine &e = H(m);
    if (e.front.density != d) {
        e.front.density = d;
        e.identifier++;
        if (e.front.fluidsteps != 0 && d > 1) e.front.fluidsteps = 0;
    }
    return AM_OK;
}
int am_set_resolution(am_morph *m, uint16_t w, uint16_t h) { CHECK(m); H(m).width = w; H(m).height = h; return AM_OK; }
int am_set_proposal(am_morph *m, unsigned k) {
    CHECK(m);
    if (k > AM_PROPOSAL_SCORED) return AM_ERR_ARG;
    H(m).front.proposal = k;
    H(m).active.proposal = k;
    return AM_OK;
}
int am_set_sweeps(am_morph *m, size_t s) { CHECK(m); H(m).front.sweeps = s; H(m).active.sweeps = s; return AM_OK; }
int am_set_tuning(am_morph *m, const char *name, double value) {
    CHECK(m);
    if (!name || !(value >= 0.0) || value > 1024.0) return AM_ERR_ARG;
    std::string n(name);
    if (n == "render_pipeline") {
        H(m).render_pipeline = value != 0.0;
        return AM_OK;
    }
    if (n == "render_bin_ctas" || n == "render_resolve_ctas") {
        if (value > 8.0 || value != (double)(uint32_t)value) return AM_ERR_ARG;
        (n == "render_bin_ctas" ? H(m).render_bin_ctas : H(m).render_resolve_ctas) = (uint32_t)value;
        return AM_OK;
    }
    amg::Params *ps[2] = {&H(m).front, &H(m).active};
    for (amg::Params *p : ps) {
        if (n == "local_self") p->local_self = (uint32_t)value;
        else if (n == "local_target") p->local_target = (uint32_t)value;
        else if (n == "local_random") p->local_random = (uint32_t)value;
        else if (n == "learned_keep") {
            if (!(value > 0.0 && value <= 1.0)) return AM_ERR_ARG;
            p->learned_keep = value;
        }
        else if (n == "guided_switch") p->guided_switch = value;
        else if (n == "learned_adaptive") p->learned_adaptive = value != 0.0;
        else return AM_ERR_ARG;
    }
    return AM_OK;
}
int am_set_fluid_sparseness(am_morph *m, double v) {
    CHECK(m);
    if (!(v > 0.0 && v <= 64.0)) return AM_ERR_ARG;
    H(m).front.fluid_sparseness = v;
    return AM_OK;
}
size_t am_get_fluid_links(am_morph *m, uint32_t *src_col, uint32_t *dst_col, size_t cap) {
    if (!m || !m->e.fluid || !m->e.fmorph) return 0;
    const size_t n = m->e.fluid->n;
    if (src_col && dst_col && cap >= n) {
        std::vector<uint32_t> v(2 * n);
        if (amg::fluid_morph_links(m->e.fmorph, v.data(), n, m->e.rstream) != AM_OK) return 0;
        std::copy(v.begin(), v.begin() + n, src_col);
        std::copy(v.begin() + n, v.end(), dst_col);
    }
    return n;
}
size_t am_get_fluid_particles(am_morph *m, double *state, size_t cap) {
    if (!m || !m->e.fluid) return 0;
    const size_t n = m->e.fluid->n;
    if (state && cap >= n && amg::fluid_get(m->e.fluid, state, m->e.rstream) != AM_OK) return 0;
    return n;
}
int am_set_motion_noise(am_morph *m, double a) {
    CHECK(m);
    if (!(a >= 0.0 && a <= 64.0)) return AM_ERR_ARG;
    H(m).front.motion_noise = a;
    return AM_OK;
}

// ---- control
int am_compute(am_morph *m) { CHECK(m); return H(m).compute(); }
int am_iterate(am_morph *m, size_t n) { CHECK(m); return H(m).iterate(n); }
int am_compute_seconds(am_morph *m, double s) { CHECK(m); return H(m).compute_seconds(s); }
int am_suspend(am_morph *m) { CHECK(m); return H(m).suspend(-1.0); }
int am_suspend_timeout(am_morph *m, double t) { CHECK(m); return H(m).suspend(t < 0 ? 0.0 : t); }
int am_is_busy(const am_morph *m) { return m && m->e.is_busy() ? 1 : 0; }
int am_synchronize(am_morph *m) { CHECK(m); return H(m).synchronize(); }
int am_next_state(am_morph *m) { CHECK(m); H(m).skip_state = true; return AM_OK; }

// ---- readout
unsigned am_get_state(const am_morph *m) { return m ? m->e.f_state : 0u; }
double am_get_energy(const am_morph *m) { return m ? m->e.f_energy : 0.0; }
int am_get_cost(am_morph *m, uint64_t *exact, double *as_double) {
    CHECK(m);
    Engine &e = H(m);
    if (e.is_busy()) return AM_ERR_BUSY;
    uint64_t v = 0;
    if (e.fN) {
        int rc = e.compute_cost(&v);
        if (rc) return rc;
    }
    if (exact) *exact = v;
    if (as_double) *as_double = (double)v;
    return AM_OK;
}
int am_get_cost_noalloc(am_morph *m, uint64_t *exact) {
    CHECK(m);
    if (!exact) return AM_ERR_ARG;
    Engine &e = H(m);
    if (e.is_busy()) return AM_ERR_BUSY;
    uint64_t v = 0;
    if (e.fN) {
        int rc = e.compute_cost_noalloc(&v);
        if (rc) return rc;
    }
    *exact = v;
    return AM_OK;
}
size_t am_get_frame_count(const am_morph *m) { return m ? m->e.frames.size() : 0; }
static long frame_index(const Engine &e, size_t key) {
    long i = 0;
    for (auto &kv : e.frames) {
        if (kv.first == key) return i;
        ++i;
    }
    return -1;
}
size_t am_get_blob_count(const am_morph *m, size_t frame) {
    if (!m) return 0;
    long i = frame_index(m->e, frame);
    if (i < 0 || (size_t)i >= m->e.f_blobs.size()) return 0;
    return m->e.f_blobs[i].size();
}
size_t am_get_blob_count_total(const am_morph *m) {
    if (!m) return 0;
    size_t n = 0;
    for (auto &b : m->e.f_blobs) n += b.size();
    return n;
}
size_t am_get_pixel_count(const am_morph *m, size_t frame) {
    if (!m) return 0;
    auto it = m->e.frames.find(frame);
    return it == m->e.frames.end() ? 0 : it->second.count;
}
// morph::get_frame_key (morph.cpp:404-423).
size_t am_get_frame_key(const am_morph *m, double t) {
    if (!m) return SIZE_MAX;
    double integ;
    t = std::modf(t, &integ);
    if (t < 0.0) t += 1.0;
    size_t f = (size_t)(t * m->e.frames.size());
    size_t i = 0;
    for (auto &kv : m->e.frames)
        if (i++ == f) return kv.first;
    return SIZE_MAX;
}
uint16_t am_get_width(const am_morph *m) { return m ? m->e.width : 0; }
uint16_t am_get_height(const am_morph *m) { return m ? m->e.height : 0; }
// morph::get_time (morph.cpp:1522-1538).
double am_get_time(const am_morph *m, size_t i, size_t n) {
    if (!m || n == 0) return 0.0;
    size_t F = m->e.frames.size();
    if (m->e.front.finite) {
        if (n == 1) {
            if (F == 0) return 0.0;
            return (1.0 - (1.0 / double(F))) / 2.0;
        }
        double t = double(i) / double(n - 1);
        t *= 1.0 - (1.0 / double(F));
        return t;
    }
    return double(i) / double(n);
}
// round(255 x mean) of a stored colour, converted HSP -> RGB when the blob
// delimiter is HSP (morph.cpp:344-351, 366-373).
static void store_rgba(const amg::Engine &e, double r, double g, double b, double a, uint8_t *rgba) {
    auto cc = [](double v) { return (uint32_t)(int)std::round(255.0 * v) & 255u; };
    uint32_t c = cc(r) | (cc(g) << 8) | (cc(b) << 16) | (cc(a) << 24);
    if (e.front.delimiter == AM_HSP) c = amg::hsp_to_rgb_host(c);
    for (int k = 0; k < 4; ++k) rgba[k] = (uint8_t)(c >> (8 * k));
}

int am_get_average_pixel(const am_morph *m, size_t frame, uint16_t *xy, uint8_t *rgba) {
    if (!m) return AM_ERR_ARG;
    auto it = m->e.frames.find(frame);
    if (it == m->e.frames.end()) return AM_ERR_NOT_FOUND;
    if (xy) { xy[0] = (uint16_t)std::round(it->second.x); xy[1] = (uint16_t)std::round(it->second.y); }
    if (rgba) {
        long i = frame_index(m->e, frame);
        double r = 0, g = 0, b = 0, a = 0, n = 0;
        if (i >= 0 && (size_t)i < m->e.f_blobs.size())
            for (auto &bl : m->e.f_blobs[i]) { r += bl.r * bl.size; g += bl.g * bl.size; b += bl.b * bl.size; a += bl.a * bl.size; n += bl.size; }
        if (n > 0) { r /= n; g /= n; b /= n; a /= n; }
        store_rgba(m->e, r, g, b, a, rgba);
    }
    return AM_OK;
}
int am_get_blob_labels(am_morph *m, size_t frame, int32_t *labels, uint32_t *w, uint32_t *h) {
    CHECK(m);
    Engine &e = H(m);
    if (e.is_busy()) return AM_ERR_BUSY;
    const long i = frame_index(e, frame);
    if (i < 0 || (size_t)i >= e.blobs.size()) return AM_ERR_NOT_FOUND;
    if (w) *w = e.CW;
    if (h) *h = e.CH;
    if (!labels) return AM_OK;
    const size_t fr = (size_t)e.CW * e.CH;
    if (!e.d_labels.p || e.d_labels.n < (size_t)(i + 1) * fr) return AM_ERR_STATE;
    AMG_CUDA(cudaMemcpy(labels, e.d_labels.p + (size_t)i * fr, fr * 4, cudaMemcpyDeviceToHost));
    return AM_OK;
}
int am_get_blob_average(const am_morph *m, size_t frame, size_t blob, uint16_t *xy, uint8_t *rgba) {
    if (!m) return AM_ERR_ARG;
    long i = frame_index(m->e, frame);
    if (i < 0 || (size_t)i >= m->e.f_blobs.size() || blob >= m->e.f_blobs[i].size()) return AM_ERR_NOT_FOUND;
    const amg::Blob &b = m->e.f_blobs[i][blob];
    if (xy) { xy[0] = (uint16_t)std::round(b.x); xy[1] = (uint16_t)std::round(b.y); }
    if (rgba) store_rgba(m->e, b.r, b.g, b.b, b.a, rgba);
    return AM_OK;
}
int am_get_blob_info(const am_morph *m, size_t frame, size_t blob, size_t *group, size_t *surface, double *xyrgba) {
    if (!m) return AM_ERR_ARG;
    const long i = frame_index(m->e, frame);
    if (i < 0 || (size_t)i >= m->e.f_blobs.size() || blob >= m->e.f_blobs[i].size()) return AM_ERR_NOT_FOUND;
    const amg::Blob &b = m->e.f_blobs[i][blob];
    if (group) *group = (size_t)i < m->e.f_group.size() && blob < m->e.f_group[i].size() ? (size_t)m->e.f_group[i][blob] : 0;
    if (surface) *surface = (size_t)b.size;
    if (xyrgba) {
        xyrgba[0] = b.x; xyrgba[1] = b.y; xyrgba[2] = b.r; xyrgba[3] = b.g; xyrgba[4] = b.b; xyrgba[5] = b.a;
    }
    return AM_OK;
}
int am_get_blob_pixels(am_morph *m, size_t blob, double t, uint16_t *xy, uint8_t *rgba, size_t cap, size_t *count) {
    CHECK(m);
    if (H(m).is_busy()) return AM_ERR_BUSY;
    std::vector<std::pair<uint32_t, uint32_t>> px;
    const int rc = H(m).blob_pixels(blob, t, px);
    if (rc) return rc;
    if (count) *count = px.size();
    const size_t n = std::min(cap, px.size());
    for (size_t k = 0; k < n; ++k) {
        if (xy) { xy[2 * k] = (uint16_t)(px[k].first & 0xFFFFu); xy[2 * k + 1] = (uint16_t)(px[k].first >> 16); }
        if (rgba) for (int c = 0; c < 4; ++c) rgba[4 * k + c] = (uint8_t)(px[k].second >> (8 * c));
    }
    return AM_OK;
}
size_t am_get_atom_count(const am_morph *m) { return m ? (size_t)m->e.fN : 0; }
size_t am_get_chain_count(const am_morph *m) { return m ? (size_t)m->e.fC : 0; }

int am_render(am_morph *m, double t, uint8_t *out, int on_dev) {
    CHECK(m);
    if (!out) return AM_ERR_ARG;
    return H(m).render(t, out, on_dev != 0);
}
size_t am_get_positions(am_morph *m, double t, int32_t *xy, size_t cap) {
    if (!m) return 0;
    size_t n = 0;
    if (H(m).positions(t, xy, cap, &n) != AM_OK) return 0;
    return n;
}
int am_render_many(am_morph *m, const double *ts, size_t n, uint8_t *out) {
    CHECK(m);
    if ((!ts || !out) && n) return AM_ERR_ARG;
    size_t fsz = (size_t)H(m).width * H(m).height * 4;
    for (size_t i = 0; i < n; ++i) {
        int rc = H(m).render(ts[i], out + i * fsz, true);
        if (rc) return rc;
    }
    return AM_OK;
}

int am_render_many_host(am_morph *m, const double *ts, size_t n, uint8_t *out) {
    CHECK(m);
    if ((!ts || !out) && n) return AM_ERR_ARG;
    return H(m).render_many_host(ts, n, out);
}

int am_export_chains(am_morph *m, uint64_t *w, uint64_t *pts, int32_t *order) {
    CHECK(m);
    return H(m).export_chains(w, pts, order);
}
int am_import_chains(am_morph *m, size_t K, size_t C, const uint64_t *w, const uint64_t *pts, const int32_t *order) {
    CHECK(m);
    return H(m).import_chains(K, C, w, pts, order);
}
int am_refine(am_morph *m, size_t sweeps, uint64_t *gains) {
    CHECK(m);
    Engine &e = H(m);
    if (e.is_busy()) return AM_ERR_BUSY;
    if (e.state != AM_STATE_ATOM_MORPHING && e.state != AM_STATE_DONE) return AM_ERR_STATE;
    e.active.proposal = e.front.proposal;
    int rc = e.refine(sweeps, gains);
    if (rc) return rc;
    return e.publish_front();
}

// ---- learned proposal
int am_record_swaps(am_morph *m, size_t cap) { CHECK(m); return H(m).record_swaps(cap); }
int am_record_outcomes(am_morph *m, size_t cap, uint32_t every) {
    CHECK(m);
    if (H(m).is_busy()) return AM_ERR_BUSY;
    return H(m).record_outcomes(cap, every);
}
size_t am_recorded_swaps(am_morph *m, float *f, float *t, size_t cap) { return m ? m->e.recorded_swaps(f, t, cap) : 0; }
int am_train_recorded(am_morph *m, size_t epochs, double lr, float *loss) {
    CHECK(m);
    if (H(m).is_busy()) return AM_ERR_BUSY;
    if (epochs == 0 || !(lr > 0.0)) return AM_ERR_ARG;
    return H(m).train_recorded(epochs, lr, loss);
}
int am_train_proposal(am_morph *m, const float *f, const float *t, size_t n, size_t epochs, double lr, float *loss) {
    CHECK(m);
    if (H(m).is_busy()) return AM_ERR_BUSY;
    return H(m).train_proposal(f, t, n, epochs, lr, loss);
}
int am_get_proposal_weights(am_morph *m, float *w, size_t count) {
    CHECK(m);
    return H(m).proposal_weights(w, count, false);
}
int am_set_proposal_weights(am_morph *m, const float *w, size_t count) {
    CHECK(m);
    return H(m).proposal_weights(const_cast<float *>(w), count, true);
}
int am_proposal_forward(am_morph *m, const float *f, size_t n, float *out) {
    CHECK(m);
    if ((!f || !out) && n) return AM_ERR_ARG;
    return H(m).proposal_forward(f, n, out);
}
int am_proposal_grad(am_morph *m, const float *f, const float *t, size_t n, float *grad, float *loss) {
    CHECK(m);
    if (!grad || ((!f || !t) && n)) return AM_ERR_ARG;
    return H(m).proposal_grad(f, t, n, grad, loss);
}

// ---- runtime
int am_profile_enable(am_morph *m, int on) {
    CHECK(m);
    m->e.prof.on = on != 0;
    m->e.prof.reset();
    return AM_OK;
}
size_t am_profile_read(am_morph *m, const char **names, double *ms, uint64_t *launches, size_t cap) {
    if (!m) return 0;
    m->e.prof.collect();
    size_t n = 0;
    for (int i = 0; i < amg::PROF_COUNT && n < cap; ++i, ++n) {
        if (names) names[n] = amg::kProfNames[i];
        if (ms) ms[n] = m->e.prof.ms[i];
        if (launches) launches[n] = m->e.prof.launches[i];
    }
    return n;
}
void *am_get_stream(am_morph *m) { return m ? (void *)m->e.rstream : nullptr; }
uint64_t am_launch_count(void) { return amg::g_launches.load(); }
int am_get_heavy_tiles(am_morph *m, uint32_t *tiles, uint32_t *helpers) {
    if (!m) return AM_ERR_ARG;
    amg::render_heavy_tiles(H(m).rw, tiles, helpers);
    return AM_OK;
}
int am_device_sync(am_morph *m) {
    CHECK(m);
    if (m->e.stream) { cudaError_t x = cudaStreamSynchronize(m->e.stream); if (x) return AM_ERR_CUDA; }
    if (m->e.rstream) { cudaError_t x = cudaStreamSynchronize(m->e.rstream); if (x) return AM_ERR_CUDA; }
    return AM_OK;
}

}  // extern "C"
