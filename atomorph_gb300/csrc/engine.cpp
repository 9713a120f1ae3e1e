// Host engine and C ABI of atomorph_gb300.
//
// The handle mirrors the reference's split between the front-end am::morph
// (key frames, settings, rendering from its own copy of the results) and the
// worker am::thread (the pipeline state machine).  The worker runs on a host
// std::thread like the reference's (thread.h:45-53, thread.cpp:173-206); every
// step it takes enqueues CUDA kernels on the handle's stream and waits for
// them, so a paused worker never has GPU work in flight.  synchronize()
// publishes the worker's results to the front copy that rendering reads
// (morph.cpp:102-269), so a frame can be rendered while the worker refines.
#include <cuda.h>

#include "engine.h"
#include "fluid.cuh"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <numeric>
#include <random>
#include <string>

namespace amg {

std::atomic<uint64_t> g_launches{0};
const char *const kProfNames[PROF_COUNT] = {"k_frame_splat", "k_scan_u32",   "k_frame_scatter", "k_frame_resolve",
                                            "pair_prep",     "k_sweep_random", "k_sweep_local", "mlp", "fluid_step",
                                            "k_frame_bin",   "fluid_manage", "fluid_draw"};
static thread_local std::string t_error;
void set_error(const std::string &msg) { t_error = msg; }
const char *last_error() { return t_error.c_str(); }

// PerlinNoise(seed) permutation (perlin.cpp:11-17): 0..255 shuffled by
// std::mt19937(seed), seed 0 replaced by the engine's default seed, repeated.
static void perlin_perm(unsigned seed, int *p) {
    if (seed == 0) seed = std::mt19937::default_seed;
    std::iota(p, p + 256, 0);
    std::shuffle(p, p + 256, std::mt19937(seed));
    for (int i = 0; i < 256; ++i) p[256 + i] = p[i];
}

Engine::Engine() {
    cudaGetDevice(&device);
    // Default-constructed PerlinNoise maps use seed 1 (perlin.h:7, morph.h:136-137).
    perlin_perm(1, perm_lag);
    perlin_perm(1, perm_slope);
    // The motion perturbation's maps: seed + 2 and seed + 3 of the morph's seed (0 until set).
    perlin_perm(2, perm_mx);
    perlin_perm(3, perm_my);
}

Engine::~Engine() {
    if (running) {
        signal_pause = true;
        signal_stop = true;
        if (th.joinable()) th.join();
    }
    if (rw) render_work_destroy(rw);
    if (bw) blob_work_destroy(bw);
    if (fluid) fluid_destroy(fluid);
    if (fmorph) fluid_morph_destroy(fmorph);
    d_raw.release(); d_stored.release(); d_display.release(); d_present.release(); d_labels.release();
    d_P.release(); d_Pf.release(); d_chain_off.release(); d_pair_off.release(); d_chain_off_f.release();
    d_singles.release(); d_rank_f.release(); d_phase.release(); d_acc.release(); d_stats.release();
    d_desc.release(); d_energy.release(); d_perm.release(); d_sorted.release(); d_keys.release();
    d_tk.release(); d_tv.release(); d_hist.release(); d_bstart.release(); d_bsize.release(); d_volxy.release();
    d_blob_of.release(); d_frame.release();
    if (h_pinned) cudaFreeHost(h_pinned);
    if (stream) cudaStreamDestroy(stream);
    if (rstream) cudaStreamDestroy(rstream);
}

static int ensure_streams(Engine *e) {
    if (e->stream) return AM_OK;
    AMG_CUDA(cudaSetDevice(e->device));
    AMG_CUDA(cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking));
    AMG_CUDA(cudaStreamCreateWithFlags(&e->rstream, cudaStreamNonBlocking));
    e->rw = render_work_create();
    e->bw = blob_work_create();
    render_set_prof(e->rw, &e->prof);
    int rc = render_set_perlin(e->rw, e->perm_lag, e->perm_slope, e->perm_mx, e->perm_my);
    return rc;
}

int Engine::ensure_streams_public() { return ensure_streams(this); }

// ------------------------------------------------------------ ingestion --
static void grow(HostFrame &f, uint32_t w, uint32_t h) {
    if (w <= f.w && h <= f.h) return;
    uint32_t nw = std::max(w, f.w), nh = std::max(h, f.h);
    std::vector<uint32_t> raw((size_t)nw * nh, 0);
    std::vector<uint8_t> pr((size_t)nw * nh, 0);
    for (uint32_t y = 0; y < f.h; ++y) {
        std::memcpy(&raw[(size_t)y * nw], &f.raw[(size_t)y * f.w], f.w * 4);
        std::memcpy(&pr[(size_t)y * nw], &f.present[(size_t)y * f.w], f.w);
    }
    f.raw.swap(raw);
    f.present.swap(pr);
    f.w = nw;
    f.h = nh;
}

int Engine::add_frame(size_t key) {
    if (frames.count(key)) return AM_ERR_ARG;
    HostFrame &f = frames[key];
    f.x = bbox_x1 <= bbox_x2 ? (bbox_x1 + bbox_x2) / 2.0 : 0.0;
    f.y = bbox_y1 <= bbox_y2 ? (bbox_y1 + bbox_y2) / 2.0 : 0.0;
    identifier++;
    return AM_OK;
}

int Engine::add_pixel(size_t key, uint16_t x, uint16_t y, uint32_t rgba) {
    if (!frames.count(key)) add_frame(key);
    HostFrame &f = frames[key];
    grow(f, (uint32_t)x + 1, (uint32_t)y + 1);
    size_t i = (size_t)y * f.w + x;
    bool fresh = !f.present[i];
    f.raw[i] = rgba;
    f.present[i] = front.delimiter == AM_HSP ? 2 : 1;
    if (fresh) f.count++;
    identifier++;
    bbox_x1 = std::min(bbox_x1, x); bbox_y1 = std::min(bbox_y1, y);
    bbox_x2 = std::max(bbox_x2, x); bbox_y2 = std::max(bbox_y2, y);
    if (f.count == 1 && fresh) { f.x = x; f.y = y; }
    else {
        double w = 1.0 / double(f.count);
        f.x = (1.0 - w) * f.x + w * x;
        f.y = (1.0 - w) * f.y + w * y;
    }
    return AM_OK;
}

int Engine::add_pixels(size_t key, const uint8_t *rgba, uint32_t w, uint32_t h) {
    if (!rgba && (size_t)w * h) return AM_ERR_ARG;
    if (w > 65536 || h > 65536) return AM_ERR_ARG;
    if (!frames.count(key)) add_frame(key);
    HostFrame &f = frames[key];
    bool any = false;
    const uint8_t mark = front.delimiter == AM_HSP ? 2 : 1;
    for (uint32_t y = 0; y < h; ++y) {
        for (uint32_t x = 0; x < w; ++x) {
            const uint8_t *p = rgba + 4 * ((size_t)y * w + x);
            if (p[3] == 0) continue;
            if (!any) { grow(f, w, h); any = true; }
            size_t i = (size_t)y * f.w + x;
            bool fresh = !f.present[i];
            uint32_t c;
            std::memcpy(&c, p, 4);
            f.raw[i] = c;
            f.present[i] = mark;
            if (fresh) f.count++;
            bbox_x1 = std::min<uint16_t>(bbox_x1, (uint16_t)x); bbox_y1 = std::min<uint16_t>(bbox_y1, (uint16_t)y);
            bbox_x2 = std::max<uint16_t>(bbox_x2, (uint16_t)x); bbox_y2 = std::max<uint16_t>(bbox_y2, (uint16_t)y);
            if (f.count == 1 && fresh) { f.x = x; f.y = y; }
            else {
                double wt = 1.0 / double(f.count);
                f.x = (1.0 - wt) * f.x + wt * x;
                f.y = (1.0 - wt) * f.y + wt * y;
            }
        }
    }
    identifier++;
    return AM_OK;
}

void Engine::set_seed(unsigned s) {
    seed = s;
    perlin_perm(s, perm_lag);
    perlin_perm(s + 1, perm_slope);
    perlin_perm(s + 2, perm_mx);
    perlin_perm(s + 3, perm_my);
    if (rw) render_set_perlin(rw, perm_lag, perm_slope, perm_mx, perm_my);
}

int Engine::clear() {
    if (running) {
        signal_pause = true;
        signal_stop = true;
        if (th.joinable()) th.join();
        running = false;
        paused = true;
        signal_stop = false;
        signal_pause = false;
    }
    frames.clear();
    identifier = 0;
    worker_identifier = SIZE_MAX;
    bbox_x1 = bbox_y1 = UINT16_MAX;
    bbox_x2 = bbox_y2 = 0;
    state = AM_STATE_BLOB_DETECTION;
    blobs.clear(); blob_real.clear(); perm.clear(); widths.clear();
    Wb = C = 0; N = 0; match_started = false; cost_valid = false;
    fK = fC = 0; fN = 0; f_widths.clear(); f_chain_off.clear(); f_rank.clear(); f_blobs.clear(); f_group.clear();
    f_state = AM_STATE_BLOB_DETECTION;
    f_energy = 0.0;
    if (rw) render_invalidate(rw);
    return AM_OK;
}

// -------------------------------------------------------------- worker ---
void Engine::run() {
    if (device >= 0) cudaSetDevice(device);
    auto start = std::chrono::steady_clock::now();
    while (!signal_stop) {
        if (!signal_pause && !paused) {
            step();
            if (iterations > 0 && --iterations == 0) signal_pause = true;
            if (seconds > 0.0) {
                auto end = std::chrono::steady_clock::now();
                if (std::chrono::duration<double>(end - start).count() > seconds) {
                    signal_pause = true;
                    seconds = 0.0;
                }
            }
        } else {
            paused = true;
            signal_pause = false;
            std::this_thread::sleep_for(std::chrono::microseconds(50));
            start = std::chrono::steady_clock::now();
        }
    }
    running = false;
    signal_stop = false;
    signal_pause = false;
    paused = true;
}

void Engine::start_thread() {
    if (th.joinable()) th.join();
    running = true;
    th = std::thread(&Engine::run, this);
}

int Engine::compute() {
    if (is_busy()) return AM_ERR_BUSY;
    int rc = ensure_streams(this);
    if (rc) return rc;
    if (!running) start_thread();
    paused = false;
    return AM_OK;
}
int Engine::iterate(size_t n) {
    if (is_busy()) return AM_ERR_BUSY;
    int rc = ensure_streams(this);
    if (rc) return rc;
    iterations = n;
    if (!running) start_thread();
    paused = false;
    return AM_OK;
}
int Engine::compute_seconds(double s) {
    if (is_busy()) return AM_ERR_BUSY;
    int rc = ensure_streams(this);
    if (rc) return rc;
    seconds = s;
    if (!running) start_thread();
    paused = false;
    return AM_OK;
}
int Engine::suspend(double timeout) {
    auto t0 = std::chrono::steady_clock::now();
    while (is_busy()) {
        signal_pause = true;
        if (paused) break;
        if (timeout >= 0.0 &&
            std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count() > timeout)
            return AM_ERR_TIMEOUT;
        std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
    return AM_OK;
}

void Engine::step() {
    if (status != AM_OK) return;
    int rc = AM_OK;
    switch (state) {
        case AM_STATE_BLOB_DETECTION:
            rc = detect();
            if (!rc) state = AM_STATE_BLOB_UNIFICATION;
            break;
        case AM_STATE_BLOB_UNIFICATION:
            // In the component regime unify_frame leaves every blob as it is.
            state = AM_STATE_BLOB_MATCHING;
            break;
        case AM_STATE_BLOB_MATCHING: {
            bool done = false;
            if (!match_started) {
                rc = match_init();
                if (!rc && worker_skip) done = true;
            } else if (worker_skip || Wb <= 1) {
                done = true;
            } else {
                rc = match_run(&done);
            }
            if (!rc && done) {
                rc = build_chains();
                if (!rc) state = (C == 0 || N == 0) ? AM_STATE_DONE : AM_STATE_ATOM_MORPHING;
            }
            break;
        }
        case AM_STATE_ATOM_MORPHING:
            if (worker_skip) state = AM_STATE_DONE;
            else rc = refine(active.sweeps, nullptr);
            break;
        default:
            break;
    }
    worker_skip = false;
    if (rc) status = rc;
}

// ------------------------------------------------------------- pipeline --
int Engine::upload_frames() {
    int rc = ensure_streams(this);
    if (rc) return rc;
    K = (uint32_t)frames.size();
    CW = 1; CH = 1;
    for (auto &kv : frames) { CW = std::max(CW, kv.second.w); CH = std::max(CH, kv.second.h); }
    frame_keys.clear();
    size_t fr = (size_t)CW * CH;
    std::vector<uint32_t> raw(fr * std::max<uint32_t>(K, 1), 0);
    std::vector<uint8_t> pr(fr * std::max<uint32_t>(K, 1), 0);
    uint32_t k = 0;
    for (auto &kv : frames) {
        frame_keys.push_back(kv.first);
        const HostFrame &f = kv.second;
        for (uint32_t y = 0; y < f.h; ++y) {
            std::memcpy(&raw[k * fr + (size_t)y * CW], &f.raw[(size_t)y * f.w], f.w * 4);
            std::memcpy(&pr[k * fr + (size_t)y * CW], &f.present[(size_t)y * f.w], f.w);
        }
        ++k;
    }
    size_t n = fr * K;
    if ((rc = d_raw.reserve(std::max<size_t>(n, 1)))) return rc;
    if ((rc = d_present.reserve(std::max<size_t>(n, 1)))) return rc;
    if ((rc = d_stored.reserve(std::max<size_t>(n, 1)))) return rc;
    if ((rc = d_display.reserve(std::max<size_t>(n, 1)))) return rc;
    if ((rc = d_labels.reserve(std::max<size_t>(n, 1)))) return rc;
    if (n) {
        AMG_CUDA(cudaMemcpyAsync(d_raw.p, raw.data(), n * 4, cudaMemcpyHostToDevice, stream));
        AMG_CUDA(cudaMemcpyAsync(d_present.p, pr.data(), n, cudaMemcpyHostToDevice, stream));
    }
    rc = launch_colour(d_raw.p, d_present.p, d_stored.p, d_display.p, n, front.delimiter == AM_HSP, stream);
    if (rc) return rc;
    AMG_CUDA(cudaStreamSynchronize(stream));
    return AM_OK;
}

int Engine::detect() {
    blobs.assign(K, {});
    blob_real.assign(K, 0);
    size_t fr = (size_t)CW * CH;
    for (uint32_t k = 0; k < K; ++k) {
        uint32_t nb = 0;
        int rc = label_components(bw, d_present.p + k * fr, d_stored.p + k * fr, CW, CH, d_labels.p + k * fr, &nb,
                                  stream);
        if (rc) return rc;
        if ((rc = d_stats.reserve(std::max<size_t>((size_t)nb * 7, 7)))) return rc;
        rc = blob_stats(bw, d_labels.p + k * fr, d_stored.p + k * fr, CW, CH, nb, d_stats.p, stream);
        if (rc) return rc;
        std::vector<unsigned long long> st((size_t)nb * 7);
        if (nb) AMG_CUDA(cudaMemcpyAsync(st.data(), d_stats.p, st.size() * 8, cudaMemcpyDeviceToHost, stream));
        AMG_CUDA(cudaStreamSynchronize(stream));
        // The components are blobify's result when every colour distance is
        // within the threshold, nothing is below the minimum size or above
        // the maximum, and blob_number does not stop the merging earlier;
        // otherwise the merge rules run (k_blobs.cu, merge_blobs).
        unsigned long long largest = 0;
        for (uint32_t b = 0; b < nb; ++b) largest = std::max(largest, st[(size_t)b * 7]);
        if (!(active.threshold >= 1.0 && active.min_size <= 1 && active.blob_number <= nb &&
              active.max_size >= largest)) {
            BlobRules br;
            br.threshold = active.threshold;
            br.blob_number = active.blob_number;
            br.min_size = active.min_size;
            br.max_size = active.max_size;
            br.box_samples = active.box_samples;
            br.box_grip = active.box_grip;
            br.seed = (uint32_t)mix64(((uint64_t)seed << 16) ^ k);
            rc = merge_blobs(bw, d_present.p + k * fr, d_stored.p + k * fr, CW, CH, br, d_labels.p + k * fr, &nb,
                             stream);
            if (rc) return rc;
            if ((rc = d_stats.reserve(std::max<size_t>((size_t)nb * 7, 7)))) return rc;
            rc = blob_stats(bw, d_labels.p + k * fr, d_stored.p + k * fr, CW, CH, nb, d_stats.p, stream);
            if (rc) return rc;
            st.assign((size_t)nb * 7, 0);
            if (nb) AMG_CUDA(cudaMemcpyAsync(st.data(), d_stats.p, st.size() * 8, cudaMemcpyDeviceToHost, stream));
            AMG_CUDA(cudaStreamSynchronize(stream));
        }
        std::vector<Blob> &bl = blobs[k];
        bl.resize(nb);
        for (uint32_t b = 0; b < nb; ++b) {
            const unsigned long long *s = &st[(size_t)b * 7];
            double c = (double)s[0];
            bl[b].size = s[0];
            bl[b].x = s[1] / c; bl[b].y = s[2] / c;
            bl[b].r = s[3] / c / 255.0; bl[b].g = s[4] / c / 255.0;
            bl[b].b = s[5] / c / 255.0; bl[b].a = s[6] / c / 255.0;
        }
        blob_real[k] = nb;
    }
    return AM_OK;
}

int Engine::match_init() {
    match_started = true;
    Wb = 0;
    for (auto &b : blobs) Wb = std::max<uint32_t>(Wb, (uint32_t)b.size());
    // Pad every frame with empty "volatile" blobs (thread.cpp:636-647) placed
    // at the frame's mean, colour of the frame's mean.
    uint32_t k = 0;
    for (auto &kv : frames) {
        const HostFrame &f = kv.second;
        Blob v;
        v.size = 0;
        if (f.count) {
            v.x = f.x; v.y = f.y;
            double r = 0, g = 0, b = 0, a = 0, n = 0;
            for (auto &bb : blobs[k]) { r += bb.r * bb.size; g += bb.g * bb.size; b += bb.b * bb.size; a += bb.a * bb.size; n += bb.size; }
            if (n > 0) { v.r = r / n; v.g = g / n; v.b = b / n; v.a = a / n; }
        } else {
            v.x = bbox_x1 <= bbox_x2 ? (bbox_x1 + bbox_x2) / 2.0 : 0.0;
            v.y = bbox_y1 <= bbox_y2 ? (bbox_y1 + bbox_y2) / 2.0 : 0.0;
        }
        while (blobs[k].size() < Wb) blobs[k].push_back(v);
        ++k;
    }
    // Random initial groups, as the reference shuffles each frame's blobs
    // (thread.cpp:649-657).
    perm.assign((size_t)K * Wb, 0);
    std::mt19937_64 rng(0x9e3779b97f4a7c15ULL ^ active_seed_mix());
    for (uint32_t kk = 0; kk < K; ++kk) {
        int32_t *row = &perm[(size_t)kk * Wb];
        std::iota(row, row + Wb, 0);
        std::shuffle(row, row + Wb, rng);
    }
    match_step = 0;
    match_energy = -1.0;
    if (Wb == 0) return AM_OK;
    int rc;
    if ((rc = d_desc.reserve((size_t)K * Wb * 7))) return rc;
    if ((rc = d_perm.reserve((size_t)K * Wb))) return rc;
    if ((rc = d_energy.reserve(1))) return rc;
    std::vector<double> desc((size_t)K * Wb * 7);
    for (uint32_t kk = 0; kk < K; ++kk)
        for (uint32_t b = 0; b < Wb; ++b) {
            const Blob &x = blobs[kk][b];
            double *d = &desc[((size_t)kk * Wb + b) * 7];
            d[0] = (double)x.size; d[1] = x.x; d[2] = x.y; d[3] = x.r; d[4] = x.g; d[5] = x.b; d[6] = x.a;
        }
    AMG_CUDA(cudaMemcpyAsync(d_desc.p, desc.data(), desc.size() * 8, cudaMemcpyHostToDevice, stream));
    AMG_CUDA(cudaMemcpyAsync(d_perm.p, perm.data(), perm.size() * 4, cudaMemcpyHostToDevice, stream));
    AMG_CUDA(cudaStreamSynchronize(stream));
    return AM_OK;
}

unsigned Engine::active_seed_mix() const { return seed; }

int Engine::match_run(bool *done) {
    *done = false;
    MatchArgs a;
    a.desc = d_desc.p;
    a.perm = d_perm.p;
    a.Wb = Wb;
    a.K = K;
    int dx = (int)bbox_x2 - (int)bbox_x1, dy = (int)bbox_y2 - (int)bbox_y1;
    a.bbox_d = bbox_x1 <= bbox_x2 ? (double)(dx * dx + dy * dy) : 0.0;
    if (a.bbox_d <= 0.0) a.bbox_d = 1.0;
    double sum = (double)(active.rgba_w * active.rgba_w + active.size_w * active.size_w + active.xy_w * active.xy_w);
    if (sum > 0) {
        a.w_rgba = (active.rgba_w * active.rgba_w) / sum;
        a.w_size = (active.size_w * active.size_w) / sum;
        a.w_xy = 1.0 - (a.w_rgba + a.w_size);
    } else {
        a.w_rgba = 0.33; a.w_size = 0.33; a.w_xy = 0.34;
    }
    a.sweeps = 64;
    a.key = mix64(((uint64_t)seed << 32) ^ (match_step + 1));
    a.degenerate = active.degeneration;
    a.energy_out = d_energy.p;
    int rc = launch_blob_match(a, stream);
    if (rc) return rc;
    double e = 0;
    AMG_CUDA(cudaMemcpyAsync(&e, d_energy.p, 8, cudaMemcpyDeviceToHost, stream));
    AMG_CUDA(cudaMemcpyAsync(perm.data(), d_perm.p, perm.size() * 4, cudaMemcpyDeviceToHost, stream));
    AMG_CUDA(cudaStreamSynchronize(stream));
    ++match_step;
    // Converged when a whole step of sweeps no longer lowers the energy
    // (the reference stops at zero energy or when told to, thread.cpp:735).
    if (match_energy >= 0.0 && e >= match_energy) *done = true;
    if (e == 0.0 || match_step >= 256) *done = true;
    match_energy = e;
    return AM_OK;
}

std::vector<std::vector<uint32_t>> phases_for(uint32_t K) {
    std::vector<std::vector<uint32_t>> ph;
    if (K == 0) return ph;
    if (K == 1) return {{0}};
    if (K == 2) return {{0}, {1}};
    std::vector<uint32_t> ev, od, last;
    for (uint32_t y = 0; y < K; ++y) {
        if (K % 2 == 1 && y == K - 1) last.push_back(y);
        else if (y % 2 == 0) ev.push_back(y);
        else od.push_back(y);
    }
    ph.push_back(ev);
    ph.push_back(od);
    if (!last.empty()) ph.push_back(last);
    return ph;
}

int Engine::set_chain_layout(const std::vector<uint64_t> &w) {
    ++layout_version;
    local_valid = false;
    guided_on = false;
    lg_state = LG_MEASURE_FULL;
    widths = w;
    C = (uint32_t)w.size();
    chain_off.assign(C + 1, 0);
    pair_off.assign(C + 1, 0);
    singles.clear();
    for (uint32_t c = 0; c < C; ++c) {
        chain_off[c + 1] = chain_off[c] + w[c];
        pair_off[c + 1] = pair_off[c] + w[c] / 2;
        if (w[c] == 1) singles.push_back(chain_off[c]);
    }
    N = chain_off[C];
    int rc;
    if ((rc = d_P.reserve(std::max<uint64_t>(N * K, 1)))) return rc;
    if ((rc = d_chain_off.reserve(C + 1))) return rc;
    if ((rc = d_pair_off.reserve(C + 1))) return rc;
    if ((rc = d_singles.reserve(std::max<size_t>(singles.size(), 1)))) return rc;
    if ((rc = d_phase.reserve(std::max<uint32_t>(K, 1)))) return rc;
    AMG_CUDA(cudaMemcpyAsync(d_chain_off.p, chain_off.data(), (C + 1) * 8, cudaMemcpyHostToDevice, stream));
    AMG_CUDA(cudaMemcpyAsync(d_pair_off.p, pair_off.data(), (C + 1) * 8, cudaMemcpyHostToDevice, stream));
    if (!singles.empty())
        AMG_CUDA(cudaMemcpyAsync(d_singles.p, singles.data(), singles.size() * 8, cudaMemcpyHostToDevice, stream));
    std::vector<uint32_t> ph;
    for (auto &p : phases_for(K)) ph.insert(ph.end(), p.begin(), p.end());
    if (!ph.empty()) AMG_CUDA(cudaMemcpyAsync(d_phase.p, ph.data(), ph.size() * 4, cudaMemcpyHostToDevice, stream));
    AMG_CUDA(cudaStreamSynchronize(stream));
    return AM_OK;
}

int Engine::build_chains() {
    if (!match_started) {
        int rc = match_init();
        if (rc) return rc;
    }
    C = 0;
    N = 0;
    if (Wb == 0 || K == 0) return AM_OK;
    // Empty blobs take positions interpolated between the group's non-empty
    // neighbours (fix_volatiles, thread.cpp:1187-1233).
    std::vector<uint32_t> volxy((size_t)K * Wb, 0);
    std::vector<int32_t> blob_of((size_t)K * Wb, -1);
    std::vector<uint64_t> w(Wb, 0);
    for (uint32_t g = 0; g < Wb; ++g) {
        std::vector<Blob *> col(K);
        for (uint32_t k = 0; k < K; ++k) col[k] = &blobs[k][perm[(size_t)k * Wb + g]];
        if (K > 1) {
            uint32_t i = 0;
            bool started = false;
            std::vector<Blob *> vol;
            Blob *first = nullptr, *prev = nullptr;
            while (true) {
                i = (i + 1) % K;
                Blob *bl = col[i];
                bool empty = bl->size == 0;
                if (!started) {
                    if (empty) { if (i == 0) break; continue; }
                    started = true; first = prev = bl; continue;
                }
                if (empty) { vol.push_back(bl); continue; }
                for (size_t v = 0; v < vol.size(); ++v) {
                    double t = (v + 1.0) / double(vol.size() + 1.0);
                    vol[v]->x = t * bl->x + (1.0 - t) * prev->x;
                    vol[v]->y = t * bl->y + (1.0 - t) * prev->y;
                }
                vol.clear();
                prev = bl;
                if (prev == first) break;
            }
        }
        uint64_t mx = 0;
        for (uint32_t k = 0; k < K; ++k) {
            int32_t b = perm[(size_t)k * Wb + g];
            const Blob &bl = blobs[k][b];
            mx = std::max<uint64_t>(mx, bl.size);
            if ((size_t)b < blob_real[k] && bl.size > 0) blob_of[(size_t)k * Wb + g] = b;
            uint32_t vx = (uint32_t)(uint16_t)std::round(bl.x), vy = (uint32_t)(uint16_t)std::round(bl.y);
            volxy[(size_t)k * Wb + g] = vx | (vy << 16);
        }
        w[g] = mx * active.density;
    }
    int rc = set_chain_layout(w);
    if (rc) return rc;
    // Sort each frame's pixels by (blob, row-major position).
    size_t fr = (size_t)CW * CH;
    uint32_t maxb = 1;
    for (uint32_t k = 0; k < K; ++k) maxb = std::max<uint32_t>(maxb, (uint32_t)blob_real[k]);
    if ((rc = d_sorted.reserve(fr * K))) return rc;
    if ((rc = d_keys.reserve(fr))) return rc;
    if ((rc = d_tk.reserve(fr))) return rc;
    if ((rc = d_tv.reserve(fr))) return rc;
    if ((rc = d_hist.reserve(radix_hist_words(fr)))) return rc;
    if ((rc = d_bstart.reserve((size_t)K * maxb))) return rc;
    if ((rc = d_bsize.reserve((size_t)K * maxb))) return rc;
    if ((rc = d_volxy.reserve((size_t)K * Wb))) return rc;
    if ((rc = d_blob_of.reserve((size_t)K * Wb))) return rc;
    std::vector<uint32_t> bstart((size_t)K * maxb, 0), bsize((size_t)K * maxb, 0);
    std::vector<uint32_t> iota_px(fr);
    std::iota(iota_px.begin(), iota_px.end(), 0u);
    for (uint32_t k = 0; k < K; ++k) {
        uint32_t nb = (uint32_t)blob_real[k];
        uint32_t acc = 0;
        for (uint32_t b = 0; b < nb; ++b) {
            bstart[(size_t)k * maxb + b] = acc;
            bsize[(size_t)k * maxb + b] = (uint32_t)blobs[k][b].size;
            acc += (uint32_t)blobs[k][b].size;
        }
        // keys = labels with absent pixels mapped past the last blob.
        int bits = 1;
        while ((1ull << bits) < (uint64_t)nb + 1) ++bits;
        rc = labels_to_keys(d_labels.p + k * fr, d_keys.p, fr, nb, stream);
        if (rc) return rc;
        AMG_CUDA(cudaMemcpyAsync(d_sorted.p + k * fr, iota_px.data(), fr * 4, cudaMemcpyHostToDevice, stream));
        rc = radix_sort_pairs(d_keys.p, d_sorted.p + k * fr, d_tk.p, d_tv.p, d_hist.p, fr, bits, stream);
        if (rc) return rc;
    }
    AMG_CUDA(cudaMemcpyAsync(d_bstart.p, bstart.data(), bstart.size() * 4, cudaMemcpyHostToDevice, stream));
    AMG_CUDA(cudaMemcpyAsync(d_bsize.p, bsize.data(), bsize.size() * 4, cudaMemcpyHostToDevice, stream));
    AMG_CUDA(cudaMemcpyAsync(d_volxy.p, volxy.data(), volxy.size() * 4, cudaMemcpyHostToDevice, stream));
    AMG_CUDA(cudaMemcpyAsync(d_blob_of.p, blob_of.data(), blob_of.size() * 4, cudaMemcpyHostToDevice, stream));
    ChainBuildArgs cb;
    cb.P = d_P.p; cb.N = N; cb.K = K; cb.C = C; cb.chain_off = d_chain_off.p; cb.blob_of = d_blob_of.p;
    cb.blob_start = d_bstart.p; cb.blob_size = d_bsize.p; cb.maxb = maxb; cb.sorted = d_sorted.p;
    cb.npx = (uint32_t)fr; cb.CW = CW; cb.vol_xy = d_volxy.p;
    cb.seed = mix64(((uint64_t)seed << 16) ^ 0xC4A1);
    rc = launch_chain_build(cb, stream);
    if (rc) return rc;
    uint64_t ex = 0;
    rc = compute_cost(&ex);
    if (rc) return rc;
    cost_exact = ex;
    cost_valid = true;
    return AM_OK;
}

int Engine::compute_cost(uint64_t *exact) {
    int rc;
    if ((rc = d_acc.reserve(8))) return rc;
    if (N == 0 || K == 0) { *exact = 0; return AM_OK; }
    rc = launch_cost(d_P.p, N, K, d_singles.p, (uint32_t)singles.size(), d_acc.p + 2, stream);
    if (rc) return rc;
    unsigned long long v = 0;
    AMG_CUDA(cudaMemcpyAsync(&v, d_acc.p + 2, 8, cudaMemcpyDeviceToHost, stream));
    AMG_CUDA(cudaStreamSynchronize(stream));
    *exact = v;
    return AM_OK;
}

// Guided and learned refinement start with the plain method's cheap uniform
// sweeps, which fix the coarse transport quickly, and switch (once per set of
// chains) to guided sweeps when a block of plain sweeps gains less than
// `guided_switch` of the cost per sweep; from then on the guided proposals
// resolve the local crossings uniform pairs almost never sample.
int Engine::refine(size_t sweeps, uint64_t *gains) {
    if (N == 0 || K == 0 || sweeps == 0) return AM_OK;
    if (active.proposal == AM_PROPOSAL_RANDOM) return refine_plain(sweeps, gains);
    if (active.proposal == AM_PROPOSAL_SCORED) {
        // The pair proposal falls back to plain sweeps until its network is
        // trained, and afterwards whenever plain sweeps gain more cost per
        // second: one call of each is timed, the better runs the next calls
        // (4 when scored won, 16 when plain did), then both are measured again.
        if (!mlp_trained) return refine_plain(sweeps, gains);
        const bool scored = ps_state == PS_MEASURE_SCORED || (ps_state == PS_RUN && ps_scored);
        const uint64_t before = cost_exact;
        const auto t0 = std::chrono::steady_clock::now();
        int rc = scored ? refine_scored(sweeps, gains) : refine_plain(sweeps, gains);
        if (rc) return rc;
        const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        const double rate = (double)(before - cost_exact) / std::max(secs, 1e-9);
        if (ps_state == PS_MEASURE_SCORED) {
            ps_rate = rate;
            ps_state = PS_MEASURE_PLAIN;
        } else if (ps_state == PS_MEASURE_PLAIN) {
            ps_scored = ps_rate > rate;
            ps_state = PS_RUN;
            ps_left = ps_scored ? 4 : 16;
        } else if (--ps_left <= 0) {
            ps_state = PS_MEASURE_SCORED;
        }
        return AM_OK;
    }
    size_t done = 0;
    if (active.guided_switch <= 0.0) guided_on = true;
    while (!guided_on && done < sweeps) {
        size_t b = std::min<size_t>(50, sweeps - done);
        uint64_t before = cost_exact;
        int rc = refine_plain(b, gains ? gains + done : nullptr);
        if (rc) return rc;
        done += b;
        double g = (double)(before - cost_exact);
        if (g < active.guided_switch * (double)b * (double)cost_exact) guided_on = true;
    }
    if (done < sweeps) return refine_guided(sweeps - done, gains ? gains + done : nullptr);
    return AM_OK;
}

int Engine::refine_plain(size_t sweeps, uint64_t *gains) {
    local_valid = false;  // plain sweeps move points without the guided index
    int rc;
    if ((rc = d_acc.reserve(std::max<size_t>(8, 2 * sweeps + 4)))) return rc;
    AMG_CUDA(cudaMemsetAsync(d_acc.p + 4, 0, 2 * sweeps * 8, stream));
    auto ph = phases_for(K);
    for (size_t s = 0; s < sweeps; ++s) {
        uint32_t pofs = 0;
        for (size_t p = 0; p < ph.size(); ++p) {
            SweepArgs a;
            a.P = d_P.p; a.N = N; a.K = K; a.C = C; a.chain_off = d_chain_off.p; a.pair_off = d_pair_off.p;
            a.frames = d_phase.p + pofs; a.nframes = (uint32_t)ph[p].size();
            a.key = sweep_key(seed, sweep_counter, (uint32_t)p);
            a.gain = d_acc.p + 4 + 2 * s; a.accepted = d_acc.p + 5 + 2 * s;
            if (recording_outcomes) {
                a.log_feat = d_rec_feat.p; a.log_label = d_rec_gain.p; a.log_count = d_rec_count.p;
                a.log_cap = rec_cap; a.log_every = outcome_every;
                a.display = d_display.p; a.CW = CW; a.CH = CH;
            }
            if (pair_off[C] > 0) {
                prof.open(stream);
                rc = launch_sweep_random(a, stream);
                if (rc) return rc;
                prof.close(PROF_SWEEP_RANDOM, stream);
            }
            pofs += (uint32_t)ph[p].size();
        }
        ++sweep_counter;
    }
    std::vector<unsigned long long> acc(2 * sweeps);
    AMG_CUDA(cudaMemcpyAsync(acc.data(), d_acc.p + 4, acc.size() * 8, cudaMemcpyDeviceToHost, stream));
    AMG_CUDA(cudaStreamSynchronize(stream));
    for (size_t s = 0; s < sweeps; ++s) {
        cost_exact -= acc[2 * s];
        if (gains) gains[s] = acc[2 * s];
    }
    return AM_OK;
}

// Sweeps of the learned pair proposal: per phase the network scores four
// random partners of every column and mutually best-scored pairs are swapped
// when the exact criterion holds; the gains are exact, as in plain sweeps.
int Engine::refine_scored(size_t sweeps, uint64_t *gains) {
    local_valid = false;
    int rc;
    size_t maxph = 0;
    for (auto &p : phases_for(K)) maxph = std::max(maxph, p.size());
    if (scored_layout != layout_version) {
        if ((rc = d_scored_chain.reserve(std::max<uint64_t>(N, 1)))) return rc;
        if ((rc = launch_chain_ids(d_chain_off.p, C, N, d_scored_chain.p, stream))) return rc;
        scored_layout = layout_version;
    }
    if ((rc = d_sclaim.reserve(std::max<size_t>(N * maxph, 1)))) return rc;
    if ((rc = d_acc.reserve(std::max<size_t>(8, 2 * sweeps + 4)))) return rc;
    AMG_CUDA(cudaMemsetAsync(d_acc.p + 4, 0, 2 * sweeps * 8, stream));
    auto ph = phases_for(K);
    for (size_t s = 0; s < sweeps; ++s) {
        uint32_t pofs = 0;
        for (size_t p = 0; p < ph.size(); ++p) {
            ScoredArgs a;
            a.P = d_P.p; a.N = N; a.K = K; a.C = C; a.chain_off = d_chain_off.p; a.chain_id = d_scored_chain.p;
            a.frames = d_phase.p + pofs; a.nframes = (uint32_t)ph[p].size();
            a.key = sweep_key(seed, sweep_counter, (uint32_t)p) ^ 0x73636f726564ull;
            a.display = d_display.p; a.CW = CW; a.CH = CH;
            a.mlp = d_mlp_dep.p; a.claim = d_sclaim.p;
            a.gain = d_acc.p + 4 + 2 * s; a.accepted = d_acc.p + 5 + 2 * s;
            a.err = d_err.p;
            if (pair_off[C] > 0) {
                prof.open(stream);
                rc = launch_scored_sweep(a, stream);
                if (rc) return rc;
                prof.close(PROF_MLP, stream);
            }
            pofs += (uint32_t)ph[p].size();
        }
        ++sweep_counter;
    }
    std::vector<unsigned long long> acc(2 * sweeps);
    AMG_CUDA(cudaMemcpyAsync(acc.data(), d_acc.p + 4, acc.size() * 8, cudaMemcpyDeviceToHost, stream));
    AMG_CUDA(cudaStreamSynchronize(stream));
    for (size_t s = 0; s < sweeps; ++s) {
        cost_exact -= acc[2 * s];
        if (gains) gains[s] = acc[2 * s];
    }
    return check_err();
}

int Engine::publish_front() {
    ++publish_count;
    fK = K; fC = C; fN = N;
    f_widths = widths; f_chain_off = chain_off; f_keys = frame_keys;
    f_blobs = blobs;
    f_group.assign(K, {});
    f_rank.assign((size_t)K * C, 0);
    for (uint32_t k = 0; k < K && k < blobs.size(); ++k) {
        f_group[k].assign(blobs[k].size(), 0);
        for (uint32_t g = 0; g < Wb && (size_t)k * Wb + g < perm.size(); ++g) {
            int32_t b = perm[(size_t)k * Wb + g];
            if ((size_t)b < f_group[k].size()) f_group[k][b] = (int32_t)g;
            if (g < C) f_rank[(size_t)k * C + g] = b;
        }
    }
    f_state = state;
    if (state == AM_STATE_BLOB_MATCHING) f_energy = match_energy;
    else if (state == AM_STATE_ATOM_MORPHING || state == AM_STATE_DONE) f_energy = cost_valid ? (double)cost_exact : 0.0;
    else f_energy = -1.0;
    if (N && K) {
        int rc;
        // frames in flight read the front chains, ranks and colour tables
        if (rstream) AMG_CUDA(cudaStreamSynchronize(rstream));
        render_quiesce(rw);
        if ((rc = d_Pf.reserve(N * K))) return rc;
        if ((rc = d_chain_off_f.reserve(C + 1))) return rc;
        if ((rc = d_rank_f.reserve((size_t)K * C))) return rc;
        AMG_CUDA(cudaMemcpyAsync(d_Pf.p, d_P.p, N * K * 8, cudaMemcpyDeviceToDevice, stream));
        AMG_CUDA(cudaMemcpyAsync(d_chain_off_f.p, chain_off.data(), (C + 1) * 8, cudaMemcpyHostToDevice, stream));
        AMG_CUDA(cudaMemcpyAsync(d_rank_f.p, f_rank.data(), f_rank.size() * 4, cudaMemcpyHostToDevice, stream));
        // show_blobs colours by blob (morph.cpp:1321-1334): AVERAGE is
        // blob2pixel (create_color of the blob's mean, HSP -> RGB when the
        // delimiter is HSP, morph.cpp:1423-1429); DISTINCT draws three bytes
        // from std::mt19937(group) as the reference does.
        const size_t kc = (size_t)K * C;
        std::vector<uint32_t> col(3 * kc, 0);
        auto cc = [](double v) { return (uint32_t)(int)std::round(v * 255.0) & 255u; };
        for (uint32_t k = 0; k < K; ++k)
            for (uint32_t g = 0; g < C; ++g) {
                const uint32_t b = (uint32_t)f_rank[(size_t)k * C + g];
                if (b >= C) continue;
                if (k < f_blobs.size() && b < f_blobs[k].size()) {
                    const Blob &bl = f_blobs[k][b];
                    const uint32_t st = cc(bl.r) | (cc(bl.g) << 8) | (cc(bl.b) << 16) | (cc(bl.a) << 24);
                    col[(size_t)k * C + b] = st;
                    col[kc + (size_t)k * C + b] = hsp_to_rgb_host(st);
                }
                std::mt19937 gen(g);
                std::uniform_int_distribution<unsigned char> byte(0, 255);
                const uint32_t r = byte(gen), gg = byte(gen), bb = byte(gen);
                col[2 * kc + (size_t)k * C + b] = r | (gg << 8) | (bb << 16) | 0xFF000000u;
            }
        if ((rc = d_blob_col.reserve(std::max<size_t>(col.size(), 1)))) return rc;
        AMG_CUDA(cudaMemcpyAsync(d_blob_col.p, col.data(), col.size() * 4, cudaMemcpyHostToDevice, stream));
        AMG_CUDA(cudaStreamSynchronize(stream));
    }
    if (rw) render_invalidate(rw);
    return AM_OK;
}

int Engine::synchronize() {
    if (is_busy()) return AM_ERR_BUSY;
    int rc = ensure_streams(this);
    if (rc) return rc;
    if (status) {
        int s = status;
        status = AM_OK;
        return s;
    }
    active = front;
    if (identifier != worker_identifier) {
        state = AM_STATE_BLOB_DETECTION;
        blobs.clear(); blob_real.clear(); perm.clear(); widths.clear();
        Wb = C = 0; N = 0; match_started = false; cost_valid = false; sweep_counter = 0;
        rc = upload_frames();
        if (rc) return rc;
        worker_identifier = identifier;
    }
    rc = publish_front();
    if (rc) return rc;
    if (skip_state) {
        worker_skip = true;
        skip_state = false;
    }
    return AM_OK;
}

// Pinned host memory is mapped into the GPU's address space: the device
// address of [p, p + bytes) when the driver reports p as mapped host memory
// whose whole allocation covers the range, else nullptr.  Pageable memory,
// a short pinned buffer or a failed query leave the frame on the copy path.
// One driver query (cuPointerGetAttributes answers pointers it does not
// know with empty attributes, not an error).
uint8_t *mapped_host_range(uint8_t *p, size_t bytes) {
    using GetAttrs = CUresult (*)(unsigned, CUpointer_attribute *, void **, CUdeviceptr);
    static GetAttrs get_attrs = [] {
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuPointerGetAttributes", &fn, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            fn = nullptr;
        return reinterpret_cast<GetAttrs>(fn);
    }();
    if (!get_attrs) return nullptr;
    CUpointer_attribute which[4] = {CU_POINTER_ATTRIBUTE_MEMORY_TYPE, CU_POINTER_ATTRIBUTE_DEVICE_POINTER,
                                    CU_POINTER_ATTRIBUTE_RANGE_START_ADDR, CU_POINTER_ATTRIBUTE_RANGE_SIZE};
    unsigned int type = 0;
    CUdeviceptr dev = 0, start = 0;
    size_t size = 0;
    void *data[4] = {&type, &dev, &start, &size};
    const CUdeviceptr hp = (CUdeviceptr)(uintptr_t)p;
    if (get_attrs(4, which, data, hp) != CUDA_SUCCESS) return nullptr;
    if (type != CU_MEMORYTYPE_HOST || !dev || !size) return nullptr;
    if (hp < start || hp - start > size || size - (hp - start) < bytes) return nullptr;
    return reinterpret_cast<uint8_t *>((uintptr_t)dev);
}

int Engine::render(double time, uint8_t *out, bool out_dev) {
    int rc = ensure_streams(this);
    if (rc) return rc;
    size_t bytes = (size_t)width * height * 4;
    if (bytes == 0) return AM_OK;
    uint8_t *dst = out;
    // An atom frame into mapped (pinned) host memory is stored there by the
    // resolve kernel directly, over the CPU-GPU link, while it resolves.
    bool direct = false;
    if (!out_dev && fN && fK && front.fluidsteps == 0) {
        if (uint8_t *d = mapped_host_range(out, bytes)) {
            dst = d;
            direct = true;
        }
    }
    if (!out_dev && !direct) {
        if ((rc = d_frame.reserve(bytes))) return rc;
        dst = d_frame.p;
    }
    double integ;
    double t = std::modf(time, &integ);
    if (t < 0.0) t += 1.0;
    if (fN == 0 || fK == 0) {
        // No chains yet: the key frame's blob pixels as they are
        // (morph.cpp:469-475), or nothing before blobs exist.
        AMG_CUDA(cudaMemsetAsync(dst, 0, bytes, rstream));
        size_t f = (size_t)(t * fK);
        bool have_blobs = f < f_blobs.size() && !f_blobs[f].empty();
        if (fK && f < fK && have_blobs) {
            rc = copy_keyframe(f, dst);
            if (rc) return rc;
        }
    } else if (front.fluidsteps > 0) {
        rc = render_fluid(t, dst);
        if (rc) return rc;
    } else {
        RenderScene sc;
        uint64_t key = 0;
        frame_scene(t, sc, &key);
        // a host frame of a sequence played in order: the next frame is
        // binned beside this one's resolve, ready when the caller asks for it
        FrameAhead nx;
        double tn = 0.0;
        const bool ahead = !out_dev && next_time(t, &tn);
        if (ahead) {
            nx.time = tn;
            frame_scene(tn, nx.sc, &nx.frame_key);
        }
        rc = render_frame(rw, sc, t, key, dst, rstream, ahead ? &nx : nullptr);
        if (rc) return rc;
    }
    // A device frame is left in flight on the render stream (am_get_stream);
    // a host frame is copied out (unless stored there directly) and waited for.
    if (!out_dev) {
        if (!direct) AMG_CUDA(cudaMemcpyAsync(out, dst, bytes, cudaMemcpyDeviceToHost, rstream));
        AMG_CUDA(cudaStreamSynchronize(rstream));
    } else {
        AMG_CUDA(cudaGetLastError());
    }
    return AM_OK;
}

// The pixels of blob `blob` of the key frame at `time` drawn alone
// (morph::get_pixels(blob, t), morph.cpp:452-678), in the reference's order:
// ascending position, or with a feather its outer layers one by one and then
// the rest.  Before chains exist, the blob's own key-frame pixels.
int Engine::blob_pixels(size_t blob, double time, std::vector<std::pair<uint32_t, uint32_t>> &out) {
    out.clear();
    int rc = ensure_streams(this);
    if (rc) return rc;
    double integ;
    double t = std::modf(time, &integ);
    if (t < 0.0) t += 1.0;
    const size_t nk = frames.size();
    if (nk == 0) return AM_ERR_NOT_FOUND;
    const size_t f = std::min<size_t>((size_t)(t * nk), nk - 1);
    if (f >= f_blobs.size() || blob >= f_blobs[f].size()) return AM_ERR_NOT_FOUND;
    if (fN == 0 || fK == 0) {
        const size_t fr = (size_t)CW * CH;
        if (!d_labels.p || d_labels.n < (f + 1) * fr) return AM_ERR_STATE;
        std::vector<int32_t> lab(fr);
        std::vector<uint32_t> disp(fr);
        AMG_CUDA(cudaMemcpy(lab.data(), d_labels.p + f * fr, fr * 4, cudaMemcpyDeviceToHost));
        AMG_CUDA(cudaMemcpy(disp.data(), d_display.p + f * fr, fr * 4, cudaMemcpyDeviceToHost));
        for (size_t q = 0; q < fr; ++q)
            if (lab[q] == (int32_t)blob) out.emplace_back((uint32_t)((q / CW) << 16 | (q % CW)), disp[q]);
        return AM_OK;
    }
    const size_t npx = (size_t)width * height;
    if (npx == 0) return AM_OK;
    if ((rc = d_frame.reserve(npx * 4))) return rc;
    if ((rc = d_aux.reserve(npx))) return rc;
    RenderScene sc;
    sc.K = fK; sc.C = fC; sc.N = fN; sc.CW = CW; sc.CH = CH; sc.width = width; sc.height = height;
    sc.bbox[0] = bbox_x1; sc.bbox[1] = bbox_y1; sc.bbox[2] = bbox_x2; sc.bbox[3] = bbox_y2;
    sc.motion = front.motion; sc.fading = front.fading; sc.density = front.density;
    sc.P = d_Pf.p; sc.chain_off = d_chain_off_f.p; sc.display = d_display.p; sc.rank = d_rank_f.p;
    sc.motion_noise = front.motion_noise;
    render_options(sc);
    sc.pipeline = 0;
    sc.only_rank = (uint32_t)blob;
    sc.aux = d_aux.p;
    const uint64_t key = f < f_keys.size() ? f_keys[f] : 0;
    if ((rc = render_frame(rw, sc, t, key, d_frame.p, rstream))) return rc;
    std::vector<uint32_t> rgba(npx);
    std::vector<uint8_t> aux(npx);
    AMG_CUDA(cudaMemcpyAsync(rgba.data(), d_frame.p, npx * 4, cudaMemcpyDeviceToHost, rstream));
    AMG_CUDA(cudaMemcpyAsync(aux.data(), d_aux.p, npx, cudaMemcpyDeviceToHost, rstream));
    AMG_CUDA(cudaStreamSynchronize(rstream));
    const uint32_t F = sc.feather;
    for (uint32_t code = 1; code <= F + 1; ++code)
        for (size_t q = 0; q < npx; ++q)
            if (aux[q] == code || (F == 0 && aux[q]))
                out.emplace_back((uint32_t)((q / width) << 16 | (q % width)), rgba[q]);
    return AM_OK;
}

// Every atom's position at time `time` as the render places it (host xy,
// 2 words per atom column); returns the atom count.
int Engine::positions(double time, int32_t *xy, size_t cap, size_t *count) {
    *count = fN;
    if (!xy || cap < fN || fN == 0 || fK == 0) return AM_OK;
    int rc = ensure_streams(this);
    if (rc) return rc;
    if ((rc = d_pos.reserve(2 * fN))) return rc;
    double integ;
    double t = std::modf(time, &integ);
    if (t < 0.0) t += 1.0;
    RenderScene sc;
    sc.K = fK; sc.C = fC; sc.N = fN; sc.CW = CW; sc.CH = CH; sc.width = width; sc.height = height;
    sc.bbox[0] = bbox_x1; sc.bbox[1] = bbox_y1; sc.bbox[2] = bbox_x2; sc.bbox[3] = bbox_y2;
    sc.motion = front.motion; sc.fading = front.fading; sc.density = front.density;
    sc.P = d_Pf.p; sc.chain_off = d_chain_off_f.p; sc.display = d_display.p; sc.rank = d_rank_f.p;
    sc.motion_noise = front.motion_noise;
    render_options(sc);
    const size_t f = (size_t)(t * fK);
    const uint64_t key = f < f_keys.size() ? f_keys[f] : 0;
    if ((rc = render_positions(rw, sc, t, key, d_pos.p, rstream))) return rc;
    AMG_CUDA(cudaMemcpyAsync(xy, d_pos.p, fN * 8, cudaMemcpyDeviceToHost, rstream));
    AMG_CUDA(cudaStreamSynchronize(rstream));
    return AM_OK;
}

// n frames into consecutive host frames.  A pinned buffer covering all of
// them is mapped: every frame is resolved straight into it, the frames
// pipelined as device frames are, and the call waits once at the end.  Other
// host memory takes the frames one at a time (render's copy path).
int Engine::render_many_host(const double *ts, size_t n, uint8_t *out) {
    const size_t fsz = (size_t)width * height * 4;
    if (n == 0 || fsz == 0) return AM_OK;
    int rc = ensure_streams(this);
    if (rc) return rc;
    uint8_t *dev = (fN && fK && front.fluidsteps == 0) ? mapped_host_range(out, n * fsz) : nullptr;
    for (size_t i = 0; i < n; ++i) {
        rc = dev ? render(ts[i], dev + i * fsz, true) : render(ts[i], out + i * fsz, false);
        if (rc) return rc;
    }
    if (dev) AMG_CUDA(cudaStreamSynchronize(rstream));
    return AM_OK;
}

// The frame after t in a sequence of host frames t_i = get_time(i, n)
// (morph.cpp:1522-1538; without `finite` i / n, with it i / (n - 1) scaled
// by 1 - 1/F), when the previous host frame was t_(i-1) of the same
// sequence: the order the reference's demo writes frames in
// (demo/main.cpp:177-190).  The prediction is exact or absent: the time is
// recomputed with get_time's own arithmetic and both known terms are
// checked bit for bit.
bool Engine::next_time(double t, double *tn) {
    const double prev = last_host_t;
    last_host_t = t;
    if (!(t > prev)) return false;  // the first frame, a repeat, a jump back or the cycle's wrap
    const size_t F = frames.size();
    const bool fin = front.finite;
    if (fin && F == 0) return false;
    const double scale = fin ? 1.0 - 1.0 / double(F) : 1.0;
    const double steps = std::round(scale / (t - prev));  // n (or n - 1 with finite)
    if (!(steps >= 2.0 && steps <= 1e9)) return false;
    const double di = std::round(t / scale * steps);
    if (!(di >= 1.0 && di <= steps)) return false;
    const size_t i = (size_t)di, n = (size_t)steps + (fin ? 1 : 0);
    auto at = [&](size_t k) {
        if (!fin) return double(k) / double(n);
        double v = double(k) / double(n - 1);
        v *= 1.0 - (1.0 / double(F));
        return v;
    };
    if (at(i) != t || at(i - 1) != prev) return false;
    if (fin && i + 1 > n - 1) return false;  // a finite sequence ends
    double nxt = at(i + 1), integ;
    nxt = std::modf(nxt, &integ);  // i + 1 == n wraps to the cycle's start
    *tn = nxt;
    return true;
}

// The published chains' scene for an atom frame at normalised time t in
// [0, 1), and the key frame of its pair.
void Engine::frame_scene(double t, RenderScene &sc, uint64_t *key) const {
    sc.K = fK; sc.C = fC; sc.N = fN; sc.CW = CW; sc.CH = CH; sc.width = width; sc.height = height;
    sc.bbox[0] = bbox_x1; sc.bbox[1] = bbox_y1; sc.bbox[2] = bbox_x2; sc.bbox[3] = bbox_y2;
    sc.motion = front.motion; sc.fading = front.fading; sc.density = front.density;
    sc.P = d_Pf.p; sc.chain_off = d_chain_off_f.p; sc.display = d_display.p; sc.rank = d_rank_f.p;
    sc.motion_noise = front.motion_noise;
    render_options(sc);
    // host frames too: the tile plan for the next frame then runs on the
    // second stream, after the resolve the caller waits for
    sc.pipeline = render_pipeline ? 1u : 0u;
    sc.bin_ctas = render_bin_ctas;
    sc.resolve_ctas = render_resolve_ctas;
    const size_t f = (size_t)(t * fK);
    *key = f < f_keys.size() ? f_keys[f] : 0;
}

// Render options of the front settings (feather, keep_background,
// show_blobs) and the tables they read.
void Engine::render_options(RenderScene &sc) const {
    sc.feather = (uint32_t)std::min<size_t>(front.feather, kMaxFeather);
    sc.keep_background = front.keep_background ? 1u : 0u;
    sc.show_blobs = front.show_blobs;
    sc.present = d_present.p;
    sc.perm = render_perm(rw);
    const size_t kc = (size_t)fK * fC;
    sc.blob_col = nullptr;
    if (d_blob_col.p && front.show_blobs == AM_AVERAGE)
        sc.blob_col = d_blob_col.p + (front.delimiter == AM_HSP ? kc : 0);
    else if (d_blob_col.p && front.show_blobs == AM_DISTINCT)
        sc.blob_col = d_blob_col.p + 2 * kc;
    if (!sc.blob_col) sc.show_blobs = AM_TEXTURE;
}

// The fluid frame (morph::get_pixels with fluid steps, morph.cpp:1417): the
// particles are stepped to time t and drawn.  Like the reference, every call
// advances the simulation, so frames are meant to be rendered in order.
int Engine::render_fluid(double t, uint8_t *dst) {
    const double sp = front.fluid_sparseness;
    const uint32_t gsx = (uint32_t)std::lround(width * sp) + 20, gsy = (uint32_t)std::lround(height * sp) + 20;
    if (!fluid || fluid->n != fN || fluid_gsx != gsx || fluid_gsy != gsy) {
        // particle count = sum of the chains' maximum surfaces = N at density 1
        // (morph.cpp:234-260); a new count or grid restarts the simulation
        if (fluid) fluid_destroy(fluid);
        if (fmorph) fluid_morph_destroy(fmorph);
        fluid = fluid_create(gsx, gsy, (uint32_t)fN);
        fmorph = fluid_morph_create();
        if (!fluid || !fmorph) { set_error("fluid: out of device memory"); return AM_ERR_NOMEM; }
        fluid_gsx = gsx;
        fluid_gsy = gsy;
        fluid_front = UINT64_MAX;
    }
    int rc;
    if (fluid_front != publish_count) {
        if ((rc = d_fchain_id.reserve(std::max<uint64_t>(fN, 1)))) return rc;
        if ((rc = launch_chain_ids(d_chain_off_f.p, fC, fN, d_fchain_id.p, rstream))) return rc;
        // surface of each chain's blob per key frame (blob_before/after ->surface.size())
        surf_host.assign((size_t)fK * fC, 0);
        for (uint32_t k = 0; k < fK && k < f_blobs.size(); ++k)
            for (uint32_t c = 0; c < fC; ++c) {
                const int32_t b = f_rank[(size_t)k * fC + c];
                if (b >= 0 && (size_t)b < f_blobs[k].size()) surf_host[(size_t)k * fC + c] = (uint32_t)f_blobs[k][b].size;
            }
        if ((rc = d_surf.reserve(std::max<size_t>(surf_host.size(), 1)))) return rc;
        AMG_CUDA(cudaMemcpyAsync(d_surf.p, surf_host.data(), surf_host.size() * 4, cudaMemcpyHostToDevice, rstream));
        fluid_front = publish_count;
    }
    FluidFrame fr;
    fr.sc.K = fK; fr.sc.C = fC; fr.sc.N = fN; fr.sc.CW = CW; fr.sc.CH = CH; fr.sc.width = width; fr.sc.height = height;
    fr.sc.bbox[0] = bbox_x1; fr.sc.bbox[1] = bbox_y1; fr.sc.bbox[2] = bbox_x2; fr.sc.bbox[3] = bbox_y2;
    fr.sc.motion = front.motion; fr.sc.fading = front.fading; fr.sc.density = front.density;
    fr.sc.motion_noise = front.motion_noise;
    fr.sc.P = d_Pf.p; fr.sc.chain_off = d_chain_off_f.p; fr.sc.display = d_display.p; fr.sc.rank = d_rank_f.p;
    render_options(fr.sc);
    const size_t f = std::min<size_t>((size_t)(t * fK), fK - 1);
    fr.time = t;
    fr.frame_key = f < f_keys.size() ? f_keys[f] : f;
    fr.sparseness = sp;
    fr.chain_id = d_fchain_id.p;
    fr.surf = d_surf.p;
    fr.surf_host = surf_host.data();
    fr.chain_off_host = f_chain_off.data();
    fr.perm = render_perm(rw);
    fr.fluidsteps = front.fluidsteps;
    fr.seed_key = mix64((uint64_t)seed << 24 ^ 0x666c7569ull);
    fr.version = publish_count;
    fr.rw = rw;
    return fluid_morph_frame(fmorph, fluid, fr, dst, rstream);
}

int Engine::import_chains(size_t k_, size_t c_, const uint64_t *w, const uint64_t *pts, const int32_t *order) {
    if (is_busy()) return AM_ERR_BUSY;
    if (k_ != frames.size() || !w || (!pts && c_)) return AM_ERR_ARG;
    int rc = ensure_streams(this);
    if (rc) return rc;
    active = front;
    if (identifier != worker_identifier) {
        rc = upload_frames();
        if (rc) return rc;
        worker_identifier = identifier;
    }
    K = (uint32_t)k_;
    Wb = (uint32_t)c_;
    perm.assign((size_t)K * Wb, 0);
    blobs.assign(K, std::vector<Blob>(Wb));
    blob_real.assign(K, Wb);
    for (uint32_t k = 0; k < K; ++k)
        for (uint32_t b = 0; b < Wb; ++b) {
            int32_t g = order ? order[(size_t)k * Wb + b] : (int32_t)b;
            if (g < 0 || (uint32_t)g >= Wb) return AM_ERR_ARG;
            perm[(size_t)k * Wb + g] = (int32_t)b;
        }
    match_started = true;
    rc = set_chain_layout(std::vector<uint64_t>(w, w + c_));
    if (rc) return rc;
    // The blobs behind the imported chains: a chain's blob at key frame k is
    // its original points there (HAS_PIXEL | HAS_FLUID, thread.cpp:800-830),
    // whose count is the blob's surface and whose mean is its position.
    for (uint32_t k = 0; k < K; ++k)
        for (uint32_t g = 0; g < Wb && g < C; ++g) {
            Blob &b = blobs[k][perm[(size_t)k * Wb + g]];
            b = Blob();
            double sx = 0.0, sy = 0.0;
            for (uint64_t x = chain_off[g]; x < chain_off[g + 1]; ++x) {
                const uint64_t p = pts[(uint64_t)k * N + x];
                if (((p >> 48) & 3u) != 3u) continue;
                ++b.size;
                sx += (double)(p & 0xFFFFu);
                sy += (double)((p >> 16) & 0xFFFFu);
            }
            if (b.size) { b.x = sx / (double)b.size; b.y = sy / (double)b.size; }
        }
    if (N * K) AMG_CUDA(cudaMemcpyAsync(d_P.p, pts, N * K * 8, cudaMemcpyHostToDevice, stream));
    uint64_t ex = 0;
    rc = compute_cost(&ex);
    if (rc) return rc;
    cost_exact = ex;
    cost_valid = true;
    state = AM_STATE_ATOM_MORPHING;
    return publish_front();
}

int Engine::export_chains(uint64_t *w, uint64_t *pts, int32_t *order) {
    if (w) for (uint32_t c = 0; c < fC; ++c) w[c] = f_widths[c];
    if (pts && fN * fK) {
        AMG_CUDA(cudaMemcpyAsync(pts, d_Pf.p, fN * fK * 8, cudaMemcpyDeviceToHost, rstream));
        AMG_CUDA(cudaStreamSynchronize(rstream));
    }
    if (order)
        for (uint32_t k = 0; k < fK; ++k)
            for (uint32_t g = 0; g < fC; ++g) order[(size_t)k * fC + f_rank[(size_t)k * fC + g]] = (int32_t)g;
    return AM_OK;
}

int Engine::copy_keyframe(size_t f, uint8_t *dst) {
    size_t fr = (size_t)CW * CH;
    return launch_keyframe_copy(d_display.p + f * fr, d_present.p + f * fr, CW, CH, width, height, dst, rstream);
}

int Engine::ensure_local_index() {
    if (local_valid) return AM_OK;
    int rc;
    uint32_t ncells = ((CW + 1) / 2) * ((CH + 1) / 2);
    size_t maxph = 0;
    for (auto &p : phases_for(K)) maxph = std::max(maxph, p.size());
    if ((rc = d_slot_pt.reserve(N * K))) return rc;
    if ((rc = d_col.reserve(N * K))) return rc;
    if ((rc = d_slot_of.reserve(N * K))) return rc;
    if ((rc = d_cell_start.reserve((size_t)K * (ncells + 1)))) return rc;
    if ((rc = d_chain_id.reserve(N))) return rc;
    if ((rc = d_chain_w1.reserve(std::max<uint32_t>(C, 1)))) return rc;
    if ((rc = d_slot_ch.reserve(N * K))) return rc;
    if ((rc = d_claim.reserve(N * maxph))) return rc;
    if ((rc = d_pgain.reserve(N * maxph))) return rc;
    if ((rc = d_lprop.reserve(N * maxph))) return rc;
    if ((rc = d_sv.reserve(N * K))) return rc;
    if ((rc = d_hot.reserve(N * K))) return rc;
    AMG_CUDA(cudaMemsetAsync(d_hot.p, 0, N * K, stream));
    if ((rc = d_lk.reserve(N))) return rc;
    if ((rc = d_lv.reserve(N))) return rc;
    if ((rc = d_tk.reserve(N))) return rc;
    if ((rc = d_tv.reserve(N))) return rc;
    if ((rc = d_hist.reserve(radix_hist_words(N)))) return rc;
    std::vector<uint8_t> w1(std::max<uint32_t>(C, 1), 0);
    for (uint32_t c = 0; c < C; ++c) w1[c] = widths[c] <= 1;
    AMG_CUDA(cudaMemcpyAsync(d_chain_w1.p, w1.data(), w1.size(), cudaMemcpyHostToDevice, stream));
    lix.slot_pt = d_slot_pt.p; lix.col = d_col.p; lix.slot_of = d_slot_of.p; lix.cell_start = d_cell_start.p;
    lix.chain_id = d_chain_id.p; lix.chain_w1 = d_chain_w1.p; lix.slot_ch = d_slot_ch.p; lix.sv = d_sv.p;
    rc = local_index_build(lix, d_P.p, N, K, CW, CH, d_chain_off.p, C, d_lk.p, d_lv.p, d_tk.p, d_tv.p, d_hist.p,
                           stream);
    if (rc) return rc;
    local_valid = true;
    return AM_OK;
}

// The learned form runs its gate only while it pays: a gated sweep scans a
// quarter of the regions (default keep) and costs about three quarters of a
// full guided sweep, so it must keep at least that share of a full sweep's
// gain.  The policy alternates one measured full block and one measured
// gated block, then runs four blocks of the better one, and measures again.
void Engine::learned_gate_next(double gain_per_s) {
    switch (lg_state) {
    case LG_MEASURE_FULL:
        lg_full_rate = gain_per_s;
        lg_state = LG_MEASURE_GATED;
        break;
    case LG_MEASURE_GATED:
        lg_state = gain_per_s >= lg_full_rate ? LG_GATED : LG_FULL;
        lg_left = 4;
        break;
    default:
        if (--lg_left <= 0) lg_state = LG_MEASURE_FULL;
        break;
    }
}

int Engine::refine_guided(size_t sweeps, uint64_t *gains) {
    if (active.proposal == AM_PROPOSAL_LEARNED && !mlp_ready()) {
        set_error("the learned proposal needs a trained network (am_train_proposal / am_set_proposal_weights)");
        return AM_ERR_STATE;
    }
    int rc = ensure_local_index();
    if (rc) return rc;
    size_t maxph = 0;
    for (auto &p : phases_for(K)) maxph = std::max(maxph, p.size());
    if (active.proposal == AM_PROPOSAL_LEARNED) {
        if ((rc = mlp_init())) return rc;
        if ((rc = d_sel.reserve(N * maxph))) return rc;
        if ((rc = d_nsel.reserve(1))) return rc;
        if (recording && (rc = d_rec_idx.reserve((N * maxph + 31) / 32 + 1))) return rc;
    }
    // Sweeps run in blocks; the learned form decides per block whether its
    // gate runs (see learned_gate_next).
    constexpr size_t kBlock = 10;
    if ((rc = d_acc.reserve(std::max<size_t>(8, 2 * kBlock + 4)))) return rc;
    auto ph = phases_for(K);
    const bool learned = active.proposal == AM_PROPOSAL_LEARNED;
    for (size_t done = 0; done < sweeps;) {
        const size_t nb = std::min(kBlock, sweeps - done);
        const bool gated = learned && (recording || !active.learned_adaptive || lg_state == LG_MEASURE_GATED ||
                                       lg_state == LG_GATED);
        const auto t_block = std::chrono::steady_clock::now();
        AMG_CUDA(cudaMemsetAsync(d_acc.p + 4, 0, 2 * nb * 8, stream));
        for (size_t s = 0; s < nb; ++s) {
            uint32_t pofs = 0;
            for (size_t p = 0; p < ph.size(); ++p) {
                LocalArgs a;
                a.P = d_P.p; a.N = N; a.K = K; a.frames = d_phase.p + pofs; a.nframes = (uint32_t)ph[p].size();
                a.slot_pt = lix.slot_pt; a.col = lix.col; a.slot_of = lix.slot_of; a.cell_start = lix.cell_start;
                a.ncx = lix.ncx; a.ncy = lix.ncy; a.ncells = lix.ncells; a.slot_ch = lix.slot_ch;
                a.cap = active.local_target;
                a.self_cap = active.local_self; a.nrandom = active.local_random; a.chain_off = d_chain_off.p;
                a.key = mix64(((uint64_t)seed << 40) ^ (sweep_counter << 4) ^ p ^ 0x5bd1e995ULL);
                a.claim = d_claim.p; a.prop = d_lprop.p; a.pgain = d_pgain.p; a.sv = d_sv.p; a.hot = d_hot.p;
                a.single_chain = C == 1;
                a.gain = d_acc.p + 4 + 2 * s; a.accepted = d_acc.p + 5 + 2 * s;
                if (gated) {
                    a.mlp = d_mlp_dep.p; a.keep = (float)active.learned_keep; a.err = d_err.p;
                    a.cost_scale = log1pf((float)((double)cost_exact / ((double)N * K) / kGainScale));
                    a.sel_out = d_sel.p; a.nsel_out = d_nsel.p;
                    a.explore = (uint32_t)mix64(sweep_counter ^ (uint64_t)p);
                    if (recording) {
                        a.rec_feat = d_rec_feat.p; a.rec_gain = d_rec_gain.p; a.rec_count = d_rec_count.p;
                        a.rec_cap = rec_cap; a.rec_idx = d_rec_idx.p;
                    }
                }
                prof.open(stream);
                if (gated) rc = launch_learned_phase(a, stream);
                else rc = launch_local_phase(a, stream);
                if (rc) return rc;
                prof.close(gated ? PROF_MLP : PROF_SWEEP_LOCAL, stream);
                pofs += (uint32_t)ph[p].size();
            }
            ++sweep_counter;
        }
        std::vector<unsigned long long> acc(2 * nb);
        AMG_CUDA(cudaMemcpyAsync(acc.data(), d_acc.p + 4, acc.size() * 8, cudaMemcpyDeviceToHost, stream));
        AMG_CUDA(cudaStreamSynchronize(stream));
        double block_gain = 0.0;
        for (size_t s = 0; s < nb; ++s) {
            cost_exact -= acc[2 * s];
            block_gain += (double)acc[2 * s];
            if (gains) gains[done + s] = acc[2 * s];
        }
        if (learned && !recording) {
            const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_block).count();
            learned_gate_next(block_gain / std::max(dt, 1e-9));
        }
        done += nb;
    }
    return AM_OK;
}

}  // namespace amg
