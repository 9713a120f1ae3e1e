// Host side of one morph handle: the GB300 counterpart of am::morph
// (morph.h:9-145) and its worker am::thread (thread.h:9-130).
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <chrono>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

#include "common.cuh"
#include "kernels.h"

namespace amg {

// The device address of pinned, CUDA-mapped host memory [p, p + bytes) when
// one allocation covers it, else null.
uint8_t *mapped_host_range(uint8_t *p, size_t bytes);

struct Params {  // defaults of morph.h:97-119
    unsigned delimiter = AM_HSP;
    double threshold = 1.0;
    size_t blob_number = 1, max_size = SIZE_MAX, min_size = 1, box_samples = 10;
    uint16_t box_grip = UINT16_MAX;
    unsigned rgba_w = 1, size_w = 1, xy_w = 1;
    size_t degeneration = 0;
    uint16_t density = 1;
    size_t threads = 0, cycle_length = 1000, feather = 0;
    bool keep_background = false, finite = false;
    unsigned fluidsteps = 0, show_blobs = AM_TEXTURE;
    unsigned motion = AM_SPLINE, fading = AM_PERLIN;
    unsigned proposal = AM_PROPOSAL_RANDOM;
    size_t sweeps = 1;
    // guided-refinement tunables (am_set_tuning; chosen by the autotuner)
    uint32_t local_self = 12, local_target = 8, local_random = 2;
    double learned_keep = 0.25;  // fraction of regions the learned gate lets scan
    bool learned_adaptive = true;  // run the gate only while it pays (learned_gate_next)
    double guided_switch = 1e-3;  // plain -> guided when a plain sweep gains less than this fraction
    double motion_noise = 0.0;
    double fluid_sparseness = 1.0;  // solver grid units per pixel (the reference's sparseness)
};

struct HostFrame {
    uint32_t w = 0, h = 0;                // canvas extent of this frame
    std::vector<uint32_t> raw;            // RGBA as given, row-major w*h
    std::vector<uint8_t> present;         // 0 absent, 1 stored as given, 2 stored as HSP
    size_t count = 0;
    double x = 0, y = 0, r = 0, g = 0, b = 0, a = 0;  // running means (morph.cpp:318-334)
};

struct Blob {
    uint64_t size = 0;
    double x = 0, y = 0, r = 0, g = 0, b = 0, a = 0;  // means; colours 0..1 of the stored value
};

template <class T>
struct DBuf {
    T *p = nullptr;
    size_t n = 0;
    DBuf() = default;
    DBuf(const DBuf &) = delete;
    DBuf &operator=(const DBuf &) = delete;
    ~DBuf() { release(); }
    int reserve(size_t count) {
        if (count <= n) return AM_OK;
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
        if (count == 0) return AM_OK;
        cudaError_t e = cudaMalloc(&p, count * sizeof(T));
        if (e != cudaSuccess) {
            cudaGetLastError();  // the failed allocation's pending error, so the caller's retry can succeed
            set_error(std::string("cudaMalloc: ") + cudaGetErrorString(e));
            p = nullptr;
            return AM_ERR_NOMEM;
        }
        n = count;
        return AM_OK;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
};

// Frames refined together (never adjacent): K=2 {0},{1}; even K evens, odds;
// odd K evens except the last, odds, the last.
std::vector<std::vector<uint32_t>> phases_for(uint32_t K);

class Engine {
  public:
    Engine();
    ~Engine();

    // front-end (morph) state
    Params front;
    std::map<size_t, HostFrame> frames;
    uint16_t bbox_x1 = UINT16_MAX, bbox_y1 = UINT16_MAX, bbox_x2 = 0, bbox_y2 = 0;
    uint16_t width = 0, height = 0;
    size_t identifier = 0;
    bool skip_state = false;
    unsigned seed = 0;
    int perm_lag[512], perm_slope[512], perm_mx[512], perm_my[512];  // Perlin maps: seed, +1, +2, +3

    int add_pixel(size_t f, uint16_t x, uint16_t y, uint32_t rgba);
    int add_pixels(size_t f, const uint8_t *rgba, uint32_t w, uint32_t h);
    int add_frame(size_t f);
    void set_seed(unsigned s);
    int clear();

    // worker control (thread.h:42-53, thread.cpp:113-206)
    int compute();
    int iterate(size_t n);
    int compute_seconds(double s);
    int suspend(double timeout);  // timeout < 0: no limit
    bool is_busy() const { return running && !paused; }
    int synchronize();

    // worker pipeline state (touched only by the worker or while paused)
    Params active;
    unsigned state = AM_STATE_BLOB_DETECTION;
    bool worker_skip = false;
    size_t worker_identifier = SIZE_MAX;
    uint32_t K = 0, CW = 0, CH = 0;
    std::vector<uint64_t> frame_keys;
    std::vector<std::vector<Blob>> blobs;  // per key frame; matched frames padded with volatile blobs
    std::vector<size_t> blob_real;         // real (non-volatile) blob count per frame
    uint32_t Wb = 0;                       // blob-map width = chain count
    std::vector<int32_t> perm;             // [K][Wb] blob of group g in frame k
    bool match_started = false;
    double match_energy = -1.0;
    uint64_t match_step = 0;
    uint32_t C = 0;
    uint64_t N = 0;
    std::vector<uint64_t> widths, chain_off, pair_off, singles;
    uint64_t sweep_counter = 0;
    uint64_t layout_version = 0;           // bumped whenever the chain layout changes
    uint64_t cost_exact = 0;               // exact cost after the last refinement step
    bool cost_valid = false;

    // front copy of the results (what rendering reads, like morph's own copy)
    uint32_t fK = 0, fC = 0;
    uint64_t fN = 0;
    std::vector<uint64_t> f_widths, f_chain_off, f_keys;
    std::vector<int32_t> f_rank;           // [K][C] composite rank of group g
    std::vector<std::vector<Blob>> f_blobs;
    std::vector<std::vector<int32_t>> f_group;  // group of blob b of frame k
    unsigned f_state = AM_STATE_BLOB_DETECTION;
    double f_energy = 0.0;

    // device
    int device = 0;
    cudaStream_t stream = nullptr, rstream = nullptr;
    DBuf<uint32_t> d_raw, d_stored, d_display;
    DBuf<uint8_t> d_present;
    DBuf<int32_t> d_labels;
    DBuf<uint64_t> d_P, d_Pf, d_chain_off, d_pair_off, d_chain_off_f, d_singles;
    DBuf<int32_t> d_rank_f;
    // [3][K][C] draw colours of the b-th blob of key frame k for show_blobs:
    // AVERAGE as stored, AVERAGE converted HSP -> RGB, DISTINCT
    DBuf<uint32_t> d_blob_col;
    DBuf<uint32_t> d_phase;
    DBuf<unsigned long long> d_acc;        // [0] gain, [1] accepted, [2] cost
    DBuf<unsigned long long> d_stats;
    DBuf<double> d_desc, d_energy;
    DBuf<int32_t> d_perm;
    DBuf<uint32_t> d_sorted, d_keys, d_tk, d_tv, d_hist, d_bstart, d_bsize, d_volxy;
    DBuf<int32_t> d_blob_of;
    DBuf<uint8_t> d_frame;                 // host-output staging frame
    // guided refinement index (valid while only guided sweeps touch P)
    LocalIndex lix;
    bool local_valid = false;
    DBuf<uint64_t> d_slot_pt;
    DBuf<uint32_t> d_col, d_slot_of, d_cell_start, d_chain_id, d_slot_ch, d_lprop, d_lk, d_lv;
    DBuf<uint8_t> d_chain_w1;
    DBuf<unsigned long long> d_claim, d_pgain, d_nsel;
    DBuf<uint64_t> d_sv;
    DBuf<uint8_t> d_hot;
    DBuf<uint32_t> d_sel, d_rec_idx;
    int ensure_local_index();

    Prof prof;
    RenderWork *rw = nullptr;
    // fluid path of the render (step_fluid + draw_fluid)
    FluidDev *fluid = nullptr;
    FluidMorph *fmorph = nullptr;
    uint32_t fluid_gsx = 0, fluid_gsy = 0;
    uint64_t publish_count = 0, fluid_front = UINT64_MAX;
    DBuf<uint32_t> d_fchain_id, d_surf;
    std::vector<uint32_t> surf_host;
    int render_fluid(double t, uint8_t *dst);
    void render_options(RenderScene &sc) const;
    void frame_scene(double t, RenderScene &sc, uint64_t *key) const;  // atom frame at t in [0, 1)
    bool next_time(double t, double *tn);  // the next host frame of a get_time sequence
    double last_host_t = -1.0;             // time of the last host frame (next_time)
    BlobWork *bw = nullptr;
    uint8_t *h_pinned = nullptr;
    size_t h_pinned_n = 0;

    // pipeline steps
    void step();
    int upload_frames();
    int detect();
    int match_init();
    int match_run(bool *done);
    int build_chains();
    int refine(size_t sweeps, uint64_t *gains);
    int compute_cost(uint64_t *exact);
    int compute_cost_noalloc(uint64_t *exact);  // noalloc.cu: static scratch, no device allocation
    int publish_front();
    int render(double t, uint8_t *out, bool out_dev);
    int render_many_host(const double *ts, size_t n, uint8_t *out);
    int positions(double time, int32_t *xy, size_t cap, size_t *count);
    DBuf<int32_t> d_pos;                   // position readout
    // morph::get_pixels(blob, t): (y << 16 | x, RGBA) in the reference's order
    int blob_pixels(size_t blob, double time, std::vector<std::pair<uint32_t, uint32_t>> &out);
    DBuf<uint8_t> d_aux;                   // per-pixel layer codes of a blob drawn alone
    int import_chains(size_t K, size_t C, const uint64_t *w, const uint64_t *pts, const int32_t *order);
    int export_chains(uint64_t *w, uint64_t *pts, int32_t *order);
    int set_chain_layout(const std::vector<uint64_t> &w);
    int refine_guided(size_t sweeps, uint64_t *gains);
    int refine_plain(size_t sweeps, uint64_t *gains);
    // learned pair proposal (AM_PROPOSAL_SCORED): outcome log of the plain
    // sweeps, per-column chain ids and claims of the scored sweeps
    int refine_scored(size_t sweeps, uint64_t *gains);
    int record_outcomes(size_t cap, uint32_t every);
    bool recording_outcomes = false;
    enum { PS_MEASURE_SCORED, PS_MEASURE_PLAIN, PS_RUN };
    int ps_state = PS_MEASURE_SCORED, ps_left = 0;
    bool ps_scored = true;
    double ps_rate = 0.0;
    uint32_t outcome_every = 1;
    DBuf<uint32_t> d_scored_chain;
    DBuf<unsigned long long> d_sclaim;
    uint64_t scored_layout = UINT64_MAX;
    bool guided_on = false;                // the guided phase of the current chains has started
    // learned form: when its gate runs (learned_gate_next)
    enum { LG_MEASURE_FULL, LG_MEASURE_GATED, LG_GATED, LG_FULL };
    int lg_state = LG_MEASURE_FULL, lg_left = 0;
    bool render_pipeline = true;           // render tuning "render_pipeline"
    uint32_t render_bin_ctas = 0, render_resolve_ctas = 0;  // "render_bin_ctas", "render_resolve_ctas" (0: all that fit)
    double lg_full_rate = 0.0;
    void learned_gate_next(double gain_per_s);
    int copy_keyframe(size_t f, uint8_t *dst);
    unsigned active_seed_mix() const;
    int status = AM_OK;                    // first failure inside the worker
    bool mlp_ready() const { return mlp_trained || recording; }
    bool mlp_trained = false;

    // proposal network (engine_mlp.cpp)
    DBuf<float> d_mlp_master, d_mlp_dep, d_mlp_grad, d_adam_m, d_adam_v, d_mlp_loss, d_rec_feat, d_rec_gain;
    DBuf<float> d_io_a, d_io_b;
    DBuf<unsigned long long> d_rec_count;
    DBuf<int> d_err;
    uint64_t rec_cap = 0, adam_t = 0;
    bool recording = false;
    int mlp_init();
    int record_swaps(size_t cap);
    size_t recorded_swaps(float *feat, float *gains, size_t cap);
    int train_proposal(const float *feat, const float *gains, size_t n, size_t epochs, double lr, float *loss_out);
    int train_recorded(size_t epochs, double lr, float *loss_out);
    int train_device(const float *feat, const float *gains, size_t n, size_t epochs, double lr, float *loss_out);
    int proposal_weights(float *w, size_t count, bool set);
    int proposal_forward(const float *feat, size_t n, float *out);
    int proposal_grad(const float *feat, const float *target, size_t n, float *grad, float *loss);
    int check_err();
    int ensure_streams_public();

  private:
    void run();
    void start_thread();
    std::thread th;
    std::atomic<bool> running{false}, paused{true}, signal_pause{false}, signal_stop{false};
    std::atomic<size_t> iterations{0};
    std::atomic<double> seconds{0.0};
};

}  // namespace amg
