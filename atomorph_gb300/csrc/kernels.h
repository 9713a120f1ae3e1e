// Host-callable launch wrappers of the atomorph_gb300 kernels.  Every wrapper
// enqueues on the given stream and returns an AM_* status.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include <algorithm>

#include "../../include/atomorph_gb300.h"

namespace amg {

struct Prof;

// ---- k_colour.cu
int launch_colour(const uint32_t *raw, const uint8_t *present, uint32_t *stored, uint32_t *display, size_t n,
                  int display_hsp, cudaStream_t s);
int launch_hsp_probe(const uint32_t *in, uint32_t *out, size_t n, int dir, cudaStream_t s);

// ---- k_chains.cu
// Exact atom cost: out += sum over atoms i, frames j of
// d(P[j][i], P[(j+1)%K][i]) (thread.cpp:1109-1125), atoms of width-1 chains
// excluded via the `single` list.
int launch_cost(const uint64_t *P, uint64_t N, uint32_t K, const uint64_t *single, uint32_t nsingle,
                unsigned long long *out, cudaStream_t s);

struct SweepArgs {
    uint64_t *P;                 // [K][N] chain points
    uint64_t N;
    uint32_t K;
    uint32_t C;                  // chains
    const uint64_t *chain_off;   // [C+1] atom offsets of the chains
    const uint64_t *pair_off;    // [C+1] prefix sums of floor(width/2)
    const uint32_t *frames;      // frames updated by this phase
    uint32_t nframes;
    uint64_t key;                // random key of this (sweep, phase)
    unsigned long long *gain;    // += exact cost decrease
    unsigned long long *accepted;
    // Optional outcome log for the learned pair proposal: a hashed sample of
    // 1 in log_every proposals writes its pair features ([cap][10]) and
    // whether the swap lowers the cost (1 when c1 > c2, else 0).
    float *log_feat = nullptr, *log_label = nullptr;
    unsigned long long *log_count = nullptr;
    uint64_t log_cap = 0;
    uint32_t log_every = 1;
    const uint32_t *display = nullptr;  // [K][CH][CW] colours the features read
    uint32_t CW = 0, CH = 0;
};
// One phase of the plain refinement: for every chain and every frame of the
// phase, a uniformly random perfect matching of the chain's columns; each pair
// is swapped when the reference's criterion c1 >= c2 holds
// (thread.cpp:1014-1039).
int launch_sweep_random(const SweepArgs &a, cudaStream_t s);

// ---- the learned pair proposal (k_mlp.cu): every column of the phase's
// frames draws kScoredCandidates random partners in its chain, the network
// scores the pairs, each column claims its best-scored partner, and mutually
// claimed pairs are swapped when the exact criterion holds (c1 >= c2,
// thread.cpp:1014-1022).
constexpr int kScoredCandidates = 4;
struct ScoredArgs {
    uint64_t *P;
    uint64_t N;
    uint32_t K, C;
    const uint64_t *chain_off;          // [C+1]
    const uint32_t *chain_id;           // [N] chain of each column
    const uint32_t *frames;
    uint32_t nframes;
    uint64_t key;
    const uint32_t *display;
    uint32_t CW, CH;
    const float *mlp;                   // deployed network
    unsigned long long *claim;          // [nframes][N], zero on entry
    unsigned long long *gain, *accepted;
    int *err;
};
int launch_scored_sweep(const ScoredArgs &a, cudaStream_t s);

// ---- k_batch.cu: many jobs' plain sweeps in one persistent launch
struct BatchJob {
    uint64_t *P;                 // the job's [K][N] chain points
    uint64_t N;
    uint32_t K, C;
    const uint64_t *chain_off, *pair_off;
    const uint32_t *frames;      // the job's phase frames, phases concatenated
    uint32_t ph_off[3], ph_n[3]; // per phase: offset into frames and frame count (0 = no such phase)
    unsigned seed;
    uint64_t sweep0;             // the job's sweep counter when the launch starts
    uint64_t pairs;              // pair_off[C]
};
struct BatchArgs {
    const BatchJob *jobs;
    uint32_t njobs;
    const uint32_t *ch_job;      // chunk -> job
    const uint64_t *ch_start;    // first pair of the chunk (within its frame)
    const uint32_t *ch_count;    // pairs in the chunk
    const uint32_t *ch_fi;       // the chunk's frame within the job's phase
    uint32_t ch_off[4];          // chunks of phase p: [ch_off[p], ch_off[p+1])
    uint32_t nphase;             // phases of the longest schedule (<= 3)
    uint32_t sweeps;
    unsigned long long *gains;   // [njobs][sweeps] exact cost decrease, zeroed before the launch
    unsigned *bar;               // [0] arrivals, [1] generation, [2] abort; zeroed before the launch
    int *err;
};
int batch_max_ctas_per_sm(uint32_t threads, int *out);
// Cooperative launch of `grid` CTAs (all co-resident) running b.sweeps sweeps.
int launch_batch_sweeps(const BatchArgs &b, uint32_t grid, uint32_t threads, cudaStream_t s);

// ---- k_local.cu: guided refinement (spatially local candidates)
struct LocalIndex {
    uint32_t ncx = 0, ncy = 0, ncells = 0;   // 2x2-pixel cells over the canvas
    uint64_t *slot_pt = nullptr;             // [K][N] points sorted by cell (static)
    uint32_t *col = nullptr;                 // [K][N] column holding slot s
    uint32_t *slot_of = nullptr;             // [K][N] slot held by column x
    uint32_t *cell_start = nullptr;          // [K][ncells+1]
    uint64_t *sv = nullptr;                  // [K][N] target sum p + n of the column at slot s
    uint32_t *chain_id = nullptr;            // [N]
    uint8_t *chain_w1 = nullptr;             // [C] 1 for width-1 chains
    uint32_t *slot_ch = nullptr;             // [K][N] chain of the column at slot s, kNoChain for width-1 chains
};
// Swaps stay within a chain and a slot's point never moves, so the chain of
// the column at a slot is fixed for the life of the index.
constexpr uint32_t kNoChain = 0xFFFFFFFFu;
struct LocalArgs {
    uint64_t *P;
    uint64_t N;
    uint32_t K;
    const uint32_t *frames;
    uint32_t nframes;
    const uint64_t *slot_pt;
    uint32_t *col, *slot_of;
    const uint32_t *cell_start;
    uint32_t ncx, ncy, ncells;
    const uint32_t *slot_ch;                 // [K][N] chain of the column at each slot (kNoChain: width 1)
    uint32_t cap;                            // candidates from the target cell
    uint32_t self_cap = 12;                  // candidates from the column's own neighbourhood
    uint32_t nrandom = 2;                    // uniform random candidates of the same chain
    const uint64_t *chain_off = nullptr;     // [C+1]
    uint64_t key;                            // random key of this (sweep, phase)
    uint64_t *sv = nullptr;                  // [K][N] target sum of the column at each slot (kept current)
    bool single_chain = false;               // C == 1: no chain lookups
    unsigned long long *claim;               // [nframes][N] by slot
    uint32_t *prop;                          // [nframes][N] proposed partner slot, by proposer slot
    unsigned long long *pgain;               // [nframes][N] exact gain of the proposal
    unsigned long long *gain, *accepted;
    uint8_t *hot = nullptr;                  // [K][N] gain bucket of each slot's last scan
    const uint32_t *sel = nullptr;           // proposing slots (t = fi*N + s) when gated,
    const unsigned long long *nsel = nullptr;//   their count,
    bool sel_groups = false;                 //   and whether entries are 32-slot regions (t / 32)
    // learned proposal only
    const float *mlp = nullptr;              // deployed network (MlpLayout)
    float keep = 0.25f;                      // fraction of the regions of each 128-region tile the network lets scan
    uint32_t explore = 0;                    // rotates the regions scanned regardless of score (1 in 8)
    float cost_scale = 0.f;                  // log1p(mean column cost / kGainScale)
    uint32_t *sel_out = nullptr;             // gate output list
    unsigned long long *nsel_out = nullptr;
    float *rec_feat = nullptr;               // optional sample log: features [cap][10]
    float *rec_gain = nullptr;               //   and the summed best gains the full scan found [cap]
    uint32_t *rec_idx = nullptr;             // [nframes*N/32] record row of each region or ~0
    unsigned long long *rec_count = nullptr;
    uint64_t rec_cap = 0;
    int *err = nullptr;                      // bounded-wait failure flag
};

// Gains enter the network and its targets as log1p(gain / kGainScale):
// kGainScale = (16 px)^2 in (1/256 px)^2.
constexpr float kGainScale = 4096.f * 4096.f;
// log2 bucket of a gain (0 = no improving partner found), 1..63.
__host__ __device__ __forceinline__ uint8_t gain_bucket(int64_t g) {
    if (g <= 0) return 0;
#ifdef __CUDA_ARCH__
    return (uint8_t)(64 - __clzll(g));
#else
    int b = 0;
    while (g) { ++b; g >>= 1; }
    return (uint8_t)b;
#endif
}

// ---- k_mlp.cu: the proposal network 10 -> 64 -> 64 -> 1 (ReLU)
// Deployed layout (floats): W1 bf16 [64][16] as 512 floats, W2 bf16 [64][64]
// as 2048 floats, b1[64], b2[64], w3[64], b3 — see MlpLayout.
constexpr int kMlpIn = 10, kMlpHid = 64;
constexpr int kMlpMasterParams = kMlpHid * kMlpIn + kMlpHid + kMlpHid * kMlpHid + kMlpHid + kMlpHid + 1;  // 4929
constexpr int kMlpDeployedFloats = 512 + 2048 + 64 + 64 + 64 + 4;
// Packs fp32 master parameters (W1[64][10], b1, W2[64][64], b2, w3, b3) into
// the deployed bf16/fp32 layout.
int mlp_deploy(const float *master, float *deployed, cudaStream_t s);
// One optimisation step over n samples: forward + backward on tensor cores,
// gradients reduced into grad (kMlpMasterParams floats), Adam on master.
int mlp_train_step(const float *feat, const float *target, uint64_t n, float *master, float *deployed, float *grad,
                   float *adam_m, float *adam_v, uint64_t t, float lr, float *loss_sum, int *err, cudaStream_t s);
// Forward only (scores for n samples), for tests and the gradient check.
int mlp_forward(const float *feat, uint64_t n, const float *deployed, float *out, int *err, cudaStream_t s);
// Gradient of the mean squared error over n samples (no update).
int mlp_grad(const float *feat, const float *target, uint64_t n, const float *deployed, float *grad,
             float *loss_sum, int *err, cudaStream_t s);
// ---- batched guided refinement (k_local.cu): every job's guided sweeps in
// one persistent cooperative launch; per phase the claims of all jobs are
// cleared, all proposals made, all winners applied, with grid barriers
// between the stages.  Each job uses its own keys and index, so the result
// is bit-identical to its own guided sweeps (refine with AM_PROPOSAL_LOCAL
// once the guided phase has started).
struct BatchLocalJob {
    LocalArgs a;                 // the job's guided index and arrays (frames, key, gain set per phase)
    const uint32_t *frames;      // the job's phase frames, phases concatenated
    uint32_t ph_off[3], ph_n[3];
    unsigned seed;
    uint64_t sweep0;
};
struct BatchLocalArgs {
    const BatchLocalJob *jobs;
    const uint32_t *ch_job, *ch_fi, *ch_count;  // chunk -> job, frame within the phase, slots
    const uint64_t *ch_start;    // first slot of the chunk
    uint32_t ch_off[4];
    uint32_t nphase, sweeps;
    unsigned long long *gains;   // [njobs][sweeps], zeroed before the launch
    unsigned *bar;
    int *err;
};
int launch_batch_local(const BatchLocalArgs &b, uint32_t grid, uint32_t threads, cudaStream_t s);
int batch_local_max_ctas_per_sm(uint32_t threads, int *out);

int local_index_build(LocalIndex &ix, const uint64_t *P, uint64_t N, uint32_t K, uint32_t CW, uint32_t CH,
                      const uint64_t *chain_off, uint32_t C, uint32_t *keys, uint32_t *vals, uint32_t *tk,
                      uint32_t *tv, uint32_t *hist, cudaStream_t s);
// One guided phase: proposals of every slot, disjoint apply.
int launch_local_phase(const LocalArgs &a, cudaStream_t s);
int launch_local_propose(const LocalArgs &a, cudaStream_t s);  // a.sel/a.nsel: listed slots only
int launch_local_apply(const LocalArgs &a, cudaStream_t s);
// Learned proposal phase (k_mlp.cu): the network scores every 32-slot region
// from cheap features of its slots on tensor cores, the best-scored `keep`
// fraction of each 128-region tile is listed, and only listed regions run the
// guided candidate scan (exact gains, disjoint apply as above).
int launch_learned_phase(const LocalArgs &a, cudaStream_t s);

// Stable LSD radix sort of (key, value) u32 pairs on the low `bits` key bits.
// tmp buffers must hold n elements each; hist needs radix_hist_words(n).
size_t radix_hist_words(size_t n);
int radix_sort_pairs(uint32_t *keys, uint32_t *vals, uint32_t *tmp_keys, uint32_t *tmp_vals, uint32_t *hist,
                     size_t n, int bits, cudaStream_t s);
// keys[i] = labels[i] >= 0 ? labels[i] : nb (absent pixels sort last).
int labels_to_keys(const int32_t *labels, uint32_t *keys, size_t n, uint32_t nb, cudaStream_t s);
// Exclusive scan of n u32 in place (single CTA; setup-sized arrays).
int launch_scan_u32(uint32_t *a, size_t n, uint32_t *total, cudaStream_t s);

struct ChainBuildArgs {
    uint64_t *P;                  // [K][N] output
    uint64_t N;
    uint32_t K;
    uint32_t C;
    const uint64_t *chain_off;    // [C+1]
    const int32_t *blob_of;       // [K][C] blob index (within frame) of group g, -1 = volatile
    const uint32_t *blob_start;   // [K][maxb] start of blob b's pixels in sorted[k]
    const uint32_t *blob_size;    // [K][maxb]
    uint32_t maxb;
    const uint32_t *sorted;       // [K][npx] pixel indices sorted by (blob, row-major)
    uint32_t npx;                 // pixels per frame canvas
    uint32_t CW;                  // canvas width
    const uint32_t *vol_xy;       // [K][C] rounded centre of volatile blobs (x | y << 16)
    uint64_t seed;
};
// init_morph (thread.cpp:770-848): surface points in row-major order,
// duplicates drawn from a random permutation with random fractions.
int launch_chain_build(const ChainBuildArgs &a, cudaStream_t s);

// ---- k_render.cu
struct RenderScene {
    uint32_t K, C;
    uint64_t N;
    uint32_t CW, CH;              // key-frame canvas
    uint32_t width, height;       // output resolution
    uint32_t bbox[4];
    uint32_t motion, fading, density;
    const uint64_t *P;            // [K][N]
    const uint64_t *chain_off;    // [C+1]
    const uint32_t *display;      // [K][CH][CW] RGB colour read by get_pixel
    const int32_t *rank;          // [K][C] composite rank of group g in frame k
    uint32_t pipeline = 1;        // a frame's binning may run beside the previous frame's resolve
    // render options (morph.h:67-70)
    uint32_t feather = 0;         // outer layers of each blob faded (TEXTURE blobs)
    uint32_t keep_background = 0; // key frames cross-faded under the blobs
    uint32_t show_blobs = 0;      // AM_TEXTURE, AM_AVERAGE or AM_DISTINCT
    const uint8_t *present = nullptr;   // [K][CH][CW] 1 where the key frame has a pixel
    const uint32_t *blob_col = nullptr; // [K][C] AVERAGE / DISTINCT colour (RGB) of the b-th blob of frame k
    const int *perm = nullptr;          // [2][512] Perlin permutations (lag, slope) for the background
    double motion_noise = 0.0;          // Perlin motion perturbation amplitude in px (0: off)
    // One blob alone (morph::get_pixels(blob, t), morph.cpp:452-678): only
    // records of this composite rank are drawn, every pixel they reach keeps
    // its mean colour (alpha 0 included) and aux[pixel] gets 1 + its feather
    // layer (feather + 1 inside, 0 where the blob has no pixel).
    uint32_t only_rank = 0xFFFFFFFFu;
    uint8_t *aux = nullptr;             // device, width * height
    // Co-resident CTAs per SM the binning and the resolve may take (0: as
    // many as fit): capping one leaves room on every SM for the other
    // kernel of the pipelined frames.
    uint32_t bin_ctas = 0, resolve_ctas = 0;
};
// Largest feather the frame render supports (three 32-px tile rings).
constexpr uint32_t kMaxFeather = 96;
// HSP -> RGB of one stored colour on the host (color.cpp:71-178).
uint32_t hsp_to_rgb_host(uint32_t c);
struct RenderWork;                // per-handle scratch (k_render.cu)
RenderWork *render_work_create();
void render_work_destroy(RenderWork *w);
void render_set_prof(RenderWork *w, Prof *p);
Prof *render_prof(RenderWork *w);  // the timer render_set_prof installed (or null)
// Uploads the Perlin permutations: lag map (seed), slope map (seed + 1) and
// the motion perturbation's x and y maps (seed + 2, seed + 3), [4][512].
int render_set_perlin(RenderWork *w, const int *perm_lag, const int *perm_slope, const int *perm_mx,
                      const int *perm_my);
// Renders the frame at normalised time `time` into out (device, width*height*4).
// A frame render_frame may bin after the frame it renders, beside that
// frame's resolve, for the call expected next (frames played in order); the
// next call uses it when it asks for exactly that time and scene.
struct FrameAhead {
    RenderScene sc;
    double time;
    uint64_t frame_key;
};
int render_frame(RenderWork *w, const RenderScene &sc, double time, uint64_t frame_key, uint8_t *out,
                 cudaStream_t s, const FrameAhead *ahead = nullptr);
// Every atom's position words (x, y) at normalised time `time` into xy
// (device, 2 * N int32; -1 where the atom is not drawn), as render_frame
// places them.
int render_positions(RenderWork *w, const RenderScene &sc, double time, uint64_t frame_key, int32_t *xy,
                     cudaStream_t s);
// Writes key frame colours (display[CH][CW]) of present, non-transparent
// pixels into a width*height RGBA8 frame (rendering before chains exist).
int launch_keyframe_copy(const uint32_t *display, const uint8_t *present, uint32_t CW, uint32_t CH,
                         uint32_t width, uint32_t height, uint8_t *out, cudaStream_t s);
// Drops cached per-key-frame-pair data (chains or settings changed).
void render_invalidate(RenderWork *w);
// Heavy tiles of the morph's recent frames (tiles resolved in row bands by
// helper CTAs): the count the last frame that had any recorded (0: none
// yet) and the helper CTAs of the last resolve launched.  Waits for the
// binning stream, whose tile plans record the counts.  w may be null (no
// GPU work yet): zeros.
void render_heavy_tiles(RenderWork *w, uint32_t *tiles, uint32_t *helpers);
// Waits for the render work's own binning stream (frames resolve on the
// caller's render stream; their binning may still be running on it).
void render_quiesce(RenderWork *w);
// One morph's frame in a batched render (render_frames_batch).
struct RenderJob {
    RenderWork *w;
    RenderScene sc;
    double time;          // normalised time in [0, 1)
    uint64_t frame_key;   // key frame of the pair at `time`
    uint8_t *out;         // device, width * height * 4
};
// Frames of several morphs on stream s: the binning, the resolve and the next
// tile plan of up to 32 frames each run as one launch; frames that cannot
// (no chains, tile grids above the fused limit, one blob alone) are rendered
// one by one on s.  Every frame equals render_frame's for its morph.  Each
// morph's own render streams must be idle.
// Two-stream form of render_frames_batch for consecutive times: bs runs the
// pair preparation, binning and next tile plans, s the resolves; binned[g]
// orders launch group g (up to 32 frames) between them, and the plans wait
// for prev_resolved (recorded on s after the previous time's resolves, the
// last readers of the slots the plans fill; null for the first time).
struct BatchPipe {
    cudaStream_t bs;
    const cudaEvent_t *binned;
    uint32_t groups;
    cudaEvent_t prev_resolved;
};
int render_frames_batch(const RenderJob *jobs, size_t n, cudaStream_t s, const BatchPipe *pipe = nullptr);

// ---- k_fluid.cu: FluidModel::step in FP32
struct FluidDev;
FluidDev *fluid_create(uint32_t gsx, uint32_t gsy, uint32_t n);
void fluid_destroy(FluidDev *f);
int fluid_set(FluidDev *f, const double *state, cudaStream_t s);  // n x 18 doubles (oracle order)
int fluid_get(FluidDev *f, double *state, cudaStream_t s);
struct FluidMorph;
// Source and destination columns of every particle's last update (host, 2n).
int fluid_morph_links(FluidMorph *m, uint32_t *out, size_t n, cudaStream_t s);
int fluid_step(FluidDev *f, uint64_t steps_left, double freedom_radius, cudaStream_t s, Prof *prof);
// nsteps steps; step k runs with steps_left = last_steps_left + (nsteps - 1 - k).
int fluid_run(FluidDev *f, uint32_t nsteps, uint64_t last_steps_left, double freedom_radius, cudaStream_t s,
              Prof *prof);

// ---- k_fluid_morph.cu: the morph's fluid path (step_fluid + draw_fluid)
struct FluidMorph;
struct FluidFrame {
    RenderScene sc;                   // published chains, key frames, output
    double time;                      // normalised global time
    uint64_t frame_key;               // index of the pair's first key frame
    double sparseness;                // solver grid units per pixel
    const uint32_t *chain_id;         // [N] chain of each column (device)
    const uint32_t *surf;             // [K][C] surface of each chain's blob (device)
    const uint32_t *surf_host;        // the same on the host
    const uint64_t *chain_off_host;   // [C+1]
    const int *perm;                  // Perlin lag / slope permutations (device)
    uint32_t fluidsteps;
    uint64_t seed_key;
    uint64_t version;                 // changes whenever the published chains change
    RenderWork *rw;                   // frame arithmetic tables
};
FluidMorph *fluid_morph_create();
void fluid_morph_destroy(FluidMorph *m);
// Steps the particles to the frame (management, update, solver) and draws
// it into out (device, width * height RGBA8).
int fluid_morph_frame(FluidMorph *m, FluidDev *fl, const FluidFrame &fr, uint8_t *out, cudaStream_t s);
// draw_fluid of the particles as they are (tests and the standalone solver):
// `feather` outward layers; bg_img (device [height][width] RGBA8, or null)
// turns keep_background on with that background.
int fluid_render_only(FluidDev *fl, uint32_t width, uint32_t height, double sparseness, const uint32_t *bbox,
                      double t, uint32_t feather, const uint32_t *bg_img, uint8_t *out, cudaStream_t s);
int launch_chain_ids(const uint64_t *chain_off, uint32_t C, uint64_t N, uint32_t *out, cudaStream_t s);
const int *render_perm(RenderWork *w);

// ---- k_blobs.cu
struct BlobWork;
BlobWork *blob_work_create();
void blob_work_destroy(BlobWork *w);
// 4-connected components of one key frame's present pixels: labels (blob
// index by first pixel in row-major order, -1 absent) and per-blob exact sums
// {count, sum x, sum y, sum r, sum g, sum b, sum a} of the stored colour.
// blobify / unify settings (morph.h:53-58).
struct BlobRules {
    double threshold = 1.0;
    size_t blob_number = 1, min_size = 1, max_size = SIZE_MAX, box_samples = 100;
    uint32_t box_grip = 65535;
    uint32_t seed = 0;
};
// Blobs by the reference's merge rules outside the component regime (parallel
// agglomeration rounds, then dust unification); labels and count as
// label_components gives them.
int merge_blobs(BlobWork *w, const uint8_t *present, const uint32_t *stored, uint32_t CW, uint32_t CH,
                const BlobRules &p, int32_t *labels, uint32_t *nblobs, cudaStream_t s);
int label_components(BlobWork *w, const uint8_t *present, const uint32_t *stored, uint32_t CW, uint32_t CH,
                     int32_t *labels, uint32_t *nblobs, cudaStream_t s);
int blob_stats(BlobWork *w, const int32_t *labels, const uint32_t *stored, uint32_t CW, uint32_t CH,
               uint32_t nblobs, unsigned long long *stats, cudaStream_t s);

struct MatchArgs {
    const double *desc;   // [K][Wb][7] blob descriptors (size, x, y, r, g, b, a)
    int32_t *perm;        // [K][Wb] blob of group g in frame k (in/out)
    uint32_t Wb, K;
    double bbox_d, w_rgba, w_size, w_xy;
    uint32_t sweeps;
    uint64_t key;
    size_t degenerate;
    double *energy_out;   // device double
};
// Blob matching (thread.cpp:669-737): disjoint random group pairs per frame,
// swapped when the blob-distance criterion c1 >= c2 holds.  One CTA.
int launch_blob_match(const MatchArgs &a, cudaStream_t s);

}  // namespace amg
