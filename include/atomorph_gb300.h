/*
 * atomorph_gb300 — C ABI of the GB300 (sm_103a) morph pipeline.
 *
 * This is the drop-in boundary for the atomorph morph path.  Every entry point
 * replaces one member of the reference's C++ class am::morph (morph.h:9-145)
 * or one step the reference's demo performs around it; the comment on each
 * declaration names the reference interface it replaces as file:line.  The
 * C++ class am::morph in include/atomorph_gb300.hpp maps these calls back to
 * the reference's own signatures (bool / no-op conventions).
 *
 * Conventions
 *   - Functions returning int return an AM_* status.  Queries return their
 *     value directly, with the reference's "missing" value (0, SIZE_MAX, ...).
 *   - Pointers are plain host pointers unless a parameter says "device".
 *   - A handle is used by one host thread at a time; its GPU work runs on
 *     the handle's own CUDA stream (am_get_stream).
 */
#ifndef ATOMORPH_GB300_H
#define ATOMORPH_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (the reference's bool/nullptr conventions, made explicit) */
#define AM_OK              0
#define AM_ERR_BUSY        1  /* worker running: reference no-ops (morph.cpp:53,60,66,103) */
#define AM_ERR_NOMEM       2  /* device or host allocation failed (reference: new(std::nothrow)) */
#define AM_ERR_CUDA        3  /* a CUDA call failed; am_last_error() has the text */
#define AM_ERR_TIMEOUT     4  /* suspend(timeout) expired (morph.cpp:80-100) / bounded wait expired */
#define AM_ERR_ARG         5  /* invalid argument */
#define AM_ERR_STATE       6  /* call not valid in the current pipeline state */
#define AM_ERR_UNSUPPORTED 7  /* setting outside what the GPU path implements */
#define AM_ERR_NOT_FOUND   8  /* frame / blob does not exist */

/* ---- constants, same values as atomorph.h:235-248, 304-306 */
#define AM_RGB     0
#define AM_HSP     1
#define AM_NONE    2
#define AM_LINEAR  3
#define AM_SPLINE  4
#define AM_COSINE  5
#define AM_PERLIN  6
#define AM_STATE_BLOB_DETECTION   0
#define AM_STATE_BLOB_UNIFICATION 1
#define AM_STATE_BLOB_MATCHING    2
#define AM_STATE_ATOM_MORPHING    3
#define AM_STATE_DONE             4
#define AM_HAS_PIXEL 1
#define AM_HAS_FLUID 2
#define AM_TEXTURE  0
#define AM_AVERAGE  1
#define AM_DISTINCT 2

/* ---- swap proposal kinds (new; the reference has only uniform random pairs) */
#define AM_PROPOSAL_RANDOM  0  /* disjoint uniform random pairs: the plain method */
#define AM_PROPOSAL_LOCAL   1  /* spatially local candidates, exact gain, greedy disjoint matching */
#define AM_PROPOSAL_LEARNED 2  /* the trained MLP picks which columns run the local scan */
#define AM_PROPOSAL_SCORED  3  /* the trained MLP ranks random partners; the best-ranked is checked exactly
                                * (calls alternate with plain sweeps by measured cost gain per second) */

typedef struct am_morph am_morph;

/* ---- lifetime */
int  am_create(am_morph **out);          /* morph::morph()  morph.cpp:9-12 */
void am_destroy(am_morph *m);            /* morph::~morph() morph.cpp:14-16 */
int  am_clear(am_morph *m);              /* morph::clear()  morph.cpp:18-50 */
const char *am_last_error(void);         /* text of the last AM_ERR_CUDA / AM_ERR_ARG in this thread */
const char *am_version(void);            /* am::get_version atomorph.cpp:1015-1017 */

/* ---- key-frame ingestion */
/* morph::add_pixel (morph.cpp:298-337): stores the pixel (HSP-converted when
 * the delimiter is HSP), updates bbox and running frame means. */
int am_add_pixel(am_morph *m, size_t frame, uint16_t x, uint16_t y,
                 uint8_t r, uint8_t g, uint8_t b, uint8_t a);
/* Bulk form of the demo's fill_morph (demo/main.cpp:96-127): every pixel of
 * a w*h RGBA8 image with alpha > 0 is added in row-major order; an image
 * with no such pixel adds an empty frame. */
int am_add_pixels(am_morph *m, size_t frame, const uint8_t *rgba, uint32_t w, uint32_t h);
int am_add_frame(am_morph *m, size_t frame);           /* morph::add_frame morph.cpp:287-296; AM_ERR_ARG if it exists */

/* ---- parameters (morph.h:52-76, morph.cpp:436-444, 1517-1570) */
int am_set_seed(am_morph *m, unsigned seed);                 /* morph::set_seed morph.cpp:436 */
int am_set_blob_delimiter(am_morph *m, unsigned d);          /* morph.h:52 */
int am_set_blob_threshold(am_morph *m, double t);            /* morph.h:53 */
int am_set_blob_max_size(am_morph *m, size_t s);             /* morph.h:54 */
int am_set_blob_min_size(am_morph *m, size_t s);             /* morph.h:55 */
int am_set_blob_box_grip(am_morph *m, uint16_t g);           /* morph.h:56 */
int am_set_blob_box_samples(am_morph *m, size_t s);          /* morph.h:57 */
int am_set_blob_number(am_morph *m, size_t n);               /* morph.h:58 */
int am_set_blob_rgba_weight(am_morph *m, unsigned w);        /* morph.h:59 */
int am_set_blob_size_weight(am_morph *m, unsigned w);        /* morph.h:60 */
int am_set_blob_xy_weight(am_morph *m, unsigned w);          /* morph.h:61 */
int am_set_degeneration(am_morph *m, size_t d);              /* morph.h:62 */
int am_set_motion(am_morph *m, unsigned motion);             /* morph.h:63 */
int am_set_fading(am_morph *m, unsigned fading);             /* morph.h:64 */
int am_set_threads(am_morph *m, size_t t);                   /* morph.h:65 (accepted; GPU width is automatic) */
int am_set_cycle_length(am_morph *m, size_t c);              /* morph.h:66: stored; a worker step here runs am_set_sweeps whole sweeps instead of cycle_length random proposals */
/* Feather fades each blob's outer f layers (morph.cpp:625-674; the fluid
 * path grows f layers outward, morph.cpp:1204-1266); f <= 96, larger values
 * return AM_ERR_UNSUPPORTED. */
int am_set_feather(am_morph *m, size_t f);                   /* morph.h:67 */
int am_set_keep_background(am_morph *m, int k);              /* morph.h:68 */
int am_set_finite(am_morph *m, int f);                       /* morph.h:69 */
/* AM_TEXTURE (atom colours), AM_AVERAGE (each blob in its mean colour) or
 * AM_DISTINCT (a colour per group from std::mt19937(group)),
 * morph.cpp:1321-1334; other values draw TEXTURE. */
int am_set_show_blobs(am_morph *m, unsigned b);              /* morph.h:70 */
int am_set_fluid(am_morph *m, unsigned steps);               /* morph::set_fluid morph.cpp:1553-1560 */
int am_set_density(am_morph *m, uint16_t d);                 /* morph::set_density morph.cpp:1562-1570 */
int am_set_resolution(am_morph *m, uint16_t w, uint16_t h);  /* morph::set_resolution morph.cpp:1517-1520 */
/* New knobs (no reference counterpart): swap proposal kind and sweeps per
 * atom-morphing step. */
int am_set_proposal(am_morph *m, unsigned kind);
int am_set_sweeps(am_morph *m, size_t sweeps_per_step);
/* Perlin motion perturbation (no reference counterpart: the reference moves
 * atoms along their LINEAR / SPLINE paths, morph.cpp:523-531).  Amplitude A
 * in pixels, 0 (the default) = off, at most 64.  An atom drawn at local time
 * t of a key-frame pair is displaced by rint(s * n) in 1/256 px per axis,
 * s = A * 256 * sin(pi t) (zero at key frames), n the 8-octave Perlin noise
 * (perlin.cpp:57-69) of maps seeded seed + 2 (x) and seed + 3 (y) at the
 * atom's first point of the pair, normalised by the key frames' bounding box
 * at frequency 8 as the colour fade's lag map is (morph.cpp:540-545); the
 * noise is evaluated in FP32, every operation rounded to nearest. */
int am_set_motion_noise(am_morph *m, double amplitude_px);
/* Fluid solver grid units per pixel (the reference's sparseness, fixed at 1
 * there): the grid is (width * s + 20) x (height * s + 20). */
int am_set_fluid_sparseness(am_morph *m, double s);
/* The morph's fluid particles (fields as am_fluid_get_particles) after the
 * last fluid frame; returns the particle count, writes when cap >= it. */
size_t am_get_fluid_particles(am_morph *m, double *state, size_t cap);
/* The columns each particle's last update_particle read (morph.cpp:687-695):
 * its source column (after the growing-area rule) and destination column,
 * whose trajectory and colours gave its gravity target and ideal colour;
 * meaningful for the active particles.  Returns the particle count, writes
 * when cap >= it. */
size_t am_get_fluid_links(am_morph *m, uint32_t *src_col, uint32_t *dst_col, size_t cap);
/* Guided-refinement tunables (the autotuner sets these): "local_self",
 * "local_target", "local_random" (candidates per column from the column's own
 * neighbourhood, its target cell, and uniform random columns),
 * "learned_keep" (fraction of 32-slot regions, 0 < f <= 1, that the learned
 * gate lets run the guided candidate scan in a gated sweep),
 * "learned_adaptive" (1, the default: the learned form runs its gate only in
 * blocks of sweeps where gated sweeps keep up with full ones; 0: always) and
 * "guided_switch" (guided/learned refinement runs plain sweeps until one gains
 * less than this fraction of the cost per sweep; 0 = guided from the start).
 * Render: "render_pipeline" (1, the default: a frame's binning and the next
 * frame's tile plan run on a second stream, beside the previous frame's
 * resolve; 0: frames run one after the other on the render stream alone, for
 * timing each kernel by itself).  "render_bin_ctas" / "render_resolve_ctas"
 * (0, the default: as many as fit; 1-8): co-resident CTAs per SM the frame's
 * binning / resolve kernel may take, so the pipelined frames' two kernels can
 * share every SM. */
int am_set_tuning(am_morph *m, const char *name, double value);

/* ---- control (morph.h:40-49, morph.cpp:52-100, 102-269) */
int am_compute(am_morph *m);                          /* morph::compute() morph.cpp:52-57 */
int am_iterate(am_morph *m, size_t iterations);       /* morph::iterate morph.cpp:59-63 */
int am_compute_seconds(am_morph *m, double seconds);  /* morph::compute(double) morph.cpp:65-70 */
int am_suspend(am_morph *m);                          /* morph::suspend() morph.cpp:72-78 */
int am_suspend_timeout(am_morph *m, double timeout);  /* morph::suspend(double) morph.cpp:80-100; AM_ERR_TIMEOUT on expiry */
int am_is_busy(const am_morph *m);                    /* morph::is_busy morph.h:49; 1 or 0 */
int am_synchronize(am_morph *m);                      /* morph::synchronize morph.cpp:102-269; AM_ERR_BUSY while running */
int am_next_state(am_morph *m);                       /* morph::next_state morph.h:39 */

/* ---- readout */
unsigned am_get_state(const am_morph *m);                   /* morph.h:38 */
double   am_get_energy(const am_morph *m);                  /* morph.h:41; the TRUE cost (see am_get_cost) */
/* Exact atom cost: sum over chains of thread::get_energy(chain*)
 * (thread.cpp:1109-1125), as an exact integer and as a double. */
int      am_get_cost(am_morph *m, uint64_t *exact, double *as_double);
/* The exact cost of am_get_cost without allocating device memory (no
 * counterpart in the reference): for callers that must not allocate while
 * other work is on the device, since cudaMalloc/cudaFree may synchronise it.
 * Scratch is one static device array shared by all calls in the process, so
 * calls that overlap in time race and must be serialised by the caller.
 * Accepts chains of at most 2^27 columns (atoms x key frames); larger ones
 * return AM_ERR_ARG.  The first call on a device looks up the array's
 * address: make it before any stream capture begins.  The call runs on the
 * handle's device and leaves the calling thread's current device as it
 * found it. */
int      am_get_cost_noalloc(am_morph *m, uint64_t *exact);
size_t   am_get_blob_count(const am_morph *m, size_t frame);  /* morph::get_blob_count(f) morph.cpp:399-402 */
size_t   am_get_blob_count_total(const am_morph *m);          /* morph::get_blob_count() morph.cpp:425-434 */
size_t   am_get_pixel_count(const am_morph *m, size_t frame); /* morph::get_pixel_count morph.cpp:394-397 */
size_t   am_get_frame_count(const am_morph *m);               /* morph.h:37 */
size_t   am_get_frame_key(const am_morph *m, double t);       /* morph::get_frame_key morph.cpp:404-423 */
uint16_t am_get_width(const am_morph *m);                     /* morph.h:35 */
uint16_t am_get_height(const am_morph *m);                    /* morph.h:36 */
double   am_get_time(const am_morph *m, size_t i, size_t n);  /* morph::get_time morph.cpp:1522-1538 */
/* morph::get_average_pixel(f) morph.cpp:339-354: x, y, r, g, b, a (RGB). */
int      am_get_average_pixel(const am_morph *m, size_t frame, uint16_t *xy, uint8_t *rgba);
/* The blobs of key frame `frame` after detection (morph::get_blob's surface
 * sets, morph.h:31): labels[y * w + x] = index of the blob holding pixel
 * (x, y), -1 where the frame has no pixel; w, h = the key-frame canvas.  With
 * labels NULL only w and h are written.  AM_ERR_BUSY while the worker runs. */
int      am_get_blob_labels(am_morph *m, size_t frame, int32_t *labels, uint32_t *w, uint32_t *h);
/* morph::get_average_pixel(f, b) morph.cpp:356-376. */
int      am_get_blob_average(const am_morph *m, size_t frame, size_t blob, uint16_t *xy, uint8_t *rgba);
/* morph::get_blob(f, b) (morph.h:40; blob, atomorph.h:256-263) as values:
 * the blob's group (its chain), surface size and means x, y, r, g, b, a
 * (colours in the stored colour space, 0..1).  AM_ERR_NOT_FOUND when the
 * frame or blob does not exist. */
int      am_get_blob_info(const am_morph *m, size_t frame, size_t blob, size_t *group, size_t *surface,
                          double *xyrgba);
/* morph::get_pixels(blob, t, to) (morph.h:29, morph.cpp:452-678): the pixels
 * of the blob-th blob of the key frame at time t drawn alone, every pixel its
 * atoms reach with its mean colour (transparent ones included), in the
 * reference's order (ascending position y * 65536 + x; with a feather the
 * outer layers first, layer by layer, then the rest).  Before chains exist,
 * the blob's own key-frame pixels.  xy (2 per pixel) and rgba (4 per pixel)
 * receive up to cap pixels, *count the number; pixels outside the morph's
 * resolution are not returned.  AM_ERR_NOT_FOUND when the blob does not
 * exist, AM_ERR_BUSY while the worker runs. */
int      am_get_blob_pixels(am_morph *m, size_t blob, double t, uint16_t *xy, uint8_t *rgba, size_t cap,
                            size_t *count);
size_t   am_get_atom_count(const am_morph *m);                /* total chain width (atoms per key frame) */
size_t   am_get_chain_count(const am_morph *m);               /* chains = blob groups */

/* Renders the frame at time t (morph::get_pixels(t, vec) morph.cpp:1405-1421)
 * as width*height RGBA8, row-major.  out is a host pointer, or a device
 * pointer when out_on_device != 0.  A host frame is complete when the call
 * returns.  When out lies in pinned (page-locked, CUDA-mapped) host memory
 * whose allocation covers the whole frame, an atom frame is stored there by
 * the GPU directly while it is resolved; other host memory receives a copy. */
int am_render(am_morph *m, double t, uint8_t *out, int out_on_device);
/* Every atom's position at time t, as the render draws it (motion path plus
 * the motion perturbation): xy[2i], xy[2i + 1] = x and y position words
 * (integer pixel * 256 + fraction byte, the point layout of atomorph.h:275-
 * 284) of atom column i (chain order, as am_export_chains), -1, -1 where the
 * atom is drawn at neither key frame of its pair.  Returns the atom count
 * and writes when cap >= it (0 when the readout failed: am_last_error).
 * Readout of get_pixels(blob, t)'s positions, morph.cpp:523-531. */
size_t am_get_positions(am_morph *m, double t, int32_t *xy, size_t cap);
/* Renders n frames at times ts[0..n) into n consecutive device frames. */
int am_render_many(am_morph *m, const double *ts, size_t n, uint8_t *out_device);
/* Renders n frames at times ts[0..n) into n consecutive host frames, complete
 * when the call returns.  When out lies in pinned host memory whose
 * allocation covers all n frames, atom frames are stored there by the GPU
 * directly and pipelined like device frames; other memory receives the frames
 * one at a time as am_render would. */
int am_render_many_host(am_morph *m, const double *ts, size_t n, uint8_t *out);

/* ---- chains (reference chain = points[width][height], atomorph.h:286-298)
 * pts is frame-major: pts[k * N + off_c + x] = point x of chain c at key
 * frame k, as the reference's 8-byte point word (atomorph.h:275-284, padding
 * byte zero).  blob_order[k * C + b] = group of the b-th blob of key frame k
 * (composite order in draw_atoms, morph.cpp:1309). */
int am_export_chains(am_morph *m, uint64_t *widths, uint64_t *pts, int32_t *blob_order);
int am_import_chains(am_morph *m, size_t K, size_t C, const uint64_t *widths,
                     const uint64_t *pts, const int32_t *blob_order);
/* Runs n refinement sweeps now on the handle's stream with the current
 * proposal kind (the synchronous form of the atom-morphing step,
 * thread.cpp:1043-1068).  gains (optional, n entries) receive the exact cost
 * decrease of each sweep. */
int am_refine(am_morph *m, size_t sweeps, uint64_t *gains);

/* ---- learned swap proposal (no reference counterpart; the reference only
 * draws uniform random pairs, thread.cpp:1000-1005).  The network maps 10
 * features of a column to a predicted gain of scanning it; its fp32 master
 * parameters are exchanged as
 * AM_PROPOSAL_PARAMS floats: W1[64][10], b1[64], W2[64][64], b2[64], w3[64], b3. */
#define AM_PROPOSAL_FEATURES 10
#define AM_PROPOSAL_PARAMS 4929
/* Makes the next learned-proposal sweeps scan every column and log up to cap
 * of them: the column's features and the target log1p(g/S^2) of the best
 * exact swap gain g its full candidate scan found (0 when none improves);
 * S = 16 px in 1/256 px units. */
int    am_record_swaps(am_morph *m, size_t cap);
size_t am_recorded_swaps(am_morph *m, float *features, float *targets, size_t cap);
/* Trains the network on the GPU (tensor-core forward/backward, Adam) on n
 * samples for `epochs` passes; loss_out gets the last epoch's mean loss. */
int    am_train_proposal(am_morph *m, const float *features, const float *targets, size_t n, size_t epochs,
                         double lr, float *loss_out);
/* The same on the samples recorded since am_record_swaps, where the
 * recording sweeps left them in device memory (no copy through the host);
 * recording stops.  AM_ERR_STATE when nothing was recorded. */
int    am_train_recorded(am_morph *m, size_t epochs, double lr, float *loss_out);
/* Training data of the learned pair proposal (AM_PROPOSAL_SCORED): makes the
 * next plain (AM_PROPOSAL_RANDOM) sweeps log 1 in `every` of their proposals,
 * up to cap, as 10 pair features (position difference and distance over
 * 16 px, colour difference of the two atoms' key-frame pixels, each column's
 * current cost log1p(d / (16 px)^2), HAS_PIXEL parity) and the outcome of the
 * swap under the reference's costs (thread.cpp:1014-1022): 1 when it lowers
 * the cost (c1 > c2), 0 otherwise (the criterion c1 >= c2 also accepts ties,
 * which gain nothing).  am_recorded_swaps reads them (targets = outcomes) and
 * am_train_recorded trains the network on them where they lie.  cap 0 stops.
 * The learned gate and the pair proposal share one network: train it for
 * the proposal kind it serves.  Until it is trained, AM_PROPOSAL_SCORED runs
 * plain sweeps. */
int    am_record_outcomes(am_morph *m, size_t cap, uint32_t every);
int    am_get_proposal_weights(am_morph *m, float *w, size_t count);
int    am_set_proposal_weights(am_morph *m, const float *w, size_t count);
/* Scores of n feature rows, and the gradient of the mean squared error of n
 * (feature, target) rows with respect to the master parameters. */
int    am_proposal_forward(am_morph *m, const float *features, size_t n, float *scores);
int    am_proposal_grad(am_morph *m, const float *features, const float *targets, size_t n, float *grad,
                        float *loss_sum);

/* ---- fluid solver (the reference's FluidModel, fluidmodel.h:103-142), FP32.
 * Particle state is exchanged as 18 doubles per particle in this order:
 * x y u v gravity_x gravity_y freedom_r active mature strength R G B A r g b a
 * (Particle, fluidmodel.h:33-79; positions in grid units). */
typedef struct am_fluid am_fluid;
int  am_fluid_create(am_fluid **out, uint32_t gsize_x, uint32_t gsize_y, uint32_t particles); /* FluidModel::FluidModel fluidmodel.cpp:107-148 */
void am_fluid_destroy(am_fluid *f);                                             /* FluidModel::~FluidModel fluidmodel.cpp:151-162 */
int  am_fluid_set_particles(am_fluid *f, const double *state);
int  am_fluid_get_particles(am_fluid *f, double *state);                        /* FluidModel::getParticles fluidmodel.cpp:595-597 */
int  am_fluid_step(am_fluid *f, size_t steps_left, double freedom_radius);      /* FluidModel::step fluidmodel.cpp:165-580 */
/* n steps with steps_left = n-1 .. 0, as morph::step_fluid runs them (morph.cpp:1054). */
int  am_fluid_steps(am_fluid *f, size_t n, double freedom_radius);
void *am_fluid_stream(am_fluid *f);
/* draw_fluid (morph.cpp:1081-1204) of the particles as they are: colour
 * correction at local time t (written back to the particles, which also
 * mature), bilinear splat, per-pixel rounded means into rgba_out (host,
 * width x height RGBA8); bbox = x1, y1, x2, y2 of the key frames. */
int  am_fluid_render(am_fluid *f, uint32_t width, uint32_t height, double sparseness, const uint32_t *bbox,
                     double t, uint8_t *rgba_out);
/* The same with `feather` outward layers (morph.cpp:1204-1266) and, when
 * `background` (host width x height RGBA8, the get_background image) is not
 * NULL, keep_background: fluid alpha x (1 - t^24) drawn over it
 * (morph.cpp:1187-1190, 1268-1299). */
int  am_fluid_render_ex(am_fluid *f, uint32_t width, uint32_t height, double sparseness, const uint32_t *bbox,
                        double t, size_t feather, const uint8_t *background, uint8_t *rgba_out);

/* ---- batched refinement (no reference counterpart: the reference refines
 * one morph per worker thread, thread.cpp:173-206).  A batch refines many
 * jobs (morph handles whose chains are built) with one persistent cooperative
 * launch per call that runs every sweep of every job, captured once into a
 * CUDA graph and replayed.  Each job draws the same random pairs as its own
 * am_refine with AM_PROPOSAL_RANDOM would, so results are bit-identical to
 * refining the jobs one by one, and each job's cost, sweep counter and
 * rendered front copy advance as after am_refine.  All jobs must be on one
 * device and idle (not computing) during batch calls; a job may appear only
 * once (AM_ERR_ARG otherwise). */
typedef struct am_batch am_batch;
int  am_batch_create(am_batch **out, am_morph *const *jobs, size_t n);
void am_batch_destroy(am_batch *b);
/* n plain sweeps of every job; gains (optional, [jobs][sweeps]) receive the
 * exact cost decrease of each job's sweeps. */
int  am_batch_refine(am_batch *b, size_t sweeps, uint64_t *gains);
/* n guided sweeps (AM_PROPOSAL_LOCAL) of every job in one persistent
 * cooperative launch, captured into a CUDA graph and replayed: per phase the
 * claims of all jobs are cleared, every column proposes, the winners are
 * applied, with grid barriers between.  Each job's result is bit-identical
 * to its own am_refine with AM_PROPOSAL_LOCAL once its guided phase has
 * started (guided_switch 0); gains as am_batch_refine. */
int  am_batch_refine_guided(am_batch *b, size_t sweeps, uint64_t *gains);
/* Schedule autotuner: for a budget of `sweeps` per job, tries 0, 1/8, 1/4
 * and 1/2 of the budget as plain sweeps followed by guided ones, from the
 * jobs' chains as they are (restored after each trial), and keeps the split
 * whose summed final cost is lowest; *plain_sweeps receives it.  The chains
 * are left as they were. */
int  am_batch_tune_schedule(am_batch *b, size_t sweeps, size_t *plain_sweeps);
/* The tuned schedule: plain sweeps (am_batch_refine), then guided ones
 * (am_batch_refine_guided), `sweeps` in all; gains [jobs][sweeps]. */
int  am_batch_refine_schedule(am_batch *b, size_t sweeps, uint64_t *gains);
/* Frames of every job at the n normalised times ts (morph::get_pixels(t),
 * morph.cpp:452-678, per job): outs[j] receives job j's n frames, each its
 * width * height * 4 RGBA8 bytes, one after the other, in device memory when
 * outs_on_device != 0, else in host memory (pinned, mapped host memory is
 * stored into by the GPU directly).  Per time, the atom frames of all jobs
 * are binned by one launch, resolved by one launch and their next tile plans
 * made by one launch (up to 32 jobs per launch); fluid frames and frames
 * before chains exist run through each job's own render.  Every frame equals
 * the job's own am_render at the same time.  The jobs must be idle; the
 * frames are complete when the call returns. */
int  am_batch_render(am_batch *b, const double *ts, size_t n, uint8_t *const *outs, int outs_on_device);
/* Autotuner: times trial_sweeps real sweeps of all jobs under each candidate
 * launch shape (threads per CTA, CTAs per SM) and work schedule (pairs per
 * chunk, job-major or interleaved chunk order) on a snapshot of the jobs'
 * chains, keeps the fastest, and leaves the chains as they were. */
int  am_batch_tune(am_batch *b, size_t trial_sweeps);
int  am_batch_get_tuning(const am_batch *b, uint32_t *threads, uint32_t *ctas_per_sm, uint32_t *chunk, uint32_t *order);
int  am_batch_set_tuning(am_batch *b, uint32_t threads, uint32_t ctas_per_sm, uint32_t chunk, uint32_t order);

/* ---- runtime (no reference counterpart) */
void    *am_get_stream(am_morph *m);        /* cudaStream_t that renders run on */
/* Per-kernel timing: when enabled, CUDA events are recorded on the launching
 * stream around every render / refinement kernel; am_profile_read waits for
 * them and returns, per kernel kind, the name, total milliseconds and launch
 * count (up to cap kinds; returns the number written). */
int      am_profile_enable(am_morph *m, int on);
size_t   am_profile_read(am_morph *m, const char **names, double *ms, uint64_t *launches, size_t cap);
uint64_t am_launch_count(void);             /* kernels launched by this library, process-wide */
/* Heavy tiles: output tiles holding more than 8192 binned atom records
 * (atoms crowded or stacked by a chain much wider than a key frame's blob)
 * are resolved in 32 row bands by helper CTAs in the frames after one of the
 * morph's frames had them.  *tiles = the heavy tiles of the last frame that
 * had any (0 when none yet), *helpers = the helper CTAs of the last resolve
 * launched.  Waits for the morph's binning work, so every frame rendered so
 * far has reported.  Either pointer may be null. */
int      am_get_heavy_tiles(am_morph *m, uint32_t *tiles, uint32_t *helpers);
int      am_device_sync(am_morph *m);       /* waits for the handle's stream */

#ifdef __cplusplus
}
#endif
#endif
