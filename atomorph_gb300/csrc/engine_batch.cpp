// Batched refinement of many morph jobs (am_batch_*).  No reference
// counterpart: the reference refines one morph per worker thread
// (thread.cpp:173-206).  See k_batch.cu for the kernel.
#include "batch.h"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace amg {

Batch::Batch(std::vector<Engine *> jobs) : jobs_(std::move(jobs)) {}

Batch::~Batch() {
    drop_graphs();
    for (cudaEvent_t e : ev_bin_) cudaEventDestroy(e);
    for (int k = 0; k < 2; ++k) {
        if (ev_time_[k]) cudaEventDestroy(ev_time_[k]);
        if (ev_copied_[k]) cudaEventDestroy(ev_copied_[k]);
    }
    if (bstream_) cudaStreamDestroy(bstream_);
    if (cstream_) cudaStreamDestroy(cstream_);
    if (h_jobs_) cudaFreeHost(h_jobs_);
    if (h_ljobs_) cudaFreeHost(h_ljobs_);
    if (h_gains_) cudaFreeHost(h_gains_);
    if (ev0_) cudaEventDestroy(ev0_);
    if (ev1_) cudaEventDestroy(ev1_);
    if (stream_) cudaStreamDestroy(stream_);
}

void Batch::drop_graphs() {
    for (auto &g : graphs_)
        if (g.second.exec) cudaGraphExecDestroy(g.second.exec);
    graphs_.clear();
    for (auto &g : lgraphs_)
        if (g.second.exec) cudaGraphExecDestroy(g.second.exec);
    lgraphs_.clear();
}

static bool refinable(const Engine *e) {
    return (e->state == AM_STATE_ATOM_MORPHING || e->state == AM_STATE_DONE) && e->N > 0 && e->K > 0;
}

int Batch::init() {
    if (jobs_.empty()) {
        set_error("am_batch_create: no jobs");
        return AM_ERR_ARG;
    }
    device_ = jobs_[0]->device;
    std::vector<Engine *> sorted(jobs_);
    std::sort(sorted.begin(), sorted.end());
    if (std::adjacent_find(sorted.begin(), sorted.end()) != sorted.end()) {
        set_error("am_batch_create: a job appears twice");
        return AM_ERR_ARG;
    }
    for (Engine *e : jobs_) {
        if (!e) { set_error("am_batch_create: null job"); return AM_ERR_ARG; }
        if (e->device != device_) { set_error("am_batch_create: jobs on different devices"); return AM_ERR_ARG; }
        if (e->is_busy()) return AM_ERR_BUSY;
        if (!refinable(e)) {
            set_error("am_batch_create: every job must have its chains built (state ATOM_MORPHING or DONE)");
            return AM_ERR_STATE;
        }
    }
    AMG_CUDA(cudaSetDevice(device_));
    AMG_CUDA(cudaDeviceGetAttribute(&sms_, cudaDevAttrMultiProcessorCount, device_));
    AMG_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
    AMG_CUDA(cudaEventCreate(&ev0_));
    AMG_CUDA(cudaEventCreate(&ev1_));
    int rc;
    AMG_CUDA(cudaMallocHost(&h_jobs_, jobs_.size() * sizeof(BatchJob)));
    AMG_CUDA(cudaMallocHost(&h_ljobs_, jobs_.size() * sizeof(BatchLocalJob)));
    if ((rc = d_ljobs_.reserve(jobs_.size()))) return rc;
    sversions_.assign(jobs_.size(), UINT64_MAX);
    if ((rc = d_jobs_.reserve(jobs_.size()))) return rc;
    if ((rc = d_bar_.reserve(4))) return rc;
    if ((rc = d_err_.reserve(1))) return rc;
    AMG_CUDA(cudaMemsetAsync(d_err_.p, 0, sizeof(int), stream_));
    versions_.assign(jobs_.size(), UINT64_MAX);
    return sync_layout();
}

// Chunk tables: for each phase p and each frame of every job's phase p, the
// job's pairs cut into chunks of at most tuning.chunk pairs.
int Batch::sync_layout() {
    bool changed = tuning.chunk != chunk_built_ || tuning.order != order_built_;
    for (size_t j = 0; j < jobs_.size(); ++j) changed |= versions_[j] != jobs_[j]->layout_version;
    if (!changed) return AM_OK;
    struct Ch { uint64_t start; uint32_t count, fi; };
    std::vector<uint32_t> job[3], cnt[3], fis[3];
    std::vector<uint64_t> start[3];
    nphase_ = 0;
    for (uint32_t p = 0; p < 3; ++p) {
        std::vector<std::vector<Ch>> per(jobs_.size());
        for (size_t j = 0; j < jobs_.size(); ++j) {
            Engine *e = jobs_[j];
            auto ph = phases_for(e->K);
            nphase_ = std::max<uint32_t>(nphase_, (uint32_t)ph.size());
            if (p >= ph.size() || e->pair_off.empty()) continue;
            const uint64_t pairs = e->pair_off[e->C];
            for (uint32_t fi = 0; fi < (uint32_t)ph[p].size(); ++fi)
                for (uint64_t s = 0; s < pairs; s += tuning.chunk)
                    per[j].push_back({s, (uint32_t)std::min<uint64_t>(tuning.chunk, pairs - s), fi});
        }
        auto put = [&](size_t j, const Ch &c) {
            job[p].push_back((uint32_t)j); start[p].push_back(c.start); cnt[p].push_back(c.count); fis[p].push_back(c.fi);
        };
        if (tuning.order == 0) {
            for (size_t j = 0; j < per.size(); ++j)
                for (auto &c : per[j]) put(j, c);
        } else {
            for (size_t k = 0;; ++k) {
                bool any = false;
                for (size_t j = 0; j < per.size(); ++j)
                    if (k < per[j].size()) { any = true; put(j, per[j][k]); }
                if (!any) break;
            }
        }
    }
    size_t total = job[0].size() + job[1].size() + job[2].size();
    if (total > UINT32_MAX) { set_error("am_batch: too many chunks"); return AM_ERR_ARG; }
    ch_off_[0] = 0;
    for (int p = 0; p < 3; ++p) ch_off_[p + 1] = ch_off_[p] + (uint32_t)job[p].size();
    std::vector<uint32_t> J, Cn, F;
    std::vector<uint64_t> S;
    for (int p = 0; p < 3; ++p) {
        J.insert(J.end(), job[p].begin(), job[p].end());
        Cn.insert(Cn.end(), cnt[p].begin(), cnt[p].end());
        F.insert(F.end(), fis[p].begin(), fis[p].end());
        S.insert(S.end(), start[p].begin(), start[p].end());
    }
    uint32_t *oj = d_ch_job_.p, *oc = d_ch_count_.p, *of = d_ch_fi_.p;
    uint64_t *os = d_ch_start_.p;
    int rc;
    if ((rc = d_ch_job_.reserve(std::max<size_t>(total, 1)))) return rc;
    if ((rc = d_ch_count_.reserve(std::max<size_t>(total, 1)))) return rc;
    if ((rc = d_ch_fi_.reserve(std::max<size_t>(total, 1)))) return rc;
    if ((rc = d_ch_start_.reserve(std::max<size_t>(total, 1)))) return rc;
    if (oj != d_ch_job_.p || oc != d_ch_count_.p || os != d_ch_start_.p || of != d_ch_fi_.p) drop_graphs();
    if (total) {
        AMG_CUDA(cudaMemcpyAsync(d_ch_job_.p, J.data(), total * 4, cudaMemcpyHostToDevice, stream_));
        AMG_CUDA(cudaMemcpyAsync(d_ch_count_.p, Cn.data(), total * 4, cudaMemcpyHostToDevice, stream_));
        AMG_CUDA(cudaMemcpyAsync(d_ch_fi_.p, F.data(), total * 4, cudaMemcpyHostToDevice, stream_));
        AMG_CUDA(cudaMemcpyAsync(d_ch_start_.p, S.data(), total * 8, cudaMemcpyHostToDevice, stream_));
    }
    AMG_CUDA(cudaStreamSynchronize(stream_));
    drop_graphs();  // chunk ranges are baked into the captured launch
    for (size_t j = 0; j < jobs_.size(); ++j) versions_[j] = jobs_[j]->layout_version;
    chunk_built_ = tuning.chunk;
    order_built_ = tuning.order;
    return AM_OK;
}

// Enqueues one call: job table in, counters zeroed, the persistent launch,
// gains out.  With `graph`, the sequence is captured once per (sweeps,
// tuning) and replayed.
int Batch::run(size_t sweeps, const BatchTuning &t, bool graph, float *ms) {
    const size_t nj = jobs_.size();
    int rc;
    unsigned long long *og = d_gains_.p;
    if ((rc = d_gains_.reserve(std::max<size_t>(nj * sweeps, 1)))) return rc;
    if (og != d_gains_.p) drop_graphs();
    if (h_gains_n_ < nj * sweeps) {
        drop_graphs();
        if (h_gains_) cudaFreeHost(h_gains_);
        h_gains_ = nullptr;
        h_gains_n_ = 0;
        AMG_CUDA(cudaMallocHost(&h_gains_, nj * sweeps * sizeof(unsigned long long)));
        h_gains_n_ = nj * sweeps;
    }
    int occ = 0;
    if ((rc = batch_max_ctas_per_sm(t.threads, &occ))) return rc;
    if (occ < 1) { set_error("am_batch: the sweep kernel does not fit on an SM"); return AM_ERR_CUDA; }
    uint32_t grid = std::min<uint32_t>(t.ctas_per_sm, (uint32_t)occ) * (uint32_t)sms_;
    BatchArgs a;
    a.jobs = d_jobs_.p; a.njobs = (uint32_t)nj;
    a.ch_job = d_ch_job_.p; a.ch_start = d_ch_start_.p; a.ch_count = d_ch_count_.p; a.ch_fi = d_ch_fi_.p;
    std::memcpy(a.ch_off, ch_off_, sizeof(ch_off_));
    a.nphase = nphase_; a.sweeps = (uint32_t)sweeps; a.gains = d_gains_.p; a.bar = d_bar_.p; a.err = d_err_.p;
    auto enqueue = [&]() -> int {
        AMG_CUDA(cudaMemcpyAsync(d_jobs_.p, h_jobs_, nj * sizeof(BatchJob), cudaMemcpyHostToDevice, stream_));
        AMG_CUDA(cudaMemsetAsync(d_bar_.p, 0, 4 * sizeof(unsigned), stream_));
        AMG_CUDA(cudaMemsetAsync(d_gains_.p, 0, nj * sweeps * sizeof(unsigned long long), stream_));
        int r = launch_batch_sweeps(a, grid, t.threads, stream_);
        if (r) return r;
        AMG_CUDA(cudaMemcpyAsync(h_gains_, d_gains_.p, nj * sweeps * sizeof(unsigned long long),
                                 cudaMemcpyDeviceToHost, stream_));
        return AM_OK;
    };
    if (ms) AMG_CUDA(cudaEventRecord(ev0_, stream_));
    if (graph) {
        Graph &g = graphs_[sweeps];
        if (g.exec && (g.t.threads != t.threads || g.t.ctas_per_sm != t.ctas_per_sm)) {
            cudaGraphExecDestroy(g.exec);
            g.exec = nullptr;
        }
        if (!g.exec) {
            cudaGraph_t gr = nullptr;
            AMG_CUDA(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
            int r = enqueue();
            cudaError_t ce = cudaStreamEndCapture(stream_, &gr);
            if (r) { if (gr) cudaGraphDestroy(gr); return r; }
            if (ce != cudaSuccess) {
                set_error(std::string("am_batch: stream capture: ") + cudaGetErrorString(ce));
                return AM_ERR_CUDA;
            }
            cudaError_t ie = cudaGraphInstantiate(&g.exec, gr, 0);
            cudaGraphDestroy(gr);
            if (ie != cudaSuccess) {
                g.exec = nullptr;
                set_error(std::string("am_batch: graph instantiate: ") + cudaGetErrorString(ie));
                return AM_ERR_CUDA;
            }
            g.t = t;
        }
        AMG_CUDA(cudaGraphLaunch(g.exec, stream_));
    } else {
        if ((rc = enqueue())) return rc;
    }
    if (ms) AMG_CUDA(cudaEventRecord(ev1_, stream_));
    AMG_CUDA(cudaStreamSynchronize(stream_));
    int err = 0;
    AMG_CUDA(cudaMemcpy(&err, d_err_.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (err) {
        set_error("am_batch: a grid barrier timed out; the jobs' chains are in an unknown state");
        return err;
    }
    if (ms) AMG_CUDA(cudaEventElapsedTime(ms, ev0_, ev1_));
    return AM_OK;
}

static void fill_jobs(const std::vector<Engine *> &jobs, BatchJob *h) {
    for (size_t j = 0; j < jobs.size(); ++j) {
        Engine *e = jobs[j];
        BatchJob &b = h[j];
        b.P = e->d_P.p; b.N = e->N; b.K = e->K; b.C = e->C;
        b.chain_off = e->d_chain_off.p; b.pair_off = e->d_pair_off.p; b.frames = e->d_phase.p;
        auto ph = phases_for(e->K);
        uint32_t off = 0;
        for (uint32_t p = 0; p < 3; ++p) {
            b.ph_off[p] = off;
            b.ph_n[p] = p < ph.size() ? (uint32_t)ph[p].size() : 0;
            off += b.ph_n[p];
        }
        b.seed = e->seed;
        b.sweep0 = e->sweep_counter;
        b.pairs = e->pair_off.empty() ? 0 : e->pair_off[e->C];
    }
}

static int check_jobs(const std::vector<Engine *> &jobs) {
    for (Engine *e : jobs) {
        if (e->is_busy()) return AM_ERR_BUSY;
        if (!refinable(e)) {
            set_error("am_batch: a job's chains are gone (state changed since am_batch_create)");
            return AM_ERR_STATE;
        }
    }
    return AM_OK;
}

int Batch::refine(size_t sweeps, uint64_t *gains) {
    if (sweeps == 0) return AM_OK;
    if (sweeps > UINT32_MAX) return AM_ERR_ARG;
    int rc = check_jobs(jobs_);
    if (rc) return rc;
    AMG_CUDA(cudaSetDevice(device_));
    if ((rc = sync_layout())) return rc;
    fill_jobs(jobs_, h_jobs_);
    if ((rc = run(sweeps, tuning, true, nullptr))) return rc;
    return apply_gains(sweeps, gains, false);
}

// Slot chunks of the guided sweeps: for each phase p and each frame of every
// job's phase p, the job's N slots cut into chunks of tuning.chunk.
int Batch::sync_slot_layout() {
    bool changed = tuning.chunk != slot_chunk_built_;
    for (size_t j = 0; j < jobs_.size(); ++j) changed |= sversions_[j] != jobs_[j]->layout_version;
    if (!changed) return AM_OK;
    std::vector<uint32_t> J, Cn, F;
    std::vector<uint64_t> S;
    uint32_t nph = 0;
    for (uint32_t p = 0; p < 3; ++p) {
        sch_off_[p] = (uint32_t)J.size();
        for (size_t j = 0; j < jobs_.size(); ++j) {
            Engine *e = jobs_[j];
            auto ph = phases_for(e->K);
            nph = std::max<uint32_t>(nph, (uint32_t)ph.size());
            if (p >= ph.size()) continue;
            for (uint32_t fi = 0; fi < (uint32_t)ph[p].size(); ++fi)
                for (uint64_t s = 0; s < e->N; s += tuning.chunk) {
                    J.push_back((uint32_t)j);
                    S.push_back(s);
                    Cn.push_back((uint32_t)std::min<uint64_t>(tuning.chunk, e->N - s));
                    F.push_back(fi);
                }
        }
    }
    sch_off_[3] = (uint32_t)J.size();
    const size_t total = J.size();
    int rc;
    if ((rc = d_sch_job_.reserve(std::max<size_t>(total, 1)))) return rc;
    if ((rc = d_sch_count_.reserve(std::max<size_t>(total, 1)))) return rc;
    if ((rc = d_sch_fi_.reserve(std::max<size_t>(total, 1)))) return rc;
    if ((rc = d_sch_start_.reserve(std::max<size_t>(total, 1)))) return rc;
    if (total) {
        AMG_CUDA(cudaMemcpyAsync(d_sch_job_.p, J.data(), total * 4, cudaMemcpyHostToDevice, stream_));
        AMG_CUDA(cudaMemcpyAsync(d_sch_count_.p, Cn.data(), total * 4, cudaMemcpyHostToDevice, stream_));
        AMG_CUDA(cudaMemcpyAsync(d_sch_fi_.p, F.data(), total * 4, cudaMemcpyHostToDevice, stream_));
        AMG_CUDA(cudaMemcpyAsync(d_sch_start_.p, S.data(), total * 8, cudaMemcpyHostToDevice, stream_));
    }
    AMG_CUDA(cudaStreamSynchronize(stream_));
    drop_graphs();  // chunk ranges are baked into the captured launch
    nphase_ = std::max(nphase_, nph);
    for (size_t j = 0; j < jobs_.size(); ++j) sversions_[j] = jobs_[j]->layout_version;
    slot_chunk_built_ = tuning.chunk;
    return AM_OK;
}

// Each job's guided index (built from its current points when missing) and
// its guided sweep arguments, as its own guided sweeps set them; the batch's
// sweeps start at the job's sweep counter + sweep_offset.
int Batch::prepare_guided(uint64_t sweep_offset) {
    int rc;
    for (size_t j = 0; j < jobs_.size(); ++j) {
        Engine *e = jobs_[j];
        if ((rc = e->ensure_local_index())) return rc;
        AMG_CUDA(cudaStreamSynchronize(e->stream));
        BatchLocalJob &b = h_ljobs_[j];
        std::memset(&b, 0, sizeof(b));
        LocalArgs &a = b.a;
        a = LocalArgs();
        a.P = e->d_P.p; a.N = e->N; a.K = e->K;
        a.slot_pt = e->lix.slot_pt; a.col = e->lix.col; a.slot_of = e->lix.slot_of; a.cell_start = e->lix.cell_start;
        a.ncx = e->lix.ncx; a.ncy = e->lix.ncy; a.ncells = e->lix.ncells; a.slot_ch = e->lix.slot_ch;
        a.cap = e->active.local_target;
        a.self_cap = e->active.local_self; a.nrandom = e->active.local_random; a.chain_off = e->d_chain_off.p;
        a.claim = e->d_claim.p; a.prop = e->d_lprop.p; a.pgain = e->d_pgain.p; a.sv = e->d_sv.p; a.hot = e->d_hot.p;
        a.single_chain = e->C == 1;
        b.frames = e->d_phase.p;
        auto ph = phases_for(e->K);
        uint32_t off = 0;
        for (uint32_t p = 0; p < 3; ++p) {
            b.ph_off[p] = off;
            b.ph_n[p] = p < ph.size() ? (uint32_t)ph[p].size() : 0;
            off += b.ph_n[p];
        }
        b.seed = e->seed;
        b.sweep0 = e->sweep_counter + sweep_offset;
    }
    return sync_slot_layout();
}

// Enqueues one call of batched guided sweeps (captured once per sweep count
// and launch shape, then replayed), like run() for the plain sweeps.
int Batch::run_local(size_t sweeps, const BatchTuning &t, bool graph, float *ms) {
    const size_t nj = jobs_.size();
    int rc;
    unsigned long long *og = d_gains_.p;
    if ((rc = d_gains_.reserve(std::max<size_t>(nj * sweeps, 1)))) return rc;
    if (og != d_gains_.p) drop_graphs();
    if (h_gains_n_ < nj * sweeps) {
        drop_graphs();
        if (h_gains_) cudaFreeHost(h_gains_);
        h_gains_ = nullptr;
        h_gains_n_ = 0;
        AMG_CUDA(cudaMallocHost(&h_gains_, nj * sweeps * sizeof(unsigned long long)));
        h_gains_n_ = nj * sweeps;
    }
    const uint32_t threads = std::min<uint32_t>(t.threads, 256);
    int occ = 0;
    if ((rc = batch_local_max_ctas_per_sm(threads, &occ))) return rc;
    if (occ < 1) { set_error("am_batch: the guided sweep kernel does not fit on an SM"); return AM_ERR_CUDA; }
    const uint32_t grid = std::min<uint32_t>(t.ctas_per_sm, (uint32_t)occ) * (uint32_t)sms_;
    BatchLocalArgs a;
    a.jobs = d_ljobs_.p;
    a.ch_job = d_sch_job_.p; a.ch_fi = d_sch_fi_.p; a.ch_count = d_sch_count_.p; a.ch_start = d_sch_start_.p;
    std::memcpy(a.ch_off, sch_off_, sizeof(sch_off_));
    a.nphase = nphase_; a.sweeps = (uint32_t)sweeps; a.gains = d_gains_.p; a.bar = d_bar_.p; a.err = d_err_.p;
    auto enqueue = [&]() -> int {
        AMG_CUDA(cudaMemcpyAsync(d_ljobs_.p, h_ljobs_, nj * sizeof(BatchLocalJob), cudaMemcpyHostToDevice, stream_));
        AMG_CUDA(cudaMemsetAsync(d_bar_.p, 0, 4 * sizeof(unsigned), stream_));
        AMG_CUDA(cudaMemsetAsync(d_gains_.p, 0, nj * sweeps * sizeof(unsigned long long), stream_));
        int r = launch_batch_local(a, grid, threads, stream_);
        if (r) return r;
        AMG_CUDA(cudaMemcpyAsync(h_gains_, d_gains_.p, nj * sweeps * sizeof(unsigned long long),
                                 cudaMemcpyDeviceToHost, stream_));
        return AM_OK;
    };
    if (ms) AMG_CUDA(cudaEventRecord(ev0_, stream_));
    if (graph) {
        Graph &g = lgraphs_[sweeps];
        if (g.exec && (g.t.threads != t.threads || g.t.ctas_per_sm != t.ctas_per_sm)) {
            cudaGraphExecDestroy(g.exec);
            g.exec = nullptr;
        }
        if (!g.exec) {
            cudaGraph_t gr = nullptr;
            AMG_CUDA(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
            int r = enqueue();
            cudaError_t ce = cudaStreamEndCapture(stream_, &gr);
            if (r) { if (gr) cudaGraphDestroy(gr); return r; }
            if (ce != cudaSuccess) {
                set_error(std::string("am_batch: stream capture: ") + cudaGetErrorString(ce));
                return AM_ERR_CUDA;
            }
            cudaError_t ie = cudaGraphInstantiate(&g.exec, gr, 0);
            cudaGraphDestroy(gr);
            if (ie != cudaSuccess) {
                g.exec = nullptr;
                set_error(std::string("am_batch: graph instantiate: ") + cudaGetErrorString(ie));
                return AM_ERR_CUDA;
            }
            g.t = t;
        }
        AMG_CUDA(cudaGraphLaunch(g.exec, stream_));
    } else {
        if ((rc = enqueue())) return rc;
    }
    if (ms) AMG_CUDA(cudaEventRecord(ev1_, stream_));
    AMG_CUDA(cudaStreamSynchronize(stream_));
    int err = 0;
    AMG_CUDA(cudaMemcpy(&err, d_err_.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (err) {
        set_error("am_batch: a grid barrier timed out; the jobs' chains are in an unknown state");
        return err;
    }
    if (ms) AMG_CUDA(cudaEventElapsedTime(ms, ev0_, ev1_));
    return AM_OK;
}

// The gains of the last call into each job's cost, sweep counter and front
// copy (guided sweeps keep the job's guided index valid, plain ones do not).
int Batch::apply_gains(size_t sweeps, uint64_t *gains, bool guided) {
    int rc;
    for (size_t j = 0; j < jobs_.size(); ++j) {
        Engine *e = jobs_[j];
        uint64_t sum = 0;
        for (size_t s = 0; s < sweeps; ++s) {
            uint64_t g = h_gains_[j * sweeps + s];
            sum += g;
            if (gains) gains[j * sweeps + s] = g;
        }
        e->sweep_counter += sweeps;
        e->cost_exact -= sum;
        e->local_valid = guided;
        if (guided) e->guided_on = true;
        if ((rc = e->publish_front())) return rc;
    }
    return AM_OK;
}

int Batch::refine_guided(size_t sweeps, uint64_t *gains) {
    if (sweeps == 0) return AM_OK;
    if (sweeps > UINT32_MAX) return AM_ERR_ARG;
    int rc = check_jobs(jobs_);
    if (rc) return rc;
    AMG_CUDA(cudaSetDevice(device_));
    if ((rc = sync_layout())) return rc;  // the phase count of the longest schedule
    if ((rc = prepare_guided(0))) return rc;
    if ((rc = run_local(sweeps, tuning, true, nullptr))) return rc;
    return apply_gains(sweeps, gains, true);
}

// The tuned schedule: tuning.plain_sweeps plain sweeps, then guided ones up
// to `sweeps` in all; gains [njobs][sweeps].
int Batch::refine_schedule(size_t sweeps, uint64_t *gains) {
    const size_t np = std::min<size_t>(tuning.plain_sweeps, sweeps);
    std::vector<uint64_t> g1, g2;
    if (gains) { g1.resize(jobs_.size() * std::max<size_t>(np, 1)); g2.resize(jobs_.size() * std::max<size_t>(sweeps - np, 1)); }
    int rc;
    if (np && (rc = refine(np, gains ? g1.data() : nullptr))) return rc;
    if (sweeps > np && (rc = refine_guided(sweeps - np, gains ? g2.data() : nullptr))) return rc;
    if (gains)
        for (size_t j = 0; j < jobs_.size(); ++j) {
            for (size_t s = 0; s < np; ++s) gains[j * sweeps + s] = g1[j * np + s];
            for (size_t s = np; s < sweeps; ++s) gains[j * sweeps + s] = g2[j * (sweeps - np) + (s - np)];
        }
    return AM_OK;
}

// Schedule autotuner: for a budget of `sweeps` per job, tries plain sweeps
// first for 0, 1/8, 1/4 and 1/2 of the budget and guided sweeps for the
// rest, each from the jobs' chains as they are (restored before each
// trial), and keeps the split whose summed final cost is lowest (on a tie,
// the faster).  The chains, sweep counters and guided indices are left as
// they were (an index is rebuilt on the next guided call).
int Batch::tune_schedule(size_t sweeps) {
    if (sweeps == 0 || sweeps > 100000) return AM_ERR_ARG;
    int rc = check_jobs(jobs_);
    if (rc) return rc;
    AMG_CUDA(cudaSetDevice(device_));
    if ((rc = sync_layout())) return rc;
    std::vector<uint64_t> off(jobs_.size() + 1, 0);
    for (size_t j = 0; j < jobs_.size(); ++j) off[j + 1] = off[j] + jobs_[j]->N * jobs_[j]->K;
    DBuf<uint64_t> snap;
    if ((rc = snap.reserve(std::max<uint64_t>(off.back(), 1)))) return rc;
    auto copy_all = [&](bool save) -> int {
        for (size_t j = 0; j < jobs_.size(); ++j) {
            size_t bytes = (off[j + 1] - off[j]) * 8;
            if (!bytes) continue;
            if (save) AMG_CUDA(cudaMemcpyAsync(snap.p + off[j], jobs_[j]->d_P.p, bytes, cudaMemcpyDeviceToDevice, stream_));
            else AMG_CUDA(cudaMemcpyAsync(jobs_[j]->d_P.p, snap.p + off[j], bytes, cudaMemcpyDeviceToDevice, stream_));
        }
        AMG_CUDA(cudaStreamSynchronize(stream_));
        for (Engine *e : jobs_) e->local_valid = false;
        return AM_OK;
    };
    if ((rc = copy_all(true))) return rc;
    const size_t cands[] = {0, sweeps / 8, sweeps / 4, sweeps / 2};
    uint64_t best_cost = UINT64_MAX;
    float best_ms = 1e30f;
    size_t best_np = 0;
    for (size_t np : cands) {
        if ((rc = copy_all(false))) return rc;
        uint64_t gain = 0;
        float ms_total = 0.f, ms = 0.f;
        if (np) {
            fill_jobs(jobs_, h_jobs_);
            if ((rc = run(np, tuning, false, &ms))) return rc;
            ms_total += ms;
            for (size_t k = 0; k < jobs_.size() * np; ++k) gain += h_gains_[k];
        }
        if (sweeps > np) {
            if ((rc = prepare_guided(np))) return rc;
            if ((rc = run_local(sweeps - np, tuning, false, &ms))) return rc;
            ms_total += ms;
            for (size_t k = 0; k < jobs_.size() * (sweeps - np); ++k) gain += h_gains_[k];
        }
        uint64_t cost = 0;
        for (Engine *e : jobs_) cost += e->cost_exact;
        cost -= gain;
        if (cost < best_cost || (cost == best_cost && ms_total < best_ms)) {
            best_cost = cost;
            best_ms = ms_total;
            best_np = np;
        }
    }
    if ((rc = copy_all(false))) return rc;
    tuning.plain_sweeps = best_np;
    return AM_OK;
}

// Times `trial_sweeps` real sweeps of every job under each candidate launch
// shape and schedule, on the jobs' chains restored from a snapshot before
// each trial, and keeps the fastest.  The chains and sweep counters are left
// as they were.
int Batch::tune(size_t trial_sweeps) {
    if (trial_sweeps == 0 || trial_sweeps > 1000) return AM_ERR_ARG;
    int rc = check_jobs(jobs_);
    if (rc) return rc;
    AMG_CUDA(cudaSetDevice(device_));
    std::vector<uint64_t> off(jobs_.size() + 1, 0);
    for (size_t j = 0; j < jobs_.size(); ++j) off[j + 1] = off[j] + jobs_[j]->N * jobs_[j]->K;
    DBuf<uint64_t> snap;
    if ((rc = snap.reserve(std::max<uint64_t>(off.back(), 1)))) return rc;
    auto copy_all = [&](bool save) -> int {
        for (size_t j = 0; j < jobs_.size(); ++j) {
            size_t bytes = (off[j + 1] - off[j]) * 8;
            if (!bytes) continue;
            if (save) AMG_CUDA(cudaMemcpyAsync(snap.p + off[j], jobs_[j]->d_P.p, bytes, cudaMemcpyDeviceToDevice, stream_));
            else AMG_CUDA(cudaMemcpyAsync(jobs_[j]->d_P.p, snap.p + off[j], bytes, cudaMemcpyDeviceToDevice, stream_));
        }
        return AM_OK;
    };
    if ((rc = copy_all(true))) return rc;
    fill_jobs(jobs_, h_jobs_);
    BatchTuning best = tuning;
    float best_ms = 1e30f;
    const uint32_t threads_c[] = {128, 256, 512};
    const uint32_t ctas_c[] = {1, 2, 4, 8, 16};
    const uint32_t chunk_c[] = {1024, 4096, 16384};
    bool warm = false;
    for (uint32_t order : {0u, 1u})
        for (uint32_t chunk : chunk_c) {
            tuning.chunk = chunk;
            tuning.order = order;
            if ((rc = sync_layout())) return rc;
            for (uint32_t th : threads_c) {
                int occ = 0;
                if ((rc = batch_max_ctas_per_sm(th, &occ))) return rc;
                for (uint32_t c : ctas_c) {
                    if ((int)c > occ) continue;
                    BatchTuning t{th, c, chunk, order};
                    float ms = 0.f, m2 = 1e30f;
                    for (int rep = 0; rep < (warm ? 2 : 3); ++rep) {
                        if ((rc = copy_all(false))) return rc;
                        if ((rc = run(trial_sweeps, t, false, &ms))) return rc;
                        m2 = std::min(m2, ms);
                    }
                    warm = true;
                    if (m2 < best_ms) { best_ms = m2; best = t; }
                }
            }
        }
    if ((rc = copy_all(false))) return rc;
    AMG_CUDA(cudaStreamSynchronize(stream_));
    tuning = best;
    drop_graphs();
    return sync_layout();
}

}  // namespace amg

namespace amg {

// Streams and events of the pipelined batched frames, for `groups` launch
// groups of up to 32 jobs.
int Batch::ensure_render_streams(uint32_t groups) {
    if (!bstream_) AMG_CUDA(cudaStreamCreateWithFlags(&bstream_, cudaStreamNonBlocking));
    if (!cstream_) AMG_CUDA(cudaStreamCreateWithFlags(&cstream_, cudaStreamNonBlocking));
    for (int k = 0; k < 2; ++k) {
        if (!ev_time_[k]) AMG_CUDA(cudaEventCreateWithFlags(&ev_time_[k], cudaEventDisableTiming));
        if (!ev_copied_[k]) AMG_CUDA(cudaEventCreateWithFlags(&ev_copied_[k], cudaEventDisableTiming));
    }
    while (ev_bin_.size() < groups) {
        cudaEvent_t e;
        AMG_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        ev_bin_.push_back(e);
    }
    return AM_OK;
}

// Frames of every job at the times ts, pipelined over the times: the atom
// frames of all jobs per time through render_frames_batch (one binning, one
// resolve and one tile-plan launch per group of up to 32 jobs), time i's
// binning on a second stream beside time i-1's resolve; fluid frames and
// frames before chains through each job's own render.  Host destinations
// the GPU can store into (pinned, mapped) are written directly; others get a
// copy from one of two staging frames per job, issued on a copy stream after
// the next time's launches so the pipeline keeps running.
int Batch::render(const double *ts, size_t n, uint8_t *const *outs, bool on_device) {
    if (n == 0) return AM_OK;
    if (!ts || !outs) return AM_ERR_ARG;
    for (size_t j = 0; j < jobs_.size(); ++j) {
        if (!outs[j]) return AM_ERR_ARG;
        if (jobs_[j]->is_busy()) return AM_ERR_BUSY;
    }
    AMG_CUDA(cudaSetDevice(device_));
    // work a failed earlier call may have left on the batch's own streams
    if (bstream_) AMG_CUDA(cudaStreamSynchronize(bstream_));
    if (cstream_) AMG_CUDA(cudaStreamSynchronize(cstream_));
    AMG_CUDA(cudaStreamSynchronize(stream_));
    const size_t nj = jobs_.size();
    std::vector<size_t> fsz(nj), stage_off(nj, SIZE_MAX);
    std::vector<uint8_t *> base(nj);
    size_t half = 0;
    int rc;
    for (size_t j = 0; j < nj; ++j) {
        Engine *e = jobs_[j];
        if ((rc = e->ensure_streams_public())) return rc;
        // the job's own frames in flight read the slots and pairs reused here
        AMG_CUDA(cudaStreamSynchronize(e->rstream));
        render_quiesce(e->rw);
        fsz[j] = (size_t)e->width * e->height * 4;
        base[j] = outs[j];
        if (!on_device) {
            uint8_t *d = mapped_host_range(outs[j], n * fsz[j]);
            if (d) {
                base[j] = d;
            } else {
                stage_off[j] = half;
                half += (fsz[j] + 255) / 256 * 256;
            }
        }
    }
    if (half && (rc = stage_.reserve(2 * half))) return rc;
    const uint32_t groups = (uint32_t)(nj + 2);  // launch groups per time: at most one per job
    if ((rc = ensure_render_streams(groups))) return rc;
    // bstream_ starts after the work already on stream_ (earlier calls)
    AMG_CUDA(cudaEventRecord(ev_time_[1], stream_));
    AMG_CUDA(cudaStreamWaitEvent(bstream_, ev_time_[1], 0));
    std::vector<RenderJob> rj;
    rj.reserve(nj);
    std::vector<char> batched(nj), was_batched(nj);
    auto copy_out = [&](size_t i) -> int {
        // time i's staged frames, once its resolves are done
        bool any = false;
        for (size_t j = 0; j < nj; ++j) any |= was_batched[j] && stage_off[j] != SIZE_MAX;
        if (!any) return AM_OK;
        AMG_CUDA(cudaStreamWaitEvent(cstream_, ev_time_[i & 1], 0));
        for (size_t j = 0; j < nj; ++j)
            if (was_batched[j] && stage_off[j] != SIZE_MAX)
                AMG_CUDA(cudaMemcpyAsync(outs[j] + i * fsz[j], stage_.p + (i & 1) * half + stage_off[j], fsz[j],
                                         cudaMemcpyDeviceToHost, cstream_));
        AMG_CUDA(cudaEventRecord(ev_copied_[i & 1], cstream_));
        return AM_OK;
    };
    for (size_t i = 0; i < n; ++i) {
        double integ;
        double t = std::modf(ts[i], &integ);
        if (t < 0.0) t += 1.0;
        rj.clear();
        bool staged = false;
        for (size_t j = 0; j < nj; ++j) {
            Engine *e = jobs_[j];
            batched[j] = 0;
            if (fsz[j] == 0) continue;
            if (e->fN == 0 || e->fK == 0 || e->front.fluidsteps > 0) {
                // the job's own render on its render stream, waited for
                if ((rc = e->render(ts[i], outs[j] + i * fsz[j], on_device))) return rc;
                AMG_CUDA(cudaStreamSynchronize(e->rstream));
            } else {
                uint8_t *dst = base[j] + i * fsz[j];
                if (stage_off[j] != SIZE_MAX) {
                    dst = stage_.p + (i & 1) * half + stage_off[j];
                    staged = true;
                }
                RenderJob r;
                r.w = e->rw;
                e->frame_scene(t, r.sc, &r.frame_key);
                r.time = t;
                r.out = dst;
                rj.push_back(r);
                batched[j] = 1;
            }
        }
        // this staging half was last copied out two times ago
        if (staged && i >= 2) AMG_CUDA(cudaStreamWaitEvent(stream_, ev_copied_[i & 1], 0));
        BatchPipe bp{bstream_, ev_bin_.data(), groups, i > 0 ? ev_time_[(i - 1) & 1] : nullptr};
        if ((rc = render_frames_batch(rj.data(), rj.size(), stream_, &bp))) return rc;
        AMG_CUDA(cudaEventRecord(ev_time_[i & 1], stream_));
        if (i > 0 && (rc = copy_out(i - 1))) return rc;
        was_batched = batched;
    }
    if ((rc = copy_out(n - 1))) return rc;
    AMG_CUDA(cudaStreamSynchronize(bstream_));
    AMG_CUDA(cudaStreamSynchronize(stream_));
    AMG_CUDA(cudaStreamSynchronize(cstream_));
    return AM_OK;
}

}  // namespace amg
