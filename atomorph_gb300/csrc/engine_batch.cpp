// Batched refinement of many morph jobs (am_batch_*).  No reference
// counterpart: the reference refines one morph per worker thread
// (thread.cpp:173-206).  See k_batch.cu for the kernel.
#include "batch.h"

#include <algorithm>
#include <cstring>

namespace amg {

Batch::Batch(std::vector<Engine *> jobs) : jobs_(std::move(jobs)) {}

Batch::~Batch() {
    drop_graphs();
    if (h_jobs_) cudaFreeHost(h_jobs_);
    if (h_gains_) cudaFreeHost(h_gains_);
    if (ev0_) cudaEventDestroy(ev0_);
    if (ev1_) cudaEventDestroy(ev1_);
    if (stream_) cudaStreamDestroy(stream_);
}

void Batch::drop_graphs() {
    for (auto &g : graphs_)
        if (g.second.exec) cudaGraphExecDestroy(g.second.exec);
    graphs_.clear();
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
    AMG_CUDA(cudaMallocHost(&h_jobs_, jobs_.size() * sizeof(BatchJob)));
    int rc;
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
        e->local_valid = false;  // plain sweeps move points without the guided index
        if ((rc = e->publish_front())) return rc;
    }
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
