// Host side of a batch of morph jobs refined together (am_batch_*): one
// persistent cooperative launch per call, captured once into a CUDA graph
// and replayed, with a launch shape and work schedule picked by an
// autotuner that times real sweeps on a snapshot of the jobs' chains.
#pragma once

#include <map>
#include <vector>

#include "engine.h"

namespace amg {

struct BatchTuning {
    uint32_t threads = 256;      // threads per CTA
    uint32_t ctas_per_sm = 4;    // co-resident CTAs per SM (<= occupancy limit)
    uint32_t chunk = 4096;       // pairs per chunk (a CTA's unit of work)
    uint32_t order = 0;          // 0: each job's chunks together; 1: jobs interleaved chunk by chunk
    uint64_t plain_sweeps = 0;   // schedule: plain sweeps before the guided ones (refine_schedule)
};

class Batch {
  public:
    explicit Batch(std::vector<Engine *> jobs);
    ~Batch();
    int init();
    int refine(size_t sweeps, uint64_t *gains);  // gains: [njobs][sweeps] or null
    int refine_guided(size_t sweeps, uint64_t *gains);
    int refine_schedule(size_t sweeps, uint64_t *gains);  // tuning.plain_sweeps plain, then guided
    int tune(size_t trial_sweeps);
    int tune_schedule(size_t sweeps);
    // frames of every job at times ts[0..n): job j's into outs[j] (n frames of
    // its width * height * 4 bytes, consecutive), device or host memory
    int render(const double *ts, size_t n, uint8_t *const *outs, bool on_device);
    BatchTuning tuning;
    size_t njobs() const { return jobs_.size(); }

  private:
    int sync_layout();                 // rebuild chunks when any job's chain layout changed
    int run(size_t sweeps, const BatchTuning &t, bool graph, float *ms);
    int run_local(size_t sweeps, const BatchTuning &t, bool graph, float *ms);
    int sync_slot_layout();            // slot chunks of the guided sweeps
    int prepare_guided(uint64_t sweep_offset);
    int apply_gains(size_t sweeps, uint64_t *gains, bool guided);
    void drop_graphs();
    std::vector<Engine *> jobs_;
    std::vector<uint64_t> versions_;
    int device_ = 0, sms_ = 0;
    cudaStream_t stream_ = nullptr;
    cudaEvent_t ev0_ = nullptr, ev1_ = nullptr;
    uint32_t nphase_ = 0;
    DBuf<BatchJob> d_jobs_;
    BatchJob *h_jobs_ = nullptr;       // pinned mirror, copied in by the graph
    DBuf<uint32_t> d_ch_job_, d_ch_count_, d_ch_fi_;
    DBuf<uint64_t> d_ch_start_;
    uint32_t ch_off_[4] = {};
    DBuf<unsigned long long> d_gains_;
    unsigned long long *h_gains_ = nullptr;  // pinned, filled by the graph
    size_t h_gains_n_ = 0;
    DBuf<unsigned> d_bar_;
    DBuf<int> d_err_;
    uint32_t chunk_built_ = 0, order_built_ = UINT32_MAX;
    struct Graph { cudaGraphExec_t exec = nullptr; BatchTuning t; };
    std::map<size_t, Graph> graphs_;   // by sweeps per call
    // batched guided sweeps
    DBuf<BatchLocalJob> d_ljobs_;
    BatchLocalJob *h_ljobs_ = nullptr; // pinned mirror
    DBuf<uint32_t> d_sch_job_, d_sch_count_, d_sch_fi_;
    DBuf<uint64_t> d_sch_start_;
    uint32_t sch_off_[4] = {};
    uint32_t slot_chunk_built_ = 0;
    std::vector<uint64_t> sversions_;
    std::map<size_t, Graph> lgraphs_;
    // batched frames: staging for host memory the GPU cannot store into
    // (two halves, alternating with the time), the binning stream, the copy
    // stream and their events (binned per launch group; a time's resolves
    // done and its copies done, per time parity)
    DBuf<uint8_t> stage_;
    cudaStream_t bstream_ = nullptr, cstream_ = nullptr;
    std::vector<cudaEvent_t> ev_bin_;
    cudaEvent_t ev_time_[2] = {nullptr, nullptr}, ev_copied_[2] = {nullptr, nullptr};
    int ensure_render_streams(uint32_t groups);
};

}  // namespace amg
