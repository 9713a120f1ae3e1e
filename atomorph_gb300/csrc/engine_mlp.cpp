// Host side of the learned swap proposal: parameter initialisation, swap
// sample recording, GPU training and weight exchange.  No reference
// counterpart (the reference refines with uniform random pairs only).
#include <cmath>
#include <cstring>
#include <random>

#include "engine.h"

namespace amg {

int Engine::check_err() {
    if (!d_err.p) return AM_OK;
    int e = 0;
    AMG_CUDA(cudaMemcpyAsync(&e, d_err.p, sizeof(int), cudaMemcpyDeviceToHost, stream));
    AMG_CUDA(cudaStreamSynchronize(stream));
    if (e) {
        AMG_CUDA(cudaMemsetAsync(d_err.p, 0, sizeof(int), stream));
        set_error("a bounded wait on a tensor-core barrier expired");
        return AM_ERR_TIMEOUT;
    }
    return AM_OK;
}

// He-initialised fp32 master weights from a fixed seed, zero biases, Adam
// state cleared, deployed copy packed.
int Engine::mlp_init() {
    if (d_mlp_master.p) return AM_OK;
    int rc = ensure_streams_public();
    if (rc) return rc;
    if ((rc = d_mlp_master.reserve(kMlpMasterParams))) return rc;
    if ((rc = d_mlp_grad.reserve(kMlpMasterParams))) return rc;
    if ((rc = d_adam_m.reserve(kMlpMasterParams))) return rc;
    if ((rc = d_adam_v.reserve(kMlpMasterParams))) return rc;
    if ((rc = d_mlp_dep.reserve(kMlpDeployedFloats))) return rc;
    if ((rc = d_mlp_loss.reserve(4))) return rc;
    if ((rc = d_err.reserve(1))) return rc;
    std::vector<float> m(kMlpMasterParams, 0.f);
    std::mt19937 g(20240917u);
    std::normal_distribution<float> n1(0.f, std::sqrt(2.f / kMlpIn)), n2(0.f, std::sqrt(2.f / kMlpHid));
    for (int i = 0; i < kMlpHid * kMlpIn; ++i) m[i] = n1(g);
    const int w2 = kMlpHid * kMlpIn + kMlpHid;
    for (int i = 0; i < kMlpHid * kMlpHid; ++i) m[w2 + i] = n2(g);
    const int w3 = w2 + kMlpHid * kMlpHid + kMlpHid;
    for (int i = 0; i < kMlpHid; ++i) m[w3 + i] = n2(g) * 0.1f;
    AMG_CUDA(cudaMemcpyAsync(d_mlp_master.p, m.data(), m.size() * 4, cudaMemcpyHostToDevice, stream));
    AMG_CUDA(cudaMemsetAsync(d_adam_m.p, 0, kMlpMasterParams * 4, stream));
    AMG_CUDA(cudaMemsetAsync(d_adam_v.p, 0, kMlpMasterParams * 4, stream));
    AMG_CUDA(cudaMemsetAsync(d_err.p, 0, sizeof(int), stream));
    adam_t = 0;
    rc = mlp_deploy(d_mlp_master.p, d_mlp_dep.p, stream);
    if (rc) return rc;
    AMG_CUDA(cudaStreamSynchronize(stream));
    return AM_OK;
}

int Engine::record_swaps(size_t cap) {
    int rc = mlp_init();
    if (rc) return rc;
    if ((rc = d_rec_feat.reserve(std::max<size_t>(cap, 1) * kMlpIn))) return rc;
    if ((rc = d_rec_gain.reserve(std::max<size_t>(cap, 1)))) return rc;
    if ((rc = d_rec_count.reserve(1))) return rc;
    AMG_CUDA(cudaMemsetAsync(d_rec_count.p, 0, 8, stream));
    AMG_CUDA(cudaStreamSynchronize(stream));
    rec_cap = cap;
    recording = cap > 0;
    recording_outcomes = false;
    return AM_OK;
}

// Makes the next plain sweeps log 1 in `every` of their proposals: pair
// features and the exact criterion's accept (1) / reject (0), the training
// data of the learned pair proposal.  cap 0 stops logging.
int Engine::record_outcomes(size_t cap, uint32_t every) {
    if (every == 0) return AM_ERR_ARG;
    int rc = mlp_init();
    if (rc) return rc;
    if ((rc = d_rec_feat.reserve(std::max<size_t>(cap, 1) * kMlpIn))) return rc;
    if ((rc = d_rec_gain.reserve(std::max<size_t>(cap, 1)))) return rc;
    if ((rc = d_rec_count.reserve(1))) return rc;
    AMG_CUDA(cudaMemsetAsync(d_rec_count.p, 0, 8, stream));
    AMG_CUDA(cudaStreamSynchronize(stream));
    rec_cap = cap;
    recording = false;
    recording_outcomes = cap > 0;
    outcome_every = every;
    return AM_OK;
}

size_t Engine::recorded_swaps(float *feat, float *gains, size_t cap) {
    if (!d_rec_count.p) return 0;
    unsigned long long n = 0;
    if (cudaMemcpy(&n, d_rec_count.p, 8, cudaMemcpyDeviceToHost) != cudaSuccess) return 0;
    size_t k = std::min<size_t>({(size_t)n, (size_t)rec_cap, cap});
    if (feat && k) cudaMemcpy(feat, d_rec_feat.p, k * kMlpIn * 4, cudaMemcpyDeviceToHost);
    if (gains && k) cudaMemcpy(gains, d_rec_gain.p, k * 4, cudaMemcpyDeviceToHost);
    return k;
}

int Engine::train_proposal(const float *feat, const float *gains, size_t n, size_t epochs, double lr,
                           float *loss_out) {
    if (!feat || !gains || n == 0) return AM_ERR_ARG;
    int rc = mlp_init();
    if (rc) return rc;
    recording = false;
    if ((rc = d_io_a.reserve(n * kMlpIn))) return rc;
    if ((rc = d_io_b.reserve(n))) return rc;
    AMG_CUDA(cudaMemcpyAsync(d_io_a.p, feat, n * kMlpIn * 4, cudaMemcpyHostToDevice, stream));
    AMG_CUDA(cudaMemcpyAsync(d_io_b.p, gains, n * 4, cudaMemcpyHostToDevice, stream));
    return train_device(d_io_a.p, d_io_b.p, n, epochs, lr, loss_out);
}

// Trains on the samples the recording sweeps logged, where they lie in device
// memory (no copy to the host and back); recording stops.
int Engine::train_recorded(size_t epochs, double lr, float *loss_out) {
    if (!d_rec_count.p) return AM_ERR_STATE;
    int rc = mlp_init();
    if (rc) return rc;
    unsigned long long cnt = 0;
    AMG_CUDA(cudaMemcpyAsync(&cnt, d_rec_count.p, 8, cudaMemcpyDeviceToHost, stream));
    AMG_CUDA(cudaStreamSynchronize(stream));
    const size_t n = std::min<size_t>((size_t)cnt, (size_t)rec_cap);
    if (n == 0) return AM_ERR_STATE;
    recording = false;
    recording_outcomes = false;
    return train_device(d_rec_feat.p, d_rec_gain.p, n, epochs, lr, loss_out);
}

int Engine::train_device(const float *feat, const float *gains, size_t n, size_t epochs, double lr,
                         float *loss_out) {
    int rc;
    const size_t batch = 16384, steps = (n + batch - 1) / batch;
    // one loss slot per minibatch, read once per epoch
    if ((rc = d_mlp_loss.reserve(steps))) return rc;
    std::vector<float> losses(steps);
    double last = 0.0;
    for (size_t e = 0; e < epochs; ++e) {
        for (size_t k = 0; k < steps; ++k) {
            const size_t b = k * batch, m = std::min(batch, n - b);
            ++adam_t;
            prof.open(stream);
            rc = mlp_train_step(feat + b * kMlpIn, gains + b, m, d_mlp_master.p, d_mlp_dep.p, d_mlp_grad.p,
                                d_adam_m.p, d_adam_v.p, adam_t, (float)lr, d_mlp_loss.p + k, d_err.p, stream);
            if (rc) return rc;
            prof.close(PROF_MLP, stream);
        }
        AMG_CUDA(cudaMemcpyAsync(losses.data(), d_mlp_loss.p, steps * 4, cudaMemcpyDeviceToHost, stream));
        AMG_CUDA(cudaStreamSynchronize(stream));
        double sum = 0.0;
        for (float l : losses) sum += l;
        last = sum / (double)n;
        rc = check_err();
        if (rc) return rc;
    }
    if (loss_out) *loss_out = (float)last;
    mlp_trained = true;
    return AM_OK;
}

int Engine::proposal_weights(float *w, size_t count, bool set) {
    if (!w || count != (size_t)kMlpMasterParams) return AM_ERR_ARG;
    int rc = mlp_init();
    if (rc) return rc;
    if (set) {
        AMG_CUDA(cudaMemcpyAsync(d_mlp_master.p, w, count * 4, cudaMemcpyHostToDevice, stream));
        rc = mlp_deploy(d_mlp_master.p, d_mlp_dep.p, stream);
        if (rc) return rc;
        mlp_trained = true;
    } else {
        AMG_CUDA(cudaMemcpyAsync(w, d_mlp_master.p, count * 4, cudaMemcpyDeviceToHost, stream));
    }
    AMG_CUDA(cudaStreamSynchronize(stream));
    return AM_OK;
}

int Engine::proposal_forward(const float *feat, size_t n, float *out) {
    int rc = mlp_init();
    if (rc) return rc;
    if ((rc = d_io_a.reserve(std::max<size_t>(n, 1) * kMlpIn))) return rc;
    if ((rc = d_io_b.reserve(std::max<size_t>(n, 1)))) return rc;
    AMG_CUDA(cudaMemcpyAsync(d_io_a.p, feat, n * kMlpIn * 4, cudaMemcpyHostToDevice, stream));
    rc = mlp_forward(d_io_a.p, n, d_mlp_dep.p, d_io_b.p, d_err.p, stream);
    if (rc) return rc;
    AMG_CUDA(cudaMemcpyAsync(out, d_io_b.p, n * 4, cudaMemcpyDeviceToHost, stream));
    AMG_CUDA(cudaStreamSynchronize(stream));
    return check_err();
}

int Engine::proposal_grad(const float *feat, const float *target, size_t n, float *grad, float *loss) {
    int rc = mlp_init();
    if (rc) return rc;
    if ((rc = d_io_a.reserve(std::max<size_t>(n, 1) * kMlpIn))) return rc;
    if ((rc = d_io_b.reserve(std::max<size_t>(n, 1)))) return rc;
    AMG_CUDA(cudaMemcpyAsync(d_io_a.p, feat, n * kMlpIn * 4, cudaMemcpyHostToDevice, stream));
    AMG_CUDA(cudaMemcpyAsync(d_io_b.p, target, n * 4, cudaMemcpyHostToDevice, stream));
    rc = mlp_grad(d_io_a.p, d_io_b.p, n, d_mlp_dep.p, d_mlp_grad.p, d_mlp_loss.p, d_err.p, stream);
    if (rc) return rc;
    AMG_CUDA(cudaMemcpyAsync(grad, d_mlp_grad.p, kMlpMasterParams * 4, cudaMemcpyDeviceToHost, stream));
    if (loss) AMG_CUDA(cudaMemcpyAsync(loss, d_mlp_loss.p, 4, cudaMemcpyDeviceToHost, stream));
    AMG_CUDA(cudaStreamSynchronize(stream));
    return check_err();
}

}  // namespace amg
