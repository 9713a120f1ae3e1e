// extern "C" entry points of batched refinement (am_batch_*; no reference
// counterpart).
#include <new>

#include "batch.h"
#include "handle.h"

struct am_batch {
    amg::Batch *b = nullptr;
};

extern "C" {

int am_batch_create(am_batch **out, am_morph *const *jobs, size_t n) {
    if (!out || !jobs || n == 0) return AM_ERR_ARG;
    *out = nullptr;
    std::vector<amg::Engine *> es;
    for (size_t i = 0; i < n; ++i) {
        if (!jobs[i]) return AM_ERR_ARG;
        es.push_back(&jobs[i]->e);
    }
    am_batch *h = new (std::nothrow) am_batch();
    if (!h) return AM_ERR_NOMEM;
    h->b = new (std::nothrow) amg::Batch(std::move(es));
    if (!h->b) { delete h; return AM_ERR_NOMEM; }
    int rc = h->b->init();
    if (rc) {
        delete h->b;
        delete h;
        return rc;
    }
    *out = h;
    return AM_OK;
}

void am_batch_destroy(am_batch *b) {
    if (!b) return;
    delete b->b;
    delete b;
}

int am_batch_refine(am_batch *b, size_t sweeps, uint64_t *gains) {
    if (!b) return AM_ERR_ARG;
    return b->b->refine(sweeps, gains);
}

int am_batch_refine_guided(am_batch *b, size_t sweeps, uint64_t *gains) {
    if (!b) return AM_ERR_ARG;
    return b->b->refine_guided(sweeps, gains);
}

int am_batch_refine_schedule(am_batch *b, size_t sweeps, uint64_t *gains) {
    if (!b) return AM_ERR_ARG;
    return b->b->refine_schedule(sweeps, gains);
}

int am_batch_tune_schedule(am_batch *b, size_t sweeps, size_t *plain_sweeps) {
    if (!b) return AM_ERR_ARG;
    int rc = b->b->tune_schedule(sweeps);
    if (!rc && plain_sweeps) *plain_sweeps = (size_t)b->b->tuning.plain_sweeps;
    return rc;
}

int am_batch_render(am_batch *b, const double *ts, size_t n, uint8_t *const *outs, int outs_on_device) {
    if (!b) return AM_ERR_ARG;
    return b->b->render(ts, n, outs, outs_on_device != 0);
}

int am_batch_tune(am_batch *b, size_t trial_sweeps) {
    if (!b) return AM_ERR_ARG;
    return b->b->tune(trial_sweeps);
}

int am_batch_get_tuning(const am_batch *b, uint32_t *threads, uint32_t *ctas_per_sm, uint32_t *chunk, uint32_t *order) {
    if (!b) return AM_ERR_ARG;
    const amg::BatchTuning &t = b->b->tuning;
    if (threads) *threads = t.threads;
    if (ctas_per_sm) *ctas_per_sm = t.ctas_per_sm;
    if (chunk) *chunk = t.chunk;
    if (order) *order = t.order;
    return AM_OK;
}

int am_batch_set_tuning(am_batch *b, uint32_t threads, uint32_t ctas_per_sm, uint32_t chunk, uint32_t order) {
    if (!b) return AM_ERR_ARG;
    if ((threads != 128 && threads != 256 && threads != 512 && threads != 1024) || ctas_per_sm == 0 ||
        ctas_per_sm > 32 || chunk == 0 || order > 1)
        return AM_ERR_ARG;
    amg::BatchTuning &t = b->b->tuning;
    t.threads = threads;
    t.ctas_per_sm = ctas_per_sm;
    t.chunk = chunk;
    t.order = order;
    return AM_OK;
}

}  // extern "C"
