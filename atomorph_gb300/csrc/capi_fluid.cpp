// extern "C" entry points of the standalone fluid solver (the GB300
// counterpart of the reference's FluidModel, fluidmodel.h:103-142).
#include <algorithm>
#include "engine.h"

struct am_fluid {
    amg::FluidDev *f = nullptr;
    cudaStream_t s = nullptr;
};

extern "C" {

int am_fluid_create(am_fluid **out, uint32_t gsx, uint32_t gsy, uint32_t n) {
    if (!out || gsx < 8 || gsy < 8) return AM_ERR_ARG;
    am_fluid *h = new (std::nothrow) am_fluid();
    if (!h) return AM_ERR_NOMEM;
    if (cudaStreamCreateWithFlags(&h->s, cudaStreamNonBlocking) != cudaSuccess) {
        delete h;
        amg::set_error("cudaStreamCreate failed");
        return AM_ERR_CUDA;
    }
    h->f = amg::fluid_create(gsx, gsy, n);
    if (!h->f) {
        cudaStreamDestroy(h->s);
        delete h;
        return AM_ERR_NOMEM;
    }
    *out = h;
    return AM_OK;
}

void am_fluid_destroy(am_fluid *h) {
    if (!h) return;
    amg::fluid_destroy(h->f);
    if (h->s) cudaStreamDestroy(h->s);
    delete h;
}

int am_fluid_set_particles(am_fluid *h, const double *state) {
    if (!h || !state) return AM_ERR_ARG;
    return amg::fluid_set(h->f, state, h->s);
}

int am_fluid_get_particles(am_fluid *h, double *state) {
    if (!h || !state) return AM_ERR_ARG;
    return amg::fluid_get(h->f, state, h->s);
}

int am_fluid_step(am_fluid *h, size_t steps_left, double freedom_radius) {
    if (!h) return AM_ERR_ARG;
    int rc = amg::fluid_step(h->f, steps_left, freedom_radius, h->s, nullptr);
    if (rc) return rc;
    return cudaStreamSynchronize(h->s) == cudaSuccess ? AM_OK : AM_ERR_CUDA;
}

int am_fluid_steps(am_fluid *h, size_t n, double freedom_radius) {
    if (!h) return AM_ERR_ARG;
    for (size_t i = 0; i < n; i += 1u << 20) {
        const uint32_t k = (uint32_t)std::min<size_t>(n - i, 1u << 20);
        int rc = amg::fluid_run(h->f, k, n - i - k, freedom_radius, h->s, nullptr);
        if (rc) return rc;
    }
    return cudaStreamSynchronize(h->s) == cudaSuccess ? AM_OK : AM_ERR_CUDA;
}

void *am_fluid_stream(am_fluid *h) { return h ? (void *)h->s : nullptr; }

int am_fluid_render_ex(am_fluid *h, uint32_t width, uint32_t height, double sparseness, const uint32_t *bbox,
                       double t, size_t feather, const uint8_t *background, uint8_t *rgba_out) {
    if (!h || !bbox || !rgba_out || !width || !height || !(sparseness > 0.0)) return AM_ERR_ARG;
    if (feather > amg::kMaxFeather) return AM_ERR_UNSUPPORTED;
    uint8_t *d = nullptr, *bg = nullptr;
    const size_t bytes = (size_t)width * height * 4;
    if (cudaMalloc(&d, bytes) != cudaSuccess || (background && cudaMalloc(&bg, bytes) != cudaSuccess)) {
        cudaGetLastError();  // the failed allocation's pending error
        cudaFree(d);
        amg::set_error("cudaMalloc failed");
        return AM_ERR_NOMEM;
    }
    int rc = AM_OK;
    if (bg && cudaMemcpy(bg, background, bytes, cudaMemcpyHostToDevice) != cudaSuccess) rc = AM_ERR_CUDA;
    if (!rc)
        rc = amg::fluid_render_only(h->f, width, height, sparseness, bbox, t, (uint32_t)feather,
                                    reinterpret_cast<const uint32_t *>(bg), d, h->s);
    if (!rc && cudaMemcpy(rgba_out, d, bytes, cudaMemcpyDeviceToHost) != cudaSuccess) rc = AM_ERR_CUDA;
    cudaFree(d);
    cudaFree(bg);
    return rc;
}

int am_fluid_render(am_fluid *h, uint32_t width, uint32_t height, double sparseness, const uint32_t *bbox, double t,
                    uint8_t *rgba_out) {
    return am_fluid_render_ex(h, width, height, sparseness, bbox, t, 0, nullptr, rgba_out);
}

}  // extern "C"
