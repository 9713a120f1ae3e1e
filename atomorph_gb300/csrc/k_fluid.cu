// Fluid solver: FluidModel::step (fluidmodel.cpp:165-580) in FP32 on
// structure-of-arrays particles and a structure-of-arrays grid.
//
// The reference's MLS-MPM liquid step is four particle passes with grid
// reductions between them:
//   k_fl_p2g      quadratic B-spline weights of the 3x3 stencil; mass,
//                 density and density gradient to the nodes; strength-weighted
//                 colour of mature particles (fluidmodel.cpp:191-249)
//   k_fl_forces   bicubic density from the 2x2 cell, pressure (clamped at 2),
//                 wall forces, scattered as node accelerations (:271-357)
//   k_fl_div      node accelerations / mass (:359-369)
//   k_fl_vel      G2P acceleration plus the attractor pull (a = 0.03 toward
//                 the particle's gravity point), momentum back to the nodes
//                 (:373-435)
//   k_fl_div      node velocities / mass (:437-443)
//   k_fl_advect   G2P velocity and node colour, advection, freedom-radius pull
//                 toward the gravity point, walls (:447-567)
// Node sums use FP32 atomics (order-independent up to rounding; the
// reference's running colour mean equals the weighted sum / weight used
// here).  The reference jitters wall contacts with rand() in [0, 0.01]; here
// the jitter is a counter hash of (step, particle) in the same range.
// Grid clearing replaces the reference's active-node list: every node a step
// touches is zero before the next step either way.
#include "common.cuh"
#include "fluid.cuh"
#include "kernels.h"

#include <vector>

namespace amg {

namespace {


struct Stencil {
    int cx, cy;
    float px[3], py[3], gx[3], gy[3];
};

// Stencil origin clamped into the grid so no state can index outside it
// (inside the walls, fluidmodel.cpp:553-566, the clamp never acts).
__device__ __forceinline__ Stencil stencil(float x, float y, uint32_t gsx, uint32_t gsy) {
    Stencil s;
    s.cx = min(max((int)(x - 0.5f), 0), (int)gsx - 3);
    s.cy = min(max((int)(y - 0.5f), 0), (int)gsy - 3);
    float u = (float)s.cx - x;
    s.px[0] = 0.5f * u * u + 1.5f * u + 1.125f; s.gx[0] = u + 1.5f; u += 1.f;
    s.px[1] = -u * u + 0.75f; s.gx[1] = -2.f * u; u += 1.f;
    s.px[2] = 0.5f * u * u - 1.5f * u + 1.125f; s.gx[2] = u - 1.5f;
    float v = (float)s.cy - y;
    s.py[0] = 0.5f * v * v + 1.5f * v + 1.125f; s.gy[0] = v + 1.5f; v += 1.f;
    s.py[1] = -v * v + 0.75f; s.gy[1] = -2.f * v; v += 1.f;
    s.py[2] = 0.5f * v * v - 1.5f * v + 1.125f; s.gy[2] = v - 1.5f;
    return s;
}

struct FlArgs {
    float *P;
    const uint8_t *flags;
    int2 *cell;
    float *G;
    uint32_t n, gsx, gsy;
    float freedom_radius, w_pull;  // w_pull = 1 / (steps_left + 1)
    uint64_t step;
};

#define FL(f, i) a.P[(size_t)(f) * a.n + (i)]
#define ND_(f, q) a.G[(size_t)(f) * ((size_t)a.gsx * a.gsy) + (q)]

// Grid index of node (i, j) = grid[i][j] of the reference (x-major).
__device__ __forceinline__ size_t node(const FlArgs &a, int i, int j) { return (size_t)i * a.gsy + j; }

__global__ void k_fl_p2g(FlArgs a) {
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < a.n; p += gridDim.x * blockDim.x) {
        uint8_t fl = a.flags[p];
        if (!(fl & 1)) continue;
        Stencil s = stencil(FL(PX, p), FL(PY, p), a.gsx, a.gsy);
        a.cell[p] = make_int2(s.cx, s.cy);
        bool colour = (fl & 2) && FL(PSTR, p) > 0.f;
        float str = FL(PSTR, p), r = FL(Pr, p), g = FL(Pg, p), b = FL(Pb, p), al = FL(Pa, p);
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                size_t q = node(a, s.cx + i, s.cy + j);
                float phi = s.px[i] * s.py[j];
                atomicAdd(&ND_(NM, q), phi);  // material mass 1
                atomicAdd(&ND_(ND, q), phi);
                atomicAdd(&ND_(NGX, q), s.gx[i] * s.py[j]);
                atomicAdd(&ND_(NGY, q), s.px[i] * s.gy[j]);
                if (colour) {
                    atomicAdd(&ND_(NW, q), str);
                    atomicAdd(&ND_(NR, q), str * r);
                    atomicAdd(&ND_(NG, q), str * g);
                    atomicAdd(&ND_(NB, q), str * b);
                    atomicAdd(&ND_(NA, q), str * al);
                }
            }
    }
}

__global__ void k_fl_forces(FlArgs a) {
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < a.n; p += gridDim.x * blockDim.x) {
        if (!(a.flags[p] & 1)) continue;
        float x = FL(PX, p), y = FL(PY, p);
        int cx = min(max((int)x, 0), (int)a.gsx - 2), cy = min(max((int)y, 0), (int)a.gsy - 2);
        size_t n01 = node(a, cx, cy), n02 = node(a, cx, cy + 1), n11 = node(a, cx + 1, cy),
               n12 = node(a, cx + 1, cy + 1);
        float d01 = ND_(ND, n01), d02 = ND_(ND, n02), d11 = ND_(ND, n11), d12 = ND_(ND, n12);
        float gx01 = ND_(NGX, n01), gx02 = ND_(NGX, n02), gx11 = ND_(NGX, n11), gx12 = ND_(NGX, n12);
        float gy01 = ND_(NGY, n01), gy02 = ND_(NGY, n02), gy11 = ND_(NGY, n11), gy12 = ND_(NGY, n12);
        float pdx = d11 - d01, pdy = d02 - d01;
        float C20 = 3.f * pdx - gx11 - 2.f * gx01, C02 = 3.f * pdy - gy02 - 2.f * gy01;
        float C30 = -2.f * pdx + gx11 + gx01, C03 = -2.f * pdy + gy02 + gy01;
        float csum1 = d01 + gy01 + C02 + C03, csum2 = d01 + gx01 + C20 + C30;
        float C21 = 3.f * d12 - 2.f * gx02 - gx12 - 3.f * csum1 - C20;
        float C31 = -2.f * d12 + gx02 + gx12 + 2.f * csum1 - C30;
        float C12 = 3.f * d12 - 2.f * gy11 - gy12 - 3.f * csum2 - C02;
        float C13 = -2.f * d12 + gy11 + gy12 + 2.f * csum2 - C03;
        float C11 = gx02 - C13 - C12 - gx01;
        float u = x - cx, u2 = u * u, u3 = u * u2, v = y - cy, v2 = v * v, v3 = v * v2;
        float density = d01 + gx01 * u + gy01 * v + C20 * u2 + C02 * v2 + C30 * u3 + C03 * v3 + C21 * u2 * v +
                        C31 * u3 * v + C12 * u * v2 + C13 * u * v3 + C11 * u * v;
        float pressure = fminf(density - 1.f, 2.f);
        float fx = 0.f, fy = 0.f;
        if (x < 4.f) fx += 4.f - x;
        else if (x > (float)(a.gsx - 5)) fx += (float)(a.gsx - 5) - x;
        if (y < 4.f) fy += 4.f - y;
        else if (y > (float)(a.gsy - 5)) fy += (float)(a.gsy - 5) - y;
        Stencil s = stencil(x, y, a.gsx, a.gsy);
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                size_t q = node(a, s.cx + i, s.cy + j);
                float phi = s.px[i] * s.py[j];
                atomicAdd(&ND_(NAX, q), -((s.gx[i] * s.py[j]) * pressure) + fx * phi);
                atomicAdd(&ND_(NAY, q), -((s.px[i] * s.gy[j]) * pressure) + fy * phi);
            }
    }
}

__global__ void k_fl_div(FlArgs a, int fa, int fb) {
    size_t G = (size_t)a.gsx * a.gsy;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < G; q += (size_t)gridDim.x * blockDim.x) {
        float m = ND_(NM, q);
        if (m > 0.f) {
            float inv = 1.f / m;
            ND_(fa, q) *= inv;
            ND_(fb, q) *= inv;
        }
    }
}

// Unit step of length `acc` toward (x2, y2), split as the reference splits it
// (fluidmodel.cpp:393-412, 513-538).
__device__ __forceinline__ void pull(float x1, float y1, float x2, float y2, float acc, float &dx, float &dy) {
    float A = fabsf(y1 - y2), B = fabsf(x1 - x2), C = sqrtf(A * A + B * B);
    dx = 0.f; dy = 0.f;
    if (acc >= C) acc = C;
    if (B <= 0.f) {
        dy = y2 <= y1 ? -acc : acc;
    } else if (C > 0.f) {
        float ddx = (acc * B) / C, ddy = (A * ddx) / B;
        dx = x1 <= x2 ? ddx : -ddx;
        dy = y1 <= y2 ? ddy : -ddy;
    }
}

__global__ void k_fl_vel(FlArgs a) {
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < a.n; p += gridDim.x * blockDim.x) {
        uint8_t fl = a.flags[p];
        if (!(fl & 1)) continue;
        float x = FL(PX, p), y = FL(PY, p);
        Stencil s = stencil(x, y, a.gsx, a.gsy);
        float cax, cay;
        pull(x, y, FL(PGX, p), FL(PGY, p), 0.03f, cax, cay);
        float u = FL(PU, p), v = FL(PV, p);
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                size_t q = node(a, s.cx + i, s.cy + j);
                float phi = s.px[i] * s.py[j];
                u += phi * (ND_(NAX, q) + cax);
                v += phi * (ND_(NAY, q) + cay);
            }
        FL(PU, p) = u;
        FL(PV, p) = v;
        float mu = (fl & 2) ? u : 0.f, mv = (fl & 2) ? v : 0.f;
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                size_t q = node(a, s.cx + i, s.cy + j);
                float phi = s.px[i] * s.py[j];
                atomicAdd(&ND_(NU, q), phi * mu);
                atomicAdd(&ND_(NV, q), phi * mv);
            }
    }
}

__global__ void k_fl_advect(FlArgs a) {
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < a.n; p += gridDim.x * blockDim.x) {
        uint8_t fl = a.flags[p];
        if (!(fl & 1)) continue;
        float x = FL(PX, p), y = FL(PY, p);
        Stencil s = stencil(x, y, a.gsx, a.gsy);
        float gu = 0.f, gv = 0.f, w = 0.f, nR = 0.f, nG = 0.f, nB = 0.f, nA = 0.f;
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                size_t q = node(a, s.cx + i, s.cy + j);
                float phi = s.px[i] * s.py[j];
                gu += phi * ND_(NU, q);
                gv += phi * ND_(NV, q);
                float nw = ND_(NW, q);
                if (nw > 0.f) {
                    w += nw;
                    nR += ND_(NR, q); nG += ND_(NG, q); nB += ND_(NB, q); nA += ND_(NA, q);
                }
            }
        if (w > 0.f) {
            nR /= w; nG /= w; nB /= w; nA /= w;
            if (!(fl & 2)) {
                FL(Pr, p) = nR; FL(Pg, p) = nG; FL(Pb, p) = nB; FL(Pa, p) = nA;
            } else {
                float wr = fabsf(nR - FL(PR_, p)), wg = fabsf(nG - FL(PG_, p));
                float wb = fabsf(nB - FL(PB_, p)), wa = fabsf(nA - FL(PA_, p));
                FL(Pr, p) = (1.f - wr) * FL(Pr, p) + wr * nR;
                FL(Pg, p) = (1.f - wg) * FL(Pg, p) + wg * nG;
                FL(Pb, p) = (1.f - wb) * FL(Pb, p) + wb * nB;
                FL(Pa, p) = (1.f - wa) * FL(Pa, p) + wa * nA;
            }
        }
        x += gu;
        y += gv;
        {
            float gxp = FL(PGX, p), gyp = FL(PGY, p);
            float A = fabsf(y - gyp), B = fabsf(x - gxp), C = sqrtf(A * A + B * B);
            float r = a.freedom_radius * FL(PFR, p);
            if (C > r) {
                float mx, my;
                pull(x, y, gxp, gyp, C - r, mx, my);
                x += mx * a.w_pull;
                y += my * a.w_pull;
            }
        }
        float u = gu, v = gv;
        uint32_t h = mix32((uint32_t)a.step * 0x9E3779B1u ^ mix32(p));
        float jit = (float)(h & 0xFFFFFFu) / 16777215.f * 0.01f;
        if (x < 1.f) { x = 1.f + jit; u = 0.f; }
        else if (x > (float)(a.gsx - 2)) { x = (float)(a.gsx - 2) - jit; u = 0.f; }
        if (y < 1.f) { y = 1.f + jit; v = 0.f; }
        else if (y > (float)(a.gsy - 2)) { y = (float)(a.gsy - 2) - jit; v = 0.f; }
        FL(PX, p) = x; FL(PY, p) = y; FL(PU, p) = u; FL(PV, p) = v;
    }
}

}  // namespace

FluidDev *fluid_create(uint32_t gsx, uint32_t gsy, uint32_t n) {
    if (gsx < 8 || gsy < 8) return nullptr;
    FluidDev *f = new FluidDev();
    f->gsx = gsx; f->gsy = gsy; f->n = n;
    size_t G = (size_t)gsx * gsy;
    if (cudaMalloc(&f->P, (size_t)kFlFields * std::max<uint32_t>(n, 1) * 4) != cudaSuccess ||
        cudaMalloc(&f->flags, std::max<uint32_t>(n, 1)) != cudaSuccess ||
        cudaMalloc(&f->cell, sizeof(int2) * std::max<uint32_t>(n, 1)) != cudaSuccess ||
        cudaMalloc(&f->G, (size_t)kFlNode * G * 4) != cudaSuccess) {
        fluid_destroy(f);
        return nullptr;
    }
    cudaMemset(f->P, 0, (size_t)kFlFields * std::max<uint32_t>(n, 1) * 4);
    cudaMemset(f->flags, 0, std::max<uint32_t>(n, 1));
    return f;
}

void fluid_destroy(FluidDev *f) {
    if (!f) return;
    if (f->P) cudaFree(f->P);
    if (f->flags) cudaFree(f->flags);
    if (f->cell) cudaFree(f->cell);
    if (f->G) cudaFree(f->G);
    delete f;
}

// Host exchange in the oracle's field order (x y u v gravity_x gravity_y
// freedom_r active mature strength R G B A r g b a), n particles x 18 doubles.
int fluid_set(FluidDev *f, const double *state, cudaStream_t s) {
    std::vector<float> P((size_t)kFlFields * f->n);
    std::vector<uint8_t> fl(f->n);
    const int map[kFlFields] = {0, 1, 2, 3, 4, 5, 6, 9, 10, 11, 12, 13, 14, 15, 16, 17};
    for (uint32_t i = 0; i < f->n; ++i) {
        const double *q = state + 18 * (size_t)i;
        for (int k = 0; k < kFlFields; ++k) P[(size_t)k * f->n + i] = (float)q[map[k]];
        fl[i] = (uint8_t)((q[7] != 0.0 ? 1 : 0) | (q[8] != 0.0 ? 2 : 0));
    }
    AMG_CUDA(cudaMemcpyAsync(f->P, P.data(), P.size() * 4, cudaMemcpyHostToDevice, s));
    AMG_CUDA(cudaMemcpyAsync(f->flags, fl.data(), fl.size(), cudaMemcpyHostToDevice, s));
    AMG_CUDA(cudaStreamSynchronize(s));
    return AM_OK;
}

int fluid_get(FluidDev *f, double *state, cudaStream_t s) {
    std::vector<float> P((size_t)kFlFields * f->n);
    std::vector<uint8_t> fl(f->n);
    AMG_CUDA(cudaMemcpyAsync(P.data(), f->P, P.size() * 4, cudaMemcpyDeviceToHost, s));
    AMG_CUDA(cudaMemcpyAsync(fl.data(), f->flags, fl.size(), cudaMemcpyDeviceToHost, s));
    AMG_CUDA(cudaStreamSynchronize(s));
    const int map[kFlFields] = {0, 1, 2, 3, 4, 5, 6, 9, 10, 11, 12, 13, 14, 15, 16, 17};
    for (uint32_t i = 0; i < f->n; ++i) {
        double *q = state + 18 * (size_t)i;
        for (int k = 0; k < kFlFields; ++k) q[map[k]] = P[(size_t)k * f->n + i];
        q[7] = (fl[i] & 1) ? 1.0 : 0.0;
        q[8] = (fl[i] & 2) ? 1.0 : 0.0;
    }
    return AM_OK;
}

int fluid_step(FluidDev *f, uint64_t steps_left, double freedom_radius, cudaStream_t s, Prof *prof) {
    FlArgs a;
    a.P = f->P; a.flags = f->flags; a.cell = f->cell; a.G = f->G; a.n = f->n; a.gsx = f->gsx; a.gsy = f->gsy;
    a.freedom_radius = (float)freedom_radius;
    a.w_pull = (float)(1.0 / (double)(steps_left + 1));
    a.step = ++f->step;
    size_t G = (size_t)f->gsx * f->gsy;
    if (prof) prof->open(s);
    AMG_CUDA(cudaMemsetAsync(f->G, 0, (size_t)kFlNode * G * 4, s));
    unsigned gp = (unsigned)std::min<uint64_t>((f->n + 255) / 256, (uint64_t)kSMs * 8);
    unsigned gg = (unsigned)std::min<uint64_t>((G + 255) / 256, (uint64_t)kSMs * 8);
    if (f->n) {
        AMG_LAUNCH(k_fl_p2g, gp, 256, 0, s, a);
        AMG_LAUNCH(k_fl_forces, gp, 256, 0, s, a);
        AMG_LAUNCH(k_fl_div, gg, 256, 0, s, a, (int)NAX, (int)NAY);
        AMG_LAUNCH(k_fl_vel, gp, 256, 0, s, a);
        AMG_LAUNCH(k_fl_div, gg, 256, 0, s, a, (int)NU, (int)NV);
        AMG_LAUNCH(k_fl_advect, gp, 256, 0, s, a);
    }
    if (prof) prof->close(PROF_FLUID, s);
    AMG_CUDA(cudaGetLastError());
    return AM_OK;
}

}  // namespace amg
