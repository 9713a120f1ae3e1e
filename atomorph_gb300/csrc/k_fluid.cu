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
//
// Particles are kept in the caller's order (the morph's particle p is atom
// column p, spatially random).  fluid_run sorts them by 8x8 cell block once
// per call, runs its steps on a gathered copy in that order and scatters the
// changed fields back.  In sorted order a CTA's 256 particles cover a compact
// patch of the grid, so the three deposit passes accumulate into a
// shared-memory copy of the patch's nodes and add it to the grid with one
// atomic per node and field; a CTA whose patch exceeds kPrivNodes nodes (sparse
// regions, block-row ends) deposits directly.
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
    float *P;                 // [kFlFields][n] particles in solver (sorted) order
    const uint8_t *flags;
    const uint32_t *ids;      // [n] caller index of each solver slot (wall-jitter hash)
    float *G;
    uint32_t n, gsx, gsy;
    float freedom_radius, w_pull;  // w_pull = 1 / (steps_left + 1)
    uint64_t step;
};

constexpr int kFlThreads = 256;    // particles per CTA of the deposit passes (one per thread)
constexpr int kPrivNodes = 1024;   // nodes of a CTA's shared-memory patch

// The particle of this thread within its CTA's 256 (a bijection): lane l of
// warp w takes particle 8 l + w.  Particles are sorted by cell, about four
// to a cell, so consecutive particles share their stencil nodes; spread this
// way, the 32 lanes of a warp lie in different cells and each shared-memory
// atomic of a deposit goes to 32 different nodes instead of queueing on a
// few.  The patch sums are integers, so the order changes nothing.
__device__ __forceinline__ uint32_t spread_lane() {
    return (threadIdx.x & 31u) * (kFlThreads / 32) + (threadIdx.x >> 5);
}

// Patch of the CTA's 3x3 stencils (origins (cx, cy) of its active
// particles): box = {x0, y0, width, height} in shared memory.  True when the
// CTA has active particles and the patch fits kPrivNodes nodes (uniform).
// The patch sums are 32-bit fixed point: `bound` is the largest magnitude
// one particle adds to one node in one field, and *scale the largest power of
// two (at most 2^24) at which the CTA's summed bounds stay below 2^31, so no
// node sum can overflow; integer sums are exact and order-free.  *scale is 0
// when that power would be below 2^12 (the patch then sums in FP32).
__device__ bool priv_box(bool act, int cx, int cy, float bound, int *box, int *red, float *scale) {
    int mnx = act ? cx : INT_MAX, mny = act ? cy : INT_MAX, mxx = act ? cx : INT_MIN, mxy = act ? cy : INT_MIN;
    float bsum = act ? bound : 0.f;
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        mnx = min(mnx, __shfl_xor_sync(0xffffffffu, mnx, o));
        mny = min(mny, __shfl_xor_sync(0xffffffffu, mny, o));
        mxx = max(mxx, __shfl_xor_sync(0xffffffffu, mxx, o));
        mxy = max(mxy, __shfl_xor_sync(0xffffffffu, mxy, o));
        bsum += __shfl_xor_sync(0xffffffffu, bsum, o);
    }
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        red[5 * w] = mnx; red[5 * w + 1] = mny; red[5 * w + 2] = mxx; red[5 * w + 3] = mxy;
        red[5 * w + 4] = __float_as_int(bsum);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < kFlThreads / 32; ++k) {
            mnx = min(mnx, red[5 * k]); mny = min(mny, red[5 * k + 1]);
            mxx = max(mxx, red[5 * k + 2]); mxy = max(mxy, red[5 * k + 3]);
            bsum += __int_as_float(red[5 * k + 4]);
        }
        box[0] = mnx; box[1] = mny;
        box[2] = mnx == INT_MAX ? 0 : mxx - mnx + 3;
        box[3] = mnx == INT_MAX ? 0 : mxy - mny + 3;
        // each rounded term adds at most 1/2 more: keep 2^10 of headroom
        int e = 24;
        while (e >= 12 && !(bsum * ldexpf(1.f, e) <= 2147483648.f - 1024.f)) --e;
        box[4] = e >= 12 ? e : 0;
    }
    __syncthreads();
    *scale = box[4] ? ldexpf(1.f, box[4]) : 0.f;
    return box[2] > 0 && box[2] * box[3] <= kPrivNodes;
}

// One term of a patch sum: fixed point at `scale`, or FP32 when scale is 0.
__device__ __forceinline__ void patch_add(float *acc, int q, float v, float scale) {
    if (scale != 0.f) atomicAdd(reinterpret_cast<int *>(acc) + q, __float2int_rn(v * scale));
    else atomicAdd(acc + q, v);
}
__device__ __forceinline__ float patch_get(const float *acc, int q, float scale) {
    return scale != 0.f ? (float)reinterpret_cast<const int *>(acc)[q] / scale : acc[q];
}
// Sum of a per-cell field over the 3x3 cells whose stencils reach patch node
// (lx, ly): cells (lx - 2 .. lx, ly - 2 .. ly) inside the patch's cell range
// [0, bw - 2) x [0, bh - 2).  In fixed point the integer terms are added
// first, so the node sum is the one the nine per-node deposits would give.
__device__ __forceinline__ float cell_sum(const float *acc, int lx, int ly, int bw, int bh, float scale) {
    int isum = 0;
    float fsum = 0.f;
#pragma unroll
    for (int di = 0; di < 3; ++di)
#pragma unroll
        for (int dj = 0; dj < 3; ++dj) {
            const int cx = lx - di, cy = ly - dj;
            if (cx < 0 || cy < 0 || cx >= bw - 2 || cy >= bh - 2) continue;
            if (scale != 0.f) isum += reinterpret_cast<const int *>(acc)[cx * bh + cy];
            else fsum += acc[cx * bh + cy];
        }
    return scale != 0.f ? (float)isum / scale : fsum;
}

#define FL(f, i) a.P[(size_t)(f) * a.n + (i)]
#define ND_(f, q) a.G[(size_t)(f) * ((size_t)a.gsx * a.gsy) + (q)]

// Grid index of node (i, j) = grid[i][j] of the reference (x-major).
__device__ __forceinline__ size_t node(const FlArgs &a, int i, int j) { return (size_t)i * a.gsy + j; }

// Deposit fields of k_fl_p2g's shared patch: mass (= density: material mass
// 1), density gradient x, y, colour weight and weighted R G B A.
enum { QM, QGX, QGY, QW, QR, QG, QB, QA, kQ };

__global__ void __launch_bounds__(kFlThreads) k_fl_p2g(FlArgs a) {
    __shared__ float acc[kQ * kPrivNodes];
    __shared__ int box[5], red[5 * (kFlThreads / 32)];
    const uint32_t p = blockIdx.x * kFlThreads + spread_lane();
    const uint8_t fl = p < a.n ? a.flags[p] : 0;
    const bool act = fl & 1;
    Stencil s{};
    float str = 0.f, r = 0.f, g = 0.f, b = 0.f, al = 0.f;
    bool colour = false;
    if (act) {
        s = stencil(FL(PX, p), FL(PY, p), a.gsx, a.gsy);
        str = FL(PSTR, p); r = FL(Pr, p); g = FL(Pg, p); b = FL(Pb, p); al = FL(Pa, p);
        colour = (fl & 2) && str > 0.f;
    }
    // per-node term bound: phi <= 0.5625, |gradient term| <= 1.5 x 0.75,
    // colour terms str and str x colour
    float bound = 1.125f;
    if (colour)
        bound = fmaxf(bound, fmaxf(fabsf(str), fabsf(str) * fmaxf(fmaxf(fabsf(r), fabsf(g)), fmaxf(fabsf(b), fabsf(al)))));
    float scale;
    if (!priv_box(act, s.cx, s.cy, bound, box, red, &scale)) {
        if (!act) return;
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
        return;
    }
    const int x0 = box[0], y0 = box[1], bw = box[2], bh = box[3], nn = bw * bh;
    for (int q = threadIdx.x; q < nn; q += kFlThreads)
#pragma unroll
        for (int f = 0; f < kQ; ++f) acc[f * kPrivNodes + q] = 0.f;
    __syncthreads();
    if (act) {
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                const int q = (s.cx + i - x0) * bh + (s.cy + j - y0);
                const float phi = s.px[i] * s.py[j];
                patch_add(acc, QM * kPrivNodes + q, phi, scale);
                patch_add(acc, QGX * kPrivNodes + q, s.gx[i] * s.py[j], scale);
                patch_add(acc, QGY * kPrivNodes + q, s.px[i] * s.gy[j], scale);
            }
        if (colour) {
            // The colour terms are the same at all nine nodes of the stencil:
            // one term per particle into its stencil cell, spread over the
            // nodes when the patch is added to the grid (5 shared atomics per
            // particle instead of 45).
            const int c = (s.cx - x0) * bh + (s.cy - y0);
            patch_add(acc, QW * kPrivNodes + c, str, scale);
            patch_add(acc, QR * kPrivNodes + c, str * r, scale);
            patch_add(acc, QG * kPrivNodes + c, str * g, scale);
            patch_add(acc, QB * kPrivNodes + c, str * b, scale);
            patch_add(acc, QA * kPrivNodes + c, str * al, scale);
        }
    }
    __syncthreads();
    for (int q = threadIdx.x; q < nn; q += kFlThreads) {
        const float m = patch_get(acc, QM * kPrivNodes + q, scale), gx = patch_get(acc, QGX * kPrivNodes + q, scale),
                    gy = patch_get(acc, QGY * kPrivNodes + q, scale);
        const int lx = q / bh, ly = q % bh;
        const size_t n = node(a, x0 + lx, y0 + ly);
        if (m != 0.f || gx != 0.f || gy != 0.f) {
            atomicAdd(&ND_(NM, n), m);
            atomicAdd(&ND_(ND, n), m);
            atomicAdd(&ND_(NGX, n), gx);
            atomicAdd(&ND_(NGY, n), gy);
        }
        const float w = cell_sum(acc + QW * kPrivNodes, lx, ly, bw, bh, scale);
        if (w != 0.f) {
            atomicAdd(&ND_(NW, n), w);
            atomicAdd(&ND_(NR, n), cell_sum(acc + QR * kPrivNodes, lx, ly, bw, bh, scale));
            atomicAdd(&ND_(NG, n), cell_sum(acc + QG * kPrivNodes, lx, ly, bw, bh, scale));
            atomicAdd(&ND_(NB, n), cell_sum(acc + QB * kPrivNodes, lx, ly, bw, bh, scale));
            atomicAdd(&ND_(NA, n), cell_sum(acc + QA * kPrivNodes, lx, ly, bw, bh, scale));
        }
    }
}

// Adds a two-field 3x3 deposit (per-node values v1, v2 of the stencil) into
// the grid fields f1, f2 through the CTA's shared patch when it fits.
struct Dep2 {
    float v1[9], v2[9];
};
__device__ __forceinline__ void deposit2(const FlArgs &a, bool act, const Stencil &s, const Dep2 &d, int f1, int f2,
                                         float *acc, int *box, int *red) {
    float bound = 0.f;
    if (act)
#pragma unroll
        for (int k = 0; k < 9; ++k) bound = fmaxf(bound, fmaxf(fabsf(d.v1[k]), fabsf(d.v2[k])));
    float scale;
    if (!priv_box(act, s.cx, s.cy, bound, box, red, &scale)) {
        if (!act) return;
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                const size_t q = node(a, s.cx + i, s.cy + j);
                atomicAdd(&ND_(f1, q), d.v1[3 * i + j]);
                atomicAdd(&ND_(f2, q), d.v2[3 * i + j]);
            }
        return;
    }
    const int x0 = box[0], y0 = box[1], bh = box[3], nn = box[2] * bh;
    for (int q = threadIdx.x; q < nn; q += kFlThreads) {
        acc[q] = 0.f;
        acc[kPrivNodes + q] = 0.f;
    }
    __syncthreads();
    if (act) {
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                const int q = (s.cx + i - x0) * bh + (s.cy + j - y0);
                patch_add(acc, q, d.v1[3 * i + j], scale);
                patch_add(acc, kPrivNodes + q, d.v2[3 * i + j], scale);
            }
    }
    __syncthreads();
    for (int q = threadIdx.x; q < nn; q += kFlThreads) {
        const float u = patch_get(acc, q, scale), v = patch_get(acc, kPrivNodes + q, scale);
        if (u != 0.f || v != 0.f) {
            const size_t n = node(a, x0 + q / bh, y0 + q % bh);
            atomicAdd(&ND_(f1, n), u);
            atomicAdd(&ND_(f2, n), v);
        }
    }
}

__global__ void __launch_bounds__(kFlThreads) k_fl_forces(FlArgs a) {
    __shared__ float acc[2 * kPrivNodes];
    __shared__ int box[5], red[5 * (kFlThreads / 32)];
    const uint32_t p = blockIdx.x * kFlThreads + spread_lane();
    const bool act = p < a.n && (a.flags[p] & 1);
    Stencil s{};
    Dep2 d;
    if (act) {
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
        s = stencil(x, y, a.gsx, a.gsy);
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                float phi = s.px[i] * s.py[j];
                d.v1[3 * i + j] = -((s.gx[i] * s.py[j]) * pressure) + fx * phi;
                d.v2[3 * i + j] = -((s.px[i] * s.gy[j]) * pressure) + fy * phi;
            }
    }
    deposit2(a, act, s, d, NAX, NAY, acc, box, red);
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

__global__ void __launch_bounds__(kFlThreads) k_fl_vel(FlArgs a) {
    __shared__ float acc[2 * kPrivNodes];
    __shared__ float pg[2 * kPrivNodes];  // the patch's node accelerations (gathered as in k_fl_advect)
    __shared__ int box[5], red[5 * (kFlThreads / 32)];
    const uint32_t p = blockIdx.x * kFlThreads + spread_lane();
    const uint8_t fl = p < a.n ? a.flags[p] : 0;
    const bool act = fl & 1;
    Stencil s{};
    Dep2 d;
    float x = 0.f, y = 0.f;
    if (act) {
        x = FL(PX, p);
        y = FL(PY, p);
        s = stencil(x, y, a.gsx, a.gsy);
    }
    float unused;
    const bool patch = priv_box(act, s.cx, s.cy, 0.f, box, red, &unused);
    const int x0 = box[0], y0 = box[1], bh = box[3];
    if (patch) {
        const int nn = box[2] * bh;
        for (int q = threadIdx.x; q < nn; q += kFlThreads) {
            const size_t n = node(a, x0 + q / bh, y0 + q % bh);
            pg[q] = ND_(NAX, n);
            pg[kPrivNodes + q] = ND_(NAY, n);
        }
        __syncthreads();
    }
    if (act) {
        float cax, cay;
        pull(x, y, FL(PGX, p), FL(PGY, p), 0.03f, cax, cay);
        float u = FL(PU, p), v = FL(PV, p);
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                float ax, ay;
                if (patch) {
                    const int q = (s.cx + i - x0) * bh + (s.cy + j - y0);
                    ax = pg[q];
                    ay = pg[kPrivNodes + q];
                } else {
                    const size_t q = node(a, s.cx + i, s.cy + j);
                    ax = ND_(NAX, q);
                    ay = ND_(NAY, q);
                }
                float phi = s.px[i] * s.py[j];
                u += phi * (ax + cax);
                v += phi * (ay + cay);
            }
        FL(PU, p) = u;
        FL(PV, p) = v;
        float mu = (fl & 2) ? u : 0.f, mv = (fl & 2) ? v : 0.f;
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                float phi = s.px[i] * s.py[j];
                d.v1[3 * i + j] = phi * mu;
                d.v2[3 * i + j] = phi * mv;
            }
    }
    deposit2(a, act, s, d, NU, NV, acc, box, red);
}

// The node fields advect reads, in the order of its shared-memory patch.
__host__ __device__ constexpr int advect_field(int f) {
    return f == 0 ? NU : f == 1 ? NV : f == 2 ? NW : f == 3 ? NR : f == 4 ? NG : f == 5 ? NB : NA;
}

__global__ void __launch_bounds__(kFlThreads) k_fl_advect(FlArgs a) {
    // The CTA's particles are neighbours in solver order, so their stencils
    // cover a compact patch: its node fields are read once into shared
    // memory and every particle gathers its 3x3 nodes from there (the grid
    // itself when the patch exceeds kPrivNodes nodes).
    __shared__ float pg[7 * kPrivNodes];
    __shared__ int box[5], red[5 * (kFlThreads / 32)];
    const uint32_t p = blockIdx.x * kFlThreads + threadIdx.x;
    const uint8_t fl = p < a.n ? a.flags[p] : 0;
    const bool act = fl & 1;
    float x = 0.f, y = 0.f;
    Stencil s{};
    if (act) {
        x = FL(PX, p);
        y = FL(PY, p);
        s = stencil(x, y, a.gsx, a.gsy);
    }
    float unused;
    const bool patch = priv_box(act, s.cx, s.cy, 0.f, box, red, &unused);
    const int x0 = box[0], y0 = box[1], bh = box[3];
    if (patch) {
        const int nn = box[2] * bh;
        for (int q = threadIdx.x; q < nn; q += kFlThreads) {
            const size_t n = node(a, x0 + q / bh, y0 + q % bh);
#pragma unroll
            for (int f = 0; f < 7; ++f) pg[f * kPrivNodes + q] = ND_(advect_field(f), n);
        }
        __syncthreads();
    }
    if (act) {
        auto nd = [&](int f, int i, int j) -> float {
            return patch ? pg[f * kPrivNodes + (s.cx + i - x0) * bh + (s.cy + j - y0)]
                         : ND_(advect_field(f), node(a, s.cx + i, s.cy + j));
        };
        float gu = 0.f, gv = 0.f, w = 0.f, nR = 0.f, nG = 0.f, nB = 0.f, nA = 0.f;
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                float phi = s.px[i] * s.py[j];
                gu += phi * nd(0, i, j);
                gv += phi * nd(1, i, j);
                float nw = nd(2, i, j);
                if (nw > 0.f) {
                    w += nw;
                    nR += nd(3, i, j); nG += nd(4, i, j); nB += nd(5, i, j); nA += nd(6, i, j);
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
        uint32_t h = mix32((uint32_t)a.step * 0x9E3779B1u ^ mix32(a.ids ? a.ids[p] : p));
        float jit = (float)(h & 0xFFFFFFu) / 16777215.f * 0.01f;
        if (x < 1.f) { x = 1.f + jit; u = 0.f; }
        else if (x > (float)(a.gsx - 2)) { x = (float)(a.gsx - 2) - jit; u = 0.f; }
        if (y < 1.f) { y = 1.f + jit; v = 0.f; }
        else if (y > (float)(a.gsy - 2)) { y = (float)(a.gsy - 2) - jit; v = 0.f; }
        FL(PX, p) = x; FL(PY, p) = y; FL(PU, p) = u; FL(PV, p) = v;
    }
}

// Sort key of a particle: its stencil cell's 8x8 block (row-major over
// blocks), then the cell inside the block; inactive particles sort last.
__global__ void k_fl_keys(const float *__restrict__ P, const uint8_t *__restrict__ flags, uint32_t n,
                          uint32_t gsx, uint32_t gsy, uint32_t *keys, uint32_t *ids) {
    const uint32_t nbx = (gsx + 7) / 8, nby = (gsy + 7) / 8;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        ids[p] = p;
        if (!(flags[p] & 1)) {
            keys[p] = nbx * nby * 64u;
            continue;
        }
        const int cx = min(max((int)(P[(size_t)PX * n + p] - 0.5f), 0), (int)gsx - 3);
        const int cy = min(max((int)(P[(size_t)PY * n + p] - 0.5f), 0), (int)gsy - 3);
        keys[p] = (((uint32_t)cy >> 3) * nbx + ((uint32_t)cx >> 3)) << 6 | ((uint32_t)cy & 7u) << 3 | ((uint32_t)cx & 7u);
    }
}

__global__ void k_fl_gather(const float *__restrict__ P, const uint8_t *__restrict__ flags,
                            const uint32_t *__restrict__ ids, uint32_t n, float *S, uint8_t *sflags) {
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        const uint32_t p = ids[j];
        sflags[j] = flags[p];
#pragma unroll
        for (int k = 0; k < kFlFields; ++k) S[(size_t)k * n + j] = P[(size_t)k * n + p];
    }
}

// The fields a step changes (position, velocity, current colour) back to the
// caller's order.
__global__ void k_fl_scatter(const float *__restrict__ S, const uint32_t *__restrict__ ids, uint32_t n, float *P) {
    const int changed[8] = {PX, PY, PU, PV, Pr, Pg, Pb, Pa};
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        const uint32_t p = ids[j];
#pragma unroll
        for (int k = 0; k < 8; ++k) P[(size_t)changed[k] * n + p] = S[(size_t)changed[k] * n + j];
    }
}

}  // namespace

FluidDev *fluid_create(uint32_t gsx, uint32_t gsy, uint32_t n) {
    if (gsx < 8 || gsy < 8) return nullptr;
    FluidDev *f = new FluidDev();
    f->gsx = gsx; f->gsy = gsy; f->n = n;
    size_t G = (size_t)gsx * gsy;
    const size_t m = std::max<uint32_t>(n, 1);
    if (cudaMalloc(&f->P, (size_t)kFlFields * m * 4) != cudaSuccess || cudaMalloc(&f->flags, m) != cudaSuccess ||
        cudaMalloc(&f->G, (size_t)kFlNode * G * 4) != cudaSuccess ||
        cudaMalloc(&f->S, (size_t)kFlFields * m * 4) != cudaSuccess || cudaMalloc(&f->sflags, m) != cudaSuccess ||
        cudaMalloc(&f->keys, m * 4) != cudaSuccess || cudaMalloc(&f->ids, m * 4) != cudaSuccess ||
        cudaMalloc(&f->tkeys, m * 4) != cudaSuccess || cudaMalloc(&f->tids, m * 4) != cudaSuccess ||
        cudaMalloc(&f->hist, radix_hist_words(m) * 4) != cudaSuccess) {
        cudaGetLastError();  // the failed allocation's pending error
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
    void *ps[] = {f->G, f->S, f->sflags, f->keys, f->ids, f->tkeys, f->tids, f->hist};
    for (void *q : ps)
        if (q) cudaFree(q);
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

// `nsteps` solver steps; step k runs with steps_left = last_steps_left +
// (nsteps - 1 - k) (the freedom-radius pull weight 1 / (steps_left + 1)).
int fluid_run(FluidDev *f, uint32_t nsteps, uint64_t last_steps_left, double freedom_radius, cudaStream_t s,
              Prof *prof) {
    if (!nsteps) return AM_OK;
    const uint32_t n = f->n;
    const size_t G = (size_t)f->gsx * f->gsy;
    const unsigned gl = (unsigned)std::min<uint64_t>((n + 255) / 256, (uint64_t)kSMs * 8);
    const unsigned gp = (unsigned)((n + kFlThreads - 1) / kFlThreads);
    const unsigned gg = (unsigned)std::min<uint64_t>((G + 255) / 256, (uint64_t)kSMs * 8);
    if (n) {
        if (prof) prof->open(s);
        AMG_LAUNCH(k_fl_keys, gl, 256, 0, s, f->P, f->flags, n, f->gsx, f->gsy, f->keys, f->ids);
        const uint64_t maxkey = (uint64_t)((f->gsx + 7) / 8) * ((f->gsy + 7) / 8) * 64;
        int bits = 1;
        while ((1ull << bits) < maxkey + 1) ++bits;
        int rc = radix_sort_pairs(f->keys, f->ids, f->tkeys, f->tids, f->hist, n, bits, s);
        if (rc) return rc;
        AMG_LAUNCH(k_fl_gather, gl, 256, 0, s, f->P, f->flags, f->ids, n, f->S, f->sflags);
        if (prof) prof->close(PROF_FLUID_MANAGE, s);
    }
    FlArgs a;
    a.P = f->S; a.flags = f->sflags; a.ids = f->ids; a.G = f->G; a.n = n; a.gsx = f->gsx; a.gsy = f->gsy;
    a.freedom_radius = (float)freedom_radius;
    for (uint32_t k = 0; k < nsteps; ++k) {
        const uint64_t steps_left = last_steps_left + (nsteps - 1 - k);
        a.w_pull = (float)(1.0 / (double)(steps_left + 1));
        a.step = ++f->step;
        if (prof) prof->open(s);
        AMG_CUDA(cudaMemsetAsync(f->G, 0, (size_t)kFlNode * G * 4, s));
        if (n) {
            AMG_LAUNCH(k_fl_p2g, gp, kFlThreads, 0, s, a);
            AMG_LAUNCH(k_fl_forces, gp, kFlThreads, 0, s, a);
            AMG_LAUNCH(k_fl_div, gg, 256, 0, s, a, (int)NAX, (int)NAY);
            AMG_LAUNCH(k_fl_vel, gp, kFlThreads, 0, s, a);
            AMG_LAUNCH(k_fl_div, gg, 256, 0, s, a, (int)NU, (int)NV);
            AMG_LAUNCH(k_fl_advect, gp, kFlThreads, 0, s, a);
        }
        if (prof) prof->close(PROF_FLUID, s);
    }
    if (n) {
        if (prof) prof->open(s);
        AMG_LAUNCH(k_fl_scatter, gl, 256, 0, s, f->S, f->ids, n, f->P);
        if (prof) prof->close(PROF_FLUID_MANAGE, s);
    }
    AMG_CUDA(cudaGetLastError());
    return AM_OK;
}

int fluid_step(FluidDev *f, uint64_t steps_left, double freedom_radius, cudaStream_t s, Prof *prof) {
    return fluid_run(f, 1, steps_left, freedom_radius, s, prof);
}

}  // namespace amg
