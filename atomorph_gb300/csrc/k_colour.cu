// Key-frame colour ingestion: RGB -> HSP on store, HSP -> RGB on read.
//
// Restates color.cpp:64-211 (RGBtoHSP / HSPtoRGB, Darel Rex Finley's public
// domain HSP model) in FP64.  This file is compiled with -fmad=false so every
// multiply and add rounds separately, exactly as the reference's x86 build
// does; CUDA's double division and square root are IEEE round-to-nearest, so
// the stored and displayed bytes are bit-identical to the reference's.
#include "common.cuh"
#include "kernels.h"

namespace amg {
namespace {

constexpr double kPr = 0.299, kPg = 0.587, kPb = 0.114;

__host__ __device__ void rgb2hsp(double R, double G, double B, double *H, double *S, double *P) {
    *P = sqrt(R * R * kPr + G * G * kPg + B * B * kPb);
    if (R == G && R == B) { *H = 0.; *S = 0.; return; }
    if (R >= G && R >= B) {
        if (B >= G) { *H = 6. / 6. - 1. / 6. * (B - G) / (R - G); *S = 1. - G / R; }
        else        { *H = 0. / 6. + 1. / 6. * (G - B) / (R - B); *S = 1. - B / R; }
    } else if (G >= R && G >= B) {
        if (R >= B) { *H = 2. / 6. - 1. / 6. * (R - B) / (G - B); *S = 1. - B / G; }
        else        { *H = 2. / 6. + 1. / 6. * (B - R) / (G - R); *S = 1. - R / G; }
    } else {
        if (G >= R) { *H = 4. / 6. - 1. / 6. * (G - R) / (B - R); *S = 1. - R / B; }
        else        { *H = 4. / 6. + 1. / 6. * (R - G) / (B - G); *S = 1. - G / B; }
    }
}

__host__ __device__ void hsp2rgb(double H, double S, double P, double *R, double *G, double *B) {
    double part, mom = 1. - S;
    if (mom > 0.) {
        if (H < 1. / 6.) {
            H = 6. * (H - 0. / 6.); part = 1. + H * (1. / mom - 1.);
            *B = P / sqrt(kPr / mom / mom + kPg * part * part + kPb); *R = (*B) / mom; *G = (*B) + H * ((*R) - (*B));
        } else if (H < 2. / 6.) {
            H = 6. * (-H + 2. / 6.); part = 1. + H * (1. / mom - 1.);
            *B = P / sqrt(kPg / mom / mom + kPr * part * part + kPb); *G = (*B) / mom; *R = (*B) + H * ((*G) - (*B));
        } else if (H < 3. / 6.) {
            H = 6. * (H - 2. / 6.); part = 1. + H * (1. / mom - 1.);
            *R = P / sqrt(kPg / mom / mom + kPb * part * part + kPr); *G = (*R) / mom; *B = (*R) + H * ((*G) - (*R));
        } else if (H < 4. / 6.) {
            H = 6. * (-H + 4. / 6.); part = 1. + H * (1. / mom - 1.);
            *R = P / sqrt(kPb / mom / mom + kPg * part * part + kPr); *B = (*R) / mom; *G = (*R) + H * ((*B) - (*R));
        } else if (H < 5. / 6.) {
            H = 6. * (H - 4. / 6.); part = 1. + H * (1. / mom - 1.);
            *G = P / sqrt(kPb / mom / mom + kPr * part * part + kPg); *B = (*G) / mom; *R = (*G) + H * ((*B) - (*G));
        } else {
            H = 6. * (-H + 6. / 6.); part = 1. + H * (1. / mom - 1.);
            *G = P / sqrt(kPr / mom / mom + kPb * part * part + kPg); *R = (*G) / mom; *B = (*G) + H * ((*R) - (*G));
        }
    } else {
        if (H < 1. / 6.)      { H = 6. * (H - 0. / 6.);  *R = sqrt(P * P / (kPr + kPg * H * H)); *G = (*R) * H; *B = 0.; }
        else if (H < 2. / 6.) { H = 6. * (-H + 2. / 6.); *G = sqrt(P * P / (kPg + kPr * H * H)); *R = (*G) * H; *B = 0.; }
        else if (H < 3. / 6.) { H = 6. * (H - 2. / 6.);  *G = sqrt(P * P / (kPg + kPb * H * H)); *B = (*G) * H; *R = 0.; }
        else if (H < 4. / 6.) { H = 6. * (-H + 4. / 6.); *B = sqrt(P * P / (kPb + kPg * H * H)); *G = (*B) * H; *R = 0.; }
        else if (H < 5. / 6.) { H = 6. * (H - 4. / 6.);  *B = sqrt(P * P / (kPb + kPr * H * H)); *R = (*B) * H; *G = 0.; }
        else                  { H = 6. * (-H + 6. / 6.); *R = sqrt(P * P / (kPr + kPb * H * H)); *B = (*R) * H; *G = 0.; }
    }
}

// Round-half-away-from-zero of a non-negative double to a byte, as
// std::round followed by the implicit conversion to uint8_t.
__host__ __device__ __forceinline__ uint32_t rbyte(double v) { return (uint32_t)(int)round(v) & 0xFFu; }

__host__ __device__ uint32_t to_hsp(uint32_t c) {
    double h, s, p;
    rgb2hsp((c & 0xFF) / 255.0, ((c >> 8) & 0xFF) / 255.0, ((c >> 16) & 0xFF) / 255.0, &h, &s, &p);
    return rbyte(h * 255.0) | (rbyte(s * 255.0) << 8) | (rbyte(p * 255.0) << 16) | (c & 0xFF000000u);
}
__host__ __device__ uint32_t to_rgb(uint32_t c) {
    double r, g, b;
    hsp2rgb((c & 0xFF) / 255.0, ((c >> 8) & 0xFF) / 255.0, ((c >> 16) & 0xFF) / 255.0, &r, &g, &b);
    return rbyte(fmin(round(r * 255.0), 255.0)) | (rbyte(fmin(round(g * 255.0), 255.0)) << 8) |
           (rbyte(fmin(round(b * 255.0), 255.0)) << 16) | (c & 0xFF000000u);
}

// present[i]: 0 absent, 1 stored as given, 2 stored after RGB->HSP
// (the delimiter in force when the pixel was added, morph.cpp:299-301).
__global__ void k_colour(const uint32_t *__restrict__ raw, const uint8_t *__restrict__ present,
                         uint32_t *__restrict__ stored, uint32_t *__restrict__ display, size_t n,
                         int display_hsp) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        uint8_t p = present[i];
        if (!p) { stored[i] = 0; display[i] = 0; continue; }
        uint32_t s = p == 2 ? to_hsp(raw[i]) : raw[i];
        stored[i] = s;
        display[i] = display_hsp ? to_rgb(s) : s;
    }
}

__global__ void k_hsp_probe(const uint32_t *in, uint32_t *out, size_t n, int dir) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i < n) out[i] = dir == 0 ? to_hsp(in[i]) : to_rgb(in[i]);
}

}  // namespace

uint32_t hsp_to_rgb_host(uint32_t c) { return to_rgb(c); }

int launch_colour(const uint32_t *raw, const uint8_t *present, uint32_t *stored, uint32_t *display, size_t n,
                  int display_hsp, cudaStream_t s) {
    if (n == 0) return AM_OK;
    unsigned grid = (unsigned)std::min<size_t>((n + 255) / 256, (size_t)kSMs * 16);
    AMG_LAUNCH(k_colour, grid, 256, 0, s, raw, present, stored, display, n, display_hsp);
    AMG_CUDA(cudaGetLastError());
    return AM_OK;
}

int launch_hsp_probe(const uint32_t *in, uint32_t *out, size_t n, int dir, cudaStream_t s) {
    if (n == 0) return AM_OK;
    AMG_LAUNCH(k_hsp_probe, (unsigned)((n + 255) / 256), 256, 0, s, in, out, n, dir);
    AMG_CUDA(cudaGetLastError());
    return AM_OK;
}

}  // namespace amg
