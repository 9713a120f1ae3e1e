// The learned swap proposal: a 10 -> 64 -> 64 -> 1 ReLU network with BF16
// weights and FP32 accumulation, run and trained on the 5th-generation tensor
// cores (tcgen05.mma, accumulators in tensor memory) from hand-written PTX.
//
// Operands live in shared memory in the canonical no-swizzle K-major layout:
// 8x16-byte core matrices, the byte offset of element (r, k) being
//   (r / 8) * SBO + (k / 8) * 128 + (r % 8) * 16 + (k % 8) * 2
// (LBO = 128 B between core matrices along K, SBO between 8-row groups).
// One elected thread issues the MMAs; tcgen05.commit arrives on an mbarrier
// every thread waits on with a bounded number of tries (a failed wait sets
// the error flag instead of spinning); each warp reads its own 32 TMEM lanes
// with tcgen05.ld.
//
// As a swap proposal the network is a gate in front of the guided candidate
// scan (k_local.cu): it scores every 32-slot region of a phase (a compact
// patch of the frame, since slots are sorted by cell) from features of the
// region's slots, and only the best-scored fraction of the regions runs the
// scan.  Its training target is log1p(G / S^2), G the sum of the best exact
// gains the full scan found in the region, S = 16 px in 1/256 px units;
// samples come from the refinement itself (am_record_swaps).
#include <cuda_bf16.h>

#include "common.cuh"
#include "kernels.h"
#include "sweep.cuh"

namespace amg {
namespace {

constexpr float kS = 4096.f;             // 16 px in 1/256 px
constexpr float kS2 = 4096.f * 4096.f;
constexpr int kTM = 128;                 // rows per MMA tile
// deployed layout offsets (floats)
constexpr int kOffW1 = 0, kOffW2 = 512, kOffB1 = 2560, kOffB2 = 2624, kOffW3 = 2688, kOffB3 = 2752;
// master layout offsets (floats)
constexpr int kMW1 = 0, kMB1 = 640, kMW2 = 704, kMB2 = 4800, kMW3 = 4864, kMB3 = 4928;

// ------------------------------------------------------------------ PTX ---
__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t make_desc(const void *base, uint32_t sbo) {
    uint32_t a = smem_u32(base);
    return (uint64_t)((a >> 4) & 0x3FFFu) | ((uint64_t)((128u >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}
// kind::f16 instruction descriptor: D f32, A/B bf16, both K-major, M x N.
__host__ __device__ constexpr uint32_t idesc_bf16(uint32_t M, uint32_t N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((N >> 3) << 17) | ((M >> 4) << 24);
}
__device__ __forceinline__ int kmaj(int r, int k, int sbo) {
    return (r >> 3) * sbo + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2;
}
__device__ __forceinline__ void put_bf16(uint8_t *base, int off, float v) {
    *reinterpret_cast<__nv_bfloat16 *>(base + off) = __float2bfloat16_rn(v);
}

__device__ __forceinline__ void tmem_alloc(uint32_t *dst, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mma(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(d),
        "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ void mbar_init(uint64_t *bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// Bounded wait: gives up after ~1M tries and flags the error.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, int *err) {
    for (uint32_t it = 0; it < (1u << 20); ++it) {
        uint32_t ok;
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            "selp.u32 %0, 1, 0, p;\n}"
            : "=r"(ok)
            : "r"(smem_u32(bar)), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    if (err) atomicExch(err, 1);
    return false;
}
// 16 consecutive fp32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// Loads W1 (B operand [64][16]) and W2 (B operand [64][64]) from the deployed
// parameters into shared memory; W2T ([i][o]) too when wanted.
__device__ void load_weights(const float *dep, uint8_t *B1, uint8_t *B2, uint8_t *B2T) {
    const __nv_bfloat16 *w1 = reinterpret_cast<const __nv_bfloat16 *>(dep + kOffW1);
    const __nv_bfloat16 *w2 = reinterpret_cast<const __nv_bfloat16 *>(dep + kOffW2);
    for (int e = threadIdx.x; e < 64 * 16; e += blockDim.x) {
        int n = e >> 4, k = e & 15;
        *reinterpret_cast<__nv_bfloat16 *>(B1 + kmaj(n, k, 256)) = w1[e];
    }
    for (int e = threadIdx.x; e < 64 * 64; e += blockDim.x) {
        int o = e >> 6, i = e & 63;
        *reinterpret_cast<__nv_bfloat16 *>(B2 + kmaj(o, i, 1024)) = w2[e];
        if (B2T) *reinterpret_cast<__nv_bfloat16 *>(B2T + kmaj(i, o, 1024)) = w2[e];
    }
}

struct FwdSmem {
    uint8_t A1[kTM * 16 * 2];   // features [128][16]
    uint8_t A2[kTM * 64 * 2];   // hidden 1 [128][64]
    uint8_t B1[64 * 16 * 2];
    uint8_t B2[64 * 64 * 2];
    float b1[64], b2[64], w3[64];
    float b3;
    uint64_t bar;
    uint32_t tmem;
};

// Forward of one 128-row tile whose features are in s.A1: returns this
// thread's score (row = threadIdx.x).  Whole CTA of 128 threads.
__device__ float forward_tile(FwdSmem &s, uint32_t &phase, int *err) {
    const int warp = threadIdx.x >> 5;
    const uint32_t lane_base = s.tmem + ((uint32_t)(32 * warp) << 16);
    fence_async_smem();
    fence_before();
    __syncthreads();
    if (threadIdx.x == 0) {
        fence_after();
        mma(s.tmem, make_desc(s.A1, 256), make_desc(s.B1, 256), idesc_bf16(128, 64), 0);
        mma_commit(&s.bar);
    }
    bool ok = mbar_wait(&s.bar, phase, err);
    phase ^= 1;
    fence_after();
    float v[16];
    const int r = threadIdx.x;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        tmem_ld16(lane_base + 16 * c, v);
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            int i = 16 * c + j;
            float h = ok ? fmaxf(v[j] + s.b1[i], 0.f) : 0.f;
            put_bf16(s.A2, kmaj(r, i, 1024), h);
        }
    }
    fence_async_smem();
    fence_before();
    __syncthreads();
    if (threadIdx.x == 0) {
        fence_after();
#pragma unroll
        for (int k = 0; k < 4; ++k)
            mma(s.tmem + 64, make_desc(s.A2 + 256 * k, 1024), make_desc(s.B2 + 256 * k, 1024), idesc_bf16(128, 64),
                k > 0);
        mma_commit(&s.bar);
    }
    ok = mbar_wait(&s.bar, phase, err) && ok;
    phase ^= 1;
    fence_after();
    float out = s.b3;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        tmem_ld16(lane_base + 64 + 16 * c, v);
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            int i = 16 * c + j;
            out += fmaxf(v[j] + s.b2[i], 0.f) * s.w3[i];
        }
    }
    fence_before();
    return ok ? out : 0.f;
}

__device__ void fwd_setup(FwdSmem &s, const float *dep) {
    load_weights(dep, s.B1, s.B2, nullptr);
    for (int i = threadIdx.x; i < 64; i += blockDim.x) {
        s.b1[i] = dep[kOffB1 + i];
        s.b2[i] = dep[kOffB2 + i];
        s.w3[i] = dep[kOffW3 + i];
    }
    if (threadIdx.x == 0) {
        s.b3 = dep[kOffB3];
        mbar_init(&s.bar);
    }
    if (threadIdx.x < 32) tmem_alloc(&s.tmem, 128);
    fence_before();
    __syncthreads();
    fence_after();
}
__device__ void fwd_teardown(FwdSmem &s) {
    fence_before();
    __syncthreads();
    fence_after();
    if (threadIdx.x < 32) tmem_dealloc(s.tmem, 128);
}

__device__ __forceinline__ void write_features(uint8_t *A1, int r, const float *f) {
#pragma unroll
    for (int k = 0; k < 16; ++k) put_bf16(A1, kmaj(r, k, 256), k < kMlpIn ? f[k] : 0.f);
}

// ------------------------------------------------------- forward kernel --
__global__ void __launch_bounds__(128) k_mlp_forward(const float *__restrict__ feat, uint64_t n,
                                                     const float *__restrict__ dep, float *out, int *err) {
    extern __shared__ __align__(1024) uint8_t smraw[];
    FwdSmem &s = *reinterpret_cast<FwdSmem *>(smraw);
    fwd_setup(s, dep);
    uint32_t phase = 0;
    for (uint64_t base = (uint64_t)blockIdx.x * kTM; base < n; base += (uint64_t)gridDim.x * kTM) {
        uint64_t row = base + threadIdx.x;
        float f[kMlpIn];
#pragma unroll
        for (int k = 0; k < kMlpIn; ++k) f[k] = row < n ? feat[row * kMlpIn + k] : 0.f;
        write_features(s.A1, threadIdx.x, f);
        float o = forward_tile(s, phase, err);
        if (row < n) out[row] = o;
    }
    fwd_teardown(s);
}

// ----------------------------------------------------- training kernel ---
// Warp sums of 64 values at once (a transposed butterfly: 62 shuffles
// instead of 320).  Lane l ends with the totals of values i and i + 1,
// i = 32 b4 + 16 b3 + 8 b2 + 4 b1 + 2 b0 (b_k the lane's bits), returned in
// v[0], v[1]; the other entries of v are clobbered.
__device__ __forceinline__ int warp_sum64(float (&v)[64], int lane) {
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        const bool up = lane & o;
        // 2 o values stay after this level
#pragma unroll
        for (int j = 0; j < 2 * o; ++j) {
            const float send = up ? v[j] : v[j + 2 * o], keep = up ? v[j + 2 * o] : v[j];
            v[j] = keep + __shfl_xor_sync(0xffffffffu, send, o);
        }
    }
    return ((lane >> 4) & 1) * 32 + ((lane >> 3) & 1) * 16 + ((lane >> 2) & 1) * 8 + ((lane >> 1) & 1) * 4 +
           (lane & 1) * 2;
}
// Adds a warp's 64 per-lane vectors into acc[64] (one shared atomic per lane
// and value pair instead of 32 same-address atomics per value).
__device__ __forceinline__ void warp_add64(float (&v)[64], float *acc) {
    const int i = warp_sum64(v, threadIdx.x & 31);
    atomicAdd(acc + i, v[0]);
    atomicAdd(acc + i + 1, v[1]);
}
__device__ __forceinline__ float warp_sum1(float v) {
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

struct TrainSmem {
    uint8_t A1[kTM * 16 * 2];        // X [b][16]
    uint8_t A2[kTM * 64 * 2];        // H1 [b][64]
    uint8_t G2[kTM * 64 * 2];        // dZ2 [b][64]
    uint8_t G2T[kTM * kTM * 2];      // dZ2^T [o pad 128][b 128]
    uint8_t H1T[64 * kTM * 2];       // H1^T [i 64][b 128]
    uint8_t G1T[kTM * kTM * 2];      // dZ1^T [o pad 128][b 128]
    uint8_t XT[16 * kTM * 2];        // X^T [i 16][b 128]
    uint8_t B1[64 * 16 * 2];
    uint8_t B2[64 * 64 * 2];
    uint8_t B2T[64 * 64 * 2];
    float b1[64], b2[64], w3[64];
    float gb1[64], gb2[64], gw3[64];
    float b3, gb3, loss;
    uint64_t bar;
    uint32_t tmem;
};

__global__ void __launch_bounds__(128) k_mlp_train(const float *__restrict__ feat, const float *__restrict__ target,
                                                   uint64_t n, const float *__restrict__ dep, float *grad,
                                                   float *loss_sum, int *err) {
    extern __shared__ __align__(1024) uint8_t smraw[];
    TrainSmem &s = *reinterpret_cast<TrainSmem *>(smraw);
    const int r = threadIdx.x, warp = r >> 5;
    load_weights(dep, s.B1, s.B2, s.B2T);
    for (int i = r; i < 64; i += 128) {
        s.b1[i] = dep[kOffB1 + i]; s.b2[i] = dep[kOffB2 + i]; s.w3[i] = dep[kOffW3 + i];
        s.gb1[i] = 0.f; s.gb2[i] = 0.f; s.gw3[i] = 0.f;
    }
    // Padding rows 64..127 of the transposed gradient operands stay zero.
    for (int e = r; e < kTM * kTM; e += 128) {
        int o = e / kTM, b = e % kTM;
        if (o >= 64) { put_bf16(s.G2T, kmaj(o, b, 2048), 0.f); put_bf16(s.G1T, kmaj(o, b, 2048), 0.f); }
    }
    if (r == 0) { s.b3 = dep[kOffB3]; s.gb3 = 0.f; s.loss = 0.f; mbar_init(&s.bar); }
    if (r < 32) tmem_alloc(&s.tmem, 256);
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t lb = s.tmem + ((uint32_t)(32 * warp) << 16);
    const uint32_t tD1 = s.tmem, tD2 = s.tmem + 64, tW2 = s.tmem + 128, tW1 = s.tmem + 192;
    uint32_t phase = 0;
    const float inv_n = 1.f / (float)n;
    int tiles = 0;
    bool ok = true;
    for (uint64_t base = (uint64_t)blockIdx.x * kTM; base < n; base += (uint64_t)gridDim.x * kTM, ++tiles) {
        uint64_t row = base + r;
        bool valid = row < n;
        float f[16];
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            float x = (valid && k < kMlpIn) ? feat[row * kMlpIn + k] : 0.f;
            f[k] = x;
            put_bf16(s.A1, kmaj(r, k, 256), x);
            put_bf16(s.XT, kmaj(k, r, 2048), x);
        }
        float tgt = valid ? target[row] : 0.f;
        // layer 1
        fence_async_smem();
        fence_before();
        __syncthreads();
        if (r == 0) {
            fence_after();
            mma(tD1, make_desc(s.A1, 256), make_desc(s.B1, 256), idesc_bf16(128, 64), 0);
            mma_commit(&s.bar);
        }
        ok = mbar_wait(&s.bar, phase, err) && ok;
        phase ^= 1;
        fence_after();
        uint32_t act1[2] = {0u, 0u};
        float v[16];
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            tmem_ld16(lb + tD1 - s.tmem + 16 * c, v);
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                int i = 16 * c + j;
                float z = v[j] + s.b1[i];
                float h = (valid && z > 0.f) ? z : 0.f;
                if (z > 0.f) act1[i >> 5] |= 1u << (i & 31);
                put_bf16(s.A2, kmaj(r, i, 1024), h);
                put_bf16(s.H1T, kmaj(i, r, 2048), h);
            }
        }
        // layer 2
        fence_async_smem();
        fence_before();
        __syncthreads();
        if (r == 0) {
            fence_after();
#pragma unroll
            for (int k = 0; k < 4; ++k)
                mma(tD2, make_desc(s.A2 + 256 * k, 1024), make_desc(s.B2 + 256 * k, 1024), idesc_bf16(128, 64), k > 0);
            mma_commit(&s.bar);
        }
        ok = mbar_wait(&s.bar, phase, err) && ok;
        phase ^= 1;
        fence_after();
        float z2[64];
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            tmem_ld16(lb + 64 + 16 * c, v);
#pragma unroll
            for (int j = 0; j < 16; ++j) z2[16 * c + j] = v[j] + s.b2[16 * c + j];
        }
        float out = s.b3;
#pragma unroll
        for (int i = 0; i < 64; ++i) out += fmaxf(z2[i], 0.f) * s.w3[i];
        float e = valid ? out - tgt : 0.f;
        float dout = 2.f * e * inv_n;
        {
            const float l = warp_sum1(e * e), d = warp_sum1(dout);
            if ((r & 31) == 0) {
                atomicAdd(&s.loss, l);
                atomicAdd(&s.gb3, d);
            }
        }
        float acc[64];
#pragma unroll
        for (int i = 0; i < 64; ++i) acc[i] = dout * fmaxf(z2[i], 0.f);
        warp_add64(acc, s.gw3);
#pragma unroll
        for (int i = 0; i < 64; ++i) {
            float g = z2[i] > 0.f ? dout * s.w3[i] : 0.f;
            acc[i] = g;
            put_bf16(s.G2, kmaj(r, i, 1024), g);
            put_bf16(s.G2T, kmaj(i, r, 2048), g);
        }
        warp_add64(acc, s.gb2);
        // dH1 = dZ2 W2  and  dW2 += dZ2^T H1
        fence_async_smem();
        fence_before();
        __syncthreads();
        if (r == 0) {
            fence_after();
#pragma unroll
            for (int k = 0; k < 4; ++k)
                mma(tD1, make_desc(s.G2 + 256 * k, 1024), make_desc(s.B2T + 256 * k, 1024), idesc_bf16(128, 64),
                    k > 0);
#pragma unroll
            for (int k = 0; k < 8; ++k)
                mma(tW2, make_desc(s.G2T + 256 * k, 2048), make_desc(s.H1T + 256 * k, 2048), idesc_bf16(128, 64),
                    (tiles > 0 || k > 0) ? 1u : 0u);
            mma_commit(&s.bar);
        }
        ok = mbar_wait(&s.bar, phase, err) && ok;
        phase ^= 1;
        fence_after();
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            tmem_ld16(lb + 16 * c, v);
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                int i = 16 * c + j;
                float g = (act1[i >> 5] >> (i & 31)) & 1u ? v[j] : 0.f;
                if (!valid) g = 0.f;
                acc[i] = g;
                put_bf16(s.G1T, kmaj(i, r, 2048), g);
            }
        }
        warp_add64(acc, s.gb1);
        // dW1 += dZ1^T X
        fence_async_smem();
        fence_before();
        __syncthreads();
        if (r == 0) {
            fence_after();
#pragma unroll
            for (int k = 0; k < 8; ++k)
                mma(tW1, make_desc(s.G1T + 256 * k, 2048), make_desc(s.XT + 256 * k, 2048), idesc_bf16(128, 16),
                    (tiles > 0 || k > 0) ? 1u : 0u);
            mma_commit(&s.bar);
        }
        ok = mbar_wait(&s.bar, phase, err) && ok;
        phase ^= 1;
        fence_after();
    }
    // Reduce the accumulated weight gradients (rows 0..63 live in warps 0-1).
    fence_before();
    __syncthreads();
    fence_after();
    ok = __all_sync(0xffffffffu, ok);
    if (tiles > 0 && warp < 2 && ok) {
        float v[16];
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            tmem_ld16(lb + 128 + 16 * c, v);
#pragma unroll
            for (int j = 0; j < 16; ++j) atomicAdd(grad + kMW2 + r * 64 + 16 * c + j, v[j]);
        }
        tmem_ld16(lb + 192, v);
#pragma unroll
        for (int j = 0; j < kMlpIn; ++j) atomicAdd(grad + kMW1 + r * kMlpIn + j, v[j]);
    }
    __syncthreads();
    if (r < 64) {
        atomicAdd(grad + kMB1 + r, s.gb1[r]);
        atomicAdd(grad + kMB2 + r, s.gb2[r]);
        atomicAdd(grad + kMW3 + r, s.gw3[r]);
    }
    if (r == 0) {
        atomicAdd(grad + kMB3, s.gb3);
        if (loss_sum) atomicAdd(loss_sum, s.loss);
    }
    fence_before();
    __syncthreads();
    fence_after();
    if (r < 32) tmem_dealloc(s.tmem, 256);
}

__global__ void k_mlp_deploy(const float *__restrict__ m, float *dep) {
    __nv_bfloat16 *w1 = reinterpret_cast<__nv_bfloat16 *>(dep + kOffW1);
    __nv_bfloat16 *w2 = reinterpret_cast<__nv_bfloat16 *>(dep + kOffW2);
    for (int e = threadIdx.x; e < 64 * 16; e += blockDim.x) {
        int o = e >> 4, i = e & 15;
        w1[e] = __float2bfloat16_rn(i < kMlpIn ? m[kMW1 + o * kMlpIn + i] : 0.f);
    }
    for (int e = threadIdx.x; e < 64 * 64; e += blockDim.x) w2[e] = __float2bfloat16_rn(m[kMW2 + e]);
    for (int i = threadIdx.x; i < 64; i += blockDim.x) {
        dep[kOffB1 + i] = m[kMB1 + i];
        dep[kOffB2 + i] = m[kMB2 + i];
        dep[kOffW3 + i] = m[kMW3 + i];
    }
    if (threadIdx.x == 0) dep[kOffB3] = m[kMB3];
}

__global__ void k_adam(float *p, const float *g, float *m, float *v, int n, float lr, float c1, float c2) {
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float gi = g[i];
        m[i] = b1 * m[i] + (1.f - b1) * gi;
        v[i] = b2 * v[i] + (1.f - b2) * gi * gi;
        p[i] -= lr * (m[i] / c1) / (sqrtf(v[i] / c2) + eps);
    }
}

// ----------------------------------------------- learned proposal gate --
// The network gates regions, not single columns: slots are sorted by 2x2-px
// cell, so 32 consecutive slots of a frame are a compact patch of the frame,
// and late in refinement the improving swaps left are concentrated in a few
// unsettled patches.  A region's features come from data the scan reads
// anyway (coalesced, one warp per region), one network row scores a region,
// and only the best-scored `keep` fraction of each 128-region tile is scanned
// (by full warps).  Features of region g (slots 32g .. 32g+31 of the phase's
// frames), S = 16 px:
//   0,1  mean and max of log1p(|a - m|^2 / S^2), a the slot's point, m its
//        column's target (p + n) / 2
//   2,3  mean and max gain bucket of the slots' last scans / 16
//   4    fraction of slots whose last scan found an improving partner
//   5,6  mean |a - m| along x and along y / S
//   7    log1p(mean column cost / S^2): how far refinement has come
//   8    fraction of slots whose target lies in their own cell
//   9    fraction of slots that can refine (chain wider than 1)
// Target: log1p(sum of the best gains the full scan found in the region / S^2).
// The seven per-slot terms summed over a region (slot 7 pads to eight).
enum { kTOk, kTLg, kTHb, kTHit, kTAx, kTAy, kTSame, kTerms = 8 };
// Raw sums of a region as staged for its owner lane: the eight sums, then
// the maxima of lg and hb (row padded to 11 floats against bank conflicts).
constexpr int kRawMaxLg = 8, kRawMaxHb = 9, kRawStride = 11;

// What the features read of one slot (lane = slot of the region).
struct SlotRaw {
    uint64_t a1, S1;  // the slot's point and its column's target sum
    uint32_t ch, h;   // the slot's chain (kNoChain: cannot refine), gain bucket of its last scan
};
// Four independent coalesced loads of slot s1 of phase frame fi.
__device__ __forceinline__ SlotRaw slot_load(const LocalArgs &a, uint32_t fi, uint32_t s1, bool in) {
    SlotRaw r{0ull, 0ull, kNoChain, 0u};
    if (in) {
        const uint64_t base = (uint64_t)a.frames[fi] * a.N + s1;
        r.ch = a.slot_ch[base];
        r.a1 = a.slot_pt[base];
        r.S1 = a.sv[base];
        r.h = a.hot[base];
    }
    return r;
}
// The slot's terms of its region's features.
__device__ __forceinline__ void slot_terms(const LocalArgs &a, const SlotRaw &r, float (&v)[kTerms]) {
#pragma unroll
    for (int k = 0; k < kTerms; ++k) v[k] = 0.f;
    if (r.ch == kNoChain) return;
    const float dx = (float)pt_X(r.a1) - 0.5f * (float)sums_x(r.S1), dy = (float)pt_Y(r.a1) - 0.5f * (float)sums_y(r.S1);
    v[kTOk] = 1.f;
    v[kTLg] = __logf(1.f + (dx * dx + dy * dy) * (1.f / kS2));
    v[kTHb] = (float)r.h * (1.f / 16.f);
    v[kTHit] = r.h ? 1.f : 0.f;
    v[kTAx] = fabsf(dx) * (1.f / kS);
    v[kTAy] = fabsf(dy) * (1.f / kS);
    const int32_t mx = sums_x(r.S1) >> 1, my = sums_y(r.S1) >> 1;
    const uint32_t own = (min((uint32_t)pt_Y(r.a1) >> 9, a.ncy - 1)) * a.ncx + min((uint32_t)pt_X(r.a1) >> 9, a.ncx - 1);
    const uint32_t tgt = (min((uint32_t)max(my, 0) >> 9, a.ncy - 1)) * a.ncx + min((uint32_t)max(mx, 0) >> 9, a.ncx - 1);
    v[kTSame] = own == tgt ? 1.f : 0.f;
}

// Warp sum of eight values at once (a transposed butterfly: 9 shuffles
// instead of 40).  Each lane ends with one total: that of value
// 4 b4 + 2 b3 + b2, b_i the lane's bits.  Every total is the same
// xor-butterfly tree a single-value reduction builds, so the sums are
// bit-identical to eight separate reductions.
__device__ __forceinline__ float warp_sum8(float (&v)[kTerms], int lane) {
    const bool u16 = lane & 16, u8 = lane & 8, u4 = lane & 4;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const float send = u16 ? v[j] : v[j + 4], keep = u16 ? v[j + 4] : v[j];
        v[j] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
    }
#pragma unroll
    for (int j = 0; j < 2; ++j) {
        const float send = u8 ? v[j] : v[j + 2], keep = u8 ? v[j + 2] : v[j];
        v[j] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
    }
    const float send = u4 ? v[0] : v[1], keep = u4 ? v[1] : v[0];
    float t = keep + __shfl_xor_sync(0xffffffffu, send, 4);
    t += __shfl_xor_sync(0xffffffffu, t, 2);
    t += __shfl_xor_sync(0xffffffffu, t, 1);
    return t;
}
// Warp maxima of two values: lanes 0-15 end with max(p), lanes 16-31 with max(q).
__device__ __forceinline__ float warp_max2(float p, float q, int lane) {
    const bool u16 = lane & 16;
    float m = fmaxf(u16 ? q : p, __shfl_xor_sync(0xffffffffu, u16 ? p : q, 16));
#pragma unroll
    for (int o = 8; o; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    return m;
}

// One CTA scores 128 regions per tile (one MMA tile): warp w reduces the
// slots of regions 32w .. 32w+31 of the tile, four regions per pass so
// their loads overlap, and stages each region's raw sums in shared memory;
// lane r then builds region 32w + r's features.  While recording, every
// eligible region is listed and its features logged.
__global__ void __launch_bounds__(128, 4) k_learned_gate(LocalArgs a) {
    extern __shared__ __align__(1024) uint8_t smraw[];
    FwdSmem &s = *reinterpret_cast<FwdSmem *>(smraw);
    __shared__ float sc[kTM];
    __shared__ float raw[kTM * kRawStride];
    fwd_setup(s, a.mlp);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint64_t total = a.N * a.nframes;
    const uint64_t ngroups = (total + 31) / 32;
    const uint64_t ntiles = (ngroups + kTM - 1) / kTM;
    const int kk = max(1, min(kTM, (int)ceilf(a.keep * (float)kTM)));
    const bool rec = a.rec_idx != nullptr;
    const uint32_t N32 = (uint32_t)a.N;  // total < 2^32 (host-checked)
    float *wraw = raw + warp * 32 * kRawStride;
    uint32_t phase = 0;
    for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        // the warp's first region: slot gw * 32 + lane, then 32 slots further
        // per region
        const uint64_t gw = tile * kTM + warp * 32;
        const uint32_t t0 = (uint32_t)(gw * 32) + lane;
        uint32_t fi = t0 / N32, s1 = t0 - fi * N32;
        // the loads of pass p + 1 are issued before pass p's reductions
        SlotRaw cur[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            cur[u] = slot_load(a, fi, s1, (gw + u) * 32 + lane < total);
            s1 += 32;
            while (s1 >= N32) { s1 -= N32; ++fi; }
        }
        for (int r0 = 0; r0 < 32; r0 += 4) {
            const uint64_t g0 = gw + r0;
            if (g0 >= ngroups) break;  // uniform across the warp
            SlotRaw nxt[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                nxt[u] = slot_load(a, fi, s1, r0 + 4 < 32 && (g0 + 4 + u) * 32 + lane < total);
                s1 += 32;
                while (s1 >= N32) { s1 -= N32; ++fi; }
            }
            float v[4][kTerms];
#pragma unroll
            for (int u = 0; u < 4; ++u) slot_terms(a, cur[u], v[u]);
#pragma unroll
            for (int u = 0; u < 4; ++u) cur[u] = nxt[u];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const float mx = warp_max2(v[u][kTLg], v[u][kTHb], lane);
                const float sum = warp_sum8(v[u], lane);
                float *row = wraw + (r0 + u) * kRawStride;
                if ((lane & 3) == 0) row[((lane >> 4) & 1) * 4 + ((lane >> 3) & 1) * 2 + ((lane >> 2) & 1)] = sum;
                if (lane == 1) row[kRawMaxLg] = mx;
                if (lane == 17) row[kRawMaxHb] = mx;
            }
        }
        __syncwarp();
        const uint64_t g = tile * kTM + threadIdx.x;
        float f[kMlpIn];
        bool elig = false;
#pragma unroll
        for (int k = 0; k < kMlpIn; ++k) f[k] = 0.f;
        if (g < ngroups) {
            const float *q = wraw + lane * kRawStride;
            const float n = q[kTOk];
            const float inv = n > 0.f ? 1.f / n : 0.f;
            f[0] = q[kTLg] * inv;
            f[1] = q[kRawMaxLg];
            f[2] = q[kTHb] * inv;
            f[3] = q[kRawMaxHb];
            f[4] = q[kTHit] * inv;
            f[5] = fminf(q[kTAx] * inv, 8.f);
            f[6] = fminf(q[kTAy] * inv, 8.f);
            f[7] = a.cost_scale;
            f[8] = q[kTSame] * inv;
            f[9] = n * (1.f / 32.f);
            elig = n > 0.f;
        }
        write_features(s.A1, threadIdx.x, f);
        float score = forward_tile(s, phase, a.err);
        bool keep;
        if (rec) {
            keep = elig;
            if (g < ngroups) {
                uint32_t j = 0xFFFFFFFFu;
                if (elig) {
                    unsigned long long r = atomicAdd(a.rec_count, 1ull);
                    if (r < a.rec_cap) {
                        j = (uint32_t)r;
#pragma unroll
                        for (int k = 0; k < kMlpIn; ++k) a.rec_feat[r * kMlpIn + k] = f[k];
                    }
                }
                a.rec_idx[g] = j;
            }
        } else {
            sc[threadIdx.x] = elig ? score : -INFINITY;
            __syncthreads();
            int rank = 0;
            const float me = sc[threadIdx.x];
            for (int j = 0; j < kTM; ++j) {
                const float o = sc[j];
                rank += (o > me) || (o == me && j < (int)threadIdx.x);
            }
            __syncthreads();
            // exploration: one region in eight is scanned whatever its score,
            // in a rotation, so a region the network ranks low is still
            // rescanned every few sweeps
            keep = elig && (rank < kk || (((uint32_t)g + a.explore) & 7u) == 0u);
        }
        unsigned m = __ballot_sync(0xffffffffu, keep);
        if (m) {
            unsigned long long base = 0;
            if (lane == 0) base = atomicAdd(a.nsel_out, (unsigned long long)__popc(m));
            base = __shfl_sync(0xffffffffu, base, 0);
            if (keep) a.sel_out[base + __popc(m & ((1u << lane) - 1u))] = (uint32_t)g;
        }
    }
    fwd_teardown(s);
}

// ----------------------------------------------- learned pair proposal --
// A score as an unsigned key whose order is the float order.
__device__ __forceinline__ uint32_t score_key(float v) {
    const uint32_t u = __float_as_uint(v);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

// Proposals: one 128-row network tile scores 32 columns x 4 candidate
// partners (row 4c + k = candidate k of column c, drawn uniformly from the
// column's chain without the column itself); each column claims its
// best-scored partner on both claim words with one 64-bit atomicMax of
// (score key, partner + 1).
__global__ void __launch_bounds__(128, 4) k_scored_propose(ScoredArgs a) {
    extern __shared__ __align__(1024) uint8_t smraw[];
    FwdSmem &s = *reinterpret_cast<FwdSmem *>(smraw);
    fwd_setup(s, a.mlp);
    uint32_t phase = 0;
    const uint64_t total = (uint64_t)a.nframes * a.N;
    const uint32_t t = threadIdx.x, cand = t & 3u;
    for (uint64_t base = (uint64_t)blockIdx.x * 32; base < total; base += (uint64_t)gridDim.x * 32) {
        const uint64_t item = base + (t >> 2);
        bool live = item < total;
        uint32_t fi = 0;
        uint64_t i = 0, j = 0;
        float f[kMlpIn];
#pragma unroll
        for (int q = 0; q < kMlpIn; ++q) f[q] = 0.f;
        if (live) {
            fi = (uint32_t)(item / a.N);
            i = item - (uint64_t)fi * a.N;
            const uint32_t c = a.C == 1 ? 0u : __ldg(a.chain_id + i);
            const uint64_t off = __ldg(a.chain_off + c), w = __ldg(a.chain_off + c + 1) - off;
            live = w >= 2;
            if (live) {
                const uint64_t h = mix64(a.key ^ mix64(item * kScoredCandidates + cand));
                const uint64_t il = i - off, jl = h % (w - 1);
                j = off + (jl >= il ? jl + 1 : jl);
                const uint32_t y = __ldg(a.frames + fi), yn = y + 1 == a.K ? 0 : y + 1, yp = y == 0 ? a.K - 1 : y - 1;
                const uint64_t *Py = a.P + (uint64_t)y * a.N, *Pp = a.P + (uint64_t)yp * a.N,
                               *Pn = a.P + (uint64_t)yn * a.N;
                const uint64_t a1 = Py[i], a2 = Py[j], p1 = Pp[i], p2 = Pp[j], n1 = Pn[i], n2 = Pn[j];
                pair_features(a1, a2, p1, n1, p2, n2, atom_colour(a.display, a.CW, a.CH, y, a1),
                              atom_colour(a.display, a.CW, a.CH, y, a2), f);
            }
        }
        write_features(s.A1, t, f);
        const float score = forward_tile(s, phase, a.err);
        uint32_t key = live ? score_key(score) : 0u;
        uint32_t part = (uint32_t)j;
#pragma unroll
        for (int o = 1; o < kScoredCandidates; o <<= 1) {
            const uint32_t k2 = __shfl_xor_sync(0xffffffffu, key, o), p2 = __shfl_xor_sync(0xffffffffu, part, o);
            if (k2 > key || (k2 == key && p2 > part)) { key = k2; part = p2; }
        }
        if (live && cand == 0 && key) {
            const uint64_t row = (uint64_t)fi * a.N;
            atomicMax(&a.claim[row + i], ((unsigned long long)key << 32) | (unsigned long long)(part + 1u));
            atomicMax(&a.claim[row + part], ((unsigned long long)key << 32) | (unsigned long long)(i + 1u));
        }
    }
    fwd_teardown(s);
}

// Mutually claimed pairs (column i's claim names j and j's names i with the
// same score) are disjoint; the lower column checks the reference's
// criterion exactly and swaps.
__global__ void __launch_bounds__(256) k_scored_apply(ScoredArgs a) {
    const uint64_t total = (uint64_t)a.nframes * a.N;
    unsigned long long gain = 0, acc = 0;
    for (uint64_t item = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; item < total;
         item += (uint64_t)gridDim.x * blockDim.x) {
        const unsigned long long c = a.claim[item];
        if (!c) continue;
        const uint32_t fi = (uint32_t)(item / a.N);
        const uint64_t i = item - (uint64_t)fi * a.N, row = (uint64_t)fi * a.N;
        const uint64_t j = (uint64_t)(uint32_t)c - 1u;
        if (j <= i) continue;
        if (a.claim[row + j] != ((c & 0xFFFFFFFF00000000ull) | (unsigned long long)(i + 1u))) continue;
        const uint32_t y = __ldg(a.frames + fi), yn = y + 1 == a.K ? 0 : y + 1, yp = y == 0 ? a.K - 1 : y - 1;
        uint64_t *Py = a.P + (uint64_t)y * a.N;
        const uint64_t *Pp = a.P + (uint64_t)yp * a.N, *Pn = a.P + (uint64_t)yn * a.N;
        const uint64_t a1 = Py[i], a2 = Py[j], p1 = Pp[i], p2 = Pp[j], n1 = Pn[i], n2 = Pn[j];
        const uint64_t c1 = pt_dist(p1, a1) + pt_dist(a1, n1) + pt_dist(p2, a2) + pt_dist(a2, n2);
        const uint64_t c2 = pt_dist(p2, a1) + pt_dist(a1, n2) + pt_dist(p1, a2) + pt_dist(a2, n1);
        if (c1 >= c2) {
            Py[i] = a2;
            Py[j] = a1;
            gain += c1 - c2;
            acc += 1;
        }
    }
    gain = warp_sum_u64(gain);
    acc = warp_sum_u64(acc);
    if ((threadIdx.x & 31) == 0) {
        if (gain) atomicAdd(a.gain, gain);
        if (acc) atomicAdd(a.accepted, acc);
    }
}

}  // namespace

static int set_smem(const void *fn, size_t bytes) {
    AMG_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    return AM_OK;
}

int mlp_deploy(const float *master, float *deployed, cudaStream_t s) {
    AMG_LAUNCH(k_mlp_deploy, 1, 256, 0, s, master, deployed);
    AMG_CUDA(cudaGetLastError());
    return AM_OK;
}

int mlp_forward(const float *feat, uint64_t n, const float *deployed, float *out, int *err, cudaStream_t s) {
    if (!n) return AM_OK;
    // 48 KB of shared memory (+1 KB the runtime reserves per CTA) lets 4 CTAs
    // share an SM's 228 KB but not 5: 4 x 128 TMEM columns at most.
    size_t smem = std::max<size_t>(sizeof(FwdSmem) + 1024, 48 * 1024);
    int rc = set_smem((const void *)k_mlp_forward, smem);
    if (rc) return rc;
    unsigned grid = (unsigned)std::min<uint64_t>((n + kTM - 1) / kTM, (uint64_t)kSMs * 4);
    AMG_LAUNCH(k_mlp_forward, grid, 128, smem, s, feat, n, deployed, out, err);
    AMG_CUDA(cudaGetLastError());
    return AM_OK;
}

int mlp_grad(const float *feat, const float *target, uint64_t n, const float *deployed, float *grad, float *loss_sum,
             int *err, cudaStream_t s) {
    AMG_CUDA(cudaMemsetAsync(grad, 0, kMlpMasterParams * sizeof(float), s));
    if (loss_sum) AMG_CUDA(cudaMemsetAsync(loss_sum, 0, sizeof(float), s));
    if (!n) return AM_OK;
    size_t smem = sizeof(TrainSmem) + 1024;
    int rc = set_smem((const void *)k_mlp_train, smem);
    if (rc) return rc;
    unsigned grid = (unsigned)std::min<uint64_t>((n + kTM - 1) / kTM, (uint64_t)kSMs);
    AMG_LAUNCH(k_mlp_train, grid, 128, smem, s, feat, target, n, deployed, grad, loss_sum, err);
    AMG_CUDA(cudaGetLastError());
    return AM_OK;
}

int mlp_train_step(const float *feat, const float *target, uint64_t n, float *master, float *deployed, float *grad,
                   float *adam_m, float *adam_v, uint64_t t, float lr, float *loss_sum, int *err, cudaStream_t s) {
    int rc = mlp_grad(feat, target, n, deployed, grad, loss_sum, err, s);
    if (rc) return rc;
    float c1 = 1.f - powf(0.9f, (float)t), c2 = 1.f - powf(0.999f, (float)t);
    AMG_LAUNCH(k_adam, (kMlpMasterParams + 255) / 256, 256, 0, s, master, grad, adam_m, adam_v, kMlpMasterParams, lr,
               c1, c2);
    return mlp_deploy(master, deployed, s);
}

int launch_learned_phase(const LocalArgs &a, cudaStream_t s) {
    uint64_t total = a.N * a.nframes;
    if (!total) return AM_OK;
    if (total >= 0xFFFFFFFFull) {
        set_error("the learned gate lists slots as 32-bit indices: too many columns in one phase");
        return AM_ERR_ARG;
    }
    AMG_CUDA(cudaMemsetAsync(a.claim, 0, total * sizeof(unsigned long long), s));
    AMG_CUDA(cudaMemsetAsync(a.nsel_out, 0, sizeof(unsigned long long), s));
    int rc;
    // 44 KB dynamic + 6.1 KB static (scores, raw sums) + 1 KB reserved per
    // CTA: 4 CTAs share an SM's 228 KB, 5 do not (4 x 128 TMEM columns at most).
    size_t smem = std::max<size_t>(sizeof(FwdSmem) + 1024, 44 * 1024);
    if ((rc = set_smem((const void *)k_learned_gate, smem))) return rc;
    const uint64_t ngroups = (total + 31) / 32;
    unsigned g = (unsigned)std::min<uint64_t>((ngroups + kTM - 1) / kTM, (uint64_t)kSMs * 4);
    AMG_LAUNCH(k_learned_gate, g, 128, smem, s, a);
    LocalArgs b = a;
    b.sel = a.sel_out;
    b.nsel = a.nsel_out;
    b.sel_groups = true;
    if ((rc = launch_local_propose(b, s))) return rc;
    return launch_local_apply(b, s);
}

int launch_scored_sweep(const ScoredArgs &a, cudaStream_t s) {
    const uint64_t total = a.N * a.nframes;
    if (!total) return AM_OK;
    if (a.N >= 0xFFFFFFFFull) {
        set_error("the learned pair proposal names partners as 32-bit columns: too many atoms");
        return AM_ERR_ARG;
    }
    AMG_CUDA(cudaMemsetAsync(a.claim, 0, total * sizeof(unsigned long long), s));
    // 48 KB per CTA keeps 4 CTAs on an SM: 4 x 128 TMEM columns at most
    const size_t smem = std::max<size_t>(sizeof(FwdSmem) + 1024, 48 * 1024);
    int rc = set_smem((const void *)k_scored_propose, smem);
    if (rc) return rc;
    unsigned g = (unsigned)std::min<uint64_t>((total + 31) / 32, (uint64_t)kSMs * 4);
    AMG_LAUNCH(k_scored_propose, g, 128, smem, s, a);
    g = (unsigned)std::min<uint64_t>((total + 255) / 256, (uint64_t)kSMs * 8);
    AMG_LAUNCH(k_scored_apply, g, 256, 0, s, a);
    AMG_CUDA(cudaGetLastError());
    return AM_OK;
}

}  // namespace amg
