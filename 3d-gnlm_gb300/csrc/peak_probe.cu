// FP32 FMA-throughput probe (measurement tool of the bench, not part of the
// NLM ABI).  Every thread runs 8 independent FFMA chains of `iters` steps, so
// the FP32 pipe, not latency, bounds it: flops = 2 * 8 * iters * threads.
// The bench times it with CUDA events to get the FP32 roofline denominator on
// the same GPU and clock as the NLM kernels.
#include <cuda_runtime.h>

__global__ void __launch_bounds__(256) fp32_fma_probe(float* out, int iters, float a, float b) {
    float x0 = threadIdx.x * 1e-3f, x1 = x0 + 1.f, x2 = x0 + 2.f, x3 = x0 + 3.f;
    float x4 = x0 + 4.f, x5 = x0 + 5.f, x6 = x0 + 6.f, x7 = x0 + 7.f;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            x0 = fmaf(x0, a, b); x1 = fmaf(x1, a, b); x2 = fmaf(x2, a, b); x3 = fmaf(x3, a, b);
            x4 = fmaf(x4, a, b); x5 = fmaf(x5, a, b); x6 = fmaf(x6, a, b); x7 = fmaf(x7, a, b);
        }
    }
    const float s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
    if (s == 123.456f) out[blockIdx.x] = s;  // keeps the chains live
}

// Same chains as packed FP32x2 FMAs (FFMA2): 16 independent lanes of work per thread.
__global__ void __launch_bounds__(256) fp32x2_fma_probe(float* out, int iters, float a, float b) {
    float2 x0 = make_float2(threadIdx.x * 1e-3f, 1.f), x1 = make_float2(2.f, 3.f);
    float2 x2 = make_float2(4.f, 5.f), x3 = make_float2(6.f, 7.f), x4 = make_float2(8.f, 9.f);
    float2 x5 = make_float2(10.f, 11.f), x6 = make_float2(12.f, 13.f), x7 = make_float2(14.f, 15.f);
    const float2 a2 = make_float2(a, a), b2 = make_float2(b, b);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            x0 = __ffma2_rn(x0, a2, b2); x1 = __ffma2_rn(x1, a2, b2);
            x2 = __ffma2_rn(x2, a2, b2); x3 = __ffma2_rn(x3, a2, b2);
            x4 = __ffma2_rn(x4, a2, b2); x5 = __ffma2_rn(x5, a2, b2);
            x6 = __ffma2_rn(x6, a2, b2); x7 = __ffma2_rn(x7, a2, b2);
        }
    }
    const float s = x0.x + x1.x + x2.x + x3.x + x4.x + x5.x + x6.x + x7.x + x0.y + x1.y + x2.y +
                    x3.y + x4.y + x5.y + x6.y + x7.y;
    if (s == 123.456f) out[blockIdx.x] = s;
}

// packed variant: 2 * 2 * 8 * 16 * iters flops per thread
extern "C" int gnlm_probe_fp32x2(float* d_out, int blocks, int iters, void* stream) {
    fp32x2_fma_probe<<<blocks, 256, 0, (cudaStream_t)stream>>>(d_out, iters, 0.9999f, 1e-4f);
    return (int)cudaGetLastError();
}

extern "C" int gnlm_probe_fp32(float* d_out, int blocks, int iters, void* stream) {
    fp32_fma_probe<<<blocks, 256, 0, (cudaStream_t)stream>>>(d_out, iters, 0.9999f, 1e-4f);
    return (int)cudaGetLastError();
}

// FMA count of one launch (each of the 16 unrolled steps issues 8 FFMAs).
extern "C" double gnlm_probe_fp32_flops(int blocks, int iters) {
    return 2.0 * 8.0 * 16.0 * (double)iters * 256.0 * (double)blocks;
}
