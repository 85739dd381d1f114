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

extern "C" int gnlm_probe_fp32(float* d_out, int blocks, int iters, void* stream) {
    fp32_fma_probe<<<blocks, 256, 0, (cudaStream_t)stream>>>(d_out, iters, 0.9999f, 1e-4f);
    return (int)cudaGetLastError();
}

// FMA count of one launch (each of the 16 unrolled steps issues 8 FFMAs).
extern "C" double gnlm_probe_fp32_flops(int blocks, int iters) {
    return 2.0 * 8.0 * 16.0 * (double)iters * 256.0 * (double)blocks;
}
