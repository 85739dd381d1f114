// Large-patch 3D forward: instances and launch (kernel in nlm3d_lp.cuh).
#include <algorithm>

#include "nlm3d_lp.cuh"
#include "nlm_internal.h"

namespace gnlm {

// out = (num_0 + num_1) / (Z_0 + Z_1) over the voxels [v0, v0 + n) of two
// accumulator buffers (the two halves of the passes), always added in that order.
__global__ void __launch_bounds__(256) lp_combine_kernel(const float2* __restrict__ acc,
                                                         size_t stride, size_t v0, size_t n,
                                                         float inv_scale, float* __restrict__ out,
                                                         float* __restrict__ zsum) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        const size_t v = v0 + i;
        const float2 h0 = acc[v], h1 = acc[stride + v];
        const float zt = h0.x + h1.x, nt = h0.y + h1.y;
        out[v] = nt / zt * inv_scale;
        if (zsum) zsum[v] = zt;
    }
}

int device_sm_count() {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
        return 1;
    return sms;
}

// Pass split of a whole volume (one CTA per SM): two half-pass CTAs per tile when
// that fills the last wave better, estimated as ceil(2n / SMs) / 2 against
// ceil(n / SMs) waves of full-pass CTAs.  Depends only on the volume, the chunk
// depth and the device, so every launch over one volume (whole or by chunk
// ranges) makes the same choice and the sums are the same bits.
int nlm3d_lp_split(int X, int Y, int Z, int tz) {
    if (tz <= 0) return 1;
    const long long n = (long long)((X + 31) / 32) * ((Y + 15) / 16) * ((Z + tz - 1) / tz);
    const long long sms = device_sm_count();
    const double one = (double)((n + sms - 1) / sms);
    const double two = (double)((2 * n + sms - 1) / sms) / 2.0;
    return two < 0.97 * one ? 2 : 1;
}

template <int M, int N>
static cudaError_t run_lp(const Staging& st, const void* staged, int tz, float inv_scale,
                          float* out, float* zsum, float2* acc, unsigned int* errword,
                          cudaStream_t stream, int zc0, int zc1) {
    using C = Lp3d<M, N>;
    CUtensorMap mapR, mapC;
    const uint64_t dims[3] = {(uint64_t)st.Xs, (uint64_t)st.Yp, (uint64_t)st.Zp};
    const uint64_t strides[2] = {(uint64_t)st.Xs * 4, (uint64_t)st.Xs * st.Yp * 4};
    const uint32_t boxR[3] = {(uint32_t)C::BWR, (uint32_t)C::HY, 1};
    const uint32_t boxC[3] = {(uint32_t)C::BWC, (uint32_t)C::HY, 1};
    void* base = const_cast<void*>(staged);
    cudaError_t e = encode_tensor_map(&mapR, false, 3, dims, strides, boxR, base);
    if (e == cudaSuccess) e = encode_tensor_map(&mapC, false, 3, dims, strides, boxC, base);
    if (e != cudaSuccess) return e;
    auto kern = nlm3d_lp_kernel<M, N>;
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM_BYTES);
    if (e != cudaSuccess) return e;
    if (zc1 < 0) zc1 = (st.Z + tz - 1) / tz;
    if (zc1 <= zc0) return cudaSuccess;
    const int nsplit = nlm3d_lp_split(st.X, st.Y, st.Z, tz);
    LpArgs a;
    a.X = st.X;
    a.Y = st.Y;
    a.Z = st.Z;
    a.TZ = tz;
    a.zc0 = zc0;
    a.nzc = zc1 - zc0;
    a.nsplit = nsplit;
    a.part_stride = (size_t)st.X * st.Y * st.Z;
    a.inv_scale = inv_scale;
    a.acc = acc;
    a.out = out;
    a.zsum = zsum;
    a.errword = errword;
    dim3 grid((st.X + C::CX - 1) / C::CX, (st.Y + C::CY - 1) / C::CY, (zc1 - zc0) * nsplit);
    kern<<<grid, C::THREADS, C::SMEM_BYTES, stream>>>(mapR, mapC, a);
    e = cudaGetLastError();
    if (e != cudaSuccess || nsplit == 1) return e;
    const size_t plane = (size_t)st.X * st.Y;
    const size_t v0 = (size_t)zc0 * tz * plane;
    const size_t v1 = (size_t)std::min(zc1 * tz, st.Z) * plane;
    const size_t blocks = std::min<size_t>((v1 - v0 + 255) / 256, (size_t)device_sm_count() * 8);
    lp_combine_kernel<<<(unsigned)blocks, 256, 0, stream>>>(acc, a.part_stride, v0, v1 - v0,
                                                            inv_scale, out, zsum);
    return cudaGetLastError();
}

// Compiled (sr, pr) instances: search radius 1..6 with patch radius 3..8 (the
// reference's NS 7..17), plus the small-patch pairs the register-brick kernel
// does not cover.
#define GNLM_LP3D_CASES(X_)                                                        \
    X_(1, 3) X_(2, 3) X_(3, 3) X_(4, 3) X_(5, 3) X_(6, 3)                          \
    X_(1, 4) X_(2, 4) X_(3, 4) X_(4, 4) X_(5, 4) X_(6, 4)                          \
    X_(1, 5) X_(2, 5) X_(3, 5) X_(4, 5) X_(5, 5) X_(6, 5)                          \
    X_(1, 6) X_(2, 6) X_(3, 6) X_(4, 6) X_(5, 6) X_(6, 6)                          \
    X_(1, 7) X_(2, 7) X_(3, 7) X_(4, 7) X_(5, 7) X_(6, 7)                          \
    X_(1, 8) X_(2, 8) X_(3, 8) X_(4, 8) X_(5, 8) X_(6, 8)                          \
    X_(6, 1) X_(1, 2) X_(2, 2) X_(4, 2) X_(6, 2)

// Chunk depth per variant (planes streamed per CTA).
static const int kLpTz[7] = {64, 32, 128, 16, 48, 96, 80};

int nlm3d_lp_tile_z(int variant) { return (variant >= 0 && variant < 7) ? kLpTz[variant] : 0; }

bool nlm3d_lp_supported(int sr, int pr) {
#define X_(m, n) \
    if (sr == m && pr == n) return true;
    GNLM_LP3D_CASES(X_)
#undef X_
    return false;
}

cudaError_t launch_nlm3d_lp(const Staging& st, const void* staged, int sr, int pr, int variant,
                            float inv_scale, float* out, float* zsum, float2* acc,
                            unsigned int* errword, cudaStream_t stream, int zc0, int zc1) {
    const int tz = nlm3d_lp_tile_z(variant);
    if (!tz) return cudaErrorInvalidValue;
#define X_(m, n)                                                                                  \
    if (sr == m && pr == n)                                                                       \
        return run_lp<m, n>(st, staged, tz, inv_scale, out, zsum, acc, errword, stream, zc0, zc1);
    GNLM_LP3D_CASES(X_)
#undef X_
    return cudaErrorNotSupported;
}

}  // namespace gnlm
