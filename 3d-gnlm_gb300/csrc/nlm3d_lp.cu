// Large-patch 3D forward: instances and launch (kernel in nlm3d_lp.cuh).
#include "nlm3d_lp.cuh"
#include "nlm_internal.h"

namespace gnlm {

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
    LpArgs a;
    a.X = st.X;
    a.Y = st.Y;
    a.Z = st.Z;
    a.TZ = tz;
    a.zc0 = zc0;
    a.inv_scale = inv_scale;
    a.acc = acc;
    a.out = out;
    a.zsum = zsum;
    a.errword = errword;
    dim3 grid((st.X + C::CX - 1) / C::CX, (st.Y + C::CY - 1) / C::CY, zc1 - zc0);
    kern<<<grid, C::THREADS, C::SMEM_BYTES, stream>>>(mapR, mapC, a);
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
