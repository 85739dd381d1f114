// Large-patch 3D forward: FP32 instances and the launch dispatch (kernel and
// launcher template in nlm3d_lp.cuh; the FP16-storage instances in nlm3d_lp_h.cu).
#include "nlm3d_lp.cuh"

namespace gnlm {

int device_sm_count() {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
        return 1;
    return sms;
}

// Pass split of a whole volume: two half-pass CTAs per tile (per x part) when that fills
// the last wave better, estimated as ceil(2n / slots) / 2 against ceil(n / slots) waves
// for n = tiles x chunks x x-parts full-pass CTAs and slots = SMs x CTAs per SM.
// Depends only on the volume, the chunk depth, the tile geometry and the device, so
// every launch over one volume (whole or by chunk ranges) makes the same choice and the
// sums are the same bits.
int nlm3d_lp_split(int X, int Y, int Z, int tz, int tile_x, int tile_y, int xparts,
                   int ctas_per_sm) {
    if (tz <= 0) return 1;
    const long long n = (long long)((X + tile_x - 1) / tile_x) * ((Y + tile_y - 1) / tile_y) *
                        ((Z + tz - 1) / tz) * xparts;
    const long long slots = (long long)device_sm_count() * ctas_per_sm;
    const double one = (double)((n + slots - 1) / slots);
    const double two = (double)((2 * n + slots - 1) / slots) / 2.0;
    return two < 0.97 * one ? 2 : 1;
}

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

cudaError_t launch_nlm3d_lp(const Staging& st, const void* staged, int sr, int pr, bool fp16,
                            int variant, float inv_scale, float* out, float* zsum, void* acc,
                            unsigned int* errword, cudaStream_t stream, int zc0, int zc1) {
    const int tz = nlm3d_lp_tile_z(variant);
    if (!tz) return cudaErrorInvalidValue;
#define X_(m, n)                                                                              \
    if (sr == m && pr == n)                                                                   \
        return fp16 ? launch_lp_h<m, n>(st, staged, tz, inv_scale, out, zsum, acc, errword,   \
                                        stream, zc0, zc1)                                     \
                    : run_lp<m, n, float>(st, staged, tz, inv_scale, out, zsum, acc, errword, \
                                          stream, zc0, zc1);
    GNLM_LP3D_CASES(X_)
#undef X_
    return cudaErrorNotSupported;
}

}  // namespace gnlm
