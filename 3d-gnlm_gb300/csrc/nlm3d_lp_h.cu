// Large-patch 3D forward, FP16-storage instances (FP16 staged volume and plane boxes,
// FP32 arithmetic, Kahan-compensated pass sums).  A translation unit of its own so
// that it compiles in parallel with the FP32 instances in nlm3d_lp.cu.
#include "nlm3d_lp.cuh"

namespace gnlm {

template <int M, int N>
cudaError_t launch_lp_h(const Staging& st, const void* staged, int tz, float inv_scale, float* out,
                        float* zsum, void* acc, unsigned int* errword, cudaStream_t stream,
                        int zc0, int zc1) {
    return run_lp<M, N, __half>(st, staged, tz, inv_scale, out, zsum, acc, errword, stream, zc0,
                                zc1);
}

#define X_(m, n)                                                                                  \
    template cudaError_t launch_lp_h<m, n>(const Staging&, const void*, int, float, float*, float*, \
                                           void*, unsigned int*, cudaStream_t, int, int);
GNLM_LP3D_CASES(X_)
#undef X_

}  // namespace gnlm
