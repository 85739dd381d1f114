// 2D non-local means forward kernel for sm_103a.
//
// Same decomposition as the 3D kernel without z: a CTA loads its tile + halo
// (H = sr + pr) by one TMA 2D box; warp w owns RY output rows, lane l owns
// column X0 + l - pr (32 - 2pr outputs per warp, as the reference's
// 33-nb_size, 2D NLM/11x11/main.cu:389).  Per search offset: squared
// differences, y box sum by a register sliding window over the thread's rows
// (the reference slides y through a global cache, 2D NLM/11x11/main.cu:428-466),
// x box sum by warp shuffles (2D NLM/11x11/main.cu:405-410), weight
// 2^(-D') on the MUFU pipe, and register accumulation.  Unlike the reference,
// whose y slide hard-codes an 11-wide patch (2D NLM/11x11/main.cu:446), any
// compiled (sr, pr) is exact.
//
// Algorithmic work per (pixel, offset): 10 FP32 flops (diff, square, 2 box-sum
// add/sub per axis, scale, weight-sum add, weighted-value FMA) + 1 exp.
#include <cuda_fp16.h>

#include "nlm_device.cuh"
#include "nlm_internal.h"

namespace gnlm {

constexpr int cgcd2(int a, int b) { return b == 0 ? a : cgcd2(b, a % b); }
constexpr int cround2(int v, int a) { return (v + a - 1) / a * a; }

template <int M, int N, typename T, int RY, int NW>
struct Fwd2d {
    static constexpr int H = M + N;
    static constexpr int XO = 32 - 2 * N;
    static constexpr int A = 16 / (int)sizeof(T);
    static constexpr int RMAX = A - cgcd2(XO, A);
    static constexpr int BX = cround2(32 + 2 * M + RMAX, A);
    static constexpr int TY = NW * RY;
    static constexpr int BY = TY + 2 * H;
    static constexpr int TILE_BYTES = BX * BY * (int)sizeof(T);
    static constexpr int BAR_OFF = cround2(TILE_BYTES, 128);
    static constexpr int SMEM_BYTES = BAR_OFF + 128;
    static constexpr int K = 2 * N + 1;
    static constexpr int ROWS = RY + 2 * N;
    static_assert(BX <= 256 && BY <= 256, "TMA box dimension > 256");
    static_assert(BAR_OFF % 128 == 0, "the tile (at offset 0) and barrier stay 128-byte aligned");
};

template <int M, int N, typename T, int RY, int NW, int MINB>
__global__ void __launch_bounds__(32 * NW, MINB)
    nlm2d_fwd_kernel(const __grid_constant__ CUtensorMap tmap, int X, int Y, float inv_scale,
                     float* __restrict__ out, float* __restrict__ zsum, unsigned int* errword) {
    using C = Fwd2d<M, N, T, RY, NW>;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    T* tile = reinterpret_cast<T*>(smem_raw);
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw + C::BAR_OFF);

    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int X0 = blockIdx.x * C::XO;
    const int Y0 = blockIdx.y * C::TY;
    const int xs = X0 & ~(C::A - 1);
    const int ral = X0 - xs;

    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        mbar_arrive_expect_tx(bar, C::TILE_BYTES);
        tma_load_2d(tile, &tmap, xs, Y0, bar);
    }
    if (!mbar_wait_bounded(bar, 0)) {
        if (threadIdx.x == 0) {
            raise_device_error(errword, DEVERR_TMA_TIMEOUT);
            mbar_wait_bounded(bar, 0);
        }
        return;
    }

    const T* aptr = tile + (warp * RY + C::H - N) * C::BX + (lane + M + ral);
    float num[RY], zs[RY];
#pragma unroll
    for (int r = 0; r < RY; ++r) {
        num[r] = 0.f;
        zs[r] = 0.f;
    }

    for (int oy = -M; oy <= M; ++oy) {
        for (int ox = -M; ox <= M; ++ox) {
            const T* bptr = aptr + oy * C::BX + ox;
            float q[C::ROWS], cand[RY];
#pragma unroll
            for (int rr = 0; rr < C::ROWS; ++rr) {
                const float a = to_f32(aptr[rr * C::BX]);
                const float b = to_f32(bptr[rr * C::BX]);
                const float t = a - b;
                q[rr] = t * t;
                if (rr >= N && rr < RY + N) cand[rr - N] = b;
            }
            float yv = 0.f;
#pragma unroll
            for (int k = 0; k < C::K; ++k) yv += q[k];
#pragma unroll
            for (int r = 0; r < RY; ++r) {
                if (r > 0) yv = yv + q[r + 2 * N] - q[r - 1];
                float xv = yv;
#pragma unroll
                for (int k = 1; k <= N; ++k)
                    xv += __shfl_down_sync(0xffffffffu, yv, k) + __shfl_up_sync(0xffffffffu, yv, k);
                const float w = ex2_neg(xv);
                zs[r] += w;
                num[r] = fmaf(w, cand[r], num[r]);
            }
        }
    }

    const int x = X0 + lane - N;
    if (lane < N || lane >= 32 - N || x >= X) return;
#pragma unroll
    for (int r = 0; r < RY; ++r) {
        const int y = Y0 + warp * RY + r;
        if (y >= Y) break;
        const size_t o = (size_t)y * X + x;
        out[o] = num[r] / zs[r] * inv_scale;
        if (zsum) zsum[o] = zs[r];
    }
}

template <int M, int N, typename T, int RY, int NW, int MINB>
static cudaError_t run_fwd2d(const Staging& st, const void* staged, float inv_scale, float* out,
                             float* zsum, unsigned int* errword, cudaStream_t stream) {
    using C = Fwd2d<M, N, T, RY, NW>;
    CUtensorMap map;
    const uint64_t dims[2] = {(uint64_t)st.Xs, (uint64_t)st.Yp};
    const uint64_t strides[1] = {(uint64_t)st.Xs * sizeof(T)};
    const uint32_t box[2] = {(uint32_t)C::BX, (uint32_t)C::BY};
    cudaError_t e = encode_tensor_map(&map, sizeof(T) == 2, 2, dims, strides, box,
                                      const_cast<void*>(staged));
    if (e != cudaSuccess) return e;
    auto kern = nlm2d_fwd_kernel<M, N, T, RY, NW, MINB>;
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM_BYTES);
    if (e != cudaSuccess) return e;
    dim3 grid((st.X + C::XO - 1) / C::XO, (st.Y + C::TY - 1) / C::TY);
    kern<<<grid, 32 * NW, C::SMEM_BYTES, stream>>>(map, st.X, st.Y, inv_scale, out, zsum, errword);
    return cudaGetLastError();
}

// Compiled (sr, pr) instances.  (5, 2) is the 11x11-search / 5x5-patch
// workload; (3, 5) and (7, 5) are the reference's 11x11-patch kernels' own
// configuration family.
#define GNLM_FWD2D_CASES(X_) \
    X_(1, 1) X_(3, 1) X_(5, 1) X_(3, 2) X_(5, 2) X_(7, 2) X_(3, 5) X_(7, 5) X_(10, 5)

bool nlm2d_fwd_supported(int sr, int pr, bool fp16) {
    (void)fp16;
#define X_(m, n) \
    if (sr == m && pr == n) return true;
    GNLM_FWD2D_CASES(X_)
#undef X_
    return false;
}

cudaError_t launch_nlm2d_fwd(const Staging& st, const void* staged, int sr, int pr, bool fp16,
                             float inv_scale, float* out, float* zsum, unsigned int* errword,
                             cudaStream_t stream) {
#define X_(m, n)                                                                            \
    if (sr == m && pr == n)                                                                 \
        return fp16 ? run_fwd2d<m, n, __half, 16, 4, 4>(st, staged, inv_scale, out, zsum,   \
                                                        errword, stream)                    \
                    : run_fwd2d<m, n, float, 16, 4, 4>(st, staged, inv_scale, out, zsum,    \
                                                       errword, stream);
    GNLM_FWD2D_CASES(X_)
#undef X_
    return cudaErrorNotSupported;
}

}  // namespace gnlm
