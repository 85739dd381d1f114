// 3D non-local means forward kernel for sm_103a.
//
// Work decomposition (one CTA per output tile of XO x TY x RZ voxels):
//   * The tile plus its halo (H = sr + pr voxels on each side) is loaded from
//     the staged volume into shared memory by one TMA box copy
//     (cp.async.bulk.tensor.3d) completing on an mbarrier.
//   * Warp w owns RY output rows, lane l owns output column X0 + l - pr; lanes
//     0..pr-1 and 32-pr..31 only feed the x box sum (the reference's
//     33-NS outputs per warp, 3DNLM/main.cu:30).  Each thread owns an RY x RZ
//     brick of voxels and keeps their weighted sums in registers across all
//     (2sr+1)^3 search offsets.
//   * Per offset: squared differences t^2 of (reference, candidate) values are
//     summed along z with a register sliding window (add the entering plane,
//     subtract the leaving one), along y from those row sums, and along x with
//     warp shuffles (3DNLM/main.cu:58-103 sums x by shuffles and z by planes;
//     its y cache in global memory, 3DNLM/main.cu:107,132-209, becomes
//     on-chip register reuse here).
//   * Weight w = 2^(-D') with D' = D log2(e)/(P h^2): the staging pass
//     pre-scaled the volume so D' is the sum of squares itself, and one MUFU
//     ex2 gives exp(-(D/P)/h^2) (3DNLM/main.cu:108-109).  num += w v, Z += w
//     (3DNLM/main.cu:110-111); out = num / Z (3DNLM/main.cu:125).
//
// Algorithmic work per (voxel, offset): 12 FP32 flops (diff, square, 2 box-sum
// add/sub per axis, scale, weight-sum add, weighted-value FMA) + 1 exp.
#include <cuda_fp16.h>

#include "nlm_device.cuh"
#include "nlm_internal.h"

namespace gnlm {

constexpr int cgcd(int a, int b) { return b == 0 ? a : cgcd(b, a % b); }
constexpr int cround(int v, int a) { return (v + a - 1) / a * a; }

template <int M, int N, typename T, int RY, int RZ, int NW>
struct Fwd3d {
    static constexpr int H = M + N;
    static constexpr int XO = 32 - 2 * N;             // output columns per warp
    static constexpr int A = 16 / (int)sizeof(T);      // elements per 16 bytes
    static constexpr int RMAX = A - cgcd(XO, A);       // max misalignment of X0
    static constexpr int BX = cround(32 + 2 * M + RMAX, A);
    static constexpr int TY = NW * RY;
    static constexpr int BY = TY + 2 * H;
    static constexpr int BZ = RZ + 2 * H;
    static constexpr int PLANE = BX * BY;
    static constexpr int TILE_BYTES = BX * BY * BZ * (int)sizeof(T);
    static constexpr int BAR_OFF = cround(TILE_BYTES, 128);
    static constexpr int SMEM_BYTES = BAR_OFF + 128;  // + mbarrier
    static constexpr int THREADS = 32 * NW;
    static constexpr int K = 2 * N + 1;                 // patch width
    static constexpr int ROWS = RY + 2 * N;             // rows a thread sums
    static constexpr int PLANES = RZ + 2 * N;           // planes a thread streams
    static_assert(BX <= 256 && BY <= 256 && BZ <= 256, "TMA box dimension > 256");
    static_assert(TILE_BYTES + 256 <= 227 * 1024, "tile exceeds shared memory");
};

template <int M, int N, typename T, int RY, int RZ, int NW, int MINB>
__global__ void __launch_bounds__(32 * NW, MINB)
    nlm3d_fwd_kernel(const __grid_constant__ CUtensorMap tmap, int X, int Y, int Z,
                     float inv_scale, float* __restrict__ out, float* __restrict__ zsum,
                     unsigned int* errword) {
    using C = Fwd3d<M, N, T, RY, RZ, NW>;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    T* tile = reinterpret_cast<T*>(smem_raw);
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw + C::BAR_OFF);

    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int X0 = blockIdx.x * C::XO;
    const int Y0 = blockIdx.y * C::TY;
    const int Z0 = blockIdx.z * RZ;
    const int xs = X0 & ~(C::A - 1);  // 16-byte aligned TMA start column
    const int ral = X0 - xs;

    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        mbar_arrive_expect_tx(bar, C::TILE_BYTES);
        tma_load_3d(tile, &tmap, xs, Y0, Z0, bar);
    }
    if (!mbar_wait_bounded(bar, 0)) {
        if (threadIdx.x == 0) {
            raise_device_error(errword, DEVERR_TMA_TIMEOUT);
            mbar_wait_bounded(bar, 0);  // give an in-flight copy a last chance to land
        }
        return;
    }

    // Reference values: lane's column, rows warp*RY + H - N + rr, planes H - N + pl.
    const T* aptr = tile + (C::H - N) * C::PLANE + (warp * RY + C::H - N) * C::BX + (lane + M + ral);

    float num[RY][RZ], zs[RY][RZ];
#pragma unroll
    for (int r = 0; r < RY; ++r)
#pragma unroll
        for (int q = 0; q < RZ; ++q) {
            num[r][q] = 0.f;
            zs[r][q] = 0.f;
        }

    for (int oz = -M; oz <= M; ++oz) {
        for (int oy = -M; oy <= M; ++oy) {
            for (int ox = -M; ox <= M; ++ox) {
                const T* bptr = aptr + oz * C::PLANE + oy * C::BX + ox;
                float S[C::ROWS];
                float tr[C::K][C::ROWS];
                float cand[N + 1][RY];
#pragma unroll
                for (int pl = 0; pl < C::PLANES; ++pl) {
#pragma unroll
                    for (int rr = 0; rr < C::ROWS; ++rr) {
                        const float a = to_f32(aptr[pl * C::PLANE + rr * C::BX]);
                        const float b = to_f32(bptr[pl * C::PLANE + rr * C::BX]);
                        const float t = a - b;
                        if (pl == 0)
                            S[rr] = t * t;
                        else
                            S[rr] = fmaf(t, t, S[rr]);
                        if (pl >= C::K) {
                            const float to = tr[(pl - C::K) % C::K][rr];
                            S[rr] = fmaf(-to, to, S[rr]);
                        }
                        tr[pl % C::K][rr] = t;
                        if (rr >= N && rr < RY + N) cand[pl % (N + 1)][rr - N] = b;
                    }
                    if (pl >= 2 * N) {
                        const int q = pl - 2 * N;
#pragma unroll
                        for (int r = 0; r < RY; ++r) {
                            float yv = S[r];
#pragma unroll
                            for (int k = 1; k < C::K; ++k) yv += S[r + k];
                            float xv = yv;
#pragma unroll
                            for (int k = 1; k <= N; ++k)
                                xv += __shfl_down_sync(0xffffffffu, yv, k) +
                                      __shfl_up_sync(0xffffffffu, yv, k);
                            const float w = ex2_neg(xv);
                            const float c = cand[(pl - N) % (N + 1)][r];
                            zs[r][q] += w;
                            num[r][q] = fmaf(w, c, num[r][q]);
                        }
                    }
                }
            }
        }
    }

    const int x = X0 + lane - N;
    if (lane < N || lane >= 32 - N || x >= X) return;
#pragma unroll
    for (int q = 0; q < RZ; ++q) {
        const int z = Z0 + q;
        if (z >= Z) break;
#pragma unroll
        for (int r = 0; r < RY; ++r) {
            const int y = Y0 + warp * RY + r;
            if (y >= Y) break;
            const size_t o = ((size_t)z * Y + y) * X + x;
            out[o] = num[r][q] / zs[r][q] * inv_scale;
            if (zsum) zsum[o] = zs[r][q];
        }
    }
}

template <int M, int N, typename T, int RY, int RZ, int NW, int MINB>
static cudaError_t run_fwd3d(const Staging& st, const void* staged, float inv_scale, float* out,
                             float* zsum, unsigned int* errword, cudaStream_t stream) {
    using C = Fwd3d<M, N, T, RY, RZ, NW>;
    CUtensorMap map;
    const uint64_t dims[3] = {(uint64_t)st.Xs, (uint64_t)st.Yp, (uint64_t)st.Zp};
    const uint64_t strides[2] = {(uint64_t)st.Xs * sizeof(T), (uint64_t)st.Xs * st.Yp * sizeof(T)};
    const uint32_t box[3] = {(uint32_t)C::BX, (uint32_t)C::BY, (uint32_t)C::BZ};
    cudaError_t e = encode_tensor_map(&map, sizeof(T) == 2, 3, dims, strides, box,
                                      const_cast<void*>(staged));
    if (e != cudaSuccess) return e;
    auto kern = nlm3d_fwd_kernel<M, N, T, RY, RZ, NW, MINB>;
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM_BYTES);
    if (e != cudaSuccess) return e;
    dim3 grid((st.X + C::XO - 1) / C::XO, (st.Y + C::TY - 1) / C::TY, (st.Z + RZ - 1) / RZ);
    kern<<<grid, C::THREADS, C::SMEM_BYTES, stream>>>(map, st.X, st.Y, st.Z, inv_scale, out, zsum,
                                                      errword);
    return cudaGetLastError();
}

// Compiled (sr, pr) instances.  Tile: 4 warps x 4 rows x 8 planes per CTA.
#define GNLM_FWD3D_CASES(X_)  \
    X_(1, 1) X_(2, 1) X_(3, 1) X_(4, 1) X_(5, 1) X_(3, 2) X_(5, 2)

bool nlm3d_fwd_supported(int sr, int pr, bool fp16) {
    (void)fp16;
#define X_(m, n) \
    if (sr == m && pr == n) return true;
    GNLM_FWD3D_CASES(X_)
#undef X_
    return false;
}

cudaError_t launch_nlm3d_fwd(const Staging& st, const void* staged, int sr, int pr, bool fp16,
                             float inv_scale, float* out, float* zsum, unsigned int* errword,
                             cudaStream_t stream) {
#define X_(m, n)                                                                                 \
    if (sr == m && pr == n)                                                                      \
        return fp16 ? run_fwd3d<m, n, __half, 4, 8, 4, 3>(st, staged, inv_scale, out, zsum,      \
                                                          errword, stream)                       \
                    : run_fwd3d<m, n, float, 4, 8, 4, 3>(st, staged, inv_scale, out, zsum,       \
                                                         errword, stream);
    GNLM_FWD3D_CASES(X_)
#undef X_
    return cudaErrorNotSupported;
}

}  // namespace gnlm
