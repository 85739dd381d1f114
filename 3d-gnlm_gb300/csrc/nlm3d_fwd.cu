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
    static_assert(BAR_OFF % 128 == 0, "the tile (at offset 0) and barrier stay 128-byte aligned");
    static_assert(TILE_BYTES + 256 <= 227 * 1024, "tile exceeds shared memory");
};

// Compensated (Kahan) accumulation of a packed pair of running sums.
struct Kahan2 {
    float2 s, c;
};
__device__ __forceinline__ void kahan_add(Kahan2& k, float2 v) {
    const float2 y = __fadd2_rn(v, make_float2(-k.c.x, -k.c.y));
    const float2 t = __fadd2_rn(k.s, y);
    k.c = __fadd2_rn(__fadd2_rn(t, make_float2(-k.s.x, -k.s.y)), make_float2(-y.x, -y.y));
    k.s = t;
}

// AREG: the thread's reference values (its column, ROWS rows, PLANES planes) are
// loaded into registers once; they are the same for every search offset.
// KAHAN: Z and num are Kahan-compensated (precision form).
// Rows are processed in pairs so that everything after the first difference runs
// as packed FP32x2 arithmetic (FFMA2/FADD2): one issue slot per two operations.
template <int M, int N, typename T, int RY, int RZ, int NW, int MINB, bool AREG, bool KAHAN>
__global__ void __launch_bounds__(32 * NW, MINB)
    nlm3d_fwd_kernel(const __grid_constant__ CUtensorMap tmap, int X, int Y, int Z,
                     float inv_scale, float* __restrict__ out, float* __restrict__ zsum,
                     unsigned int* errword) {
    using C = Fwd3d<M, N, T, RY, RZ, NW>;
    static_assert(RY % 2 == 0, "rows are processed in pairs");
    constexpr int RP = C::ROWS / 2;  // row pairs a thread sums
    constexpr int OP = RY / 2;       // output row pairs
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

    float2 areg[AREG ? C::PLANES : 1][AREG ? RP : 1];
    if constexpr (AREG) {
#pragma unroll
        for (int pl = 0; pl < C::PLANES; ++pl)
#pragma unroll
            for (int rp = 0; rp < RP; ++rp)
                areg[pl][rp] = make_float2(to_f32(aptr[pl * C::PLANE + (2 * rp) * C::BX]),
                                           to_f32(aptr[pl * C::PLANE + (2 * rp + 1) * C::BX]));
    }

    // Accumulators for output row pairs (r, r+1) and planes q.
    Kahan2 zacc[OP][RZ], nacc[OP][RZ];
#pragma unroll
    for (int r = 0; r < OP; ++r)
#pragma unroll
        for (int q = 0; q < RZ; ++q) {
            zacc[r][q].s = nacc[r][q].s = make_float2(0.f, 0.f);
            zacc[r][q].c = nacc[r][q].c = make_float2(0.f, 0.f);
        }
    const float2 minus1 = make_float2(-1.f, -1.f);

    for (int oz = -M; oz <= M; ++oz) {
        for (int oy = -M; oy <= M; ++oy) {
            for (int ox = -M; ox <= M; ++ox) {
                const T* bptr = aptr + oz * C::PLANE + oy * C::BX + ox;
                float2 S[RP];          // z-window sums of t^2, row pairs
                float2 tr[C::K][RP];   // ring of the last K planes of t, row pairs
                float cand[N + 1][RY]; // candidate centre values of the last N+1 planes
#pragma unroll
                for (int pl = 0; pl < C::PLANES; ++pl) {
#pragma unroll
                    for (int rp = 0; rp < RP; ++rp) {
                        const float b0 = to_f32(bptr[pl * C::PLANE + (2 * rp) * C::BX]);
                        const float b1 = to_f32(bptr[pl * C::PLANE + (2 * rp + 1) * C::BX]);
                        float2 a2;
                        if constexpr (AREG)
                            a2 = areg[pl][rp];
                        else
                            a2 = make_float2(to_f32(aptr[pl * C::PLANE + (2 * rp) * C::BX]),
                                             to_f32(aptr[pl * C::PLANE + (2 * rp + 1) * C::BX]));
                        const float2 t = __ffma2_rn(make_float2(b0, b1), minus1, a2);  // a - b
                        if (pl == 0)
                            S[rp] = __fmul2_rn(t, t);
                        else
                            S[rp] = __ffma2_rn(t, t, S[rp]);
                        if (pl >= C::K) {
                            const float2 to = tr[(pl - C::K) % C::K][rp];
                            S[rp] = __ffma2_rn(make_float2(-to.x, -to.y), to, S[rp]);
                        }
                        tr[pl % C::K][rp] = t;
                        const int r0 = 2 * rp, r1 = 2 * rp + 1;
                        if (r0 >= N && r0 < RY + N) cand[pl % (N + 1)][r0 - N] = b0;
                        if (r1 >= N && r1 < RY + N) cand[pl % (N + 1)][r1 - N] = b1;
                    }
                    if (pl >= 2 * N) {
                        const int q = pl - 2 * N;
                        // y box over rows: Yv[r] = sum_{k<K} Srow[r+k]
                        float Srow[C::ROWS];
#pragma unroll
                        for (int rp = 0; rp < RP; ++rp) {
                            Srow[2 * rp] = S[rp].x;
                            Srow[2 * rp + 1] = S[rp].y;
                        }
                        float Yv[RY];
                        if constexpr (N == 1) {
#pragma unroll
                            for (int r = 0; r < RY; r += 2) {  // 3 adds per 2 outputs
                                const float u = Srow[r + 1] + Srow[r + 2];
                                Yv[r] = Srow[r] + u;
                                Yv[r + 1] = u + Srow[r + 3];
                            }
                        } else {
                            float acc = 0.f;
#pragma unroll
                            for (int k = 0; k < C::K; ++k) acc += Srow[k];
                            Yv[0] = acc;
#pragma unroll
                            for (int r = 1; r < RY; ++r) {
                                acc = acc + Srow[r + C::K - 1] - Srow[r - 1];
                                Yv[r] = acc;
                            }
                        }
#pragma unroll
                        for (int op = 0; op < OP; ++op) {
                            float2 xv = make_float2(Yv[2 * op], Yv[2 * op + 1]);
#pragma unroll
                            for (int k = 1; k <= N; ++k) {
                                const float2 dn =
                                    make_float2(__shfl_down_sync(0xffffffffu, Yv[2 * op], k),
                                                __shfl_down_sync(0xffffffffu, Yv[2 * op + 1], k));
                                const float2 up =
                                    make_float2(__shfl_up_sync(0xffffffffu, Yv[2 * op], k),
                                                __shfl_up_sync(0xffffffffu, Yv[2 * op + 1], k));
                                xv = __fadd2_rn(xv, __fadd2_rn(dn, up));
                            }
                            const float2 w = make_float2(ex2_neg(xv.x), ex2_neg(xv.y));
                            const float2 c = make_float2(cand[(pl - N) % (N + 1)][2 * op],
                                                         cand[(pl - N) % (N + 1)][2 * op + 1]);
                            if constexpr (KAHAN) {
                                kahan_add(zacc[op][q], w);
                                kahan_add(nacc[op][q], __fmul2_rn(w, c));
                            } else {
                                zacc[op][q].s = __fadd2_rn(zacc[op][q].s, w);
                                nacc[op][q].s = __ffma2_rn(w, c, nacc[op][q].s);
                            }
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
            const float2 zz = zacc[r / 2][q].s, nn = nacc[r / 2][q].s;
            const float zs = (r & 1) ? zz.y : zz.x;
            const float nm = (r & 1) ? nn.y : nn.x;
            out[o] = nm / zs * inv_scale;
            if (zsum) zsum[o] = zs;
        }
    }
}

template <int M, int N, typename T, int RY, int RZ, int NW, int MINB, bool AREG, bool KAHAN>
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
    auto kern = nlm3d_fwd_kernel<M, N, T, RY, RZ, NW, MINB, AREG, KAHAN>;
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM_BYTES);
    if (e != cudaSuccess) return e;
    dim3 grid((st.X + C::XO - 1) / C::XO, (st.Y + C::TY - 1) / C::TY, (st.Z + RZ - 1) / RZ);
    kern<<<grid, C::THREADS, C::SMEM_BYTES, stream>>>(map, st.X, st.Y, st.Z, inv_scale, out, zsum,
                                                      errword);
    return cudaGetLastError();
}

// Compiled (sr, pr) instances.
#define GNLM_FWD3D_CASES(X_)  \
    X_(1, 1) X_(2, 1) X_(3, 1) X_(4, 1) X_(5, 1) X_(3, 2) X_(5, 2)

// Tile-shape variants (the autotuner's search space).  FP32 form:
//   0: 4 rows x 8 planes per thread, reference values in registers, 2 CTAs/SM
//   1: 4 x 8, reference values re-read from shared memory, 3 CTAs/SM
//   2: 4 x 4, registers, 3 CTAs/SM
//   3: 2 x 8, registers, 3 CTAs/SM
// FP16-storage form (Kahan-compensated sums):
//   0: 4 x 4, registers, 3 CTAs/SM;  1: 4 x 8, shared memory, 2 CTAs/SM;  2: 2 x 8, registers
template <int m, int n>
static cudaError_t run_variant(const Staging& st, const void* staged, bool fp16, int v,
                               float inv_scale, float* out, float* zsum, unsigned int* ew,
                               cudaStream_t s) {
    if (!fp16) {
        switch (v) {
            case 0: return run_fwd3d<m, n, float, 4, 8, 4, 2, true, false>(st, staged, inv_scale, out, zsum, ew, s);
            case 1: return run_fwd3d<m, n, float, 4, 8, 4, 3, false, false>(st, staged, inv_scale, out, zsum, ew, s);
            case 2: return run_fwd3d<m, n, float, 4, 4, 4, 3, true, false>(st, staged, inv_scale, out, zsum, ew, s);
            case 3: return run_fwd3d<m, n, float, 2, 8, 4, 3, true, false>(st, staged, inv_scale, out, zsum, ew, s);
        }
    } else {
        switch (v) {
            case 0: return run_fwd3d<m, n, __half, 4, 4, 4, 3, true, true>(st, staged, inv_scale, out, zsum, ew, s);
            case 1: return run_fwd3d<m, n, __half, 4, 8, 4, 2, false, true>(st, staged, inv_scale, out, zsum, ew, s);
            case 2: return run_fwd3d<m, n, __half, 2, 8, 4, 3, true, true>(st, staged, inv_scale, out, zsum, ew, s);
        }
    }
    return cudaErrorInvalidValue;
}

int nlm3d_fwd_variant_count(bool fp16) { return fp16 ? 3 : 4; }

bool nlm3d_fwd_supported(int sr, int pr, bool fp16) {
    (void)fp16;
#define X_(m, n) \
    if (sr == m && pr == n) return true;
    GNLM_FWD3D_CASES(X_)
#undef X_
    return false;
}

cudaError_t launch_nlm3d_fwd(const Staging& st, const void* staged, int sr, int pr, bool fp16,
                             int variant, float inv_scale, float* out, float* zsum,
                             unsigned int* errword, cudaStream_t stream) {
    if (variant < 0 || variant >= nlm3d_fwd_variant_count(fp16)) return cudaErrorInvalidValue;
#define X_(m, n)                                                                                \
    if (sr == m && pr == n)                                                                     \
        return run_variant<m, n>(st, staged, fp16, variant, inv_scale, out, zsum, errword, stream);
    GNLM_FWD3D_CASES(X_)
#undef X_
    return cudaErrorNotSupported;
}

}  // namespace gnlm
