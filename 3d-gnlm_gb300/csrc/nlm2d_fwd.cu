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

#include <type_traits>

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

// Thread = one column (lane) x RY rows; the reference rows sit in registers
// for all offsets; rows are processed in pairs as packed FP32x2 arithmetic.
// G > 1: the y offsets (ox, oy+g), g < G, share one pass over the candidate rows
// (offset oy+g's candidate for thread row r is row r+g of offset oy's), so candidate
// loads per (pixel, offset) drop from (RY+2N)/RY to (RY+2N+G-1)/(G RY).
template <int M, int N, typename T, int RY, int NW, int MINB, int G>
__global__ void __launch_bounds__(32 * NW, MINB)
    nlm2d_fwd_kernel(const __grid_constant__ CUtensorMap tmap, int X, int Y, float inv_scale,
                     float* __restrict__ out, float* __restrict__ zsum, unsigned int* errword) {
    using C = Fwd2d<M, N, T, RY, NW>;
    static_assert(RY % 2 == 0, "row pairs");
    constexpr int RP = C::ROWS / 2;
    constexpr int OP = RY / 2;
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
    const bool skip = inject_skip_copy(errword, blockIdx.x, blockIdx.y, 0);  // test builds only
    if (threadIdx.x == 0) {
        mbar_arrive_expect_tx(bar, C::TILE_BYTES);
        if (!skip) tma_load_2d(tile, &tmap, xs, Y0, bar);
    }
    if (!tile_copy_wait(bar, 0, errword, skip)) return;

    const T* aptr = tile + (warp * RY + C::H - N) * C::BX + (lane + M + ral);
    if constexpr (kBoundsCheck) {  // offsets +-M around ROWS rows (groups reach the same rows)
        const long long a0 = aptr - tile, reach = (long long)M * (C::BX + 1);
        if (!range_ok(errword, a0 - reach, a0 + reach + (C::ROWS - 1) * C::BX,
                      (long long)C::BX * C::BY))
            aptr = tile + (C::H - N) * C::BX + M;  // warp 0, lane 0
    }
    float2 areg[RP];
#pragma unroll
    for (int rp = 0; rp < RP; ++rp)
        areg[rp] = make_float2(to_f32(aptr[(2 * rp) * C::BX]), to_f32(aptr[(2 * rp + 1) * C::BX]));
    float2 zacc[OP], nacc[OP];
#pragma unroll
    for (int r = 0; r < OP; ++r) zacc[r] = nacc[r] = make_float2(0.f, 0.f);
    const float2 minus1 = make_float2(-1.f, -1.f);

    if constexpr (G > 1) {
        auto group = [&](const T* bptr, auto size_tag) {
            constexpr int GG = decltype(size_tag)::value;
            float c[C::ROWS + GG - 1];
#pragma unroll
            for (int j = 0; j < C::ROWS + GG - 1; ++j) c[j] = to_f32(bptr[j * C::BX]);
#pragma unroll
            for (int g = 0; g < GG; ++g) {
                float q[C::ROWS];
#pragma unroll
                for (int rp = 0; rp < RP; ++rp) {
                    const float2 t = __ffma2_rn(make_float2(c[2 * rp + g], c[2 * rp + 1 + g]), minus1,
                                                areg[rp]);
                    const float2 t2 = __fmul2_rn(t, t);
                    q[2 * rp] = t2.x;
                    q[2 * rp + 1] = t2.y;
                }
                float Yv[RY];
                if constexpr (N == 1) {
#pragma unroll
                    for (int r = 0; r < RY; r += 2) {
                        const float u = q[r + 1] + q[r + 2];
                        Yv[r] = q[r] + u;
                        Yv[r + 1] = u + q[r + 3];
                    }
                } else {
                    float acc = 0.f;
#pragma unroll
                    for (int k = 0; k < C::K; ++k) acc += q[k];
                    Yv[0] = acc;
#pragma unroll
                    for (int r = 1; r < RY; ++r) {
                        acc = acc + q[r + 2 * N] - q[r - 1];
                        Yv[r] = acc;
                    }
                }
#pragma unroll
                for (int op = 0; op < OP; ++op) {
                    const float x0 = xbox_lanes<N>(Yv[2 * op]);
                    const float x1 = xbox_lanes<N>(Yv[2 * op + 1]);
                    const float2 w = make_float2(ex2_neg(x0), ex2_neg(x1));
                    zacc[op] = __fadd2_rn(zacc[op], w);
                    nacc[op] = __ffma2_rn(
                        w, make_float2(c[2 * op + N + g], c[2 * op + 1 + N + g]), nacc[op]);
                }
            }
        };
        constexpr int REM = (2 * M + 1) % G;
        for (int ox = -M; ox <= M; ++ox) {
#pragma unroll 1
            for (int oy = -M; oy + G - 1 <= M; oy += G)
                group(aptr + oy * C::BX + ox, std::integral_constant<int, G>());
            if constexpr (REM > 0)
                group(aptr + (M - REM + 1) * C::BX + ox, std::integral_constant<int, REM>());
        }
    } else
    for (int oy = -M; oy <= M; ++oy) {
        for (int ox = -M; ox <= M; ++ox) {
            const T* bptr = aptr + oy * C::BX + ox;
            float q[C::ROWS], cand[RY];
#pragma unroll
            for (int rp = 0; rp < RP; ++rp) {
                const float b0 = to_f32(bptr[(2 * rp) * C::BX]);
                const float b1 = to_f32(bptr[(2 * rp + 1) * C::BX]);
                const float2 t = __ffma2_rn(make_float2(b0, b1), minus1, areg[rp]);
                const float2 t2 = __fmul2_rn(t, t);
                q[2 * rp] = t2.x;
                q[2 * rp + 1] = t2.y;
                if (2 * rp >= N && 2 * rp < RY + N) cand[2 * rp - N] = b0;
                if (2 * rp + 1 >= N && 2 * rp + 1 < RY + N) cand[2 * rp + 1 - N] = b1;
            }
            float Yv[RY];
            if constexpr (N == 1) {
#pragma unroll
                for (int r = 0; r < RY; r += 2) {
                    const float u = q[r + 1] + q[r + 2];
                    Yv[r] = q[r] + u;
                    Yv[r + 1] = u + q[r + 3];
                }
            } else {
                float acc = 0.f;
#pragma unroll
                for (int k = 0; k < C::K; ++k) acc += q[k];
                Yv[0] = acc;
#pragma unroll
                for (int r = 1; r < RY; ++r) {
                    acc = acc + q[r + 2 * N] - q[r - 1];
                    Yv[r] = acc;
                }
            }
#pragma unroll
            for (int op = 0; op < OP; ++op) {
                const float x0 = xbox_lanes<N>(Yv[2 * op]);
                const float x1 = xbox_lanes<N>(Yv[2 * op + 1]);
                const float2 w = make_float2(ex2_neg(x0), ex2_neg(x1));
                zacc[op] = __fadd2_rn(zacc[op], w);
                nacc[op] = __ffma2_rn(w, make_float2(cand[2 * op], cand[2 * op + 1]), nacc[op]);
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
        const float zs = (r & 1) ? zacc[r / 2].y : zacc[r / 2].x;
        const float nm = (r & 1) ? nacc[r / 2].y : nacc[r / 2].x;
        out[o] = nm / zs * inv_scale;
        if (zsum) zsum[o] = zs;
    }
}

// Two columns per lane (FP32): a warp is two row groups of 16 lanes, lane l of a group
// owning halo columns 2l and 2l+1, so differences, squares and both box sums run as
// packed column pairs and the x box sum is assembled from pair sums P = y0 + y1 of the
// neighbouring lanes: patch 5 takes 2 shuffles per output instead of 3, patch 11 takes
// 3 instead of 6.  Candidate pairs come in one 8-byte shared load, from the tile when
// the column is even, else from a copy of the tile shifted by one float (built in
// shared memory after the TMA copy).  y offsets in groups of G as in nlm2d_fwd_kernel.
template <int M, int N, int RY, int NW>
struct Fwd2dC2 {
    static constexpr int H = M + N;
    static constexpr int XO = 32 - 2 * N;
    static constexpr int RMAX = 4 - cgcd2(XO, 4);
    static constexpr int BX = cround2(32 + 2 * M + RMAX, 4);
    static constexpr int TY = NW * 2 * RY;
    static constexpr int BY = TY + 2 * H;
    static constexpr int TILE_FLOATS = BX * BY;
    static constexpr int COPY_OFF = cround2(TILE_FLOATS * 4, 128);
    static constexpr int BAR_OFF = 2 * COPY_OFF;
    static constexpr int SMEM_BYTES = BAR_OFF + 128;
    static constexpr int K = 2 * N + 1;
    static constexpr int ROWS = RY + 2 * N;
    static_assert(BX % 2 == 0 && XO % 2 == 0, "8-byte aligned column pairs");
    static_assert(BX <= 256 && BY <= 256, "TMA box dimension > 256");
    static_assert(SMEM_BYTES <= 227 * 1024, "tile exceeds shared memory");
};

// Sum of p over the lanes l+A .. l+B of a 16-lane segment (power-of-two windows).
template <int A, int B>
__device__ __forceinline__ float seg_window(float p) {
    constexpr int L = B - A + 1;
    if constexpr (L <= 0) {
        return 0.f;
    } else {
        float pw[5];  // pw[j] = sum over lanes l .. l + 2^j - 1
        pw[0] = p;
#pragma unroll
        for (int j = 1; j < 5; ++j)
            pw[j] = (1 << j) <= L ? pw[j - 1] + __shfl_down_sync(0xffffffffu, pw[j - 1], 1 << (j - 1), 16)
                                  : 0.f;
        float x = 0.f;
        int start = A;
#pragma unroll
        for (int j = 4; j >= 0; --j) {
            if (L & (1 << j)) {
                x += start < 0 ? __shfl_up_sync(0xffffffffu, pw[j], -start, 16)
                               : (start == 0 ? pw[j] : __shfl_down_sync(0xffffffffu, pw[j], start, 16));
                start += 1 << j;
            }
        }
        return x;
    }
}

// x box sums (columns 2l - N .. 2l + N and 2l + 1 - N .. 2l + 1 + N) of lane l's pair y.
template <int N>
__device__ __forceinline__ float2 xbox_pairs(float2 y) {
    const float p = y.x + y.y;
    if constexpr (N % 2 == 1) {
        constexpr int m = (N - 1) / 2;  // pairs l-m .. l+m, then one column on each side
        const float w = seg_window<-m, m>(p);
        return make_float2(w + __shfl_up_sync(0xffffffffu, y.y, m + 1, 16),
                           w + __shfl_down_sync(0xffffffffu, y.x, m + 1, 16));
    } else {
        constexpr int m = N / 2;  // shared pairs l-m+1 .. l+m-1, one more pair and column
        const float v = seg_window<-m + 1, m - 1>(p);
        return make_float2(v + __shfl_up_sync(0xffffffffu, p, m, 16) +
                               __shfl_down_sync(0xffffffffu, y.x, m, 16),
                           v + __shfl_down_sync(0xffffffffu, p, m, 16) +
                               __shfl_up_sync(0xffffffffu, y.y, m, 16));
    }
}

template <int M, int N, int RY, int NW, int MINB, int G>
__global__ void __launch_bounds__(32 * NW, MINB)
    nlm2d_fwd_c2_kernel(const __grid_constant__ CUtensorMap tmap, int X, int Y, float inv_scale,
                        float* __restrict__ out, float* __restrict__ zsum, unsigned int* errword) {
    using C = Fwd2dC2<M, N, RY, NW>;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    float* tile = reinterpret_cast<float*>(smem_raw);
    float* shifted = reinterpret_cast<float*>(smem_raw + C::COPY_OFF);
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw + C::BAR_OFF);

    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int l16 = lane & 15, rg = lane >> 4;
    const int X0 = blockIdx.x * C::XO;
    const int Y0 = blockIdx.y * C::TY;
    const int xs = X0 & ~3;
    const int ral = X0 - xs;  // even: XO is even

    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    const bool skip = inject_skip_copy(errword, blockIdx.x, blockIdx.y, 0);  // test builds only
    if (threadIdx.x == 0) {
        mbar_arrive_expect_tx(bar, C::TILE_FLOATS * 4);
        if (!skip) tma_load_2d(tile, &tmap, xs, Y0, bar);
    }
    if (!tile_copy_wait(bar, 0, errword, skip)) return;
    for (int i = threadIdx.x; i < C::TILE_FLOATS - 1; i += 32 * NW) shifted[i] = tile[i + 1];
    __syncthreads();

    int rowbase = warp * 2 * RY + rg * RY + (C::H - N);
    int colbase = 2 * l16 + M + ral;
    if constexpr (kBoundsCheck) {  // pair loads: columns colbase-M .. colbase+M+1, rows +-M
        // (the shifted copy is read at column colbase+ox-1 only when M+ral+ox is odd,
        // i.e. never for ox = -M: ral is even)
        const long long lo = (long long)(rowbase - M) * C::BX + colbase - M;
        const long long hi = (long long)(rowbase + M + C::ROWS - 1) * C::BX + colbase + M + 1;
        if (!range_ok(errword, lo, hi, C::TILE_FLOATS)) {
            rowbase = C::H - N;  // warp 0, lane 0
            colbase = M + ral;
        }
    }
    auto src = [&](int ox) -> const float* {  // 8-byte aligned base for column offset ox
        return ((M + ral + ox) & 1) ? shifted + (colbase + ox - 1) : tile + (colbase + ox);
    };
    float2 areg[C::ROWS];
    {
        const float* a = src(0) + rowbase * C::BX;
#pragma unroll
        for (int r = 0; r < C::ROWS; ++r) areg[r] = *reinterpret_cast<const float2*>(a + r * C::BX);
    }
    float2 zacc[RY], nacc[RY];
#pragma unroll
    for (int r = 0; r < RY; ++r) zacc[r] = nacc[r] = make_float2(0.f, 0.f);
    const float2 minus1 = make_float2(-1.f, -1.f);

    auto group = [&](const float* bptr, auto size_tag) {
        constexpr int GG = decltype(size_tag)::value;
        float2 c[C::ROWS + GG - 1];
#pragma unroll
        for (int j = 0; j < C::ROWS + GG - 1; ++j) c[j] = *reinterpret_cast<const float2*>(bptr + j * C::BX);
#pragma unroll
        for (int g = 0; g < GG; ++g) {
            float2 q[C::ROWS];
#pragma unroll
            for (int r = 0; r < C::ROWS; ++r) {
                const float2 t = __ffma2_rn(c[r + g], minus1, areg[r]);
                q[r] = __fmul2_rn(t, t);
            }
            float2 acc = q[0];
#pragma unroll
            for (int k = 1; k < C::K; ++k) acc = __fadd2_rn(acc, q[k]);
#pragma unroll
            for (int r = 0; r < RY; ++r) {
                if (r > 0)
                    acc = __fadd2_rn(acc, __fadd2_rn(q[r + 2 * N], make_float2(-q[r - 1].x, -q[r - 1].y)));
                const float2 xv = xbox_pairs<N>(acc);
                const float2 w = make_float2(ex2_neg(xv.x), ex2_neg(xv.y));
                zacc[r] = __fadd2_rn(zacc[r], w);
                nacc[r] = __ffma2_rn(w, c[r + N + g], nacc[r]);
            }
        }
    };
    constexpr int REM = (2 * M + 1) % G;
    for (int ox = -M; ox <= M; ++ox) {
        const float* bx = src(ox) + rowbase * C::BX;
#pragma unroll 1
        for (int oy = -M; oy + G - 1 <= M; oy += G)
            group(bx + oy * C::BX, std::integral_constant<int, G>());
        if constexpr (REM > 0)
            group(bx + (M - REM + 1) * C::BX, std::integral_constant<int, REM>());
    }

#pragma unroll
    for (int cc = 0; cc < 2; ++cc) {
        const int jcol = 2 * l16 + cc;
        const int x = X0 + jcol - N;
        if (jcol < N || jcol >= 32 - N || x >= X) continue;
#pragma unroll
        for (int r = 0; r < RY; ++r) {
            const int y = Y0 + warp * 2 * RY + rg * RY + r;
            if (y >= Y) break;
            const size_t o = (size_t)y * X + x;
            const float zs = cc ? zacc[r].y : zacc[r].x;
            const float nm = cc ? nacc[r].y : nacc[r].x;
            out[o] = nm / zs * inv_scale;
            if (zsum) zsum[o] = zs;
        }
    }
}

template <int M, int N, int RY, int NW, int MINB, int G>
static cudaError_t run_fwd2d_c2(const Staging& st, const void* staged, float inv_scale,
                                float* out, float* zsum, unsigned int* errword,
                                cudaStream_t stream) {
    using C = Fwd2dC2<M, N, RY, NW>;
    CUtensorMap map;
    const uint64_t dims[2] = {(uint64_t)st.Xs, (uint64_t)st.Yp};
    const uint64_t strides[1] = {(uint64_t)st.Xs * 4};
    const uint32_t box[2] = {(uint32_t)C::BX, (uint32_t)C::BY};
    cudaError_t e = encode_tensor_map(&map, false, 2, dims, strides, box, const_cast<void*>(staged));
    if (e != cudaSuccess) return e;
    auto kern = nlm2d_fwd_c2_kernel<M, N, RY, NW, MINB, G>;
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM_BYTES);
    if (e != cudaSuccess) return e;
    dim3 grid((st.X + C::XO - 1) / C::XO, (st.Y + C::TY - 1) / C::TY);
    kern<<<grid, 32 * NW, C::SMEM_BYTES, stream>>>(map, st.X, st.Y, inv_scale, out, zsum, errword);
    return cudaGetLastError();
}

template <int M, int N, typename T, int RY, int NW, int MINB, int G = 1>
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
    auto kern = nlm2d_fwd_kernel<M, N, T, RY, NW, MINB, G>;
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

// Tile variants: 0: 16 rows per thread, 4 warps; 1: 8 rows, 4 warps; 2: 16 rows, 8 warps;
// 3, 4: as 0 and 2 with y offsets in groups of three; 5, 6: two columns per lane
// (nlm2d_fwd_c2_kernel) with 8 rows x 4 warps in groups of six and 4 rows x 8 warps in
// groups of three (FP32; FP16 storage runs variant 4 for them).
template <int m, int n>
static cudaError_t run2d_variant(const Staging& st, const void* staged, bool fp16, int v,
                                 float inv_scale, float* out, float* zsum, unsigned int* ew,
                                 cudaStream_t s) {
    if (fp16) {
        switch (v) {
            case 0: return run_fwd2d<m, n, __half, 16, 4, 3>(st, staged, inv_scale, out, zsum, ew, s);
            case 1: return run_fwd2d<m, n, __half, 8, 4, 4>(st, staged, inv_scale, out, zsum, ew, s);
            case 2: return run_fwd2d<m, n, __half, 16, 8, 2>(st, staged, inv_scale, out, zsum, ew, s);
            case 3: return run_fwd2d<m, n, __half, 16, 4, 3, 3>(st, staged, inv_scale, out, zsum, ew, s);
            case 4:
            case 5:
            case 6: return run_fwd2d<m, n, __half, 16, 8, 2, 3>(st, staged, inv_scale, out, zsum, ew, s);
        }
    } else {
        switch (v) {
            case 0: return run_fwd2d<m, n, float, 16, 4, 3>(st, staged, inv_scale, out, zsum, ew, s);
            case 1: return run_fwd2d<m, n, float, 8, 4, 4>(st, staged, inv_scale, out, zsum, ew, s);
            case 2: return run_fwd2d<m, n, float, 16, 8, 2>(st, staged, inv_scale, out, zsum, ew, s);
            case 3: return run_fwd2d<m, n, float, 16, 4, 3, 3>(st, staged, inv_scale, out, zsum, ew, s);
            case 4: return run_fwd2d<m, n, float, 16, 8, 2, 3>(st, staged, inv_scale, out, zsum, ew, s);
            case 5: return run_fwd2d_c2<m, n, 8, 4, 3, 6>(st, staged, inv_scale, out, zsum, ew, s);
            case 6: return run_fwd2d_c2<m, n, 4, 8, 2, 3>(st, staged, inv_scale, out, zsum, ew, s);
        }
    }
    return cudaErrorInvalidValue;
}

int nlm2d_fwd_variant_count() { return 7; }

bool nlm2d_fwd_supported(int sr, int pr, bool fp16) {
    (void)fp16;
#define X_(m, n) \
    if (sr == m && pr == n) return true;
    GNLM_FWD2D_CASES(X_)
#undef X_
    return false;
}

cudaError_t launch_nlm2d_fwd(const Staging& st, const void* staged, int sr, int pr, bool fp16,
                             int variant, float inv_scale, float* out, float* zsum,
                             unsigned int* errword, cudaStream_t stream) {
    if (variant < 0 || variant >= nlm2d_fwd_variant_count()) return cudaErrorInvalidValue;
#define X_(m, n)                                                                                \
    if (sr == m && pr == n)                                                                     \
        return run2d_variant<m, n>(st, staged, fp16, variant, inv_scale, out, zsum, errword,    \
                                   stream);
    GNLM_FWD2D_CASES(X_)
#undef X_
    return cudaErrorNotSupported;
}

}  // namespace gnlm
