// The per-tile body of the fused 3D NLM forward, shared by the single-volume
// kernel (nlm3d_fwd.cu) and the persistent batched kernel (nlm3d_batch.cu).
//
// Work decomposition (one output tile of XO x TY x RZ voxels):
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
#pragma once

#include <cuda_fp16.h>

#include <type_traits>

#include "nlm_device.cuh"

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
// One output tile (bx, by, bz) of a staged volume: thread 0 issues the TMA box
// copy of tile + halo into `tile` (completing on `bar`), every thread waits for
// phase `parity`, computes its brick over all offsets and stores.  Returns false
// if the copy did not land within the wait limit (the error word is set).
template <int M, int N, typename T, int RY, int RZ, int NW, bool AREG, bool KAHAN>
__device__ __forceinline__ bool fwd3d_tile(const CUtensorMap* map, T* tile, uint64_t* bar,
                                           uint32_t parity, int bx, int by, int bz, int X, int Y,
                                           int Z, float inv_scale, float* __restrict__ out,
                                           float* __restrict__ zsum, unsigned int* errword) {
    using C = Fwd3d<M, N, T, RY, RZ, NW>;
    static_assert(RY % 2 == 0, "rows are processed in pairs");
    static_assert(N != 1 || RZ % 2 == 0, "patch 3: output planes are processed in pairs");
    constexpr int RP = C::ROWS / 2;  // row pairs a thread sums
    constexpr int OP = RY / 2;       // output row pairs

    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int X0 = bx * C::XO;
    const int Y0 = by * C::TY;
    const int Z0 = bz * RZ;
    const int xs = X0 & ~(C::A - 1);  // 16-byte aligned TMA start column
    const int ral = X0 - xs;

    const bool skip = inject_skip_copy(errword, bx, by, bz);  // false outside test builds
    if (threadIdx.x == 0) {
        fence_proxy_async_smem();  // earlier generic reads of the tile before the async write
        mbar_arrive_expect_tx(bar, C::TILE_BYTES);
        if (!skip) tma_load_3d(tile, map, xs, Y0, Z0, bar);
    }
    if (!tile_copy_wait(bar, parity, errword, skip)) return false;

    // Reference values: lane's column, rows warp*RY + H - N + rr, planes H - N + pl.
    const T* aptr = tile + (C::H - N) * C::PLANE + (warp * RY + C::H - N) * C::BX + (lane + M + ral);
    if constexpr (kBoundsCheck) {  // offsets +-M in every axis around ROWS x PLANES
        const long long a0 = aptr - tile, reach = (long long)M * (C::PLANE + C::BX + 1);
        if (!range_ok(errword, a0 - reach,
                      a0 + reach + (C::ROWS - 1) * C::BX + (C::PLANES - 1) * C::PLANE,
                      (long long)C::BX * C::BY * C::BZ))
            aptr = tile + (C::H - N) * C::PLANE + (C::H - N) * C::BX + M;  // warp 0, lane 0
    }

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
                float2 tr[C::K][RP];   // ring of the last K planes of t (patch 3: of t^2)
                float2 mid[RP];        // patch 3: middle terms shared by an output plane pair
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
                        if constexpr (N == 1) {
                            // three planes' squares summed directly (see fwd3d_tile_pz)
                            const float2 sq = __fmul2_rn(t, t);
                            tr[pl % 3][rp] = sq;
                            if (pl >= 2) {
                                if (((pl - 2) & 1) == 0) {
                                    mid[rp] = __fadd2_rn(tr[(pl - 1) % 3][rp], sq);
                                    S[rp] = __fadd2_rn(tr[(pl - 2) % 3][rp], mid[rp]);
                                } else {
                                    S[rp] = __fadd2_rn(mid[rp], sq);
                                }
                            }
                        } else {
                            if (pl == 0)
                                S[rp] = __fmul2_rn(t, t);
                            else
                                S[rp] = __ffma2_rn(t, t, S[rp]);
                            if (pl >= C::K) {
                                const float2 to = tr[(pl - C::K) % C::K][rp];
                                S[rp] = __ffma2_rn(make_float2(-to.x, -to.y), to, S[rp]);
                            }
                            tr[pl % C::K][rp] = t;
                        }
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
                            if constexpr (N == 1) {
                                const float2 dn =
                                    make_float2(__shfl_down_sync(0xffffffffu, Yv[2 * op], 1),
                                                __shfl_down_sync(0xffffffffu, Yv[2 * op + 1], 1));
                                const float2 up =
                                    make_float2(__shfl_up_sync(0xffffffffu, Yv[2 * op], 1),
                                                __shfl_up_sync(0xffffffffu, Yv[2 * op + 1], 1));
                                xv = __fadd2_rn(xv, __fadd2_rn(dn, up));
                            } else {
                                xv = make_float2(xbox_lanes<N>(Yv[2 * op]), xbox_lanes<N>(Yv[2 * op + 1]));
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
    if (lane >= N && lane < 32 - N && x < X) {
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
    return true;
}

// Window row of element e of row pair p in the grouped kernel's packed arithmetic.
// With patch radius 1 the two halo rows (0 and RY + 1) form pair 0 and pairs 1..RY/2
// are rows (2p - 1, 2p): the centre rows of output rows (2k, 2k + 1) are then the
// aligned pair k + 1, and the candidate centre values enter the packed weighted-sum
// FMA without register moves.  Other radii pair rows (2p, 2p + 1).
template <int N, int RY>
__host__ __device__ constexpr int pz_row(int p, int e) {
    return N == 1 ? (p == 0 ? (e == 0 ? 0 : RY + 1) : 2 * p - 1 + e) : 2 * p + e;
}

// Grouped z offsets (FP32, reference values in registers): the GZ offsets
// (ox, oy, oz+g), g < GZ, share every candidate plane.  With c(j) the candidate plane
// j of offset oz's stream, offset oz+g's difference at the thread's plane pl is
// a(pl) - c(pl+g); streaming j = 0..PLANES+GZ-2, plane j feeds offset oz+g at
// pl = j-g, and every output a member completes at that step (plane j-g-2N) takes
// the same candidate centre c(j-N).  With patch 3 the z window of an output plane is
// the sum of three planes' squares taken directly (the two outputs of a plane pair
// share the middle pair), which issues fewer instructions than a running sum that
// must subtract a negated square (measured at 256^3: 4 x 8 tiles 2.645 -> 2.513 ms).  Shared loads per (voxel, offset):
// (RY+2)(RZ+2N+GZ-1) / (GZ RY RZ) instead of (RY+2)(RZ+2N) / (RY RZ).  The 2M+1 z
// offsets make (2M+1)/GZ full groups and one shorter group for the rest.
template <int M, int N, int RY, int RZ, int NW, int GZ>
__device__ __forceinline__ bool fwd3d_tile_pz(const CUtensorMap* map, float* tile, uint64_t* bar,
                                              uint32_t parity, int bx, int by, int bz, int X, int Y,
                                              int Z, float inv_scale, float* __restrict__ out,
                                              float* __restrict__ zsum, unsigned int* errword) {
    using C = Fwd3d<M, N, float, RY, RZ, NW>;
    static_assert(RY % 2 == 0, "rows are processed in pairs");
    static_assert(N != 1 || RZ % 2 == 0, "patch 3: output planes are processed in pairs");
    constexpr int RP = C::ROWS / 2;
    constexpr int OP = RY / 2;

    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int X0 = bx * C::XO;
    const int Y0 = by * C::TY;
    const int Z0 = bz * RZ;
    const int xs = X0 & ~(C::A - 1);
    const int ral = X0 - xs;

    const bool skip = inject_skip_copy(errword, bx, by, bz);  // false outside test builds
    if (threadIdx.x == 0) {
        fence_proxy_async_smem();
        mbar_arrive_expect_tx(bar, C::TILE_BYTES);
        if (!skip) tma_load_3d(tile, map, xs, Y0, Z0, bar);
    }
    if (!tile_copy_wait(bar, parity, errword, skip)) return false;

    const float* aptr =
        tile + (C::H - N) * C::PLANE + (warp * RY + C::H - N) * C::BX + (lane + M + ral);
    if constexpr (kBoundsCheck) {  // a group of GZ reads planes up to oz + PLANES + GZ - 2 <= M + PLANES - 1
        const long long a0 = aptr - tile, reach = (long long)M * (C::PLANE + C::BX + 1);
        if (!range_ok(errword, a0 - reach,
                      a0 + reach + (C::ROWS - 1) * C::BX + (C::PLANES - 1) * C::PLANE,
                      (long long)C::BX * C::BY * C::BZ))
            aptr = tile + (C::H - N) * C::PLANE + (C::H - N) * C::BX + M;  // warp 0, lane 0
    }
    float2 areg[C::PLANES][RP];
#pragma unroll
    for (int pl = 0; pl < C::PLANES; ++pl)
#pragma unroll
        for (int rp = 0; rp < RP; ++rp)
            areg[pl][rp] = make_float2(aptr[pl * C::PLANE + pz_row<N, RY>(rp, 0) * C::BX],
                                       aptr[pl * C::PLANE + pz_row<N, RY>(rp, 1) * C::BX]);

    float2 zacc[OP][RZ], nacc[OP][RZ];
#pragma unroll
    for (int r = 0; r < OP; ++r)
#pragma unroll
        for (int q = 0; q < RZ; ++q) zacc[r][q] = nacc[r][q] = make_float2(0.f, 0.f);
    const float2 minus1 = make_float2(-1.f, -1.f);

    // y box, x box, weight and accumulation of output plane q from the z-window sums S
    // of the row pairs, with candidate centres cc (output rows 2op, 2op + 1 in cc[op]).
    auto emit = [&](const float2 (&S)[RP], const int q, const float2 (&cc)[OP]) {
        float Srow[C::ROWS];
#pragma unroll
        for (int rp = 0; rp < RP; ++rp) {
            Srow[pz_row<N, RY>(rp, 0)] = S[rp].x;
            Srow[pz_row<N, RY>(rp, 1)] = S[rp].y;
        }
        float Yv[RY];
        if constexpr (N == 1) {
#pragma unroll
            for (int r = 0; r < RY; r += 2) {
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
            if constexpr (N == 1) {
                const float2 dn = make_float2(__shfl_down_sync(0xffffffffu, Yv[2 * op], 1),
                                              __shfl_down_sync(0xffffffffu, Yv[2 * op + 1], 1));
                const float2 up = make_float2(__shfl_up_sync(0xffffffffu, Yv[2 * op], 1),
                                              __shfl_up_sync(0xffffffffu, Yv[2 * op + 1], 1));
                xv = __fadd2_rn(xv, __fadd2_rn(dn, up));
            } else {
                xv = make_float2(xbox_lanes<N>(Yv[2 * op]), xbox_lanes<N>(Yv[2 * op + 1]));
            }
            const float2 w = make_float2(ex2_neg(xv.x), ex2_neg(xv.y));
            zacc[op][q] = __fadd2_rn(zacc[op][q], w);
            nacc[op][q] = __ffma2_rn(w, cc[op], nacc[op][q]);
        }
    };

    auto zgroup = [&](const float* bptr, auto size_tag) {
        constexpr int G = decltype(size_tag)::value;
        constexpr int JEND = C::PLANES + G - 1;
        float2 S[G][RP];
        float2 tr[G][C::K][RP];  // patch 3: squares of the last 3 planes; else differences
        [[maybe_unused]] float2 mid[G][RP];  // patch 3: middle terms shared by a plane pair
        float2 cand[N + 1][OP];  // candidate centres of the last N + 1 planes, output row pairs
#pragma unroll
        for (int j = 0; j < JEND; ++j) {
            float2 c2[RP];
#pragma unroll
            for (int rp = 0; rp < RP; ++rp) {
                const float b0 = bptr[j * C::PLANE + pz_row<N, RY>(rp, 0) * C::BX];
                const float b1 = bptr[j * C::PLANE + pz_row<N, RY>(rp, 1) * C::BX];
                c2[rp] = make_float2(b0, b1);
                if constexpr (N == 1) {
                    if (rp >= 1) cand[j % 2][rp - 1] = c2[rp];  // rows (2rp - 1, 2rp)
                } else {
                    const int r0 = pz_row<N, RY>(rp, 0), r1 = pz_row<N, RY>(rp, 1);
                    if (r0 >= N && r0 < RY + N) {
                        if ((r0 - N) & 1) cand[j % (N + 1)][(r0 - N) / 2].y = b0;
                        else cand[j % (N + 1)][(r0 - N) / 2].x = b0;
                    }
                    if (r1 >= N && r1 < RY + N) {
                        if ((r1 - N) & 1) cand[j % (N + 1)][(r1 - N) / 2].y = b1;
                        else cand[j % (N + 1)][(r1 - N) / 2].x = b1;
                    }
                }
            }
#pragma unroll
            for (int g = 0; g < G; ++g) {
                const int pl = j - g;  // offset oz+g, thread plane pl
                if (pl < 0 || pl >= C::PLANES) continue;
#pragma unroll
                for (int rp = 0; rp < RP; ++rp) {
                    const float2 t = __ffma2_rn(c2[rp], minus1, areg[pl][rp]);
                    if constexpr (N == 1) {
                        // z window of three planes summed directly from the squares of the
                        // last three planes (no running sum to subtract from); the two
                        // outputs of a plane pair share their middle two terms.  RZ is even,
                        // so output planes come in pairs (q even: q, q + 1).
                        const float2 sq = __fmul2_rn(t, t);
                        tr[g][pl % 3][rp] = sq;
                        if (pl >= 2) {
                            if (((pl - 2) & 1) == 0) {
                                mid[g][rp] = __fadd2_rn(tr[g][(pl - 1) % 3][rp], sq);
                                S[g][rp] = __fadd2_rn(tr[g][(pl - 2) % 3][rp], mid[g][rp]);
                            } else {
                                S[g][rp] = __fadd2_rn(mid[g][rp], sq);
                            }
                        }
                    } else {
                        if (pl == 0)
                            S[g][rp] = __fmul2_rn(t, t);
                        else
                            S[g][rp] = __ffma2_rn(t, t, S[g][rp]);
                        if (pl >= C::K) {
                            const float2 to = tr[g][(pl - C::K) % C::K][rp];
                            S[g][rp] = __ffma2_rn(make_float2(-to.x, -to.y), to, S[g][rp]);
                        }
                        tr[g][pl % C::K][rp] = t;
                    }
                }
                if (pl >= 2 * N) emit(S[g], pl - 2 * N, cand[(j - N) % (N + 1)]);
            }
        }
    };

    constexpr int NZ = 2 * M + 1;
    constexpr int REM = NZ % GZ;
    for (int oy = -M; oy <= M; ++oy) {
        for (int ox = -M; ox <= M; ++ox) {
            const float* bxy = aptr + oy * C::BX + ox;
#pragma unroll 1
            for (int oz = -M; oz + GZ - 1 <= M; oz += GZ)
                zgroup(bxy + oz * C::PLANE, std::integral_constant<int, GZ>());
            if constexpr (REM > 0)
                zgroup(bxy + (M - REM + 1) * C::PLANE, std::integral_constant<int, REM>());
        }
    }

    const int x = X0 + lane - N;
    if (lane >= N && lane < 32 - N && x < X) {
#pragma unroll
        for (int q = 0; q < RZ; ++q) {
            const int z = Z0 + q;
            if (z >= Z) break;
#pragma unroll
            for (int r = 0; r < RY; ++r) {
                const int y = Y0 + warp * RY + r;
                if (y >= Y) break;
                const size_t o = ((size_t)z * Y + y) * X + x;
                const float zs = (r & 1) ? zacc[r / 2][q].y : zacc[r / 2][q].x;
                const float nm = (r & 1) ? nacc[r / 2][q].y : nacc[r / 2][q].x;
                out[o] = nm / zs * inv_scale;
                if (zsum) zsum[o] = zs;
            }
        }
    }
    return true;
}

// ---------------------------------------------------------------------------
// FP16-storage form (precision form).  The staged volume is the row-pair layout
// (two copies of half2 pairs, see Staging::pairs), so one 32-bit shared load gives
// a candidate voxel of two adjacent rows: half the shared-memory traffic of FP32.
// Reference values are held as FP32 in registers; each difference is one
// mixed-precision subtraction (FP16 candidate, FP32 reference, FP32 result), so
// no conversion instructions are needed and every square and sum is FP32.  The
// weight sum Z is Kahan-compensated; the weighted sum is kept as
// T = sum w (v_{p+o} - v_p), so that out = v_p + T / Z.  The weights of each
// run of 2M+1 offsets (the innermost x loop) are summed plainly and the run sums
// are added with Kahan compensation.
template <int M, int N, int RY, int RZ, int NW>
struct Fwd3dH2 {
    static constexpr int H = M + N;
    static constexpr int XO = 32 - 2 * N;
    static constexpr int RMAX = 4 - cgcd(XO, 4);
    static constexpr int BX = cround(32 + 2 * M + RMAX, 4);  // half2 columns
    static constexpr int TY = NW * RY;
    static constexpr int BYQ = TY / 2 + H;                    // row pairs per copy
    static constexpr int BZ = RZ + 2 * H;
    static constexpr int PLANEQ = BX * BYQ;
    static constexpr int COPY_BYTES = BX * BYQ * BZ * 4;
    static constexpr int COPY_STRIDE = cround(COPY_BYTES, 128);  // TMA destination alignment
    static constexpr int BAR_OFF = 2 * COPY_STRIDE;
    static constexpr int SMEM_BYTES = BAR_OFF + 128;
    static constexpr int K = 2 * N + 1;
    static constexpr int ROWS = RY + 2 * N;
    static constexpr int PLANES = RZ + 2 * N;
    static_assert(BX <= 256 && BYQ <= 256 && BZ <= 256, "TMA box dimension > 256");
    static_assert(COPY_STRIDE % 128 == 0, "TMA destination alignment");
    static_assert(SMEM_BYTES <= 227 * 1024, "tile exceeds shared memory");
    static_assert(RY % 2 == 0 && (NW * RY) % 2 == 0, "row pairs");
};

// (b_lo - a0, b_hi - a1) in FP32 from a half2 of candidates and FP32 references:
// PTX sub.rn.f32.f16 converts the f16 operand and subtracts in FP32 (one op each).
__device__ __forceinline__ float2 sub_f32_f16x2(__half2 b2, float a0, float a1) {
    float2 r;
    asm("{\n\t.reg .f16 lo, hi;\n\tmov.b32 {lo, hi}, %2;\n\t"
        "sub.rn.f32.f16 %0, lo, %3;\n\tsub.rn.f32.f16 %1, hi, %4;\n\t}"
        : "=f"(r.x), "=f"(r.y)
        : "r"(*reinterpret_cast<const unsigned int*>(&b2)), "f"(a0), "f"(a1));
    return r;
}

template <int M, int N, int RY, int RZ, int NW, bool KAHAN>
__device__ __forceinline__ bool fwd3d_tile_h2(const CUtensorMap* mapE, const CUtensorMap* mapO,
                                              unsigned char* smem, uint64_t* bar, uint32_t parity,
                                              int bx, int by, int bz, int X, int Y, int Z,
                                              float inv_scale, float* __restrict__ out,
                                              float* __restrict__ zsum, unsigned int* errword) {
    using C = Fwd3dH2<M, N, RY, RZ, NW>;
    static_assert(N != 1 || RZ % 2 == 0, "patch 3: output planes are processed in pairs");
    constexpr int RP = C::ROWS / 2;
    constexpr int OP = RY / 2;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int X0 = bx * C::XO, Y0 = by * C::TY, Z0 = bz * RZ;
    const int xs = X0 & ~3;
    const int ral = X0 - xs;
    const __half2* E = reinterpret_cast<const __half2*>(smem);
    const __half2* O = reinterpret_cast<const __half2*>(smem + C::COPY_STRIDE);

    const bool skip = inject_skip_copy(errword, bx, by, bz);  // false outside test builds
    if (threadIdx.x == 0) {
        fence_proxy_async_smem();
        mbar_arrive_expect_tx(bar, 2 * C::COPY_BYTES);
        // E pair k = rows (2k, 2k+1) from pair Y0/2; O pair k = rows (2k+1, 2k+2) from Y0/2 - 1
        if (!skip) {
            tma_load_3d(smem, mapE, xs, Y0 / 2, Z0, bar);
            tma_load_3d(smem + C::COPY_STRIDE, mapO, xs, Y0 / 2 - 1, Z0, bar);
        }
    }
    if (!tile_copy_wait(bar, parity, errword, skip)) return false;

    // Row pair (r, r+1) of the tile, r = Y0 + j: in E at index j/2 if r is even, in O at
    // (j+1)/2 if odd.  The thread's rows start at j = warp*RY + M (+ oy for candidates).
    int col = lane + M + ral;
    int j0 = warp * RY + M;
    if constexpr (kBoundsCheck) {  // row pairs of every oy in both copies, planes and columns +-M
        long long lo = 1LL << 62, hi = -1;
        for (int oy = -M; oy <= M; ++oy) {
            const int jb = j0 + oy;
            const long long pr0 = ((M + oy) & 1) ? (jb + 1) >> 1 : jb >> 1;
            lo = min(lo, pr0 * C::BX + (long long)(C::H - N - M) * C::PLANEQ + col - M);
            hi = max(hi, (pr0 + C::ROWS / 2 - 1) * C::BX +
                             (long long)(C::H - N + M + C::PLANES - 1) * C::PLANEQ + col + M);
        }
        if (!range_ok(errword, lo, hi, (long long)C::BX * C::BYQ * C::BZ)) {
            col = M;  // lane 0 of warp 0
            j0 = M;
        }
    }
    const __half2* abase = (M & 1) ? O + ((j0 + 1) >> 1) * C::BX : E + (j0 >> 1) * C::BX;
    abase += (C::H - N) * C::PLANEQ + col;
    float2 areg[C::PLANES][RP];
#pragma unroll
    for (int pl = 0; pl < C::PLANES; ++pl)
#pragma unroll
        for (int rp = 0; rp < RP; ++rp) areg[pl][rp] = __half22float2(abase[pl * C::PLANEQ + rp * C::BX]);

    Kahan2 zacc[OP][RZ];
    float tacc[RY][RZ];
#pragma unroll
    for (int r = 0; r < OP; ++r)
#pragma unroll
        for (int q = 0; q < RZ; ++q) zacc[r][q].s = zacc[r][q].c = make_float2(0.f, 0.f);
#pragma unroll
    for (int r = 0; r < RY; ++r)
#pragma unroll
        for (int q = 0; q < RZ; ++q) tacc[r][q] = 0.f;

    for (int oy = -M; oy <= M; ++oy) {
        const int jb = j0 + oy;  // >= 0
        const __half2* brow = ((M + oy) & 1) ? O + ((jb + 1) >> 1) * C::BX : E + (jb >> 1) * C::BX;
        for (int oz = -M; oz <= M; ++oz) {
            // plain packed sums of the weights over this run of 2M+1 offsets, folded into
            // the Kahan-compensated total once per run
            float2 zrun[OP][RZ];
#pragma unroll
            for (int r = 0; r < OP; ++r)
#pragma unroll
                for (int q = 0; q < RZ; ++q) zrun[r][q] = make_float2(0.f, 0.f);
            for (int ox = -M; ox <= M; ++ox) {
                const __half2* bptr = brow + (C::H - N + oz) * C::PLANEQ + col + ox;
                float2 S[RP];
                float2 tr[C::K][RP];
                float2 sqr[3][RP], mid[RP];  // patch 3: squares of the last 3 planes, shared pair
#pragma unroll
                for (int pl = 0; pl < C::PLANES; ++pl) {
#pragma unroll
                    for (int rp = 0; rp < RP; ++rp) {
                        const __half2 b2 = bptr[pl * C::PLANEQ + rp * C::BX];
                        // t = v_{p+o} - v_p (sign is irrelevant to the squares)
                        const float2 t = sub_f32_f16x2(b2, areg[pl][rp].x, areg[pl][rp].y);
                        if constexpr (N == 1) {
                            // three planes' squares summed directly, the two outputs of a
                            // plane pair sharing the middle pair (as in fwd3d_tile_pz)
                            const float2 sq = __fmul2_rn(t, t);
                            sqr[pl % 3][rp] = sq;
                            if (pl >= 2) {
                                if (((pl - 2) & 1) == 0) {
                                    mid[rp] = __fadd2_rn(sqr[(pl - 1) % 3][rp], sq);
                                    S[rp] = __fadd2_rn(sqr[(pl - 2) % 3][rp], mid[rp]);
                                } else {
                                    S[rp] = __fadd2_rn(mid[rp], sq);
                                }
                            }
                        } else {
                            if (pl == 0)
                                S[rp] = __fmul2_rn(t, t);
                            else
                                S[rp] = __ffma2_rn(t, t, S[rp]);
                            if (pl >= C::K) {
                                const float2 to = tr[(pl - C::K) % C::K][rp];
                                S[rp] = __ffma2_rn(make_float2(-to.x, -to.y), to, S[rp]);
                            }
                        }
                        tr[pl % C::K][rp] = t;
                    }
                    if (pl >= 2 * N) {
                        const int q = pl - 2 * N;
                        float Srow[C::ROWS], tc[C::ROWS];
#pragma unroll
                        for (int rp = 0; rp < RP; ++rp) {
                            Srow[2 * rp] = S[rp].x;
                            Srow[2 * rp + 1] = S[rp].y;
                            const float2 c2 = tr[(pl - N) % C::K][rp];  // centre plane q + N
                            tc[2 * rp] = c2.x;
                            tc[2 * rp + 1] = c2.y;
                        }
                        float Yv[RY];
                        if constexpr (N == 1) {
#pragma unroll
                            for (int r = 0; r < RY; r += 2) {
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
                            if constexpr (N == 1) {
                                const float2 dn =
                                    make_float2(__shfl_down_sync(0xffffffffu, Yv[2 * op], 1),
                                                __shfl_down_sync(0xffffffffu, Yv[2 * op + 1], 1));
                                const float2 up =
                                    make_float2(__shfl_up_sync(0xffffffffu, Yv[2 * op], 1),
                                                __shfl_up_sync(0xffffffffu, Yv[2 * op + 1], 1));
                                xv = __fadd2_rn(xv, __fadd2_rn(dn, up));
                            } else {
                                xv = make_float2(xbox_lanes<N>(Yv[2 * op]), xbox_lanes<N>(Yv[2 * op + 1]));
                            }
                            const float2 w = make_float2(ex2_neg(xv.x), ex2_neg(xv.y));
                            zrun[op][q] = __fadd2_rn(zrun[op][q], w);
                            tacc[2 * op][q] = fmaf(w.x, tc[2 * op + N], tacc[2 * op][q]);
                            tacc[2 * op + 1][q] = fmaf(w.y, tc[2 * op + 1 + N], tacc[2 * op + 1][q]);
                        }
                    }
                }
            }
#pragma unroll
            for (int r = 0; r < OP; ++r)
#pragma unroll
                for (int q = 0; q < RZ; ++q) {
                    if constexpr (KAHAN)
                        kahan_add(zacc[r][q], zrun[r][q]);
                    else
                        zacc[r][q].s = __fadd2_rn(zacc[r][q].s, zrun[r][q]);
                }
        }
    }

    const int x = X0 + lane - N;
    if (lane >= N && lane < 32 - N && x < X) {
#pragma unroll
        for (int q = 0; q < RZ; ++q) {
            const int z = Z0 + q;
            if (z >= Z) break;
#pragma unroll
            for (int r = 0; r < RY; ++r) {
                const int y = Y0 + warp * RY + r;
                if (y >= Y) break;
                const size_t o = ((size_t)z * Y + y) * X + x;
                const float2 zz = zacc[r / 2][q].s;
                const float zs = (r & 1) ? zz.y : zz.x;
                const float2 a2 = areg[q + N][(r + N) / 2];  // reference value v_p
                const float vp = ((r + N) & 1) ? a2.y : a2.x;
                out[o] = (vp + tacc[r][q] / zs) * inv_scale;
                if (zsum) zsum[o] = zs;
            }
        }
    }
    return true;
}

}  // namespace gnlm
