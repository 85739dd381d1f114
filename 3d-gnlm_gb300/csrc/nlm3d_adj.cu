// Adjoint of the 3D NLM forward (no counterpart in the reference).
//
// Notation (scaled units of the staging pass, s = sqrt(log2(e)/(P h^2)), v' = s v):
//   D'_p(o) = sum_t (v'_{p+t} - v'_{p+o+t})^2,  e_p(o) = 2^(-D'_p(o)) = w_p(o),
//   Z_p = sum_o e_p(o),  out'_p = s out_p,  G(p) = g_p / (s Z_p) inside the volume, 0 outside.
// For L = sum_p g_p out_p the gradient with respect to the padded volume is
//   gpad'(q) = sum_o [ G(q+o) e_q(o) + 2 (v'_q - v'_{q+o}) sum_{u in q+box} a_o(u) ]
//   a_o(u)   = -ln2 e_u(o) [ G(u) (v'_{u+o} - out'_u) + G(u+o) (v'_u - out'_{u+o}) ]
// (the two patch-difference terms of dD/dv' collapse into one box sum because
// D'_p(o) = D'_{p+o}(-o)), dL/dv = s * (gpad' folded back through REFLECT_101), and
//   dL/dh = -(2/h) sum_{p in volume} sum_o a1_o(p) D'_p(o),
//   a1_o(p) = -ln2 e_p(o) G(p) (v'_{p+o} - out'_p).
// Every weight is recomputed from the staged volume (nothing per offset is stored),
// each output voxel is written by exactly one thread (a gather, no atomics), and the
// h reduction is two fixed-order passes, so results are bitwise reproducible.
//
// Kernels: adj_aux_kernel ((G, out') pairs padded like the staged volume),
// nlm3d_adj_kernel (gpad' over the padded domain + per-CTA h partial sums; the
// tiles of a last, partial wave are split by offset runs over several CTAs whose
// partial gpad' adj_tail_combine_kernel adds in part order; with patch radius 1 the z
// offsets go in groups that stream each candidate and (G, out') plane once, adj_zgroup),
// adj_fold_kernel (REFLECT_101 fold, times s), adj_hgrad_kernel (fixed-order sum).
#include <cuda_fp16.h>

#include <algorithm>

#include "nlm_device.cuh"
#include "nlm_internal.h"

namespace gnlm {

constexpr int adj_round(int v, int a) { return (v + a - 1) / a * a; }

template <int M, int N, int RY, int RZ, int NW>
struct Adj3d {
    static constexpr int H = M + N;
    static constexpr int HE = H + N;            // tile halo: offset + two box sums
    static constexpr int XO = 32 - 4 * N;       // output lanes per warp (2 box sums across lanes)
    static constexpr int BX = adj_round(32 + 2 * HE + 3, 4);
    static constexpr int TY = NW * RY;
    static constexpr int BY = TY + 2 * HE;
    static constexpr int BZ = RZ + 2 * HE;
    static constexpr int PLANE = BX * BY;
    static constexpr int FIELD_BYTES = BX * BY * BZ * 4;     // v' tile
    static constexpr int GO_BYTES = 2 * FIELD_BYTES;         // (G, out') pair tile
    // each tile starts on a 128-byte boundary: TMA tensor-copy destinations must
    static constexpr int FIELD_STRIDE = adj_round(FIELD_BYTES, 128);
    static constexpr int GO_STRIDE = adj_round(GO_BYTES, 128);
    static constexpr int BAR_OFF = FIELD_STRIDE + GO_STRIDE;  // mbarrier
    static constexpr int RED_OFF = BAR_OFF + 128;             // per-warp h partials
    static constexpr int SMEM_BYTES = RED_OFF + 32 * 8;
    static_assert(FIELD_STRIDE % 128 == 0 && BAR_OFF % 128 == 0, "TMA destination alignment");
    static constexpr int K = 2 * N + 1;
    static constexpr int TILE_VOX = RZ * TY * 32;           // floats of a partial brick tile
    static constexpr int RT = RY + 4 * N, PT = RZ + 4 * N;  // difference window
    static constexpr int RD = RY + 2 * N, PD = RZ + 2 * N;  // distance window
    static_assert(2 * BX <= 256 && BY <= 256 && BZ <= 256, "TMA box dimension > 256");
    static_assert(SMEM_BYTES <= 227 * 1024, "adjoint tile exceeds shared memory");
    static_assert(RY % 2 == 0 && RZ % 2 == 0, "outputs are processed in pairs");
};

// (G, out') = (g / (s Z), s out) pairs, padded like the staged volume (zero outside).
// One warp per padded row (8 rows per block, rows ordered (plane, row)).
__global__ void __launch_bounds__(256) adj_aux_kernel(const float* __restrict__ g,
                                                      const float* __restrict__ out,
                                                      const float* __restrict__ zsum, int X,
                                                      int Y, int Z, int H, int Xs, int Yp,
                                                      long long nrows, float s,
                                                      float2* __restrict__ GO) {
    const long long r = (long long)blockIdx.x * 8 + (threadIdx.x >> 5);
    if (r >= nrows) return;
    const int py = (int)(r % Yp), pz = (int)(r / Yp);
    const int y = py - H, z = pz - H;
    const bool inside_yz = y >= 0 && y < Y && z >= 0 && z < Z;
    float2* row = GO + ((size_t)pz * Yp + py) * Xs;
    for (int px = threadIdx.x & 31; px < Xs; px += 32) {
        const int x = px - H;
        float2 go = make_float2(0.f, 0.f);
        if (inside_yz && x >= 0 && x < X) {
            const size_t i = ((size_t)z * Y + y) * X + x;
            go = make_float2(g[i] / (s * zsum[i]), s * out[i]);
        }
        row[px] = go;
    }
}

// out[i] = in[i] + ... + in[i + K - 1] for i < NO (NO even); each pair of outputs
// shares its K - 1 middle terms.
template <int K, int NO>
__device__ __forceinline__ void box_pairs(const float (&in)[NO + K - 1], float (&out)[NO]) {
    static_assert(NO % 2 == 0, "pairs");
#pragma unroll
    for (int i = 0; i < NO; i += 2) {
        float u = in[i + 1];
#pragma unroll
        for (int k = 2; k < K; ++k) u += in[i + k];
        out[i] = in[i] + u;
        out[i + 1] = u + in[i + K];
    }
}

// x box sum across lanes of a pair of values: the shuffles per value, the adds packed.
template <int N>
__device__ __forceinline__ float2 xbox_pair(float2 y) {
    if constexpr (N == 1) {
        const float2 dn = make_float2(__shfl_down_sync(0xffffffffu, y.x, 1),
                                      __shfl_down_sync(0xffffffffu, y.y, 1));
        const float2 up = make_float2(__shfl_up_sync(0xffffffffu, y.x, 1),
                                      __shfl_up_sync(0xffffffffu, y.y, 1));
        return __fadd2_rn(y, __fadd2_rn(dn, up));
    } else {
        return make_float2(xbox_lanes<N>(y.x), xbox_lanes<N>(y.y));
    }
}

// Offset runs of one tile: (oz, oy) pairs, or (z group, oy) pairs when the z offsets are
// grouped by GZ.
template <int M, int GZ>
__host__ __device__ constexpr int adj_runs() {
    return GZ > 0 ? (2 * M + 1 + GZ - 1) / GZ * (2 * M + 1) : (2 * M + 1) * (2 * M + 1);
}

// The offsets (ox, oy, oz + g), g < G, of one z group, ox = -M..M, for patch radius 1.
// The thread streams the group's candidate planes c = 0 .. PT + G - 2 of its difference
// window once: plane c is difference plane c - g of offset oz + g, so one candidate load
// serves G offsets, and the (G, out') plane c - 2 serves distance plane c - 2 - g of each.
// Per offset the stream keeps three-plane rings of squared differences (z box of t^2),
// of t at the output rows (the t A term) and of the field a (z box of a); distance plane
// pd completes at difference plane pd + 2 and output plane q at distance plane q + 2.
// Within each offset the arithmetic is the window form's (the same sums in the same
// order: plane pairs share the middle terms of their z boxes, row pairs of their y boxes).
template <int M, int RY, int RZ, int NW, int G>
__device__ __forceinline__ void adj_zgroup(const float* vt, const float2* got, int sx, int sy,
                                           int sz, int oz, int oy,
                                           const float2 (&av)[(RY + 4) / 2][RZ + 4],
                                           const float2 (&gref)[RY + 2][RZ + 2],
                                           float (&acc_e)[RY][RZ], float (&acc_t)[RY][RZ],
                                           float& hrun) {
    constexpr int N = 1;
    using C = Adj3d<M, N, RY, RZ, NW>;
    constexpr int RT = C::RT, PT = C::PT, RD = C::RD, RTP = RT / 2;
    constexpr int CEND = PT + G - 1;
    const float2 minus1 = make_float2(-1.f, -1.f);
    auto avs = [&](int r, int p) { return (r & 1) ? av[r >> 1][p].y : av[r >> 1][p].x; };
    for (int ox = -M; ox <= M; ++ox) {
        const int off = oz * C::PLANE + oy * C::BX + ox;
        const float* cb = vt + (sz - 2 * N) * C::PLANE + (sy - 2 * N) * C::BX + sx + off;
        const float2* gb = got + (sz - N) * C::PLANE + (sy - N) * C::BX + sx + off;
        float2 sq[G][3][RTP];  // t^2 of difference planes jj % 3, row pairs
        float2 zmid[G][RTP];   // sq(pd + 1) + sq(pd + 2) of an even distance plane pd
        float2 tt[G][3][RY / 2];  // t at rows 2 .. RY + 1 of difference planes jj % 3
        float ar[G][3][RD];    // a of distance planes pd % 3
        float amid[G][RD];     // a(q + 1) + a(q + 2) of an even output plane q
        float bprev[RT];       // the previous candidate plane (v'_{w+o} of distance plane pd)
#pragma unroll
        for (int c = 0; c < CEND; ++c) {
            float bc[RT];
#pragma unroll
            for (int r = 0; r < RT; ++r) bc[r] = cb[c * C::PLANE + r * C::BX];
            float2 gpl[RD];  // (G, out') at plane c - 2 of the distance window (offset oz)
            if (c >= 2 * N) {
#pragma unroll
                for (int r = 0; r < RD; ++r) gpl[r] = gb[(c - 2 * N) * C::PLANE + r * C::BX];
            }
#pragma unroll
            for (int g = 0; g < G; ++g) {
                const int jj = c - g;  // difference plane of offset oz + g
                if (jj < 0 || jj >= PT) continue;
                float2 s2[RTP];
#pragma unroll
                for (int rp = 0; rp < RTP; ++rp) {
                    const float2 t = __ffma2_rn(make_float2(bc[2 * rp], bc[2 * rp + 1]), minus1,
                                                av[rp][jj]);
                    s2[rp] = __fmul2_rn(t, t);
                    if (rp >= 1 && rp <= RY / 2) tt[g][jj % 3][rp - 1] = t;
                }
                if (jj >= 2 * N) {
                    const int pd = jj - 2 * N;  // distance plane completed by this plane
                    float zrow[RT];
#pragma unroll
                    for (int rp = 0; rp < RTP; ++rp) {
                        float2 z;
                        if ((pd & 1) == 0) {
                            zmid[g][rp] = __fadd2_rn(sq[g][(jj - 1) % 3][rp], s2[rp]);
                            z = __fadd2_rn(sq[g][(jj - 2) % 3][rp], zmid[g][rp]);
                        } else {
                            z = __fadd2_rn(zmid[g][rp], s2[rp]);
                        }
                        zrow[2 * rp] = z.x;
                        zrow[2 * rp + 1] = z.y;
                    }
                    float D[RD];
                    box_pairs<3, RD>(zrow, D);
#pragma unroll
                    for (int r = 0; r < RD; r += 2) {
                        const float2 x2 = xbox_pair<N>(make_float2(D[r], D[r + 1]));
                        D[r] = x2.x;
                        D[r + 1] = x2.y;
                    }
#pragma unroll
                    for (int r = 0; r < RD; ++r) {
                        const float2 go2 = gpl[r];
                        const float e = ex2_neg(D[r]);
                        const float gd = gref[r][pd].x * (bprev[r + N] - gref[r][pd].y);
                        ar[g][pd % 3][r] = e * fmaf(go2.x, avs(r + N, pd + N) - go2.y, gd);
                        const int q = pd - N;
                        if (r >= N && r < N + RY && q >= 0 && q < RZ) {
                            acc_e[r - N][q] = fmaf(go2.x, e, acc_e[r - N][q]);
                            hrun = fmaf(e * gd, D[r], hrun);
                        }
                    }
                    if (pd >= 2 * N) {
                        const int q = pd - 2 * N;  // output plane completed
                        float za[RD];
#pragma unroll
                        for (int r = 0; r < RD; ++r) {
                            if ((q & 1) == 0) {
                                amid[g][r] = ar[g][(pd - 1) % 3][r] + ar[g][pd % 3][r];
                                za[r] = ar[g][(pd - 2) % 3][r] + amid[g][r];
                            } else {
                                za[r] = amid[g][r] + ar[g][pd % 3][r];
                            }
                        }
                        float Ay[RY];
                        box_pairs<3, RY>(za, Ay);
#pragma unroll
                        for (int r = 0; r < RY; r += 2) {
                            const float2 A = xbox_pair<N>(make_float2(Ay[r], Ay[r + 1]));
                            const float2 t = tt[g][pd % 3][r / 2];  // t at rows r + 2, r + 3
                            acc_t[r][q] = fmaf(t.x, A.x, acc_t[r][q]);
                            acc_t[r + 1][q] = fmaf(t.y, A.y, acc_t[r + 1][q]);
                        }
                    }
                }
#pragma unroll
                for (int rp = 0; rp < RTP; ++rp) sq[g][jj % 3][rp] = s2[rp];
            }
#pragma unroll
            for (int r = 0; r < RT; ++r) bprev[r] = bc[r];
        }
    }
}

// Work split of one launch (1D grid): CTAs [0, full) own tiles [0, full) whole;
// each of the ntail tiles after them is split into S parts, CTA full + t*S + p
// making part p of the (2M+1)^2 (oz, oy) offset runs of tile full + t and writing
// its partial gpad' brick to side[(p * ntail + t) * tile_vox ...].
struct AdjTail {
    int nx, ny;   // tiles along x and y
    int full;     // tiles made whole by one CTA
    int S;        // parts per tail tile
    int ntail;    // tail tiles
    float* side;  // S * ntail partial bricks (tile_vox floats each)
};

// GZ = 0: one offset at a time over the whole window.  GZ > 0 (patch radius 1): the z
// offsets in groups of GZ, streamed plane by plane (adj_zgroup below).
template <int M, int N, int RY, int RZ, int NW, int GZ>
__global__ void __launch_bounds__(32 * NW, 1)
    nlm3d_adj_kernel(const __grid_constant__ CUtensorMap vmap,
                     const __grid_constant__ CUtensorMap gomap, int X, int Y, int Z, int Xs, int Yp,
                     float* __restrict__ gpad, double* __restrict__ hpart, const AdjTail tl,
                     unsigned int* errword) {
    using C = Adj3d<M, N, RY, RZ, NW>;
    constexpr float kLn2 = 0.69314718055994531f;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    float* vt = reinterpret_cast<float*>(smem_raw);
    float2* got = reinterpret_cast<float2*>(smem_raw + C::FIELD_STRIDE);
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw + C::BAR_OFF);
    double* red = reinterpret_cast<double*>(smem_raw + C::RED_OFF);

    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int Xp = X + 2 * C::H, Ypd = Y + 2 * C::H, Zp = Z + 2 * C::H;
    // Tile and offset runs of this CTA (uniform over the CTA): (oz, oy) pairs, or (z group,
    // oy) pairs with grouped z offsets.
    constexpr int RUNS = adj_runs<M, GZ>();
    int tile, part = 0, nparts = 1;
    if ((int)blockIdx.x < tl.full) {
        tile = blockIdx.x;
    } else {
        const int j = blockIdx.x - tl.full;
        tile = tl.full + j / tl.S;
        part = j - (j / tl.S) * tl.S;
        nparts = tl.S;
    }
    const int run0 = part * RUNS / nparts, run1 = (part + 1) * RUNS / nparts;
    const int bx = tile % tl.nx, by = (tile / tl.nx) % tl.ny, bz = tile / (tl.nx * tl.ny);
    // Output positions are padded-domain voxels, staged coordinates [0, Xp) etc.
    // smem column 0 starts HE voxels before lane 0's voxel (staged x = bx*XO - 2N)
    const int base_x = bx * C::XO - 2 * N - C::HE;
    const int org_x = base_x & ~3;                  // 16-byte aligned TMA start (may be < 0)
    const int ral = base_x - org_x;
    const int Y0 = by * C::TY, Z0 = bz * RZ;
    const int org_y = Y0 - C::HE, org_z = Z0 - C::HE;

    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    const bool skip = inject_skip_copy(errword, bx, by, bz);  // test builds only
    if (threadIdx.x == 0) {
        mbar_arrive_expect_tx(bar, C::FIELD_BYTES + C::GO_BYTES);
        if (!skip) {
            tma_load_3d(vt, &vmap, org_x, org_y, org_z, bar);
            tma_load_3d(got, &gomap, 2 * org_x, org_y, org_z, bar);
        }
    }
    if (!tile_copy_wait(bar, 0, errword, skip)) return;

    // smem position of this thread's (row 0, plane 0) output voxel
    int sx = lane + C::HE + ral;
    int sy = warp * RY + C::HE;
    const int sz = C::HE;
    if constexpr (kBoundsCheck) {  // v' window +-2N around the brick, offsets +-M; G/out' +-N
        const long long reach = (long long)M * (C::PLANE + C::BX + 1), n = (long long)C::PLANE * C::BZ;
        const long long v0 = (long long)(sz - 2 * N) * C::PLANE + (sy - 2 * N) * C::BX + sx;
        const long long g0 = (long long)(sz - N) * C::PLANE + (sy - N) * C::BX + sx;
        const bool ok =
            range_ok(errword, v0 - reach, v0 + reach + (C::RT - 1) * C::BX + (C::PT - 1) * C::PLANE, n) &&
            range_ok(errword, g0 - reach, g0 + reach + (C::RD - 1) * C::BX + (C::PD - 1) * C::PLANE, n);
        if (!ok) {
            sx = C::HE + ral;  // lane 0 of warp 0
            sy = C::HE;
        }
    }
    // v' values of the difference window (same for every offset), as row pairs
    static_assert(C::RT % 2 == 0, "row pairs");
    constexpr int K = C::K, RTP = C::RT / 2, RD = C::RD, PD = C::PD;
    float2 av[RTP][C::PT];
    // (G, out') at the distance window (same for every offset)
    float2 gref[RD][PD];
#pragma unroll
    for (int rp = 0; rp < RTP; ++rp)
#pragma unroll
        for (int p = 0; p < C::PT; ++p) {
            const int i = (sz + p - 2 * N) * C::PLANE + (sy + 2 * rp - 2 * N) * C::BX + sx;
            av[rp][p] = make_float2(vt[i], vt[i + C::BX]);
        }
#pragma unroll
    for (int r = 0; r < RD; ++r)
#pragma unroll
        for (int p = 0; p < PD; ++p) gref[r][p] = got[(sz + p - N) * C::PLANE + (sy + r - N) * C::BX + sx];
    auto avs = [&](int r, int p) { return (r & 1) ? av[r >> 1][p].y : av[r >> 1][p].x; };

    // gpad' = acc_e + (-2 ln2) acc_t: the G(q+o) e_q(o) terms and the t A terms
    float acc_e[RY][RZ], acc_t[RY][RZ];
#pragma unroll
    for (int r = 0; r < RY; ++r)
#pragma unroll
        for (int q = 0; q < RZ; ++q) acc_e[r][q] = acc_t[r][q] = 0.f;
    double hacc = 0.0;
    const float2 minus1 = make_float2(-1.f, -1.f);

    if constexpr (GZ > 0) {
        constexpr int ZG = (2 * M + 1 + GZ - 1) / GZ, GR = (2 * M + 1) - (ZG - 1) * GZ;
        for (int run = run0; run < run1; ++run) {
            const int gi = run / (2 * M + 1), oy = run % (2 * M + 1) - M;
            const int oz = -M + gi * GZ;
            float hrun = 0.f;
            if (gi < ZG - 1)
                adj_zgroup<M, RY, RZ, NW, GZ>(vt, got, sx, sy, sz, oz, oy, av, gref, acc_e, acc_t, hrun);
            else
                adj_zgroup<M, RY, RZ, NW, GR>(vt, got, sx, sy, sz, oz, oy, av, gref, acc_e, acc_t, hrun);
            hacc += (double)hrun;
        }
    } else
    for (int run = run0; run < run1; ++run) {
        const int oz = run / (2 * M + 1) - M, oy = run % (2 * M + 1) - M;
        {
            // dL/dh terms of this run of 2M+1 offsets, summed in FP32, then added to
            // the FP64 total once per run
            float hrun = 0.f;
            for (int ox = -M; ox <= M; ++ox) {
                const int off = oz * C::PLANE + oy * C::BX + ox;
                // differences t = v'_u - v'_{u+o} over the window (row pairs), candidates b
                float2 t2[RTP][C::PT];
                float bv[RD][PD];
#pragma unroll
                for (int rp = 0; rp < RTP; ++rp)
#pragma unroll
                    for (int p = 0; p < C::PT; ++p) {
                        const int i =
                            (sz + p - 2 * N) * C::PLANE + (sy + 2 * rp - 2 * N) * C::BX + sx + off;
                        const float b0 = vt[i], b1 = vt[i + C::BX];
                        t2[rp][p] = __ffma2_rn(make_float2(b0, b1), minus1, av[rp][p]);
                        const int r0 = 2 * rp, r1 = 2 * rp + 1;
                        if (p >= N && p < N + PD) {
                            if (r0 >= N && r0 < N + RD) bv[r0 - N][p - N] = b0;
                            if (r1 >= N && r1 < N + RD) bv[r1 - N][p - N] = b1;
                        }
                    }
                auto ts = [&](int r, int p) { return (r & 1) ? t2[r >> 1][p].y : t2[r >> 1][p].x; };
                // distance D' on the distance window: z sums of t^2 (sliding window over
                // packed row pairs), y sums (pairs of rows share the middle terms), x
                // across lanes (adds packed over pairs of planes)
                float zrow[C::RT][PD];
#pragma unroll
                for (int rp = 0; rp < RTP; ++rp) {
                    if constexpr (N == 1 && PD % 2 == 0) {
                        // three planes' squares summed directly; pairs of output planes
                        // share their middle pair (no running sum to subtract from)
                        float2 sq[C::PT];
#pragma unroll
                        for (int p = 0; p < C::PT; ++p) sq[p] = __fmul2_rn(t2[rp][p], t2[rp][p]);
#pragma unroll
                        for (int p = 0; p < PD; p += 2) {
                            const float2 m2 = __fadd2_rn(sq[p + 1], sq[p + 2]);
                            const float2 z0 = __fadd2_rn(sq[p], m2), z1 = __fadd2_rn(m2, sq[p + 3]);
                            zrow[2 * rp][p] = z0.x;
                            zrow[2 * rp + 1][p] = z0.y;
                            zrow[2 * rp][p + 1] = z1.x;
                            zrow[2 * rp + 1][p + 1] = z1.y;
                        }
                    } else {
                        float2 run = __fmul2_rn(t2[rp][0], t2[rp][0]);
#pragma unroll
                        for (int k = 1; k < K; ++k) run = __ffma2_rn(t2[rp][k], t2[rp][k], run);
                        zrow[2 * rp][0] = run.x;
                        zrow[2 * rp + 1][0] = run.y;
#pragma unroll
                        for (int p = 1; p < PD; ++p) {
                            const float2 tn = t2[rp][p + K - 1], to = t2[rp][p - 1];
                            run = __ffma2_rn(tn, tn, run);
                            run = __ffma2_rn(make_float2(-to.x, -to.y), to, run);
                            zrow[2 * rp][p] = run.x;
                            zrow[2 * rp + 1][p] = run.y;
                        }
                    }
                }
                float D[RD][PD];
#pragma unroll
                for (int p = 0; p < PD; ++p) {
                    float col[C::RT], dcol[RD];
#pragma unroll
                    for (int r = 0; r < C::RT; ++r) col[r] = zrow[r][p];
                    box_pairs<K, RD>(col, dcol);
#pragma unroll
                    for (int r = 0; r < RD; ++r) D[r][p] = dcol[r];
                }
#pragma unroll
                for (int r = 0; r < RD; ++r)
#pragma unroll
                    for (int p = 0; p < PD; p += 2) {
                        const float2 x2 = xbox_pair<N>(make_float2(D[r][p], D[r][p + 1]));
                        D[r][p] = x2.x;
                        D[r][p + 1] = x2.y;
                    }
                // weights, (G, out') at u+o, and the field a_o(u) (without the -ln2);
                // gd = G(u) (v'_{u+o} - out'_u) is shared with the dL/dh term
                float e[RD][PD], a[RD][PD], gd[RD][PD], guo[RD][PD];
#pragma unroll
                for (int r = 0; r < RD; ++r)
#pragma unroll
                    for (int p = 0; p < PD; ++p) {
                        const int i = (sz + p - N) * C::PLANE + (sy + r - N) * C::BX + sx + off;
                        const float2 go2 = got[i];
                        e[r][p] = ex2_neg(D[r][p]);
                        guo[r][p] = go2.x;
                        const float vu = avs(r + N, p + N);
                        gd[r][p] = gref[r][p].x * (bv[r][p] - gref[r][p].y);
                        a[r][p] = e[r][p] * fmaf(go2.x, vu - go2.y, gd[r][p]);
                    }
                // box sum of a over the patch: z, then y (pairs share the middle terms),
                // then x across lanes
                float za[RD][RZ];
#pragma unroll
                for (int r = 0; r < RD; ++r) box_pairs<K, RZ>(a[r], za[r]);
#pragma unroll
                for (int q = 0; q < RZ; q += 2) {
                    float c0[RD], c1[RD], y0[RY], y1[RY];
#pragma unroll
                    for (int r = 0; r < RD; ++r) {
                        c0[r] = za[r][q];
                        c1[r] = za[r][q + 1];
                    }
                    box_pairs<K, RY>(c0, y0);
                    box_pairs<K, RY>(c1, y1);
#pragma unroll
                    for (int r = 0; r < RY; ++r) {
                        const float2 xv = xbox_pair<N>(make_float2(y0[r], y1[r]));
#pragma unroll
                        for (int h = 0; h < 2; ++h) {
                            const int qq = q + h;
                            const float A = h ? xv.y : xv.x;
                            // gpad' += G(q+o) e_q(o) + 2 (v'_q - v'_{q+o}) (-ln2) A(q)
                            acc_e[r][qq] = fmaf(guo[r + N][qq + N], e[r + N][qq + N], acc_e[r][qq]);
                            acc_t[r][qq] = fmaf(ts(r + 2 * N, qq + 2 * N), A, acc_t[r][qq]);
                            // dL/dh partial: a1_o(q) D'_q(o), a1 = -ln2 e G(q) (v'_{q+o} - out'_q)
                            hrun = fmaf(e[r + N][qq + N] * gd[r + N][qq + N], D[r + N][qq + N], hrun);
                        }
                    }
                }
            }
            hacc += (double)hrun;
        }
    }
    float acc[RY][RZ];
#pragma unroll
    for (int r = 0; r < RY; ++r)
#pragma unroll
        for (int q = 0; q < RZ; ++q) acc[r][q] = fmaf(-2.f * kLn2, acc_t[r][q], acc_e[r][q]);

    // store gpad' for the thread's padded-domain voxels (or this part's partial
    // brick, every lane); reduce the h partial
    const int px = bx * C::XO + lane - 2 * N;  // staged x of this lane
    const bool lane_ok = lane >= 2 * N && lane < 32 - 2 * N && px < Xp;
    double hsum = 0.0;
    if (nparts == 1) {
#pragma unroll
        for (int q = 0; q < RZ; ++q) {
            const int pz = Z0 + q;
#pragma unroll
            for (int r = 0; r < RY; ++r) {
                const int py = Y0 + warp * RY + r;
                if (lane_ok && py < Ypd && pz < Zp) gpad[((size_t)pz * Yp + py) * Xs + px] = acc[r][q];
            }
        }
    } else {
        float* brick = tl.side + ((size_t)part * tl.ntail + (tile - tl.full)) * C::TILE_VOX;
#pragma unroll
        for (int q = 0; q < RZ; ++q)
#pragma unroll
            for (int r = 0; r < RY; ++r) brick[(q * C::TY + warp * RY + r) * 32 + lane] = acc[r][q];
    }
    // Halo lanes duplicate a neighbouring CTA's voxels: only output lanes count.
    // Voxels outside the volume (padding, rows/planes past the end) have G = 0 and
    // add nothing.
    hsum = lane_ok ? hacc : 0.0;
    for (int k = 16; k > 0; k >>= 1) hsum += __shfl_down_sync(0xffffffffu, hsum, k);
    if (lane == 0) red[warp] = hsum;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < NW; ++w) s += red[w];
        hpart[blockIdx.x] = -kLn2 * s;
    }
}

// gpad' of the tail tiles: the sum of their S partial bricks, in part order.  Grid
// (tail tiles, slices): the blocks of a tile split its voxels.
template <int N, int RZ, int TY, int XO>
__global__ void __launch_bounds__(256) adj_tail_combine_kernel(const AdjTail tl, int Xp, int Ypd,
                                                               int Zp, int Xs, int Yp,
                                                               float* __restrict__ gpad) {
    constexpr int TILE_VOX = RZ * TY * 32;
    const int t = blockIdx.x, tile = tl.full + t;
    const int bx = tile % tl.nx, by = (tile / tl.nx) % tl.ny, bz = tile / (tl.nx * tl.ny);
    for (int k = blockIdx.y * blockDim.x + threadIdx.x; k < TILE_VOX; k += gridDim.y * blockDim.x) {
        const int lane = k & 31, row = (k >> 5) % TY, q = (k >> 5) / TY;
        const int px = bx * XO + lane - 2 * N, py = by * TY + row, pz = bz * RZ + q;
        if (lane < 2 * N || lane >= 32 - 2 * N || px >= Xp || py >= Ypd || pz >= Zp) continue;
        float sum = 0.f;
        for (int p = 0; p < tl.S; ++p) sum += tl.side[((size_t)p * tl.ntail + t) * TILE_VOX + k];
        gpad[((size_t)pz * Yp + py) * Xs + px] = sum;
    }
}

// Padded positions along one axis whose REFLECT_101 source is i: i + H, plus any of
// the 2H border positions that reflect onto i.  Returns the count (<= 1 + 2H).
__device__ __forceinline__ int preimages(int i, int n, int H, int* p) {
    int k = 0;
    p[k++] = i + H;
    for (int b = 0; b < H; ++b) {
        if (reflect101_near(b - H, n) == i) p[k++] = b;
        if (reflect101_near(n + b, n) == i) p[k++] = n + H + b;
    }
    return k;
}

// gin(x) = s * sum of gpad' over the padded positions that REFLECT_101 maps to x.
// Columns H+1 .. X-2-H have the one preimage x + H (no border column reflects onto
// them) and skip the preimage search; the summation order is the same either way.
constexpr int kMaxHalo = 16;
__global__ void __launch_bounds__(256) adj_fold_kernel(const float* __restrict__ gpad, int X,
                                                       int Y, int Z, int H, int Xs, int Yp,
                                                       float s, float* __restrict__ gin) {
    const int y = blockIdx.x, z = blockIdx.y;
    int pz[1 + 2 * kMaxHalo], py[1 + 2 * kMaxHalo], px[1 + 2 * kMaxHalo];
    const int nz = preimages(z, Z, H, pz);
    const int ny = preimages(y, Y, H, py);
    for (int x = threadIdx.x; x < X; x += blockDim.x) {
        float sum = 0.f;
        if (x > H && x < X - 1 - H) {
            for (int a = 0; a < nz; ++a)
                for (int b = 0; b < ny; ++b) sum += gpad[((size_t)pz[a] * Yp + py[b]) * Xs + x + H];
        } else {
            const int nx = preimages(x, X, H, px);
            for (int a = 0; a < nz; ++a)
                for (int b = 0; b < ny; ++b) {
                    const float* row = gpad + ((size_t)pz[a] * Yp + py[b]) * Xs;
                    for (int c = 0; c < nx; ++c) sum += row[px[c]];
                }
        }
        gin[((size_t)z * Y + y) * X + x] = s * sum;
    }
}

// dL/dh = -(2/h) * sum of the per-CTA partials.  One block: thread t sums partials
// t, t + 256, ... in index order, then a fixed binary tree adds the 256 thread sums.
// The order never changes, so the result is bitwise reproducible.
constexpr int kHgradThreads = 256;
__global__ void __launch_bounds__(kHgradThreads) adj_hgrad_kernel(const double* __restrict__ hpart,
                                                                  int n, double coef,
                                                                  double* __restrict__ hgrad) {
    __shared__ double red[kHgradThreads];
    double s = 0.0;
    for (int i = threadIdx.x; i < n; i += kHgradThreads) s += hpart[i];
    red[threadIdx.x] = s;
    __syncthreads();
#pragma unroll
    for (int w = kHgradThreads / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) *hgrad = coef * red[0];
}

// Tail split bounds: S * ntail <= min(SMs, kAdjMaxTailCtas), S <= kAdjMaxParts.
constexpr int kAdjMaxTailCtas = 1024;
constexpr int kAdjMaxParts = 16;

// With one CTA per SM, n tiles fill n / SMs whole waves; the tiles of a last,
// partial wave are split into S parts of their offset runs so that the tail wave
// holds S * ntail <= SMs CTAs of 1/S of the work.
static AdjTail adj_tail_plan(int nx, int ny, int nz, int runs) {
    AdjTail t{};
    t.nx = nx;
    t.ny = ny;
    const int n = nx * ny * nz;
    const int slots = std::min(device_sm_count(), kAdjMaxTailCtas);
    const int tail = n % slots;
    const int S = tail ? std::min(std::min(slots / tail, runs), kAdjMaxParts) : 1;
    if (S < 2) {
        t.full = n;
        t.S = 1;
        t.ntail = 0;
    } else {
        t.full = n - tail;
        t.S = S;
        t.ntail = tail;
    }
    return t;
}

template <int M, int N, int RY, int RZ, int NW, int GZ>
static cudaError_t run_adj3d(const Staging& st, const void* staged, const float* d_out,
                             const float* d_zsum, const float* d_gout, float s, float h,
                             float* gin, double* hgrad, float2* GO, float* gpad,
                             double* hpart, float* side, unsigned int* errword,
                             cudaStream_t stream) {
    using C = Adj3d<M, N, RY, RZ, NW>;
    const long long nrows = (long long)st.Yp * st.Zp;
    adj_aux_kernel<<<(unsigned)((nrows + 7) / 8), 256, 0, stream>>>(
        d_gout, d_out, d_zsum, st.X, st.Y, st.Z, st.H, st.Xs, st.Yp, nrows, s, GO);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    CUtensorMap vmap, gomap;
    const uint64_t dims[3] = {(uint64_t)st.Xs, (uint64_t)st.Yp, (uint64_t)st.Zp};
    const uint64_t strides[2] = {(uint64_t)st.Xs * 4, (uint64_t)st.Xs * st.Yp * 4};
    const uint32_t box[3] = {(uint32_t)C::BX, (uint32_t)C::BY, (uint32_t)C::BZ};
    // (G, out') pairs: the same geometry with twice the floats per row
    const uint64_t dims2[3] = {2 * (uint64_t)st.Xs, (uint64_t)st.Yp, (uint64_t)st.Zp};
    const uint64_t strides2[2] = {(uint64_t)st.Xs * 8, (uint64_t)st.Xs * st.Yp * 8};
    const uint32_t box2[3] = {2 * (uint32_t)C::BX, (uint32_t)C::BY, (uint32_t)C::BZ};
    if ((e = encode_tensor_map(&vmap, false, 3, dims, strides, box, const_cast<void*>(staged))))
        return e;
    if ((e = encode_tensor_map(&gomap, false, 3, dims2, strides2, box2, GO))) return e;
    auto kern = nlm3d_adj_kernel<M, N, RY, RZ, NW, GZ>;
    if ((e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM_BYTES)))
        return e;
    AdjTail tl = adj_tail_plan((st.Xp + C::XO - 1) / C::XO, (st.Yp + C::TY - 1) / C::TY,
                               (st.Zp + RZ - 1) / RZ, adj_runs<M, GZ>());
    tl.side = side;
    const int nblk = tl.full + tl.S * tl.ntail;
    kern<<<nblk, 32 * NW, C::SMEM_BYTES, stream>>>(vmap, gomap, st.X, st.Y, st.Z, st.Xs, st.Yp,
                                                   gpad, hpart, tl, errword);
    if ((e = cudaGetLastError())) return e;
    if (tl.ntail > 0) {
        const dim3 cgrid(tl.ntail, (C::TILE_VOX + 255) / 256);
        adj_tail_combine_kernel<N, RZ, C::TY, C::XO><<<cgrid, 256, 0, stream>>>(
            tl, st.Xp, st.Yp, st.Zp, st.Xs, st.Yp, gpad);
        if ((e = cudaGetLastError())) return e;
    }
    dim3 out_rows(st.Y, st.Z);
    adj_fold_kernel<<<out_rows, 128, 0, stream>>>(gpad, st.X, st.Y, st.Z, st.H, st.Xs, st.Yp, s,
                                                  gin);
    if ((e = cudaGetLastError())) return e;
    if (hgrad) {
        adj_hgrad_kernel<<<1, kHgradThreads, 0, stream>>>(hpart, nblk, -2.0 / (double)h, hgrad);
        e = cudaGetLastError();
    }
    return e;
}

// Z offsets per group of the patch-radius-1 adjoint: at most GMAX, the 2M + 1 offsets
// split into equal groups where they divide (9 -> 5 + 4, 11 -> 6 + 5, 7 -> 2+2+2+1).
constexpr int adj_group(int n, int gmax) {
    const int groups = (n + gmax - 1) / gmax;
    return (n + groups - 1) / groups;
}

// Tile shape per (sr, pr): 8 warps x 2 rows x 4 planes, or 4 x 2 x 2 where the
// three FP32 tiles of a larger halo would not fit in shared memory.
template <int M, int N>
struct AdjShape {
    static constexpr bool SMALL = M + 2 * N > 5;
    static constexpr int RY = 2, RZ = SMALL ? 2 : 4, NW = SMALL ? 4 : 8;
    // z offsets per group (patch 3): the 2-plane tiles hold six offsets' rings within the
    // register budget (232-254 registers), the 4-plane tiles two (252 registers)
    static constexpr int GZ = N == 1 ? adj_group(2 * M + 1, SMALL ? 6 : 2) : 0;
    using C = Adj3d<M, N, RY, RZ, NW>;
};

#define GNLM_ADJ3D_CASES(X_) X_(1, 1) X_(2, 1) X_(3, 1) X_(4, 1) X_(5, 1) X_(3, 2)

bool nlm3d_adj_supported(int sr, int pr) {
#define X_(m, n) \
    if (sr == m && pr == n) return true;
    GNLM_ADJ3D_CASES(X_)
#undef X_
    return false;
}

// Upper bound on the CTAs of the adjoint kernel (one double of h partials each):
// the tiles plus at most kAdjMaxTailCtas tail-part CTAs.
size_t adj3d_ctas(const Staging& st, int sr, int pr) {
#define X_(m, n)                                                                             \
    if (sr == m && pr == n) {                                                                \
        using C = AdjShape<m, n>::C;                                                         \
        return (size_t)((st.Xp + C::XO - 1) / C::XO) * ((st.Yp + C::TY - 1) / C::TY) *     \
                   ((st.Zp + AdjShape<m, n>::RZ - 1) / AdjShape<m, n>::RZ) +                 \
               kAdjMaxTailCtas;                                                              \
    }
    GNLM_ADJ3D_CASES(X_)
#undef X_
    return 0;
}

// Bytes of the tail parts' partial bricks.
size_t adj3d_side_bytes(int sr, int pr) {
#define X_(m, n) \
    if (sr == m && pr == n) return (size_t)kAdjMaxTailCtas * AdjShape<m, n>::C::TILE_VOX * 4;
    GNLM_ADJ3D_CASES(X_)
#undef X_
    return 0;
}

cudaError_t launch_nlm3d_adj(const Staging& st, const void* staged, const float* d_out,
                             const float* d_zsum, const float* d_gout, int sr, int pr, float s,
                             float h, float* gin, double* hgrad, float2* GO, float* gpad,
                             double* hpart, float* side, unsigned int* errword,
                             cudaStream_t stream) {
    if (st.H > kMaxHalo) return cudaErrorNotSupported;
#define X_(m, n)                                                                                \
    if (sr == m && pr == n)                                                                     \
        return run_adj3d<m, n, AdjShape<m, n>::RY, AdjShape<m, n>::RZ, AdjShape<m, n>::NW,     \
                         AdjShape<m, n>::GZ>(                                                   \
            st, staged, d_out, d_zsum, d_gout, s, h, gin, hgrad, GO, gpad, hpart, side,         \
            errword, stream);
    GNLM_ADJ3D_CASES(X_)
#undef X_
    return cudaErrorNotSupported;
}

}  // namespace gnlm
