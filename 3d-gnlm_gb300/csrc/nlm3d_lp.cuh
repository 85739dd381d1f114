// Large-patch 3D NLM forward (patch radius up to 8, search radius up to 6): the
// reference's NS = 7..17 configurations (3DNLM/main.cu:1005-7599, swept with
// SS 11/13 and NS 13/15/17 by 3DNLM/run.sh:25-34).
//
// The register-brick kernel (nlm3d_tile.cuh) recomputes a (RY+2pr) x (RZ+2pr)
// block of differences per offset and sums x by 2pr shuffles, so its cost grows
// with the patch; here every box sum is a running sum and the cost per (voxel,
// offset) does not depend on the patch width.
//
// One CTA owns a column tile of 32 x 16 output voxels and a chunk of TZ planes.
// It makes (2sr+1)^2 passes, one per (oz, oy); a pass covers all 2sr+1 x
// offsets and streams the chunk's planes (plus the patch halo) in z:
//   A  each thread owns 4 halo columns of one halo row and keeps, per x offset,
//      the running z-sum Sz of squared differences over the 2pr+1 planes around
//      the current plane (add the entering plane, subtract the leaving one; the
//      first window is built two planes per step); the reference plane and the
//      candidate plane of a step come in as TMA boxes (double-buffered,
//      prefetched one step ahead), and one 4-column candidate window serves all
//      2sr+1 x offsets;
//   B  x box sum of Sz along each halo row (shared memory, running sum);
//   C  y box sum down each output column, in place (running sum) -> D;
//   D  w = 2^(-D) (the staging pass pre-scaled the volume so D is the base-2
//      exponent of exp(-(D/P)/h^2), 3DNLM/main.cu:108-109), Z += w, num += w v
//      over the pass's x offsets, then one read-add-write of the voxel's (Z, num)
//      pair in the accumulator buffer (L2-resident: a chunk's pairs are re-read
//      once per pass, in pass order, so the sums are deterministic).  The last
//      pass writes out = num / Z (3DNLM/main.cu:125).
// With one CTA per SM, a grid of a few waves can leave most of the last wave
// idle; the launcher may then split each tile's passes into two halves run by
// two CTAs with separate accumulator buffers, and a combine kernel adds the two
// halves (always in the same order) and writes num / Z.
//
// Storage type T: float, or __half for the FP16-storage form (the staged volume and
// the TMA plane boxes hold FP16, halving their bytes; every difference, square and
// sum is FP32, and the per-pass weight sums are added across passes with Kahan
// compensation, the (Z, num) accumulator then holding (Z, num, cZ, cnum)).  TMA needs
// 16-byte aligned box starts and widths, so for FP16 the boxes start 8 elements
// before the tile (candidate box) or on the 8-element boundary below the first
// halo group (reference box) and the in-box column offsets CB and RO absorb that.
#pragma once

#include <algorithm>

#include "nlm3d_tile.cuh"
#include "nlm_device.cuh"
#include "nlm_internal.h"

namespace gnlm {

template <int M, int N, typename T>
struct Lp3d {
    static constexpr int ES = (int)sizeof(T);  // bytes per staged element
    static constexpr int EA = 16 / ES;         // elements per 16 bytes (TMA alignment)
    static constexpr bool KAHAN = ES == 2;     // FP16-storage form: compensated pass sums
    static constexpr int K = 2 * M + 1;        // x offsets per pass
    static constexpr int CX = 32;              // output columns per CTA
    static constexpr int CY = 16;              // output rows per CTA
    static constexpr int H = M + N;
    static constexpr int HX = CX + 2 * N;      // halo columns
    static constexpr int HY = CY + 2 * N;      // halo rows
    // Column i of the 4-column group layout is padded column X0 - 4 + i (halo column
    // xh is i = 4 + M + xh).  The candidate box starts at padded column X0 - 4 - CB and
    // the reference box at X0 - 4 + 4*G0 - RO (16-byte aligned starts), so layout
    // column i sits at candidate-box column i + CB.
    static constexpr int R = (M + 3) / 4;      // candidate 4-column groups either side
    static constexpr int G0 = 1 + M / 4;       // first 4-column group holding a halo column
    static constexpr int G1 = (4 + M + HX + 3) / 4;
    static constexpr int NG = G1 - G0;         // groups per halo row
    static constexpr int MA = M % 4;           // halo column 0 in an Sz row
    static constexpr int CB = EA - 4;          // 0 (FP32) or 4 (FP16)
    static constexpr int RO = (4 * G0 - 4) % EA;
    static constexpr int BWR = cround(4 * NG + RO, EA);     // reference box width (elements)
    static constexpr int BWC = cround(4 * (G1 + R) + CB, EA);  // candidate box width
    static constexpr int PSZ = ((4 * NG) % 8 == 4) ? 4 * NG : 4 * NG + 4;  // Sz pitch, PSZ/4 odd
    static constexpr int PSX = 36;             // Sx row pitch (32 used), PSX/4 odd
    static constexpr int THREADS = 512;
    static constexpr int NA = 16 * HY;         // stage A threads (16 per halo row, NG used)
    static constexpr int NB = K * HY;          // stage B items (k, halo row)
    static constexpr int NC = K * CX;          // stage C items (k, column)
    static constexpr int REF_TX = BWR * HY * ES;   // bytes of a reference plane box
    static constexpr int CAND_TX = BWC * HY * ES;  // bytes of a candidate plane box
    static constexpr int REF_SLOT = cround(REF_TX, 128);
    static constexpr int CAND_SLOT = cround(CAND_TX, 128);
    static constexpr int DC_TX = BWC * CY * ES;    // bytes of a stage-D candidate box (CY rows)
    static constexpr int DC_SLOT = cround(DC_TX, 128);
    static constexpr int ABUF = 2 * REF_SLOT + 2 * CAND_SLOT;  // entering/leaving ref + cand
    static constexpr int SZ_OFF = 0;
    static constexpr int SX_OFF = SZ_OFF + cround(K * HY * PSZ * 4, 128);
    static constexpr int A_OFF = SX_OFF + cround(K * HY * PSX * 4, 128);
    static constexpr int D_OFF = A_OFF + 2 * ABUF;
    static constexpr int BAR_OFF = D_OFF + 2 * DC_SLOT;
    static constexpr int SMEM_BYTES = BAR_OFF + 64;
    static_assert(M >= 1 && N >= 1, "radii");
    static_assert(NG <= 16 && NA <= THREADS && NB <= THREADS && NC <= THREADS,
                  "one item per thread");
    static_assert(CX == 32 && CY == 16, "stage B/C split outputs into two runs");
    static_assert(CX * CY == THREADS, "one stage-D voxel per thread");
    static_assert(4 * R >= M, "candidate window covers the x offsets");
    static_assert(4 * NG >= MA + HX, "Sz row covers the halo");
    static_assert(BWC <= 256 && BWR <= 256 && HY <= 256, "TMA box dimension > 256");
    static_assert(CB + 4 + N + 31 + 2 * M < BWC, "stage D candidates inside the box");
    static_assert((BWR * ES) % 16 == 0 && (BWC * ES) % 16 == 0, "TMA box rows of 16-byte units");
    static_assert(SMEM_BYTES <= 227 * 1024, "shared memory");
};

// Geometry of one launch (all CTAs): tensor maps + extents + pass/step counts.
struct LpArgs {
    int X, Y, Z;
    int TZ;           // planes per chunk
    int zc0;          // first chunk of this launch
    int nzc;          // chunks in this launch (grid z = nzc * nsplit)
    int nsplit;       // 1: a CTA makes every pass; 2: each half of the passes
    size_t part_stride;  // float2 pairs per accumulator buffer (X * Y * Z)
    float inv_scale;
    void* acc;        // [nsplit][Z][Y][X] of (Z, num) float2, or (Z, num, cZ, cnum) float4
                      // for the FP16-storage form
    float* out;
    float* zsum;
    unsigned int* errword;
};

// Four consecutive staged elements (8 bytes of FP16 or 16 of FP32) as FP32.
__device__ __forceinline__ float4 load4(const float* p) { return *reinterpret_cast<const float4*>(p); }
__device__ __forceinline__ float4 load4(const __half* p) {
    const uint2 u = *reinterpret_cast<const uint2*>(p);
    const float2 lo = __half22float2(*reinterpret_cast<const __half2*>(&u.x));
    const float2 hi = __half22float2(*reinterpret_cast<const __half2*>(&u.y));
    return make_float4(lo.x, lo.y, hi.x, hi.y);
}

// Adds a pass's (Z, num) increment to a Kahan pair (sum, compensation) per component.
__device__ __forceinline__ float4 kahan_step(float4 acc, float dz, float dn) {
    const float yz = dz - acc.z, yn = dn - acc.w;
    const float tz = acc.x + yz, tn = acc.y + yn;
    return make_float4(tz, tn, (tz - acc.x) - yz, (tn - acc.y) - yn);
}

template <int M, int N, typename Elem>
__global__ void __launch_bounds__(512, 1)
    nlm3d_lp_kernel(const __grid_constant__ CUtensorMap mapR,
                    const __grid_constant__ CUtensorMap mapC,
                    const __grid_constant__ CUtensorMap mapD, const LpArgs a) {
    using C = Lp3d<M, N, Elem>;
    extern __shared__ __align__(128) unsigned char smem[];
    float* Szb = reinterpret_cast<float*>(smem + C::SZ_OFF);
    float* Sxb = reinterpret_cast<float*>(smem + C::SX_OFF);
    uint64_t* barA = reinterpret_cast<uint64_t*>(smem + C::BAR_OFF);
    uint64_t* barD = barA + 2;
    __shared__ int s_abort;

    const int tid = threadIdx.x;
    const int X0 = blockIdx.x * C::CX, Y0 = blockIdx.y * C::CY;
    const int chunk = blockIdx.z % a.nzc, part = blockIdx.z / a.nzc;
    const int Z0 = (chunk + a.zc0) * a.TZ;
    const int TZc = min(a.TZ, a.Z - Z0);
    if (TZc <= 0) return;  // uniform over the CTA
    // This CTA's passes [pb, pb + P) of the (2sr+1)^2, and its accumulator buffer.
    const int pb = part * (C::K * C::K) / a.nsplit;
    const int P = (part + 1) * (C::K * C::K) / a.nsplit - pb;
    float2* const acc = static_cast<float2*>(a.acc) + part * a.part_stride;
    float4* const acck = static_cast<float4*>(a.acc) + part * a.part_stride;
    // A pass is N warm-up steps, each adding two planes of the first window
    // (padded planes Z0+M .. Z0+M+2N-1), then TZc output steps: output plane
    // Z0+q adds padded plane Z0+M+2N+q and, for q >= 1, drops Z0+M+q-1.
    const int SPP = N + TZc;
    const int T = P * SPP;      // steps
    const int TD = P * TZc;     // output steps

    auto abuf = [&](int b) { return smem + C::A_OFF + b * C::ABUF; };
    auto dbuf = [&](int b) { return smem + C::D_OFF + b * C::DC_SLOT; };

    // Thread 0: loads of step t's planes into A buffer t&1 (slot 0: the entering
    // plane, slot 1: the second warm-up plane or the leaving plane).
    auto issueA = [&](int t) {
        const int b = t & 1, lp = t / SPP, s = t - lp * SPP, pass = pb + lp;
        const int oz = pass / C::K - M, oy = pass % C::K - M;
        int p0, p1 = -1;
        if (s < N) {
            p0 = Z0 + M + 2 * s;
            p1 = p0 + 1;
        } else {
            const int q = s - N;
            p0 = Z0 + M + 2 * N + q;
            if (q >= 1) p1 = Z0 + M + q - 1;
        }
        unsigned char* base = abuf(b);
        const int xr = X0 - 4 + 4 * C::G0, yr = Y0 + M;
        fence_proxy_async_smem();
        mbar_arrive_expect_tx(&barA[b], (p1 >= 0 ? 2u : 1u) * (C::REF_TX + C::CAND_TX));
        tma_load_3d(base, &mapR, xr - C::RO, yr, p0, &barA[b]);
        tma_load_3d(base + 2 * C::REF_SLOT, &mapC, X0 - 4 - C::CB, yr + oy, p0 + oz, &barA[b]);
        if (p1 >= 0) {
            tma_load_3d(base + C::REF_SLOT, &mapR, xr - C::RO, yr, p1, &barA[b]);
            tma_load_3d(base + 2 * C::REF_SLOT + C::CAND_SLOT, &mapC, X0 - 4 - C::CB, yr + oy,
                        p1 + oz, &barA[b]);
        }
    };
    // Thread 0: the candidate plane of output step d (stage D's centre values: the CY
    // output rows only, shifted by oy).
    auto issueD = [&](int d) {
        const int b = d & 1, lp = d / TZc, q = d - lp * TZc, pass = pb + lp;
        const int oz = pass / C::K - M, oy = pass % C::K - M;
        fence_proxy_async_smem();
        mbar_arrive_expect_tx(&barD[b], C::DC_TX);
        tma_load_3d(dbuf(b), &mapD, X0 - 4 - C::CB, Y0 + C::H + oy, Z0 + q + C::H + oz, &barD[b]);
    };

    if (tid == 0) {
        for (int i = 0; i < 4; ++i) mbar_init(&barA[i], 1);
        fence_mbar_init();
        s_abort = 0;
    }
    __syncthreads();
    int lastA = 0, lastD = 0;  // thread 0: latest step whose loads were issued
    if (tid == 0) {
        issueA(0);
        issueD(0);
    }

    // Stage A ownership: 16 lanes per halo row (conflict-free shared loads), lane
    // gi < NG owns columns 4*(G0+gi) .. +3 of the box.
    const int gi = tid & 15, ya = tid >> 4;
    bool hasA = gi < C::NG && ya < C::HY;
    // Stages B-D own fixed items too; a thread whose ranges leave their buffers
    // (possible only through a defect, caught by NLM_BOUNDS_CHECK builds) skips its work.
    // Items fill whole warps (shared-memory wavefronts are counted per warp access, so
    // spreading them over more, partly filled warps costs bandwidth).
    bool okB = tid < C::NB, okC = tid < C::NC, okD = true;
    if constexpr (kBoundsCheck) {
        const long long szn = (long long)C::K * C::HY * C::PSZ, sxn = (long long)C::K * C::HY * C::PSX;
        if (hasA) {
            const int g = C::G0 + gi;
            hasA = range_ok(a.errword, ya * C::BWR + 4 * gi + C::RO,
                            ya * C::BWR + 4 * gi + C::RO + 3, C::REF_TX / C::ES) &&
                   range_ok(a.errword, ya * C::BWC + 4 * (g - C::R) + C::CB,
                            ya * C::BWC + 4 * (g + C::R) + C::CB + 3, C::CAND_TX / C::ES) &&
                   range_ok(a.errword, ya * C::PSZ + 4 * gi,
                            ((C::K - 1) * C::HY + ya) * C::PSZ + 4 * gi + 3, szn);
        }
        if (okB) {
            const int k = tid / C::HY, yh = tid - k * C::HY;
            constexpr int NV = (C::MA + C::HX + 3) / 4;
            okB = range_ok(a.errword, (k * C::HY + yh) * C::PSZ,
                           (k * C::HY + yh) * C::PSZ + 4 * NV - 1, szn) &&
                  range_ok(a.errword, (k * C::HY + yh) * C::PSX,
                           (k * C::HY + yh) * C::PSX + C::CX - 1, sxn);
        }
        if (okC) {
            const int k = tid >> 5, j = tid & 31;
            okC = range_ok(a.errword, k * C::HY * C::PSX + j,
                           k * C::HY * C::PSX + j + (C::HY - 1) * C::PSX, sxn);
        }
        const int y = tid >> 5, j = tid & 31;
        okD = range_ok(a.errword, y * C::PSX + j, ((C::K - 1) * C::HY + y) * C::PSX + j, sxn) &&
              range_ok(a.errword, y * C::BWC + 4 + N + j + C::CB,
                       y * C::BWC + 4 + N + j + C::CB + C::K - 1, C::DC_TX / C::ES);
    }
    float Sz[C::K][4];

    int d = 0;  // output steps done
    for (int t = 0; t < T; ++t) {
        const int pass = t / SPP, s = t - pass * SPP;
        if (tid == 0 && t + 1 < T) issueA(lastA = t + 1);
        if (s == 0) {
#pragma unroll
            for (int k = 0; k < C::K; ++k)
#pragma unroll
                for (int c = 0; c < 4; ++c) Sz[k][c] = 0.f;
        }
        const bool out_step = s >= N;
        // Stage D's partial sums of this voxel from earlier passes, requested now so
        // the load overlaps stages A-C.
        const int vy = tid >> 5, vj = tid & 31;
        const int vx = X0 + vj, vyy = Y0 + vy, vz = Z0 + (s - N);
        const bool vin = out_step && vx < a.X && vyy < a.Y;
        const size_t vo = ((size_t)vz * a.Y + vyy) * a.X + vx;
        float2 prev = make_float2(0.f, 0.f);
        float4 prevk = make_float4(0.f, 0.f, 0.f, 0.f);
        if (vin && pass > 0) {
            if constexpr (C::KAHAN)
                prevk = acck[vo];
            else
                prev = acc[vo];
        }
        const int b = t & 1;
        const bool okA = mbar_wait_bounded(&barA[b], (t >> 1) & 1);
        if (!okA) {
            raise_device_error(a.errword, DEVERR_TMA_TIMEOUT);
            s_abort = 1;
        }
        if (okA && hasA) {
            const Elem* ref0 = reinterpret_cast<const Elem*>(abuf(b)) + C::RO;
            const Elem* ref1 = ref0 + C::REF_SLOT / C::ES;
            const Elem* cand0 = reinterpret_cast<const Elem*>(abuf(b) + 2 * C::REF_SLOT) + C::CB;
            const Elem* cand1 = cand0 + C::CAND_SLOT / C::ES;
            const int g = C::G0 + gi;
            const float4 a0 = load4(ref0 + ya * C::BWR + 4 * gi);
            const float av[4] = {a0.x, a0.y, a0.z, a0.w};
            float c0[4 * (2 * C::R + 1)];
#pragma unroll
            for (int r = 0; r <= 2 * C::R; ++r)
                *reinterpret_cast<float4*>(&c0[4 * r]) = load4(cand0 + ya * C::BWC + 4 * (g - C::R + r));
            if (s != N) {
                // second plane: added (warm-up) or dropped (leaving)
                const float4 a1 = load4(ref1 + ya * C::BWR + 4 * gi);
                const float lv[4] = {a1.x, a1.y, a1.z, a1.w};
                float c1[4 * (2 * C::R + 1)];
#pragma unroll
                for (int r = 0; r <= 2 * C::R; ++r)
                    *reinterpret_cast<float4*>(&c1[4 * r]) =
                        load4(cand1 + ya * C::BWC + 4 * (g - C::R + r));
                if (s < N) {
#pragma unroll
                    for (int k = 0; k < C::K; ++k)
#pragma unroll
                        for (int c = 0; c < 4; ++c) {
                            const int i = 4 * C::R + c + k - M;
                            const float de = av[c] - c0[i];
                            const float dl = lv[c] - c1[i];
                            Sz[k][c] = fmaf(dl, dl, fmaf(de, de, Sz[k][c]));
                        }
                } else {
#pragma unroll
                    for (int k = 0; k < C::K; ++k)
#pragma unroll
                        for (int c = 0; c < 4; ++c) {
                            const int i = 4 * C::R + c + k - M;
                            const float de = av[c] - c0[i];
                            const float dl = lv[c] - c1[i];
                            Sz[k][c] = fmaf(-dl, dl, fmaf(de, de, Sz[k][c]));
                        }
                }
            } else {
#pragma unroll
                for (int k = 0; k < C::K; ++k)
#pragma unroll
                    for (int c = 0; c < 4; ++c) {
                        const float de = av[c] - c0[4 * C::R + c + k - M];
                        Sz[k][c] = fmaf(de, de, Sz[k][c]);
                    }
            }
            if (out_step) {
#pragma unroll
                for (int k = 0; k < C::K; ++k)
                    *reinterpret_cast<float4*>(Szb + (k * C::HY + ya) * C::PSZ + 4 * gi) =
                        make_float4(Sz[k][0], Sz[k][1], Sz[k][2], Sz[k][3]);
            }
        }
        __syncthreads();  // Sz rows written; step t's A buffer free
        if (s_abort) break;
        if (!out_step) continue;
        if (tid == 0 && d + 1 < TD) issueD(lastD = d + 1);

        // B: x box sums along halo rows, two independent running sums of 16 outputs.
        if (okB) {
            const int k = tid / C::HY, yh = tid - k * C::HY;
            const float* row = Szb + (k * C::HY + yh) * C::PSZ;
            constexpr int NV = (C::MA + C::HX + 3) / 4;
            float v[4 * NV];
#pragma unroll
            for (int q = 0; q < NV; ++q)
                *reinterpret_cast<float4*>(&v[4 * q]) = *reinterpret_cast<const float4*>(row + 4 * q);
            float o[C::CX];
            float acc[2];
#pragma unroll
            for (int sg = 0; sg < 2; ++sg) {
                acc[sg] = 0.f;
#pragma unroll
                for (int x = 0; x <= 2 * N; ++x) acc[sg] += v[C::MA + 16 * sg + x];
                o[16 * sg] = acc[sg];
            }
#pragma unroll
            for (int j = 1; j < 16; ++j)
#pragma unroll
                for (int sg = 0; sg < 2; ++sg) {
                    const int jj = 16 * sg + j;
                    acc[sg] += v[C::MA + jj + 2 * N] - v[C::MA + jj - 1];
                    o[jj] = acc[sg];
                }
            float* sx = Sxb + (k * C::HY + yh) * C::PSX;
#pragma unroll
            for (int q = 0; q < C::CX / 4; ++q)
                *reinterpret_cast<float4*>(sx + 4 * q) =
                    make_float4(o[4 * q], o[4 * q + 1], o[4 * q + 2], o[4 * q + 3]);
        }
        __syncthreads();
        // C: y box sums down output columns, in place (row y of the column becomes D),
        // two independent running sums of 8 outputs.
        if (okC) {
            const int k = tid >> 5, j = tid & 31;
            float* col = Sxb + k * C::HY * C::PSX + j;
            float u[C::HY];
#pragma unroll
            for (int yh = 0; yh < C::HY; ++yh) u[yh] = col[yh * C::PSX];
            float acc[2];
#pragma unroll
            for (int sg = 0; sg < 2; ++sg) {
                acc[sg] = 0.f;
#pragma unroll
                for (int y = 0; y <= 2 * N; ++y) acc[sg] += u[8 * sg + y];
                col[8 * sg * C::PSX] = acc[sg];
            }
#pragma unroll
            for (int y = 1; y < 8; ++y)
#pragma unroll
                for (int sg = 0; sg < 2; ++sg) {
                    const int yy = 8 * sg + y;
                    acc[sg] += u[yy + 2 * N] - u[yy - 1];
                    col[yy * C::PSX] = acc[sg];
                }
        }
        __syncthreads();
        // D: weights and accumulation for voxel (X0 + j, Y0 + y, z).
        {
            const int db = d & 1;
            const bool okDw = mbar_wait_bounded(&barD[db], (d >> 1) & 1);
            if (!okDw) {
                raise_device_error(a.errword, DEVERR_TMA_TIMEOUT);
                s_abort = 1;
            } else if (okD) {
                const int y = vy, j = vj;
                const Elem* cpl =
                    reinterpret_cast<const Elem*>(dbuf(db)) + y * C::BWC + 4 + N + j + C::CB;
                float zl[2] = {0.f, 0.f}, nl[2] = {0.f, 0.f};
#pragma unroll
                for (int k = 0; k < C::K; ++k) {
                    const float w = ex2_neg(Sxb[(k * C::HY + y) * C::PSX + j]);
                    zl[k & 1] += w;
                    nl[k & 1] = fmaf(w, to_f32(cpl[k]), nl[k & 1]);
                }
                if (vin) {
                    float zt, nt;
                    float4 nk;
                    if constexpr (C::KAHAN) {
                        nk = kahan_step(prevk, zl[0] + zl[1], nl[0] + nl[1]);
                        zt = nk.x;
                        nt = nk.y;
                    } else {
                        zt = prev.x + (zl[0] + zl[1]);
                        nt = prev.y + (nl[0] + nl[1]);
                    }
                    if (pass == P - 1 && a.nsplit == 1) {
                        a.out[vo] = nt / zt * a.inv_scale;
                        if (a.zsum) a.zsum[vo] = zt;
                    } else if constexpr (C::KAHAN) {
                        acck[vo] = nk;
                    } else {
                        acc[vo] = make_float2(zt, nt);
                    }
                }
            }
        }
        ++d;
    }
    if (tid == 0 && s_abort) {
        // Let the copies still in flight land before the CTA exits (bounded).
        mbar_wait_bounded(&barA[lastA & 1], (lastA >> 1) & 1);
        mbar_wait_bounded(&barD[lastD & 1], (lastD >> 1) & 1);
    }
}

// The x-offset halves.  Each CTA takes half of a pass's x offsets (half 0: ox = -M..0,
// half 1: ox = 1..M) of the same column tile and chunk, which halves the z sums a stage-A
// thread keeps per halo row (two rows per thread fit) and the shared buffer that hands
// them to stage B.  That room goes to a taller tile: 48 output rows under 64 halo rows
// (512 threads, one CTA per SM) or 32 under 48 (384 threads), against the one-CTA
// kernel's 16 under 32; a 16-row tile (256 threads) fits two CTAs per SM instead, so one
// runs its stages while the other waits at a barrier.  Stage B writes its x sums in place
// over the Sz row it read (no separate Sx buffer), the candidate plane boxes cover only
// the half's window, and every CTA accumulates into its own (Z, num) buffer: part
// 2 * (pass half) + (x half), added in that order by lp_combine_kernel.
template <int M, int N, typename T, int CYT = 16>
struct Lpx3d {
    using G = Lp3d<M, N, T>;
    static constexpr int ES = G::ES, EA = G::EA, K = G::K, CX = G::CX, H = G::H;
    static constexpr int HX = G::HX, R = G::R, G0 = G::G0, NG = G::NG, MA = G::MA;
    static constexpr int PSZ = G::PSZ, BWR = G::BWR, RO = G::RO, BWC = G::BWC, CB = G::CB;
    static constexpr bool KAHAN = G::KAHAN;
    static constexpr int CY = CYT;             // output rows per tile (16 or 32)
    static constexpr int HY = CY + 2 * N;      // halo rows
    static constexpr int KH = M + 1;           // x offsets of half 0 (half 1 has M)
    static constexpr int THREADS = CY == 16 ? 256 : (CY == 32 ? 384 : 512);
    static constexpr int RS = THREADS / 16;    // stage-A row slots: rows ya and ya + RS
    static constexpr int ND = (CX * CY + THREADS - 1) / THREADS;  // stage-D voxels per thread
    static constexpr int MINB = CY == 16 ? 2 : 1;                 // CTAs per SM
    static constexpr int WG = NG + R;          // 4-column groups of a half's candidate box
    // Half h's candidate box starts at layout group h ? G0 : G0 - R; FP16 boxes start on a
    // 16-byte (8-element) boundary, 4 elements early when that group is even.
    static constexpr int CB0 = ES == 2 && (G0 - R) % 2 == 0 ? 4 : 0;
    static constexpr int CB1 = ES == 2 && G0 % 2 == 0 ? 4 : 0;
    static constexpr int BWH = cround(4 * WG + (ES == 2 ? 4 : 0), EA);  // half box width
    static constexpr int REF_TX = BWR * HY * ES;
    static constexpr int CAND_TX = BWH * HY * ES;
    static constexpr int REF_SLOT = cround(REF_TX, 128);
    static constexpr int CAND_SLOT = cround(CAND_TX, 128);
    static constexpr int DC_TX = BWC * CY * ES;  // stage-D candidates: the full window
    static constexpr int DC_SLOT = cround(DC_TX, 128);
    static constexpr int ABUF = 2 * REF_SLOT + 2 * CAND_SLOT;
    static constexpr int SZ_OFF = 0;
    static constexpr int A_OFF = cround(KH * HY * PSZ * 4, 128);
    static constexpr int NDB = CY >= 48 ? 1 : 2;  // stage-D candidate buffers
    static constexpr int D_OFF = A_OFF + 2 * ABUF;
    static constexpr int BAR_OFF = D_OFF + NDB * DC_SLOT;
    static constexpr int SMEM_BYTES = BAR_OFF + 64;
    static_assert(HY <= 2 * RS, "stage A: two halo rows per thread");
    static_assert(KH * HY <= THREADS && KH * CX <= THREADS, "one stage B / C item per thread");
    static_assert(THREADS % 32 == 0 && CY % 2 == 0, "stage D: whole warps, two y chains");
    static_assert(4 * WG + CB0 <= BWH && 4 * WG + CB1 <= BWH, "half box");
    static_assert(BWH <= 256 && (BWH * ES) % 16 == 0 && HY <= 256, "TMA box");
    static_assert((SMEM_BYTES + 1024) * MINB <= 228 * 1024, "CTAs per SM");
};

template <int M, int N, typename Elem, int HALF, int CYT>
__device__ __forceinline__ void lpx_body(const CUtensorMap* mapR, const CUtensorMap* mapC,
                                         const CUtensorMap* mapD, const LpArgs& a,
                                         unsigned char* smem, int chunk, int part) {
    using C = Lpx3d<M, N, Elem, CYT>;
    constexpr int KL = HALF ? M : M + 1;          // x offsets of this half
    constexpr int KB = HALF ? M + 1 : 0;          // ox + M of the half's first x offset
    constexpr int OG = HALF ? C::G0 : C::G0 - C::R;  // candidate box origin (layout group)
    constexpr int CBh = HALF ? C::CB1 : C::CB0;
    constexpr int IB = HALF ? 1 : 4 * C::R - M;   // window index of (column 0, offset 0)
    float* Szb = reinterpret_cast<float*>(smem + C::SZ_OFF);
    uint64_t* barA = reinterpret_cast<uint64_t*>(smem + C::BAR_OFF);
    uint64_t* barD = barA + 2;
    __shared__ int s_abort;

    const int tid = threadIdx.x;
    const int X0 = blockIdx.x * C::CX, Y0 = blockIdx.y * C::CY;
    const int Z0 = (chunk + a.zc0) * a.TZ;
    const int TZc = min(a.TZ, a.Z - Z0);
    if (TZc <= 0) return;  // uniform over the CTA
    const int sp = part >> 1;  // pass half
    const int pb = sp * (C::K * C::K) / a.nsplit;
    const int P = (sp + 1) * (C::K * C::K) / a.nsplit - pb;
    float2* const acc = static_cast<float2*>(a.acc) + part * a.part_stride;
    float4* const acck = static_cast<float4*>(a.acc) + part * a.part_stride;
    const int SPP = N + TZc;
    const int T = P * SPP;
    const int TD = P * TZc;

    auto abuf = [&](int b) { return smem + C::A_OFF + b * C::ABUF; };
    auto dbuf = [&](int b) { return smem + C::D_OFF + (C::NDB == 1 ? 0 : b) * C::DC_SLOT; };
    // Thread 0: loads of step t's planes (as in nlm3d_lp_kernel; candidates: the half's box).
    auto issueA = [&](int t) {
        const int b = t & 1, lp = t / SPP, s = t - lp * SPP, pass = pb + lp;
        const int oz = pass / C::K - M, oy = pass % C::K - M;
        int p0, p1 = -1;
        if (s < N) {
            p0 = Z0 + M + 2 * s;
            p1 = p0 + 1;
        } else {
            const int q = s - N;
            p0 = Z0 + M + 2 * N + q;
            if (q >= 1) p1 = Z0 + M + q - 1;
        }
        unsigned char* base = abuf(b);
        const int xr = X0 - 4 + 4 * C::G0, yr = Y0 + M, xc = X0 - 4 + 4 * OG - CBh;
        fence_proxy_async_smem();
        mbar_arrive_expect_tx(&barA[b], (p1 >= 0 ? 2u : 1u) * (C::REF_TX + C::CAND_TX));
        tma_load_3d(base, mapR, xr - C::RO, yr, p0, &barA[b]);
        tma_load_3d(base + 2 * C::REF_SLOT, mapC, xc, yr + oy, p0 + oz, &barA[b]);
        if (p1 >= 0) {
            tma_load_3d(base + C::REF_SLOT, mapR, xr - C::RO, yr, p1, &barA[b]);
            tma_load_3d(base + 2 * C::REF_SLOT + C::CAND_SLOT, mapC, xc, yr + oy, p1 + oz,
                        &barA[b]);
        }
    };
    // Thread 0: stage D's candidate plane of output step d (CY rows, full x window).
    auto issueD = [&](int d) {
        const int b = C::NDB == 1 ? 0 : d & 1, lp = d / TZc, q = d - lp * TZc, pass = pb + lp;
        const int oz = pass / C::K - M, oy = pass % C::K - M;
        fence_proxy_async_smem();
        mbar_arrive_expect_tx(&barD[b], C::DC_TX);
        tma_load_3d(dbuf(b), mapD, X0 - 4 - C::CB, Y0 + C::H + oy, Z0 + q + C::H + oz, &barD[b]);
    };

    if (tid == 0) {
        for (int i = 0; i < 4; ++i) mbar_init(&barA[i], 1);
        fence_mbar_init();
        s_abort = 0;
    }
    __syncthreads();
    int lastA = 0, lastD = 0;
    if (tid == 0) {
        issueA(0);
        issueD(0);
    }

    // Stage A: 16 lanes per halo row, lane gi < NG owns columns 4*(G0+gi) .. +3 of rows
    // ya0 and ya0 + RS.
    const int gi = tid & 15, ya0 = tid >> 4;
    bool hasA[2];
#pragma unroll
    for (int r = 0; r < 2; ++r) hasA[r] = gi < C::NG && ya0 + C::RS * r < C::HY;
    bool okB = tid < KL * C::HY, okC = tid < KL * C::CX, okD = true;
    if constexpr (kBoundsCheck) {
        const long long szn = (long long)KL * C::HY * C::PSZ;
#pragma unroll
        for (int r = 0; r < 2; ++r)
            if (hasA[r]) {
                const int ya = ya0 + C::RS * r;
                hasA[r] = range_ok(a.errword, ya * C::BWR + 4 * gi + C::RO,
                                   ya * C::BWR + 4 * gi + C::RO + 3, C::REF_TX / C::ES) &&
                          range_ok(a.errword, ya * C::BWH + 4 * gi + CBh,
                                   ya * C::BWH + 4 * (gi + C::R) + CBh + 3, C::CAND_TX / C::ES) &&
                          range_ok(a.errword, ya * C::PSZ + 4 * gi,
                                   ((KL - 1) * C::HY + ya) * C::PSZ + 4 * gi + 3, szn);
            }
        if (okB) {
            constexpr int NV = (C::MA + C::HX + 3) / 4;
            okB = range_ok(a.errword, tid * C::PSZ, tid * C::PSZ + 4 * NV - 1, szn);
        }
        if (okC) {
            const int k = tid >> 5, j = tid & 31;
            okC = range_ok(a.errword, k * C::HY * C::PSZ + j,
                           k * C::HY * C::PSZ + j + (C::HY - 1) * C::PSZ, szn);
        }
        const int y = tid >> 5, j = tid & 31, yl = min(C::CY - 1, y + (C::ND - 1) * (C::THREADS / 32));
        okD = range_ok(a.errword, y * C::PSZ + j, ((KL - 1) * C::HY + yl) * C::PSZ + j, szn) &&
              range_ok(a.errword, y * C::BWC + 4 + N + j + C::CB + KB,
                       yl * C::BWC + 4 + N + j + C::CB + KB + KL - 1, C::DC_TX / C::ES);
    }
    float Sz[2][KL][4];

    int d = 0;
    for (int t = 0; t < T; ++t) {
        const int pass = t / SPP, s = t - pass * SPP;
        if (tid == 0 && t + 1 < T) issueA(lastA = t + 1);
        if (s == 0) {
#pragma unroll
            for (int r = 0; r < 2; ++r)
#pragma unroll
                for (int k = 0; k < KL; ++k)
#pragma unroll
                    for (int c = 0; c < 4; ++c) Sz[r][k][c] = 0.f;
        }
        const bool out_step = s >= N;
        // the thread's voxels' sums from earlier passes, requested early (voxel u: tile row
        // vy + u * THREADS / 32, column vj)
        const int vy = tid >> 5, vj = tid & 31;
        const int vx = X0 + vj, vz = Z0 + (s - N);
        size_t vo[C::ND];
        bool vin[C::ND];
        float2 prev[C::ND];
        float4 prevk[C::ND];
#pragma unroll
        for (int u = 0; u < C::ND; ++u) {
            const int vr = vy + u * (C::THREADS / 32), vyy = Y0 + vr;
            vin[u] = out_step && vr < C::CY && vx < a.X && vyy < a.Y;
            vo[u] = ((size_t)vz * a.Y + vyy) * a.X + vx;
            prev[u] = make_float2(0.f, 0.f);
            prevk[u] = make_float4(0.f, 0.f, 0.f, 0.f);
            if (vin[u] && pass > 0) {
                if constexpr (C::KAHAN)
                    prevk[u] = acck[vo[u]];
                else
                    prev[u] = acc[vo[u]];
            }
        }
        const int b = t & 1;
        const bool okA = mbar_wait_bounded(&barA[b], (t >> 1) & 1);
        if (!okA) {
            raise_device_error(a.errword, DEVERR_TMA_TIMEOUT);
            s_abort = 1;
        }
        if (okA) {
#pragma unroll
            for (int r = 0; r < 2; ++r) {
                if (!hasA[r]) continue;
                const int ya = ya0 + C::RS * r;
                const Elem* ref0 = reinterpret_cast<const Elem*>(abuf(b)) + C::RO;
                const Elem* ref1 = ref0 + C::REF_SLOT / C::ES;
                const Elem* cand0 = reinterpret_cast<const Elem*>(abuf(b) + 2 * C::REF_SLOT) + CBh;
                const Elem* cand1 = cand0 + C::CAND_SLOT / C::ES;
                const float4 a0 = load4(ref0 + ya * C::BWR + 4 * gi);
                const float av[4] = {a0.x, a0.y, a0.z, a0.w};
                float c0[4 * (C::R + 1)];
#pragma unroll
                for (int w = 0; w <= C::R; ++w)
                    *reinterpret_cast<float4*>(&c0[4 * w]) = load4(cand0 + ya * C::BWH + 4 * (gi + w));
                if (s != N) {
                    const float4 a1 = load4(ref1 + ya * C::BWR + 4 * gi);
                    const float lv[4] = {a1.x, a1.y, a1.z, a1.w};
                    float c1[4 * (C::R + 1)];
#pragma unroll
                    for (int w = 0; w <= C::R; ++w)
                        *reinterpret_cast<float4*>(&c1[4 * w]) =
                            load4(cand1 + ya * C::BWH + 4 * (gi + w));
                    if (s < N) {  // warm-up: both planes enter
#pragma unroll
                        for (int k = 0; k < KL; ++k)
#pragma unroll
                            for (int c = 0; c < 4; ++c) {
                                const float de = av[c] - c0[IB + c + k];
                                const float dl = lv[c] - c1[IB + c + k];
                                Sz[r][k][c] = fmaf(dl, dl, fmaf(de, de, Sz[r][k][c]));
                            }
                    } else {  // the second plane leaves
#pragma unroll
                        for (int k = 0; k < KL; ++k)
#pragma unroll
                            for (int c = 0; c < 4; ++c) {
                                const float de = av[c] - c0[IB + c + k];
                                const float dl = lv[c] - c1[IB + c + k];
                                Sz[r][k][c] = fmaf(-dl, dl, fmaf(de, de, Sz[r][k][c]));
                            }
                    }
                } else {
#pragma unroll
                    for (int k = 0; k < KL; ++k)
#pragma unroll
                        for (int c = 0; c < 4; ++c) {
                            const float de = av[c] - c0[IB + c + k];
                            Sz[r][k][c] = fmaf(de, de, Sz[r][k][c]);
                        }
                }
                if (out_step) {
#pragma unroll
                    for (int k = 0; k < KL; ++k)
                        *reinterpret_cast<float4*>(Szb + (k * C::HY + ya) * C::PSZ + 4 * gi) =
                            make_float4(Sz[r][k][0], Sz[r][k][1], Sz[r][k][2], Sz[r][k][3]);
                }
            }
        }
        __syncthreads();  // Sz rows written; step t's A buffer free
        if (s_abort) break;
        if (!out_step) continue;
        if constexpr (C::NDB == 2) {
            if (tid == 0 && d + 1 < TD) issueD(lastD = d + 1);
        } else {  // one buffer: step d's box, once stage D of step d - 1 is done (barrier above)
            if (tid == 0 && d >= 1) issueD(lastD = d);
        }

        // B: x box sums along a halo row, written over the first 32 floats of the same row
        // (the whole row is in registers first).
        if (okB) {
            float* row = Szb + tid * C::PSZ;
            constexpr int NV = (C::MA + C::HX + 3) / 4;
            float v[4 * NV];
#pragma unroll
            for (int q = 0; q < NV; ++q)
                *reinterpret_cast<float4*>(&v[4 * q]) = *reinterpret_cast<const float4*>(row + 4 * q);
            float o[C::CX];
            float run[2];
#pragma unroll
            for (int sg = 0; sg < 2; ++sg) {
                run[sg] = 0.f;
#pragma unroll
                for (int x = 0; x <= 2 * N; ++x) run[sg] += v[C::MA + 16 * sg + x];
                o[16 * sg] = run[sg];
            }
#pragma unroll
            for (int j = 1; j < 16; ++j)
#pragma unroll
                for (int sg = 0; sg < 2; ++sg) {
                    const int jj = 16 * sg + j;
                    run[sg] += v[C::MA + jj + 2 * N] - v[C::MA + jj - 1];
                    o[jj] = run[sg];
                }
#pragma unroll
            for (int q = 0; q < C::CX / 4; ++q)
                *reinterpret_cast<float4*>(row + 4 * q) =
                    make_float4(o[4 * q], o[4 * q + 1], o[4 * q + 2], o[4 * q + 3]);
        }
        __syncthreads();
        // C: y box sums down the output columns, in place (row y becomes D).
        if (okC) {
            const int k = tid >> 5, j = tid & 31;
            float* col = Szb + k * C::HY * C::PSZ + j;
            float u[C::HY];
#pragma unroll
            for (int yh = 0; yh < C::HY; ++yh) u[yh] = col[yh * C::PSZ];
            constexpr int HC = C::CY / 2;  // outputs per running sum
            float run[2];
#pragma unroll
            for (int sg = 0; sg < 2; ++sg) {
                run[sg] = 0.f;
#pragma unroll
                for (int y = 0; y <= 2 * N; ++y) run[sg] += u[HC * sg + y];
                col[HC * sg * C::PSZ] = run[sg];
            }
#pragma unroll
            for (int y = 1; y < HC; ++y)
#pragma unroll
                for (int sg = 0; sg < 2; ++sg) {
                    const int yy = HC * sg + y;
                    run[sg] += u[yy + 2 * N] - u[yy - 1];
                    col[yy * C::PSZ] = run[sg];
                }
        }
        __syncthreads();
        // D: weights and accumulation for the thread's voxels (X0 + j, Y0 + y, z).
        {
            const int db = C::NDB == 1 ? 0 : d & 1;
            const bool okDw = mbar_wait_bounded(&barD[db], C::NDB == 1 ? d & 1 : (d >> 1) & 1);
            if (!okDw) {
                raise_device_error(a.errword, DEVERR_TMA_TIMEOUT);
                s_abort = 1;
            } else if (okD) {
#pragma unroll
                for (int u = 0; u < C::ND; ++u) {
                    const int y = vy + u * (C::THREADS / 32), j = vj;
                    if (y >= C::CY) continue;
                    const Elem* cpl = reinterpret_cast<const Elem*>(dbuf(db)) + y * C::BWC + 4 + N +
                                      j + C::CB + KB;
                    float zl[2] = {0.f, 0.f}, nl[2] = {0.f, 0.f};
#pragma unroll
                    for (int k = 0; k < KL; ++k) {
                        const float w = ex2_neg(Szb[(k * C::HY + y) * C::PSZ + j]);
                        zl[k & 1] += w;
                        nl[k & 1] = fmaf(w, to_f32(cpl[k]), nl[k & 1]);
                    }
                    if (vin[u]) {
                        if constexpr (C::KAHAN) {
                            acck[vo[u]] = kahan_step(prevk[u], zl[0] + zl[1], nl[0] + nl[1]);
                        } else {
                            acc[vo[u]] = make_float2(prev[u].x + (zl[0] + zl[1]),
                                                     prev[u].y + (nl[0] + nl[1]));
                        }
                    }
                }
            }
        }
        ++d;
    }
    if (tid == 0 && s_abort) {
        mbar_wait_bounded(&barA[lastA & 1], (lastA >> 1) & 1);
        if constexpr (C::NDB == 1)
            mbar_wait_bounded(&barD[0], lastD & 1);
        else
            mbar_wait_bounded(&barD[lastD & 1], (lastD >> 1) & 1);
    }
}

template <int M, int N, typename Elem, int CYT>
__global__ void __launch_bounds__(Lpx3d<M, N, Elem, CYT>::THREADS, Lpx3d<M, N, Elem, CYT>::MINB)
    nlm3d_lpx_kernel(const __grid_constant__ CUtensorMap mapR,
                     const __grid_constant__ CUtensorMap mapC,
                     const __grid_constant__ CUtensorMap mapD, const LpArgs a) {
    extern __shared__ __align__(128) unsigned char smem[];
    const int chunk = blockIdx.z % a.nzc, part = blockIdx.z / a.nzc;  // part = 2 * split + half
    if (part & 1)
        lpx_body<M, N, Elem, 1, CYT>(&mapR, &mapC, &mapD, a, smem, chunk, part);
    else
        lpx_body<M, N, Elem, 0, CYT>(&mapR, &mapC, &mapD, a, smem, chunk, part);
}

// out = (num_0 + ... + num_{P-1}) / (Z_0 + ... + Z_{P-1}) over the voxels [v0, v0 + n) of
// P accumulator buffers (pass halves and x-offset halves), always added in buffer order.
// KAHAN: the buffers hold (Z, num, cZ, cnum) Kahan pairs; each contributes its sum minus
// its compensation.
template <bool KAHAN>
__global__ void __launch_bounds__(256) lp_combine_kernel(const void* __restrict__ accv,
                                                         size_t stride, int nparts, size_t v0,
                                                         size_t n, float inv_scale,
                                                         float* __restrict__ out,
                                                         float* __restrict__ zsum) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        const size_t v = v0 + i;
        float zt = 0.f, nt = 0.f;
        for (int p = 0; p < nparts; ++p) {
            if constexpr (KAHAN) {
                const float4 h = static_cast<const float4*>(accv)[p * stride + v];
                zt += h.x - h.z;
                nt += h.y - h.w;
            } else {
                const float2 h = static_cast<const float2*>(accv)[p * stride + v];
                zt += h.x;
                nt += h.y;
            }
        }
        out[v] = nt / zt * inv_scale;
        if (zsum) zsum[v] = zt;
    }
}

// Search radii that run the x-half form (nlm3d_lpx_kernel); the others keep every x
// offset of a pass in one CTA (nlm3d_lp_kernel).  Measured on 512 x 512 x 16 with 48-row
// x-half tiles against the one-CTA kernel: search 13 -10 to -22 %, search 11 -1 to -16 %,
// search 9 -4 to -14 %, search 7 -1 to -9 %; search 5 and 3 +1 to +2 % (with few x offsets,
// halving them halves the candidate windows' reuse).
template <int M>
constexpr bool kLpXHalf = M >= 3;
// Output rows per x-half tile: 48 (one CTA of 512 threads per SM, 64 halo rows for 48 output
// rows, one stage-D candidate buffer so that the plane boxes fit), the tallest tile whose
// FP32 buffers fit the shared memory.  At search 13, patch 17 on 512 x 512 x 128: 16-row
// tiles (two CTAs of 256 threads per SM) 207 ms, 32-row tiles (384 threads) 183 ms, 48-row
// tiles 167 ms.
constexpr int kLpXHalfRows = 48;

template <int M, int N, typename T>
inline cudaError_t run_lp(const Staging& st, const void* staged, int tz, float inv_scale,
                          float* out, float* zsum, void* acc, unsigned int* errword,
                          cudaStream_t stream, int zc0, int zc1) {
    using C = Lp3d<M, N, T>;
    if (st.elem != C::ES) return cudaErrorInvalidValue;
    CUtensorMap mapR, mapC, mapD;
    const uint64_t dims[3] = {(uint64_t)st.Xs, (uint64_t)st.Yp, (uint64_t)st.Zp};
    const uint64_t strides[2] = {(uint64_t)st.Xs * C::ES, (uint64_t)st.Xs * st.Yp * C::ES};
    const uint32_t boxR[3] = {(uint32_t)C::BWR, (uint32_t)C::HY, 1};
    const uint32_t boxC[3] = {(uint32_t)C::BWC, (uint32_t)C::HY, 1};
    const uint32_t boxD[3] = {(uint32_t)C::BWC, (uint32_t)C::CY, 1};
    void* base = const_cast<void*>(staged);
    cudaError_t e = encode_tensor_map(&mapR, C::ES == 2, 3, dims, strides, boxR, base);
    if (e == cudaSuccess) e = encode_tensor_map(&mapC, C::ES == 2, 3, dims, strides, boxC, base);
    if (e == cudaSuccess) e = encode_tensor_map(&mapD, C::ES == 2, 3, dims, strides, boxD, base);
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
    int nparts = nsplit;
    if constexpr (kLpXHalf<M>) {
        // CTAs with half of the x offsets each: parts 2 * split + half
        using X = Lpx3d<M, N, T, kLpXHalfRows>;
        const uint32_t boxRx[3] = {(uint32_t)X::BWR, (uint32_t)X::HY, 1};
        const uint32_t boxH[3] = {(uint32_t)X::BWH, (uint32_t)X::HY, 1};
        const uint32_t boxDx[3] = {(uint32_t)X::BWC, (uint32_t)X::CY, 1};
        e = encode_tensor_map(&mapR, X::ES == 2, 3, dims, strides, boxRx, base);
        if (e == cudaSuccess) e = encode_tensor_map(&mapC, X::ES == 2, 3, dims, strides, boxH, base);
        if (e == cudaSuccess) e = encode_tensor_map(&mapD, X::ES == 2, 3, dims, strides, boxDx, base);
        if (e != cudaSuccess) return e;
        auto kern = nlm3d_lpx_kernel<M, N, T, kLpXHalfRows>;
        e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, X::SMEM_BYTES);
        if (e != cudaSuccess) return e;
        nparts = 2 * nsplit;
        dim3 grid((st.X + X::CX - 1) / X::CX, (st.Y + X::CY - 1) / X::CY, (zc1 - zc0) * nparts);
        kern<<<grid, X::THREADS, X::SMEM_BYTES, stream>>>(mapR, mapC, mapD, a);
    } else {
        auto kern = nlm3d_lp_kernel<M, N, T>;
        e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM_BYTES);
        if (e != cudaSuccess) return e;
        dim3 grid((st.X + C::CX - 1) / C::CX, (st.Y + C::CY - 1) / C::CY, (zc1 - zc0) * nsplit);
        kern<<<grid, C::THREADS, C::SMEM_BYTES, stream>>>(mapR, mapC, mapD, a);
    }
    e = cudaGetLastError();
    if (e != cudaSuccess || nparts == 1) return e;
    const size_t plane = (size_t)st.X * st.Y;
    const size_t v0 = (size_t)zc0 * tz * plane;
    const size_t v1 = (size_t)std::min(zc1 * tz, st.Z) * plane;
    const size_t blocks = std::min<size_t>((v1 - v0 + 255) / 256, (size_t)device_sm_count() * 8);
    lp_combine_kernel<C::KAHAN><<<(unsigned)blocks, 256, 0, stream>>>(acc, a.part_stride, nparts,
                                                                      v0, v1 - v0, inv_scale,
                                                                      out, zsum);
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

// FP16-storage launches (nlm3d_lp_h.cu), one explicit instance per compiled pair.
template <int M, int N>
cudaError_t launch_lp_h(const Staging& st, const void* staged, int tz, float inv_scale, float* out,
                        float* zsum, void* acc, unsigned int* errword, cudaStream_t stream,
                        int zc0, int zc1);

}  // namespace gnlm
