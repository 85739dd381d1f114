// Large-patch 3D NLM forward (patch radius up to 8, search radius up to 6): the
// reference's NS = 7..17 configurations (3DNLM/main.cu:1005-7599, swept with
// SS 11/13 and NS 13/15/17 by 3DNLM/run.sh:25-34).
//
// The register-brick kernel (nlm3d_tile.cuh) recomputes a (RY+2pr) x (RZ+2pr)
// block of differences per offset and sums x by 2pr shuffles, so its cost grows
// with the patch; here every box sum is a running sum and the cost per (voxel,
// offset) does not depend on the patch width.
//
// A CTA owns a column tile of 32 x 48 output voxels (32 x 64 where the buffers fit), a
// chunk of TZ planes and, from search radius 3, one half of the x offsets (ox = -M..0
// or 1..M; below that every x offset).  It makes (2sr+1)^2 passes, one per (oz, oy); a pass streams the chunk's
// planes (plus the patch halo) in z, each step in four barrier-separated stages:
//   A  each thread owns 4 halo columns of two (or three) halo rows and keeps, per x offset, the
//      running z-sum Sz of squared differences over the 2pr+1 planes around the
//      current plane (add the entering plane, subtract the leaving one; the first
//      window is built two planes per step); the reference and candidate planes of
//      a step come in as TMA boxes (double-buffered, prefetched one step ahead), and
//      one 4-column candidate window serves all of the CTA's x offsets;
//   B  x box sum of Sz along each halo row (running sum), written over the row it read;
//   C  y box sum down each output column, in place (running sum) -> D;
//   D  w = 2^(-D) (the staging pass pre-scaled the volume so D is the base-2
//      exponent of exp(-(D/P)/h^2), 3DNLM/main.cu:108-109), Z += w, num += w v
//      over the CTA's x offsets, then one read-add-write of the voxel's (Z, num)
//      pair in the CTA's accumulator buffer (L2-resident: a chunk's pairs are re-read
//      once per pass, in pass order, so the sums are deterministic).
// A combine kernel adds the accumulator buffers (the x halves, and the two halves of
// the passes where the launcher splits them to fill the last wave) in a fixed order
// and writes out = num / Z (3DNLM/main.cu:125).

// Storage type T: float, or __half for the FP16-storage form (the staged volume and
// the TMA plane boxes hold FP16, halving their bytes; every difference, square and
// sum is FP32, and the per-pass weight sums are added across passes with Kahan
// compensation, the (Z, num) accumulator then holding (Z, num, cZ, cnum)).  TMA needs
// 16-byte aligned box starts and widths, so for FP16 each box starts on the 8-element
// boundary at or below its first 4-column group and the in-box column offsets (CB, RO,
// CB0, CB1) absorb that.
#pragma once

#include <algorithm>

#include "nlm3d_tile.cuh"
#include "nlm_device.cuh"
#include "nlm_internal.h"

namespace gnlm {

// Column geometry shared by the tile forms: 32 output columns per tile.
template <int M, int N, typename T>
struct Lp3d {
    static constexpr int ES = (int)sizeof(T);  // bytes per staged element
    static constexpr int EA = 16 / ES;         // elements per 16 bytes (TMA alignment)
    static constexpr bool KAHAN = ES == 2;     // FP16-storage form: compensated pass sums
    static constexpr int K = 2 * M + 1;        // x offsets per pass
    static constexpr int CX = 32;              // output columns per CTA
    static constexpr int H = M + N;
    static constexpr int HX = CX + 2 * N;      // halo columns
    // Column i of the 4-column group layout is padded column X0 - 4 + i (halo column
    // xh is i = 4 + M + xh).  Boxes start on 16-byte aligned columns: the stage-D
    // candidate box at padded column X0 - 4 - CB and the reference box at
    // X0 - 4 + 4*G0 - RO, so layout column i sits at candidate-box column i + CB.
    static constexpr int R = (M + 3) / 4;      // candidate 4-column groups either side
    static constexpr int G0 = 1 + M / 4;       // first 4-column group holding a halo column
    static constexpr int G1 = (4 + M + HX + 3) / 4;
    static constexpr int NG = G1 - G0;         // groups per halo row
    static constexpr int MA = M % 4;           // halo column 0 in an Sz row
    static constexpr int CB = EA - 4;          // 0 (FP32) or 4 (FP16)
    static constexpr int RO = (4 * G0 - 4) % EA;
    static constexpr int BWR = cround(4 * NG + RO, EA);     // reference box width (elements)
    static constexpr int BWC = cround(4 * (G1 + R) + CB, EA);  // stage-D candidate box width
    static constexpr int PSZ = ((4 * NG) % 8 == 4) ? 4 * NG : 4 * NG + 4;  // Sz pitch, PSZ/4 odd
    static_assert(M >= 1 && N >= 1, "radii");
    static_assert(NG <= 16, "16 lanes per halo row");
    static_assert(4 * R >= M, "candidate window covers the x offsets");
    static_assert(4 * NG >= MA + HX, "Sz row covers the halo");
    static_assert(BWC <= 256 && BWR <= 256, "TMA box dimension > 256");
    static_assert(CB + 4 + N + 31 + 2 * M < BWC, "stage D candidates inside the box");
    static_assert((BWR * ES) % 16 == 0 && (BWC * ES) % 16 == 0, "TMA box rows of 16-byte units");
};

// Geometry of one launch (all CTAs): tensor maps + extents + pass/step counts.
struct LpArgs {
    int X, Y, Z;
    int TZ;           // planes per chunk
    int zc0;          // first chunk of this launch
    int nzc;          // chunks in this launch (grid z = nzc * parts)
    int nsplit;       // 1: a CTA makes every pass; 2: each half of the passes
    size_t part_stride;  // accumulator elements per buffer (X * Y * Z)
    float inv_scale;
    void* acc;        // [parts][Z][Y][X] of (Z, num) float2, or (Z, num, cZ, cnum) float4
                      // for the FP16-storage form
    float* out;       // written by the combine kernel
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

// Tile layout.  From search radius 3 each CTA takes half of a pass's x offsets (XS = 2;
// half 0: ox = -M..0, half 1: ox = 1..M) of the same column tile and chunk, which halves
// the z sums a stage-A thread keeps per halo row so that two halo rows fit per thread, and
// halves the shared buffer that hands them to stage B; below that (2M + 1 <= 5) a CTA keeps
// every x offset (XS = 1).  The room goes to a tall tile: CY = 48 output rows under 64
// halo rows (512 threads, one CTA per SM).  Stage B writes its x sums in place over the Sz
// row it read, the candidate plane boxes cover only the CTA's window, and every CTA
// accumulates into its own (Z, num) buffer: part XS * (pass half) + (x half).  CY = 16
// (256 threads, two CTAs per SM) and 32 (384 threads) are the smaller layouts of the same
// code.
template <int M, int N, typename T, int CYT = 16, int XS = 2>
struct Lpx3d {
    using G = Lp3d<M, N, T>;
    static constexpr int ES = G::ES, EA = G::EA, K = G::K, CX = G::CX, H = G::H;
    static constexpr int HX = G::HX, R = G::R, G0 = G::G0, NG = G::NG, MA = G::MA;
    static constexpr int PSZ = G::PSZ, BWR = G::BWR, RO = G::RO, BWC = G::BWC, CB = G::CB;
    static constexpr bool KAHAN = G::KAHAN;
    static constexpr int CY = CYT;             // output rows per tile (16, 32 or 48)
    static constexpr int HY = CY + 2 * N;      // halo rows
    // XS = 2: x-offset halves (KH = M + 1 offsets for half 0, M for half 1); XS = 1: every
    // x offset in one CTA (the same tall-tile layout for small search radii)
    static constexpr int KH = XS == 2 ? M + 1 : 2 * M + 1;
    static constexpr int THREADS = CY == 16 ? 256 : (CY == 32 ? 384 : (CY == 48 ? 512 : 448));
    static constexpr int RS = THREADS / 16;    // stage-A row slots: rows ya + r * RS
    static constexpr int RA = (HY + RS - 1) / RS;  // halo rows per stage-A thread
    static constexpr int ND = (CX * CY + THREADS - 1) / THREADS;  // stage-D voxels per thread
    static constexpr int MINB = CY == 16 ? 2 : 1;                 // CTAs per SM
    static constexpr int WN = XS == 2 ? R + 1 : 2 * R + 1;  // candidate float4s per row
    static constexpr int WG = NG + WN - 1;     // 4-column groups of a candidate box
    // The candidate box starts at layout group G0 - R (half 0, or every x offset) or G0
    // (half 1); FP16 boxes start on a 16-byte (8-element) boundary, 4 elements early when
    // that group is even.
    static constexpr int CB0 = ES == 2 && (G0 - R) % 2 == 0 ? 4 : 0;
    static constexpr int CB1 = ES == 2 && G0 % 2 == 0 ? 4 : 0;
    static constexpr int BWH = cround(4 * WG + (ES == 2 ? 4 : 0), EA);  // candidate box width
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
    static constexpr int NB = KH * HY;         // stage-B items (offset, halo row)
    static constexpr int D_OFF = A_OFF + 2 * ABUF;
    static constexpr int BAR_OFF = D_OFF + NDB * DC_SLOT;
    static constexpr int SMEM_BYTES = BAR_OFF + 64;
    static_assert(RA <= 3, "stage A: at most three halo rows per thread");
    static_assert(KH * CX <= THREADS, "one stage C item per thread");
    static_assert(THREADS % 32 == 0 && CY % 2 == 0, "stage D: whole warps, two y chains");
    static_assert(4 * WG + CB0 <= BWH && 4 * WG + CB1 <= BWH, "candidate box");
    static_assert(BWH <= 256 && (BWH * ES) % 16 == 0 && HY <= 256, "TMA box");
    static_assert((SMEM_BYTES + 1024) * MINB <= 228 * 1024, "CTAs per SM");
};

// HALF: 0 or 1 for the x-offset halves (ox = -M..0, 1..M), 2 for every x offset.
template <int M, int N, typename Elem, int HALF, int CYT>
__device__ __forceinline__ void lpx_body(const CUtensorMap* mapR, const CUtensorMap* mapC,
                                         const CUtensorMap* mapD, const LpArgs& a,
                                         unsigned char* smem, int chunk, int part) {
    using C = Lpx3d<M, N, Elem, CYT, HALF == 2 ? 1 : 2>;
    constexpr int KL = HALF == 2 ? 2 * M + 1 : (HALF ? M : M + 1);  // x offsets of this CTA
    constexpr int KB = HALF == 1 ? M + 1 : 0;     // ox + M of the first x offset
    constexpr int OG = HALF == 1 ? C::G0 : C::G0 - C::R;  // candidate box origin (layout group)
    constexpr int CBh = HALF == 1 ? C::CB1 : C::CB0;
    constexpr int IB = HALF == 1 ? 1 : 4 * C::R - M;  // window index of (column 0, offset 0)
    constexpr int WN = C::WN;                     // candidate float4s per row
    float* Szb = reinterpret_cast<float*>(smem + C::SZ_OFF);
    uint64_t* barA = reinterpret_cast<uint64_t*>(smem + C::BAR_OFF);
    uint64_t* barD = barA + 2;
    __shared__ int s_abort;

    const int tid = threadIdx.x;
    const int X0 = blockIdx.x * C::CX, Y0 = blockIdx.y * C::CY;
    const int Z0 = (chunk + a.zc0) * a.TZ;
    const int TZc = min(a.TZ, a.Z - Z0);
    if (TZc <= 0) return;  // uniform over the CTA
    const int sp = HALF == 2 ? part : part >> 1;  // pass half
    const int pb = sp * (C::K * C::K) / a.nsplit;
    const int P = (sp + 1) * (C::K * C::K) / a.nsplit - pb;
    float2* const acc = static_cast<float2*>(a.acc) + part * a.part_stride;
    float4* const acck = static_cast<float4*>(a.acc) + part * a.part_stride;
    const int SPP = N + TZc;
    const int T = P * SPP;
    const int TD = P * TZc;

    // test builds: the CTA at grid origin arms its first plane copy without issuing it
    // (nlm_test_set_fault), so its first wait runs out after the short injected limit
    const bool skip = inject_skip_copy(a.errword, blockIdx.x, blockIdx.y, blockIdx.z);
    auto abuf = [&](int b) { return smem + C::A_OFF + b * C::ABUF; };
    auto dbuf = [&](int b) { return smem + C::D_OFF + (C::NDB == 1 ? 0 : b) * C::DC_SLOT; };
    // Thread 0: loads of step t's planes into A buffer t&1 (slot 0: the entering plane,
    // slot 1: the second warm-up plane or the leaving plane; candidates: the CTA's box).
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
        if (skip && t == 0) return;
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
    bool hasA[C::RA];
#pragma unroll
    for (int r = 0; r < C::RA; ++r) hasA[r] = gi < C::NG && ya0 + C::RS * r < C::HY;
    bool okB = true, okC = tid < KL * C::CX, okD = true;
    if constexpr (kBoundsCheck) {
        const long long szn = (long long)KL * C::HY * C::PSZ;
#pragma unroll
        for (int r = 0; r < C::RA; ++r)
            if (hasA[r]) {
                const int ya = ya0 + C::RS * r;
                hasA[r] = range_ok(a.errword, ya * C::BWR + 4 * gi + C::RO,
                                   ya * C::BWR + 4 * gi + C::RO + 3, C::REF_TX / C::ES) &&
                          range_ok(a.errword, ya * C::BWH + 4 * gi + CBh,
                                   ya * C::BWH + 4 * (gi + WN - 1) + CBh + 3, C::CAND_TX / C::ES) &&
                          range_ok(a.errword, ya * C::PSZ + 4 * gi,
                                   ((KL - 1) * C::HY + ya) * C::PSZ + 4 * gi + 3, szn);
            }
        {  // stage-B rows: items tid, tid + THREADS, ... < KL * HY
            constexpr int NV = (C::MA + C::HX + 3) / 4;
            const int last = tid + ((KL * C::HY - 1 - tid) / C::THREADS) * C::THREADS;
            if (tid < KL * C::HY)
                okB = range_ok(a.errword, tid * C::PSZ, last * C::PSZ + 4 * NV - 1, szn);
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
    float Sz[C::RA][KL][4];

    int d = 0;
    for (int t = 0; t < T; ++t) {
        const int pass = t / SPP, s = t - pass * SPP;
        if (tid == 0 && t + 1 < T) issueA(lastA = t + 1);
        if (s == 0) {
#pragma unroll
            for (int r = 0; r < C::RA; ++r)
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
        const bool okA = mbar_wait_bounded(&barA[b], (t >> 1) & 1,
                                           skip && t == 0 ? kInjectedWaitPolls : kMaxWaitPolls);
        if (!okA) {
            raise_device_error(a.errword, DEVERR_TMA_TIMEOUT);
            s_abort = 1;
        }
        if (okA) {
#pragma unroll
            for (int r = 0; r < C::RA; ++r) {
                if (!hasA[r]) continue;
                const int ya = ya0 + C::RS * r;
                const Elem* ref0 = reinterpret_cast<const Elem*>(abuf(b)) + C::RO;
                const Elem* ref1 = ref0 + C::REF_SLOT / C::ES;
                const Elem* cand0 = reinterpret_cast<const Elem*>(abuf(b) + 2 * C::REF_SLOT) + CBh;
                const Elem* cand1 = cand0 + C::CAND_SLOT / C::ES;
                const float4 a0 = load4(ref0 + ya * C::BWR + 4 * gi);
                const float av[4] = {a0.x, a0.y, a0.z, a0.w};
                float c0[4 * WN];
#pragma unroll
                for (int w = 0; w < WN; ++w)
                    *reinterpret_cast<float4*>(&c0[4 * w]) = load4(cand0 + ya * C::BWH + 4 * (gi + w));
                if (s != N) {
                    const float4 a1 = load4(ref1 + ya * C::BWR + 4 * gi);
                    const float lv[4] = {a1.x, a1.y, a1.z, a1.w};
                    float c1[4 * WN];
#pragma unroll
                    for (int w = 0; w < WN; ++w)
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
        for (int bi = tid; okB && bi < KL * C::HY; bi += C::THREADS) {
            float* row = Szb + bi * C::PSZ;
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
            constexpr int HC = C::CY / 2;  // outputs per running sum
            if constexpr (C::HY <= 64) {
                // the whole column in registers, two interleaved running sums
                float u[C::HY];
#pragma unroll
                for (int yh = 0; yh < C::HY; ++yh) u[yh] = col[yh * C::PSZ];
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
            } else {
                // one half column at a time (fewer registers beside the z sums); the second
                // half's rows are read before the first's writes could reach them
#pragma unroll
                for (int sg = 0; sg < 2; ++sg) {
                    float u[HC + 2 * N];
#pragma unroll
                    for (int yh = 0; yh < HC + 2 * N; ++yh) u[yh] = col[(HC * sg + yh) * C::PSZ];
                    float run = 0.f;
#pragma unroll
                    for (int y = 0; y <= 2 * N; ++y) run += u[y];
                    col[HC * sg * C::PSZ] = run;
#pragma unroll
                    for (int y = 1; y < HC; ++y) {
                        run += u[y + 2 * N] - u[y - 1];
                        col[(HC * sg + y) * C::PSZ] = run;
                    }
                }
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

template <int M, int N, typename Elem, int CYT, int XS>
__global__ void __launch_bounds__(Lpx3d<M, N, Elem, CYT, XS>::THREADS,
                                  Lpx3d<M, N, Elem, CYT, XS>::MINB)
    nlm3d_lpx_kernel(const __grid_constant__ CUtensorMap mapR,
                     const __grid_constant__ CUtensorMap mapC,
                     const __grid_constant__ CUtensorMap mapD, const LpArgs a) {
    extern __shared__ __align__(128) unsigned char smem[];
    // part = 2 * split + half (XS = 2) or the split (XS = 1)
    const int chunk = blockIdx.z % a.nzc, part = blockIdx.z / a.nzc;
    if constexpr (XS == 1)
        lpx_body<M, N, Elem, 2, CYT>(&mapR, &mapC, &mapD, a, smem, chunk, part);
    else if (part & 1)
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

// Search radii whose CTAs take half of the x offsets (the others keep all 2M + 1).  With
// 48-row tiles on 512 x 512 x 16, halves against all offsets per CTA: search 13 -10 to
// -22 %, search 11 -1 to -16 %, search 9 -4 to -14 %, search 7 -1 to -9 %; search 5 and 3
// +1 to +2 % (with few x offsets, halving them halves the candidate windows' reuse).
template <int M>
constexpr bool kLpXHalf = M >= 3;
// Output rows per tile: 48 (one CTA of 512 threads per SM, 64 halo rows for 48 output
// rows, one stage-D candidate buffer so that the plane boxes fit), the tallest tile whose
// FP32 buffers fit the shared memory.  Search 13, patch 17 on 512 x 512 x 128: 16-row tiles
// with every x offset per CTA (the first form of this kernel) 214 ms; x halves in 16-row
// tiles (two CTAs of 256 threads per SM) 207 ms, 32-row tiles (384 threads) 183 ms, 48-row
// tiles 167 ms.  Search 3 and 5 with every x offset per CTA: 48-row against 16-row tiles
// -18 to -28 %.
// With every x offset per CTA and FP16 plane boxes (search 3 and 5), or FP32 ones at search
// 3 (three z sums per row), the buffers also fit 64 output rows under 80 halo rows (448
// threads, three halo rows per stage-A thread): 11-16 % faster than 48 rows in FP16.  The
// x-half CTAs keep 48 rows (64 measured 22 % slower in FP16: the seven z sums of three rows
// crowd the registers; in FP32 the plane boxes do not fit).
template <int M, typename T, int XS>
constexpr int kLpRows = XS == 1 && (sizeof(T) == 2 || M == 1) ? 64 : 48;

template <int M, int N, typename T>
inline cudaError_t run_lp(const Staging& st, const void* staged, int tz, float inv_scale,
                          float* out, float* zsum, void* acc, unsigned int* errword,
                          cudaStream_t stream, int zc0, int zc1) {
    // x-offset halves (parts 2 * split + half) or every x offset (parts = splits) per CTA
    constexpr int XS = kLpXHalf<M> ? 2 : 1;
    using X = Lpx3d<M, N, T, kLpRows<M, T, XS>, XS>;
    if (st.elem != X::ES) return cudaErrorInvalidValue;
    CUtensorMap mapR, mapC, mapD;
    const uint64_t dims[3] = {(uint64_t)st.Xs, (uint64_t)st.Yp, (uint64_t)st.Zp};
    const uint64_t strides[2] = {(uint64_t)st.Xs * X::ES, (uint64_t)st.Xs * st.Yp * X::ES};
    const uint32_t boxR[3] = {(uint32_t)X::BWR, (uint32_t)X::HY, 1};
    const uint32_t boxC[3] = {(uint32_t)X::BWH, (uint32_t)X::HY, 1};
    const uint32_t boxD[3] = {(uint32_t)X::BWC, (uint32_t)X::CY, 1};
    void* base = const_cast<void*>(staged);
    cudaError_t e = encode_tensor_map(&mapR, X::ES == 2, 3, dims, strides, boxR, base);
    if (e == cudaSuccess) e = encode_tensor_map(&mapC, X::ES == 2, 3, dims, strides, boxC, base);
    if (e == cudaSuccess) e = encode_tensor_map(&mapD, X::ES == 2, 3, dims, strides, boxD, base);
    if (e != cudaSuccess) return e;
    auto kern = nlm3d_lpx_kernel<M, N, T, kLpRows<M, T, XS>, XS>;
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, X::SMEM_BYTES);
    if (e != cudaSuccess) return e;
    if (zc1 < 0) zc1 = (st.Z + tz - 1) / tz;
    if (zc1 <= zc0) return cudaSuccess;
    const int nsplit = nlm3d_lp_split(st.X, st.Y, st.Z, tz, X::CX, X::CY, XS, X::MINB);
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
    const int nparts = XS * nsplit;
    dim3 grid((st.X + X::CX - 1) / X::CX, (st.Y + X::CY - 1) / X::CY, (zc1 - zc0) * nparts);
    kern<<<grid, X::THREADS, X::SMEM_BYTES, stream>>>(mapR, mapC, mapD, a);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    // the kernel leaves its sums in the accumulator buffers (even with one part)
    const size_t plane = (size_t)st.X * st.Y;
    const size_t v0 = (size_t)zc0 * tz * plane;
    const size_t v1 = (size_t)std::min(zc1 * tz, st.Z) * plane;
    const size_t blocks = std::min<size_t>((v1 - v0 + 255) / 256, (size_t)device_sm_count() * 8);
    lp_combine_kernel<X::KAHAN><<<(unsigned)blocks, 256, 0, stream>>>(acc, a.part_stride, nparts,
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
