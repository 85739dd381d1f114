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
//      the current plane (add the entering plane, subtract the leaving one);
//      the reference plane and the candidate plane of a step come in as TMA
//      boxes (double-buffered, prefetched one step ahead), and one 4-column
//      candidate window serves all 2sr+1 x offsets;
//   B  x box sum of Sz along each halo row (shared memory, running sum);
//   C  y box sum down each output column, in place (running sum) -> D;
//   D  w = 2^(-D) (the staging pass pre-scaled the volume so D is the base-2
//      exponent of exp(-(D/P)/h^2), 3DNLM/main.cu:108-109), Z += w, num += w v
//      over the pass's x offsets, then one read-add-write of the voxel's (Z, num)
//      pair in the accumulator buffer (L2-resident: a chunk's pairs are re-read
//      once per pass, in pass order, so the sums are deterministic).  The last
//      pass writes out = num / Z (3DNLM/main.cu:125).
#pragma once

#include "nlm3d_tile.cuh"
#include "nlm_device.cuh"

namespace gnlm {

template <int M, int N>
struct Lp3d {
    static constexpr int K = 2 * M + 1;        // x offsets per pass
    static constexpr int CX = 32;              // output columns per CTA
    static constexpr int CY = 16;              // output rows per CTA
    static constexpr int H = M + N;
    static constexpr int HX = CX + 2 * N;      // halo columns
    static constexpr int HY = CY + 2 * N;      // halo rows
    // Boxes start at padded column X0 - 4 (16-byte aligned); box column i is
    // padded column X0 - 4 + i, halo column xh is i = 4 + M + xh.
    static constexpr int R = (M + 3) / 4;      // candidate float4s either side of a group
    static constexpr int G0 = 1 + M / 4;       // first 4-column group holding a halo column
    static constexpr int G1 = (4 + M + HX + 3) / 4;
    static constexpr int NG = G1 - G0;         // groups per halo row
    static constexpr int MA = M % 4;           // halo column 0 in an Sz row
    static constexpr int BWR = 4 * NG;         // reference box width (columns 4*G0 ..)
    static constexpr int BWC = 4 * (G1 + R);   // candidate box width (columns 0 ..)
    static constexpr int PSZ = (BWR % 8 == 4) ? BWR : BWR + 4;  // Sz row pitch, PSZ/4 odd
    static constexpr int PSX = 36;             // Sx row pitch (32 used), PSX/4 odd
    static constexpr int THREADS = 512;
    static constexpr int NA = NG * HY;         // stage A items (one per thread)
    static constexpr int NB = K * HY;          // stage B items (k, halo row)
    static constexpr int NC = K * CX;          // stage C items (k, column)
    static constexpr int REF_TX = BWR * HY * 4;    // bytes of a reference plane box
    static constexpr int CAND_TX = BWC * HY * 4;   // bytes of a candidate plane box
    static constexpr int REF_SLOT = cround(REF_TX, 128);
    static constexpr int CAND_SLOT = cround(CAND_TX, 128);
    static constexpr int ABUF = 2 * REF_SLOT + 2 * CAND_SLOT;  // entering/leaving ref + cand
    static constexpr int SZ_OFF = 0;
    static constexpr int SX_OFF = SZ_OFF + cround(K * HY * PSZ * 4, 128);
    static constexpr int A_OFF = SX_OFF + cround(K * HY * PSX * 4, 128);
    static constexpr int D_OFF = A_OFF + 2 * ABUF;
    static constexpr int BAR_OFF = D_OFF + 2 * CAND_SLOT;
    static constexpr int SMEM_BYTES = BAR_OFF + 64;
    static_assert(M >= 1 && N >= 1, "radii");
    static_assert(NA <= THREADS && NB <= THREADS && NC <= THREADS, "one item per thread");
    static_assert(CX * CY == THREADS, "one stage-D voxel per thread");
    static_assert(4 * R >= M, "candidate window covers the x offsets");
    static_assert(BWR >= MA + HX, "Sz row covers the halo");
    static_assert(BWC <= 256 && BWR <= 256 && HY <= 256, "TMA box dimension > 256");
    static_assert(4 + N + 31 + 2 * M < BWC, "stage D candidates inside the box");
    static_assert(SMEM_BYTES <= 227 * 1024, "shared memory");
};

// Geometry of one launch (all CTAs): tensor maps + extents + pass/step counts.
struct LpArgs {
    int X, Y, Z;
    int TZ;           // planes per chunk
    int zc0;          // first chunk of this launch
    float inv_scale;
    float2* acc;      // (Z, num) pairs, [Z][Y][X]
    float* out;
    float* zsum;
    unsigned int* errword;
};

template <int M, int N>
__global__ void __launch_bounds__(512, 1)
    nlm3d_lp_kernel(const __grid_constant__ CUtensorMap mapR,
                    const __grid_constant__ CUtensorMap mapC, const LpArgs a) {
    using C = Lp3d<M, N>;
    extern __shared__ __align__(128) unsigned char smem[];
    float* Szb = reinterpret_cast<float*>(smem + C::SZ_OFF);
    float* Sxb = reinterpret_cast<float*>(smem + C::SX_OFF);
    uint64_t* barA = reinterpret_cast<uint64_t*>(smem + C::BAR_OFF);
    uint64_t* barD = barA + 2;
    __shared__ int s_abort;

    const int tid = threadIdx.x;
    const int X0 = blockIdx.x * C::CX, Y0 = blockIdx.y * C::CY;
    const int Z0 = (blockIdx.z + a.zc0) * a.TZ;
    const int TZc = min(a.TZ, a.Z - Z0);
    if (TZc <= 0) return;  // uniform over the CTA
    const int SPP = TZc + 2 * N;            // steps per pass
    const int P = C::K * C::K;              // passes
    const int T = P * SPP;                  // steps
    const int TD = P * TZc;                 // steps with output (stage B..D)

    auto abuf = [&](int b) { return smem + C::A_OFF + b * C::ABUF; };
    auto dbuf = [&](int b) { return smem + C::D_OFF + b * C::CAND_SLOT; };

    // Thread 0: prefetch of step t's entering (and leaving) planes.
    auto issueA = [&](int t) {
        const int b = t & 1, pass = t / SPP, s = t - pass * SPP;
        const int oz = pass / C::K - M, oy = pass % C::K - M;
        const int ep = Z0 + M + s;  // padded plane of the entering plane (unpadded Z0 - N + s)
        const bool leave = s >= 2 * N + 1;
        unsigned char* base = abuf(b);
        fence_proxy_async_smem();
        mbar_arrive_expect_tx(&barA[b], (leave ? 2u : 1u) * (C::REF_TX + C::CAND_TX));
        tma_load_3d(base, &mapR, X0 - 4 + 4 * C::G0, Y0 + M, ep, &barA[b]);
        tma_load_3d(base + 2 * C::REF_SLOT, &mapC, X0 - 4, Y0 + M + oy, ep + oz, &barA[b]);
        if (leave) {
            const int lp = ep - (2 * N + 1);
            tma_load_3d(base + C::REF_SLOT, &mapR, X0 - 4 + 4 * C::G0, Y0 + M, lp, &barA[b]);
            tma_load_3d(base + 2 * C::REF_SLOT + C::CAND_SLOT, &mapC, X0 - 4, Y0 + M + oy, lp + oz,
                        &barA[b]);
        }
    };
    // Thread 0: the candidate plane of output step d (stage D's centre values).
    auto issueD = [&](int d) {
        const int b = d & 1, pass = d / TZc, q = d - pass * TZc;
        const int oz = pass / C::K - M, oy = pass % C::K - M;
        fence_proxy_async_smem();
        mbar_arrive_expect_tx(&barD[b], C::CAND_TX);
        tma_load_3d(dbuf(b), &mapC, X0 - 4, Y0 + M + oy, Z0 + q + C::H + oz, &barD[b]);
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

    // Stage A ownership: group gi (columns 4*(G0+gi) .. +3 of the box), halo row ya.
    const int gi = tid % C::NG, ya = tid / C::NG;
    const bool hasA = tid < C::NA;
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
        const int b = t & 1;
        const bool okA = mbar_wait_bounded(&barA[b], (t >> 1) & 1);
        if (!okA) {
            raise_device_error(a.errword, DEVERR_TMA_TIMEOUT);
            s_abort = 1;
        }
        const bool out_step = s >= 2 * N;
        if (okA && hasA) {
            const float* refE = reinterpret_cast<const float*>(abuf(b));
            const float* refL = refE + C::REF_SLOT / 4;
            const float* candE = refE + 2 * C::REF_SLOT / 4;
            const float* candL = candE + C::CAND_SLOT / 4;
            const float4 ae = *reinterpret_cast<const float4*>(refE + ya * C::BWR + 4 * gi);
            float ce[4 * (2 * C::R + 1)];
            const int g = C::G0 + gi;
#pragma unroll
            for (int r = 0; r <= 2 * C::R; ++r)
                *reinterpret_cast<float4*>(&ce[4 * r]) =
                    *reinterpret_cast<const float4*>(candE + ya * C::BWC + 4 * (g - C::R + r));
            const float av[4] = {ae.x, ae.y, ae.z, ae.w};
            if (s >= 2 * N + 1) {
                const float4 al = *reinterpret_cast<const float4*>(refL + ya * C::BWR + 4 * gi);
                float cl[4 * (2 * C::R + 1)];
#pragma unroll
                for (int r = 0; r <= 2 * C::R; ++r)
                    *reinterpret_cast<float4*>(&cl[4 * r]) =
                        *reinterpret_cast<const float4*>(candL + ya * C::BWC + 4 * (g - C::R + r));
                const float lv[4] = {al.x, al.y, al.z, al.w};
#pragma unroll
                for (int k = 0; k < C::K; ++k)
#pragma unroll
                    for (int c = 0; c < 4; ++c) {
                        const int i = 4 * C::R + c + k - M;
                        const float de = av[c] - ce[i];
                        const float dl = lv[c] - cl[i];
                        Sz[k][c] = fmaf(-dl, dl, fmaf(de, de, Sz[k][c]));
                    }
            } else {
#pragma unroll
                for (int k = 0; k < C::K; ++k)
#pragma unroll
                    for (int c = 0; c < 4; ++c) {
                        const float de = av[c] - ce[4 * C::R + c + k - M];
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

        // B: x box sums along halo rows.
        if (tid < C::NB) {
            const int k = tid / C::HY, yh = tid - k * C::HY;
            const float* row = Szb + (k * C::HY + yh) * C::PSZ;
            constexpr int NV = (C::MA + C::HX + 3) / 4;
            float v[4 * NV];
#pragma unroll
            for (int q = 0; q < NV; ++q)
                *reinterpret_cast<float4*>(&v[4 * q]) = *reinterpret_cast<const float4*>(row + 4 * q);
            float* sx = Sxb + (k * C::HY + yh) * C::PSX;
            float acc = 0.f;
#pragma unroll
            for (int x = 0; x <= 2 * N; ++x) acc += v[C::MA + x];
            float o[4];
            o[0] = acc;
#pragma unroll
            for (int j = 1; j < C::CX; ++j) {
                acc += v[C::MA + j + 2 * N] - v[C::MA + j - 1];
                o[j & 3] = acc;
                if ((j & 3) == 3)
                    *reinterpret_cast<float4*>(sx + j - 3) = make_float4(o[0], o[1], o[2], o[3]);
            }
        }
        __syncthreads();
        // C: y box sums down output columns, in place (row y of the column becomes D).
        if (tid < C::NC) {
            const int k = tid >> 5, j = tid & 31;
            float* col = Sxb + k * C::HY * C::PSX + j;
            float u[C::HY];
#pragma unroll
            for (int yh = 0; yh < C::HY; ++yh) u[yh] = col[yh * C::PSX];
            float acc = 0.f;
#pragma unroll
            for (int y = 0; y <= 2 * N; ++y) acc += u[y];
            col[0] = acc;
#pragma unroll
            for (int y = 1; y < C::CY; ++y) {
                acc += u[y + 2 * N] - u[y - 1];
                col[y * C::PSX] = acc;
            }
        }
        __syncthreads();
        // D: weights and accumulation for voxel (X0 + j, Y0 + y, z).
        {
            const int db = d & 1;
            const bool okD = mbar_wait_bounded(&barD[db], (d >> 1) & 1);
            if (!okD) {
                raise_device_error(a.errword, DEVERR_TMA_TIMEOUT);
                s_abort = 1;
            } else {
                const int y = tid >> 5, j = tid & 31;
                const int dpass = d / TZc, q = d - dpass * TZc;
                const int x = X0 + j, yy = Y0 + y, z = Z0 + q;
                const bool inside = x < a.X && yy < a.Y;
                const size_t o = ((size_t)z * a.Y + yy) * a.X + x;
                float2 prev = make_float2(0.f, 0.f);
                if (inside && dpass > 0) prev = a.acc[o];
                const float* cpl = reinterpret_cast<const float*>(dbuf(db)) + (N + y) * C::BWC + 4 + N + j;
                float zl = 0.f, nl = 0.f;
#pragma unroll
                for (int k = 0; k < C::K; ++k) {
                    const float w = ex2_neg(Sxb[(k * C::HY + y) * C::PSX + j]);
                    zl += w;
                    nl = fmaf(w, cpl[k], nl);
                }
                if (inside) {
                    zl = prev.x + zl;
                    nl = prev.y + nl;
                    if (dpass == P - 1) {
                        a.out[o] = nl / zl * a.inv_scale;
                        if (a.zsum) a.zsum[o] = zl;
                    } else {
                        a.acc[o] = make_float2(zl, nl);
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

}  // namespace gnlm
