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
    static constexpr int NA = 16 * HY;         // stage A threads (16 per halo row, NG used)
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
    static_assert(NG <= 16 && NA <= THREADS && NB <= THREADS && NC <= THREADS,
                  "one item per thread");
    static_assert(CX == 32 && CY == 16, "stage B/C split outputs into two runs");
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
    int nzc;          // chunks in this launch (grid z = nzc * nsplit)
    int nsplit;       // 1: a CTA makes every pass; 2: each half of the passes
    size_t part_stride;  // float2 pairs per accumulator buffer (X * Y * Z)
    float inv_scale;
    float2* acc;      // (Z, num) pairs, [nsplit][Z][Y][X]
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
    const int chunk = blockIdx.z % a.nzc, part = blockIdx.z / a.nzc;
    const int Z0 = (chunk + a.zc0) * a.TZ;
    const int TZc = min(a.TZ, a.Z - Z0);
    if (TZc <= 0) return;  // uniform over the CTA
    // This CTA's passes [pb, pb + P) of the (2sr+1)^2, and its accumulator buffer.
    const int pb = part * (C::K * C::K) / a.nsplit;
    const int P = (part + 1) * (C::K * C::K) / a.nsplit - pb;
    float2* const acc = a.acc + part * a.part_stride;
    // A pass is N warm-up steps, each adding two planes of the first window
    // (padded planes Z0+M .. Z0+M+2N-1), then TZc output steps: output plane
    // Z0+q adds padded plane Z0+M+2N+q and, for q >= 1, drops Z0+M+q-1.
    const int SPP = N + TZc;
    const int T = P * SPP;      // steps
    const int TD = P * TZc;     // output steps

    auto abuf = [&](int b) { return smem + C::A_OFF + b * C::ABUF; };
    auto dbuf = [&](int b) { return smem + C::D_OFF + b * C::CAND_SLOT; };

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
        tma_load_3d(base, &mapR, xr, yr, p0, &barA[b]);
        tma_load_3d(base + 2 * C::REF_SLOT, &mapC, X0 - 4, yr + oy, p0 + oz, &barA[b]);
        if (p1 >= 0) {
            tma_load_3d(base + C::REF_SLOT, &mapR, xr, yr, p1, &barA[b]);
            tma_load_3d(base + 2 * C::REF_SLOT + C::CAND_SLOT, &mapC, X0 - 4, yr + oy, p1 + oz,
                        &barA[b]);
        }
    };
    // Thread 0: the candidate plane of output step d (stage D's centre values).
    auto issueD = [&](int d) {
        const int b = d & 1, lp = d / TZc, q = d - lp * TZc, pass = pb + lp;
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

    // Stage A ownership: 16 lanes per halo row (conflict-free shared loads), lane
    // gi < NG owns columns 4*(G0+gi) .. +3 of the box.
    const int gi = tid & 15, ya = tid >> 4;
    bool hasA = gi < C::NG && ya < C::HY;
    // Stages B-D own fixed items too; a thread whose ranges leave their buffers
    // (possible only through a defect, caught by NLM_BOUNDS_CHECK builds) skips its work.
    bool okB = tid < C::NB, okC = tid < C::NC, okD = true;
    if constexpr (kBoundsCheck) {
        const long long szn = (long long)C::K * C::HY * C::PSZ, sxn = (long long)C::K * C::HY * C::PSX;
        if (hasA) {
            const int g = C::G0 + gi;
            hasA = range_ok(a.errword, ya * C::BWR + 4 * gi, ya * C::BWR + 4 * gi + 3, C::REF_TX / 4) &&
                   range_ok(a.errword, ya * C::BWC + 4 * (g - C::R),
                            ya * C::BWC + 4 * (g + C::R) + 3, C::CAND_TX / 4) &&
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
              range_ok(a.errword, (N + y) * C::BWC + 4 + N + j,
                       (N + y) * C::BWC + 4 + N + j + C::K - 1, C::CAND_TX / 4);
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
        if (vin && pass > 0) prev = acc[vo];
        const int b = t & 1;
        const bool okA = mbar_wait_bounded(&barA[b], (t >> 1) & 1);
        if (!okA) {
            raise_device_error(a.errword, DEVERR_TMA_TIMEOUT);
            s_abort = 1;
        }
        if (okA && hasA) {
            const float* ref0 = reinterpret_cast<const float*>(abuf(b));
            const float* ref1 = ref0 + C::REF_SLOT / 4;
            const float* cand0 = ref0 + 2 * C::REF_SLOT / 4;
            const float* cand1 = cand0 + C::CAND_SLOT / 4;
            const int g = C::G0 + gi;
            const float4 a0 = *reinterpret_cast<const float4*>(ref0 + ya * C::BWR + 4 * gi);
            const float av[4] = {a0.x, a0.y, a0.z, a0.w};
            float c0[4 * (2 * C::R + 1)];
#pragma unroll
            for (int r = 0; r <= 2 * C::R; ++r)
                *reinterpret_cast<float4*>(&c0[4 * r]) =
                    *reinterpret_cast<const float4*>(cand0 + ya * C::BWC + 4 * (g - C::R + r));
            if (s != N) {
                // second plane: added (warm-up) or dropped (leaving)
                const float4 a1 = *reinterpret_cast<const float4*>(ref1 + ya * C::BWR + 4 * gi);
                const float lv[4] = {a1.x, a1.y, a1.z, a1.w};
                float c1[4 * (2 * C::R + 1)];
#pragma unroll
                for (int r = 0; r <= 2 * C::R; ++r)
                    *reinterpret_cast<float4*>(&c1[4 * r]) =
                        *reinterpret_cast<const float4*>(cand1 + ya * C::BWC + 4 * (g - C::R + r));
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
                const float* cpl =
                    reinterpret_cast<const float*>(dbuf(db)) + (N + y) * C::BWC + 4 + N + j;
                float zl[2] = {0.f, 0.f}, nl[2] = {0.f, 0.f};
#pragma unroll
                for (int k = 0; k < C::K; ++k) {
                    const float w = ex2_neg(Sxb[(k * C::HY + y) * C::PSX + j]);
                    zl[k & 1] += w;
                    nl[k & 1] = fmaf(w, cpl[k], nl[k & 1]);
                }
                if (vin) {
                    const float zt = prev.x + (zl[0] + zl[1]);
                    const float nt = prev.y + (nl[0] + nl[1]);
                    if (pass == P - 1 && a.nsplit == 1) {
                        a.out[vo] = nt / zt * a.inv_scale;
                        if (a.zsum) a.zsum[vo] = zt;
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

}  // namespace gnlm
