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
// Kernels: adj_aux_kernel (G and out' padded like the staged volume),
// nlm3d_adj_kernel (gpad' over the padded domain + per-CTA h partial sums),
// adj_fold_kernel (REFLECT_101 fold, times s), adj_hgrad_kernel (ordered sum).
#include <cuda_fp16.h>

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
    static constexpr int FIELD_BYTES = BX * BY * BZ * 4;
    // each field starts on a 128-byte boundary: TMA tensor-copy destinations must
    static constexpr int FIELD_STRIDE = adj_round(FIELD_BYTES, 128);
    static constexpr int BAR_OFF = 3 * FIELD_STRIDE;          // mbarrier
    static constexpr int RED_OFF = BAR_OFF + 128;             // per-warp h partials
    static constexpr int SMEM_BYTES = RED_OFF + 32 * 8;
    static_assert(FIELD_STRIDE % 128 == 0 && BAR_OFF % 128 == 0, "TMA destination alignment");
    static constexpr int K = 2 * N + 1;
    static constexpr int RT = RY + 4 * N, PT = RZ + 4 * N;  // difference window
    static constexpr int RD = RY + 2 * N, PD = RZ + 2 * N;  // distance window
    static_assert(BX <= 256 && BY <= 256 && BZ <= 256, "TMA box dimension > 256");
    static_assert(SMEM_BYTES <= 227 * 1024, "adjoint tile exceeds shared memory");
};

// G = g / (s Z) and out' = s out, padded like the staged volume (zero outside).
__global__ void __launch_bounds__(256) adj_aux_kernel(const float* __restrict__ g,
                                                      const float* __restrict__ out,
                                                      const float* __restrict__ zsum, int X,
                                                      int Y, int Z, int H, int Xs, int Yp,
                                                      float s, float* __restrict__ G,
                                                      float* __restrict__ O) {
    const int py = blockIdx.x, pz = blockIdx.y;
    const int y = py - H, z = pz - H;
    const bool inside_yz = y >= 0 && y < Y && z >= 0 && z < Z;
    float* grow = G + ((size_t)pz * Yp + py) * Xs;
    float* orow = O + ((size_t)pz * Yp + py) * Xs;
    for (int px = threadIdx.x; px < Xs; px += blockDim.x) {
        const int x = px - H;
        float gv = 0.f, ov = 0.f;
        if (inside_yz && x >= 0 && x < X) {
            const size_t i = ((size_t)z * Y + y) * X + x;
            gv = g[i] / (s * zsum[i]);
            ov = s * out[i];
        }
        grow[px] = gv;
        orow[px] = ov;
    }
}

template <int M, int N, int RY, int RZ, int NW>
__global__ void __launch_bounds__(32 * NW, 1)
    nlm3d_adj_kernel(const __grid_constant__ CUtensorMap vmap,
                     const __grid_constant__ CUtensorMap gmap,
                     const __grid_constant__ CUtensorMap omap, int X, int Y, int Z, int Xs, int Yp,
                     float* __restrict__ gpad, double* __restrict__ hpart,
                     unsigned int* errword) {
    using C = Adj3d<M, N, RY, RZ, NW>;
    constexpr float kLn2 = 0.69314718055994531f;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    float* vt = reinterpret_cast<float*>(smem_raw);
    float* gt = reinterpret_cast<float*>(smem_raw + C::FIELD_STRIDE);
    float* ot = reinterpret_cast<float*>(smem_raw + 2 * C::FIELD_STRIDE);
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw + C::BAR_OFF);
    double* red = reinterpret_cast<double*>(smem_raw + C::RED_OFF);

    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int Xp = X + 2 * C::H, Ypd = Y + 2 * C::H, Zp = Z + 2 * C::H;
    // Output positions are padded-domain voxels, staged coordinates [0, Xp) etc.
    // smem column 0 starts HE voxels before lane 0's voxel (staged x = bx*XO - 2N)
    const int base_x = blockIdx.x * C::XO - 2 * N - C::HE;
    const int org_x = base_x & ~3;                  // 16-byte aligned TMA start (may be < 0)
    const int ral = base_x - org_x;
    const int Y0 = blockIdx.y * C::TY, Z0 = blockIdx.z * RZ;
    const int org_y = Y0 - C::HE, org_z = Z0 - C::HE;

    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        mbar_arrive_expect_tx(bar, 3 * C::FIELD_BYTES);
        tma_load_3d(vt, &vmap, org_x, org_y, org_z, bar);
        tma_load_3d(gt, &gmap, org_x, org_y, org_z, bar);
        tma_load_3d(ot, &omap, org_x, org_y, org_z, bar);
    }
    if (!mbar_wait_bounded(bar, 0)) {
        if (threadIdx.x == 0) {
            raise_device_error(errword, DEVERR_TMA_TIMEOUT);
            mbar_wait_bounded(bar, 0);
        }
        return;
    }

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
    constexpr int RTP = C::RT / 2;
    float2 av[RTP][C::PT];
    // G and out' at the distance window (same for every offset)
    float gu[C::RD][C::PD], ou[C::RD][C::PD];
#pragma unroll
    for (int rp = 0; rp < RTP; ++rp)
#pragma unroll
        for (int p = 0; p < C::PT; ++p) {
            const int i = (sz + p - 2 * N) * C::PLANE + (sy + 2 * rp - 2 * N) * C::BX + sx;
            av[rp][p] = make_float2(vt[i], vt[i + C::BX]);
        }
#pragma unroll
    for (int r = 0; r < C::RD; ++r)
#pragma unroll
        for (int p = 0; p < C::PD; ++p) {
            const int i = (sz + p - N) * C::PLANE + (sy + r - N) * C::BX + sx;
            gu[r][p] = gt[i];
            ou[r][p] = ot[i];
        }
    auto avs = [&](int r, int p) { return (r & 1) ? av[r >> 1][p].y : av[r >> 1][p].x; };

    float acc[RY][RZ];
#pragma unroll
    for (int r = 0; r < RY; ++r)
#pragma unroll
        for (int q = 0; q < RZ; ++q) acc[r][q] = 0.f;
    double hacc = 0.0;
    const float2 minus1 = make_float2(-1.f, -1.f);

    for (int oz = -M; oz <= M; ++oz) {
        for (int oy = -M; oy <= M; ++oy) {
            // dL/dh terms of this run of 2M+1 offsets, summed in FP32, then added to
            // the FP64 total once per run
            float hrun = 0.f;
            for (int ox = -M; ox <= M; ++ox) {
                const int off = oz * C::PLANE + oy * C::BX + ox;
                // differences t = v'_u - v'_{u+o} over the window (row pairs), candidates b
                float2 t2[RTP][C::PT];
                float bv[C::RD][C::PD];
#pragma unroll
                for (int rp = 0; rp < RTP; ++rp)
#pragma unroll
                    for (int p = 0; p < C::PT; ++p) {
                        const int i =
                            (sz + p - 2 * N) * C::PLANE + (sy + 2 * rp - 2 * N) * C::BX + sx + off;
                        const float b0 = vt[i], b1 = vt[i + C::BX];
                        t2[rp][p] = __ffma2_rn(make_float2(b0, b1), minus1, av[rp][p]);
                        const int r0 = 2 * rp, r1 = 2 * rp + 1;
                        if (p >= N && p < N + C::PD) {
                            if (r0 >= N && r0 < N + C::RD) bv[r0 - N][p - N] = b0;
                            if (r1 >= N && r1 < N + C::RD) bv[r1 - N][p - N] = b1;
                        }
                    }
                auto ts = [&](int r, int p) { return (r & 1) ? t2[r >> 1][p].y : t2[r >> 1][p].x; };
                // distance D' on the distance window: z sums of t^2 (packed row pairs),
                // then y sums, then x across lanes
                float2 zs[RTP][C::PD];
#pragma unroll
                for (int rp = 0; rp < RTP; ++rp)
#pragma unroll
                    for (int p = 0; p < C::PD; ++p) {
                        float2 sum = __fmul2_rn(t2[rp][p], t2[rp][p]);
#pragma unroll
                        for (int kz = 1; kz < C::K; ++kz)
                            sum = __ffma2_rn(t2[rp][p + kz], t2[rp][p + kz], sum);
                        zs[rp][p] = sum;
                    }
                auto zss = [&](int r, int p) { return (r & 1) ? zs[r >> 1][p].y : zs[r >> 1][p].x; };
                float D[C::RD][C::PD];
#pragma unroll
                for (int r = 0; r < C::RD; ++r)
#pragma unroll
                    for (int p = 0; p < C::PD; ++p) {
                        float sum = zss(r, p);
#pragma unroll
                        for (int ky = 1; ky < C::K; ++ky) sum += zss(r + ky, p);
                        D[r][p] = sum;
                    }
#pragma unroll
                for (int r = 0; r < C::RD; ++r)
#pragma unroll
                    for (int p = 0; p < C::PD; ++p) {
                        D[r][p] = xbox_lanes<N>(D[r][p]);
                    }
                // weights, G(u+o), and the field a_o(u) (without the -ln2)
                float e[C::RD][C::PD], a[C::RD][C::PD], guo[C::RD][C::PD];
#pragma unroll
                for (int r = 0; r < C::RD; ++r)
#pragma unroll
                    for (int p = 0; p < C::PD; ++p) {
                        const int i = (sz + p - N) * C::PLANE + (sy + r - N) * C::BX + sx + off;
                        const float g2 = gt[i], o2 = ot[i];
                        e[r][p] = ex2_neg(D[r][p]);
                        guo[r][p] = g2;
                        const float vu = avs(r + N, p + N);
                        a[r][p] = e[r][p] * fmaf(gu[r][p], bv[r][p] - ou[r][p], g2 * (vu - o2));
                    }
                // box sum of a over the patch: z, then y, then x across lanes
                float za[C::RD][RZ];
#pragma unroll
                for (int r = 0; r < C::RD; ++r)
#pragma unroll
                    for (int q = 0; q < RZ; ++q) {
                        float sum = a[r][q];
#pragma unroll
                        for (int kz = 1; kz < C::K; ++kz) sum += a[r][q + kz];
                        za[r][q] = sum;
                    }
#pragma unroll
                for (int r = 0; r < RY; ++r)
#pragma unroll
                    for (int q = 0; q < RZ; ++q) {
                        float yv = za[r][q];
#pragma unroll
                        for (int ky = 1; ky < C::K; ++ky) yv += za[r + ky][q];
                        const float xv = xbox_lanes<N>(yv);
                        // gpad' += G(q+o) e_q(o) + 2 (v'_q - v'_{q+o}) (-ln2) A(q)
                        acc[r][q] = fmaf(guo[r + N][q + N], e[r + N][q + N], acc[r][q]);
                        acc[r][q] = fmaf(-2.f * kLn2 * ts(r + 2 * N, q + 2 * N), xv, acc[r][q]);
                        // dL/dh partial: a1_o(q) D'_q(o), a1 = -ln2 e G(q) (v'_{q+o} - out'_q)
                        const float a1 = e[r + N][q + N] * gu[r + N][q + N] *
                                         (bv[r + N][q + N] - ou[r + N][q + N]);
                        hrun = fmaf(a1, D[r + N][q + N], hrun);
                    }
            }
            hacc += (double)hrun;
        }
    }

    // store gpad' for the thread's padded-domain voxels; reduce the h partial
    const int px = blockIdx.x * C::XO + lane - 2 * N;  // staged x of this lane
    const bool lane_ok = lane >= 2 * N && lane < 32 - 2 * N && px < Xp;
    double hsum = 0.0;
#pragma unroll
    for (int q = 0; q < RZ; ++q) {
        const int pz = Z0 + q;
#pragma unroll
        for (int r = 0; r < RY; ++r) {
            const int py = Y0 + warp * RY + r;
            if (lane_ok && py < Ypd && pz < Zp) gpad[((size_t)pz * Yp + py) * Xs + px] = acc[r][q];
        }
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
        hpart[((size_t)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x] = -kLn2 * s;
    }
}

// Padded positions along one axis whose REFLECT_101 source is i: i + H, plus any of
// the 2H border positions that reflect onto i.  Returns the count (<= 1 + 2H).
__device__ __forceinline__ int preimages(int i, int n, int H, int* p) {
    int k = 0;
    p[k++] = i + H;
    for (int b = 0; b < H; ++b) {
        if (reflect101(b - H, n) == i) p[k++] = b;
        if (reflect101(n + b, n) == i) p[k++] = n + H + b;
    }
    return k;
}

// gin(x) = s * sum of gpad' over the padded positions that REFLECT_101 maps to x.
constexpr int kMaxHalo = 16;
__global__ void __launch_bounds__(256) adj_fold_kernel(const float* __restrict__ gpad, int X,
                                                       int Y, int Z, int H, int Xs, int Yp,
                                                       float s, float* __restrict__ gin) {
    const int y = blockIdx.x, z = blockIdx.y;
    int pz[1 + 2 * kMaxHalo], py[1 + 2 * kMaxHalo], px[1 + 2 * kMaxHalo];
    const int nz = preimages(z, Z, H, pz);
    const int ny = preimages(y, Y, H, py);
    for (int x = threadIdx.x; x < X; x += blockDim.x) {
        const int nx = preimages(x, X, H, px);
        float sum = 0.f;
        for (int a = 0; a < nz; ++a)
            for (int b = 0; b < ny; ++b) {
                const float* row = gpad + ((size_t)pz[a] * Yp + py[b]) * Xs;
                for (int c = 0; c < nx; ++c) sum += row[px[c]];
            }
        gin[((size_t)z * Y + y) * X + x] = s * sum;
    }
}

// dL/dh = -(2/h) * sum of the per-CTA partials, summed in index order by one thread.
__global__ void adj_hgrad_kernel(const double* __restrict__ hpart, int n, double coef,
                                 double* __restrict__ hgrad) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        double s = 0.0;
        for (int i = 0; i < n; ++i) s += hpart[i];
        *hgrad = coef * s;
    }
}

template <int M, int N, int RY, int RZ, int NW>
static cudaError_t run_adj3d(const Staging& st, const void* staged, const float* d_out,
                             const float* d_zsum, const float* d_gout, float s, float h,
                             float* gin, double* hgrad, float* G, float* O, float* gpad,
                             double* hpart, unsigned int* errword, cudaStream_t stream) {
    using C = Adj3d<M, N, RY, RZ, NW>;
    dim3 rows(st.Yp, st.Zp);
    adj_aux_kernel<<<rows, 256, 0, stream>>>(d_gout, d_out, d_zsum, st.X, st.Y, st.Z, st.H, st.Xs,
                                              st.Yp, s, G, O);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    CUtensorMap vmap, gmap, omap;
    const uint64_t dims[3] = {(uint64_t)st.Xs, (uint64_t)st.Yp, (uint64_t)st.Zp};
    const uint64_t strides[2] = {(uint64_t)st.Xs * 4, (uint64_t)st.Xs * st.Yp * 4};
    const uint32_t box[3] = {(uint32_t)C::BX, (uint32_t)C::BY, (uint32_t)C::BZ};
    if ((e = encode_tensor_map(&vmap, false, 3, dims, strides, box, const_cast<void*>(staged))))
        return e;
    if ((e = encode_tensor_map(&gmap, false, 3, dims, strides, box, G))) return e;
    if ((e = encode_tensor_map(&omap, false, 3, dims, strides, box, O))) return e;
    auto kern = nlm3d_adj_kernel<M, N, RY, RZ, NW>;
    if ((e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM_BYTES)))
        return e;
    dim3 grid((st.Xp + C::XO - 1) / C::XO, (st.Yp + C::TY - 1) / C::TY, (st.Zp + RZ - 1) / RZ);
    kern<<<grid, 32 * NW, C::SMEM_BYTES, stream>>>(vmap, gmap, omap, st.X, st.Y, st.Z, st.Xs,
                                                   st.Yp, gpad, hpart, errword);
    if ((e = cudaGetLastError())) return e;
    dim3 out_rows(st.Y, st.Z);
    adj_fold_kernel<<<out_rows, 128, 0, stream>>>(gpad, st.X, st.Y, st.Z, st.H, st.Xs, st.Yp, s,
                                                  gin);
    if ((e = cudaGetLastError())) return e;
    if (hgrad) {
        const int nblk = grid.x * grid.y * grid.z;
        adj_hgrad_kernel<<<1, 32, 0, stream>>>(hpart, nblk, -2.0 / (double)h, hgrad);
        e = cudaGetLastError();
    }
    return e;
}

// Tile shape per (sr, pr): 8 warps x 2 rows x 4 planes, or 4 x 2 x 2 where the
// three FP32 tiles of a larger halo would not fit in shared memory.
template <int M, int N>
struct AdjShape {
    static constexpr bool SMALL = M + 2 * N > 5;
    static constexpr int RY = 2, RZ = SMALL ? 2 : 4, NW = SMALL ? 4 : 8;
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

// Number of CTAs of the adjoint kernel (one double of h partials each).
size_t adj3d_ctas(const Staging& st, int sr, int pr) {
#define X_(m, n)                                                                             \
    if (sr == m && pr == n) {                                                                \
        using C = AdjShape<m, n>::C;                                                         \
        return (size_t)((st.Xp + C::XO - 1) / C::XO) * ((st.Yp + C::TY - 1) / C::TY) *     \
               ((st.Zp + AdjShape<m, n>::RZ - 1) / AdjShape<m, n>::RZ);                      \
    }
    GNLM_ADJ3D_CASES(X_)
#undef X_
    return 0;
}

cudaError_t launch_nlm3d_adj(const Staging& st, const void* staged, const float* d_out,
                             const float* d_zsum, const float* d_gout, int sr, int pr, float s,
                             float h, float* gin, double* hgrad, float* G, float* O, float* gpad,
                             double* hpart, unsigned int* errword, cudaStream_t stream) {
    if (st.H > kMaxHalo) return cudaErrorNotSupported;
#define X_(m, n)                                                                                \
    if (sr == m && pr == n)                                                                     \
        return run_adj3d<m, n, AdjShape<m, n>::RY, AdjShape<m, n>::RZ, AdjShape<m, n>::NW>(    \
            st, staged, d_out, d_zsum, d_gout, s, h, gin, hgrad, G, O, gpad, hpart, errword,    \
            stream);
    GNLM_ADJ3D_CASES(X_)
#undef X_
    return cudaErrorNotSupported;
}

}  // namespace gnlm
