// 3D non-local means forward kernel for sm_103a: one CTA per output tile.
// The per-tile body (TMA staging, register bricks, sliding-window box sums,
// exp weights, accumulation) is fwd3d_tile in nlm3d_tile.cuh.
#include "nlm3d_tile.cuh"
#include "nlm_internal.h"

namespace gnlm {

// Single-volume kernel: one CTA per output tile.
template <int M, int N, typename T, int RY, int RZ, int NW, int MINB, bool AREG, bool KAHAN>
__global__ void __launch_bounds__(32 * NW, MINB)
    nlm3d_fwd_kernel(const __grid_constant__ CUtensorMap tmap, int X, int Y, int Z,
                     float inv_scale, float* __restrict__ out, float* __restrict__ zsum,
                     unsigned int* errword, int bz0) {
    using C = Fwd3d<M, N, T, RY, RZ, NW>;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    T* tile = reinterpret_cast<T*>(smem_raw);
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw + C::BAR_OFF);
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    fwd3d_tile<M, N, T, RY, RZ, NW, AREG, KAHAN>(&tmap, tile, bar, 0, blockIdx.x, blockIdx.y,
                                                  blockIdx.z + bz0, X, Y, Z, inv_scale, out, zsum,
                                                  errword);
}

// Single-volume kernel with grouped z offsets (fwd3d_tile_pz).
template <int M, int N, int RY, int RZ, int NW, int MINB, int GZ>
__global__ void __launch_bounds__(32 * NW, MINB)
    nlm3d_fwd_pz_kernel(const __grid_constant__ CUtensorMap tmap, int X, int Y, int Z,
                        float inv_scale, float* __restrict__ out, float* __restrict__ zsum,
                        unsigned int* errword, int bz0) {
    using C = Fwd3d<M, N, float, RY, RZ, NW>;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    float* tile = reinterpret_cast<float*>(smem_raw);
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw + C::BAR_OFF);
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    fwd3d_tile_pz<M, N, RY, RZ, NW, GZ>(&tmap, tile, bar, 0, blockIdx.x, blockIdx.y, blockIdx.z + bz0,
                                    X, Y, Z, inv_scale, out, zsum, errword);
}

// FP16-storage single-volume kernel (row-pair layout, two tensor maps).
template <int M, int N, int RY, int RZ, int NW, int MINB, bool KAHAN>
__global__ void __launch_bounds__(32 * NW, MINB)
    nlm3d_fwd_h2_kernel(const __grid_constant__ CUtensorMap mapE,
                        const __grid_constant__ CUtensorMap mapO, int X, int Y, int Z,
                        float inv_scale, float* __restrict__ out, float* __restrict__ zsum,
                        unsigned int* errword, int bz0) {
    using C = Fwd3dH2<M, N, RY, RZ, NW>;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw + C::BAR_OFF);
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    fwd3d_tile_h2<M, N, RY, RZ, NW, KAHAN>(&mapE, &mapO, smem_raw, bar, 0, blockIdx.x,
                                           blockIdx.y, blockIdx.z + bz0, X, Y, Z, inv_scale, out, zsum,
                                           errword);
}

template <int M, int N, int RY, int RZ, int NW, int MINB, bool KAHAN>
static cudaError_t run_fwd3d_h2(const Staging& st, const void* staged, float inv_scale,
                                float* out, float* zsum, unsigned int* errword,
                                cudaStream_t stream, int zt0, int zt1) {
    using C = Fwd3dH2<M, N, RY, RZ, NW>;
    CUtensorMap mapE, mapO;
    const uint64_t dims[3] = {(uint64_t)st.Xs, (uint64_t)st.Yq, (uint64_t)st.Zp};
    const uint64_t strides[2] = {(uint64_t)st.Xs * 4, (uint64_t)st.Xs * st.Yq * 4};
    const uint32_t box[3] = {(uint32_t)C::BX, (uint32_t)C::BYQ, (uint32_t)C::BZ};
    char* base = static_cast<char*>(const_cast<void*>(staged));
    cudaError_t e = encode_tensor_map(&mapE, false, 3, dims, strides, box, base);
    if (e == cudaSuccess)
        e = encode_tensor_map(&mapO, false, 3, dims, strides, box, base + st.copy_bytes());
    if (e != cudaSuccess) return e;
    auto kern = nlm3d_fwd_h2_kernel<M, N, RY, RZ, NW, MINB, KAHAN>;
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM_BYTES);
    if (e != cudaSuccess) return e;
    if (zt1 < 0) zt1 = (st.Z + RZ - 1) / RZ;
    if (zt1 <= zt0) return cudaSuccess;
    dim3 grid((st.X + C::XO - 1) / C::XO, (st.Y + C::TY - 1) / C::TY, zt1 - zt0);
    kern<<<grid, 32 * NW, C::SMEM_BYTES, stream>>>(mapE, mapO, st.X, st.Y, st.Z, inv_scale, out,
                                                   zsum, errword, zt0);
    return cudaGetLastError();
}

template <int M, int N, int RY, int RZ, int NW, int MINB, int GZ>
static cudaError_t run_fwd3d_pz(const Staging& st, const void* staged, float inv_scale, float* out,
                                float* zsum, unsigned int* errword, cudaStream_t stream, int zt0,
                                int zt1) {
    using C = Fwd3d<M, N, float, RY, RZ, NW>;
    CUtensorMap map;
    const uint64_t dims[3] = {(uint64_t)st.Xs, (uint64_t)st.Yp, (uint64_t)st.Zp};
    const uint64_t strides[2] = {(uint64_t)st.Xs * 4, (uint64_t)st.Xs * st.Yp * 4};
    const uint32_t box[3] = {(uint32_t)C::BX, (uint32_t)C::BY, (uint32_t)C::BZ};
    cudaError_t e = encode_tensor_map(&map, false, 3, dims, strides, box, const_cast<void*>(staged));
    if (e != cudaSuccess) return e;
    auto kern = nlm3d_fwd_pz_kernel<M, N, RY, RZ, NW, MINB, GZ>;
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM_BYTES);
    if (e != cudaSuccess) return e;
    if (zt1 < 0) zt1 = (st.Z + RZ - 1) / RZ;
    if (zt1 <= zt0) return cudaSuccess;
    dim3 grid((st.X + C::XO - 1) / C::XO, (st.Y + C::TY - 1) / C::TY, zt1 - zt0);
    kern<<<grid, C::THREADS, C::SMEM_BYTES, stream>>>(map, st.X, st.Y, st.Z, inv_scale, out, zsum,
                                                      errword, zt0);
    return cudaGetLastError();
}

template <int M, int N, typename T, int RY, int RZ, int NW, int MINB, bool AREG, bool KAHAN>
static cudaError_t run_fwd3d(const Staging& st, const void* staged, float inv_scale, float* out,
                             float* zsum, unsigned int* errword, cudaStream_t stream, int zt0,
                             int zt1) {
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
    if (zt1 < 0) zt1 = (st.Z + RZ - 1) / RZ;
    if (zt1 <= zt0) return cudaSuccess;
    dim3 grid((st.X + C::XO - 1) / C::XO, (st.Y + C::TY - 1) / C::TY, zt1 - zt0);
    kern<<<grid, C::THREADS, C::SMEM_BYTES, stream>>>(map, st.X, st.Y, st.Z, inv_scale, out, zsum,
                                                      errword, zt0);
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
//   4: 4 x 6, z offsets in groups of four sharing candidate planes (the 2M+1 z offsets
//      split as 4 + 3 for search 7), 2 CTAs/SM
//   5: 4 x 6, groups of three (3 + 3 + 1 for search 7), 2 CTAs/SM
//   6: 4 x 8, groups of four, 2 CTAs/SM
// FP16-storage form (row-pair layout, Kahan-compensated weight sum):
//   0: 4 x 6, 2 CTAs/SM;  1: 4 x 8, 2 CTAs/SM;  2: 2 x 8, 3 CTAs/SM
template <int m, int n>
static cudaError_t run_variant(const Staging& st, const void* staged, bool fp16, int v,
                               float inv_scale, float* out, float* zsum, unsigned int* ew,
                               cudaStream_t s, int zt0, int zt1) {
    if (!fp16) {
        switch (v) {
            case 0: return run_fwd3d<m, n, float, 4, 8, 4, 2, true, false>(st, staged, inv_scale, out, zsum, ew, s, zt0, zt1);
            case 1: return run_fwd3d<m, n, float, 4, 8, 4, 3, false, false>(st, staged, inv_scale, out, zsum, ew, s, zt0, zt1);
            case 2: return run_fwd3d<m, n, float, 4, 4, 4, 3, true, false>(st, staged, inv_scale, out, zsum, ew, s, zt0, zt1);
            case 3: return run_fwd3d<m, n, float, 2, 8, 4, 3, true, false>(st, staged, inv_scale, out, zsum, ew, s, zt0, zt1);
            case 4: return run_fwd3d_pz<m, n, 4, 6, 4, 2, 4>(st, staged, inv_scale, out, zsum, ew, s, zt0, zt1);
            case 5: return run_fwd3d_pz<m, n, 4, 6, 4, 2, 3>(st, staged, inv_scale, out, zsum, ew, s, zt0, zt1);
            case 6: return run_fwd3d_pz<m, n, 4, 8, 4, 2, 4>(st, staged, inv_scale, out, zsum, ew, s, zt0, zt1);
        }
    } else {
        switch (v) {
            case 0: return run_fwd3d_h2<m, n, 4, 6, 4, 2, true>(st, staged, inv_scale, out, zsum, ew, s, zt0, zt1);
            case 1: return run_fwd3d_h2<m, n, 4, 8, 4, 2, true>(st, staged, inv_scale, out, zsum, ew, s, zt0, zt1);
            case 2: return run_fwd3d_h2<m, n, 2, 8, 4, 3, true>(st, staged, inv_scale, out, zsum, ew, s, zt0, zt1);
        }
    }
    return cudaErrorInvalidValue;
}

int nlm3d_fwd_variant_count(bool fp16) { return fp16 ? 3 : 7; }

static bool small_case(int sr, int pr) {
#define X_(m, n) \
    if (sr == m && pr == n) return true;
    GNLM_FWD3D_CASES(X_)
#undef X_
    return false;
}

// Pairs without a register-brick instance run on the large-patch kernel (FP32 or
// plain FP16 staging).
bool nlm3d_fwd_large_patch(int sr, int pr, bool fp16) {
    (void)fp16;
    return !small_case(sr, pr) && nlm3d_lp_supported(sr, pr);
}

// Up to four accumulator buffers: the large-patch launcher may split each tile's passes
// into two halves (nlm3d_lp_split) and, from search radius 3, each pass's x offsets into
// two halves run by separate CTAs (kLpXHalf).  (Z, num) float2 per voxel, or with FP16
// storage the Kahan pairs (Z, num, cZ, cnum) float4.
size_t nlm3d_fwd_extra_bytes(int X, int Y, int Z, int sr, int pr, bool fp16) {
    if (!nlm3d_fwd_large_patch(sr, pr, fp16)) return 0;
    const size_t parts = sr >= 3 ? 4 : 2;
    return align_up(parts * X * Y * Z * (fp16 ? sizeof(float4) : sizeof(float2)), kAlign);
}

Staging staging3d(int X, int Y, int Z, int sr, int pr, bool fp16) {
    const int H = sr + pr;
    if (!fp16) return make_staging(X, Y, Z, H, H, false);
    return nlm3d_fwd_large_patch(sr, pr, true) ? make_staging(X, Y, Z, H, H, true)
                                               : make_staging_pairs(X, Y, Z, H);
}

int nlm3d_fwd_tile_z(int sr, int pr, bool fp16, int v) {
    static const int f32[7] = {8, 8, 4, 8, 6, 6, 8}, f16[3] = {6, 8, 8};
    if (v < 0 || v >= nlm3d_fwd_variant_count(fp16)) return 0;
    if (nlm3d_fwd_large_patch(sr, pr, fp16)) return nlm3d_lp_tile_z(v);
    return fp16 ? f16[v] : f32[v];
}

bool nlm3d_fwd_supported(int sr, int pr, bool fp16) {
    return small_case(sr, pr) || nlm3d_fwd_large_patch(sr, pr, fp16);
}

cudaError_t launch_nlm3d_fwd(const Staging& st, const void* staged, int sr, int pr, bool fp16,
                             int variant, float inv_scale, float* out, float* zsum,
                             unsigned int* errword, cudaStream_t stream, int zt0, int zt1) {
    if (variant < 0 || variant >= nlm3d_fwd_variant_count(fp16)) return cudaErrorInvalidValue;
#define X_(m, n)                                                                                \
    if (sr == m && pr == n)                                                                     \
        return run_variant<m, n>(st, staged, fp16, variant, inv_scale, out, zsum, errword, stream, \
                                 zt0, zt1);
    GNLM_FWD3D_CASES(X_)
#undef X_
    if (nlm3d_fwd_large_patch(sr, pr, fp16)) {
        void* acc = static_cast<char*>(const_cast<void*>(staged)) + st.bytes();
        return launch_nlm3d_lp(st, staged, sr, pr, fp16, variant, inv_scale, out, zsum, acc,
                               errword, stream, zt0, zt1);
    }
    return cudaErrorNotSupported;
}

}  // namespace gnlm
