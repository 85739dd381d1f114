// Staging pass: REFLECT_101 padding + dtype conversion + exponent pre-scaling.
//
// Replaces the host-side padding of the reference's driver
// (3DNLM/nlm.cpp:36-61: copyMakeBorder(BORDER_REFLECT_101) in x/y, slice
// replication in z; 2D NLM/11x11/nlm.cpp:15-19) with one HBM-streaming kernel
// that reflects on every axis.  It reads the input once and writes the padded
// copy once: algorithmic traffic = X*Y*Z*in_bytes + Xs*Yp*Zp*elem.
#include <cuda_fp16.h>
#include <stdint.h>

#include <algorithm>

#include "../../include/nlm.h"
#include "nlm_device.cuh"
#include "nlm_internal.h"

namespace gnlm {

Staging make_staging(int X, int Y, int Z, int H, int Hz, bool fp16) {
    Staging s;
    s.X = X;
    s.Y = Y;
    s.Z = Z;
    s.H = H;
    s.Hz = Hz;
    s.Xp = X + 2 * H;
    s.Yp = Y + 2 * H;
    s.Zp = Z + 2 * Hz;
    s.elem = fp16 ? 2 : 4;
    const int per16 = 16 / s.elem;
    s.Xs = (s.Xp + per16 - 1) / per16 * per16;
    return s;
}

Staging make_staging_pairs(int X, int Y, int Z, int H) {
    Staging s = make_staging(X, Y, Z, H, H, false);
    s.pairs = true;
    s.elem = 4;
    s.Xs = (s.Xp + 3) / 4 * 4;  // half2 elements, 16-byte rows
    s.Yq = (s.Yp + 2) / 2;
    return s;
}

// One 16-byte output chunk: 4 FP32 or 8 FP16 values.
template <typename Tout>
struct Vec16;
template <>
struct Vec16<float> {
    static constexpr int N = 4;
    using T = float4;
    __device__ static T pack(const float* v) { return make_float4(v[0], v[1], v[2], v[3]); }
};
template <>
struct Vec16<__half> {
    static constexpr int N = 8;
    using T = uint4;
    __device__ static T pack(const float* v) {
        uint4 r;
        __half2 h0 = __floats2half2_rn(v[0], v[1]), h1 = __floats2half2_rn(v[2], v[3]);
        __half2 h2 = __floats2half2_rn(v[4], v[5]), h3 = __floats2half2_rn(v[6], v[7]);
        r.x = *reinterpret_cast<unsigned int*>(&h0);
        r.y = *reinterpret_cast<unsigned int*>(&h1);
        r.z = *reinterpret_cast<unsigned int*>(&h2);
        r.w = *reinterpret_cast<unsigned int*>(&h3);
        return r;
    }
};

// NV consecutive input elements as floats in one vector load (the address is a
// multiple of NV * sizeof(Tin), checked by the launcher).
template <typename Tin, int NV>
__device__ __forceinline__ void load_vec(const Tin* p, float* v) {
    if constexpr (sizeof(Tin) * NV == 16) {
        const uint4 u = *reinterpret_cast<const uint4*>(p);
        const Tin* e = reinterpret_cast<const Tin*>(&u);
#pragma unroll
        for (int i = 0; i < NV; ++i) v[i] = to_f32(e[i]);
    } else if constexpr (sizeof(Tin) * NV == 32) {
        const uint4 u0 = *reinterpret_cast<const uint4*>(p);
        const uint4 u1 = *reinterpret_cast<const uint4*>(p + NV / 2);
        const Tin* e0 = reinterpret_cast<const Tin*>(&u0);
        const Tin* e1 = reinterpret_cast<const Tin*>(&u1);
#pragma unroll
        for (int i = 0; i < NV / 2; ++i) {
            v[i] = to_f32(e0[i]);
            v[NV / 2 + i] = to_f32(e1[i]);
        }
    } else if constexpr (sizeof(Tin) * NV == 8) {
        const uint2 u = *reinterpret_cast<const uint2*>(p);
        const Tin* e = reinterpret_cast<const Tin*>(&u);
#pragma unroll
        for (int i = 0; i < NV; ++i) v[i] = to_f32(e[i]);
    } else {
        static_assert(sizeof(Tin) * NV == 4, "vector width");
        const unsigned int u = *reinterpret_cast<const unsigned int*>(p);
        const Tin* e = reinterpret_cast<const Tin*>(&u);
#pragma unroll
        for (int i = 0; i < NV; ++i) v[i] = to_f32(e[i]);
    }
}

// Staging kernels, both layouts.  A warp copies whole padded rows: each lane owns the
// 16-byte output chunks at indices lane, lane + 32, ... of a row (the chunk order is
// rotated, see `rot` in the kernels) and issues the loads of all
// its chunks of kStageRows rows (kStageSlots per row and pass) before the first
// store, so a warp keeps about 2 KB in flight.  Blocks stay resident (grid = SMs x
// blocks per SM) and stride over row groups; a thread divides once, at the start,
// and then advances its (row, plane) by adds.  Columns inside the volume map to the
// source row directly (VEC: one vector load per chunk); only the 2H border columns
// reflect, without divisions in the common case (reflect101_near).  Row indices are
// 32-bit: the launcher splits launches to at most 2^30 rows.
constexpr int kStageRows = 2;
constexpr int kStageSlots = 3;  // a row of up to 96 chunks (1.5 KB) in one pass

template <typename Tin, int NV, bool PREPADDED, bool VEC>
__device__ __forceinline__ void stage_chunk(const Tin* srow, int px0, int X, int H, int Xp,
                                            float* v) {
    const int sh = PREPADDED ? 0 : H;      // source column = padded column - sh
    const int slen = PREPADDED ? Xp : X;   // source row length
    if (VEC && px0 >= sh && px0 - sh + NV <= slen) {
        load_vec<Tin, NV>(srow + (px0 - sh), v);
    } else {
#pragma unroll
        for (int i = 0; i < NV; ++i) {
            const int px = px0 + i;
            float x = 0.f;
            if (px < Xp) x = to_f32(srow[PREPADDED ? px : reflect101_near(px - H, X)]);
            v[i] = x;
        }
    }
}

// Resident blocks of 256 threads for a staging kernel instance: SMs x blocks per SM
// (the occupancy is queried once per instance).
template <auto Kernel>
static unsigned stage_grid(long long groups) {
    static const int per_sm = [] {
        int n = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, Kernel, 256, 0) != cudaSuccess ||
            n <= 0) {
            cudaGetLastError();  // consume a non-sticky error; fall back to one block per SM
            n = 1;
        }
        return n;
    }();
    const long long resident = (long long)device_sm_count() * per_sm;
    return (unsigned)std::max<long long>(1, std::min(groups, resident));
}

// Plain layout [Zp][Yp][Xs]: rows of planes [pz0, pz0 + nplanes), kStageRows per warp.
template <typename Tin, typename Tout, bool PREPADDED, bool VEC>
__global__ void __launch_bounds__(256) stage_kernel(const Tin* __restrict__ in, int X, int Y,
                                                    int Z, int H, int Hz, int Xp, int Yp, int pz0,
                                                    int nplanes, int Xs, float scale,
                                                    Tout* __restrict__ dst) {
    using V = Vec16<Tout>;
    const int lane = threadIdx.x & 31;
    const int nrows = nplanes * Yp;
    const int nchunk = Xs / V::N;
    // Lane order rotated by the chunks past the source row's end: index i holds chunk
    // (i - rot) mod nchunk, so the right and left border chunks (the scalar reflect
    // path) fall in the first slot of neighbouring lanes and a row diverges once.
    const int rot = PREPADDED ? 0 : nchunk - min(nchunk, (X + H) / V::N);
    auto chunk_of = [&](int i) { return i < rot ? i + nchunk - rot : i - rot; };
    const int wstep = gridDim.x * 8 * kStageRows;
    int rb = (blockIdx.x * 8 + (threadIdx.x >> 5)) * kStageRows;
    int py = rb % Yp, pz = pz0 + rb / Yp;  // of row rb
    const int dpy = wstep % Yp, dpz = wstep / Yp;
    for (; rb < nrows; rb += wstep) {
        const Tin* srow[kStageRows];
        typename V::T* drow[kStageRows];
        bool live[kStageRows];
#pragma unroll
        for (int r = 0; r < kStageRows; ++r) {
            live[r] = rb + r < nrows;
            int ry = py + (live[r] ? r : 0), rz = pz;
            while (ry >= Yp) {
                ry -= Yp;
                ++rz;
            }
            drow[r] = reinterpret_cast<typename V::T*>(dst + ((size_t)rz * Yp + ry) * Xs);
            srow[r] = PREPADDED ? in + ((size_t)rz * Yp + ry) * Xp
                                : in + ((size_t)reflect101_near(rz - Hz, Z) * Y +
                                        reflect101_near(ry - H, Y)) * X;
        }
        for (int c0 = lane; c0 < nchunk; c0 += 32 * kStageSlots) {
            float v[kStageRows][kStageSlots][V::N];
#pragma unroll
            for (int r = 0; r < kStageRows; ++r)
#pragma unroll
                for (int k = 0; k < kStageSlots; ++k)
                    if (live[r] && c0 + 32 * k < nchunk)
                        stage_chunk<Tin, V::N, PREPADDED, VEC>(
                            srow[r], chunk_of(c0 + 32 * k) * V::N, X, H, Xp, v[r][k]);
#pragma unroll
            for (int r = 0; r < kStageRows; ++r)
#pragma unroll
                for (int k = 0; k < kStageSlots; ++k)
                    if (live[r] && c0 + 32 * k < nchunk) {
#pragma unroll
                        for (int i = 0; i < V::N; ++i) v[r][k][i] *= scale;
                        drow[r][chunk_of(c0 + 32 * k)] = V::pack(v[r][k]);
                    }
        }
        py += dpy;
        pz += dpz;
        while (py >= Yp) {
            py -= Yp;
            ++pz;
        }
    }
}

// Row-pair layout: copy c, plane pz, pair k holds the padded rows 2k+c and 2k+c+1 as
// half2.  A warp takes one (plane, pair k) per step and writes both copies' rows
// from the three source rows 2k, 2k+1, 2k+2 (read once, instead of once per copy);
// a 16-byte chunk is 4 columns.
template <typename Tin, bool PREPADDED, bool VEC>
__global__ void __launch_bounds__(256) stage_pairs_kernel(const Tin* __restrict__ in, int X, int Y,
                                                          int Z, int H, int Xp, int Yp, int Xs,
                                                          int Yq, size_t copy_elems, float scale,
                                                          __half2* __restrict__ dst, int pz0,
                                                          int nplanes) {
    const int lane = threadIdx.x & 31;
    const int npairs = nplanes * Yq;
    const int nchunk = Xs / 4;
    // border chunks in the first slot of neighbouring lanes (as in stage_kernel)
    const int rot = PREPADDED ? 0 : nchunk - min(nchunk, (X + H) / 4);
    auto chunk_of = [&](int i) { return i < rot ? i + nchunk - rot : i - rot; };
    const int wstep = gridDim.x * 8;
    int q = blockIdx.x * 8 + (threadIdx.x >> 5);
    int k = q % Yq, pz = pz0 + q / Yq;
    const int dk = wstep % Yq, dpz = wstep / Yq;
    for (; q < npairs; q += wstep) {
        const Tin* src[3];
#pragma unroll
        for (int e = 0; e < 3; ++e) {
            const int row = 2 * k + e;
            src[e] = nullptr;
            if (row < Yp)
                src[e] = PREPADDED ? in + ((size_t)pz * Yp + row) * Xp
                                   : in + ((size_t)reflect101_near(pz - H, Z) * Y +
                                           reflect101_near(row - H, Y)) * X;
        }
        uint4* drow0 = reinterpret_cast<uint4*>(dst + ((size_t)pz * Yq + k) * Xs);
        uint4* drow1 = reinterpret_cast<uint4*>(dst + copy_elems + ((size_t)pz * Yq + k) * Xs);
        for (int c0 = lane; c0 < nchunk; c0 += 32 * kStageSlots) {
            float v[kStageSlots][3][4];
#pragma unroll
            for (int j = 0; j < kStageSlots; ++j)
                if (c0 + 32 * j < nchunk) {
#pragma unroll
                    for (int e = 0; e < 3; ++e) {
                        if (src[e])
                            stage_chunk<Tin, 4, PREPADDED, VEC>(src[e], chunk_of(c0 + 32 * j) * 4, X,
                                                                H, Xp, v[j][e]);
                        else
#pragma unroll
                            for (int i = 0; i < 4; ++i) v[j][e][i] = 0.f;
                    }
                }
#pragma unroll
            for (int j = 0; j < kStageSlots; ++j)
                if (c0 + 32 * j < nchunk) {
                    unsigned int w0[4], w1[4];
#pragma unroll
                    for (int i = 0; i < 4; ++i) {
                        const float a = v[j][0][i] * scale, b = v[j][1][i] * scale,
                                    c = v[j][2][i] * scale;
                        const __half2 e0 = __floats2half2_rn(a, b), e1 = __floats2half2_rn(b, c);
                        w0[i] = *reinterpret_cast<const unsigned int*>(&e0);
                        w1[i] = *reinterpret_cast<const unsigned int*>(&e1);
                    }
                    drow0[chunk_of(c0 + 32 * j)] = make_uint4(w0[0], w0[1], w0[2], w0[3]);
                    drow1[chunk_of(c0 + 32 * j)] = make_uint4(w1[0], w1[1], w1[2], w1[3]);
                }
        }
        k += dk;
        pz += dpz;
        while (k >= Yq) {
            k -= Yq;
            ++pz;
        }
    }
}

// Planes per launch so that a launch covers at most 2^30 rows: row indices, and a row
// index plus a grid stride, stay within 32 bits.
static int stage_planes_per_launch(long long rows_per_plane) {
    return (int)std::max<long long>(1, (1LL << 30) / std::max<long long>(1, rows_per_plane));
}

template <typename Tin>
static cudaError_t stage_pairs_typed(const void* in, bool prepadded, float scale, const Staging& st,
                                     void* dst, cudaStream_t stream, int pz0, int pz1) {
    const size_t copy_elems = st.copy_bytes() / 4;
    const bool vec = reinterpret_cast<uintptr_t>(in) % (4 * sizeof(Tin)) == 0 &&
                     (prepadded ? st.Xp % 4 == 0 : (st.X % 4 == 0 && st.H % 4 == 0));
    const int step = stage_planes_per_launch(st.Yq);
    for (int p0 = pz0; p0 < pz1; p0 += step) {
        const int np = std::min(step, pz1 - p0);
        const long long groups = ((long long)np * st.Yq + 7) / 8;
#define GNLM_PAIRS_LAUNCH(P, VEC)                                                                  \
    stage_pairs_kernel<Tin, P, VEC><<<stage_grid<stage_pairs_kernel<Tin, P, VEC>>(groups), 256, 0, \
                                      stream>>>((const Tin*)in, st.X, st.Y, st.Z, st.H, st.Xp,      \
                                                st.Yp, st.Xs, st.Yq, copy_elems, scale,             \
                                                (__half2*)dst, p0, np)
        if (prepadded) {
            if (vec) GNLM_PAIRS_LAUNCH(true, true); else GNLM_PAIRS_LAUNCH(true, false);
        } else {
            if (vec) GNLM_PAIRS_LAUNCH(false, true); else GNLM_PAIRS_LAUNCH(false, false);
        }
#undef GNLM_PAIRS_LAUNCH
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

template <typename Tin, typename Tout>
static cudaError_t stage_typed(const void* in, bool prepadded, float scale, const Staging& st,
                               void* dst, cudaStream_t stream, int pz0, int pz1) {
    constexpr int NV = Vec16<Tout>::N;
    const size_t vbytes = sizeof(Tin) * NV;
    const bool vec = reinterpret_cast<uintptr_t>(in) % vbytes == 0 &&
                     (prepadded ? st.Xp % NV == 0 : (st.X % NV == 0 && st.H % NV == 0));
    const int step = stage_planes_per_launch(st.Yp);
    for (int p0 = pz0; p0 < pz1; p0 += step) {
        const int np = std::min(step, pz1 - p0);
        const long long groups = ((long long)np * st.Yp + 8 * kStageRows - 1) / (8 * kStageRows);
#define GNLM_STAGE_LAUNCH(P, VEC)                                                                   \
    stage_kernel<Tin, Tout, P, VEC><<<stage_grid<stage_kernel<Tin, Tout, P, VEC>>(groups), 256, 0, \
                                      stream>>>((const Tin*)in, st.X, st.Y, st.Z, st.H, st.Hz,      \
                                                st.Xp, st.Yp, p0, np, st.Xs, scale, (Tout*)dst)
        if (prepadded) {
            if (vec) GNLM_STAGE_LAUNCH(true, true); else GNLM_STAGE_LAUNCH(true, false);
        } else {
            if (vec) GNLM_STAGE_LAUNCH(false, true); else GNLM_STAGE_LAUNCH(false, false);
        }
#undef GNLM_STAGE_LAUNCH
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t launch_stage(const void* in, int in_dtype, bool prepadded, float scale,
                         const Staging& st, void* dst, cudaStream_t stream, int pz0, int pz1) {
    if (pz1 < 0 || pz1 > st.Zp) pz1 = st.Zp;
    if (pz0 < 0) pz0 = 0;
    if (pz1 <= pz0) return cudaSuccess;
    if (st.pairs) {
        switch (in_dtype) {
            case NLM_U8: return stage_pairs_typed<unsigned char>(in, prepadded, scale, st, dst, stream, pz0, pz1);
            case NLM_F16: return stage_pairs_typed<__half>(in, prepadded, scale, st, dst, stream, pz0, pz1);
            case NLM_F32: return stage_pairs_typed<float>(in, prepadded, scale, st, dst, stream, pz0, pz1);
            default: return cudaErrorInvalidValue;
        }
    }
    const bool fp16 = st.elem == 2;
    switch (in_dtype) {
        case NLM_U8:
            return fp16 ? stage_typed<unsigned char, __half>(in, prepadded, scale, st, dst, stream, pz0, pz1)
                        : stage_typed<unsigned char, float>(in, prepadded, scale, st, dst, stream, pz0, pz1);
        case NLM_F16:
            return fp16 ? stage_typed<__half, __half>(in, prepadded, scale, st, dst, stream, pz0, pz1)
                        : stage_typed<__half, float>(in, prepadded, scale, st, dst, stream, pz0, pz1);
        case NLM_F32:
            return fp16 ? stage_typed<float, __half>(in, prepadded, scale, st, dst, stream, pz0, pz1)
                        : stage_typed<float, float>(in, prepadded, scale, st, dst, stream, pz0, pz1);
        default:
            return cudaErrorInvalidValue;
    }
}

}  // namespace gnlm
