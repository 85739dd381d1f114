// Staging pass: REFLECT_101 padding + dtype conversion + exponent pre-scaling.
//
// Replaces the host-side padding of the reference's driver
// (3DNLM/nlm.cpp:36-61: copyMakeBorder(BORDER_REFLECT_101) in x/y, slice
// replication in z; 2D NLM/11x11/nlm.cpp:15-19) with one HBM-streaming kernel
// that reflects on every axis.  It reads the input once and writes the padded
// copy once: algorithmic traffic = X*Y*Z*in_bytes + Xs*Yp*Zp*elem.
#include <cuda_fp16.h>
#include <stdint.h>

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

// Row-pair layout: block = (pair k, plane, copy c); rows 2k+c and 2k+c+1.
template <typename Tin, bool PREPADDED>
__global__ void __launch_bounds__(256) stage_pairs_kernel(const Tin* __restrict__ in, int X, int Y,
                                                          int Z, int H, int Xp, int Yp, int Xs,
                                                          int Yq, size_t copy_elems, float scale,
                                                          __half2* __restrict__ dst, int pz0) {
    const int k = blockIdx.x, pz = blockIdx.y + pz0, c = blockIdx.z;
    const int r0 = 2 * k + c, r1 = r0 + 1;
    __half2* drow = dst + c * copy_elems + ((size_t)pz * Yq + k) * Xs;
    const Tin *s0 = nullptr, *s1 = nullptr;
    if (PREPADDED) {
        if (r0 < Yp) s0 = in + ((size_t)pz * Yp + r0) * Xp;
        if (r1 < Yp) s1 = in + ((size_t)pz * Yp + r1) * Xp;
    } else {
        const int sz = reflect101(pz - H, Z);
        if (r0 < Yp) s0 = in + ((size_t)sz * Y + reflect101(r0 - H, Y)) * X;
        if (r1 < Yp) s1 = in + ((size_t)sz * Y + reflect101(r1 - H, Y)) * X;
    }
    for (int px = threadIdx.x; px < Xs; px += blockDim.x) {
        float v0 = 0.f, v1 = 0.f;
        if (px < Xp) {
            const int sx = PREPADDED ? px : reflect101(px - H, X);
            if (s0) v0 = to_f32(s0[sx]) * scale;
            if (s1) v1 = to_f32(s1[sx]) * scale;
        }
        drow[px] = __floats2half2_rn(v0, v1);
    }
}

template <typename Tin>
static cudaError_t stage_pairs_typed(const void* in, bool prepadded, float scale, const Staging& st,
                                     void* dst, cudaStream_t stream, int pz0, int pz1) {
    dim3 grid(st.Yq, pz1 - pz0, 2);
    const size_t copy_elems = st.copy_bytes() / 4;
    if (prepadded)
        stage_pairs_kernel<Tin, true><<<grid, 256, 0, stream>>>(
            (const Tin*)in, st.X, st.Y, st.Z, st.H, st.Xp, st.Yp, st.Xs, st.Yq, copy_elems, scale,
            (__half2*)dst, pz0);
    else
        stage_pairs_kernel<Tin, false><<<grid, 256, 0, stream>>>(
            (const Tin*)in, st.X, st.Y, st.Z, st.H, st.Xp, st.Yp, st.Xs, st.Yq, copy_elems, scale,
            (__half2*)dst, pz0);
    return cudaGetLastError();
}

// Warp per padded row (8 rows per 256-thread block, rows flattened over planes).
// Each lane writes 16-byte vectors (4 FP32 or 8 FP16 values); columns inside the
// volume map to the source row directly, only the 2H border columns reflect.
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

// VEC: every source row starts on a multiple of V::N elements and the halo H is one
// too (not prepadded), so the chunks that lie inside the source row are one vector
// load each; the 2H border columns and the stride padding take the scalar path.
template <typename Tin, typename Tout, bool PREPADDED, bool VEC>
__global__ void __launch_bounds__(256) stage_kernel(const Tin* __restrict__ in, int X, int Y,
                                                    int Z, int H, int Hz, int Xp, int Yp,
                                                    long long row0, long long row1, int Xs,
                                                    float scale, Tout* __restrict__ dst) {
    using V = Vec16<Tout>;
    const long long row = row0 + (long long)blockIdx.x * 8 + (threadIdx.x >> 5);
    if (row >= row1) return;
    const int lane = threadIdx.x & 31;
    const int py = (int)(row % Yp), pz = (int)(row / Yp);
    typename V::T* drow = reinterpret_cast<typename V::T*>(dst + row * Xs);
    const Tin* srow;
    if (PREPADDED) {
        srow = in + row * Xp;
    } else {
        const int sz = reflect101(pz - Hz, Z);
        const int sy = reflect101(py - H, Y);
        srow = in + ((size_t)sz * Y + sy) * X;
    }
    const int sh = PREPADDED ? 0 : H;      // source column = padded column - sh
    const int slen = PREPADDED ? Xp : X;   // source row length
    auto chunk = [&](int c, float* v) {
        const int px0 = c * V::N;
        if (VEC && px0 >= sh && px0 - sh + V::N <= slen) {
            load_vec<Tin, V::N>(srow + (px0 - sh), v);
        } else {
#pragma unroll
            for (int i = 0; i < V::N; ++i) {
                const int px = px0 + i;
                float x = 0.f;
                if (px < Xp) {
                    int sx = px;
                    if (!PREPADDED) {
                        sx = px - H;
                        if (sx < 0 || sx >= X) sx = reflect101(sx, X);
                    }
                    x = to_f32(srow[sx]);
                }
                v[i] = x;
            }
        }
#pragma unroll
        for (int i = 0; i < V::N; ++i) v[i] *= scale;
    };
    // two chunks per iteration, both loads issued before either store
    const int nchunk = Xs / V::N;
    int c = lane;
    for (; c + 32 < nchunk; c += 64) {
        float v0[V::N], v1[V::N];
        chunk(c, v0);
        chunk(c + 32, v1);
        drow[c] = V::pack(v0);
        drow[c + 32] = V::pack(v1);
    }
    if (c < nchunk) {
        float v0[V::N];
        chunk(c, v0);
        drow[c] = V::pack(v0);
    }
}

template <typename Tin, typename Tout>
static cudaError_t stage_typed(const void* in, bool prepadded, float scale, const Staging& st,
                               void* dst, cudaStream_t stream, int pz0, int pz1) {
    const long long row0 = (long long)st.Yp * pz0, row1 = (long long)st.Yp * pz1;
    const unsigned blocks = (unsigned)((row1 - row0 + 7) / 8);
    constexpr int NV = Vec16<Tout>::N;
    const size_t vbytes = sizeof(Tin) * NV;
    const bool vec = reinterpret_cast<uintptr_t>(in) % vbytes == 0 &&
                     (prepadded ? st.Xp % NV == 0 : (st.X % NV == 0 && st.H % NV == 0));
#define GNLM_STAGE_LAUNCH(P, VEC)                                                              \
    stage_kernel<Tin, Tout, P, VEC><<<blocks, 256, 0, stream>>>(                                \
        (const Tin*)in, st.X, st.Y, st.Z, st.H, st.Hz, st.Xp, st.Yp, row0, row1, st.Xs, scale, \
        (Tout*)dst)
    if (prepadded) {
        if (vec) GNLM_STAGE_LAUNCH(true, true); else GNLM_STAGE_LAUNCH(true, false);
    } else {
        if (vec) GNLM_STAGE_LAUNCH(false, true); else GNLM_STAGE_LAUNCH(false, false);
    }
#undef GNLM_STAGE_LAUNCH
    return cudaGetLastError();
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
