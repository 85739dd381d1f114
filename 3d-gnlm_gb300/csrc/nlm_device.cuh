// Device-side building blocks shared by the NLM kernels (sm_103a):
// TMA tile loads, mbarrier waits with an iteration limit, the MUFU ex2 weight,
// and the device error word.
#pragma once

#include <cuda.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace gnlm {

// Bits of the device error word (one 32-bit word per device, see nlm_abi.cu).
enum : unsigned int {
    DEVERR_TMA_TIMEOUT = 0x1u,     // a tile load did not complete within the wait limit
    DEVERR_QUEUE_TIMEOUT = 0x2u,   // reserved: the batch work queue takes items with one
                                   // atomicAdd and never waits, so no kernel sets this bit
    DEVERR_BAD_DESC = 0x4u,        // a work item failed its own bounds check
    DEVERR_BOUNDS = 0x8u,          // NLM_BOUNDS_CHECK build: an index range left its buffer
};

// The word after the error word is a control word that only NLM_BOUNDS_CHECK builds
// (the test library libgnlm_checked.so) read: with FAULT_SKIP_TILE_COPY set, the CTA of
// tile (0, 0, 0) of each 3D/2D forward or adjoint launch arms its barrier for the tile
// copy but never issues the copy, so its bounded wait runs out exactly as it would for
// a copy that never lands (the large-patch kernel: the CTA at grid origin, for the planes
// of its first step).  Nothing is in flight for that barrier when the CTA gives up, and
// its wait limit is kInjectedWaitPolls so the test does not spend the full limit.
enum : unsigned int { FAULT_SKIP_TILE_COPY = 0x1u };

// Builds compiled with -DNLM_BOUNDS_CHECK verify, once per tile or work item, that
// the whole index range a thread is about to touch lies inside its buffer; a
// violation sets DEVERR_BOUNDS and the caller redirects the thread to a range
// known to be valid (no access leaves the buffer, no thread leaves a warp-wide
// shuffle).  In normal builds the check compiles to nothing.
#ifdef NLM_BOUNDS_CHECK
constexpr bool kBoundsCheck = true;
#else
constexpr bool kBoundsCheck = false;
#endif

__device__ __forceinline__ void raise_device_error(unsigned int* word, unsigned int bits);

// true when [lo, hi] lies inside [0, n) (always true unless NLM_BOUNDS_CHECK)
__device__ __forceinline__ bool range_ok(unsigned int* errword, long long lo, long long hi,
                                         long long n) {
    if constexpr (kBoundsCheck) {
        if (lo < 0 || hi >= n) {
            raise_device_error(errword, DEVERR_BOUNDS);
            return false;
        }
    }
    return true;
}

// Upper bound on mbarrier.try_wait polls before a wait gives up.  Each poll may
// suspend the thread for a hardware-defined interval, so this bounds the wait
// at well under a second on a healthy device.
constexpr uint32_t kMaxWaitPolls = 1u << 22;
constexpr uint32_t kInjectedWaitPolls = 1u << 10;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
                 : "memory");
}

// Makes the initialised barrier visible to the async (TMA) proxy.
__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Waits for phase `parity` of `bar` with an iteration limit.  Returns false if
// the limit ran out (the caller records the error and abandons the tile).
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity,
                                                  uint32_t polls = kMaxWaitPolls) {
    for (uint32_t i = 0; i < polls; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// True in the CTA that must skip its tile copy (see FAULT_SKIP_TILE_COPY); always
// false outside NLM_BOUNDS_CHECK builds.  Uniform over the CTA.
__device__ __forceinline__ bool inject_skip_copy(const unsigned int* errword, int bx, int by,
                                                 int bz) {
    if constexpr (kBoundsCheck) {
        if (errword && (bx | by | bz) == 0)
            return (*reinterpret_cast<const volatile unsigned int*>(errword + 1) &
                    FAULT_SKIP_TILE_COPY) != 0;
    }
    return false;
}

__device__ __forceinline__ void raise_device_error(unsigned int* word, unsigned int bits);

// Waits for the tile copy of phase `parity`.  If the wait runs out, thread 0 records
// DEVERR_TMA_TIMEOUT and waits once more for a copy that may still be landing, and the
// caller abandons the tile (false).  `skipped`: the copy was never issued (test hook).
__device__ __forceinline__ bool tile_copy_wait(uint64_t* bar, uint32_t parity,
                                               unsigned int* errword, bool skipped) {
    const uint32_t polls = skipped ? kInjectedWaitPolls : kMaxWaitPolls;
    if (mbar_wait_bounded(bar, parity, polls)) return true;
    if (threadIdx.x == 0) {
        raise_device_error(errword, DEVERR_TMA_TIMEOUT);
        mbar_wait_bounded(bar, parity, polls);
    }
    return false;
}

// 3D tiled TMA load of one box into shared memory, completing on `bar`.
// Coordinates are element indices (x innermost); x * sizeof(elem) must be a
// multiple of 16 bytes, which every caller guarantees by rounding x down.
__device__ __forceinline__ void tma_load_3d(void* smem_dst, const CUtensorMap* map, int x, int y,
                                            int z, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(smem_dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void tma_load_2d(void* smem_dst, const CUtensorMap* map, int x, int y,
                                            uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(smem_dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

// 2^(-x) on the MUFU pipe (PTX ex2.approx.ftz.f32: about 2 ulp; 0 for large x).
__device__ __forceinline__ float ex2_neg(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(-x));
    return y;
}

__device__ __forceinline__ float to_f32(float v) { return v; }
__device__ __forceinline__ float to_f32(__half v) { return __half2float(v); }
__device__ __forceinline__ float to_f32(unsigned char v) { return static_cast<float>(v); }

template <typename T>
__device__ __forceinline__ T from_f32(float v);
template <>
__device__ __forceinline__ float from_f32<float>(float v) { return v; }
template <>
__device__ __forceinline__ __half from_f32<__half>(float v) { return __float2half_rn(v); }

// OpenCV BORDER_REFLECT_101 for any offset (repeated reflection, period 2n-2).
__host__ __device__ __forceinline__ int reflect101(int i, int n) {
    if (n <= 1) return 0;
    const int period = 2 * n - 2;
    i %= period;
    if (i < 0) i += period;
    return i < n ? i : period - i;
}

// reflect101 with the common case first: one reflection on each side covers
// -n < i < 2n - 1 with two compares and no division; other offsets fall back.
__device__ __forceinline__ int reflect101_near(int i, int n) {
    int r = i < 0 ? -i : i;
    r = r >= n ? 2 * n - 2 - r : r;
    return (unsigned)r < (unsigned)n ? r : reflect101(i, n);
}

// Sum of y over the lanes [l - N, l + N] (valid for lanes N .. 31 - N).  N = 1: two
// shuffles; N = 2: three (from pair sums); wider windows are assembled from
// power-of-two window sums, e.g. 11 = 8 + 2 + 1 takes 6 shuffles instead of 10.
template <int N>
__device__ __forceinline__ float xbox_lanes(float y) {
    if constexpr (N == 2) {
        // P = y(l) + y(l+1); box = P(l-2) + P(l) + y(l+2): three shuffles
        const float yr = __shfl_down_sync(0xffffffffu, y, 1);
        const float p = y + yr;
        return __shfl_up_sync(0xffffffffu, p, 2) + p + __shfl_down_sync(0xffffffffu, y, 2);
    } else if constexpr (N <= 2) {
        float x = y;
#pragma unroll
        for (int k = 1; k <= N; ++k)
            x += __shfl_down_sync(0xffffffffu, y, k) + __shfl_up_sync(0xffffffffu, y, k);
        return x;
    } else {
        constexpr int K = 2 * N + 1;
        float p[5];  // p[j] = sum over lanes l .. l + 2^j - 1
        p[0] = y;
#pragma unroll
        for (int j = 1; j < 5; ++j)
            p[j] = (1 << j) <= K ? p[j - 1] + __shfl_down_sync(0xffffffffu, p[j - 1], 1 << (j - 1))
                                 : 0.f;
        float x = 0.f;
        int start = -N;  // window start relative to this lane
#pragma unroll
        for (int j = 4; j >= 0; --j) {
            if (K & (1 << j)) {
                x += start < 0 ? __shfl_up_sync(0xffffffffu, p[j], -start)
                               : (start == 0 ? p[j] : __shfl_down_sync(0xffffffffu, p[j], start));
                start += 1 << j;
            }
        }
        return x;
    }
}

__device__ __forceinline__ void raise_device_error(unsigned int* word, unsigned int bits) {
    if (word) atomicOr(word, bits);
}

}  // namespace gnlm
