// Allocation-free 3D forward: nlm3d_forward_noalloc (declared in include/nlm.h).
//
// Who needs it: some callers must never allocate device memory while they run.
// Examples are plug-ins hosted by an application that owns all of the GPU's memory
// through its own pool, and fixed-budget real-time imaging pipelines that reserve
// everything at start-up.  For them a cudaMalloc can fail in the middle of a scan,
// fragments the host's pool, and cudaFree stalls the whole device at a moment the
// caller does not choose.  nlm3d_forward with a NULL workspace allocates (it grows a
// cache with cudaMalloc); with a caller workspace it does not, but then the caller
// must allocate that workspace.  This entry point needs neither: the staging scratch
// lives in a fixed array compiled into this library.
//
// The array is kNoAllocScratchBytes (16 MiB) of device memory.  It is reserved on a
// device when this library's module is loaded there: at context creation with eager
// module loading, and at the latest by the first call of this entry point with CUDA's
// default lazy loading; from then on the device holds it until the process exits.
// A call whose staged volume needs more (padded (X+2H)(Y+2H)(Z+2H) voxels, H = sr + pr,
// 4 bytes each in FP32; FP16 storage keeps two row-paired copies of 2 bytes per voxel,
// so about the same; x rows rounded up to 16 bytes; the large-patch configurations add
// two (Z, num) float pairs per voxel) is rejected with NLM_ERR_WORKSPACE: for sr 3,
// pr 1 that is up to 152^3 (160^3 padded), FP32 or FP16 storage.
//
// Set-up: the first call in each context (one per device, the primary context, unless
// the caller makes its own) looks up the array's device address with
// cudaGetSymbolAddress while that device is current, and caches it under the
// context's unique ID; a device reset makes a new context, which gets a new lookup
// instead of a stale address.  That first call may also load the module, so make it
// before any stream capture.
//
// Every call on a device shares the one array, so calls whose GPU work overlaps (on two
// streams, or from two threads) race on it: serialise them, for example on one stream.
// The array keeps whatever the last call left in it.  Nothing needs to start at zero:
// the staging pass rewrites every byte that the NLM kernels later read, and the
// large-patch accumulators are written before they are read.
#include <cuda_runtime.h>
#include <stdio.h>

#include <map>
#include <mutex>

#include "../../include/nlm.h"
#include "nlm_internal.h"

namespace gnlm {

constexpr size_t kNoAllocScratchBytes = size_t(16) << 20;

// File-scope scratch.  In host code this name is only a host-side stand-in for the
// symbol, not a device address: the address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

namespace {
std::mutex g_noalloc_mu;
std::map<unsigned long long, void*> g_noalloc_addr;  // context ID -> device address

// Device address of the array in the calling thread's current context.
int noalloc_scratch(void** out) {
    unsigned long long ctx = 0;
    bool have_ctx = current_context_id(&ctx);
    if (have_ctx) {
        std::lock_guard<std::mutex> lk(g_noalloc_mu);
        auto it = g_noalloc_addr.find(ctx);
        if (it != g_noalloc_addr.end()) {
            *out = it->second;
            return NLM_OK;
        }
    }
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress((void**)&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
        cudaGetLastError();
        char msg[160];
        snprintf(msg, sizeof(msg), "cudaGetSymbolAddress(scratch) failed: %s",
                 cudaGetErrorString(e));
        return report_error(NLM_ERR_CUDA, msg);
    }
    if (!have_ctx) have_ctx = current_context_id(&ctx);  // the lookup made one current
    if (have_ctx) {
        std::lock_guard<std::mutex> lk(g_noalloc_mu);
        g_noalloc_addr[ctx] = p;
    }
    *out = p;
    return NLM_OK;
}
}  // namespace

}  // namespace gnlm

extern "C" int nlm3d_forward_noalloc(const void* d_in, int in_dtype, int X, int Y, int Z, int sr,
                                     int pr, float h, float* d_out, float* d_zsum,
                                     unsigned int flags, nlm_stream_t stream) {
    using namespace gnlm;
    // The same argument checks as nlm3d_forward, before the size check, so that a bad
    // pointer, dtype, radius, h or flag is reported as such whatever the volume's size.
    int rc = validate_forward3d(d_in, d_out, in_dtype, X, Y, Z, sr, pr, h, flags);
    if (rc != NLM_OK) return rc;
    const size_t need = nlm3d_workspace_bytes(X, Y, Z, sr, pr, flags);
    if (need > kNoAllocScratchBytes) {
        char msg[200];
        snprintf(msg, sizeof(msg),
                 "volume needs %zu bytes of staging scratch; the allocation-free entry point "
                 "holds at most %zu (use nlm3d_forward with a workspace)",
                 need, kNoAllocScratchBytes);
        return report_error(NLM_ERR_WORKSPACE, msg);
    }
    void* scratch = nullptr;
    if ((rc = noalloc_scratch(&scratch)) != NLM_OK) return rc;
    // With a caller-provided workspace nlm3d_forward neither allocates nor frees.
    return nlm3d_forward(d_in, in_dtype, X, Y, Z, sr, pr, h, d_out, d_zsum, flags, scratch,
                         kNoAllocScratchBytes, stream);
}
