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
// The array is kNoAllocScratchBytes (16 MiB) of device memory.  Every GPU that loads
// the library holds it until the process exits, whether or not this entry point is
// ever called.  A call whose staged volume needs more (padded (X+2H)(Y+2H)(Z+2H)
// voxels, H = sr + pr, 4 bytes each in FP32; FP16 storage keeps two row-paired copies
// of 2 bytes per voxel, so about the same; x rows rounded up to 16 bytes) is rejected
// with NLM_ERR_WORKSPACE: for sr 3, pr 1 that is up to 152^3 (about 160^3 padded).
//
// Every call on a device shares the one array, so calls whose GPU work overlaps (on two
// streams, or from two threads) race on it: serialise them, for example on one stream.
// The array keeps whatever the last call left in it.  Nothing needs to start at zero:
// the staging pass rewrites every byte that the NLM kernel later reads.
#include <cuda_runtime.h>
#include <stdio.h>

#include <mutex>

#include "../../include/nlm.h"
#include "nlm_internal.h"

namespace gnlm {

constexpr size_t kNoAllocScratchBytes = size_t(16) << 20;
constexpr int kNoAllocMaxDevices = 64;

// File-scope scratch.  In host code this name is only a host-side stand-in for the
// symbol, not a device address: the address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

namespace {
std::mutex g_noalloc_mu;
void* g_noalloc_addr[kNoAllocMaxDevices] = {};  // device address of the array, per device

// Set-up, once per device, with that device current: look up the array's device
// address.  Runs inside the first call on each device.
int noalloc_scratch(void** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return report_error(NLM_ERR_CUDA, "cudaGetDevice failed");
    if (dev < 0 || dev >= kNoAllocMaxDevices)
        return report_error(NLM_ERR_NO_DEVICE, "device ordinal beyond 63");
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            char msg[160];
            snprintf(msg, sizeof(msg), "cudaGetSymbolAddress(scratch) failed: %s",
                     cudaGetErrorString(e));
            return report_error(NLM_ERR_CUDA, msg);
        }
        g_noalloc_addr[dev] = p;
    }
    *out = g_noalloc_addr[dev];
    return NLM_OK;
}
}  // namespace

}  // namespace gnlm

extern "C" int nlm3d_forward_noalloc(const void* d_in, int in_dtype, int X, int Y, int Z, int sr,
                                     int pr, float h, float* d_out, float* d_zsum,
                                     unsigned int flags, nlm_stream_t stream) {
    using namespace gnlm;
    const size_t need = nlm3d_workspace_bytes(X, Y, Z, sr, pr, flags);
    if (need == 0) return report_error(NLM_ERR_INVALID_ARG, "invalid extent or radius");
    if (need > kNoAllocScratchBytes) {
        char msg[200];
        snprintf(msg, sizeof(msg),
                 "volume needs %zu bytes of staging scratch; the allocation-free entry point "
                 "holds at most %zu (use nlm3d_forward with a workspace)",
                 need, kNoAllocScratchBytes);
        return report_error(NLM_ERR_WORKSPACE, msg);
    }
    void* scratch = nullptr;
    int rc = noalloc_scratch(&scratch);
    if (rc != NLM_OK) return rc;
    // With a caller-provided workspace nlm3d_forward neither allocates nor frees.
    return nlm3d_forward(d_in, in_dtype, X, Y, Z, sr, pr, h, d_out, d_zsum, flags, scratch,
                         kNoAllocScratchBytes, stream);
}
