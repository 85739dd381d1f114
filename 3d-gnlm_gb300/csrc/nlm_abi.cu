// C ABI of libgnlm.so (declared in include/nlm.h): argument checks, status codes,
// the per-thread error message, workspace management and the host-buffer path.
#include <cudaTypedefs.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <vector>
#include <mutex>
#include <utility>

#include "../../include/nlm.h"
#include "nlm_internal.h"

namespace gnlm {

// Per device: [0] the error word, which kernels OR DEVERR_* bits into when a bounded
// wait gives up (see nlm_device_status); [1] the fault-injection control word that
// only the NLM_BOUNDS_CHECK test build reads (see nlm_test_set_fault).
__device__ unsigned int g_device_error_word[2];

namespace {

thread_local char t_last_error[512] = "";

int fail(int code, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(t_last_error, sizeof(t_last_error), fmt, ap);
    va_end(ap);
    return code;
}

int cuda_fail(cudaError_t e, const char* what) {
    // Consume a non-sticky error (e.g. a failed cudaMalloc) so that the next
    // call's post-launch cudaGetLastError() does not report it again.
    cudaGetLastError();
    if (e == cudaErrorNotSupported)
        return fail(NLM_ERR_UNSUPPORTED, "%s: combination not compiled in", what);
    return fail(NLM_ERR_CUDA, "%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
}

std::mutex g_mutex;
std::map<std::pair<int, cudaStream_t>, std::pair<void*, size_t>> g_ws;  // cached workspaces

struct HostPath {
    cudaStream_t stream = nullptr;  // staging + compute (even chunks of the pipelined path)
    cudaStream_t s_c2 = nullptr;    // staging + compute of odd chunks
    cudaStream_t s_h2d = nullptr, s_d2h = nullptr;
    std::vector<cudaEvent_t> ev_in, ev_out, ev_st;
    void* d_in = nullptr;
    size_t in_bytes = 0;
    float* d_out = nullptr;
    size_t out_bytes = 0;
    void* d_ws = nullptr;
    size_t ws_bytes = 0;
    std::mutex mu;
};
std::map<int, HostPath*> g_host;

PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;

// Autotuned tile-shape variant per (dims, sr, pr, fp16); absent = variant 0.
std::map<long long, int> g_tuned;
long long tune_key(int dims, int sr, int pr, bool fp16) {
    return ((long long)dims << 40) | ((long long)(sr & 0xffff) << 24) | ((long long)(pr & 0xffff) << 8) |
           (fp16 ? 1 : 0);
}

bool valid_dtype(int d) { return d == NLM_U8 || d == NLM_F16 || d == NLM_F32; }
size_t dtype_bytes(int d) { return d == NLM_U8 ? 1 : (d == NLM_F16 ? 2 : 4); }

// Grows (never shrinks) a cached device buffer.  Refuses to allocate while the
// stream is being captured.
int ensure_buffer(void** ptr, size_t* have, size_t need, cudaStream_t stream) {
    if (*have >= need && *ptr) return NLM_OK;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (stream) cudaStreamIsCapturing(stream, &cs);
    if (cs != cudaStreamCaptureStatusNone)
        return fail(NLM_ERR_WORKSPACE,
                    "workspace cache must grow (%zu bytes) during stream capture; pass a "
                    "workspace or warm the cache before capturing",
                    need);
    if (*ptr) {
        cudaStreamSynchronize(stream);
        cudaFree(*ptr);
        *ptr = nullptr;
        *have = 0;
    }
    cudaError_t e = cudaMalloc(ptr, need);
    if (e != cudaSuccess) {
        *ptr = nullptr;
        return cuda_fail(e, "cudaMalloc(workspace)");
    }
    *have = need;
    return NLM_OK;
}

// Resolves the workspace: caller-provided or the (device, stream) cache.
int resolve_ws(void** d_ws, size_t* ws_bytes, size_t need, cudaStream_t stream) {
    if (*d_ws) {
        if (*ws_bytes < need)
            return fail(NLM_ERR_WORKSPACE, "workspace of %zu bytes < %zu required", *ws_bytes,
                        need);
        if (reinterpret_cast<uintptr_t>(*d_ws) % kAlign)
            return fail(NLM_ERR_INVALID_ARG, "workspace must be %zu-byte aligned", kAlign);
        return NLM_OK;
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    std::lock_guard<std::mutex> lk(g_mutex);
    auto& slot = g_ws[{dev, stream}];
    int rc = ensure_buffer(&slot.first, &slot.second, need, stream);
    if (rc != NLM_OK) return rc;
    *d_ws = slot.first;
    *ws_bytes = slot.second;
    return NLM_OK;
}


float weight_scale(int pr, int dims, float h) {
    const double k = 2.0 * pr + 1.0;
    const double P = dims == 3 ? k * k * k : k * k;
    return (float)sqrt(1.4426950408889634 / (P * (double)h * (double)h));
}

int check_common(const void* in, const void* out, int in_dtype, int sr, int pr, float h,
                 unsigned int flags) {
    if (!in || !out) return fail(NLM_ERR_INVALID_ARG, "null input or output pointer");
    if (!valid_dtype(in_dtype)) return fail(NLM_ERR_INVALID_ARG, "invalid in_dtype %d", in_dtype);
    if (sr < 0 || pr < 0) return fail(NLM_ERR_INVALID_ARG, "negative radius (sr=%d pr=%d)", sr, pr);
    if (!(h > 0.f) || !isfinite(h)) return fail(NLM_ERR_INVALID_ARG, "h must be finite and > 0");
    if (flags & ~(NLM_FLAG_FP16_STORAGE | NLM_FLAG_PREPADDED))
        return fail(NLM_ERR_INVALID_ARG, "unknown flag bits 0x%x", flags);
    return NLM_OK;
}

int check_dims3(int X, int Y, int Z, int H) {
    if (X < 1 || Y < 1 || Z < 1) return fail(NLM_ERR_INVALID_ARG, "non-positive extent");
    // staging grid: one block per padded row (grid.y = padded planes <= 65535);
    // TMA global extents < 2^32; 64-bit element indices everywhere.
    if ((long long)Z + 2LL * H > 65535 || (long long)Y + 2LL * H > (1LL << 30) ||
        (long long)X + 2LL * H > (1LL << 30))
        return fail(NLM_ERR_INVALID_ARG, "volume too large (%d x %d x %d)", X, Y, Z);
    return NLM_OK;
}

}  // namespace

int report_error(int code, const char* msg) { return fail(code, "%s", msg); }

int validate_forward3d(const void* in, const void* out, int in_dtype, int X, int Y, int Z, int sr,
                       int pr, float h, unsigned int flags) {
    int rc = check_common(in, out, in_dtype, sr, pr, h, flags);
    if (rc) return rc;
    if ((rc = check_dims3(X, Y, Z, sr + pr))) return rc;
    if (!nlm3d_fwd_supported(sr, pr, (flags & NLM_FLAG_FP16_STORAGE) != 0))
        return fail(NLM_ERR_UNSUPPORTED, "3D (sr=%d, pr=%d) not compiled in", sr, pr);
    return NLM_OK;
}

namespace {
using PFN_ctxGetCurrent = CUresult (*)(CUcontext*);
using PFN_ctxGetId = CUresult (*)(CUcontext, unsigned long long*);
PFN_ctxGetCurrent g_ctx_current = nullptr;
PFN_ctxGetId g_ctx_id = nullptr;
std::map<std::pair<unsigned long long, const void*>, void*> g_symbols;  // (context, symbol)

}  // namespace

// Unique ID of the calling thread's current context (false if there is none yet).
bool current_context_id(unsigned long long* id) {
    {
        std::lock_guard<std::mutex> lk(g_mutex);
        if (!g_ctx_current || !g_ctx_id) {
            cudaDriverEntryPointQueryResult q;
            void* f1 = nullptr;
            void* f2 = nullptr;
            if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault,
                                                 &q) != cudaSuccess ||
                q != cudaDriverEntryPointSuccess ||
                cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault,
                                                 &q) != cudaSuccess ||
                q != cudaDriverEntryPointSuccess || !f1 || !f2)
                return false;
            g_ctx_current = reinterpret_cast<PFN_ctxGetCurrent>(f1);
            g_ctx_id = reinterpret_cast<PFN_ctxGetId>(f2);
        }
    }
    CUcontext ctx = nullptr;
    if (g_ctx_current(&ctx) != CUDA_SUCCESS || !ctx) return false;
    return g_ctx_id(ctx, id) == CUDA_SUCCESS;
}

// Device address of a __device__ variable (given by its host-side shadow) in the
// calling thread's current context.  Cached per context ID, never per device ordinal:
// a device reset makes a new primary context, which loads the module again and may
// place the variable elsewhere, and a new context has a new ID.
void* symbol_address(const void* symbol) {
    unsigned long long id = 0;
    bool have_id = current_context_id(&id);
    if (have_id) {
        std::lock_guard<std::mutex> lk(g_mutex);
        auto it = g_symbols.find({id, symbol});
        if (it != g_symbols.end()) return it->second;
    }
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, symbol) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (!have_id) have_id = current_context_id(&id);  // the lookup made the context current
    if (have_id) {
        std::lock_guard<std::mutex> lk(g_mutex);
        g_symbols[{id, symbol}] = p;
    }
    return p;
}

// Variant used before any autotuning: the fastest measured on a GB300 for the
// configuration family (3D FP32 patch 3: z offsets in groups of four, 4 x 6 tiles,
// fastest from 128^3 to 256^3; search 11 / patch 5: groups of three, 4 x 6, whose
// groups of four spill registers; 2D FP32: two columns per lane, 8 rows x 4 warps),
// else variant 0.
int default_variant(int dims, int sr, int pr, bool fp16) {
    if (fp16) return 0;
    if (dims == 3) {
        if (nlm3d_fwd_large_patch(sr, pr, fp16)) return 0;
        if (pr == 1) return 4;
        if (pr == 2 && sr == 5) return 5;
        return 0;
    }
    return 5;
}

int tuned_variant(int dims, int sr, int pr, bool fp16) {
    std::lock_guard<std::mutex> lk(g_mutex);
    auto it = g_tuned.find(tune_key(dims, sr, pr, fp16));
    return it == g_tuned.end() ? default_variant(dims, sr, pr, fp16) : it->second;
}

unsigned int* device_error_word() {
    return static_cast<unsigned int*>(symbol_address(g_device_error_word));
}

cudaError_t encode_tensor_map(CUtensorMap* map, bool fp16, int rank, const uint64_t* dims,
                              const uint64_t* strides_bytes, const uint32_t* box, void* base) {
    {
        std::lock_guard<std::mutex> lk(g_mutex);
        if (!g_encode) {
            cudaDriverEntryPointQueryResult q;
            void* fn = nullptr;
            cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000,
                                                             cudaEnableDefault, &q);
            if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !fn)
                return e != cudaSuccess ? e : cudaErrorNotSupported;
            g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
        }
    }
    cuuint64_t d[5];
    cuuint64_t s[4];
    cuuint32_t b[5], es[5];
    for (int i = 0; i < rank; ++i) {
        d[i] = dims[i];
        b[i] = box[i];
        es[i] = 1;
        if (i + 1 < rank) s[i] = strides_bytes[i];
    }
    CUresult r = g_encode(map, fp16 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32,
                          (cuuint32_t)rank, base, d, s, b, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                          CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

}  // namespace gnlm

using namespace gnlm;

extern "C" {

const char* nlm_version(void) { return "gnlm 0.1 sm_103a"; }

const char* nlm_last_error(void) { return t_last_error; }

int nlm_device_status(unsigned int* flags) {
    unsigned int* w = device_error_word();
    if (!w) return fail(NLM_ERR_CUDA, "no device error word (no CUDA device?)");
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return cuda_fail(e, "cudaDeviceSynchronize");
    unsigned int v = 0;
    e = cudaMemcpy(&v, w, sizeof(v), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "read device error word");
    const unsigned int zero = 0;
    e = cudaMemcpy(w, &zero, sizeof(zero), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(e, "clear device error word");
    if (flags) *flags = v;
    if (v) return fail(NLM_ERR_DEVICE, "device error word 0x%x", v);
    return NLM_OK;
}

int nlm_test_set_fault(unsigned int bits) {
#ifdef NLM_BOUNDS_CHECK
    unsigned int* w = device_error_word();
    if (!w) return fail(NLM_ERR_CUDA, "no device error word (no CUDA device?)");
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return cuda_fail(e, "cudaDeviceSynchronize");
    e = cudaMemcpy(w + 1, &bits, sizeof(bits), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(e, "write fault-injection word");
    return NLM_OK;
#else
    (void)bits;
    return fail(NLM_ERR_UNSUPPORTED,
                "fault injection exists only in the bounds-checked test build (libgnlm_checked.so)");
#endif
}

int nlm_release_cached(void) {
    std::lock_guard<std::mutex> lk(g_mutex);
    int prev = 0;
    cudaGetDevice(&prev);
    // A device-wide synchronise rather than one per cached stream: the caller may
    // already have destroyed a stream whose workspace is cached.
    int synced = -1;
    for (auto& kv : g_ws) {
        if (kv.second.first) {
            if (kv.first.first != synced) {
                cudaSetDevice(kv.first.first);
                cudaDeviceSynchronize();
                synced = kv.first.first;
            }
            cudaFree(kv.second.first);
        }
    }
    g_ws.clear();
    for (auto& kv : g_host) {
        HostPath* hp = kv.second;
        cudaSetDevice(kv.first);
        std::lock_guard<std::mutex> hl(hp->mu);
        for (cudaStream_t st : {hp->stream, hp->s_c2, hp->s_h2d, hp->s_d2h})
            if (st) cudaStreamSynchronize(st);
        cudaFree(hp->d_in);
        cudaFree(hp->d_out);
        cudaFree(hp->d_ws);
        hp->d_in = hp->d_out = nullptr;
        hp->d_ws = nullptr;
        hp->in_bytes = hp->out_bytes = hp->ws_bytes = 0;
    }
    cudaSetDevice(prev);
    return NLM_OK;
}

size_t nlm3d_workspace_bytes(int X, int Y, int Z, int sr, int pr, unsigned int flags) {
    if (X < 1 || Y < 1 || Z < 1 || sr < 0 || pr < 0) return 0;
    const bool fp16 = (flags & NLM_FLAG_FP16_STORAGE) != 0;
    return staging3d(X, Y, Z, sr, pr, fp16).bytes() + nlm3d_fwd_extra_bytes(X, Y, Z, sr, pr, fp16);
}

static int stage3d_impl(const void* d_in, int in_dtype, int X, int Y, int Z, int sr, int pr,
                        float h, unsigned int flags, void** d_ws, size_t* ws_bytes,
                        cudaStream_t stream) {
    const bool fp16 = (flags & NLM_FLAG_FP16_STORAGE) != 0;
    if (!nlm3d_fwd_supported(sr, pr, fp16))
        return fail(NLM_ERR_UNSUPPORTED, "3D (sr=%d, pr=%d) not compiled in", sr, pr);
    Staging st = staging3d(X, Y, Z, sr, pr, fp16);
    int rc = resolve_ws(d_ws, ws_bytes, nlm3d_workspace_bytes(X, Y, Z, sr, pr, flags), stream);
    if (rc) return rc;
    cudaError_t e = launch_stage(d_in, in_dtype, (flags & NLM_FLAG_PREPADDED) != 0,
                                 weight_scale(pr, 3, h), st, *d_ws, stream);
    if (e != cudaSuccess) return cuda_fail(e, "stage3d launch");
    return NLM_OK;
}

static int fwd3d_staged_impl(const void* d_ws, int X, int Y, int Z, int sr, int pr, float h,
                             float* d_out, float* d_zsum, unsigned int flags,
                             cudaStream_t stream) {
    const bool fp16 = (flags & NLM_FLAG_FP16_STORAGE) != 0;
    Staging st = staging3d(X, Y, Z, sr, pr, fp16);
    cudaError_t e = launch_nlm3d_fwd(st, d_ws, sr, pr, fp16, tuned_variant(3, sr, pr, fp16),
                                     1.0f / weight_scale(pr, 3, h), d_out, d_zsum,
                                     device_error_word(), stream);
    if (e != cudaSuccess) return cuda_fail(e, "nlm3d_fwd launch");
    return NLM_OK;
}

int nlm3d_stage(const void* d_in, int in_dtype, int X, int Y, int Z, int sr, int pr, float h,
                unsigned int flags, void* d_ws, size_t ws_bytes, nlm_stream_t stream) {
    int rc = check_common(d_in, d_ws ? d_ws : d_in, in_dtype, sr, pr, h, flags);
    if (rc) return rc;
    if (!d_ws) return fail(NLM_ERR_INVALID_ARG, "nlm3d_stage needs a caller workspace");
    if ((rc = check_dims3(X, Y, Z, sr + pr))) return rc;
    return stage3d_impl(d_in, in_dtype, X, Y, Z, sr, pr, h, flags, &d_ws, &ws_bytes,
                        (cudaStream_t)stream);
}

int nlm3d_forward_staged(const void* d_ws, size_t ws_bytes, int X, int Y, int Z, int sr, int pr,
                         float h, float* d_out, float* d_zsum, unsigned int flags,
                         nlm_stream_t stream) {
    int rc = check_common(d_ws, d_out, NLM_F32, sr, pr, h, flags);
    if (rc) return rc;
    if ((rc = check_dims3(X, Y, Z, sr + pr))) return rc;
    const bool fp16 = (flags & NLM_FLAG_FP16_STORAGE) != 0;
    if (!nlm3d_fwd_supported(sr, pr, fp16))
        return fail(NLM_ERR_UNSUPPORTED, "3D (sr=%d, pr=%d) not compiled in", sr, pr);
    const size_t need = nlm3d_workspace_bytes(X, Y, Z, sr, pr, flags);
    if (ws_bytes < need)
        return fail(NLM_ERR_WORKSPACE, "staged workspace of %zu bytes < %zu required", ws_bytes,
                    need);
    return fwd3d_staged_impl(d_ws, X, Y, Z, sr, pr, h, d_out, d_zsum, flags, (cudaStream_t)stream);
}

int nlm3d_forward(const void* d_in, int in_dtype, int X, int Y, int Z, int sr, int pr, float h,
                  float* d_out, float* d_zsum, unsigned int flags, void* d_ws, size_t ws_bytes,
                  nlm_stream_t stream_) {
    cudaStream_t stream = (cudaStream_t)stream_;
    int rc = check_common(d_in, d_out, in_dtype, sr, pr, h, flags);
    if (rc) return rc;
    if ((rc = check_dims3(X, Y, Z, sr + pr))) return rc;
    if ((rc = stage3d_impl(d_in, in_dtype, X, Y, Z, sr, pr, h, flags, &d_ws, &ws_bytes, stream)))
        return rc;
    return fwd3d_staged_impl(d_ws, X, Y, Z, sr, pr, h, d_out, d_zsum, flags, stream);
}

size_t nlm2d_workspace_bytes(int X, int Y, int sr, int pr, unsigned int flags) {
    if (X < 1 || Y < 1 || sr < 0 || pr < 0) return 0;
    return make_staging(X, Y, 1, sr + pr, 0, (flags & NLM_FLAG_FP16_STORAGE) != 0).bytes();
}

int nlm2d_forward(const void* d_in, int in_dtype, int X, int Y, int sr, int pr, float h,
                  float* d_out, float* d_zsum, unsigned int flags, void* d_ws, size_t ws_bytes,
                  nlm_stream_t stream_) {
    cudaStream_t stream = (cudaStream_t)stream_;
    int rc = check_common(d_in, d_out, in_dtype, sr, pr, h, flags);
    if (rc) return rc;
    const int H = sr + pr;
    if ((rc = check_dims3(X, Y, 1, H))) return rc;
    const bool fp16 = (flags & NLM_FLAG_FP16_STORAGE) != 0;
    if (!nlm2d_fwd_supported(sr, pr, fp16))
        return fail(NLM_ERR_UNSUPPORTED, "2D (sr=%d, pr=%d) not compiled in", sr, pr);
    Staging st = make_staging(X, Y, 1, H, 0, fp16);
    if ((rc = resolve_ws(&d_ws, &ws_bytes, st.bytes(), stream))) return rc;
    unsigned int* ew = device_error_word();
    const float s = weight_scale(pr, 2, h);
    cudaError_t e = launch_stage(d_in, in_dtype, (flags & NLM_FLAG_PREPADDED) != 0, s, st, d_ws, stream);
    if (e != cudaSuccess) return cuda_fail(e, "stage2d launch");
    e = launch_nlm2d_fwd(st, d_ws, sr, pr, fp16, tuned_variant(2, sr, pr, fp16), 1.0f / s, d_out,
                         d_zsum, ew, stream);
    if (e != cudaSuccess) return cuda_fail(e, "nlm2d_fwd launch");
    return NLM_OK;
}

size_t nlm3d_adjoint_workspace_bytes(int X, int Y, int Z, int sr, int pr) {
    if (X < 1 || Y < 1 || Z < 1 || sr < 0 || pr < 0 || !nlm3d_adj_supported(sr, pr)) return 0;
    const Staging st = make_staging(X, Y, Z, sr + pr, sr + pr, false);
    return 4 * st.bytes() + align_up(adj3d_ctas(st, sr, pr) * sizeof(double), kAlign) +
           align_up(adj3d_side_bytes(sr, pr), kAlign);
}

int nlm3d_adjoint(const float* d_in, const float* d_out, const float* d_zsum, const float* d_gout,
                  int X, int Y, int Z, int sr, int pr, float h, float* d_gin, double* d_hgrad,
                  void* d_ws, size_t ws_bytes, nlm_stream_t stream_) {
    cudaStream_t stream = (cudaStream_t)stream_;
    int rc = check_common(d_in, d_gin, NLM_F32, sr, pr, h, 0);
    if (rc) return rc;
    if (!d_out || !d_zsum || !d_gout)
        return fail(NLM_ERR_INVALID_ARG, "adjoint needs out, zsum and the upstream gradient");
    if ((rc = check_dims3(X, Y, Z, sr + pr))) return rc;
    if (!nlm3d_adj_supported(sr, pr))
        return fail(NLM_ERR_UNSUPPORTED, "3D adjoint (sr=%d, pr=%d) not compiled in", sr, pr);
    const Staging st = make_staging(X, Y, Z, sr + pr, sr + pr, false);
    if ((rc = resolve_ws(&d_ws, &ws_bytes, nlm3d_adjoint_workspace_bytes(X, Y, Z, sr, pr), stream)))
        return rc;
    char* base = static_cast<char*>(d_ws);
    void* staged = base;
    float2* GO = reinterpret_cast<float2*>(base + st.bytes());  // 2 * st.bytes()
    float* gpad = reinterpret_cast<float*>(base + 3 * st.bytes());
    double* hpart = reinterpret_cast<double*>(base + 4 * st.bytes());
    float* side = reinterpret_cast<float*>(
        base + 4 * st.bytes() + align_up(adj3d_ctas(st, sr, pr) * sizeof(double), kAlign));
    const float s = weight_scale(pr, 3, h);
    cudaError_t e = launch_stage(d_in, NLM_F32, false, s, st, staged, stream);
    if (e != cudaSuccess) return cuda_fail(e, "adjoint staging");
    e = launch_nlm3d_adj(st, staged, d_out, d_zsum, d_gout, sr, pr, s, h, d_gin, d_hgrad, GO,
                         gpad, hpart, side, device_error_word(), stream);
    if (e != cudaSuccess) return cuda_fail(e, "nlm3d_adjoint launch");
    return NLM_OK;
}

int nlm_variant_count(int dims, unsigned int flags) {
    if (dims == 3) return nlm3d_fwd_variant_count((flags & NLM_FLAG_FP16_STORAGE) != 0);
    if (dims == 2) return nlm2d_fwd_variant_count();
    return fail(NLM_ERR_INVALID_ARG, "dims must be 2 or 3");
}

int nlm_set_variant(int dims, int sr, int pr, unsigned int flags, int variant) {
    const int n = nlm_variant_count(dims, flags);
    if (n < 0) return n;
    if (variant < -1 || variant >= n)
        return fail(NLM_ERR_INVALID_ARG, "variant %d outside [-1, %d)", variant, n);
    std::lock_guard<std::mutex> lk(g_mutex);
    const long long k = tune_key(dims, sr, pr, (flags & NLM_FLAG_FP16_STORAGE) != 0);
    if (variant < 0)
        g_tuned.erase(k);
    else
        g_tuned[k] = variant;
    return NLM_OK;
}

int nlm_get_variant(int dims, int sr, int pr, unsigned int flags) {
    if (dims != 2 && dims != 3) return fail(NLM_ERR_INVALID_ARG, "dims must be 2 or 3");
    return tuned_variant(dims, sr, pr, (flags & NLM_FLAG_FP16_STORAGE) != 0);
}

int nlm_autotune(int dims, int X, int Y, int Z, int sr, int pr, unsigned int flags,
                 float* times_ms, nlm_stream_t stream_) {
    cudaStream_t stream = (cudaStream_t)stream_;
    if (dims != 2 && dims != 3) return fail(NLM_ERR_INVALID_ARG, "dims must be 2 or 3");
    if (dims == 2) Z = 1;
    const bool fp16 = (flags & NLM_FLAG_FP16_STORAGE) != 0;
    int rc = check_dims3(X, Y, Z, sr + pr);
    if (rc) return rc;
    const bool ok = dims == 3 ? nlm3d_fwd_supported(sr, pr, fp16) : nlm2d_fwd_supported(sr, pr, fp16);
    if (!ok) return fail(NLM_ERR_UNSUPPORTED, "%dD (sr=%d, pr=%d) not compiled in", dims, sr, pr);
    const Staging st = dims == 3 ? staging3d(X, Y, Z, sr, pr, fp16)
                                 : make_staging(X, Y, 1, sr + pr, 0, fp16);
    const size_t nvox = (size_t)X * Y * Z;
    void *d_in = nullptr, *d_ws = nullptr;
    float* d_out = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int best = -1;
    float best_ms = 0.f;
    const int nv = nlm_variant_count(dims, flags);
    cudaError_t e = cudaMalloc(&d_in, nvox * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc((void**)&d_out, nvox * sizeof(float));
    const size_t ws_need = dims == 3 ? nlm3d_workspace_bytes(X, Y, Z, sr, pr, flags) : st.bytes();
    if (e == cudaSuccess) e = cudaMalloc(&d_ws, ws_need);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_in, 0, nvox * sizeof(float), stream);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    const float s = weight_scale(pr, dims, 0.05f);
    if (e == cudaSuccess) e = launch_stage(d_in, NLM_F32, false, s, st, d_ws, stream);
    for (int v = 0; v < nv && e == cudaSuccess; ++v) {
        float ms = 1e30f;
        for (int rep = 0; rep < 4 && e == cudaSuccess; ++rep) {
            e = cudaEventRecord(e0, stream);
            if (e == cudaSuccess)
                e = dims == 3 ? launch_nlm3d_fwd(st, d_ws, sr, pr, fp16, v, 1.0f / s, d_out,
                                                 nullptr, device_error_word(), stream)
                              : launch_nlm2d_fwd(st, d_ws, sr, pr, fp16, v, 1.0f / s, d_out,
                                                 nullptr, device_error_word(), stream);
            if (e == cudaSuccess) e = cudaEventRecord(e1, stream);
            if (e == cudaSuccess) e = cudaEventSynchronize(e1);
            float t = 0.f;
            if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
            if (rep > 0 && t < ms) ms = t;  // first run is a warm-up
        }
        if (times_ms) times_ms[v] = ms;
        if (e == cudaSuccess && (best < 0 || ms < best_ms)) {
            best = v;
            best_ms = ms;
        }
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(d_in);
    cudaFree(d_out);
    cudaFree(d_ws);
    if (e != cudaSuccess) return cuda_fail(e, "nlm_autotune");
    nlm_set_variant(dims, sr, pr, flags, best);
    return best;
}

static HostPath* host_path(int dev) {
    std::lock_guard<std::mutex> lk(g_mutex);
    HostPath*& hp = g_host[dev];
    if (!hp) hp = new HostPath();
    return hp;
}

static int ensure_events(std::vector<cudaEvent_t>& v, size_t n) {
    while (v.size() < n) {
        cudaEvent_t e;
        cudaError_t r = cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
        if (r != cudaSuccess) return cuda_fail(r, "cudaEventCreate");
        v.push_back(e);
    }
    return NLM_OK;
}

// 3D host path pipelined over z chunks: the host->device copy of later input
// chunks and the device->host copy of finished output chunks overlap the staging
// and NLM kernels of the current chunk.  Output chunks are whole z tiles: a first and
// a last chunk of one tile (so the first kernel waits only for the input planes its
// REFLECT_101 halo reaches from one tile, and the last output copy is short) and
// chunks of CZ planes between them.  Input plane k is copied in the chunk of the first
// output chunk that reads it, so the copies run ahead of the kernels in the order they
// are needed.  Chunks alternate between two compute streams so that the kernels of
// chunk k+1 fill the SMs that chunk k's last wave leaves idle: chunk k stages padded
// planes [z0 + 2H, z1 + 2H) (all of [0, z1 + 2H) for k = 0), which no earlier chunk
// reads, and its NLM kernel waits for the staging of chunk k-1, which wrote the lower
// 2H planes it reads.  Returns 1 when the volume is too thin to split.
static int host_forward3d_pipelined(HostPath* hp, const void* h_in, int in_dtype, int X, int Y,
                                    int Z, int sr, int pr, float h, float* h_out,
                                    unsigned int flags) {
    const bool fp16 = (flags & NLM_FLAG_FP16_STORAGE) != 0;
    const bool prepadded = (flags & NLM_FLAG_PREPADDED) != 0;
    const int H = sr + pr;
    const int variant = tuned_variant(3, sr, pr, fp16);
    const int RZ = nlm3d_fwd_tile_z(sr, pr, fp16, variant);
    if (RZ <= 0) return 1;
    // about Z / 8 planes per middle chunk (256^3 end to end: 8 chunks 6794, 6: 6787,
    // 12: 6705, 16: 6748, 24: 6688 Mvoxel/s)
    const int CZ = std::max(1, (Z / 8 + RZ - 1) / RZ) * RZ;
    std::vector<int> zb{0};                  // output chunk boundaries
    const int zlast = ((Z - 1) / RZ) * RZ;   // first plane of the last z tile
    for (int z = RZ; z < zlast; z = std::min(z + CZ, zlast)) zb.push_back(z);
    if (zlast > 0) zb.push_back(zlast);
    zb.push_back(Z);
    const int nch = (int)zb.size() - 1;
    if (nch < 2) return 1;
    cudaError_t e = cudaSuccess;
    if (!hp->s_h2d) e = cudaStreamCreateWithFlags(&hp->s_h2d, cudaStreamNonBlocking);
    if (e == cudaSuccess && !hp->s_d2h) e = cudaStreamCreateWithFlags(&hp->s_d2h, cudaStreamNonBlocking);
    if (e == cudaSuccess && !hp->s_c2) e = cudaStreamCreateWithFlags(&hp->s_c2, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamCreate");
    const Staging st = staging3d(X, Y, Z, sr, pr, fp16);
    const size_t plane_in =
        (prepadded ? (size_t)(X + 2 * H) * (Y + 2 * H) : (size_t)X * Y) * dtype_bytes(in_dtype);
    int rc = ensure_events(hp->ev_in, nch);
    if (rc == NLM_OK) rc = ensure_events(hp->ev_out, nch);
    if (rc == NLM_OK) rc = ensure_events(hp->ev_st, nch);
    if (rc != NLM_OK) return rc;
    // input planes [0, need(k)) are read by output chunks 0..k
    auto need = [&](int k) {
        return prepadded ? zb[k + 1] + 2 * H : std::min(Z, zb[k + 1] + H);
    };
    const char* src = static_cast<const char*>(h_in);
    char* din = static_cast<char*>(hp->d_in);
    for (int k = 0, p0 = 0; k < nch; ++k) {
        const int p1 = need(k);
        if (p1 > p0)
            e = cudaMemcpyAsync(din + (size_t)p0 * plane_in, src + (size_t)p0 * plane_in,
                                (size_t)(p1 - p0) * plane_in, cudaMemcpyHostToDevice, hp->s_h2d);
        if (e == cudaSuccess) e = cudaEventRecord(hp->ev_in[k], hp->s_h2d);
        if (e != cudaSuccess) return cuda_fail(e, "host->device chunk copy");
        p0 = std::max(p0, p1);
    }
    const float s = weight_scale(pr, 3, h);
    unsigned int* ew = device_error_word();
    const size_t plane_out = (size_t)X * Y;
    for (int k = 0; k < nch; ++k) {
        const int z0 = zb[k], z1 = zb[k + 1];
        const int p0 = k == 0 ? 0 : z0 + 2 * H, p1 = z1 + 2 * H;  // new padded planes
        cudaStream_t cs = (k & 1) ? hp->s_c2 : hp->stream;
        e = cudaStreamWaitEvent(cs, hp->ev_in[k], 0);
        if (e == cudaSuccess) e = launch_stage(hp->d_in, in_dtype, prepadded, s, st, hp->d_ws, cs, p0, p1);
        if (e == cudaSuccess) e = cudaEventRecord(hp->ev_st[k], cs);
        if (e == cudaSuccess && k > 0) e = cudaStreamWaitEvent(cs, hp->ev_st[k - 1], 0);
        if (e == cudaSuccess)
            e = launch_nlm3d_fwd(st, hp->d_ws, sr, pr, fp16, variant, 1.0f / s, hp->d_out, nullptr,
                                 ew, cs, z0 / RZ, (z1 + RZ - 1) / RZ);
        if (e == cudaSuccess) e = cudaEventRecord(hp->ev_out[k], cs);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(hp->s_d2h, hp->ev_out[k], 0);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(h_out + (size_t)z0 * plane_out, hp->d_out + (size_t)z0 * plane_out,
                                (size_t)(z1 - z0) * plane_out * sizeof(float),
                                cudaMemcpyDeviceToHost, hp->s_d2h);
        if (e != cudaSuccess) return cuda_fail(e, "pipelined forward");
    }
    e = cudaStreamSynchronize(hp->s_d2h);
    if (e == cudaSuccess) e = cudaStreamSynchronize(hp->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(hp->s_c2);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamSynchronize");
    return NLM_OK;
}

static int host_forward(const void* h_in, int in_dtype, int X, int Y, int Z, int sr, int pr,
                        float h, float* h_out, unsigned int flags, int dims) {
    int rc = check_common(h_in, h_out, in_dtype, sr, pr, h, flags);
    if (rc) return rc;
    const int H = sr + pr;
    if ((rc = check_dims3(X, Y, Z, H))) return rc;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    HostPath* hp = host_path(dev);
    std::lock_guard<std::mutex> lk(hp->mu);
    if (!hp->stream) {
        e = cudaStreamCreateWithFlags(&hp->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) return cuda_fail(e, "cudaStreamCreate");
    }
    const bool prepadded = (flags & NLM_FLAG_PREPADDED) != 0;
    const int Hz = dims == 3 ? H : 0;
    const size_t nin = prepadded ? (size_t)(X + 2 * H) * (Y + 2 * H) * (Z + 2 * Hz)
                                 : (size_t)X * Y * Z;
    const size_t in_bytes = nin * dtype_bytes(in_dtype);
    const size_t out_bytes = (size_t)X * Y * Z * sizeof(float);
    const size_t ws = dims == 3 ? nlm3d_workspace_bytes(X, Y, Z, sr, pr, flags)
                                : nlm2d_workspace_bytes(X, Y, sr, pr, flags);
    if ((rc = ensure_buffer(&hp->d_in, &hp->in_bytes, in_bytes, hp->stream))) return rc;
    if ((rc = ensure_buffer((void**)&hp->d_out, &hp->out_bytes, out_bytes, hp->stream))) return rc;
    if ((rc = ensure_buffer(&hp->d_ws, &hp->ws_bytes, ws, hp->stream))) return rc;
    if (dims == 3 && nlm3d_fwd_supported(sr, pr, (flags & NLM_FLAG_FP16_STORAGE) != 0)) {
        rc = host_forward3d_pipelined(hp, h_in, in_dtype, X, Y, Z, sr, pr, h, h_out, flags);
        if (rc != 1) return rc;
    }
    e = cudaMemcpyAsync(hp->d_in, h_in, in_bytes, cudaMemcpyHostToDevice, hp->stream);
    if (e != cudaSuccess) return cuda_fail(e, "host->device copy");
    rc = dims == 3 ? nlm3d_forward(hp->d_in, in_dtype, X, Y, Z, sr, pr, h, hp->d_out, nullptr,
                                   flags, hp->d_ws, hp->ws_bytes, (nlm_stream_t)hp->stream)
                   : nlm2d_forward(hp->d_in, in_dtype, X, Y, sr, pr, h, hp->d_out, nullptr, flags,
                                   hp->d_ws, hp->ws_bytes, (nlm_stream_t)hp->stream);
    if (rc) return rc;
    e = cudaMemcpyAsync(h_out, hp->d_out, out_bytes, cudaMemcpyDeviceToHost, hp->stream);
    if (e != cudaSuccess) return cuda_fail(e, "device->host copy");
    e = cudaStreamSynchronize(hp->stream);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamSynchronize");
    return NLM_OK;
}

int nlm3d_forward_host(const void* h_in, int in_dtype, int X, int Y, int Z, int sr, int pr,
                       float h, float* h_out, unsigned int flags) {
    return host_forward(h_in, in_dtype, X, Y, Z, sr, pr, h, h_out, flags, 3);
}

int nlm2d_forward_host(const void* h_in, int in_dtype, int X, int Y, int sr, int pr, float h,
                       float* h_out, unsigned int flags) {
    return host_forward(h_in, in_dtype, X, Y, 1, sr, pr, h, h_out, flags, 2);
}

}  // extern "C"
