/*
 * nlm.h - C ABI of the GB300 (sm_103a) non-local-means denoiser.
 *
 * One shared library (libgnlm.so) exports these entry points.  Every argument is
 * a plain pointer, size or scalar; no C++ or framework types cross the boundary.
 *
 * Conventions
 *   - Volumes are dense, x fastest: index = (z * Y + y) * X + x.  Images are
 *     [Y][X].  Inputs are UNPADDED: borders are handled as OpenCV
 *     BORDER_REFLECT_101 (gfedcb|abcdefgh|gfedcba) on every axis, the padding the
 *     reference's driver applies before calling its kernels
 *     (3DNLM/nlm.cpp:36-41, 2D NLM/11x11/nlm.cpp:15-19).  With NLM_FLAG_PREPADDED
 *     the input is instead the reference's pre-padded layout (halo
 *     (SS+NS-2)/2 = sr+pr on every side), used as given.
 *   - sr is the search radius m (search window SS = 2m+1), pr the patch radius n
 *     (patch NS = 2n+1), h the filtering parameter: w = exp(-(D / NS^d) / h^2),
 *     D the summed squared patch difference (3DNLM/main.cu:108-109).  The centre
 *     offset is included; out = sum(w v) / sum(w) (3DNLM/main.cu:110-111,125).
 *   - d_* pointers are device memory owned by the caller; h_* pointers are host
 *     memory (pinned is fastest).  Calls are asynchronous on `stream` unless they
 *     say otherwise.
 *   - Return value: NLM_OK (0) or a negative nlm_status.  Nothing aborts or
 *     exits; nlm_last_error() gives the calling thread's last message.
 *   - Scratch: each forward call needs a workspace.  Pass d_ws/ws_bytes (size
 *     from the *_workspace_bytes query), or d_ws = NULL to use a buffer the
 *     library caches per (device, stream) and grows with cudaMalloc; the cache
 *     grows only outside stream capture, so warm it before capturing.  Each
 *     distinct stream keeps its own buffer until nlm_release_cached(): callers
 *     that create a new stream per call should pass their own workspace.
 *   - Thread safety: calls are thread-safe; calls on different streams with the
 *     library cache use different buffers.
 */
#ifndef GNLM_NLM_H
#define GNLM_NLM_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Same type as cudaStream_t (struct CUstream_st*); NULL is the legacy stream. */
typedef struct CUstream_st* nlm_stream_t;

typedef enum nlm_status {
    NLM_OK = 0,
    NLM_ERR_INVALID_ARG = -1,  /* null pointer, non-positive size, h <= 0, ... */
    NLM_ERR_UNSUPPORTED = -2,  /* (sr, pr, dtype) combination not compiled in */
    NLM_ERR_CUDA = -3,         /* a CUDA runtime/driver call failed */
    NLM_ERR_WORKSPACE = -4,    /* caller workspace smaller than required */
    NLM_ERR_DEVICE = -5,       /* a kernel raised its device-side error word */
    NLM_ERR_NO_DEVICE = -6     /* no CUDA device / not an sm_103 device */
} nlm_status;

/* Element type of an input volume. */
typedef enum nlm_dtype {
    NLM_U8 = 0,   /* unsigned char, as the reference's input (3DNLM/main.h:6) */
    NLM_F16 = 1,  /* IEEE binary16 */
    NLM_F32 = 2   /* IEEE binary32 */
} nlm_dtype;

/* Flags for the forward calls. */
#define NLM_FLAG_FP16_STORAGE 0x1u /* precision form: volume staged as FP16, FP32
                                      distances, Kahan-compensated weight sums */
#define NLM_FLAG_PREPADDED 0x2u    /* input is already padded by sr+pr per side */

/* Library identification, e.g. "gnlm 0.1 sm_103a" (no counterpart in the reference). */
const char* nlm_version(void);

/* Message of the calling thread's last failing call ("" if none).  With the status
 * codes, replaces the reference's CUDA_CHECK printing to stderr
 * (3DNLM/cuda_utility.h:9-16), which its NL_Means ignores. */
const char* nlm_last_error(void);

/* Synchronises the current device, then reads and clears the device-side error
 * word that kernels set when a bounded wait gives up.  *flags receives the word
 * (0 = no error; 0x1 a tile copy timed out, 0x2 reserved (the batch work queue
 * never waits, so no kernel sets it), 0x4 a batch work item failed its own check,
 * 0x8 an index range left its buffer — reported only by the NLM_BOUNDS_CHECK build,
 * libgnlm_checked.so).
 * Returns NLM_OK, or NLM_ERR_DEVICE when the word was set. */
int nlm_device_status(unsigned int* flags);

/* Test hook (no counterpart in the reference): in the bounds-checked test build,
 * libgnlm_checked.so, bits = 0x1 makes the first tile (0, 0, 0) of every later 3D/2D
 * forward (large-patch included) and adjoint launch on the current device skip its tile
 * copy (the large-patch kernel: the planes of its first step), so its bounded
 * wait runs out and the kernel reports 0x1 in the device error word instead of
 * hanging; that tile's outputs are left unwritten.  bits = 0 turns it off.  The
 * production library (libgnlm.so) returns NLM_ERR_UNSUPPORTED and changes nothing. */
int nlm_test_set_fault(unsigned int bits);

/* Frees the library-cached workspaces and host-path buffers of every device (the
 * reference allocates and frees its buffers inside every NL_Means call,
 * 3DNLM/main.cu:7616-7618,7674-7676). */
int nlm_release_cached(void);

/* ---------------------------------------------------------------- 3D ------ */

/* Bytes of scratch nlm3d_forward needs for this shape (0 on invalid input).
 * Compiled (sr, pr): sr 1..5 with pr 1, sr 3 and 5 with pr 2 (register-brick
 * kernel), and sr 1..6 with pr 1..8 otherwise (large-patch kernel: the
 * reference's NS 7..17 configurations), each in FP32 or FP16 storage; for the
 * latter kernel the scratch also holds four (Z, num) float pairs per voxel for
 * sr >= 3 and two below (halves of the passes and of the x offsets), or as many
 * (Z, num, cZ, cnum) Kahan pairs with FP16 storage. */
size_t nlm3d_workspace_bytes(int X, int Y, int Z, int sr, int pr, unsigned int flags);

/*
 * 3D NLM of one volume: d_in (X*Y*Z elements of in_dtype; with
 * NLM_FLAG_PREPADDED (X+2H)*(Y+2H)*(Z+2H), H = sr+pr) -> d_out (X*Y*Z floats).
 * d_zsum (nullable) receives the per-voxel weight sum Z_p, which the adjoint
 * takes.  Replaces the device part of NLMeansProcessor::NL_Means
 * (3DNLM/main.h:6, 3DNLM/main.cu:7607-7680): its four kernel variants x 10 runs
 * become one staging pass and one fused kernel; allocation moves to the caller.
 */
int nlm3d_forward(const void* d_in, int in_dtype, int X, int Y, int Z, int sr, int pr,
                  float h, float* d_out, float* d_zsum, unsigned int flags, void* d_ws,
                  size_t ws_bytes, nlm_stream_t stream);

/*
 * The two halves of nlm3d_forward, for callers that reuse one staged volume
 * (several outputs, the adjoint) or time the fused kernel alone.
 * nlm3d_stage writes the padded, converted, pre-scaled volume into d_ws (at
 * least nlm3d_workspace_bytes); nlm3d_forward_staged runs the fused NLM kernel
 * on it.  Same (sr, pr, h, flags) must be given to both.  Replace the
 * H2D-then-launch sequence of 3DNLM/main.cu:7620-7634.
 */
int nlm3d_stage(const void* d_in, int in_dtype, int X, int Y, int Z, int sr, int pr, float h,
                unsigned int flags, void* d_ws, size_t ws_bytes, nlm_stream_t stream);
int nlm3d_forward_staged(const void* d_ws, size_t ws_bytes, int X, int Y, int Z, int sr, int pr,
                         float h, float* d_out, float* d_zsum, unsigned int flags,
                         nlm_stream_t stream);

/*
 * Allocation-free form of nlm3d_forward (no counterpart in the reference).  For
 * callers that must not allocate device memory while they run: plug-ins whose host
 * application owns all GPU memory through its own pool, and fixed-budget real-time
 * pipelines that reserve everything at start-up, where a cudaMalloc can fail
 * mid-run and a cudaFree stalls the whole device.  The staging scratch is a 16 MiB
 * array compiled into libgnlm.so: a GPU reserves it when the library's module is
 * loaded there (with CUDA's default lazy loading, at the latest on the first call
 * of this entry point) and holds it until the process exits.  Arguments are checked
 * as nlm3d_forward checks them; then volumes whose staged copy needs more (sr 3,
 * pr 1: beyond 152^3, FP32 or FP16 storage) return NLM_ERR_WORKSPACE.  The first
 * call in each CUDA context looks up the array's device address (a device reset
 * makes a new context and a new lookup); make that first call before any stream
 * capture, since it may also load the module.  All calls on a device share the
 * array: calls whose GPU work overlaps race, so serialise them (e.g. on one
 * stream).  The array keeps the last call's contents; nothing in it needs to start
 * at zero.
 */
int nlm3d_forward_noalloc(const void* d_in, int in_dtype, int X, int Y, int Z, int sr, int pr,
                          float h, float* d_out, float* d_zsum, unsigned int flags,
                          nlm_stream_t stream);

/*
 * Host-buffer form with the reference's calling semantics: synchronous, host
 * pointers in and out, device memory owned by the library (cached per device).
 * The host->device copy, the kernels and the device->host copy run in order on a
 * library stream; returns when h_out is written.  This is what
 * NLMeansProcessor::NL_Means(unsigned char*, float*) (3DNLM/main.h:6) does.
 */
int nlm3d_forward_host(const void* h_in, int in_dtype, int X, int Y, int Z, int sr, int pr,
                       float h, float* h_out, unsigned int flags);

/*
 * Adjoint of nlm3d_forward (no counterpart in the reference): for an upstream
 * gradient d_gout = dL/dout it writes dL/dv into d_gin (X*Y*Z floats) and, if
 * d_hgrad is not NULL, dL/dh into the one device double d_hgrad.  Takes the
 * forward's input d_in (FP32), output d_out and weight sums d_zsum.  The
 * per-offset weights are recomputed, not stored; gradients that land on padding
 * voxels are folded back onto their REFLECT_101 sources; every output is a
 * gather and dL/dh a fixed-order sum, so results are bitwise reproducible.
 */
size_t nlm3d_adjoint_workspace_bytes(int X, int Y, int Z, int sr, int pr);
int nlm3d_adjoint(const float* d_in, const float* d_out, const float* d_zsum, const float* d_gout,
                  int X, int Y, int Z, int sr, int pr, float h, float* d_gin, double* d_hgrad,
                  void* d_ws, size_t ws_bytes, nlm_stream_t stream);

/* -------------------------------------------------------------- batched -- */

/* One volume of a batch: device pointers owned by the caller, kept alive and
 * unchanged in address for the life of the plan (their contents may change). */
typedef struct nlm_volume {
    const void* d_in;  /* X*Y*Z elements of in_dtype, unpadded */
    int in_dtype;
    int X, Y, Z;
    int sr, pr;        /* batched form: pr = 1, sr in 1..5 */
    float h;
    float* d_out;      /* X*Y*Z floats */
    float* d_zsum;     /* nullable */
} nlm_volume;

typedef struct nlm_batch_plan nlm_batch_plan;

/*
 * Many volumes of uneven sizes, each with its own h and search radius, denoised
 * by one persistent kernel launch (no counterpart in the reference, whose sweeps
 * rerun one compile-time configuration at a time, 3DNLM/run.sh:25-34).
 * nlm3d_batch_create stages nothing yet; it allocates the plan's device memory
 * (staged copies, descriptor tables, work list), builds the tile work list (most
 * expensive first) and captures a CUDA graph [reset work counter -> stage all
 * volumes -> persistent NLM kernel].  nlm3d_batch_run replays the graph on
 * `stream` (asynchronous).  nlm3d_batch_autotune times each tile shape on the
 * batch, keeps the fastest, and returns its index (times_ms: NLM_BATCH_VARIANTS
 * entries, one per shape, nullable).  flags must be 0 (FP32).
 */
#define NLM_BATCH_VARIANTS 4
int nlm3d_batch_create(const nlm_volume* vols, int n, unsigned int flags, nlm_batch_plan** plan);
int nlm3d_batch_run(nlm_batch_plan* plan, nlm_stream_t stream);
int nlm3d_batch_autotune(nlm_batch_plan* plan, float* times_ms, nlm_stream_t stream);
int nlm3d_batch_set_variant(nlm_batch_plan* plan, int variant);
int nlm3d_batch_info(const nlm_batch_plan* plan, int* n_items, int* variant, size_t* device_bytes);
int nlm3d_batch_destroy(nlm_batch_plan* plan);
/* One-shot form of the above (no counterpart in the reference): builds a plan
 * with the default tile shape, runs it once on `stream`, waits for it and frees
 * it.  Synchronous; callers that denoise the same batch repeatedly keep a plan. */
int nlm3d_forward_batched(const nlm_volume* vols, int n, nlm_stream_t stream);

/* ------------------------------------------------------------ autotuner -- */

/*
 * Tile-shape variants of the fused kernels (no counterpart in the reference,
 * whose block/grid shape is fixed by macros, 3DNLM/main.cu:15-21).  Forward calls
 * use the recorded variant for (dims, sr, pr, FP16 flag), or, when none is
 * recorded (or after a reset with -1), a per-configuration default measured on a
 * GB300; nlm_get_variant reports whichever applies.
 */
int nlm_variant_count(int dims, unsigned int flags);
int nlm_set_variant(int dims, int sr, int pr, unsigned int flags, int variant); /* -1 = reset */
int nlm_get_variant(int dims, int sr, int pr, unsigned int flags);

/*
 * Times every variant for (dims, sr, pr, flags) on an X x Y x Z volume (temporary
 * buffers allocated here; synchronises `stream`), records the fastest and returns
 * its index (>= 0) or a negative status.  times_ms (nullable) receives
 * nlm_variant_count() per-variant best-of-3 times in milliseconds.
 */
int nlm_autotune(int dims, int X, int Y, int Z, int sr, int pr, unsigned int flags,
                 float* times_ms, nlm_stream_t stream);

/* ---------------------------------------------------------------- 2D ------ */

size_t nlm2d_workspace_bytes(int X, int Y, int sr, int pr, unsigned int flags);

/*
 * 2D NLM of one image [Y][X].  Replaces the device part of the 2D
 * NLMeansProcessor::NL_Means (2D NLM/11x11/main.h:6, 2D NLM/11x11/main.cu:472-539),
 * whose kernels only support an 11x11 patch; here any compiled (sr, pr).
 */
int nlm2d_forward(const void* d_in, int in_dtype, int X, int Y, int sr, int pr, float h,
                  float* d_out, float* d_zsum, unsigned int flags, void* d_ws,
                  size_t ws_bytes, nlm_stream_t stream);

/* Host-buffer 2D form (2D NLM/11x11/main.h:6 semantics; synchronous). */
int nlm2d_forward_host(const void* h_in, int in_dtype, int X, int Y, int sr, int pr, float h,
                       float* h_out, unsigned int flags);

#ifdef __cplusplus
}
#endif

#endif /* GNLM_NLM_H */
