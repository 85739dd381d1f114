// Host-side declarations shared by the translation units of libgnlm.so.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace gnlm {

constexpr size_t kAlign = 256;
inline size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// Device-resident staging copy of one volume: REFLECT_101-padded by `H` voxels
// in x and y and by `Hz` in z (Hz = 0 for 2D), converted to the storage type
// and pre-multiplied by `scale` = sqrt(log2(e) / (P h^2)) so that the kernels
// get the base-2 exponent of the weight directly as a sum of squared
// differences.  Layout [Zp][Yp][Xs], x stride Xs a multiple of 16 bytes (the
// TMA global-stride rule).
//
// 3D FP16 storage uses the row-pair layout instead (pairs = true): two copies,
// E and O, each [Zp][Yq][Xs] of half2, where E pair k holds padded rows (2k, 2k+1)
// and O pair k holds rows (2k+1, 2k+2) (zero past the last row).  One 32-bit
// load then yields one voxel of two adjacent rows, whichever row a search offset
// starts on.
struct Staging {
    int X = 0, Y = 0, Z = 0;  // unpadded extents
    int H = 0, Hz = 0;        // halo in x/y and in z
    int Xp = 0, Yp = 0, Zp = 0;
    int Xs = 0;               // x stride in elements
    int elem = 4;             // 4 (FP32, or a half2 pair), 2 (FP16)
    bool pairs = false;       // row-pair FP16 layout (two copies)
    int Yq = 0;               // row pairs per copy
    size_t copy_bytes() const { return align_up((size_t)Xs * Yq * Zp * 4, kAlign); }
    size_t bytes() const {
        return pairs ? 2 * copy_bytes() : align_up((size_t)Xs * Yp * Zp * elem, kAlign);
    }
};

Staging make_staging(int X, int Y, int Z, int H, int Hz, bool fp16);
// 3D FP16-storage staging (row-pair layout).
Staging make_staging_pairs(int X, int Y, int Z, int H);
// The staging layout the 3D forward uses for (sr, pr, fp16): FP32; FP16 row pairs
// (register-brick kernel); or plain FP16 (large-patch kernel).
Staging staging3d(int X, int Y, int Z, int sr, int pr, bool fp16);

// Pads, converts and scales `in` into `dst` (layout of `st`).  in_dtype is an
// nlm_dtype; with `prepadded` the input already has the halo (layout
// [Zp][Yp][Xp], no stride padding) and is copied, converted and scaled only.
// [pz0, pz1): range of padded planes to stage (pz1 < 0: through the last).
cudaError_t launch_stage(const void* in, int in_dtype, bool prepadded, float scale,
                         const Staging& st, void* dst, cudaStream_t stream, int pz0 = 0,
                         int pz1 = -1);

// 3D forward over a staged volume.  Returns cudaErrorNotSupported when the
// (sr, pr, fp16) combination has no compiled instance.
// [zt0, zt1): range of z tiles to compute (zt1 < 0: through the last); a z tile
// is nlm3d_fwd_tile_z(sr, pr, fp16, variant) output planes.
// Large-patch configurations (nlm3d_fwd_large_patch) keep per-voxel (Z, num)
// accumulator pairs (two buffers; Kahan pairs with FP16 storage) in the workspace right
// after the staged volume: nlm3d_fwd_extra_bytes() more bytes at staged + st.bytes().
cudaError_t launch_nlm3d_fwd(const Staging& st, const void* staged, int sr, int pr, bool fp16,
                             int variant, float inv_scale, float* out, float* zsum,
                             unsigned int* errword, cudaStream_t stream, int zt0 = 0,
                             int zt1 = -1);
bool nlm3d_fwd_supported(int sr, int pr, bool fp16);
int nlm3d_fwd_variant_count(bool fp16);
int nlm3d_fwd_tile_z(int sr, int pr, bool fp16, int variant);
bool nlm3d_fwd_large_patch(int sr, int pr, bool fp16);
size_t nlm3d_fwd_extra_bytes(int X, int Y, int Z, int sr, int pr, bool fp16);

// Large-patch kernel (nlm3d_lp.cu): chunk depth per variant, compiled pairs, launch.
// FP32 staging, or (fp16) plain FP16 staging [Zp][Yp][Xs]; `acc` holds two buffers of
// per-voxel (Z, num) float2, or (Z, num, cZ, cnum) float4 Kahan pairs for FP16.
int nlm3d_lp_tile_z(int variant);
bool nlm3d_lp_supported(int sr, int pr);
int nlm3d_lp_split(int X, int Y, int Z, int tz, int tile_x, int tile_y, int xparts,
                   int ctas_per_sm);
cudaError_t launch_nlm3d_lp(const Staging& st, const void* staged, int sr, int pr, bool fp16,
                            int variant, float inv_scale, float* out, float* zsum, void* acc,
                            unsigned int* errword, cudaStream_t stream, int zc0, int zc1);

// 3D adjoint (see nlm3d_adj.cu).  Scratch: (G, out') pairs (2 st.bytes()), gpad'
// (st.bytes()), adj3d_ctas() doubles of h partial sums and adj3d_side_bytes() of
// partial bricks of split tail tiles.
bool nlm3d_adj_supported(int sr, int pr);
size_t adj3d_ctas(const Staging& st, int sr, int pr);
size_t adj3d_side_bytes(int sr, int pr);
cudaError_t launch_nlm3d_adj(const Staging& st, const void* staged, const float* d_out,
                             const float* d_zsum, const float* d_gout, int sr, int pr, float s,
                             float h, float* gin, double* hgrad, float2* GO, float* gpad,
                             double* hpart, float* side, unsigned int* errword,
                             cudaStream_t stream);

// Multiprocessors of the current device (1 if it cannot be queried).
int device_sm_count();

// Tile-shape variant the forward uses for (dims, sr, pr, fp16): the autotuned
// choice if one was recorded, else default_variant().
int tuned_variant(int dims, int sr, int pr, bool fp16);
int default_variant(int dims, int sr, int pr, bool fp16);

// 2D forward over a staged image (Z = 1, Hz = 0).
cudaError_t launch_nlm2d_fwd(const Staging& st, const void* staged, int sr, int pr, bool fp16,
                             int variant, float inv_scale, float* out, float* zsum,
                             unsigned int* errword, cudaStream_t stream);
bool nlm2d_fwd_supported(int sr, int pr, bool fp16);
int nlm2d_fwd_variant_count();

// cuTensorMapEncodeTiled through the runtime's driver entry point (no -lcuda).
// dims/strides follow the driver API: dims[0] innermost, strides in bytes for
// dims 1..rank-1.
cudaError_t encode_tensor_map(CUtensorMap* map, bool fp16, int rank, const uint64_t* dims,
                              const uint64_t* strides_bytes, const uint32_t* box, void* base);

// Address of the calling device's error word (see nlm_device_status).
unsigned int* device_error_word();

// Unique ID (cuCtxGetId) of the calling thread's current context; false if no
// context is current yet or the driver entry points are unavailable.
bool current_context_id(unsigned long long* id);

// Device address of a __device__ variable, given by its host-side shadow, in the
// calling thread's current context (cached per context ID); nullptr on failure.
void* symbol_address(const void* symbol);

// The argument checks of nlm3d_forward (pointers, dtype, radii, h, flags, extents,
// compiled (sr, pr)); NLM_OK or the status it would return (message recorded).
int validate_forward3d(const void* in, const void* out, int in_dtype, int X, int Y, int Z, int sr,
                       int pr, float h, unsigned int flags);

// Records `msg` as the calling thread's nlm_last_error() text; returns `code`.
int report_error(int code, const char* msg);

}  // namespace gnlm
