// Batched 3D NLM: many volumes of uneven sizes (each with its own h and search
// radius) denoised by one persistent kernel launch, replayed as a CUDA graph.
// No counterpart in the reference, whose sweeps recompile and rerun one
// configuration at a time (3DNLM/run.sh:25-34).
//
// Plan (built once on the host):
//   * every volume is staged (REFLECT_101 pad + pre-scale with its own h) into one
//     workspace by a single batched staging launch;
//   * a device table holds, per volume, its TMA tensor map, output pointers,
//     extents, search radius and output scale;
//   * a work list holds one item per output tile of every volume, the most
//     expensive first (search radius 5 tiles cost (11/7)^3 = 3.9x those of
//     radius 3), so the greedy dynamic schedule ends balanced;
//   * graph = [zero the work counter] -> [batched staging] -> [persistent kernel].
// The persistent kernel runs (occupancy x SMs) CTAs; each CTA takes the next work
// item with one atomicAdd (no waiting: an index past the end means done), loads the
// item's tile with TMA on its mbarrier (the phase flips per item) and runs the
// single-volume kernel's tile body with z offsets in groups of four
// (fwd3d_tile_pz in nlm3d_tile.cuh; 2M+1 = 7 splits 4 + 3, 11 splits 4 + 4 + 3).  The tile shape is a template
// parameter; the plan's autotuner times each shape on the batch and keeps the
// fastest.
#include <stdio.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "../../include/nlm.h"
#include "nlm3d_tile.cuh"
#include "nlm_internal.h"

namespace gnlm {

// Per-volume device descriptor.  The tensor map must be 64-byte aligned; the
// struct takes its alignment, and cudaMalloc bases are 256-byte aligned.
struct BatchVol {  // aligned as CUtensorMap (64+ bytes) by its first member
    CUtensorMap map;
    float* out;
    float* zsum;
    int X, Y, Z, sr;
    float inv_scale;
};

// Per-volume staging descriptor and the prefix of padded rows before it.
struct StageDesc {
    const void* in;
    void* dst;
    int in_dtype, X, Y, Z, H, Xp, Yp, Xs;
    float scale;
    long long row0;  // first global padded row of this volume
};

// Padded rows of every volume (row r of volume v: y = r % Yp, z = r / Yp), one warp
// per row, resident blocks striding over the rows.  A warp finds its first row's
// volume by binary search and then advances the volume index linearly (rows are
// ordered by volume and a stride crosses few volumes), reloading the descriptor only
// when the volume changes.  Each lane owns 16-byte output chunks (4 columns) c = lane
// and lane + 32 of a row and issues both chunks' loads before either store; only the
// 2H border columns reflect (reflect101_near, no division in the common case).
__global__ void __launch_bounds__(256) batch_stage_kernel(const StageDesc* __restrict__ descs,
                                                          int n, long long total_rows) {
    const int lane = threadIdx.x & 31;
    const long long wstep = (long long)gridDim.x * 8;
    long long row = (long long)blockIdx.x * 8 + (threadIdx.x >> 5);
    if (row >= total_rows) return;
    int lo = 0, hi = n - 1;
    while (lo < hi) {  // last volume whose row0 <= row
        const int mid = (lo + hi + 1) >> 1;
        if (descs[mid].row0 <= row) lo = mid; else hi = mid - 1;
    }
    StageDesc d = descs[lo];
    long long next0 = lo + 1 < n ? descs[lo + 1].row0 : total_rows;
    for (; row < total_rows; row += wstep) {
        if (row >= next0) {
            do {
                ++lo;
                next0 = lo + 1 < n ? descs[lo + 1].row0 : total_rows;
            } while (row >= next0);
            d = descs[lo];
        }
        const unsigned r = (unsigned)(row - d.row0);  // < Zp * Yp of one volume
        const int py = (int)(r % (unsigned)d.Yp), pz = (int)(r / (unsigned)d.Yp);
        const int sy = reflect101_near(py - d.H, d.Y), sz = reflect101_near(pz - d.H, d.Z);
        float4* drow = reinterpret_cast<float4*>(static_cast<float*>(d.dst) +
                                                 ((size_t)pz * d.Yp + py) * d.Xs);
        const size_t src = ((size_t)sz * d.Y + sy) * d.X;
        const int nchunk = d.Xs / 4;
        auto load = [&](int px) -> float {
            if (px >= d.Xp) return 0.f;
            const size_t i = src + reflect101_near(px - d.H, d.X);
            float v;
            if (d.in_dtype == NLM_U8)
                v = (float)static_cast<const unsigned char*>(d.in)[i];
            else if (d.in_dtype == NLM_F16)
                v = __half2float(static_cast<const __half*>(d.in)[i]);
            else
                v = static_cast<const float*>(d.in)[i];
            return v * d.scale;
        };
        for (int c0 = lane; c0 < nchunk; c0 += 64) {
            float v[2][4];
#pragma unroll
            for (int k = 0; k < 2; ++k)
                if (c0 + 32 * k < nchunk)
#pragma unroll
                    for (int i = 0; i < 4; ++i) v[k][i] = load(4 * (c0 + 32 * k) + i);
#pragma unroll
            for (int k = 0; k < 2; ++k)
                if (c0 + 32 * k < nchunk)
                    drow[c0 + 32 * k] = make_float4(v[k][0], v[k][1], v[k][2], v[k][3]);
        }
    }
}

// Search radii the batched kernel handles (patch radius 1).
#define GNLM_BATCH_RADII(X_) X_(1) X_(2) X_(3) X_(4) X_(5)

template <int RY, int RZ, int NW>
struct BatchShape {
    // shared memory of the largest search radius compiled in
    static constexpr int SMEM = Fwd3d<5, 1, float, RY, RZ, NW>::SMEM_BYTES;
};

template <int RY, int RZ, int NW, int MINB>
__global__ void __launch_bounds__(32 * NW, MINB)
    nlm3d_batch_kernel(const BatchVol* __restrict__ vols, const int4* __restrict__ items,
                       int n_items, int* __restrict__ counter, unsigned int* errword) {
    // No static shared memory: the dynamic region (tile at offset 0) stays 128-byte
    // aligned for TMA.  The barrier and the work index sit after the largest tile.
    extern __shared__ __align__(128) unsigned char smem_raw[];
    float* tile = reinterpret_cast<float*>(smem_raw);
    constexpr int kBar = Fwd3d<5, 1, float, RY, RZ, NW>::BAR_OFF;
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw + kBar);
    int& s_item = *reinterpret_cast<int*>(smem_raw + kBar + 64);
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    for (uint32_t k = 0;; ++k) {
        if (threadIdx.x == 0) s_item = atomicAdd(counter, 1);
        __syncthreads();
        const int it = s_item;
        if (it >= n_items) break;
        const int4 item = items[it];
        const BatchVol* v = vols + item.x;
        bool ok = true;
        switch (v->sr) {
#define X_(m)                                                                                     \
    case m:                                                                                       \
        ok = fwd3d_tile_pz<m, 1, RY, RZ, NW, 4>(&v->map, tile, bar, k & 1u, item.y, item.z,      \
                                                 item.w, v->X, v->Y, v->Z, v->inv_scale, v->out,   \
                                                 v->zsum, errword);                                \
        break;
            GNLM_BATCH_RADII(X_)
#undef X_
            default:
                if (threadIdx.x == 0) raise_device_error(errword, DEVERR_BAD_DESC);
        }
        if (!ok) break;  // copy timed out: error word set, stop this CTA
        __syncthreads();  // everyone is done with the tile before the next copy
    }
}

constexpr int kBatchXO = 32 - 2 * 1;  // output columns per warp (pr = 1)

}  // namespace gnlm

using namespace gnlm;

struct nlm_batch_plan {
    int n = 0;
    int n_items = 0;
    int variant = 0;
    int device = 0;
    std::vector<nlm_volume> vols;
    std::vector<int4> items_host;
    BatchVol* d_vols = nullptr;
    int4* d_items = nullptr;
    int* d_counter = nullptr;
    StageDesc* d_stage = nullptr;
    long long total_rows = 0;
    void* d_staged = nullptr;
    size_t staged_bytes = 0;
    std::vector<Staging> st;        // staging geometry per volume
    std::vector<BatchVol> hv;       // host copy of the device volume table
    std::vector<void*> dst;         // staged copy of each volume
    cudaStream_t cap_stream = nullptr;
    cudaGraphExec_t exec = nullptr;
    int exec_variant = -1;
    std::mutex mu;
};

namespace {

constexpr int kBatchVariants = NLM_BATCH_VARIANTS;  // (RY, RZ): (4, 8), (4, 4), (2, 8), (4, 6); 4 warps

// Sets the kernel's shared-memory limit and returns its persistent grid size.
template <int RY, int RZ, int MINB>
cudaError_t config_batch(nlm_batch_plan* p, int* ctas) {
    auto kern = nlm3d_batch_kernel<RY, RZ, 4, MINB>;
    const int smem = BatchShape<RY, RZ, 4>::SMEM;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0, sms = 0;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 128, smem))) return e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, p->device))) return e;
    *ctas = std::max(1, std::min(std::max(per_sm, 1) * sms, p->n_items));
    return cudaSuccess;
}

template <int RY, int RZ, int MINB>
cudaError_t launch_batch(nlm_batch_plan* p, cudaStream_t s, int ctas, unsigned int* ew) {
    nlm3d_batch_kernel<RY, RZ, 4, MINB><<<ctas, 128, BatchShape<RY, RZ, 4>::SMEM, s>>>(
        p->d_vols, p->d_items, p->n_items, p->d_counter, ew);
    return cudaGetLastError();
}

cudaError_t config_variant(nlm_batch_plan* p, int v, int* ctas) {
    switch (v) {
        case 0: return config_batch<4, 8, 2>(p, ctas);
        case 1: return config_batch<4, 4, 2>(p, ctas);
        case 2: return config_batch<2, 8, 2>(p, ctas);
        case 3: return config_batch<4, 6, 2>(p, ctas);
    }
    return cudaErrorInvalidValue;
}

cudaError_t launch_variant(nlm_batch_plan* p, int v, cudaStream_t s, int ctas, unsigned int* ew) {
    switch (v) {
        case 0: return launch_batch<4, 8, 2>(p, s, ctas, ew);
        case 1: return launch_batch<4, 4, 2>(p, s, ctas, ew);
        case 2: return launch_batch<2, 8, 2>(p, s, ctas, ew);
        case 3: return launch_batch<4, 6, 2>(p, s, ctas, ew);
    }
    return cudaErrorInvalidValue;
}

int tile_ty(int v) { return v == 2 ? 8 : 16; }  // NW (4) x RY
int tile_rz(int v) { return v == 1 ? 4 : v == 3 ? 6 : 8; }

// Work list for tile shape v: all tiles of all volumes, most expensive first.
void build_items(nlm_batch_plan* p, int v) {
    std::vector<std::pair<long long, int4>> list;
    for (int i = 0; i < p->n; ++i) {
        const nlm_volume& vol = p->vols[i];
        const int XO = kBatchXO, TY = tile_ty(v), RZ = tile_rz(v);
        const long long cost = (long long)(2 * vol.sr + 1) * (2 * vol.sr + 1) * (2 * vol.sr + 1);
        for (int bz = 0; bz < (vol.Z + RZ - 1) / RZ; ++bz)
            for (int by = 0; by < (vol.Y + TY - 1) / TY; ++by)
                for (int bx = 0; bx < (vol.X + XO - 1) / XO; ++bx)
                    list.push_back({cost, make_int4(i, bx, by, bz)});
    }
    std::stable_sort(list.begin(), list.end(),
                     [](const auto& a, const auto& b) { return a.first > b.first; });
    p->items_host.clear();
    for (auto& e : list) p->items_host.push_back(e.second);
    p->n_items = (int)p->items_host.size();
}

int set_error(int code, const char* msg) {
    if (code == NLM_ERR_CUDA) cudaGetLastError();  // consume a non-sticky error
    return report_error(code, msg);
}

// TMA boxes of tile shape v: the box must equal the tile the kernel expects for
// the volume's search radius (columns 32 + 2 sr + 2 rounded to 16 bytes, TY + 2H
// rows, RZ + 2H planes) because its byte count is what the mbarrier waits for.
cudaError_t encode_maps(nlm_batch_plan* p, int v) {
    for (int i = 0; i < p->n; ++i) {
        const Staging& st = p->st[i];
        const int sr = p->vols[i].sr, H = st.H;
        const uint64_t dims[3] = {(uint64_t)st.Xs, (uint64_t)st.Yp, (uint64_t)st.Zp};
        const uint64_t strides[2] = {(uint64_t)st.Xs * 4, (uint64_t)st.Xs * st.Yp * 4};
        const uint32_t box[3] = {(uint32_t)((32 + 2 * sr + 2 + 3) / 4 * 4),
                                 (uint32_t)(tile_ty(v) + 2 * H), (uint32_t)(tile_rz(v) + 2 * H)};
        cudaError_t e = encode_tensor_map(&p->hv[i].map, false, 3, dims, strides, box, p->dst[i]);
        if (e != cudaSuccess) return e;
    }
    return cudaMemcpy(p->d_vols, p->hv.data(), sizeof(BatchVol) * p->n, cudaMemcpyHostToDevice);
}

// (Re)writes the device work list and tensor maps for tile shape v, then
// re-captures the graph.
int prepare(nlm_batch_plan* p, int v) {
    build_items(p, v);
    if (encode_maps(p, v) != cudaSuccess)
        return set_error(NLM_ERR_CUDA, "batch tensor map encoding failed");
    int ctas = 0;
    if (config_variant(p, v, &ctas) != cudaSuccess)
        return set_error(NLM_ERR_CUDA, "batch kernel configuration failed");
    unsigned int* ew = device_error_word();
    cudaFree(p->d_items);
    p->d_items = nullptr;
    cudaError_t e = cudaMalloc((void**)&p->d_items, sizeof(int4) * p->items_host.size());
    if (e == cudaSuccess)
        e = cudaMemcpy(p->d_items, p->items_host.data(), sizeof(int4) * p->items_host.size(),
                       cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return set_error(NLM_ERR_CUDA, "batch work list upload failed");
    if (p->exec) {
        cudaGraphExecDestroy(p->exec);
        p->exec = nullptr;
    }
    // staging grid: resident blocks (SMs x blocks per SM), queried before the capture
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_stage_kernel, 256, 0) !=
            cudaSuccess || per_sm <= 0) {
        cudaGetLastError();
        per_sm = 1;
    }
    const unsigned stage_blocks = (unsigned)std::max(
        1LL, std::min((p->total_rows + 7) / 8, (long long)device_sm_count() * per_sm));
    cudaGraph_t graph = nullptr;
    e = cudaStreamBeginCapture(p->cap_stream, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) e = cudaMemsetAsync(p->d_counter, 0, sizeof(int), p->cap_stream);
    if (e == cudaSuccess) {
        batch_stage_kernel<<<stage_blocks, 256, 0, p->cap_stream>>>(p->d_stage, p->n,
                                                                   p->total_rows);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = launch_variant(p, v, p->cap_stream, ctas, ew);
    cudaError_t e2 = cudaStreamEndCapture(p->cap_stream, &graph);
    if (e == cudaSuccess) e = e2;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&p->exec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
        char msg[160];
        snprintf(msg, sizeof(msg), "batch graph capture failed: %s", cudaGetErrorString(e));
        return set_error(NLM_ERR_CUDA, msg);
    }
    p->variant = p->exec_variant = v;
    return NLM_OK;
}

void free_plan(nlm_batch_plan* p) {
    if (p->exec) cudaGraphExecDestroy(p->exec);
    if (p->cap_stream) cudaStreamDestroy(p->cap_stream);
    cudaFree(p->d_vols);
    cudaFree(p->d_items);
    cudaFree(p->d_counter);
    cudaFree(p->d_stage);
    cudaFree(p->d_staged);
    delete p;
}

}  // namespace

extern "C" {

int nlm3d_batch_create(const nlm_volume* vols, int n, unsigned int flags, nlm_batch_plan** out) {
    if (!out) return set_error(NLM_ERR_INVALID_ARG, "plan pointer is NULL");
    *out = nullptr;
    if (!vols || n < 1) return set_error(NLM_ERR_INVALID_ARG, "empty batch");
    if (flags != 0) return set_error(NLM_ERR_INVALID_ARG, "batched form takes no flags (FP32)");
    for (int i = 0; i < n; ++i) {
        const nlm_volume& v = vols[i];
        char msg[160];
        if (!v.d_in || !v.d_out || v.X < 1 || v.Y < 1 || v.Z < 1 || !(v.h > 0.f) ||
            (v.in_dtype != NLM_U8 && v.in_dtype != NLM_F16 && v.in_dtype != NLM_F32) ||
            v.Z + 2 * (v.sr + v.pr) > 65535) {
            snprintf(msg, sizeof(msg), "volume %d: invalid descriptor", i);
            return set_error(NLM_ERR_INVALID_ARG, msg);
        }
        if (v.pr != 1 || v.sr < 1 || v.sr > 5) {
            snprintf(msg, sizeof(msg), "volume %d: batched form supports pr 1, sr 1..5", i);
            return set_error(NLM_ERR_UNSUPPORTED, msg);
        }
    }
    nlm_batch_plan* p = new nlm_batch_plan();
    p->n = n;
    p->vols.assign(vols, vols + n);
    cudaGetDevice(&p->device);
    std::vector<BatchVol> hv(n);
    std::vector<StageDesc> hs(n);
    std::vector<Staging> st(n);
    size_t off = 0;
    long long rows = 0;
    for (int i = 0; i < n; ++i) {
        const nlm_volume& v = vols[i];
        st[i] = make_staging(v.X, v.Y, v.Z, v.sr + v.pr, v.sr + v.pr, false);
        hs[i].in = v.d_in;
        hs[i].dst = reinterpret_cast<void*>(off);  // offset; rebased after allocation
        hs[i].in_dtype = v.in_dtype;
        hs[i].X = v.X;
        hs[i].Y = v.Y;
        hs[i].Z = v.Z;
        hs[i].H = st[i].H;
        hs[i].Xp = st[i].Xp;
        hs[i].Yp = st[i].Yp;
        hs[i].Xs = st[i].Xs;
        const double k = 3.0;
        hs[i].scale = (float)sqrt(1.4426950408889634 / (k * k * k * (double)v.h * (double)v.h));
        hs[i].row0 = rows;
        rows += (long long)st[i].Yp * st[i].Zp;
        off += st[i].bytes();
    }
    p->total_rows = rows;
    p->staged_bytes = off;
    cudaError_t e = cudaMalloc(&p->d_staged, off);
    if (e == cudaSuccess) e = cudaMalloc((void**)&p->d_vols, sizeof(BatchVol) * n);
    if (e == cudaSuccess) e = cudaMalloc((void**)&p->d_stage, sizeof(StageDesc) * n);
    if (e == cudaSuccess) e = cudaMalloc((void**)&p->d_counter, sizeof(int));
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&p->cap_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        free_plan(p);
        return set_error(NLM_ERR_CUDA, "batch plan allocation failed");
    }
    p->st = st;
    p->dst.resize(n);
    for (int i = 0; i < n; ++i) {
        void* dst = static_cast<char*>(p->d_staged) + reinterpret_cast<size_t>(hs[i].dst);
        hs[i].dst = dst;
        p->dst[i] = dst;
        const nlm_volume& v = vols[i];
        hv[i].out = v.d_out;
        hv[i].zsum = v.d_zsum;
        hv[i].X = v.X;
        hv[i].Y = v.Y;
        hv[i].Z = v.Z;
        hv[i].sr = v.sr;
        hv[i].inv_scale = 1.0f / hs[i].scale;
    }
    p->hv = hv;
    e = cudaMemcpy(p->d_stage, hs.data(), sizeof(StageDesc) * n, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        free_plan(p);
        return set_error(NLM_ERR_CUDA, "batch descriptor upload failed");
    }
    int rc = prepare(p, 0);
    if (rc != NLM_OK) {
        free_plan(p);
        return rc;
    }
    *out = p;
    return NLM_OK;
}

int nlm3d_batch_run(nlm_batch_plan* p, nlm_stream_t stream) {
    if (!p) return set_error(NLM_ERR_INVALID_ARG, "plan is NULL");
    std::lock_guard<std::mutex> lk(p->mu);
    cudaError_t e = cudaGraphLaunch(p->exec, (cudaStream_t)stream);
    if (e != cudaSuccess) return set_error(NLM_ERR_CUDA, "batch graph launch failed");
    return NLM_OK;
}

int nlm3d_batch_set_variant(nlm_batch_plan* p, int variant) {
    if (!p) return set_error(NLM_ERR_INVALID_ARG, "plan is NULL");
    if (variant < 0 || variant >= kBatchVariants)
        return set_error(NLM_ERR_INVALID_ARG, "batch tile variant out of range");
    std::lock_guard<std::mutex> lk(p->mu);
    cudaDeviceSynchronize();
    return prepare(p, variant);
}

int nlm3d_batch_autotune(nlm_batch_plan* p, float* times_ms, nlm_stream_t stream_) {
    if (!p) return set_error(NLM_ERR_INVALID_ARG, "plan is NULL");
    cudaStream_t stream = (cudaStream_t)stream_;
    int best = -1;
    float best_ms = 0.f;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    auto done = [&](int rc) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        return rc;
    };
    for (int v = 0; v < kBatchVariants; ++v) {
        int rc = nlm3d_batch_set_variant(p, v);
        if (rc != NLM_OK) return done(rc);
        float ms = 1e30f;
        for (int rep = 0; rep < 3; ++rep) {
            cudaEventRecord(e0, stream);
            rc = nlm3d_batch_run(p, stream_);
            if (rc != NLM_OK) return done(rc);
            cudaEventRecord(e1, stream);
            cudaEventSynchronize(e1);
            float t = 0.f;
            cudaEventElapsedTime(&t, e0, e1);
            if (rep > 0 && t < ms) ms = t;
        }
        if (times_ms) times_ms[v] = ms;
        if (best < 0 || ms < best_ms) {
            best = v;
            best_ms = ms;
        }
    }
    done(NLM_OK);
    int rc = nlm3d_batch_set_variant(p, best);
    return rc == NLM_OK ? best : rc;
}

int nlm3d_batch_info(const nlm_batch_plan* p, int* n_items, int* variant, size_t* device_bytes) {
    if (!p) return set_error(NLM_ERR_INVALID_ARG, "plan is NULL");
    if (n_items) *n_items = p->n_items;
    if (variant) *variant = p->variant;
    if (device_bytes)
        *device_bytes = p->staged_bytes + sizeof(BatchVol) * p->n + sizeof(StageDesc) * p->n +
                        sizeof(int4) * p->n_items + sizeof(int);
    return NLM_OK;
}

int nlm3d_batch_destroy(nlm_batch_plan* p) {
    if (!p) return NLM_OK;
    cudaDeviceSynchronize();
    free_plan(p);
    return NLM_OK;
}

int nlm3d_forward_batched(const nlm_volume* vols, int n, nlm_stream_t stream) {
    nlm_batch_plan* p = nullptr;
    int rc = nlm3d_batch_create(vols, n, 0, &p);
    if (rc != NLM_OK) return rc;
    rc = nlm3d_batch_run(p, stream);
    const cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
    nlm3d_batch_destroy(p);
    if (rc != NLM_OK) return rc;
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_error(NLM_ERR_CUDA, "batched forward failed");
    }
    return NLM_OK;
}

}  // extern "C"
