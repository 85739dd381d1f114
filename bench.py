#!/usr/bin/env python3
"""Throughput of the GB300 NLM denoiser on the 3D 256^3 workload.

Workload: one 256x256x256 float32 volume (64 seeded ellipsoids, sigma 0.05),
search 7^3 (sr 3), patch 3^3 (pr 1), h 0.05.  A step is one forward pass over
the volume: the staging pass (REFLECT_101 pad + pre-scale) and the fused NLM
kernel, input resident in HBM.  Between timed steps a 256 MiB buffer is
written to flush the 129 MB L2.  ``value`` is Mvoxel/s of the plain FP32 form;
the FP16-storage form is reported beside it.  ``e2e`` is the same metric through
the host-buffer C-ABI call (nlm3d_forward_host) with the host<->device copies
inside the timed region.

``--impl reference`` times the reference's path on the host cores instead.  The
reference ships no CPU implementation of NLM (its nlm.cpp only calls the GPU),
so that arm runs the oracle's FP32 separable restatement of the reference's
arithmetic with every host thread, on a bounded z-slab sample of the same
volume per step.

Multi-GPU: the path does not shard; under torchrun every rank denoises its own
replica and ``value`` sums the ranks' voxels over the slowest rank's time.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "3d-gnlm_gb300"))
sys.path.insert(0, os.path.join(REPO, "oracle"))

import numpy as np  # noqa: E402

METRIC = "Mvoxel/s 3D NLM 256³ S7³ P3³ (fp32 vs fp16-store/batched); fwd+adjoint ms"
UNIT = "Mvoxel/s"
SHAPE = (256, 256, 256)
SR, PR, H = 3, 1, 0.05
N_ELLIPSOIDS, SIGMA, SEED = 64, 0.05, 2
OFFSETS = (2 * SR + 1) ** 3
FLOPS_PER_PAIR = 12  # diff, square, 6 box-sum add/sub, scale, Z add, num FMA (2)
# Adjoint, per (padded voxel, offset): distance recomputed (diff, square, 6 box-sum
# add/sub, scale = 9); a = e [G(u)(v'(u+o) - out'(u)) + G(u+o)(v'(u) - out'(u+o))]
# (2 differences, 2 products, 1 add, times e = 6); box sum of a (6 add/sub); gathered
# terms G(q+o) e + (-2 ln2) t A (FMA 2, product + FMA 3 = 5); dL/dh term a1 D'
# (product + FMA = 3).  The padded domain is the unit: halo gradients fold back
# through REFLECT_101.
ADJ_FLOPS_PER_PAIR = 29
L2_FLUSH_BYTES = 256 << 20
WORKLOAD_NAME = "nlm3d_256cubed_sr3_pr1_fp32"


def env_rank():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


def max_over_ranks(dist, value, device):
    """The largest `value` over all ranks (the slowest replica sets the job's time);
    `value` itself without a process group.  `device` is where the reduction tensor
    lives: "cuda" for NCCL, "cpu" for gloo."""
    if dist is None:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(units_per_rank, world, seconds_max):
    """Whole-job throughput of `world` independent replicas, each processing
    `units_per_rank` units: all units over the slowest replica's time."""
    return world * units_per_rank / seconds_max


class ClockSampler:
    """nvidia-smi clock/throttle samples every 200 ms while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": reasons,
                "samples": len(rows)}


def fp32_peak_tflops(torch, packed=False):
    """FP32 FMA throughput of this GPU, measured by the probe kernel (best of 3).
    packed=True measures the FFMA2 (f32x2) form instead."""
    import gnlm
    path = os.path.join(gnlm.LIB_DIR, "libgnlm_probe.so")
    P = ctypes.CDLL(path)
    P.gnlm_probe_fp32.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
    P.gnlm_probe_fp32x2.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
    probe = P.gnlm_probe_fp32x2 if packed else P.gnlm_probe_fp32
    P.gnlm_probe_fp32_flops.argtypes = [ctypes.c_int, ctypes.c_int]
    P.gnlm_probe_fp32_flops.restype = ctypes.c_double
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    blocks, iters = sms * 8, 2048
    buf = torch.empty(blocks, device="cuda")
    s = torch.cuda.current_stream()
    best = 0.0
    for i in range(4):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        probe(ctypes.c_void_p(buf.data_ptr()), blocks, iters, ctypes.c_void_p(s.cuda_stream))
        e1.record()
        e1.synchronize()
        if i > 0:
            flops = P.gnlm_probe_fp32_flops(blocks, iters) * (2 if packed else 1)
            best = max(best, flops / (e0.elapsed_time(e1) * 1e-3))
    return best / 1e12


TRAFFIC_SOURCE = ("from the committed ncu capture (profiles/traffic.txt: dram__bytes_read.sum + "
                  "dram__bytes_write.sum of one launch of this workload), not measured in this run")


def read_profile_traffic(kernel_key):
    """Per-launch DRAM bytes of a kernel from profiles/traffic.txt, an ncu capture
    committed with the repository (a lookup, not a measurement of the current run)."""
    path = os.path.join(REPO, "profiles", "traffic.txt")
    if not os.path.exists(path):
        return None
    for line in open(path):
        parts = line.split()
        if len(parts) >= 3 and not line.startswith("#") and parts[0] == kernel_key:
            return float(parts[2])
    return None


def measured_hbm_peak():
    """(GB/s, source) of the HBM copy peak: MEASURED_PEAKS.json at the repository root
    (a STREAM-style copy measured on the GB300s), else the fallback figure."""
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            v = float(json.load(f)["hbm_gbs"])
        if v > 0:
            return v, "of measured (MEASURED_PEAKS.json hbm_gbs, copy)"
    except (OSError, KeyError, ValueError, TypeError):
        pass
    return 6800.0, "of fallback (6.8 TB/s copy on a GB300)"


def staging_bytes(shape, sr, pr, in_bytes=4, elem=4):
    """Algorithmic bytes of one staging pass: the input read once and the padded
    volume ([Z+2H][Y+2H][X+2H rounded up to 16 bytes]) written once."""
    Z, Y, X = shape
    H = sr + pr
    per16 = 16 // elem
    xs = (X + 2 * H + per16 - 1) // per16 * per16
    return Z * Y * X * in_bytes + (Z + 2 * H) * (Y + 2 * H) * xs * elem


def cpu_baseline(shape, budget_s=10.0):
    """Oracle FP32 separable form on a z-slab of the workload, all host threads."""
    import oracle as O
    from gnlm import phantom
    threads = os.cpu_count() or 1
    O.set_threads(threads)
    Z, Y, X = shape
    vol, _ = phantom.ellipsoid_phantom(shape, n_ellipsoids=N_ELLIPSOIDS, sigma=SIGMA, seed=SEED)
    nz = 16  # calibration slab
    t0 = time.perf_counter()
    O.nlm3d(np.ascontiguousarray(vol[:nz]), SR, PR, H)
    dt = time.perf_counter() - t0
    rate = nz * Y * X / dt
    nz = int(min(Z, max(4, budget_s * rate / (Y * X))))
    slab = np.ascontiguousarray(vol[Z // 2 - nz // 2:Z // 2 - nz // 2 + nz])
    t0 = time.perf_counter()
    O.nlm3d(slab, SR, PR, H)
    dt = time.perf_counter() - t0
    # the same port on one thread, on a thinner slab
    O.set_threads(1)
    slab1 = np.ascontiguousarray(vol[Z // 2 - 2:Z // 2 + 2])
    t1 = time.perf_counter()
    O.nlm3d(slab1, SR, PR, H)
    dt1 = time.perf_counter() - t1
    O.set_threads(threads)
    return {"value": round(nz * Y * X / dt / 1e6, 3), "unit": UNIT, "cores": threads,
            "kind": "port",
            "single_thread_value": round(slab1.size / dt1 / 1e6, 3),
            "sample": f"z-slab {nz}x{Y}x{X} of the 256^3 volume, oracle FP32 separable form "
                      f"(reflect borders at the slab ends), {dt:.1f} s; single thread: "
                      f"z-slab 4x{Y}x{X}, {dt1:.1f} s"}


def bench_batched(torch, gnlm, reps=3):
    """64 uneven volumes (dims in {32..192}, sr 3 for half and 5 for the other
    half, pr 1, h = sigma): one graph-captured persistent launch against 64
    sequential single-volume launches on the same stream, both device-timed."""
    from gnlm import phantom
    specs = phantom.batch_specs()
    vols = [(torch.from_numpy(v).cuda(), s["sr"], 1, s["h"])
            for v, s in zip(phantom.batch_volumes(specs), specs)]
    nvox = sum(t.numel() for t, *_ in vols)
    plan = gnlm.BatchPlan(vols)
    best, tune_ms = plan.autotune()
    stream = torch.cuda.current_stream()

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        ms = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
        return min(ms)

    batch_ms = timed(plan.run)
    outs = [torch.empty_like(t) for t, *_ in vols]

    def sequential():
        for (t, sr, pr, h), o in zip(vols, outs):
            gnlm.nlm3d_forward(t, sr, pr, h, out=o)

    seq_ms = timed(sequential)
    same = max(float((a - b).abs().max()) for a, b in zip(plan.outputs, outs))
    info = plan.info()
    # every voxel of all 64 batched outputs against the FP64 separable oracle
    import oracle as O
    emax, sq = 0.0, 0.0
    for (t, sr, pr, h), o in zip(vols, plan.outputs):
        ref = O.nlm3d(t.cpu().numpy(), sr, pr, h, dtype=np.float64)
        d = o.cpu().numpy().astype(np.float64) - ref
        emax = max(emax, float(np.abs(d).max()))
        sq += float((d * d).sum())
    plan.close()
    return {"volumes": len(vols), "voxels": nvox, "work_items": info["items"],
            "max_abs_err_vs_fp64": emax, "rms_err_vs_fp64": (sq / nvox) ** 0.5,
            "error_sample": "every voxel of the 64 volumes vs the FP64 separable oracle",
            "value": round(nvox / (batch_ms * 1e-3) / 1e6, 2), "ms": round(batch_ms, 3),
            "sequential_value": round(nvox / (seq_ms * 1e-3) / 1e6, 2),
            "sequential_ms": round(seq_ms, 3), "speedup_vs_sequential": round(seq_ms / batch_ms, 3),
            "variant": best, "autotune_ms": [round(t, 3) for t in tune_ms],
            "max_abs_diff_vs_sequential": same}


def bench_2d(torch, gnlm, reps=5):
    """2048^2 image (32 discs/rectangles, sigma 0.08), search 11^2, patch 5^2, h 0.08."""
    from gnlm import phantom
    im, _ = phantom.disc_rect_phantom((2048, 2048), n_shapes=32, sigma=0.08, seed=0)
    x = torch.from_numpy(im).cuda()
    best, tune = gnlm.autotune(2, (1, 2048, 2048), 5, 2)
    out = torch.empty_like(x)
    gnlm.nlm2d_forward(x, 5, 2, 0.08, out=out)
    torch.cuda.synchronize()
    ms = []
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        gnlm.nlm2d_forward(x, 5, 2, 0.08, out=out)
        e1.record()
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
    t = min(ms)
    import oracle as O
    d = out.cpu().numpy().astype(np.float64) - O.nlm2d(im, 5, 2, 0.08, dtype=np.float64)
    return {"shape": [2048, 2048], "search_radius": 5, "patch_radius": 2, "ms": round(t, 4),
            "max_abs_err_vs_fp64": float(np.abs(d).max()),
            "rms_err_vs_fp64": float(np.sqrt(np.mean(d * d))),
            "error_sample": "every pixel vs the FP64 separable oracle",
            "value": round(2048 * 2048 / (t * 1e-3) / 1e6, 1), "unit": "Mpixel/s",
            "tflops": round(10 * 121 * 2048 * 2048 / (t * 1e-3) / 1e12, 2), "variant": best,
            "autotune_ms": [round(v, 4) for v in tune]}


def bench_large_patch(torch, gnlm, reps=3):
    """The largest configuration of the reference's large-patch sweep: 512 x 512 x 128,
    search 13^3 (sr 6), patch 17^3 (pr 8), h 0.05, 48 ellipsoids sigma 0.05; staging +
    large-patch kernel per call."""
    from gnlm import phantom
    shape, sr, pr = (128, 512, 512), 6, 8
    v, _ = phantom.ellipsoid_phantom(shape, n_ellipsoids=48, sigma=0.05, seed=4)
    x = torch.from_numpy(v).cuda()
    best, tune = gnlm.autotune(3, shape, sr, pr)
    out = torch.empty_like(x)
    gnlm.nlm3d_forward(x, sr, pr, 0.05, out=out)
    torch.cuda.synchronize()
    ms = []
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        gnlm.nlm3d_forward(x, sr, pr, 0.05, out=out)
        e1.record()
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
    t = min(ms)
    nvox = shape[0] * shape[1] * shape[2]
    pairs = nvox * (2 * sr + 1) ** 3
    gnlm.set_variant(3, sr, pr, -1)
    g = out.cpu().numpy()
    # the FP16-storage form of the same configuration
    best16, tune16 = gnlm.autotune(3, shape, sr, pr, fp16_storage=True)
    gnlm.nlm3d_forward(x, sr, pr, 0.05, out=out, fp16_storage=True)
    torch.cuda.synchronize()
    ms16 = []
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        gnlm.nlm3d_forward(x, sr, pr, 0.05, out=out, fp16_storage=True)
        e1.record()
        e1.synchronize()
        ms16.append(e0.elapsed_time(e1))
    t16 = min(ms16)
    g16 = out.cpu().numpy()
    gnlm.set_variant(3, sr, pr, -1, fp16_storage=True)
    # FP64 oracle on 16^3 boxes at the 8 corners, the 6 face centres and the centre
    import oracle as O
    blk = (16, 16, 16)
    origins = O.border_blocks(shape, blk)
    ref = O.nlm3d_blocks(v, sr, pr, 0.05, origins, blk)
    d = np.stack([g[z:z + 16, y:y + 16, x:x + 16] for (z, y, x) in origins]).astype(np.float64) - ref
    d16 = np.stack([g16[z:z + 16, y:y + 16, x:x + 16]
                    for (z, y, x) in origins]).astype(np.float64) - ref
    return {"shape": list(shape), "search_radius": sr, "patch_radius": pr, "ms": round(t, 3),
            "max_abs_err_vs_fp64": float(np.abs(d).max()),
            "rms_err_vs_fp64": float(np.sqrt(np.mean(d * d))),
            "error_sample": f"{len(origins)} boxes of 16^3 (8 corners, 6 face centres, centre; "
                            f"{d.size} voxels) vs the FP64 separable oracle",
            "value": round(nvox / (t * 1e-3) / 1e6, 2), "unit": "Mvoxel/s",
            "gpairs_per_s": round(pairs / (t * 1e-3) / 1e9, 1),
            "tflops": round(FLOPS_PER_PAIR * pairs / (t * 1e-3) / 1e12, 2),
            "kernel": "nlm3d_lpx_kernel<6,8,float,48> (x-offset halves, 48-row tiles)",
            "variant": best,
            "fp16_storage": {"ms": round(t16, 3), "value": round(nvox / (t16 * 1e-3) / 1e6, 2),
                             "variant": best16, "autotune_ms": [round(v, 3) for v in tune16],
                             "max_abs_err_vs_fp64": float(np.abs(d16).max()),
                             "rms_err_vs_fp64": float(np.sqrt(np.mean(d16 * d16)))},
            "autotune_ms": [round(v, 3) for v in tune]}


def bench_adjoint(torch, gnlm, peak_tflops, steps=50, reps=20):
    """128^3 (ellipsoids, sigma 0.05, sr 3, pr 1): forward + adjoint per step (median
    of `reps` device-timed pairs), then used to fit h by gradient descent on the MSE
    to the clean phantom.  The forward's tile shape is autotuned on this volume first
    (the project's autotuner, as for the 2D and large-patch workloads)."""
    from gnlm import phantom
    noisy, clean = phantom.ellipsoid_phantom((128, 128, 128), n_ellipsoids=16, sigma=0.05, seed=4)
    fwd_variant, _ = gnlm.autotune(3, (128, 128, 128), SR, PR)
    x, c = torch.from_numpy(noisy).cuda(), torch.from_numpy(clean).cuda()
    n = x.numel()
    ws = torch.empty(gnlm.lib().nlm3d_adjoint_workspace_bytes(128, 128, 128, SR, PR),
                     dtype=torch.uint8, device="cuda")
    out, zs, gin = torch.empty_like(x), torch.empty_like(x), torch.empty_like(x)
    hg = torch.zeros(1, dtype=torch.float64, device="cuda")
    g = torch.randn(x.shape, device="cuda", generator=torch.Generator("cuda").manual_seed(0))
    stream = torch.cuda.current_stream()
    for _ in range(2):  # warm-up
        gnlm.nlm3d_forward(x, SR, PR, 0.05, out=out, zsum=zs, return_zsum=True)
        gnlm.nlm3d_adjoint(x, out, zs, g, SR, PR, 0.05, gin=gin, hgrad=hg, workspace=ws)
    torch.cuda.synchronize()
    fwd_t, adj_t = [], []
    for _ in range(reps):
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        ev[0].record(stream)
        gnlm.nlm3d_forward(x, SR, PR, 0.05, out=out, zsum=zs, return_zsum=True)
        ev[1].record(stream)
        gnlm.nlm3d_adjoint(x, out, zs, g, SR, PR, 0.05, gin=gin, hgrad=hg, workspace=ws)
        ev[2].record(stream)
        ev[2].synchronize()
        fwd_t.append(ev[0].elapsed_time(ev[1]))
        adj_t.append(ev[1].elapsed_time(ev[2]))
    fwd_ms, adj_ms = statistics.median(fwd_t), statistics.median(adj_t)
    # the kernels' gradients against FP64 central differences: dL/dv on 256 voxels
    # (corners, faces, random), dL/dh from two full FP64 forwards
    import oracle as O
    g64 = g.cpu().numpy().astype(np.float64)
    vox = O.fd_sample_voxels((128, 128, 128), 256, seed=6)
    fd = O.fd_voxel_grad(noisy, SR, PR, 0.05, g64, vox, eps=1e-5)
    gin_h = gin.cpu().numpy()
    fd_rel_v = float(np.abs(np.array([gin_h[i] for i in vox], np.float64) - fd).max()
                     / np.abs(fd).max())
    fdh = O.fd_h_grad(noisy, SR, PR, 0.05, g64, eps=1e-6)
    fd_rel_h = abs(float(hg.item()) - fdh) / abs(fdh)
    padded = (128 + 2 * (SR + PR)) ** 3
    adj_tflops = ADJ_FLOPS_PER_PAIR * OFFSETS * padded / (adj_ms * 1e-3) / 1e12
    # h fit: 50 steps of normalised gradient descent on MSE(out(h), clean)

    def fit_step(hh):
        gnlm.nlm3d_forward(x, SR, PR, hh, out=out, zsum=zs, return_zsum=True)
        d = out - c
        gnlm.nlm3d_adjoint(x, out, zs, d * (2.0 / n), SR, PR, hh, gin=gin, hgrad=hg, workspace=ws)
        return float((d * d).mean()), float(hg.item())  # host read of the step's loss

    for _ in range(3):  # untimed: first use of the loss and read-back ops in this process
        fit_step(0.02)
    h = 0.02
    mse0 = None
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    for _ in range(steps):
        mse, grad = fit_step(h)
        mse0 = mse if mse0 is None else mse0
        h = max(1e-3, h - 0.002 * (1.0 if grad > 0 else -1.0))
    t1.record(stream)
    t1.synchronize()
    return {"shape": [128, 128, 128], "search_radius": SR, "patch_radius": PR,
            "fwd_ms": round(fwd_ms, 3), "adjoint_ms": round(adj_ms, 3),
            "fwd_adjoint_ms_per_step": round(fwd_ms + adj_ms, 3), "timing": f"median of {reps}",
            "fwd_variant": fwd_variant,
            "grad_rel_err_vs_fp64_fd": {"dL_dv": fd_rel_v, "dL_dh": fd_rel_h,
                                        "sample": "256 voxels (8 corners, 6 faces, 242 random), "
                                                  "max |adjoint - FD| / max |FD|; h: relative"},
            "adjoint_tflops": round(adj_tflops, 3),
            "adjoint_frac_fp32_peak": round(adj_tflops / peak_tflops, 4) if peak_tflops else None,
            "adjoint_algorithmic": f"{ADJ_FLOPS_PER_PAIR} flops x {OFFSETS} offsets x {padded} "
                                   f"padded voxels (shared-memory bound: ncu in profiles/)",
            "h_fit": {"steps": steps, "h0": 0.02, "h": round(h, 4), "mse0": mse0, "mse": mse,
                      "ms_per_step_with_loss_readback": round(t0.elapsed_time(t1) / steps, 3)}}


def run_reference(args):
    rank, world, _ = env_rank()
    if rank != 0:
        return 0
    import oracle as O
    from gnlm import phantom
    threads = os.cpu_count() or 1
    O.set_threads(threads)
    vol, _ = phantom.ellipsoid_phantom(SHAPE, n_ellipsoids=N_ELLIPSOIDS, sigma=SIGMA, seed=SEED)
    Z, Y, X = SHAPE
    # 64 planes: the oracle parallelises over 4-plane z chunks, so this keeps every
    # host thread busy (16 chunks) while one step stays well under a second
    nz = 64
    slab = np.ascontiguousarray(vol[Z // 2 - nz // 2:Z // 2 + nz // 2])
    for _ in range(args.warmup):
        O.nlm3d(slab, SR, PR, H)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        O.nlm3d(slab, SR, PR, H)
    dt = (time.perf_counter() - t0) / args.steps
    value = nz * Y * X / dt / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(dt * 1e3, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD_NAME, "shape": list(SHAPE), "search_radius": SR,
                   "patch_radius": PR, "h": H, "sample": f"z-slab {nz}x{Y}x{X} per step"},
        "cpu_baseline": {"value": round(value, 3), "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"z-slab {nz}x{Y}x{X} of the 256^3 volume per step; the "
                                   "reference has no CPU NLM, this is the oracle's FP32 "
                                   "separable restatement of its arithmetic"},
        "e2e": {"value": round(value, 3), "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def run_gnlm(args):
    import torch
    import gnlm
    from gnlm import phantom

    rank, world, local = env_rank()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    gnlm.lib()

    vol, _ = phantom.ellipsoid_phantom(SHAPE, n_ellipsoids=N_ELLIPSOIDS, sigma=SIGMA, seed=SEED)
    Z, Y, X = SHAPE
    nvox = Z * Y * X
    # the project's autotuner: time every tile-shape variant on this shape, keep the fastest
    tuned32 = gnlm.autotune(3, SHAPE, SR, PR, fp16_storage=False)
    tuned16 = gnlm.autotune(3, SHAPE, SR, PR, fp16_storage=True)
    x = torch.from_numpy(vol).cuda()
    out = torch.empty_like(x)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()

    def timed_form(fp16, steps, warmup):
        ws = torch.empty(gnlm.nlm3d_workspace_bytes(SHAPE, SR, PR, fp16), dtype=torch.uint8,
                         device="cuda")
        for _ in range(warmup):
            gnlm.nlm3d_stage(x, SR, PR, H, ws, fp16_storage=fp16)
            gnlm.nlm3d_forward_staged(ws, SHAPE, SR, PR, H, out, fp16_storage=fp16)
        torch.cuda.synchronize()
        ev = []
        for _ in range(steps):
            flush.zero_()
            e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
            e0.record(stream)
            gnlm.nlm3d_stage(x, SR, PR, H, ws, fp16_storage=fp16)
            e1.record(stream)
            gnlm.nlm3d_forward_staged(ws, SHAPE, SR, PR, H, out, fp16_storage=fp16)
            e2.record(stream)
            ev.append((e0, e1, e2))
        torch.cuda.synchronize()
        step_ms = [a.elapsed_time(c) for a, b, c in ev]
        stage_ms = [a.elapsed_time(b) for a, b, c in ev]
        fused_ms = [b.elapsed_time(c) for a, b, c in ev]
        return step_ms, stage_ms, fused_ms, ws

    # warm-up + the timed FP32 region, bracketed by barrier + synchronize
    sampler = ClockSampler(local)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    sampler.start()
    step_ms, stage_ms, fused_ms, ws32 = timed_form(False, args.steps, args.warmup)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    if dist:
        dist.barrier()
    total_ms = max_over_ranks(dist, sum(step_ms), "cuda")
    ms_per_step = total_ms / args.steps
    value = replica_throughput(nvox, world, ms_per_step * 1e-3) / 1e6
    out32 = out.clone()

    # FP16-storage form (same loop)
    s16, st16, f16, _ = timed_form(True, max(3, args.steps // 2), max(3, args.warmup))
    out16 = out.clone()
    fp16_value = nvox / (statistics.mean(s16) * 1e-3) / 1e6

    # end-to-end through the host-buffer C-ABI call (pinned host memory)
    h_in = torch.from_numpy(vol).pin_memory()
    h_out = torch.empty(SHAPE, dtype=torch.float32).pin_memory()
    a_in, a_out = h_in.numpy(), h_out.numpy()
    for _ in range(max(1, args.warmup)):
        gnlm.nlm3d_forward_host(a_in, SR, PR, H, out=a_out)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        gnlm.nlm3d_forward_host(a_in, SR, PR, H, out=a_out)
    e2e_s = max_over_ranks(dist, (time.perf_counter() - t0) / args.steps, "cuda")
    e2e_value = replica_throughput(nvox, world, e2e_s) / 1e6
    assert np.array_equal(a_out, out32.cpu().numpy()), "host path disagrees with device path"
    # the FP16-storage form end to end from an FP16 host volume: half the host->device bytes
    h_in16 = torch.from_numpy(vol.astype(np.float16)).pin_memory()
    a_in16 = h_in16.numpy()
    h_out16 = torch.empty(SHAPE, dtype=torch.float32).pin_memory()
    a_out16 = h_out16.numpy()
    for _ in range(max(1, args.warmup)):
        gnlm.nlm3d_forward_host(a_in16, SR, PR, H, fp16_storage=True, out=a_out16)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        gnlm.nlm3d_forward_host(a_in16, SR, PR, H, fp16_storage=True, out=a_out16)
    e2e16_s = max_over_ranks(dist, (time.perf_counter() - t0) / args.steps, "cuda")
    e2e16_value = replica_throughput(nvox, world, e2e16_s) / 1e6

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return 0

    # accuracy of every voxel against the FP64 separable oracle
    import oracle as O
    ref64 = O.nlm3d(vol, SR, PR, H, dtype=np.float64)
    d32 = out32.cpu().numpy().astype(np.float64) - ref64
    err32, rms32 = float(np.abs(d32).max()), float(np.sqrt(np.mean(d32 * d32)))
    del d32
    d16 = out16.cpu().numpy().astype(np.float64) - ref64
    err16, rms16 = float(np.abs(d16).max()), float(np.sqrt(np.mean(d16 * d16)))
    # FP16 host input: the volume itself rounded to FP16 before the call
    d16h = a_out16.astype(np.float64) - ref64
    err16h, rms16h = float(np.abs(d16h).max()), float(np.sqrt(np.mean(d16h * d16h)))
    del d16, d16h, ref64

    peak = fp32_peak_tflops(torch)
    peak_x2 = fp32_peak_tflops(torch, packed=True)
    batched = bench_batched(torch, gnlm) if not args.skip_extra else None
    adjoint = bench_adjoint(torch, gnlm, peak) if not args.skip_extra else None
    image2d = bench_2d(torch, gnlm) if not args.skip_extra else None
    large = bench_large_patch(torch, gnlm) if not args.skip_extra else None
    fused_mean = statistics.mean(fused_ms)
    stage_mean = statistics.mean(stage_ms)
    hbm_peak, hbm_src = measured_hbm_peak()
    stage_gbs = staging_bytes(SHAPE, SR, PR) / (stage_mean * 1e-3) / 1e9
    achieved = FLOPS_PER_PAIR * OFFSETS * nvox / (fused_mean * 1e-3) / 1e12
    # FP32 variants 4-6 are the grouped-z kernel, 0-3 the one-offset-at-a-time kernel
    kname = "nlm3d_fwd_pz_kernel" if tuned32[0] >= 4 else "nlm3d_fwd_kernel"
    traffic = read_profile_traffic(kname)
    line = {
        "metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_per_step, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": WORKLOAD_NAME, "shape": list(SHAPE), "search_radius": SR,
                   "patch_radius": PR, "h": H, "phantom": f"{N_ELLIPSOIDS} ellipsoids, sigma {SIGMA}",
                   "l2": "256 MiB buffer written between timed steps"},
        "e2e": {"value": round(e2e_value, 2), "unit": UNIT,
                "h2d_bytes_per_step": int(vol.nbytes), "d2h_bytes_per_step": int(vol.nbytes)},
        "gpu_launches": 2 * args.steps,
        "roofline": {"bound": "fp32", "achieved": round(achieved, 3),
                     "peak": round(peak, 3), "unit": "TFLOP/s",
                     "frac": round(achieved / peak, 4) if peak else None,
                     "traffic": traffic,
                     "traffic_source": TRAFFIC_SOURCE,
                     "kernel": f"{kname}<3,1> (FP32 variant {tuned32[0]})",
                     "peak_source": "FFMA probe kernel measured in this run (FP32 pipe; "
                                    "MEASURED_PEAKS.json has HBM and bf16 only)",
                     "algorithmic": f"{FLOPS_PER_PAIR} flops x {OFFSETS} offsets x {nvox} voxels"},
        "staging_roofline": {"kernel": "stage_kernel<float,float> (REFLECT_101 pad + pre-scale)",
                             "bound": "hbm", "achieved": round(stage_gbs, 1),
                             "peak": round(hbm_peak, 1), "unit": "GB/s",
                             "frac": round(stage_gbs / hbm_peak, 4), "peak_source": hbm_src,
                             "traffic": read_profile_traffic("stage_kernel"),
                             "traffic_source": TRAFFIC_SOURCE,
                             "algorithmic": "input read once + padded volume written once "
                                            f"({staging_bytes(SHAPE, SR, PR)} bytes)"},
        "autotune": {"fp32": {"chosen": tuned32[0], "ms": [round(t, 4) for t in tuned32[1]]},
                     "fp16_storage": {"chosen": tuned16[0], "ms": [round(t, 4) for t in tuned16[1]]}},
        "fp32x2_probe_tflops": round(peak_x2, 3),
        "kernels_ms": {"stage": round(stage_mean, 4),
                       "fused_fp32": round(fused_mean, 4),
                       "fused_fp16": round(statistics.mean(f16), 4)},
        "forms": {"fp32": {"value": round(value, 2), "max_abs_err_vs_fp64": err32,
                           "rms_err_vs_fp64": rms32},
                  "fp16_storage": {"value": round(fp16_value, 2), "max_abs_err_vs_fp64": err16,
                                   "rms_err_vs_fp64": rms16,
                                   "e2e": {"value": round(e2e16_value, 2), "unit": UNIT,
                                           "h2d_bytes_per_step": int(a_in16.nbytes),
                                           "d2h_bytes_per_step": int(a_out16.nbytes),
                                           "input": "FP16 host volume (the FP32 phantom rounded)",
                                           "max_abs_err_vs_fp64": err16h,
                                           "rms_err_vs_fp64": rms16h},
                                   "faster_than_fp32": {
                                       "device_resident": fp16_value > value,
                                       "e2e": e2e16_value > e2e_value}},
                  "error_sample": "every voxel of the 256^3 output vs the FP64 separable oracle",
                  "batched": batched},
        "adjoint": adjoint,
        "nlm2d": image2d,
        "large_patch": large,
        "clocks": clocks,
    }
    if world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(SHAPE)
    print(json.dumps(line))
    if dist:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gnlm", "reference"], default="gnlm")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--skip-extra", action="store_true",
                    help="skip the batched and adjoint workloads (profiling runs)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_gnlm(args)


if __name__ == "__main__":
    sys.exit(main())
