"""The reference's own CUDA kernels timed on this GPU next to this repo's kernels.

The reference kernels are compiled from the reference sources by
oracle/ref_build.sh (git-ignored cubins in oracle/_ref/) and launched with the
reference launcher's grids and scratch sizes (3DNLM/main.cu:7611-7667,
2D NLM/11x11/main.cu:476-525) on the same pre-padded unsigned char inputs that
this repo's kernels take with NLM_FLAG_PREPADDED.  At these sizes the reference
kernels read a few elements past their row ends, so their input buffers carry
slack beyond the largest index any of them reads (computed below).  The test is
skipped where the cubins were not built.  Each kernel is timed with CUDA events
(best of 3 after a warm-up); the results are printed and the repo's kernel must
be the faster one.
"""
import ctypes
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

pytestmark = pytest.mark.gpu

import make_ref_golden as R  # noqa: E402

CUBIN3D = os.path.join(R.REF_DIR, "ref3d_ss7_ns3_x256_y256_d256.cubin")
CUBIN2D = os.path.join(R.REF_DIR, "ref2d.cubin")


def _time(torch, fn, reps=3):
    fn()
    torch.cuda.synchronize()
    best = 1e30
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1))
    return best


@pytest.mark.skipif(not os.path.exists(CUBIN3D), reason="reference cubins not built here")
def test_reference_3d_kernel_vs_repo_kernel_256cubed(torch_cuda, gnlm_lib):
    torch = torch_cuda
    SS, NS, X, Y, D = 7, 3, 256, 256, 256
    top, size, (W, H, G) = R.max_read_3d(SS, NS, X, Y, D)
    padded = R.inputs3d(SS, NS, X, Y, D, "phantom", seed=41)
    assert padded.size == size
    buf = torch.zeros(size + max(0, top + 1 - size) + 4096, dtype=torch.uint8, device="cuda")
    buf[:size].copy_(torch.from_numpy(padded.ravel()))
    out = torch.zeros(D * Y * X, dtype=torch.float32, device="cuda")
    weight = torch.zeros(G * 32 * 64 * 4 * SS ** 3, dtype=torch.float32, device="cuda")
    drv = R.Driver()
    fn = drv.function(CUBIN3D, R.K3D)
    P = ctypes.c_void_p
    args = [P(buf.data_ptr()), P(out.data_ptr()), P(weight.data_ptr())]

    def ref():
        drv.launch(fn, (G, 16, 4), (32, 4, 1), args)

    x = buf[:size].reshape(padded.shape)
    mine_out = torch.empty((D, Y, X), dtype=torch.float32, device="cuda")

    def mine():
        gnlm_lib.nlm3d_forward(x, 3, 1, 10.0, prepadded=True, shape=(D, Y, X), out=mine_out)

    t_ref, t_mine = _time(torch, ref), _time(torch, mine)
    print(f"\n3D 256^3 SS7 NS3: reference generic kernel {t_ref:.3f} ms "
          f"({X * Y * D / t_ref / 1e3:.1f} Mvoxel/s), this repo {t_mine:.3f} ms "
          f"({X * Y * D / t_mine / 1e3:.1f} Mvoxel/s), speed-up {t_ref / t_mine:.2f}x")
    assert t_mine < t_ref


@pytest.mark.skipif(not os.path.exists(CUBIN2D), reason="reference cubins not built here")
def test_reference_2d_kernels_vs_repo_kernel_2048(torch_cuda, gnlm_lib):
    """Search 21 / patch 11 at 2048^2: the configuration of the reference's only
    published numbers (2D NLM/11x11/resource-11.txt:663-807)."""
    torch = torch_cuda
    sr, nb, X = 21, 11, 2048
    W = X + sr + nb - 2
    m, n = (sr - 1) // 2, (nb - 1) // 2
    from gnlm import phantom
    import oracle as O
    im, _ = phantom.disc_rect_phantom((X, X), n_shapes=32, sigma=0.03, seed=42)
    img = np.clip(im * 255, 0, 255).astype(np.uint8)
    padded = np.ascontiguousarray(O.pad_reflect101(img, (sr + nb - 2) // 2))
    grids = {"generic": ((X + 32 - nb) // (33 - nb), R.K2D),
             "shift_1": ((X + 30) // 31, R._mangle("NLmeansOnGPU_shift_1", "PhPfS0_iiiiii")),
             "shift_2": ((X + 29) // 30, R._mangle("NLmeansOnGPU_shift_2", "PhPfS0_iiiiii")),
             "shift_3": ((X + 28) // 29, R._mangle("NLmeansOnGPU_shift_3", "PhPfS0_iiiiii"))}
    # largest read of any variant: column <= ix + sr - 1 + 10, row <= W - 1
    ix_max = max((g - 1) * (32 - s) + 31 for (g, _), s in zip(grids.values(), (nb - 1, 1, 2, 3)))
    top = ix_max + sr + 10 + (W - 1) * W
    buf = torch.zeros(max(W * W, top + 1) + 4096, dtype=torch.uint8, device="cuda")
    buf[:W * W].copy_(torch.from_numpy(padded.ravel()))
    out = torch.zeros(X * X, dtype=torch.float32, device="cuda")
    G0 = grids["generic"][0]
    weight = torch.zeros(G0 * 32 * 64 * sr * sr, dtype=torch.float32, device="cuda")  # main.cu:480
    drv = R.Driver()
    P, I = ctypes.c_void_p, ctypes.c_int
    args = [P(buf.data_ptr()), P(out.data_ptr()), P(weight.data_ptr()), I(W), I(W), I(sr), I(nb),
            I(X), I(X)]
    times = {}
    for name, (g, sym) in grids.items():
        fn = drv.function(CUBIN2D, sym)
        times[name] = _time(torch, lambda: drv.launch(fn, (g, 16, 1), (32, 4, 1), args))
    x = buf[:W * W].reshape(W, W)
    mine_out = torch.empty((X, X), dtype=torch.float32, device="cuda")

    def mine():
        gnlm_lib.nlm2d_forward(x, m, n, 10.0, prepadded=True, shape=(X, X), out=mine_out)

    t_mine = _time(torch, mine)
    best = min(times.values())
    print("\n2D 2048^2 search 21 patch 11: reference " +
          ", ".join(f"{k} {v:.3f} ms" for k, v in times.items()) +
          f"; this repo {t_mine:.3f} ms ({X * X / t_mine / 1e3:.1f} Mpixel/s), "
          f"speed-up vs fastest reference variant {best / t_mine:.2f}x")
    assert t_mine < best


def _ref3d_variants(SS, NS, X):
    """(name, grid.x, mangled symbol) of the four kernels the reference's launcher
    runs (3DNLM/main.cu:7626-7666): the generic kernel and shift_1..3."""
    gen = ("generic", (X + 32 - NS) // (33 - NS), R.K3D)
    shifts = [(f"shift_{s}", (X + 31 - s) // (32 - s), R._mangle(f"NLmeansOnGPU_shift_{s}", "PhPfS0_"))
              for s in (1, 2, 3)]
    return [gen] + shifts


def _ref3d_slack_top(SS, NS, X, Y, depth):
    """Upper bound of the element index any of the four kernels reads.  Their row
    and plane indices stay inside the padded volume at these sizes; the x index of
    a lane runs at most (SS - 1) + (NS - 1) past its lane column ix (3DNLM/main.cu
    :59,111 and the shift kernels' `k + ix + c` terms with c <= NS - 1, e.g.
    :6254-7599 for NS = 17), and ix <= (grid.x - 1) * step + 31."""
    W, H, Dp = X + SS + NS - 2, Y + SS + NS - 2, depth + SS + NS - 2
    steps = {"generic": 33 - NS, "shift_1": 31, "shift_2": 30, "shift_3": 29}
    ix_max = max((g - 1) * steps[name] + 31 for name, g, _ in _ref3d_variants(SS, NS, X))
    return (Dp * H - 1) * W + ix_max + SS + NS


@pytest.mark.parametrize("SS,NS", [(11, 13), (11, 15), (11, 17), (13, 13), (13, 15), (13, 17)])
def test_reference_large_patch_kernels_vs_repo_kernel(torch_cuda, gnlm_lib, SS, NS):
    """The reference's sweep sizes (3DNLM/run.sh:25-34) at depth 16: its four kernels
    against this repo's large-patch kernel on the same pre-padded uchar volume."""
    torch = torch_cuda
    X = Y = 512
    D = 16
    cubin = os.path.join(R.REF_DIR, f"ref3d_ss{SS}_ns{NS}_x{X}_y{Y}_d{D}.cubin")
    if not os.path.exists(cubin):
        pytest.skip("reference cubins not built here")
    W, H, Dp = X + SS + NS - 2, Y + SS + NS - 2, D + SS + NS - 2
    size = W * H * Dp
    top = _ref3d_slack_top(SS, NS, X, Y, D)
    from gnlm import phantom
    import oracle as O
    img = np.clip(phantom.disc_rect_phantom((Y, X), n_shapes=32, sigma=0.03, seed=NS)[0] * 255,
                  0, 255).astype(np.uint8)
    p2 = O.pad_reflect101(img, (SS + NS - 2) // 2)
    padded = np.ascontiguousarray(np.broadcast_to(p2, (Dp, H, W)))
    buf = torch.zeros(max(size, top + 1) + 4096, dtype=torch.uint8, device="cuda")
    buf[:size].copy_(torch.from_numpy(padded.ravel()))
    out = torch.zeros(D * Y * X, dtype=torch.float32, device="cuda")
    variants = _ref3d_variants(SS, NS, X)
    n_w = max(g for _, g, _ in variants) * 32 * 64 * 4 * SS ** 3  # 3DNLM/main.cu:7618
    weight = torch.zeros(n_w, dtype=torch.float32, device="cuda")
    drv = R.Driver()
    P = ctypes.c_void_p
    args = [P(buf.data_ptr()), P(out.data_ptr()), P(weight.data_ptr())]
    times = {}
    for name, g, sym in variants:
        fn = drv.function(cubin, sym)
        times[name] = _time(torch, lambda: drv.launch(fn, (g, 16, 4), (32, 4, 1), args), reps=1)
    x = buf[:size].reshape(Dp, H, W)
    mine_out = torch.empty((D, Y, X), dtype=torch.float32, device="cuda")
    sr, pr = (SS - 1) // 2, (NS - 1) // 2

    def mine():
        gnlm_lib.nlm3d_forward(x, sr, pr, 10.0, prepadded=True, shape=(D, Y, X), out=mine_out)

    t_mine = _time(torch, mine)
    best = min(times.values())
    print(f"\n3D 512x512x{D} SS{SS} NS{NS}: reference " +
          ", ".join(f"{k} {v:.1f} ms" for k, v in times.items()) +
          f"; this repo {t_mine:.2f} ms ({X * Y * D / t_mine / 1e3:.1f} Mvoxel/s), "
          f"speed-up vs fastest reference kernel {best / t_mine:.1f}x")
    assert t_mine < best
