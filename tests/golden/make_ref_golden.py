"""Generates golden vectors by running the reference's own generic NLM kernels.

Run on a GB300 after ``bash oracle/ref_build.sh`` has built the cubins (from the
reference sources) into oracle/_ref/:

    python tests/golden/make_ref_golden.py <out_dir>

Each case launches the reference kernel ``shuffle_without_optimization`` once,
with the reference launcher's geometry and scratch size (3DNLM/main.cu:7611-7634,
2D NLM/11x11/main.cu:476-494), on a pre-padded unsigned char input built the way
the reference driver builds it (REFLECT_101 padding, 3DNLM/nlm.cpp:36-61), and
saves input, configuration and output as .npz.  Before any launch, the largest
index each kernel reads is computed from its index formulas on the CPU and
checked against the buffer sizes.
"""
import ctypes
import os
import sys

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(REPO, "3d-gnlm_gb300"))
sys.path.insert(0, os.path.join(REPO, "oracle"))

REF_DIR = os.path.join(REPO, "oracle", "_ref")


def _mangle(name, params):
    return f"_Z{len(name)}{name}{params}"


# shuffle_without_optimization(unsigned char*, float*, float*)          (3DNLM/main.cu:28)
K3D = _mangle("shuffle_without_optimization", "PhPfS0_")
# shuffle_without_optimization(uchar*, float*, float*, int x 6)         (2D NLM/11x11/main.cu:383)
K2D = _mangle("shuffle_without_optimization", "PhPfS0_iiiiii")


class Driver:
    def __init__(self):
        import torch
        torch.cuda.init()
        torch.zeros(1, device="cuda")  # make the primary context current
        self.torch = torch
        self.cu = ctypes.CDLL("libcuda.so.1")

    def check(self, rc, what):
        if rc != 0:
            raise RuntimeError(f"{what} failed: CUresult {rc}")

    def function(self, cubin_path, name):
        data = open(cubin_path, "rb").read()
        mod = ctypes.c_void_p()
        self.check(self.cu.cuModuleLoadData(ctypes.byref(mod), ctypes.c_char_p(data)), "cuModuleLoadData")
        fn = ctypes.c_void_p()
        self.check(self.cu.cuModuleGetFunction(ctypes.byref(fn), mod, name.encode()),
                   f"cuModuleGetFunction({name})")
        return fn

    def launch(self, fn, grid, block, args):
        """args: ctypes scalars in kernel-parameter order (c_void_p pointers, c_int ints)."""
        ptrs = (ctypes.c_void_p * len(args))()
        for i, a in enumerate(args):
            ptrs[i] = ctypes.cast(ctypes.byref(a), ctypes.c_void_p)
        self.check(self.cu.cuLaunchKernel(fn, grid[0], grid[1], grid[2], block[0], block[1],
                                          block[2], 0, None, ptrs, None), "cuLaunchKernel")
        self.check(self.cu.cuCtxSynchronize(), "cuCtxSynchronize")


def _top(exprs, W, H=1):
    """Largest linear index over read expressions given as (col, row, plane) maxima."""
    return max(c + r * W + p * W * H for c, r, p in exprs)


def max_read_3d(SS, NS, X, Y, depth):
    """Largest element index 3DNLM/main.cu:28-238 reads, from its index expressions."""
    G = (X + 32 - NS) // (33 - NS)
    W, H = X + SS + NS - 2, Y + SS + NS - 2
    m, n = (SS - 1) // 2, (NS - 1) // 2
    cpb, cpz = Y // 16, depth // 4
    cpt = cpb // 4
    ix = (G - 1) * (33 - NS) + 31           # largest x of any lane
    Yb = 15 * cpb + 3 * cpt                 # largest row base iy*cpb + wy*cpt
    Zb = (cpz - 2) + 3 * cpz                # largest plane base itra_z + iz*cpz
    ty = cpt - 1                            # largest itra_y
    exprs = [
        (ix + m, NS - 1 + m + Yb, NS + m + Zb),                      # reference patch, :59
        (ix + SS - 1, NS - 1 + SS - 1 + Yb, NS + SS - 1 + Zb),       # candidate patch, :59
        (ix + n + SS - 1, SS - 1 + n + Yb, SS + n + Zb),             # candidate centre, :111,118
        (ix + m, ty + NS - 1 + m + Yb, NS + m + Zb),                 # slide, reference, :146
        (ix + SS - 1, ty + NS - 1 + SS - 1 + Yb, NS + SS - 1 + Zb),  # slide, candidate, :147
        (ix + n + SS - 1, ty + SS - 1 + n + Yb, SS + n + Zb),        # slide, centre, :217,223
    ]
    return _top(exprs, W, H), W * H * (depth + SS + NS - 2), (W, H, G)


def max_read_2d(sr, nb, X, Y):
    """Largest element index 2D NLM/11x11/main.cu:383-468 reads (row stride W)."""
    G = (X + 32 - nb) // (33 - nb)
    W = X + sr + nb - 2
    m, n = (sr - 1) // 2, (nb - 1) // 2
    col = Y // 16
    ct = col // 4
    ix = (G - 1) * (33 - nb) + 31
    Yb = 15 * col + 3 * ct
    ty = ct - 1
    exprs = [
        (ix + m, nb - 1 + m + Yb, 0),              # reference patch, :404
        (ix + sr - 1, nb - 1 + sr - 1 + Yb, 0),    # candidate patch, :404
        (ix + n + sr - 1, sr - 1 + n + Yb, 0),     # candidate centre, :418
        (ix + m, ty + 10 + m + Yb, 0),             # slide, reference, :446
        (ix + sr - 1, ty + 10 + sr - 1 + Yb, 0),   # slide, candidate, :446
        (ix + n + sr - 1, sr - 1 + n + ty + Yb, 0),  # slide, centre, :460
    ]
    return _top(exprs, W), W * W, (W, G)


def run3d(drv, SS, NS, X, Y, depth, padded):
    torch = drv.torch
    top, size, (W, H, G) = max_read_3d(SS, NS, X, Y, depth)
    assert padded.shape == (depth + SS + NS - 2, H, W) and padded.size == size
    assert top < size, f"reference kernel would read index {top} >= {size}"
    fn = drv.function(os.path.join(REF_DIR, f"ref3d_ss{SS}_ns{NS}_x{X}_y{Y}_d{depth}.cubin"), K3D)
    d_in = torch.from_numpy(np.ascontiguousarray(padded)).cuda()
    d_out = torch.zeros(depth * Y * X, dtype=torch.float32, device="cuda")
    n_w = G * 32 * 64 * 4 * SS ** 3  # 3DNLM/main.cu:7618
    d_w = torch.zeros(n_w, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    P = ctypes.c_void_p
    drv.launch(fn, (G, 16, 4), (32, 4, 1), [P(d_in.data_ptr()), P(d_out.data_ptr()), P(d_w.data_ptr())])
    return d_out.cpu().numpy().reshape(depth, Y, X)


def run2d(drv, sr, nb, X, padded):
    torch = drv.torch
    top, size, (W, G) = max_read_2d(sr, nb, X, X)
    assert padded.shape == (W, W) and top < size, (top, size)
    fn = drv.function(os.path.join(REF_DIR, "ref2d.cubin"), K2D)
    d_in = torch.from_numpy(np.ascontiguousarray(padded)).cuda()
    d_out = torch.zeros(X * X, dtype=torch.float32, device="cuda")
    d_w = torch.zeros(G * 32 * 64 * sr * sr, dtype=torch.float32, device="cuda")  # main.cu:480
    torch.cuda.synchronize()
    P, I = ctypes.c_void_p, ctypes.c_int
    drv.launch(fn, (G, 16, 1), (32, 4, 1),
               [P(d_in.data_ptr()), P(d_out.data_ptr()), P(d_w.data_ptr()), I(W), I(W), I(sr),
                I(nb), I(X), I(X)])
    return d_out.cpu().numpy().reshape(X, X)


def inputs3d(SS, NS, X, Y, depth, kind, seed):
    import oracle as O
    from gnlm import phantom
    pad = (SS + NS - 2) // 2
    if kind == "zconst":  # one slice, replicated in z as 3DNLM/nlm.cpp:55-61 does
        im, _ = phantom.disc_rect_phantom((Y, X), n_shapes=12, sigma=0.03, seed=seed)
        sl = np.clip(im * 255, 0, 255).astype(np.uint8)
        p2 = O.pad_reflect101(sl, pad)
        return np.ascontiguousarray(np.broadcast_to(p2, (depth + 2 * pad,) + p2.shape))
    vol, _ = phantom.ellipsoid_phantom((depth, Y, X), n_ellipsoids=12, sigma=0.03, seed=seed,
                                       radii=(3.0, 30.0))
    vol = np.clip(vol * 255, 0, 255).astype(np.uint8)
    return np.ascontiguousarray(O.pad_reflect101(vol, pad))


def main(out_dir):
    os.makedirs(out_dir, exist_ok=True)
    drv = Driver()
    cases = [(7, 3, 120, 16, [("zconst", 31), ("phantom", 32)]),
             (7, 5, 112, 16, [("zconst", 31), ("phantom", 32)]),
             # large patches (the reference's NS 13..17 family), z-constant inputs
             (11, 13, 120, 8, [("zconst", 34)]),
             (13, 17, 128, 8, [("zconst", 35)])]
    for (SS, NS, X, depth, kinds) in cases:
        Y = 128
        for kind, seed in kinds:
            padded = inputs3d(SS, NS, X, Y, depth, kind, seed)
            out = run3d(drv, SS, NS, X, Y, depth, padded)
            path = os.path.join(out_dir, f"ref3d_ss{SS}_ns{NS}_{kind}.npz")
            np.savez_compressed(path, padded=padded, out=out,
                                cfg=np.array([SS, NS, X, Y, depth, 10], np.int32),
                                kernel=np.array(K3D), kind=np.array(kind))
            print(path, out.shape, float(out.min()), float(out.max()))
    # 2D: search 7, patch 11 (the patch width the reference's 2D kernels support)
    from gnlm import phantom
    import oracle as O
    X, sr, nb = 704, 7, 11
    im, _ = phantom.disc_rect_phantom((X, X), n_shapes=24, sigma=0.03, seed=33)
    img = np.clip(im * 255, 0, 255).astype(np.uint8)
    padded = np.ascontiguousarray(O.pad_reflect101(img, (sr + nb - 2) // 2))
    out = run2d(drv, sr, nb, X, padded)
    rows = np.r_[0:48, 328:376, 656:704]  # kept rows: both borders and the middle
    path = os.path.join(out_dir, "ref2d_sr7_nb11.npz")
    np.savez_compressed(path, image=img, out_rows=out[rows], rows=rows,
                        cfg=np.array([sr, nb, X, X, 10], np.int32), kernel=np.array(K2D))
    print(path, out.shape, float(out.min()), float(out.max()))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.join(REPO, "tests", "golden"))
