"""Runs every kernel family on small, ragged shapes and saves the outputs.

Used by tests/test_gpu_failures.py twice: once in-process with the normal build and
once in a child process with GNLM_LIB pointing at the NLM_BOUNDS_CHECK build; the
two must agree bit for bit and the checked build must leave the device error word
clean.  Usage: python checked_cases.py OUT.npz (prints the device status as JSON).
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
for p in (os.path.join(REPO, "3d-gnlm_gb300"), os.path.join(REPO, "oracle"), REPO):
    if p not in sys.path:
        sys.path.insert(0, p)


def run_cases(gnlm, torch):
    from gnlm import phantom
    res = {}
    v3, _ = phantom.ellipsoid_phantom((13, 37, 67), n_ellipsoids=5, sigma=0.05, seed=3,
                                      radii=(2.0, 8.0))
    x3 = torch.from_numpy(v3).cuda()
    for fp16 in (False, True):
        for var in range(gnlm.variant_count(3, fp16)):
            gnlm.set_variant(3, 3, 1, var, fp16)
            res[f"3d_s3p1_f{int(fp16)}_v{var}"] = gnlm.nlm3d_forward(x3, 3, 1, 0.05,
                                                                     fp16_storage=fp16).cpu().numpy()
        gnlm.set_variant(3, 3, 1, -1, fp16)
    for var in (0, 5):
        gnlm.set_variant(3, 5, 2, var)
        res[f"3d_s5p2_v{var}"] = gnlm.nlm3d_forward(x3, 5, 2, 0.05).cpu().numpy()
    gnlm.set_variant(3, 5, 2, -1)
    vl, _ = phantom.ellipsoid_phantom((19, 23, 41), n_ellipsoids=5, sigma=0.05, seed=4,
                                      radii=(2.0, 9.0))
    xl = torch.from_numpy(vl).cuda()
    for sr, pr in [(6, 8), (2, 4), (6, 1)]:
        res[f"lp_{sr}_{pr}"] = gnlm.nlm3d_forward(xl, sr, pr, 0.05).cpu().numpy()
    for sr, pr in [(6, 8), (1, 3)]:
        res[f"lp16_{sr}_{pr}"] = gnlm.nlm3d_forward(xl, sr, pr, 0.05,
                                                    fp16_storage=True).cpu().numpy()
    # every compiled 3D pair in both storage forms, on a shape with a second tile on every
    # tiled axis of every kernel (50 rows: two 48-row large-patch tiles, one 64-row tile)
    vp, _ = phantom.ellipsoid_phantom((9, 50, 37), n_ellipsoids=4, sigma=0.05, seed=77,
                                      radii=(1.5, 8.0))
    xp = torch.from_numpy(vp).cuda()
    for sr in range(1, 7):
        for pr in range(1, 9):
            for fp16 in (False, True):
                res[f"pair_{sr}_{pr}_f{int(fp16)}"] = gnlm.nlm3d_forward(
                    xp, sr, pr, 0.05, fp16_storage=fp16).cpu().numpy()
    im, _ = phantom.disc_rect_phantom((61, 90), n_shapes=6, sigma=0.08, seed=5)
    x2 = torch.from_numpy(im).cuda()
    for var in range(gnlm.variant_count(2, False)):
        gnlm.set_variant(2, 5, 2, var)
        res[f"2d_s5p2_v{var}"] = gnlm.nlm2d_forward(x2, 5, 2, 0.08).cpu().numpy()
    gnlm.set_variant(2, 5, 2, -1)
    for sr, pr in [(1, 1), (3, 1), (5, 1), (3, 2), (7, 2), (3, 5), (7, 5), (10, 5)]:
        for fp16 in (False, True):
            res[f"2d_s{sr}p{pr}_f{int(fp16)}"] = gnlm.nlm2d_forward(
                x2, sr, pr, 0.08, fp16_storage=fp16).cpu().numpy()
    va, _ = phantom.ellipsoid_phantom((10, 12, 40), n_ellipsoids=3, sigma=0.05, seed=6,
                                      radii=(1.5, 5.0))
    xa = torch.from_numpy(va).cuda()
    g = torch.from_numpy(np.random.default_rng(7).standard_normal(va.shape).astype(np.float32)).cuda()
    for sr, pr in [(3, 1), (3, 2), (1, 1), (4, 1), (5, 1)]:
        out, zs = gnlm.nlm3d_forward(xa, sr, pr, 0.06, return_zsum=True)
        gin, hg = gnlm.nlm3d_adjoint(xa, out, zs, g, sr, pr, 0.06)
        res[f"adj_{sr}_{pr}"] = gin.cpu().numpy()
        res[f"adjh_{sr}_{pr}"] = np.array([float(hg.item())])
    vols = [(xa, 3, 1, 0.05), (x3, 5, 1, 0.05)]
    plan = gnlm.BatchPlan(vols)
    plan.run()
    torch.cuda.synchronize()
    for k, o in enumerate(plan.outputs):
        res[f"batch_{k}"] = o.cpu().numpy()
    return res


if __name__ == "__main__":
    import torch

    import gnlm
    out = run_cases(gnlm, torch)
    np.savez(sys.argv[1], **out)
    rc, flags = gnlm.device_status()
    print(json.dumps({"lib": gnlm.LIB_PATH, "rc": rc, "flags": flags}))
