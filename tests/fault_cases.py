"""Drives every bounded tile-copy wait to its limit, without faulting the GPU.

Run as a child process with GNLM_LIB pointing at the NLM_BOUNDS_CHECK build
(lib/libgnlm_checked.so), whose kernels read a fault-injection control word: with
nlm_test_set_fault(0x1) the CTA of tile (0, 0, 0) of each launch arms its barrier but
never issues its tile copy, so its wait runs out after a short poll limit, the kernel
sets 0x1 (tile copy timed out) in the device error word and returns.  No copy is in
flight when it does.  For each kernel family the case records the call's status, the
error word, then turns injection off and checks that the next call is clean and
correct.  Prints one JSON line.  Used by tests/test_gpu_failures.py.
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


def main():
    import torch

    import gnlm
    import oracle as O
    from gnlm import phantom

    L = gnlm.lib()
    v, _ = phantom.ellipsoid_phantom((12, 20, 45), n_ellipsoids=3, sigma=0.05, seed=8,
                                     radii=(2.0, 6.0))
    x = torch.from_numpy(v).cuda()
    im, _ = phantom.disc_rect_phantom((40, 70), n_shapes=5, sigma=0.08, seed=9)
    x2 = torch.from_numpy(im).cuda()
    g = torch.from_numpy(np.random.default_rng(3).standard_normal(v.shape).astype(np.float32)).cuda()
    out0, zs0 = gnlm.nlm3d_forward(x, 3, 1, 0.05, return_zsum=True)
    torch.cuda.synchronize()

    cases = {
        "3d_fp32": lambda: gnlm.nlm3d_forward(x, 3, 1, 0.05),
        "3d_fp16_storage": lambda: gnlm.nlm3d_forward(x, 3, 1, 0.05, fp16_storage=True),
        "2d": lambda: gnlm.nlm2d_forward(x2, 5, 2, 0.08),
        "batched": lambda: gnlm.nlm3d_forward_batched([(x, 3, 1, 0.05), (x, 2, 1, 0.06)]),
        "adjoint": lambda: gnlm.nlm3d_adjoint(x, out0, zs0, g, 3, 1, 0.05),
        "large_patch": lambda: gnlm.nlm3d_forward(x, 4, 3, 0.05),
    }
    res = {"lib": gnlm.LIB_PATH, "cases": {}}
    for name, call in cases.items():
        r = {"set": L.nlm_test_set_fault(1)}
        try:
            call()
            r["call"] = 0
        except gnlm.NLMError as e:
            r["call"] = e.code
        r["status"], r["flags"] = gnlm.device_status()
        r["unset"] = L.nlm_test_set_fault(0)
        call()
        r["after_status"], r["after_flags"] = gnlm.device_status()
        res["cases"][name] = r
    # clean and correct once injection is off
    got = gnlm.nlm3d_forward(x, 3, 1, 0.05).cpu().numpy()
    res["after_err_vs_fp64"] = float(np.abs(got - O.nlm3d(v, 3, 1, 0.05, dtype=np.float64)).max())
    res["final_status"] = list(gnlm.device_status())
    print(json.dumps(res))


if __name__ == "__main__":
    main()
