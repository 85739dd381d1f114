"""GPU test of nlm3d_forward_noalloc, the allocation-free 3D entry point.

That entry point exists for callers that may not allocate device memory while
they run (plug-ins inside an application that owns every GPU allocation, and
fixed-budget real-time pipelines), so its staging scratch is a fixed array
inside libgnlm.so instead of a cudaMalloc'd or caller-provided workspace.  Here
it is called through the C ABI and must reproduce nlm3d_forward, on two calls
in a row with different inputs (the shared array keeps the previous call's
contents, which must not leak into the next result).  This file is collected
last so a run that stops at the first failure has run every other test first.
"""
import ctypes

import numpy as np
import pytest

from gnlm import phantom

pytestmark = pytest.mark.gpu

TOL_F32 = 1e-5


def _call_noalloc(gnlm, torch, x, sr, pr, h, flags=0, zsum=False):
    Z, Y, X = x.shape
    out = torch.empty((Z, Y, X), dtype=torch.float32, device="cuda")
    zs = torch.empty_like(out) if zsum else None
    rc = gnlm.lib().nlm3d_forward_noalloc(
        ctypes.c_void_p(x.data_ptr()), gnlm._dtype_code(x), X, Y, Z, sr, pr, float(h),
        ctypes.c_void_p(out.data_ptr()), None if zs is None else ctypes.c_void_p(zs.data_ptr()),
        flags, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    return rc, out, zs


def test_noalloc_matches_forward_on_two_calls(torch_cuda, gnlm_lib):
    torch = torch_cuda
    cases = [((40, 50, 64), 3, 1, 0.05, 0), ((96, 64, 33), 2, 1, 0.08, 0),
             ((128, 128, 128), 3, 1, 0.05, gnlm_lib.NLM_FLAG_FP16_STORAGE)]
    for k, (shape, sr, pr, h, flags) in enumerate(cases):
        v, _ = phantom.ellipsoid_phantom(shape, n_ellipsoids=8, sigma=h, seed=100 + k)
        x = torch.from_numpy(v).cuda()
        ref, ref_z = gnlm_lib.nlm3d_forward(x, sr, pr, h, return_zsum=True,
                                            fp16_storage=bool(flags))
        rc, out, zs = _call_noalloc(gnlm_lib, torch, x, sr, pr, h, flags, zsum=True)
        assert rc == gnlm_lib.NLM_OK, gnlm_lib.last_error()
        torch.cuda.synchronize()
        assert float((out - ref).abs().max()) <= TOL_F32
        assert float(((zs - ref_z).abs() / ref_z).max()) <= TOL_F32


def test_noalloc_rejects_volumes_beyond_its_scratch(torch_cuda, gnlm_lib):
    torch = torch_cuda
    x = torch.zeros((160, 160, 160), dtype=torch.float32, device="cuda")
    rc, _, _ = _call_noalloc(gnlm_lib, torch, x, 3, 1, 0.05)
    assert rc == gnlm_lib.NLM_ERR_WORKSPACE
    assert "at most" in gnlm_lib.last_error()
    # the largest FP32 volume that fits (sr 3, pr 1) still runs
    v, _ = phantom.ellipsoid_phantom((152, 152, 152), n_ellipsoids=8, sigma=0.05, seed=7)
    x = torch.from_numpy(v).cuda()
    rc, out, _ = _call_noalloc(gnlm_lib, torch, x, 3, 1, 0.05)
    assert rc == gnlm_lib.NLM_OK, gnlm_lib.last_error()
    ref = gnlm_lib.nlm3d_forward(x, 3, 1, 0.05)
    assert float((out - ref).abs().max()) <= TOL_F32
    assert gnlm_lib.device_status() == (0, 0)
