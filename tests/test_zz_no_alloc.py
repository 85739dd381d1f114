"""GPU tests of nlm3d_forward_noalloc, the allocation-free 3D entry point.

That entry point exists for callers that may not allocate device memory while
they run (plug-ins inside an application that owns every GPU allocation through
its own pool, and fixed-budget real-time pipelines that reserve everything at
start-up), so its staging scratch is a fixed 16 MiB array inside libgnlm.so
instead of a cudaMalloc'd or caller-provided workspace.  Here it is called
through the C ABI and must:

* reproduce nlm3d_forward, on two calls in a row with different inputs (the
  shared array keeps the previous call's contents, which must not leak into the
  next result), and the FP32 oracle directly;
* leave the device's free memory unchanged when called on a stream the library
  has never seen with a volume near the size limit (where nlm3d_forward with no
  workspace grows its cache by 16 MB);
* accept the largest volumes whose staging fits the array, in FP32 and FP16
  storage, and reject the next size up with NLM_ERR_WORKSPACE;
* run a large-patch configuration, whose (Z, num) accumulators also live in the
  array.

This file is collected last, so a run that stops at the first failure has run
every other test first; it also passes when run alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

import oracle as O
from gnlm import phantom

pytestmark = pytest.mark.gpu

TOL_F32 = 1e-5
SCRATCH_BYTES = 16 << 20


def _call_noalloc(gnlm, torch, x, sr, pr, h, flags=0, zsum=False, stream=None, out=None):
    Z, Y, X = x.shape
    if out is None:
        out = torch.empty((Z, Y, X), dtype=torch.float32, device="cuda")
    zs = torch.empty_like(out) if zsum else None
    s = stream if stream is not None else torch.cuda.current_stream()
    rc = gnlm.lib().nlm3d_forward_noalloc(
        ctypes.c_void_p(x.data_ptr()), gnlm._dtype_code(x), X, Y, Z, sr, pr, float(h),
        ctypes.c_void_p(out.data_ptr()), None if zs is None else ctypes.c_void_p(zs.data_ptr()),
        flags, ctypes.c_void_p(s.cuda_stream))
    return rc, out, zs


def test_noalloc_matches_forward_on_two_calls(torch_cuda, gnlm_lib):
    torch = torch_cuda
    cases = [((40, 50, 64), 3, 1, 0.05, 0), ((96, 64, 33), 2, 1, 0.08, 0),
             ((128, 128, 128), 3, 1, 0.05, gnlm_lib.NLM_FLAG_FP16_STORAGE),
             ((30, 41, 52), 2, 3, 0.06, 0)]  # large-patch kernel: accumulators in the array
    for k, (shape, sr, pr, h, flags) in enumerate(cases):
        v, _ = phantom.ellipsoid_phantom(shape, n_ellipsoids=8, sigma=h, seed=100 + k)
        x = torch.from_numpy(v).cuda()
        ref, ref_z = gnlm_lib.nlm3d_forward(x, sr, pr, h, return_zsum=True,
                                            fp16_storage=bool(flags))
        rc, out, zs = _call_noalloc(gnlm_lib, torch, x, sr, pr, h, flags, zsum=True)
        assert rc == gnlm_lib.NLM_OK, gnlm_lib.last_error()
        torch.cuda.synchronize()
        assert float((out - ref).abs().max()) <= TOL_F32, (shape, sr, pr)
        assert float(((zs - ref_z).abs() / ref_z).max()) <= TOL_F32, (shape, sr, pr)
        if k == 0:  # and the CPU restatement of the reference's arithmetic itself
            assert float(np.abs(out.cpu().numpy() - O.nlm3d(v, sr, pr, h)).max()) <= TOL_F32
    assert gnlm_lib.device_status() == (0, 0)


def test_noalloc_leaves_free_device_memory_unchanged(torch_cuda, gnlm_lib):
    """On a stream the library has never seen, nlm3d_forward_noalloc of a 152^3 volume
    (16.4 MB of staging, just inside the array) leaves the device's free memory unchanged,
    while nlm3d_forward of the same volume on another new stream lowers it by at least
    the 16 MB its cached workspace takes.  The volume is large on purpose: a cudaMalloc of
    a few hundred KB can be served from memory the driver already holds and would not
    show in the free-memory count."""
    torch = torch_cuda
    v, _ = phantom.ellipsoid_phantom((48, 56, 64), n_ellipsoids=6, sigma=0.05, seed=21)
    x = torch.from_numpy(v).cuda()
    out = torch.empty_like(x)
    # first call in this process: may load the module (which reserves the array itself)
    rc, _, _ = _call_noalloc(gnlm_lib, torch, x, 3, 1, 0.05, out=out)
    assert rc == gnlm_lib.NLM_OK, gnlm_lib.last_error()
    torch.cuda.synchronize()
    assert float(np.abs(out.cpu().numpy() - O.nlm3d(v, 3, 1, 0.05)).max()) <= TOL_F32
    vb, _ = phantom.ellipsoid_phantom((152, 152, 152), n_ellipsoids=8, sigma=0.05, seed=22)
    xb = torch.from_numpy(vb).cuda()
    ob = torch.empty_like(xb)
    ref = gnlm_lib.nlm3d_forward(xb, 3, 1, 0.05)
    fresh = torch.cuda.Stream()  # a stream the library has never seen: no cached workspace
    with torch.cuda.stream(fresh):  # first work on the new stream, outside the library
        ob.mul_(1.0)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    rc, _, _ = _call_noalloc(gnlm_lib, torch, xb, 3, 1, 0.05, stream=fresh, out=ob)
    assert rc == gnlm_lib.NLM_OK, gnlm_lib.last_error()
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    assert float((ob - ref).abs().max()) <= TOL_F32
    # the measurement sees an allocation: nlm3d_forward with no workspace on another new
    # stream grows the library's cache with cudaMalloc
    other = torch.cuda.Stream()
    L = gnlm_lib.lib()
    rc = L.nlm3d_forward(ctypes.c_void_p(xb.data_ptr()), gnlm_lib.NLM_F32, 152, 152, 152, 3, 1,
                         0.05, ctypes.c_void_p(ob.data_ptr()), None, 0, None, 0,
                         ctypes.c_void_p(other.cuda_stream))
    assert rc == gnlm_lib.NLM_OK, gnlm_lib.last_error()
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] <= free0 - (16 << 20)
    assert L.nlm_release_cached() == gnlm_lib.NLM_OK
    assert gnlm_lib.device_status() == (0, 0)


@pytest.mark.parametrize("fp16", [False, True])
def test_noalloc_size_limit(torch_cuda, gnlm_lib, fp16):
    """sr 3, pr 1: 152^3 is the largest cube whose staging fits the array (FP32
    16,384,000 bytes; FP16 storage 16,588,800), 153^3 is rejected."""
    torch = torch_cuda
    flags = gnlm_lib.NLM_FLAG_FP16_STORAGE if fp16 else 0
    L = gnlm_lib.lib()
    assert L.nlm3d_workspace_bytes(152, 152, 152, 3, 1, flags) <= SCRATCH_BYTES
    assert L.nlm3d_workspace_bytes(153, 153, 153, 3, 1, flags) > SCRATCH_BYTES
    x = torch.zeros((153, 153, 153), dtype=torch.float32, device="cuda")
    rc, _, _ = _call_noalloc(gnlm_lib, torch, x, 3, 1, 0.05, flags)
    assert rc == gnlm_lib.NLM_ERR_WORKSPACE
    assert "at most" in gnlm_lib.last_error()
    v, _ = phantom.ellipsoid_phantom((152, 152, 152), n_ellipsoids=8, sigma=0.05, seed=7)
    x = torch.from_numpy(v).cuda()
    for _ in range(2):
        rc, out, _ = _call_noalloc(gnlm_lib, torch, x, 3, 1, 0.05, flags)
        assert rc == gnlm_lib.NLM_OK, gnlm_lib.last_error()
        ref = gnlm_lib.nlm3d_forward(x, 3, 1, 0.05, fp16_storage=fp16)
        assert float((out - ref).abs().max()) <= TOL_F32
    assert gnlm_lib.device_status() == (0, 0)
