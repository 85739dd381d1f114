"""Failure handling on the GPU without faulting it: a workspace the device cannot
hold is reported as a status (no kernel is launched), and the library keeps
working afterwards with no stale error carried into the next call."""
import ctypes

import numpy as np
import pytest

import oracle as O
from gnlm import phantom

pytestmark = pytest.mark.gpu


def test_workspace_allocation_failure_is_reported_and_recoverable(torch_cuda, gnlm_lib):
    torch = torch_cuda
    L = gnlm_lib.lib()
    small = torch.zeros(64, device="cuda")
    out = torch.zeros(64, device="cuda")
    P = ctypes.c_void_p
    # 8000^3 voxels: about 2 TB of staging workspace, far beyond the device; the
    # library allocates before it launches anything, so the small buffers are never read
    need = L.nlm3d_workspace_bytes(8000, 8000, 8000, 3, 1, 0)
    assert need > 10 ** 12
    rc = L.nlm3d_forward(P(small.data_ptr()), gnlm_lib.NLM_F32, 8000, 8000, 8000, 3, 1, 0.05,
                         P(out.data_ptr()), None, 0, None, 0, None)
    assert rc == gnlm_lib.NLM_ERR_CUDA
    assert "cudaMalloc" in gnlm_lib.last_error()
    # the next calls succeed and are correct
    v, _ = phantom.ellipsoid_phantom((9, 14, 37), n_ellipsoids=3, sigma=0.05, seed=31,
                                     radii=(1.5, 5.0))
    for sr, pr in [(3, 1), (5, 6)]:
        g = gnlm_lib.nlm3d_forward(torch.from_numpy(v).cuda(), sr, pr, 0.05).cpu().numpy()
        assert np.abs(g - O.nlm3d(v, sr, pr, 0.05, dtype=np.float64)).max() <= 1e-5
    assert gnlm_lib.device_status() == (0, 0)


def test_bounds_checked_build_is_clean_and_identical(torch_cuda, gnlm_lib, tmp_path):
    """The NLM_BOUNDS_CHECK build (lib/libgnlm_checked.so) checks every kernel's index
    ranges at run time: on the cases of tests/checked_cases.py its error word stays
    clean and its results equal the normal build's bit for bit."""
    import json
    import os
    import subprocess
    import sys

    import checked_cases
    if not os.path.exists(gnlm_lib.CHECKED_LIB_PATH):
        pytest.skip("checked build not present")
    ref = checked_cases.run_cases(gnlm_lib, torch_cuda)
    assert gnlm_lib.device_status() == (0, 0)
    path = tmp_path / "checked.npz"
    env = dict(os.environ, GNLM_LIB=gnlm_lib.CHECKED_LIB_PATH)
    here = os.path.dirname(os.path.abspath(__file__))
    proc = subprocess.run([sys.executable, os.path.join(here, "checked_cases.py"), str(path)],
                          env=env, capture_output=True, text=True, timeout=600)
    assert proc.returncode == 0, proc.stderr[-2000:]
    status = json.loads(proc.stdout.strip().splitlines()[-1])
    assert status["lib"].endswith("libgnlm_checked.so")
    assert status["rc"] == 0 and status["flags"] == 0, status
    got = np.load(path)
    assert sorted(got.files) == sorted(ref)
    for k, v in ref.items():
        assert np.array_equal(got[k], v), k


def test_bounded_tile_copy_waits_run_out_and_report(torch_cuda, gnlm_lib):
    """Every kernel family's bounded tile-copy wait is driven to its limit in the
    checked test build (tests/fault_cases.py, a child process): the call returns, the
    device error word reports 0x1 (tile copy timed out), and once injection is off the
    next call is clean and matches the FP64 oracle.  No GPU fault is involved: the
    injected CTA never issues its copy, so nothing is in flight when it gives up."""
    import json
    import os
    import subprocess
    import sys

    if not os.path.exists(gnlm_lib.CHECKED_LIB_PATH):
        pytest.skip("checked build not present")
    env = dict(os.environ, GNLM_LIB=gnlm_lib.CHECKED_LIB_PATH)
    here = os.path.dirname(os.path.abspath(__file__))
    proc = subprocess.run([sys.executable, os.path.join(here, "fault_cases.py")], env=env,
                          capture_output=True, text=True, timeout=600)
    assert proc.returncode == 0, proc.stderr[-2000:]
    res = json.loads(proc.stdout.strip().splitlines()[-1])
    assert res["lib"].endswith("libgnlm_checked.so")
    assert set(res["cases"]) == {"3d_fp32", "3d_fp16_storage", "2d", "batched", "adjoint",
                                 "large_patch"}
    for name, r in res["cases"].items():
        assert r["set"] == 0 and r["unset"] == 0, (name, r)
        assert r["status"] == gnlm_lib.NLM_ERR_DEVICE and r["flags"] == 0x1, (name, r)
        assert r["after_status"] == 0 and r["after_flags"] == 0, (name, r)
    assert res["after_err_vs_fp64"] <= 1e-5
    assert res["final_status"] == [0, 0]
