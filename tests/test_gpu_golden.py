"""The CUDA path against the reference kernels' golden outputs (GPU).

Inputs are the reference's pre-padded unsigned char layout (NLM_FLAG_PREPADDED),
h = 10 on the 0..255 scale; bar 1e-5 of full scale.  On z-varying inputs the
reference's own odd-slice/odd-row error set is excluded (see test_golden.py).
"""
import os

import numpy as np
import pytest

from test_golden import CASES_3D, GOLDEN, TOL, load3d, reference_error_set

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", CASES_3D)
def test_cuda_matches_reference_kernel_3d(torch_cuda, gnlm_lib, name):
    f, SS, NS, X, Y, D, h = load3d(name)
    x = torch_cuda.from_numpy(f["padded"]).cuda()
    got = gnlm_lib.nlm3d_forward(x, (SS - 1) // 2, (NS - 1) // 2, h, prepadded=True,
                                 shape=(D, Y, X)).cpu().numpy()
    diff = np.abs(got - f["out"])
    if "zconst" in name:
        assert diff.max() <= TOL
    else:
        assert diff[~reference_error_set(D, Y, X)].max() <= TOL


def test_cuda_matches_reference_kernel_2d(torch_cuda, gnlm_lib):
    import oracle as O
    f = np.load(os.path.join(GOLDEN, "ref2d_sr7_nb11.npz"))
    sr, nb, X, Y, h = (int(v) for v in f["cfg"])
    padded = np.ascontiguousarray(O.pad_reflect101(f["image"], (sr + nb - 2) // 2))
    x = torch_cuda.from_numpy(padded).cuda()
    got = gnlm_lib.nlm2d_forward(x, (sr - 1) // 2, (nb - 1) // 2, float(h), prepadded=True,
                                 shape=(Y, X)).cpu().numpy()
    assert np.abs(got[f["rows"]] - f["out_rows"]).max() <= TOL
    # FP16-storage form against the same reference output, 1e-3 of full scale
    got16 = gnlm_lib.nlm2d_forward(x, (sr - 1) // 2, (nb - 1) // 2, float(h), prepadded=True,
                                   fp16_storage=True, shape=(Y, X)).cpu().numpy()
    assert np.abs(got16[f["rows"]] - f["out_rows"]).max() <= 1e-3 * 255
