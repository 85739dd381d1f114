"""Every compiled (search radius, patch radius) pair, 3D and 2D, FP32 and FP16 storage,
against the FP64 oracle on small ragged volumes (two or more tiles on every tiled axis).
The pair lists restate the library's compiled instance lists (GNLM_FWD3D_CASES,
GNLM_LP3D_CASES, GNLM_FWD2D_CASES); a pair outside them must be refused with
NLM_ERR_UNSUPPORTED."""
import numpy as np
import pytest

import oracle as O
from gnlm import phantom

TOL_F32 = 1e-5
TOL_F16 = 1e-3
# the weight sum Z of up to 13^3 = 2197 offsets, each weight a 2-ulp ex2 of an FP32 distance,
# summed in FP32: relative (measured up to 1.1e-5 at search 11, patch 5)
TOL_Z = 5e-5

_ORACLE = {}


def _oracle(fn, a, sr, pr, h):
    """FP64 oracle (output, weight sum Z), computed once per (input, pair) for both storage
    forms."""
    key = (fn.__name__, a.shape, sr, pr)
    if key not in _ORACLE:
        _ORACLE[key] = fn(a, sr, pr, h, dtype=np.float64, return_z=True)
    return _ORACLE[key]

BRICK3D = [(1, 1), (2, 1), (3, 1), (4, 1), (5, 1), (3, 2), (5, 2)]
LP3D = [(sr, pr) for pr in range(3, 9) for sr in range(1, 7)] + \
       [(6, 1), (1, 2), (2, 2), (4, 2), (6, 2)]
FWD2D = [(1, 1), (3, 1), (5, 1), (3, 2), (5, 2), (7, 2), (3, 5), (7, 5), (10, 5)]


def test_pair_lists_cover_every_search_patch_combination():
    """The two 3D kernels together cover sr 1..6 with pr 1..8, the whole grid of the
    reference's search widths 3..13 and patch widths 3..17, each pair once."""
    both = set(BRICK3D) | set(LP3D)
    assert len(both) == len(BRICK3D) + len(LP3D) == 48
    assert both == {(sr, pr) for sr in range(1, 7) for pr in range(1, 9)}


# (9, 50, 37): a second tile on every tiled axis; (2, 3, 5) and (1, 1, 1): every extent
# below the halo, so REFLECT_101 folds each axis repeatedly (a single voxel reflects onto
# itself, out = in).
@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(9, 50, 37), (2, 3, 5), (1, 1, 1)])
@pytest.mark.parametrize("fp16", [False, True], ids=["f32", "f16"])
def test_3d_every_compiled_pair(torch_cuda, gnlm_lib, fp16, shape):
    torch = torch_cuda
    v, _ = phantom.ellipsoid_phantom(shape, n_ellipsoids=4, sigma=0.05, seed=77,
                                     radii=(1.5, 8.0))
    x = torch.from_numpy(v).cuda()
    tol = TOL_F16 if fp16 else TOL_F32
    worst = {}
    for sr, pr in BRICK3D + LP3D:
        o, oz = _oracle(O.nlm3d, v, sr, pr, 0.05)
        g, gz = gnlm_lib.nlm3d_forward(x, sr, pr, 0.05, fp16_storage=fp16, return_zsum=True)
        err = float(np.abs(g.cpu().numpy() - o).max())
        zerr = 0.0 if fp16 else float(np.abs(gz.cpu().numpy() / oz - 1).max())
        worst[(sr, pr)] = (err, zerr)
    bad = {k: e for k, e in worst.items() if not (e[0] <= tol and e[1] <= TOL_Z)}
    assert not bad, bad
    assert gnlm_lib.device_status() == (0, 0)


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(45, 131), (3, 5), (1, 1)])
@pytest.mark.parametrize("fp16", [False, True], ids=["f32", "f16"])
def test_2d_every_compiled_pair(torch_cuda, gnlm_lib, fp16, shape):
    torch = torch_cuda
    im, _ = phantom.disc_rect_phantom(shape, n_shapes=6, sigma=0.08, seed=78)
    x = torch.from_numpy(im).cuda()
    tol = TOL_F16 if fp16 else TOL_F32
    worst = {}
    for sr, pr in FWD2D:
        o, oz = _oracle(O.nlm2d, im, sr, pr, 0.08)
        g, gz = gnlm_lib.nlm2d_forward(x, sr, pr, 0.08, fp16_storage=fp16, return_zsum=True)
        err = float(np.abs(g.cpu().numpy() - o).max())
        zerr = 0.0 if fp16 else float(np.abs(gz.cpu().numpy() / oz - 1).max())
        worst[(sr, pr)] = (err, zerr)
    bad = {k: e for k, e in worst.items() if not (e[0] <= tol and e[1] <= TOL_Z)}
    assert not bad, bad
    assert gnlm_lib.device_status() == (0, 0)


@pytest.mark.gpu
def test_uncompiled_pairs_refused(torch_cuda, gnlm_lib):
    torch = torch_cuda
    x3 = torch.rand(9, 20, 20, device="cuda")
    x2 = torch.rand(20, 20, device="cuda")
    for sr, pr in [(7, 3), (1, 9), (0, 3)]:
        with pytest.raises(gnlm_lib.NLMError) as e:
            gnlm_lib.nlm3d_forward(x3, sr, pr, 0.05)
        assert e.value.code in (gnlm_lib.NLM_ERR_UNSUPPORTED, gnlm_lib.NLM_ERR_INVALID_ARG)
    for sr, pr in [(2, 1), (4, 4), (11, 5)]:
        with pytest.raises(gnlm_lib.NLMError) as e:
            gnlm_lib.nlm2d_forward(x2, sr, pr, 0.05)
        assert e.value.code == gnlm_lib.NLM_ERR_UNSUPPORTED
    assert gnlm_lib.device_status() == (0, 0)
