"""CPU tests of the oracle: known-answer tests, form agreement, border rule,
legacy layout and the FP64 adjoint against central finite differences."""
import numpy as np
import pytest

import oracle as O
from gnlm import phantom


def test_reflect101_matches_numpy_reflect():
    # OpenCV BORDER_REFLECT_101 == numpy 'reflect' (edge voxel not repeated)
    for n in (1, 2, 3, 7):
        a = np.arange(n)
        for H in (0, 1, 3, 9):
            if n == 1:
                exp = np.zeros(n + 2 * H, int)
            else:
                exp = np.pad(a, H, mode="reflect")
            got = np.array([O.reflect101(i - H, n) for i in range(n + 2 * H)])
            assert np.array_equal(got, exp), (n, H)


@pytest.mark.parametrize("sr,pr", [(1, 1), (3, 1), (2, 2)])
def test_direct_vs_separable_3d(sr, pr):
    v, _ = phantom.ellipsoid_phantom((9, 11, 13), sigma=0.05, seed=4)
    a = O.nlm3d(v, sr, pr, 0.05, form=O.FORM_DIRECT)
    b = O.nlm3d(v, sr, pr, 0.05, form=O.FORM_SEPARABLE)
    c = O.nlm3d(v, sr, pr, 0.05, form=O.FORM_DIRECT, dtype=np.float64)
    d = O.nlm3d(v, sr, pr, 0.05, form=O.FORM_SEPARABLE, dtype=np.float64)
    assert np.abs(a - b).max() < 1e-6
    assert np.abs(a - c).max() < 2e-6
    assert np.abs(c - d).max() < 1e-12


@pytest.mark.parametrize("sr,pr,shape,size", [(2, 2, (24, 30, 36), (6, 7, 8)),
                                               (1, 3, (12, 14, 10), (5, 4, 3))])
def test_block_separable_form_matches_full_volume(sr, pr, shape, size):
    """Boxes at every corner, face centre and the centre, each with its halo gathered
    through REFLECT_101, against the full-volume separable and direct forms."""
    v, _ = phantom.ellipsoid_phantom(shape, n_ellipsoids=6, sigma=0.05, seed=3, radii=(2, 8))
    full = O.nlm3d(v, sr, pr, 0.05, dtype=np.float64)
    origins = O.border_blocks(shape, size)
    assert len(set(origins)) == 15
    blocks = O.nlm3d_blocks(v, sr, pr, 0.05, origins, size)
    nz, ny, nx = size
    for b, (z, y, x) in zip(blocks, origins):
        assert np.abs(b - full[z:z + nz, y:y + ny, x:x + nx]).max() < 1e-14
    d = O.nlm3d_region(v, sr, pr, 0.05, origins[7], size)
    assert np.abs(d - blocks[7]).max() < 1e-14
    b32 = O.nlm3d_blocks(v, sr, pr, 0.05, origins[:2], size, dtype=np.float32)
    assert np.abs(b32 - blocks[:2]).max() < 1e-6


def test_constant_volume_is_fixed_point():
    k = np.full((7, 8, 9), 0.37, np.float32)
    assert np.abs(O.nlm3d(k, 3, 1, 0.05) - 0.37).max() < 2e-6
    k64 = k.astype(np.float64)
    assert np.abs(O.nlm3d(k64, 3, 1, 0.05, dtype=np.float64) - k64).max() < 1e-14


def test_large_h_gives_search_window_mean():
    v = np.random.default_rng(1).random((8, 9, 10))
    out = O.nlm3d(v, 2, 1, 1e8, dtype=np.float64)
    vp = O.pad_reflect101(v, 2)
    from numpy.lib.stride_tricks import sliding_window_view
    bm = sliding_window_view(vp, (5, 5, 5)).mean(axis=(-1, -2, -3))
    assert np.abs(out - bm).max() < 1e-12


def test_small_h_is_identity():
    v = np.random.default_rng(2).random((6, 7, 8))
    out = O.nlm3d(v, 2, 1, 1e-4, dtype=np.float64)
    assert np.abs(out - v).max() < 1e-12


def test_single_impulse_symmetry():
    # an impulse at the centre of a zero volume: the output is symmetric under
    # the reflections of each axis about that centre.
    v = np.zeros((9, 9, 9))
    v[4, 4, 4] = 1.0
    out = O.nlm3d(v, 2, 1, 0.5, dtype=np.float64)
    assert np.allclose(out, out[::-1], atol=1e-15)
    assert np.allclose(out, out[:, ::-1], atol=1e-15)
    assert np.allclose(out, out[:, :, ::-1], atol=1e-15)
    assert np.allclose(out, out.transpose(0, 2, 1), atol=1e-15)


def test_2d_forms_agree():
    im, _ = phantom.disc_rect_phantom((33, 41), sigma=0.08, seed=5)
    a = O.nlm2d(im, 5, 2, 0.08, form=O.FORM_DIRECT)
    b = O.nlm2d(im, 5, 2, 0.08, form=O.FORM_SEPARABLE)
    c = O.nlm2d(im, 5, 2, 0.08, form=O.FORM_DIRECT, dtype=np.float64)
    assert np.abs(a - b).max() < 1e-6
    assert np.abs(a - c).max() < 2e-6


def test_2d_is_3d_of_single_slice_when_z_constant():
    # z-constant volume with patch/search in 3D == 2D NLM with the same radii
    # only when the weights match; check the 2D oracle against a direct formula
    im = np.random.default_rng(3).random((12, 13))
    sr, pr, h = 2, 1, 0.4
    out = O.nlm2d(im, sr, pr, h, dtype=np.float64)
    vp = O.pad_reflect101(im, sr + pr)
    H = sr + pr
    y, x = 5, 7
    num = zs = 0.0
    for oy in range(-sr, sr + 1):
        for ox in range(-sr, sr + 1):
            a = vp[y + H - pr:y + H + pr + 1, x + H - pr:x + H + pr + 1]
            b = vp[y + H + oy - pr:y + H + oy + pr + 1, x + H + ox - pr:x + H + ox + pr + 1]
            w = np.exp(-((a - b) ** 2).mean() / h ** 2)
            num += w * vp[y + H + oy, x + H + ox]
            zs += w
    assert abs(out[y, x] - num / zs) < 1e-14


def test_legacy_padded_u8_matches_unpadded():
    rng = np.random.default_rng(6)
    img = rng.integers(0, 256, (10, 12, 14), dtype=np.uint8)
    SS, NS = 7, 3
    H = (SS + NS - 2) // 2
    padded = O.pad_reflect101(img, H)
    a = O.nlm3d_padded_u8(padded, 14, 12, 10, SS, NS, 10.0)
    b = O.nlm3d(img.astype(np.float32), 3, 1, 10.0)
    assert np.abs(a - b).max() < 1e-3  # values on the 0..255 scale


@pytest.mark.parametrize("sr,pr", [(2, 1), (1, 1)])
def test_adjoint_matches_central_differences(sr, pr):
    v, _ = phantom.ellipsoid_phantom((6, 7, 8), sigma=0.05, seed=7)
    v = v.astype(np.float64)
    h = 0.06
    g = np.random.default_rng(8).standard_normal(v.shape)
    gin, gh, out = O.nlm3d_adjoint(v, sr, pr, h, g)
    assert np.abs(out - O.nlm3d(v, sr, pr, h, dtype=np.float64)).max() < 1e-13

    def L(vv, hh):
        return float((O.nlm3d(vv, sr, pr, hh, dtype=np.float64, form=O.FORM_DIRECT) * g).sum())

    eps = 1e-6
    rng = np.random.default_rng(9)
    for _ in range(6):
        idx = tuple(int(rng.integers(0, s)) for s in v.shape)
        vp, vm = v.copy(), v.copy()
        vp[idx] += eps
        vm[idx] -= eps
        fd = (L(vp, h) - L(vm, h)) / (2 * eps)
        assert abs(fd - gin[idx]) <= 1e-6 * max(1.0, abs(fd)), (idx, fd, gin[idx])
    fdh = (L(v, h + eps) - L(v, h - eps)) / (2 * eps)
    assert abs(fdh - gh) <= 1e-6 * max(1.0, abs(fdh))


def test_phantoms_are_seeded():
    a, ca = phantom.ellipsoid_phantom((16, 16, 16), seed=3)
    b, cb = phantom.ellipsoid_phantom((16, 16, 16), seed=3)
    assert np.array_equal(a, b) and np.array_equal(ca, cb)
    specs = phantom.batch_specs()
    assert len(specs) == 64
    assert sum(s["sr"] == 3 for s in specs) == 32 and sum(s["sr"] == 5 for s in specs) == 32
    assert all(d in phantom.BATCH_DIMS for s in specs for d in s["shape"])
