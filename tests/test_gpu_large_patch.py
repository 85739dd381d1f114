"""GPU parity tests of the large-patch 3D kernel (patch radius 3..8, and the
(search, patch) pairs the register-brick kernel does not compile), through the
C ABI, against the FP64 oracle.  Bars: 1e-5 max abs on data in [0, 1] for FP32
storage, 1e-3 for FP16 storage.

The reference sweeps search windows 11 and 13 with patches 13, 15 and 17 on
512 x 512 slices of depth 16..128 (3DNLM/run.sh:25-34); the last test runs one of
those sizes and checks blocks of it against the direct-form oracle.
"""
import numpy as np
import pytest

import oracle as O
from gnlm import phantom

pytestmark = pytest.mark.gpu

TOL = 1e-5

LARGE = [(1, 3), (3, 3), (6, 3), (2, 4), (5, 4), (4, 5), (1, 6), (5, 6), (6, 6), (3, 7), (5, 7),
         (6, 7), (1, 8), (5, 8), (6, 8), (6, 1), (1, 2), (2, 2), (4, 2), (6, 2)]


def _gpu3d(torch, gnlm, v, sr, pr, h, **kw):
    x = torch.from_numpy(np.ascontiguousarray(v)).cuda()
    r = gnlm.nlm3d_forward(x, sr, pr, h, **kw)
    if isinstance(r, tuple):
        return tuple(t.cpu().numpy() for t in r)
    return r.cpu().numpy()


@pytest.mark.parametrize("sr,pr", LARGE)
def test_large_patch_vs_fp64_oracle(torch_cuda, gnlm_lib, sr, pr):
    """Ragged in every axis: 41 columns (two x tiles), 23 rows (two y tiles), 19 planes."""
    shape = (19, 23, 41)
    v, _ = phantom.ellipsoid_phantom(shape, n_ellipsoids=5, sigma=0.05, seed=100 + 10 * sr + pr,
                                     radii=(2.0, 9.0))
    h = 0.05
    g, gz = _gpu3d(torch_cuda, gnlm_lib, v, sr, pr, h, return_zsum=True)
    o, oz = O.nlm3d(v, sr, pr, h, dtype=np.float64, return_z=True)
    assert np.abs(g - o).max() <= TOL
    assert np.abs(gz / oz - 1).max() <= 1e-5
    assert gnlm_lib.device_status() == (0, 0)


@pytest.mark.parametrize("shape", [(1, 1, 1), (2, 3, 5), (5, 17, 33), (3, 40, 70)])
def test_large_patch_tiny_and_thin_volumes(torch_cuda, gnlm_lib, shape):
    """Volumes thinner than the halo: REFLECT_101 folds the halo back many times."""
    v, _ = phantom.ellipsoid_phantom(shape, n_ellipsoids=3, sigma=0.05, seed=sum(shape),
                                     radii=(1.0, 5.0))
    for sr, pr in [(5, 6), (6, 8)]:
        g = _gpu3d(torch_cuda, gnlm_lib, v, sr, pr, 0.05)
        o = O.nlm3d(v, sr, pr, 0.05, dtype=np.float64)
        assert np.abs(g - o).max() <= TOL, (shape, sr, pr)
        g16 = _gpu3d(torch_cuda, gnlm_lib, v, sr, pr, 0.05, fp16_storage=True)
        assert np.abs(g16 - o).max() <= 1e-3, (shape, sr, pr)


@pytest.mark.parametrize("sr,pr", [(2, 4), (6, 3), (4, 5)])
def test_large_patch_every_chunk_variant(torch_cuda, gnlm_lib, sr, pr):
    """Each chunk depth (64, 32, 128, 16, 48, 96, 80 planes) on 37 planes: partial last
    chunks, several chunks per column; search 9 and 13 run the x-half form (two CTAs per
    tile, each with half of the x offsets, 48-row tiles), whose repeated calls give the
    same bits."""
    shape = (37, 20, 36)
    v, _ = phantom.ellipsoid_phantom(shape, n_ellipsoids=5, sigma=0.05, seed=7, radii=(2.0, 8.0))
    o = O.nlm3d(v, sr, pr, 0.05, dtype=np.float64)
    try:
        for var in range(gnlm_lib.variant_count(3, False)):
            gnlm_lib.set_variant(3, sr, pr, var)
            g = _gpu3d(torch_cuda, gnlm_lib, v, sr, pr, 0.05)
            assert np.abs(g - o).max() <= TOL, var
            assert np.array_equal(g, _gpu3d(torch_cuda, gnlm_lib, v, sr, pr, 0.05)), var
    finally:
        gnlm_lib.set_variant(3, sr, pr, -1)
    best, times = gnlm_lib.autotune(3, (40, 64, 64), sr, pr)
    assert 0 <= best < len(times) and times[best] == min(times)
    gnlm_lib.set_variant(3, sr, pr, -1)


def test_large_patch_reference_layout_u8(torch_cuda, gnlm_lib):
    """The reference driver's pre-padded uchar input at SS 11, NS 13 (h = PARAMETER = 10)."""
    SS, NS = 11, 13
    X, Y, Z = 40, 36, 16
    pad = (SS + NS - 2) // 2
    img = np.clip(phantom.disc_rect_phantom((Y, X), n_shapes=5, sigma=0.03, seed=3)[0] * 255,
                  0, 255).astype(np.uint8)
    p2 = O.pad_reflect101(img, pad)
    padded = np.ascontiguousarray(np.broadcast_to(p2, (Z + 2 * pad,) + p2.shape))
    g = _gpu3d(torch_cuda, gnlm_lib, padded, 5, 6, 10.0, prepadded=True, shape=(Z, Y, X))
    o = O.nlm3d_padded_u8(padded, X, Y, Z, SS, NS, 10.0)
    assert np.abs(g - o).max() <= TOL * 255


def test_large_patch_host_path_and_workspace(torch_cuda, gnlm_lib):
    """Host-buffer (pipelined over z chunks) and caller-workspace calls equal the
    device call; the workspace query includes the accumulator pairs."""
    torch = torch_cuda
    shape, sr, pr = (70, 24, 33), 5, 6
    v, _ = phantom.ellipsoid_phantom(shape, n_ellipsoids=6, sigma=0.05, seed=9)
    dev = _gpu3d(torch, gnlm_lib, v, sr, pr, 0.05)
    pinned = torch.from_numpy(v).pin_memory().numpy()
    host = gnlm_lib.nlm3d_forward_host(pinned, sr, pr, 0.05)
    assert np.array_equal(dev, host)
    Z, Y, X = shape
    nbytes = gnlm_lib.lib().nlm3d_workspace_bytes(X, Y, Z, sr, pr, 0)
    assert nbytes >= X * Y * Z * 8
    ws = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    c = gnlm_lib.nlm3d_forward(torch.from_numpy(v).cuda(), sr, pr, 0.05, workspace=ws)
    assert np.array_equal(dev, c.cpu().numpy())
    short = torch.empty(nbytes - X * Y * Z * 8, dtype=torch.uint8, device="cuda")
    with pytest.raises(gnlm_lib.NLMError) as ei:
        gnlm_lib.nlm3d_forward(torch.from_numpy(v).cuda(), sr, pr, 0.05, workspace=short)
    assert ei.value.code == gnlm_lib.NLM_ERR_WORKSPACE


TOL_F16 = 1e-3


@pytest.mark.parametrize("sr,pr", LARGE)
def test_large_patch_fp16_storage_vs_fp64_oracle(torch_cuda, gnlm_lib, sr, pr):
    """FP16 storage (FP16 staged volume and plane boxes, FP32 arithmetic, Kahan pass
    sums) on the ragged shape of the FP32 test: within 1e-3 of the FP64 oracle."""
    shape = (19, 23, 41)
    v, _ = phantom.ellipsoid_phantom(shape, n_ellipsoids=5, sigma=0.05, seed=100 + 10 * sr + pr,
                                     radii=(2.0, 9.0))
    g, gz = _gpu3d(torch_cuda, gnlm_lib, v, sr, pr, 0.05, return_zsum=True, fp16_storage=True)
    o, oz = O.nlm3d(v, sr, pr, 0.05, dtype=np.float64, return_z=True)
    assert np.abs(g - o).max() <= TOL_F16
    # the weight sums are exponentials of distances between FP16-rounded values, so
    # they move by about 1e-3 relative; the 1e-3 bar applies to the output above
    assert np.abs(gz / oz - 1).max() <= 1e-2
    assert gnlm_lib.device_status() == (0, 0)


def test_large_patch_fp16_storage_variants_split_and_host_path(torch_cuda, gnlm_lib):
    """FP16 storage: every chunk depth; a split grid (Kahan halves added by the combine
    kernel) and a whole-wave grid; the pipelined host path equals the device call; the
    workspace query counts the FP16 volume and the Kahan accumulator pairs."""
    torch = torch_cuda
    shape, sr, pr = (37, 20, 36), 2, 4
    v, _ = phantom.ellipsoid_phantom(shape, n_ellipsoids=5, sigma=0.05, seed=7, radii=(2.0, 8.0))
    o = O.nlm3d(v, sr, pr, 0.05, dtype=np.float64)
    try:
        for var in range(gnlm_lib.variant_count(3, True)):
            gnlm_lib.set_variant(3, sr, pr, var, fp16_storage=True)
            g = _gpu3d(torch, gnlm_lib, v, sr, pr, 0.05, fp16_storage=True)
            assert np.abs(g - o).max() <= TOL_F16, var
    finally:
        gnlm_lib.set_variant(3, sr, pr, -1, fp16_storage=True)
    for shp in [(4, 912, 250), (4, 432, 250)]:  # one whole wave, a split grid (see below)
        w, _ = phantom.ellipsoid_phantom(shp, n_ellipsoids=8, sigma=0.05, seed=shp[1],
                                         radii=(3.0, 20.0))
        g = _gpu3d(torch, gnlm_lib, w, 1, 3, 0.05, fp16_storage=True)
        assert np.abs(g - O.nlm3d(w, 1, 3, 0.05, dtype=np.float64)).max() <= TOL_F16, shp
        assert np.array_equal(g, _gpu3d(torch, gnlm_lib, w, 1, 3, 0.05, fp16_storage=True))
    shape, sr, pr = (70, 24, 33), 5, 6
    v, _ = phantom.ellipsoid_phantom(shape, n_ellipsoids=6, sigma=0.05, seed=9)
    dev = _gpu3d(torch, gnlm_lib, v, sr, pr, 0.05, fp16_storage=True)
    host = gnlm_lib.nlm3d_forward_host(torch.from_numpy(v).pin_memory().numpy(), sr, pr, 0.05,
                                       fp16_storage=True)
    assert np.array_equal(dev, host)
    assert np.abs(dev - O.nlm3d(v, sr, pr, 0.05, dtype=np.float64)).max() <= TOL_F16
    Z, Y, X = shape
    H = sr + pr
    xs = (X + 2 * H + 7) // 8 * 8
    staged = ((xs * (Y + 2 * H) * (Z + 2 * H) * 2 + 255) // 256) * 256
    # four Kahan accumulator buffers from search radius 3 (pass halves x x-offset halves)
    assert gnlm_lib.lib().nlm3d_workspace_bytes(X, Y, Z, sr, pr, gnlm_lib.NLM_FLAG_FP16_STORAGE) == \
        staged + ((4 * X * Y * Z * 16 + 255) // 256) * 256
    assert gnlm_lib.device_status() == (0, 0)


def test_large_patch_sweep_size_spot_checks(torch_cuda, gnlm_lib):
    """512 x 512 x 16, search 13^3, patch 17^3 (the largest window of the
    reference's sweep): corner, edge and interior blocks against the direct form."""
    v, _ = phantom.ellipsoid_phantom((16, 512, 512), n_ellipsoids=48, sigma=0.05, seed=4)
    g = _gpu3d(torch_cuda, gnlm_lib, v, 6, 8, 0.05)
    assert np.isfinite(g).all()
    rng = np.random.default_rng(5)
    boxes = [(0, 0, 0), (12, 508, 508), (6, 0, 300), (0, 255, 508)]
    boxes += [(int(rng.integers(0, 12)), int(rng.integers(0, 508)), int(rng.integers(0, 508)))
              for _ in range(2)]
    for (z0, y0, x0) in boxes:
        o = O.nlm3d_region(v, 6, 8, 0.05, (z0, y0, x0), (4, 4, 4))
        assert np.abs(g[z0:z0 + 4, y0:y0 + 4, x0:x0 + 4] - o).max() <= TOL, (z0, y0, x0)
    assert gnlm_lib.device_status() == (0, 0)


def test_large_patch_sweep_size_fp16_storage(torch_cuda, gnlm_lib):
    """512 x 512 x 16, search 13^3, patch 17^3 with FP16 storage: 15 boxes of 8^3 (the 8
    corners, 6 face centres, the centre) against the FP64 block-separable oracle."""
    v, _ = phantom.ellipsoid_phantom((16, 512, 512), n_ellipsoids=48, sigma=0.05, seed=4)
    g = _gpu3d(torch_cuda, gnlm_lib, v, 6, 8, 0.05, fp16_storage=True)
    origins = O.border_blocks(v.shape, (8, 8, 8))
    ref = O.nlm3d_blocks(v, 6, 8, 0.05, origins, (8, 8, 8))
    for b, (z0, y0, x0) in zip(ref, origins):
        assert np.abs(g[z0:z0 + 8, y0:y0 + 8, x0:x0 + 8] - b).max() <= TOL_F16, (z0, y0, x0)
    assert gnlm_lib.device_status() == (0, 0)


def test_large_patch_split_and_whole_passes(torch_cuda, gnlm_lib):
    """One CTA per SM: a grid that leaves the last wave mostly idle splits each tile's
    passes into two halves with separate accumulators, added by a combine kernel;
    a grid of whole waves does not (and the combine kernel still writes num / Z from the
    one buffer).  On a 152-SM GB300 with 32 x 48 tiles and every x offset per CTA (search
    3), 250 x 912 x 4 is 8 x 19 tiles = exactly one wave (no split) and 250 x 432 x 4 is
    8 x 9 tiles, under half a wave (split).  Both match the FP64 oracle, and repeated calls
    give the same bits."""
    for shape in [(4, 912, 250), (4, 432, 250)]:
        v, _ = phantom.ellipsoid_phantom(shape, n_ellipsoids=8, sigma=0.05, seed=shape[1],
                                         radii=(3.0, 20.0))
        g = _gpu3d(torch_cuda, gnlm_lib, v, 1, 3, 0.05)
        o = O.nlm3d(v, 1, 3, 0.05, dtype=np.float64)
        assert np.abs(g - o).max() <= TOL, shape
        assert np.array_equal(g, _gpu3d(torch_cuda, gnlm_lib, v, 1, 3, 0.05))
    assert gnlm_lib.device_status() == (0, 0)
