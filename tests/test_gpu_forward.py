"""GPU parity tests of the forward kernels through the C ABI.

Bars: plain FP32 form within 1e-5 max abs of the FP32 oracle (the CPU
restatement of the reference's arithmetic) on data in [0, 1]; the error against
the FP64 oracle is asserted with the same bound.  FP16-storage form within 1e-3
max abs of the FP64 oracle.
"""
import os
import subprocess

import numpy as np
import pytest

import oracle as O
from gnlm import phantom

pytestmark = pytest.mark.gpu

TOL_F32 = 1e-5
TOL_F16 = 1e-3


def _gpu3d(torch, gnlm, v, sr, pr, h, **kw):
    x = torch.from_numpy(np.ascontiguousarray(v)).cuda()
    r = gnlm.nlm3d_forward(x, sr, pr, h, **kw)
    if isinstance(r, tuple):
        return tuple(t.cpu().numpy() for t in r)
    return r.cpu().numpy()


def _gpu2d(torch, gnlm, v, sr, pr, h, **kw):
    x = torch.from_numpy(np.ascontiguousarray(v)).cuda()
    r = gnlm.nlm2d_forward(x, sr, pr, h, **kw)
    if isinstance(r, tuple):
        return tuple(t.cpu().numpy() for t in r)
    return r.cpu().numpy()


def test_3d_64cubed_workload(torch_cuda, gnlm_lib):
    """64^3, 8 ellipsoids, sigma 0.05, search 7^3, patch 3^3, h 0.05."""
    v, _ = phantom.ellipsoid_phantom((64, 64, 64), n_ellipsoids=8, sigma=0.05, seed=0)
    g = _gpu3d(torch_cuda, gnlm_lib, v, 3, 1, 0.05)
    o32 = O.nlm3d(v, 3, 1, 0.05)
    o64 = O.nlm3d(v, 3, 1, 0.05, dtype=np.float64)
    assert np.abs(g - o32).max() <= TOL_F32
    assert np.abs(g - o64).max() <= TOL_F32
    assert gnlm_lib.device_status() == (0, 0)


SHAPES = [(1, 1, 1), (2, 3, 5), (5, 9, 31), (8, 17, 30), (7, 31, 33), (13, 40, 61), (9, 20, 95)]


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("sr,pr", [(3, 1), (1, 1), (5, 1), (2, 1), (3, 2)])
def test_3d_shapes_and_radii(torch_cuda, gnlm_lib, shape, sr, pr):
    v, _ = phantom.ellipsoid_phantom(shape, n_ellipsoids=4, sigma=0.05, seed=sum(shape),
                                     radii=(1.0, 6.0))
    h = 0.05
    g, gz = _gpu3d(torch_cuda, gnlm_lib, v, sr, pr, h, return_zsum=True)
    o, oz = O.nlm3d(v, sr, pr, h, dtype=np.float64, form=O.FORM_SEPARABLE, return_z=True)
    assert np.abs(g - o).max() <= TOL_F32
    assert np.abs(gz / oz - 1).max() <= 1e-5


@pytest.mark.parametrize("sr,pr", [(3, 1), (5, 1)])
def test_3d_fp16_storage(torch_cuda, gnlm_lib, sr, pr):
    v, _ = phantom.ellipsoid_phantom((24, 40, 70), n_ellipsoids=8, sigma=0.05, seed=11)
    g = _gpu3d(torch_cuda, gnlm_lib, v, sr, pr, 0.05, fp16_storage=True)
    o = O.nlm3d(v, sr, pr, 0.05, dtype=np.float64)
    assert np.abs(g - o).max() <= TOL_F16


def test_3d_input_dtypes(torch_cuda, gnlm_lib):
    rng = np.random.default_rng(12)
    u8 = rng.integers(0, 256, (12, 33, 45), dtype=np.uint8)
    g = _gpu3d(torch_cuda, gnlm_lib, u8, 3, 1, 10.0)
    o = O.nlm3d(u8.astype(np.float64), 3, 1, 10.0, dtype=np.float64)
    assert np.abs(g - o).max() <= TOL_F32 * 255
    v, _ = phantom.ellipsoid_phantom((12, 33, 45), sigma=0.05, seed=13)
    f16 = v.astype(np.float16)
    g = _gpu3d(torch_cuda, gnlm_lib, f16, 3, 1, 0.05)
    o = O.nlm3d(f16.astype(np.float64), 3, 1, 0.05, dtype=np.float64)
    assert np.abs(g - o).max() <= TOL_F32


def test_3d_prepadded_reference_layout(torch_cuda, gnlm_lib):
    """The reference driver's input: one uchar slice padded REFLECT_101 in x/y and
    replicated over depth+SS+NS-2 planes (3DNLM/nlm.cpp:36-61)."""
    SS, NS = 7, 3
    X, Y, Z = 40, 36, 16
    pad = (SS + NS - 2) // 2
    img = np.random.default_rng(14).integers(0, 256, (Y, X), dtype=np.uint8)
    p2 = O.pad_reflect101(img, pad)
    padded = np.ascontiguousarray(np.broadcast_to(p2, (Z + 2 * pad,) + p2.shape))
    g = _gpu3d(torch_cuda, gnlm_lib, padded, 3, 1, 10.0, prepadded=True, shape=(Z, Y, X))
    o = O.nlm3d_padded_u8(padded, X, Y, Z, SS, NS, 10.0)
    assert np.abs(g - o).max() <= TOL_F32 * 255


def _staging_scale(pr, h, dims=3):
    """The pre-scale sqrt(log2(e) / (P h^2)) as the library computes it (double, then float)."""
    P = float((2 * pr + 1) ** dims)
    return np.float32(np.sqrt(1.4426950408889634 / (P * float(np.float32(h)) ** 2)))


@pytest.mark.parametrize("shape", [(20, 24, 64), (9, 17, 45), (5, 6, 7)])
@pytest.mark.parametrize("dt", [np.uint8, np.float16, np.float32])
@pytest.mark.parametrize("fp16", [False, True])
def test_3d_staging_layout_bit_exact(torch_cuda, gnlm_lib, shape, dt, fp16):
    """The staging pass (REFLECT_101 on every axis, conversion, pre-scale) equals a numpy
    construction of the same layout bit for bit: the plain [Zp][Yp][Xs] FP32 layout and
    the FP16 row-pair copies E (rows 2k, 2k+1) and O (rows 2k+1, 2k+2), zero past the
    last row and in the stride padding.  X = 64 takes the vector-load paths, X = 45 and
    the 5 x 6 x 7 volume (halo as wide as the volume) the scalar ones."""
    torch = torch_cuda
    Z, Y, X = shape
    sr, pr, h = 3, 1, 0.05
    rng = np.random.default_rng(sum(shape))
    if dt == np.uint8:
        v = rng.integers(0, 256, shape, dtype=np.uint8)
    else:
        v = rng.random(shape).astype(dt)
    x = torch.from_numpy(v).cuda()
    nbytes = gnlm_lib.nlm3d_workspace_bytes(shape, sr, pr, fp16)
    ws = torch.full((nbytes,), 0xAB, dtype=torch.uint8, device="cuda")
    gnlm_lib.nlm3d_stage(x, sr, pr, h, ws, fp16_storage=fp16)
    torch.cuda.synchronize()
    host = ws.cpu().numpy()
    H = sr + pr
    pv = O.pad_reflect101(v.astype(np.float32), H) * _staging_scale(pr, h)  # float32 product
    Zp, Yp, Xp = pv.shape
    if not fp16:
        Xs = (Xp + 3) // 4 * 4
        st = host[:Zp * Yp * Xs * 4].view(np.float32).reshape(Zp, Yp, Xs)
        assert np.array_equal(st[..., :Xp], pv)
        assert not st[..., Xp:].any()
    else:
        Xs, Yq = (Xp + 3) // 4 * 4, (Yp + 2) // 2
        copy_bytes = (Xs * Yq * Zp * 4 + 255) // 256 * 256
        rows = np.zeros((Zp, 2 * Yq + 2, Xp), np.float16)
        rows[:, :Yp] = pv.astype(np.float16)
        for c in range(2):
            cp = host[c * copy_bytes:c * copy_bytes + Xs * Yq * Zp * 4].view(np.float16)
            cp = cp.reshape(Zp, Yq, Xs, 2)
            for e in range(2):  # half e of pair k is padded row 2k + c + e
                want = rows[:, c + e:c + e + 2 * Yq:2, :]
                assert np.array_equal(cp[:, :, :Xp, e].view(np.uint16), want.view(np.uint16)), (c, e)
            assert not cp[:, :, Xp:].view(np.uint16).any()


def test_3d_host_path_and_workspace_forms_agree(torch_cuda, gnlm_lib):
    torch = torch_cuda
    v, _ = phantom.ellipsoid_phantom((20, 30, 50), sigma=0.05, seed=15)
    a = _gpu3d(torch, gnlm_lib, v, 3, 1, 0.05)
    b = gnlm_lib.nlm3d_forward_host(v, 3, 1, 0.05)
    assert np.array_equal(a, b)
    nbytes = gnlm_lib.lib().nlm3d_workspace_bytes(50, 30, 20, 3, 1, 0)
    ws = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    s = torch.cuda.Stream()
    x = torch.from_numpy(v).cuda()
    torch.cuda.synchronize()
    with torch.cuda.stream(s):
        c = gnlm_lib.nlm3d_forward(x, 3, 1, 0.05, workspace=ws, stream=s)
    s.synchronize()
    assert np.array_equal(a, c.cpu().numpy())
    # the query covers every tile variant's layout; a quarter of it fits none
    too_small = torch.empty(nbytes // 4 // 256 * 256, dtype=torch.uint8, device="cuda")
    with pytest.raises(gnlm_lib.NLMError) as ei:
        gnlm_lib.nlm3d_forward(x, 3, 1, 0.05, workspace=too_small)
    assert ei.value.code == gnlm_lib.NLM_ERR_WORKSPACE
    assert gnlm_lib.device_status() == (0, 0)


def test_3d_256cubed_full_volume(torch_cuda, gnlm_lib):
    """The headline workload, every voxel: 256^3 (64 ellipsoids, sigma 0.05), search 7^3,
    patch 3^3, h 0.05.  Each FP32 tile variant (the default, variant 4, included)
    against the whole FP32 separable oracle volume within 1e-5 max abs, and against the
    whole FP64 separable oracle volume (max abs and RMS stated); FP16 storage against
    the FP64 volume within 1e-3."""
    v, _ = phantom.ellipsoid_phantom((256, 256, 256), n_ellipsoids=64, sigma=0.05, seed=2)
    o32 = O.nlm3d(v, 3, 1, 0.05)
    o64 = O.nlm3d(v, 3, 1, 0.05, dtype=np.float64)
    x = torch_cuda.from_numpy(v).cuda()
    lines = []
    try:
        for var in range(gnlm_lib.variant_count(3)):
            gnlm_lib.set_variant(3, 3, 1, var)
            g = gnlm_lib.nlm3d_forward(x, 3, 1, 0.05).cpu().numpy()
            e32 = float(np.abs(g - o32).max())
            d64 = g.astype(np.float64) - o64
            e64, r64 = float(np.abs(d64).max()), float(np.sqrt(np.mean(d64 * d64)))
            lines.append(f"variant {var}: max abs vs FP32 oracle {e32:.3e}, vs FP64 {e64:.3e}, "
                         f"RMS vs FP64 {r64:.3e}")
            assert e32 <= TOL_F32, lines[-1]
            assert e64 <= TOL_F32, lines[-1]
    finally:
        gnlm_lib.set_variant(3, 3, 1, -1)
    g16 = gnlm_lib.nlm3d_forward(x, 3, 1, 0.05, fp16_storage=True).cpu().numpy()
    d16 = g16.astype(np.float64) - o64
    lines.append(f"FP16 storage: max abs vs FP64 {np.abs(d16).max():.3e}, "
                 f"RMS {np.sqrt(np.mean(d16 * d16)):.3e}")
    assert np.abs(d16).max() <= TOL_F16, lines[-1]
    print("\n".join(lines))
    assert gnlm_lib.device_status() == (0, 0)


def test_2d_2048_workload(torch_cuda, gnlm_lib):
    """2048^2, 32 discs/rectangles, sigma 0.08, search 11^2, patch 5^2, h 0.08."""
    im, _ = phantom.disc_rect_phantom((2048, 2048), n_shapes=32, sigma=0.08, seed=0)
    g = _gpu2d(torch_cuda, gnlm_lib, im, 5, 2, 0.08)
    o32 = O.nlm2d(im, 5, 2, 0.08)
    assert np.abs(g - o32).max() <= TOL_F32
    o64 = O.nlm2d(im, 5, 2, 0.08, dtype=np.float64)
    assert np.abs(g - o64).max() <= TOL_F32


@pytest.mark.parametrize("shape", [(1, 1), (3, 7), (31, 29), (64, 100), (130, 77)])
@pytest.mark.parametrize("sr,pr", [(5, 2), (3, 1), (1, 1), (7, 2), (3, 5)])
def test_2d_shapes_and_radii(torch_cuda, gnlm_lib, shape, sr, pr):
    im, _ = phantom.disc_rect_phantom(shape, n_shapes=6, sigma=0.08, seed=sum(shape))
    g, gz = _gpu2d(torch_cuda, gnlm_lib, im, sr, pr, 0.08, return_zsum=True)
    o, oz = O.nlm2d(im, sr, pr, 0.08, dtype=np.float64, return_z=True)
    assert np.abs(g - o).max() <= TOL_F32
    assert np.abs(gz / oz - 1).max() <= 1e-5


def test_2d_fp16_and_prepadded(torch_cuda, gnlm_lib):
    im, _ = phantom.disc_rect_phantom((96, 96), sigma=0.08, seed=18)
    g = _gpu2d(torch_cuda, gnlm_lib, im, 5, 2, 0.08, fp16_storage=True)
    assert np.abs(g - O.nlm2d(im, 5, 2, 0.08, dtype=np.float64)).max() <= TOL_F16
    # reference 2D driver layout: REFLECT_101-padded uchar, search 7, patch 11
    img = np.random.default_rng(19).integers(0, 256, (64, 64), dtype=np.uint8)
    padded = np.ascontiguousarray(O.pad_reflect101(img, 3 + 5))
    g = _gpu2d(torch_cuda, gnlm_lib, padded, 3, 5, 10.0, prepadded=True, shape=(64, 64))
    o = O.nlm2d_padded_u8(padded, 64, 64, 7, 11, 10.0)
    assert np.abs(g - o).max() <= TOL_F32 * 255


def test_legacy_driver_binary(torch_cuda, gnlm_lib, tmp_path):
    """The raw-array nlm driver (reference 3DNLM/nlm.cpp flow) through the
    NLMeansProcessor shim: output.bin header and truncated uchar voxels."""
    exe = os.path.join(gnlm_lib.LIB_DIR, "nlm_legacy")
    X = Y = Z = 64
    noisy, _ = phantom.disc_rect_phantom((Y, X), n_shapes=8, sigma=0.03, seed=20)
    img = np.clip(noisy * 255.0, 0, 255).astype(np.uint8)
    src = tmp_path / "in.raw"
    img.tofile(src)
    dst = tmp_path / "output.bin"
    subprocess.run([exe, str(src), str(dst)], check=True, timeout=120)
    raw = np.fromfile(dst, dtype=np.uint8)
    hdr = np.frombuffer(raw[:12].tobytes(), dtype=np.int32)
    assert list(hdr) == [Z, Y, X]
    got = raw[12:].reshape(Z, Y, X).astype(int)
    pad = 4
    p2 = O.pad_reflect101(img, pad)
    padded = np.ascontiguousarray(np.broadcast_to(p2, (Z + 2 * pad,) + p2.shape))
    ref_f = O.nlm3d_padded_u8(padded, X, Y, Z, 7, 3, 10.0)
    ref = np.floor(ref_f).astype(int)  # nlm.cpp:68-72 truncates float -> uchar
    frac = ref_f - ref
    away = (frac > 1e-3) & (frac < 1 - 1e-3)  # truncation is stable away from integers
    assert away.mean() > 0.5
    assert np.array_equal(got[away], ref[away])
    assert np.abs(got - ref).max() <= 1


def test_device_status_clean(torch_cuda, gnlm_lib):
    assert gnlm_lib.device_status() == (0, 0)


@pytest.mark.parametrize("fp16", [False, True])
def test_3d_every_tile_variant(torch_cuda, gnlm_lib, fp16):
    """Each autotuner variant (tile shape, register/shared reference values, Kahan
    sums for FP16 storage) against the FP64 oracle, on sizes with ragged edges."""
    tol = TOL_F16 if fp16 else TOL_F32
    cases = [((13, 37, 67), 3, 1), ((9, 20, 95), 5, 1), ((11, 23, 41), 3, 2)]
    for shape, sr, pr in cases:
        v, _ = phantom.ellipsoid_phantom(shape, n_ellipsoids=5, sigma=0.05, seed=sum(shape) + sr,
                                         radii=(2.0, 8.0))
        o = O.nlm3d(v, sr, pr, 0.05, dtype=np.float64)
        try:
            for var in range(gnlm_lib.variant_count(3, fp16)):
                gnlm_lib.set_variant(3, sr, pr, var, fp16)
                g = _gpu3d(torch_cuda, gnlm_lib, v, sr, pr, 0.05, fp16_storage=fp16)
                assert np.abs(g - o).max() <= tol, (shape, sr, pr, var)
        finally:
            gnlm_lib.set_variant(3, sr, pr, -1, fp16)
    assert gnlm_lib.device_status() == (0, 0)


def test_autotune_records_a_variant(torch_cuda, gnlm_lib):
    best, times = gnlm_lib.autotune(3, (32, 64, 90), 3, 1)
    assert 0 <= best < len(times) and all(t > 0 for t in times)
    assert gnlm_lib.get_variant(3, 3, 1) == best
    assert times[best] == min(times)
    gnlm_lib.set_variant(3, 3, 1, -1)
    # reset: back to the measured default (z offsets in groups of four, 4 x 6)
    assert gnlm_lib.get_variant(3, 3, 1) == 4


def test_3d_default_tile_shape(torch_cuda, gnlm_lib):
    """With no recorded variant a patch-3 forward runs on the 4 x 6 tiles with z offsets
    in groups of four (variant 4), the fastest shape measured from 128^3 to 256^3; the
    library reports that choice.  Where another shape gives other bits, the default's
    output shows which shape ran; all agree within the FP32 bar."""
    torch = torch_cuda
    try:
        gnlm_lib.set_variant(3, 3, 1, -1)
        assert gnlm_lib.get_variant(3, 3, 1) == 4
        v, _ = phantom.ellipsoid_phantom((64, 64, 64), n_ellipsoids=8, sigma=0.05, seed=31)
        x = torch.from_numpy(v).cuda()
        outs = {}
        for var in (4, 5, 6):
            gnlm_lib.set_variant(3, 3, 1, var)
            outs[var] = gnlm_lib.nlm3d_forward(x, 3, 1, 0.05).cpu().numpy()
        gnlm_lib.set_variant(3, 3, 1, -1)
        d = gnlm_lib.nlm3d_forward(x, 3, 1, 0.05).cpu().numpy()
        assert np.array_equal(d, outs[4])
        for other in (5, 6):
            if not np.array_equal(outs[4], outs[other]):
                assert not np.array_equal(d, outs[other])
            assert np.abs(outs[4] - outs[other]).max() <= TOL_F32
    finally:
        gnlm_lib.set_variant(3, 3, 1, -1)


@pytest.mark.parametrize("fp16", [False, True])
def test_2d_every_tile_variant(torch_cuda, gnlm_lib, fp16):
    tol = TOL_F16 if fp16 else TOL_F32
    for shape, sr, pr in [((61, 90), 5, 2), ((40, 33), 10, 5), ((37, 70), 3, 1), ((29, 64), 7, 2)]:
        im, _ = phantom.disc_rect_phantom(shape, n_shapes=6, sigma=0.08, seed=sum(shape) + pr)
        o = O.nlm2d(im, sr, pr, 0.08, dtype=np.float64)
        try:
            for var in range(gnlm_lib.variant_count(2, fp16)):
                gnlm_lib.set_variant(2, sr, pr, var, fp16)
                g = _gpu2d(torch_cuda, gnlm_lib, im, sr, pr, 0.08, fp16_storage=fp16)
                assert np.abs(g - o).max() <= tol, (shape, sr, pr, var)
        finally:
            gnlm_lib.set_variant(2, sr, pr, -1, fp16)
    best, times = gnlm_lib.autotune(2, (1, 128, 256), 5, 2)
    assert 0 <= best < len(times) and times[best] == min(times)
    gnlm_lib.set_variant(2, 5, 2, -1)


@pytest.mark.parametrize("shape,sr,pr,fp16,u8_prepadded", [
    ((37, 30, 50), 3, 1, False, False), ((64, 20, 33), 5, 1, False, False),
    ((41, 28, 40), 3, 1, True, False), ((33, 24, 31), 3, 2, False, False),
    ((48, 36, 40), 3, 1, False, True), ((7, 20, 30), 3, 1, False, False),
    ((13, 20, 30), 3, 1, False, False), ((130, 17, 23), 2, 1, False, False),
    ((70, 40, 36), 4, 5, False, False)])
def test_3d_pipelined_host_path_matches_device_path(torch_cuda, gnlm_lib, shape, sr, pr, fp16,
                                                    u8_prepadded):
    """The host-buffer call overlaps its copies with compute over z chunks (a first and
    a last chunk of one z tile, larger ones between; 7 and 13 planes give two and three
    chunks, 130 planes many, the large-patch case chunks by its chunk depth); the result
    must equal the device-buffer call exactly."""
    torch = torch_cuda
    v, _ = phantom.ellipsoid_phantom(shape, n_ellipsoids=6, sigma=0.05, seed=sum(shape) + sr)
    h = 0.05
    if u8_prepadded:
        v = np.ascontiguousarray(O.pad_reflect101(np.clip(v * 255, 0, 255).astype(np.uint8), sr + pr))
        h = 10.0
    dev = gnlm_lib.nlm3d_forward(torch.from_numpy(v).cuda(), sr, pr, h, fp16_storage=fp16,
                                 prepadded=u8_prepadded, shape=shape).cpu().numpy()
    pinned = torch.from_numpy(v).pin_memory().numpy()
    host = gnlm_lib.nlm3d_forward_host(pinned, sr, pr, h, fp16_storage=fp16,
                                       prepadded=u8_prepadded, shape=shape)
    assert np.array_equal(dev, host)


def test_3d_volume_beyond_2_31_voxels(torch_cuda, gnlm_lib):
    """40 x 6000 x 9000 = 2.16 G voxels (64-bit element indices in staging, kernel
    output and the host-visible result): blocks at the corners and inside against
    the FP64 direct form, each computed on a host crop that contains the block plus
    its search+patch halo (crops that start at a volume border keep that border's
    REFLECT_101; blocks stay H away from a crop's inner faces)."""
    torch = torch_cuda
    Z, Y, X = 40, 6000, 9000
    assert Z * Y * X > 2 ** 31
    g = torch.Generator(device="cuda").manual_seed(21)
    v = torch.rand((Z, Y, X), device="cuda", generator=g)
    # smooth structure plus noise: blend with a shifted copy so weights vary
    v = (0.6 * v + 0.4 * torch.roll(v, shifts=(1, 2, 3), dims=(0, 1, 2))).contiguous()
    out = gnlm_lib.nlm3d_forward(v, 3, 1, 0.05)
    H = 4
    blocks = [(0, 0, 0), (Z - 8, Y - 8, X - 8), (16, 3000, 4500), (0, Y - 8, 0), (32, 5100, 8200)]
    for (z0, y0, x0) in blocks:
        cz0, cy0, cx0 = max(0, z0 - 2 * H), max(0, y0 - 2 * H), max(0, x0 - 2 * H)
        cz1, cy1, cx1 = min(Z, z0 + 8 + 2 * H), min(Y, y0 + 8 + 2 * H), min(X, x0 + 8 + 2 * H)
        crop = v[cz0:cz1, cy0:cy1, cx0:cx1].cpu().numpy().astype(np.float64)
        ref = O.nlm3d_region(crop, 3, 1, 0.05, (z0 - cz0, y0 - cy0, x0 - cx0), (8, 8, 8))
        got = out[z0:z0 + 8, y0:y0 + 8, x0:x0 + 8].cpu().numpy()
        assert np.abs(got - ref).max() <= TOL_F32, (z0, y0, x0)
    del v, out
    torch.cuda.empty_cache()
    assert gnlm_lib.device_status() == (0, 0)


def test_3d_forward_captured_in_a_cuda_graph(torch_cuda, gnlm_lib):
    """nlm3d_forward with a caller workspace is capturable: the staging pass and the
    NLM kernel replay from a CUDA graph (tensor maps travel as kernel parameters) and
    follow new input data written into the same buffer."""
    torch = torch_cuda
    shape = (24, 40, 70)
    v1, _ = phantom.ellipsoid_phantom(shape, n_ellipsoids=5, sigma=0.05, seed=61)
    v2, _ = phantom.ellipsoid_phantom(shape, n_ellipsoids=5, sigma=0.05, seed=62)
    Z, Y, X = shape
    x = torch.from_numpy(v1).cuda()
    out = torch.empty_like(x)
    ws = torch.empty(gnlm_lib.lib().nlm3d_workspace_bytes(X, Y, Z, 3, 1, 0), dtype=torch.uint8,
                     device="cuda")
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        gnlm_lib.nlm3d_forward(x, 3, 1, 0.05, out=out, workspace=ws, stream=s)  # warm-up
    s.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        gnlm_lib.nlm3d_forward(x, 3, 1, 0.05, out=out, workspace=ws,
                               stream=torch.cuda.current_stream())
    for v in (v1, v2):
        x.copy_(torch.from_numpy(v))
        out.zero_()
        g.replay()
        torch.cuda.synchronize()
        direct = gnlm_lib.nlm3d_forward(torch.from_numpy(v).cuda(), 3, 1, 0.05).cpu().numpy()
        assert np.array_equal(out.cpu().numpy(), direct)
    assert gnlm_lib.device_status() == (0, 0)


def test_concurrent_calls_from_host_threads(torch_cuda, gnlm_lib):
    """Four host threads, each on its own stream (its own cached workspace), call the
    3D forward (small- and large-patch kernels) and the 2D forward concurrently; every
    result equals the same call made alone."""
    import threading
    torch = torch_cuda
    v, _ = phantom.ellipsoid_phantom((20, 33, 47), n_ellipsoids=5, sigma=0.05, seed=71)
    im, _ = phantom.disc_rect_phantom((90, 130), n_shapes=6, sigma=0.08, seed=72)
    jobs = [(3, 3, 1, 0.05), (3, 5, 6, 0.05), (3, 2, 1, 0.07), (2, 5, 2, 0.08)]

    def run(dims, sr, pr, h, stream=None):
        if dims == 3:
            return gnlm_lib.nlm3d_forward(torch.from_numpy(v).cuda(), sr, pr, h, stream=stream)
        return gnlm_lib.nlm2d_forward(torch.from_numpy(im).cuda(), sr, pr, h, stream=stream)

    expected = [run(*j).cpu().numpy() for j in jobs]
    results = [None] * len(jobs)
    errors = []

    def worker(i):
        try:
            s = torch.cuda.Stream()
            with torch.cuda.stream(s):
                outs = [run(*jobs[i], stream=s) for _ in range(5)]
            s.synchronize()
            results[i] = [o.cpu().numpy() for o in outs]
        except Exception as e:  # reported below
            errors.append(repr(e))

    threads = [threading.Thread(target=worker, args=(i,)) for i in range(len(jobs))]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    for i, outs in enumerate(results):
        for o in outs:
            assert np.array_equal(o, expected[i]), jobs[i]
    assert gnlm_lib.device_status() == (0, 0)
