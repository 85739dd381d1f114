"""GPU tests of the 3D adjoint (nlm3d_adjoint) through the C ABI.

* against the FP64 oracle adjoint (direct form), which is itself checked against
  FP64 central differences in test_oracle.py;
* bitwise determinism (gather form, fixed-order h reduction);
* a torch.autograd.Function harness (forward and backward both the CUDA kernels)
  checked against FP64 central differences of the FP64 oracle forward, on random
  voxels and on h;
* a few gradient-descent steps on h that lower the error to the clean phantom.
FP32 kernels against FP64 references: bar 2e-4 of the gradient's scale.
"""
import numpy as np
import pytest

import oracle as O
from gnlm import phantom

pytestmark = pytest.mark.gpu

REL = 2e-4


def _run(torch, gnlm, v, sr, pr, h, g):
    x = torch.from_numpy(np.ascontiguousarray(v, dtype=np.float32)).cuda()
    out, zs = gnlm.nlm3d_forward(x, sr, pr, h, return_zsum=True)
    gin, hg = gnlm.nlm3d_adjoint(x, out, zs, torch.from_numpy(g.astype(np.float32)).cuda(), sr, pr, h)
    torch.cuda.synchronize()
    return gin.cpu().numpy(), float(hg.item()), out.cpu().numpy()


# One CTA per SM: grids under a wave split every tile into offset-run parts; on a
# 152-SM GB300, (40, 60, 56) is 180 tiles = 152 whole + 28 tail tiles in 5 parts each,
# and (50, 40, 48) is 90 tiles, too many for a split (each tile made whole).  Search 9 and
# 11 run 2-plane tiles with z offsets in groups of 5 + 4 and 6 + 5: (24, 30, 28) is 170
# tiles (18 tail tiles in 8 parts), (20, 30, 26) 192 (40 in 3 parts).
@pytest.mark.parametrize("shape,sr,pr", [((8, 10, 12), 2, 1), ((12, 13, 14), 3, 1),
                                         ((9, 11, 40), 1, 1), ((10, 12, 12), 3, 2),
                                         ((7, 9, 11), 5, 1), ((3, 4, 5), 3, 1),
                                         ((40, 60, 56), 3, 1), ((50, 40, 48), 3, 1),
                                         ((11, 14, 13), 4, 1), ((24, 30, 28), 4, 1),
                                         ((20, 30, 26), 5, 1)])
def test_adjoint_matches_fp64_oracle(torch_cuda, gnlm_lib, shape, sr, pr):
    v, _ = phantom.ellipsoid_phantom(shape, n_ellipsoids=4, sigma=0.05, seed=sum(shape) + sr,
                                     radii=(1.5, 6.0))
    h = 0.06
    g = np.random.default_rng(sr * 7 + pr).standard_normal(shape)
    gin, hg, out = _run(torch_cuda, gnlm_lib, v, sr, pr, h, g)
    rgin, rhg, rout = O.nlm3d_adjoint(v.astype(np.float64), sr, pr, h, g)
    assert np.abs(out - rout).max() <= 1e-5
    scale = np.abs(rgin).max()
    assert np.abs(gin - rgin).max() <= REL * scale, (np.abs(gin - rgin).max(), scale)
    assert abs(hg - rhg) <= REL * max(abs(rhg), 1.0), (hg, rhg)
    assert gnlm_lib.device_status() == (0, 0)


def test_adjoint_is_deterministic(torch_cuda, gnlm_lib):
    v, _ = phantom.ellipsoid_phantom((20, 24, 60), sigma=0.05, seed=5)
    g = np.random.default_rng(1).standard_normal(v.shape)
    a = _run(torch_cuda, gnlm_lib, v, 3, 1, 0.05, g)
    b = _run(torch_cuda, gnlm_lib, v, 3, 1, 0.05, g)
    assert np.array_equal(a[0], b[0]) and a[1] == b[1]


class NLMFunction:
    """torch.autograd.Function over the CUDA forward and adjoint (test harness only)."""

    @staticmethod
    def make(torch, gnlm, sr, pr):
        class _F(torch.autograd.Function):
            @staticmethod
            def forward(ctx, x, h):
                out, zs = gnlm.nlm3d_forward(x.detach().contiguous(), sr, pr, float(h),
                                             return_zsum=True)
                ctx.save_for_backward(x, out, zs, h)
                return out

            @staticmethod
            def backward(ctx, gout):
                x, out, zs, h = ctx.saved_tensors
                gin, hg = gnlm.nlm3d_adjoint(x.contiguous(), out, zs, gout.contiguous(), sr, pr,
                                             float(h))
                return gin, hg.to(h.dtype).reshape(h.shape)

        return _F.apply


def test_autograd_harness_against_fp64_finite_differences(torch_cuda, gnlm_lib):
    torch = torch_cuda
    sr, pr, h0 = 2, 1, 0.07
    v, _ = phantom.ellipsoid_phantom((8, 9, 10), n_ellipsoids=3, sigma=0.05, seed=9, radii=(2.0, 5.0))
    g = np.random.default_rng(2).standard_normal(v.shape)
    f = NLMFunction.make(torch, gnlm_lib, sr, pr)
    x = torch.from_numpy(v).cuda().requires_grad_(True)
    h = torch.tensor([h0], dtype=torch.float64, device="cuda", requires_grad=True)
    out = f(x, h)
    (out * torch.from_numpy(g.astype(np.float32)).cuda()).sum().backward()
    gx = x.grad.cpu().numpy()
    gh = float(h.grad.item())
    v64 = v.astype(np.float64)

    def L(vv, hh):
        return float((O.nlm3d(vv, sr, pr, hh, dtype=np.float64, form=O.FORM_DIRECT) * g).sum())

    eps = 1e-6
    rng = np.random.default_rng(3)
    scale = np.abs(gx).max()
    for _ in range(8):
        idx = tuple(int(rng.integers(0, s)) for s in v.shape)
        vp, vm = v64.copy(), v64.copy()
        vp[idx] += eps
        vm[idx] -= eps
        fd = (L(vp, h0) - L(vm, h0)) / (2 * eps)
        assert abs(gx[idx] - fd) <= REL * scale, (idx, gx[idx], fd)
    fdh = (L(v64, h0 + eps) - L(v64, h0 - eps)) / (2 * eps)
    assert abs(gh - fdh) <= REL * max(1.0, abs(fdh)), (gh, fdh)


def test_h_fit_by_gradient_descent_lowers_error(torch_cuda, gnlm_lib):
    """Fit h against the clean phantom with the adjoint's dL/dh (L = MSE)."""
    torch = torch_cuda
    noisy, clean = phantom.ellipsoid_phantom((24, 32, 40), n_ellipsoids=6, sigma=0.05, seed=11)
    x = torch.from_numpy(noisy).cuda()
    c = torch.from_numpy(clean).cuda()
    h = 0.02
    losses = []
    for _ in range(8):
        out, zs = gnlm_lib.nlm3d_forward(x, 3, 1, h, return_zsum=True)
        diff = out - c
        losses.append(float((diff * diff).mean()))
        gout = 2.0 * diff / diff.numel()
        _, hg = gnlm_lib.nlm3d_adjoint(x, out, zs, gout, 3, 1, h)
        h = max(1e-3, h - 0.004 * float(np.sign(hg.item())))  # normalised step
    assert losses[-1] < losses[0]


def test_adjoint_128cubed_against_fp64_finite_differences(torch_cuda, gnlm_lib):
    """The differentiable workload: 128^3 (ellipsoid phantom, sigma 0.05), search 7^3,
    patch 3^3, h 0.05, upstream gradient i.i.d. N(0, 1).  dL/dv on 256 voxels (corners,
    faces, random) and dL/dh against FP64 central differences: only the outputs within
    sr + pr of a perturbed voxel (its REFLECT_101 images included) are re-evaluated,
    and dL/dh comes from two full FP64 forwards.  The FP32 kernels are held to 2e-4 of
    the gradient scale, the FP64 oracle adjoint to 1e-6 (relative)."""
    shape, sr, pr, h = (128, 128, 128), 3, 1, 0.05
    v, _ = phantom.ellipsoid_phantom(shape, n_ellipsoids=16, sigma=0.05, seed=4)
    g = np.random.default_rng(5).standard_normal(shape)
    gin, hg, out = _run(torch_cuda, gnlm_lib, v, sr, pr, h, g)
    vox = O.fd_sample_voxels(shape, 256, seed=6)
    assert len(set(vox)) == 256
    fd = O.fd_voxel_grad(v, sr, pr, h, g, vox, eps=1e-5)
    fdh = O.fd_h_grad(v, sr, pr, h, g, eps=1e-6)
    scale = float(np.abs(fd).max())
    gpu = np.array([gin[i] for i in vox], np.float64)
    rel_v = float(np.abs(gpu - fd).max()) / scale
    rel_h = abs(hg - fdh) / abs(fdh)
    rgin, rhg, rout = O.nlm3d_adjoint(v, sr, pr, h, g)
    ora = np.array([rgin[i] for i in vox])
    orel_v = float(np.abs(ora - fd).max()) / scale
    orel_h = abs(rhg - fdh) / abs(fdh)
    print(f"128^3 adjoint vs FP64 FD: GPU dL/dv {rel_v:.2e}, dL/dh {rel_h:.2e}; "
          f"FP64 oracle dL/dv {orel_v:.2e}, dL/dh {orel_h:.2e}")
    assert orel_v <= 1e-6 and orel_h <= 1e-6
    assert rel_v <= REL and rel_h <= REL
    assert float(np.abs(out - rout).max()) <= 1e-5
    assert gnlm_lib.device_status() == (0, 0)
