"""The oracle's FP64 adjoint against an independent reference gradient: the same NLM
written as torch float64 operations on the CPU (torch's reflect padding is REFLECT_101,
gfedcb|abcdefgh|gfedcba) and differentiated by torch.autograd.  No GPU is used.

Forward restated from the reference's arithmetic (3DNLM/main.cu:59-61 squared
differences, :108-109 w = exp(-(D/P)/h^2) with the centre offset included, :125
out = sum w v / sum w); the REFLECT_101 borders follow 3DNLM/nlm.cpp:36-61 on every axis.
"""
import itertools

import numpy as np
import pytest

import oracle as O
from gnlm import phantom

torch = pytest.importorskip("torch")


def _nlm3d_torch(v, sr, pr, h):
    """Direct-form 3D NLM of a float64 tensor [Z, Y, X] (differentiable in v and h)."""
    F = torch.nn.functional
    H = sr + pr
    K = 2 * pr + 1
    P = K ** 3
    Z, Y, X = v.shape
    vp = F.pad(v[None, None], (H,) * 6, mode="reflect")[0, 0]
    ref = vp[H - pr:H + Z + pr, H - pr:H + Y + pr, H - pr:H + X + pr]
    num = torch.zeros_like(v)
    zs = torch.zeros_like(v)
    for oz, oy, ox in itertools.product(range(-sr, sr + 1), repeat=3):
        cand = vp[H - pr + oz:H + Z + pr + oz, H - pr + oy:H + Y + pr + oy,
                  H - pr + ox:H + X + pr + ox]
        d = (ref - cand) ** 2
        D = F.avg_pool3d(d[None, None], kernel_size=K, stride=1)[0, 0] * P
        w = torch.exp(-(D / P) / h ** 2)
        num = num + w * vp[H + oz:H + oz + Z, H + oy:H + oy + Y, H + ox:H + ox + X]
        zs = zs + w
    return num / zs


@pytest.mark.parametrize("shape,sr,pr", [((6, 7, 8), 1, 1), ((7, 8, 9), 2, 1), ((9, 8, 10), 1, 2),
                                         ((8, 9, 9), 3, 1)])
def test_oracle_adjoint_matches_torch_autograd(shape, sr, pr):
    v, _ = phantom.ellipsoid_phantom(shape, n_ellipsoids=3, sigma=0.05, seed=sum(shape) + sr,
                                     radii=(1.5, 4.0))
    v = v.astype(np.float64)
    h0 = 0.07
    g = np.random.default_rng(11 + sr).standard_normal(v.shape)

    vt = torch.tensor(v, dtype=torch.float64, requires_grad=True)
    ht = torch.tensor(h0, dtype=torch.float64, requires_grad=True)
    out_t = _nlm3d_torch(vt, sr, pr, ht)
    (out_t * torch.tensor(g)).sum().backward()

    gin, gh, out = O.nlm3d_adjoint(v, sr, pr, h0, g)
    # forward: the oracle's direct FP64 form and the torch restatement
    assert np.abs(out - out_t.detach().numpy()).max() <= 1e-12
    # reference gradients: dL/dv (folded back through REFLECT_101 by the pad's
    # backward) and dL/dh
    ref_gin = vt.grad.numpy()
    assert np.abs(gin - ref_gin).max() <= 1e-9 * max(1.0, np.abs(ref_gin).max())
    assert abs(gh - float(ht.grad)) <= 1e-9 * max(1.0, abs(float(ht.grad)))
