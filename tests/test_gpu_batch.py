"""GPU tests of the batched form (one persistent, CUDA-graph-captured launch over
volumes of uneven sizes, search radii and h), against the FP64 oracle and the
single-volume path."""
import numpy as np
import pytest

import oracle as O
from gnlm import phantom

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _volumes(torch, specs):
    vols, hosts = [], []
    for s in specs:
        v, _ = phantom.ellipsoid_phantom(s["shape"], n_ellipsoids=6, sigma=s["sigma"],
                                         seed=s["seed"], radii=(2.0, 10.0))
        hosts.append(v)
        vols.append((torch.from_numpy(v).cuda(), s["sr"], 1, s["h"]))
    return vols, hosts


SPECS = [dict(shape=(32, 48, 64), sigma=0.05, h=0.05, sr=3, seed=1),
         dict(shape=(20, 33, 47), sigma=0.08, h=0.08, sr=5, seed=2),
         dict(shape=(9, 17, 95), sigma=0.02, h=0.02, sr=3, seed=3),
         dict(shape=(40, 24, 30), sigma=0.1, h=0.1, sr=5, seed=4),
         dict(shape=(5, 6, 7), sigma=0.05, h=0.05, sr=2, seed=5),
         dict(shape=(16, 64, 33), sigma=0.03, h=0.03, sr=1, seed=6),
         dict(shape=(12, 20, 28), sigma=0.06, h=0.06, sr=4, seed=7)]


def test_batch_every_variant_matches_oracle(torch_cuda, gnlm_lib):
    torch = torch_cuda
    vols, hosts = _volumes(torch, SPECS)
    plan = gnlm_lib.BatchPlan(vols, with_zsum=True)
    refs = [O.nlm3d(h, s["sr"], 1, s["h"], dtype=np.float64, return_z=True)
            for h, s in zip(hosts, SPECS)]
    try:
        for var in range(gnlm_lib.BatchPlan.N_VARIANTS):
            plan.set_variant(var)
            for o in plan.outputs:
                o.fill_(float("nan"))
            plan.run()
            torch.cuda.synchronize()
            for k, (o, zs) in enumerate(zip(plan.outputs, plan.zsums)):
                ro, rz = refs[k]
                assert np.abs(o.cpu().numpy() - ro).max() <= TOL, (var, k)
                assert np.abs(zs.cpu().numpy() / rz - 1).max() <= TOL, (var, k)
    finally:
        plan.close()
    assert gnlm_lib.device_status() == (0, 0)


def test_batch_replay_is_deterministic_and_matches_single_volume(torch_cuda, gnlm_lib):
    torch = torch_cuda
    vols, _ = _volumes(torch, SPECS[:4])
    plan = gnlm_lib.BatchPlan(vols)
    try:
        a = [o.clone() for o in plan.run()]
        b = [o.clone() for o in plan.run()]
        torch.cuda.synchronize()
        for x, y in zip(a, b):
            assert torch.equal(x, y)
        for (t, sr, pr, h), o in zip(vols, a):
            single = gnlm_lib.nlm3d_forward(t, sr, pr, h)
            assert float((single - o).abs().max()) <= TOL
        info = plan.info()
        assert info["items"] > 0 and info["device_bytes"] > 0
    finally:
        plan.close()


def test_batch_autotune_and_uneven_batch_from_specs(torch_cuda, gnlm_lib):
    """A slice of the 64-volume uneven batch (dims from {32..192}, sr 3 / 5, h = sigma)."""
    torch = torch_cuda
    specs = phantom.batch_specs()
    pick = [specs[i] for i in (0, 1, 2, 40, 41, 42)]
    vols = []
    for s in pick:
        shape = tuple(min(d, 64) for d in s["shape"])  # oracle-checkable sizes
        v, _ = phantom.ellipsoid_phantom(shape, n_ellipsoids=6, sigma=s["sigma"], seed=s["seed"])
        vols.append((torch.from_numpy(v).cuda(), s["sr"], 1, s["h"]))
    plan = gnlm_lib.BatchPlan(vols)
    try:
        best, times = plan.autotune()
        assert 0 <= best < len(times) and times[best] == min(times)
        assert plan.info()["variant"] == best
        plan.run()
        torch.cuda.synchronize()
        for (t, sr, pr, h), o in zip(vols, plan.outputs):
            ref = O.nlm3d(t.cpu().numpy(), sr, 1, h, dtype=np.float64)
            assert np.abs(o.cpu().numpy() - ref).max() <= TOL
    finally:
        plan.close()


def test_batch_rejects_unsupported(torch_cuda, gnlm_lib):
    torch = torch_cuda
    x = torch.zeros((8, 8, 8), device="cuda")
    with pytest.raises(gnlm_lib.NLMError) as ei:
        gnlm_lib.BatchPlan([(x, 3, 2, 0.05)])
    assert ei.value.code == gnlm_lib.NLM_ERR_UNSUPPORTED


def test_one_shot_batched_forward_equals_plan(torch_cuda, gnlm_lib):
    """nlm3d_forward_batched (plan built, run once, freed) gives the plan's bits and
    rejects what nlm3d_batch_create rejects."""
    torch = torch_cuda
    vols, hosts = _volumes(torch, SPECS[:5])
    plan = gnlm_lib.BatchPlan(vols)
    try:
        ref = [o.clone() for o in plan.run()]
        torch.cuda.synchronize()
    finally:
        plan.close()
    outs = gnlm_lib.nlm3d_forward_batched(vols)
    for o, r in zip(outs, ref):
        assert torch.equal(o, r)
    with pytest.raises(gnlm_lib.NLMError) as ei:
        gnlm_lib.nlm3d_forward_batched([(vols[0][0], 3, 2, 0.05)])
    assert ei.value.code == gnlm_lib.NLM_ERR_UNSUPPORTED
    assert gnlm_lib.device_status() == (0, 0)
