"""Continuous-batching serving loop on the GPU, through the native pool
(mo_pool_*, the product) and the Python engine that restates its schedule
over the same kernels (kept as the tests' reference schedule).

* Every request's result is bit-identical alone and inside the mixed stream
  (each pair's arithmetic depends only on its own state).
* Results match the single-pair fused loop over the GPU pyDeform, and the
  saturated and Poisson-paced runs give the same results.
* A malformed request fails alone without disturbing the others.
"""
import numpy as np
import pytest
import torch

from meshode_gb300 import fused, meshgen, pool, serving
from meshode_gb300 import pyDeform as PD

pytestmark = pytest.mark.gpu


def _stream(n=10, seed=21):
    specs = meshgen.serving_requests(n=n, seed=seed, rate=400.0, steps=60, v_range=(300, 3000),
                                     t_range=(500, 8000), grids=(16, 32))
    meshes = [meshgen.request_meshes(s) for s in specs]
    return specs, meshes


def _fresh(reqs):
    return [serving.Request(r.id, r.srcV, r.srcF, r.tarV, r.tarF, N=r.N, steps=r.steps, arrival=r.arrival)
            for r in reqs]


def _engine(kind, **kw):
    return pool.NativePool(**kw) if kind == "native" else serving.ServingEngine(**kw)


@pytest.mark.parametrize("kind", ["native", "python"])
def test_alone_vs_mix_and_realtime(cuda, kind):
    specs, meshes = _stream()
    base = serving.requests_from_meshes(meshes, specs, device=None, pin=True)
    eng = _engine(kind, group_steps=8, max_building=3)
    mix = _fresh(base)
    eng.run(mix)
    assert all(r.error is None for r in mix)
    paced = _fresh(base)
    eng.run(paced, realtime=True)
    for a, b in zip(mix, paced):
        assert torch.equal(a.out, b.out)
        assert b.latency is not None and b.latency > 0
    for r in (mix[0], mix[3], mix[-1]):
        solo = _fresh([r])
        _engine(kind, group_steps=5).run(solo)
        assert torch.equal(solo[0].out, r.out)
        assert torch.equal(solo[0].out_normalized, r.out_normalized)


@pytest.mark.parametrize("kind", ["native", "python"])
def test_serving_matches_fused_fit(cuda, kind):
    specs, meshes = _stream(n=3, seed=5)
    reqs = serving.requests_from_meshes(meshes, specs, device=cuda)
    src_before = [r.srcV.clone() for r in reqs]
    _engine(kind, group_steps=7).run(reqs)
    for r, (Vs, Fs, Vt, Ft), v0 in zip(reqs, meshes, src_before):
        assert torch.equal(r.srcV, v0), "device-resident inputs must not be modified"
        pid = PD.InitializeDeformTemplate(torch.from_numpy(Vt), torch.from_numpy(Ft), 0, r.N)
        V = torch.from_numpy(Vs.copy()).to(cuda)
        PD.NormalizeByTemplate(V, pid)
        PD.StoreRigidityInformation(V, torch.from_numpy(Fs).to(cuda), pid)
        out, _ = fused.fused_fit(pid, V, r.steps, group_steps=9)
        assert torch.equal(out, r.out_normalized)
        den = out.clone()
        PD.DenormalizeByTemplate(den, pid)
        assert torch.equal(den.cpu(), r.out.cpu())


@pytest.mark.parametrize("kind", ["native", "python"])
def test_bad_request_is_isolated(cuda, kind):
    specs, meshes = _stream(n=4, seed=8)
    reqs = serving.requests_from_meshes(meshes, specs, device=None, pin=True)
    bad = reqs[1]
    F = bad.srcF.clone()
    F[0, 0] = 10 ** 7
    reqs[1] = serving.Request(bad.id, bad.srcV, F, bad.tarV, bad.tarF, N=bad.N, steps=bad.steps)
    _engine(kind, group_steps=8).run(reqs)
    assert reqs[1].error is not None and reqs[1].out is None
    for i in (0, 2, 3):
        assert reqs[i].error is None and reqs[i].out is not None


def test_admission_respects_budget(cuda):
    specs, meshes = _stream(n=6, seed=9)
    reqs = serving.requests_from_meshes(meshes, specs, device=None, pin=True)
    one = max(serving.estimate_bytes(r.srcV.shape[0], r.srcF.shape[0], r.tarV.shape[0], r.tarF.shape[0], r.N)
              for r in reqs)
    eng = serving.ServingEngine(group_steps=8, hbm_budget_bytes=int(one * 1.5))
    eng.run(reqs)
    assert all(r.out is not None for r in reqs)
    assert eng.peak_in_use <= int(one * 1.5)
