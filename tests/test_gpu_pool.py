"""The native serving pool (mo_pool_* in libmeshode.so) on the GPU.

* Results (DF built with the loss-preserving band) are bit-identical to the
  Python serving engine's on exact grids, to each request
  run alone, to the single-pair fused loop over the GPU pyDeform, with and
  without CUDA graphs, under Poisson pacing, and under a tile budget that
  forces requests to wait for room.
* The loss a request reports is the fused loop's last-step loss.
* A malformed mesh fails its request only; host-side rejections raise.
* Admission keeps the byte estimate under the budget.
"""
import pytest
import torch

from meshode_gb300 import _lib as L
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


def test_pool_matches_python_engine_alone_and_paced(cuda):
    specs, meshes = _stream()
    base = serving.requests_from_meshes(meshes, specs, device=None, pin=True)
    ref = _fresh(base)
    # the Python engine on exact grids; the pool on the loss-preserving band
    serving.ServingEngine(group_steps=8, max_building=3, df_band=0.0).run(ref)
    P = pool.NativePool(group_steps=8, max_building=3)
    mix = _fresh(base)
    P.run(mix)
    assert all(r.error is None for r in mix)
    for a, b in zip(ref, mix):
        assert torch.equal(a.out, b.out)
        assert torch.equal(a.out_normalized, b.out_normalized)
    paced = _fresh(base)
    P.run(paced, realtime=True)
    for a, b in zip(mix, paced):
        assert torch.equal(a.out, b.out)
        assert b.latency is not None and b.latency > 0
    gbs, secs = P.step_roofline()
    assert gbs > 0 and secs > 0
    assert P.launches > 0
    P.close()
    for r in (mix[0], mix[-1]):
        solo = _fresh([r])
        pool.NativePool(group_steps=5).run(solo)
        assert torch.equal(solo[0].out, r.out)


def test_pool_matches_fused_fit_and_loss(cuda):
    specs, meshes = _stream(n=3, seed=5)
    reqs = serving.requests_from_meshes(meshes, specs, device=cuda)
    src_before = [r.srcV.clone() for r in reqs]
    pool.NativePool(group_steps=7, results_to_host=False).run(reqs)
    for r, (Vs, Fs, Vt, Ft), v0 in zip(reqs, meshes, src_before):
        assert torch.equal(r.srcV, v0), "device-resident inputs must not be modified"
        pid = PD.InitializeDeformTemplate(torch.from_numpy(Vt), torch.from_numpy(Ft), 0, r.N)
        V = torch.from_numpy(Vs.copy()).to(cuda)
        PD.NormalizeByTemplate(V, pid)
        PD.StoreRigidityInformation(V, torch.from_numpy(Fs).to(cuda), pid)
        out, losses = fused.fused_fit(pid, V, r.steps, group_steps=9, record_loss=True)
        assert torch.equal(out, r.out_normalized)
        den = out.clone()
        PD.DenormalizeByTemplate(den, pid)
        assert torch.equal(den, r.out)
        assert r.loss == float(losses[-1])
        PD.ReleaseTemplate(pid)


@pytest.mark.parametrize("use_graph", [False, True])
def test_pool_tile_budget_and_graph(cuda, use_graph):
    specs, meshes = _stream(n=6, seed=13)
    base = serving.requests_from_meshes(meshes, specs, device=None, pin=True)
    ref = _fresh(base)
    pool.NativePool(group_steps=6).run(ref)
    most = max((int(r.srcV.shape[0]) + 255) // 256 for r in base)  # tiles of the largest request
    tight = _fresh(base)
    P = pool.NativePool(group_steps=6, max_tiles=most, use_graph=use_graph)
    P.run(tight)
    for a, b in zip(ref, tight):
        assert b.error is None
        assert torch.equal(a.out, b.out)


def test_pool_bad_request_is_isolated(cuda):
    specs, meshes = _stream(n=4, seed=8)
    reqs = serving.requests_from_meshes(meshes, specs, device=None, pin=True)
    bad = reqs[1]
    F = bad.srcF.clone()
    F[0, 0] = 10 ** 7
    reqs[1] = serving.Request(bad.id, bad.srcV, F, bad.tarV, bad.tarF, N=bad.N, steps=bad.steps)
    rej = reqs[2]
    reqs[2] = serving.Request(rej.id, rej.srcV, rej.srcF, rej.tarV, rej.tarF, N=1, steps=rej.steps)
    pool.NativePool(group_steps=8).run(reqs)
    assert reqs[1].error and "invalid mesh" in reqs[1].error and reqs[1].out is None
    assert reqs[2].error and "resolution" in reqs[2].error and reqs[2].out is None
    for i in (0, 3):
        assert reqs[i].error is None and reqs[i].out is not None


def test_pool_admission_respects_budget(cuda):
    specs, meshes = _stream(n=6, seed=9)
    reqs = serving.requests_from_meshes(meshes, specs, device=None, pin=True)
    for mode in (L.MO_DF_FULL, L.MO_DF_ON_DEMAND):
        one = max(serving.estimate_bytes(r.srcV.shape[0], r.srcF.shape[0], r.tarV.shape[0], r.tarF.shape[0], r.N,
                                         df_mode=mode) for r in reqs)
        P = pool.NativePool(group_steps=8, hbm_budget_bytes=int(one * 1.5), df_mode=mode)
        part = _fresh(reqs)
        P.run(part)
        assert all(r.out is not None for r in part)
        assert 0 < P.peak_in_use <= int(one * 1.5)
        P.close()


def test_pool_steady_state(cuda):
    specs, meshes = _stream(n=5, seed=3)
    reqs = serving.requests_from_meshes(meshes, specs, device=cuda)
    for r in reqs:
        r.steps = 1000
    P = pool.NativePool(group_steps=10)
    t, nbytes, nv = P.steady_state(reqs, groups=2)
    assert t > 0 and nv == sum(int(r.srcV.shape[0]) for r in reqs)
    assert nbytes == sum(104 * int(r.srcV.shape[0]) + 44 * 3 * int(r.srcF.shape[0]) for r in reqs)
    P.close()


def test_pool_c_abi_direct(cuda):
    """The pool driven through the C ABI alone (as a C host would): host
    inputs, no output buffers, mo_pool_wait, then mo_pool_result into host
    arrays; equal to the facade's results."""
    import ctypes
    import numpy as np
    from meshode_gb300 import _lib as L
    specs, meshes = _stream(n=3, seed=17)
    base = serving.requests_from_meshes(meshes, specs, device=None, pin=True)
    ref = _fresh(base)
    pool.NativePool(group_steps=9).run(ref)
    lib = L.lib()
    cfg = L.MoPoolConfig(max_pairs=8, max_tiles=4096, group_steps=9, use_graph=1, layout=L.MO_LAYOUT_CELL)
    h = ctypes.c_void_p()
    L.check(lib.mo_pool_create(ctypes.byref(cfg), ctypes.byref(h)), "create")
    arrays = [[np.ascontiguousarray(a) for a in m] for m in meshes]
    ids = []
    for (Vs, Fs, Vt, Ft), r in zip(arrays, base):
        q = L.MoRequest(srcV=Vs.ctypes.data, srcF=Fs.ctypes.data, tarV=Vt.ctypes.data, tarF=Ft.ctypes.data,
                        nv=len(Vs), nf=len(Fs), ntv=len(Vt), ntf=len(Ft), inputs_on_host=1, N=r.N, steps=r.steps,
                        w_edge=1.0, lr=1e-3, layout=-1, df_band=-1.0)
        rid = ctypes.c_int64()
        L.check(lib.mo_pool_submit(h, ctypes.byref(q), ctypes.byref(rid)), "submit")
        ids.append(rid.value)
    L.check(lib.mo_pool_wait(h), "wait")
    st = L.MoPoolStats()
    L.check(lib.mo_pool_stats(h, ctypes.byref(st)), "stats")
    assert st.submitted == 3 and st.done == 3 and st.failed == 0 and st.active == 0 and st.fused_launches > 0
    got = (ctypes.c_int64 * 8)()
    n = ctypes.c_int()
    L.check(lib.mo_pool_completed(h, got, 8, ctypes.byref(n)), "completed")
    assert sorted(got[:n.value]) == sorted(ids)
    for rid, r, (Vs, _, _, _) in zip(ids, ref, arrays):
        out = np.empty_like(Vs)
        loss = ctypes.c_double()
        L.check(lib.mo_pool_result(h, rid, out.ctypes.data, None, 1, ctypes.byref(loss)), "result")
        assert np.array_equal(out, r.out.numpy())
        assert loss.value == r.loss
        state = ctypes.c_int32()
        L.check(lib.mo_pool_state(h, rid, ctypes.byref(state)), "state")
        assert state.value == L.MO_REQ_DONE
        L.check(lib.mo_pool_release(h, rid), "release")
    assert lib.mo_pool_state(h, ids[0], ctypes.byref(state)) == L.MO_ERR_INVALID
    L.check(lib.mo_pool_trim(h, 0), "trim")
    L.check(lib.mo_pool_destroy(h), "destroy")
