"""The autotuner's knobs change speed only: every LBVH packet shape and the
brute force give the same grid bit for bit, every step layout and tile
width the same trajectory, and the serving loop's results are identical with
and without the tuner."""
import ctypes

import numpy as np
import pytest
import torch

from meshode_gb300 import _lib as L
from meshode_gb300 import autotune, fused, meshgen, serving
from meshode_gb300 import pyDeform as PD

pytestmark = pytest.mark.gpu


def test_packet_shapes_and_methods_agree(cuda):
    rng = np.random.Generator(np.random.PCG64(2))
    V, F = meshgen.icosphere(4)
    T = torch.from_numpy(meshgen.displace(V, rng).astype(np.float32)).to(cuda)
    Fd = torch.from_numpy(F.astype(np.int32)).to(cuda)
    s = L.stream_ptr()
    bbox = torch.empty(6, dtype=torch.int32, device=cuda)
    prm = torch.empty(4, dtype=torch.float64, device=cuda)
    L.call("mo_bbox", L.ptr(T), T.shape[0], L.ptr(bbox), s)
    L.call("mo_norm_params", L.ptr(bbox), L.ptr(prm), s)
    grids = []
    N = 37
    cands = [(L.MO_DF_LBVH, p) for p in autotune.PACKETS.values()] + [(L.MO_DF_BRUTE, 0)]
    for method, packet in cands:
        g = torch.empty(N ** 3, dtype=torch.float32, device=cuda)
        opt = L.MoDfOptions(method, packet)
        L.call("mo_df_build_ex", L.ptr(T), T.shape[0], L.ptr(Fd), Fd.shape[0], N, L.ptr(prm), ctypes.byref(opt),
               None, 0, L.ptr(g), None, s)
        grids.append(g)
    for g in grids[1:]:
        assert torch.equal(g, grids[0])


def test_layouts_and_tile_widths_agree(cuda):
    rng = np.random.Generator(np.random.PCG64(3))
    V, F = meshgen.icosphere(3)
    T = meshgen.displace(V, rng).astype(np.float32)
    pid = PD.InitializeDeformTemplate(torch.from_numpy(T), torch.from_numpy(F.astype(np.int32)), 0, 30,
                                      layout=L.MO_LAYOUT_LINEAR)
    Vs = torch.from_numpy(V.astype(np.float32)).to(cuda)
    PD.NormalizeByTemplate(Vs, pid)
    PD.StoreRigidityInformation(Vs, torch.from_numpy(F.astype(np.int32)).to(cuda), pid)
    P = PD.GetParams(pid)
    outs = []
    for lay in (L.MO_LAYOUT_LINEAR, L.MO_LAYOUT_CELL, L.MO_LAYOUT_BRICK4):
        g = torch.empty(L.lib().mo_grid_bytes(30, lay) // 4, dtype=torch.float32, device=cuda)
        L.call("mo_grid_relayout", L.ptr(P.grid_linear), 30, lay, L.ptr(g), L.stream_ptr())
        for spt in (1, 4, 8):
            pr = fused.Pair(g, 30, lay, Vs, P.edge.csr, P.edge.nh, P.edge.rest, 40, slices_per_tile=spt)
            runner = fused.StepGroupRunner(cuda, 1, pr.ntiles, group_steps=8)
            while not pr.done:
                runner.upload([pr], [pr.t])
                runner.run_group()
                pr.t = min(pr.steps, pr.t + 8)
            outs.append(pr.positions())
    for o in outs[1:]:
        assert torch.equal(o, outs[0])


def test_serving_with_tuner_is_identical(cuda, tmp_path):
    specs = meshgen.serving_requests(n=6, seed=31, steps=30, v_range=(500, 4000), t_range=(1000, 20000),
                                     grids=(24, 40))
    meshes = [meshgen.request_meshes(s) for s in specs]
    base = serving.requests_from_meshes(meshes, specs, device=cuda)

    def fresh():
        return [serving.Request(r.id, r.srcV, r.srcF, r.tarV, r.tarF, N=r.N, steps=r.steps) for r in base]

    tuner = autotune.Autotuner(cache_path=str(tmp_path / "tune.json"))
    tuner.tune_for(base)
    assert (tmp_path / "tune.json").exists()
    a = fresh()
    serving.ServingEngine(group_steps=10, results_to_host=False).run(a)
    b = fresh()
    serving.ServingEngine(group_steps=10, results_to_host=False, autotuner=tuner).run(b)
    for x, y in zip(a, b):
        assert torch.equal(x.out, y.out)
    reloaded = autotune.Autotuner(cache_path=str(tmp_path / "tune.json"))
    assert reloaded.table == tuner.table


def test_counting_build_same_grid_and_counts(cuda):
    """mo_df_build_count (the measurement build of the bench's DF roofline)
    gives every packet shape's grid bit for bit, with and without the band;
    the brute force counts N^3 * triangles tests and no visits; the LBVH
    walks count visits and far fewer tests; counts accumulate."""
    rng = np.random.Generator(np.random.PCG64(3))
    V, F = meshgen.icosphere(4)
    T = torch.from_numpy(meshgen.displace(V, rng).astype(np.float32)).to(cuda)
    Fd = torch.from_numpy(F.astype(np.int32)).to(cuda)
    s = L.stream_ptr()
    bbox = torch.empty(6, dtype=torch.int32, device=cuda)
    prm = torch.empty(4, dtype=torch.float64, device=cuda)
    L.call("mo_bbox", L.ptr(T), T.shape[0], L.ptr(bbox), s)
    L.call("mo_norm_params", L.ptr(bbox), L.ptr(prm), s)
    N = 29
    nf = Fd.shape[0]
    for band in (0.0, L.lib().mo_df_loss_band(N)):
        cands = [(L.MO_DF_LBVH, p) for p in autotune.PACKETS.values()] + [(L.MO_DF_BRUTE, 0)]
        for method, packet in cands:
            opt = L.MoDfOptions(method, packet, band)
            g0 = torch.empty(N ** 3, dtype=torch.float32, device=cuda)
            g1 = torch.full((N ** 3,), float("nan"), dtype=torch.float32, device=cuda)
            c = torch.zeros(2, dtype=torch.int64, device=cuda)
            L.call("mo_df_build_ex", L.ptr(T), T.shape[0], L.ptr(Fd), nf, N, L.ptr(prm), ctypes.byref(opt),
                   None, 0, L.ptr(g0), None, s)
            L.call("mo_df_build_count", L.ptr(T), T.shape[0], L.ptr(Fd), nf, N, L.ptr(prm), ctypes.byref(opt),
                   None, 0, L.ptr(g1), None, L.ptr(c), s)
            assert torch.equal(g0, g1), (method, packet, band)
            visits, tests = c.cpu().tolist()
            if method == L.MO_DF_BRUTE:
                assert (visits, tests) == (0, N ** 3 * nf)
            else:
                assert visits > 0 and 0 < tests < N ** 3 * nf // 20, (packet, visits, tests)
                L.call("mo_df_build_count", L.ptr(T), T.shape[0], L.ptr(Fd), nf, N, L.ptr(prm),
                       ctypes.byref(opt), None, 0, L.ptr(g1), None, L.ptr(c), s)
                assert c.cpu().tolist() == [2 * visits, 2 * tests]
