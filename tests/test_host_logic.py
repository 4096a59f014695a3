"""Host-side logic that needs no GPU: OBJ reading quirks, argument
validation of the pyDeform mirror, generators, admission accounting,
the Chamfer metric."""
import numpy as np
import pytest
import torch

from meshode_gb300 import fused, meshgen, metrics, objio, serving
from meshode_gb300 import pyDeform as PD


def test_obj_reader_quirks(tmp_path):
    p = tmp_path / "m.obj"
    lines = ["# comment", "v 0 0 0", "v 1.5 0 0", "vn 0 0 1", "v 0 2 0", "v 0 0 3",
             "f 1/1/1 2/2/2 3/3/3", "f  1//1 3//3 4//4 2//2", "", "vt 0 0", "f 4 3 2"]
    p.write_text("\n".join(lines) + "\n" + "v " + "1 " * 200 + "\n" + "v 9 9 9\n")
    V, F = objio.read_obj(str(p))
    assert V.shape == (4, 3) and V[1, 0] == 1.5
    assert F.tolist() == [[0, 1, 2], [0, 2, 3], [3, 2, 1]]   # quads keep 3 corners; long line stops reading


def test_obj_roundtrip(tmp_path):
    V, F = meshgen.icosphere(1)
    p = tmp_path / "o.obj"
    PD.SaveMesh(str(p), torch.from_numpy(V.astype(np.float32)), torch.from_numpy(F.astype(np.int32)))
    V2, F2 = PD.LoadMesh(str(p))
    assert V2.dtype == torch.float32 and F2.dtype == torch.int32
    assert np.abs(V2.numpy() - V).max() < 1e-5 and np.array_equal(F2.numpy(), F)


def test_validation_errors_without_gpu():
    with pytest.raises(RuntimeError):
        PD.DistanceFieldLoss_forward(torch.zeros(5, 3, dtype=torch.float64), 0)
    with pytest.raises(RuntimeError):
        PD.DistanceFieldLoss_backward(torch.zeros(5, 4), 0)
    with pytest.raises(RuntimeError):
        PD.RigidEdgeLoss_forward(torch.zeros(5, 3), torch.zeros(2, 3, dtype=torch.int64), 0)
    with pytest.raises(RuntimeError):
        PD.InitializeDeformTemplate(torch.zeros(5, 3), torch.zeros(0, 3, dtype=torch.int32), 0, 64)
    with pytest.raises(RuntimeError):
        PD.InitializeDeformTemplate(torch.zeros(5, 3), torch.zeros(2, 3, dtype=torch.int32), 0, 1)
    with pytest.raises(FileNotFoundError):
        PD.LoadCadMesh("x.obj")
    with pytest.raises(RuntimeError):
        PD.StoreCadInformation(None, None, None, 0)
    with pytest.raises(RuntimeError):
        PD.CadEdgeLoss_forward(torch.zeros(5, 3), torch.zeros(2, 3, dtype=torch.int32),
                               torch.zeros(1, 3, dtype=torch.int32), 0)


def test_generators():
    V, F = meshgen.icosphere(3)
    assert V.shape == (642, 3) and F.shape == (1280, 3)
    V, F = meshgen.cubesphere(9)
    assert V.shape == (6 * 81 + 2, 3) and F.shape == (12 * 81, 3)
    e = np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]])
    assert len({tuple(x) for x in e}) == len(e)                      # consistently oriented
    assert all((b, a) in {tuple(x) for x in e} for a, b in e[:50])    # closed
    specs = meshgen.serving_requests(n=512)
    nv = np.array([s["nv"] for s in specs])
    nt = np.array([s["nt"] for s in specs])
    assert nv.min() >= 2000 and nv.max() <= 100000 and nt.min() >= 5000 and nt.max() <= 500000
    assert set(s["N"] for s in specs) == {64, 128}
    gaps = np.diff([s["arrival"] for s in specs])
    assert abs(gaps.mean() - 1 / 200.0) < 1e-3
    a = meshgen.serving_requests(n=8, seed=5)
    b = meshgen.serving_requests(n=8, seed=5)
    assert a == b


def test_admission_estimate_and_tiles():
    e1 = serving.estimate_bytes(1000, 2000, 1000, 2000, 64)
    e2 = serving.estimate_bytes(2000, 4000, 1000, 2000, 64)
    e3 = serving.estimate_bytes(1000, 2000, 1000, 2000, 128)
    assert e1 < e2 and e1 < e3
    assert fused.tiles_for(1) == 1 and fused.tiles_for(8) == 1 and fused.tiles_for(9) == 2


def test_chamfer_metric():
    V, F = meshgen.icosphere(2)
    assert metrics.chamfer(V, F, V, F, samples=2000) == pytest.approx(0.0, abs=1e-12)
    d = metrics.chamfer(V, F, V + np.array([0.01, 0, 0]), F, samples=2000)
    assert 0.005 < d <= 0.0101


def test_mesh_utilities_restated():
    from meshode_gb300 import meshops
    V = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [1e-8, 0, 0], [0, 0, 1]], np.float64)
    F = np.array([[0, 1, 2], [3, 1, 2], [0, 0, 4], [2, 1, 0], [0, 1, 4]])
    V2, F2 = meshops.merge_duplex(V, F)
    # vertex 3 truncates onto vertex 0; face [3,1,2] duplicates [0,1,2], [2,1,0] too; [0,0,4] is degenerate
    assert V2.shape[0] == 4 and F2.tolist() == [[0, 1, 2], [0, 1, 3]]
    Vd, Fd = meshops.remove_degenerated(V, np.array([[0, 1, 2], [0, 1, 3], [4, 4, 2]]))
    assert Fd.tolist() == [[0, 1, 2]]
    Vr, Fr = meshops.reflection_symmetrize(V[:3], F[:1])
    assert Vr.shape == (6, 3) and Vr[4, 0] == -1.0 and Fr.tolist() == [[0, 1, 2], [3, 4, 5]]
    Vs, Fs = meshops.subdivide_to(V[:3], F[:1], 10)
    assert Vs.shape[0] >= 10 and Fs.shape[0] == 16


def test_cli_usage_without_gpu(capsys):
    from meshode_gb300 import cli
    assert cli.main(["rigid_deform", "a.obj", "b.obj", "c.obj"]) == 0
    assert "GRID_RESOLUTION" in capsys.readouterr().out
    assert cli.main(["cad_deform"]) == 0
    assert "flow_output" in capsys.readouterr().out
    assert cli.main(["inverse_deform", "a.obj"]) == 0
    assert "inverse_deform.py source.obj" in capsys.readouterr().out


def test_autotune_buckets():
    from meshode_gb300 import autotune
    assert autotune.t_bucket(5000) == 12 and autotune.t_bucket(8192) == 13
    assert autotune.v_bucket(1) == 0 and autotune.v_bucket(100000) == 16


def test_cpu_baseline_strata():
    """bench.py's CPU sample: one request from each of the 12 strata (grid x
    source-vertex tercile x target-triangle half) of the 512-request stream,
    and the stream-weighted estimate (exact for a constant cost; a stratum's
    weight is its share of the stream)."""
    import argparse
    import bench
    specs, _ = bench.make_stream(argparse.Namespace(requests=512, req_steps=500), 5)
    strata = bench.cpu_strata(specs)
    assert len(strata) == 12 and sum(len(v) for v in strata.values()) == 512
    ids = bench.cpu_sample_ids(specs)
    assert len(ids) == 12 and len(set(ids)) == 12
    assert sorted(strata) == [k for k in sorted(strata) if any(i in strata[k] for i in ids)]
    assert abs(bench.stream_mean_seconds(specs, {i: [2.0] for i in ids}) - 2.0) < 1e-12
    # cost proportional to the stratum's index: the estimate is the share-weighted mean
    keys = sorted(strata)
    cost = {i: [float(keys.index(k))] for k in keys for i in ids if i in strata[k]}
    want = sum(len(strata[k]) / 512 * keys.index(k) for k in keys)
    assert abs(bench.stream_mean_seconds(specs, cost) - want) < 1e-12


def test_reference_arm_covers_every_stratum_each_step(monkeypatch, capsys):
    """bench.py --impl reference: every timed step is one pass over all 12
    sampled requests (so a short run is not biased toward the first strata),
    and the reported value is 1 / the stream-weighted mean of their costs."""
    import argparse
    import json
    import bench
    calls = []

    def fake_model(specs, meshes, i, threads, loop_steps=50, voxel_stride=1):
        calls.append((i, voxel_stride))
        return 1.0 + (i % 7), 0.0, 0.0

    monkeypatch.setattr(bench, "cpu_request_model", fake_model)
    monkeypatch.setattr(bench, "run_cpu_port", lambda *a, **k: (0.0, []))
    monkeypatch.setattr(bench, "make_stream", lambda args, seed: (_bench_specs(), [None] * 512))
    args = argparse.Namespace(requests=512, req_steps=500, warmup=1, steps=2, gpus=1)
    bench.reference_arm(args, 1, 0)
    out = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    ids = bench.cpu_sample_ids(_bench_specs())
    assert [c[0] for c in calls] == ids + ids
    assert all(c[1] == bench.REF_VOXEL_STRIDE for c in calls)
    want = 1.0 / bench.stream_mean_seconds(_bench_specs(), {i: [1.0 + (i % 7)] * 2 for i in ids})
    assert abs(out["value"] - want) < 1e-12 and out["impl"] == "reference"
    assert out["cpu_baseline"]["kind"] == "port" and out["e2e"]["h2d_bytes_per_step"] == 0


def _bench_specs():
    from meshode_gb300 import meshgen
    return meshgen.serving_requests(n=512, seed=5, steps=500)
