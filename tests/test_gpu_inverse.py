"""The inverse_deform loop (src/python/inverse_deform.py: RigidLossLayer * 10
+ ReverseLossLayer, torch Adam) on the GPU against the same loop on the
oracle (CPU pyDeform restatement on the same grid, cKDTree reverse loss,
torch CPU Adam), and the command-line program end to end."""
import numpy as np
import pytest
import torch

from meshode_gb300 import cli, layers, meshgen, metrics, objio
from meshode_gb300 import pyDeform as PD

pytestmark = pytest.mark.gpu


def _meshes(seed=6):
    rng = np.random.Generator(np.random.PCG64(seed))
    V, F = meshgen.icosphere(3)
    T = meshgen.displace(V, rng)
    return (V * 0.8).astype(np.float32), F.astype(np.int32), T.astype(np.float32), F.astype(np.int32)


def test_inverse_loop_vs_oracle(cuda, orc):
    Vs, Fs, Vt, Ft = _meshes()
    K = 30
    out_gpu, iters = cli.inverse_fit(Vs, Fs, Vt, Ft, steps=K, log=lambda *_: None)
    assert iters == K
    # the oracle on the GPU's own 64^3 grid (the DF build is tested on its own)
    pid = PD.InitializeDeformTemplate(torch.from_numpy(Vt), torch.from_numpy(Ft), 0, 64)
    opid = orc.InitializeDeformTemplate(Vt, Ft, 0, 64, grid=PD.GetDistanceField(pid).cpu().numpy())
    sV = torch.from_numpy(Vs.copy())
    orc.NormalizeByTemplate(sV, opid)
    orc.StoreRigidityInformation(sV, torch.from_numpy(Fs), opid)
    tV = torch.from_numpy(Vt.copy())
    orc.NormalizeByTemplate(tV, opid)
    ref = orc.inverse_fit(sV, torch.from_numpy(Fs), tV, opid, K)
    orc.DenormalizeByTemplate(ref, opid)
    diag = float(np.linalg.norm(Vt.max(0) - Vt.min(0)))
    err = np.abs(out_gpu - ref.numpy().astype(np.float64)).max()
    assert err <= 1e-5 * diag, err
    PD.ReleaseTemplate(pid)


def test_inverse_deform_cli(cuda, tmp_path):
    Vs, Fs, Vt, Ft = _meshes(seed=9)
    objio.write_obj(str(tmp_path / "src.obj"), Vs, Fs)
    objio.write_obj(str(tmp_path / "ref.obj"), Vt, Ft)
    out = tmp_path / "out.obj"
    assert cli.main(["inverse_deform", "--steps", "300", str(tmp_path / "src.obj"), str(tmp_path / "ref.obj"),
                     str(out)]) == 0
    Vo, Fo = objio.read_obj(str(out))
    assert Vo.shape == Vs.shape and np.array_equal(Fo, Fs)
    before = metrics.chamfer(Vs.astype(np.float64), Fs, Vt.astype(np.float64), Ft, samples=5000)
    after = metrics.chamfer(Vo, Fs, Vt.astype(np.float64), Ft, samples=5000)
    assert after < 0.7 * before, (before, after)
