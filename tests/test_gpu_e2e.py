"""End to end on the plain rigid-deform workload (ico-5 source, displaced ico-5
target, 64^3 grid, Adam lr 1e-3): the fused GPU loop and the plain GPU loop
(the reference's rigid_deform.py loop over the GPU pyDeform) against the CPU
oracle loop with its own FP64 distance field.  Bar: the final meshes' Chamfer
distances to the target agree within 1e-4 (unit-cube units).
"""
import numpy as np
import pytest
import torch

from meshode_gb300 import fused, layers, meshgen, metrics
from meshode_gb300 import pyDeform as PD

pytestmark = pytest.mark.gpu

CHAMFER_TOL = 1e-4


@pytest.fixture(scope="module")
def workload():
    Vs, Fs, Vt, Ft = meshgen.rigid_pair_ico5(seed=1)
    return Vs, Fs, Vt, Ft


def _target_normalised(orc, Vt):
    scale, trans = orc.normalize_params(Vt)
    return orc.normalized_double(Vt, scale, trans)


@pytest.mark.parametrize("steps", [300, 1000])
def test_rigid_fit_chamfer(cuda, orc, workload, steps):
    Vs, Fs, Vt, Ft = workload
    N = 64
    # oracle: CPU DF in FP64 + the reference's loop with torch.optim.Adam on the CPU
    opid = orc.InitializeDeformTemplate(Vt, Ft, 0, N)
    Vo = torch.from_numpy(Vs.copy())
    orc.NormalizeByTemplate(Vo, opid)
    orc.StoreRigidityInformation(Vo, torch.from_numpy(Fs), opid)
    ref, _ = orc.rigid_fit(Vo, torch.from_numpy(Fs), opid, steps)
    # GPU fused loop
    pid = PD.InitializeDeformTemplate(torch.from_numpy(Vt), torch.from_numpy(Ft), 0, N)
    Vg = torch.from_numpy(Vs.copy()).to(cuda)
    PD.NormalizeByTemplate(Vg, pid)
    assert torch.equal(Vg.cpu(), Vo), "NormalizeByTemplate differs from the oracle"
    PD.StoreRigidityInformation(Vg, torch.from_numpy(Fs).to(cuda), pid)
    out, _ = fused.fused_fit(pid, Vg, steps)
    Tn = _target_normalised(orc, Vt)
    c_ref = metrics.chamfer(ref.numpy(), Fs, Tn, Ft, samples=20000)
    c_gpu = metrics.chamfer(out.cpu().numpy(), Fs, Tn, Ft, samples=20000)
    assert abs(c_gpu - c_ref) <= CHAMFER_TOL, (c_gpu, c_ref)
    # the two fitted meshes themselves are close
    assert metrics.chamfer(out.cpu().numpy(), Fs, ref.numpy(), Fs, samples=0) <= CHAMFER_TOL


def test_plain_gpu_loop_matches(cuda, orc, workload):
    """The reference's loop verbatim (RigidLossLayer + torch.optim.Adam) on
    CUDA tensors, against the fused loop.  torch's CUDA Adam rounds
    differently from the fused update, and the distance lookup is
    discontinuous (the 0.2 cutoff, cell boundaries) and its gradient jumps
    across cell faces, so vertices sitting on such a face take different
    branches and drift by up to a few learning-rate steps, dragging their
    neighbours through the edge terms; the median vertex must agree to 1e-5
    and the meshes within the Chamfer tolerance."""
    Vs, Fs, Vt, Ft = workload
    steps = 200
    src_V = torch.from_numpy(Vs.copy()).to(cuda)
    src_F = torch.from_numpy(Fs).to(cuda)
    layer = layers.RigidLossLayer(src_V, src_F, torch.from_numpy(Vt), torch.from_numpy(Ft))
    V0 = src_V.clone()
    P = torch.nn.Parameter(src_V)
    opt = torch.optim.Adam([P], lr=1e-3)
    for _ in range(steps):
        opt.zero_grad()
        loss = layer(P, src_F)
        loss.backward()
        opt.step()
    out, _ = fused.fused_fit(int(layer.param_id), V0, steps)
    err = (out - P.detach()).abs().amax(1)
    assert torch.median(err).item() <= 1e-5, torch.median(err).item()
    assert err.max().item() <= 10 * 1e-3, err.max().item()
    assert metrics.chamfer(out.cpu().numpy(), Fs, P.detach().cpu().numpy(), Fs, samples=0) <= CHAMFER_TOL
    # Finalize denormalises in place
    Vf = P.detach().clone()
    layers.Finalize(Vf, layer.param_id)
    Vn = Vf.clone()
    PD.NormalizeByTemplate(Vn, int(layer.param_id))
    assert (Vn - P.detach()).abs().max().item() < 1e-5
