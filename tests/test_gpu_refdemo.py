"""The reference's own demo pairs, against fixtures made by the reference.

tests/golden/ref_demo_meshes.npz and ref_demo_rigid.npz come from
oracle/_ref (the reference's pyDeform loops compiled unchanged) and the
reference's own RigidLossLayer (src/python/layers/rigid_loss_layer.py) run
over it; tests/golden/gen_ref_fixtures.py made them and
tests/test_ref_pin.py checks them against the reference where it is
mounted.  Here, on the GPU:

* data/target.obj as rigid_deform.py sets it up (64^3): the GPU template's
  transform equals the reference's bit for bit, its grid is within 1e-5 of
  the bounding-box diagonal of the reference's, and NormalizeByTemplate of
  data/source.obj gives the reference's normalised source bit for bit;
* DistanceFieldLoss and RigidEdgeLoss forward/backward through the C ABI on
  the reference's own grid, at the normalised source and at a seeded
  perturbation: the reference's outputs bit for bit (SHA-256 of the bytes);
* the loop of rigid_deform.py:32-39 for 1000 steps, over the GPU layers
  (torch Adam on CUDA) and with the fused step: the Chamfer distance of the
  fitted source to the target within 1e-4 of the reference loop's;
* data/cad-source.obj -> cad-target.obj (``f a//n`` records) through the
  LoadCadMesh pipeline and the graph + reverse-loss loop of
  cad_deform2.py:30-57 on the GPU, against the same loop on the oracle:
  the pipeline's invariants, and Chamfer within 1e-4.
"""
import hashlib
import os

import numpy as np
import pytest
import torch

from meshode_gb300 import _lib as L
from meshode_gb300 import cadmesh, fused, layers, metrics
from meshode_gb300 import pyDeform as PD

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CHAMFER_TOL = 1e-4
DF_TOL_REL_DIAG = 1e-5


@pytest.fixture(scope="module")
def demo():
    m = dict(np.load(os.path.join(GOLDEN, "ref_demo_meshes.npz")))
    r = dict(np.load(os.path.join(GOLDEN, "ref_demo_rigid.npz")))
    return m, r


def _sha(t):
    return hashlib.sha256(np.ascontiguousarray(t.detach().cpu().numpy()).tobytes()).hexdigest()


def _perturbed(Vn, r):
    seed, sigma = r["perturb"]
    rng = np.random.Generator(np.random.PCG64(int(seed)))
    return (Vn + torch.from_numpy(rng.normal(0, float(sigma), Vn.shape).astype(np.float32))).contiguous()


def _target_normalized(orc, m, r):
    return orc.normalized_double(m["target_V"], float(r["scale"]), r["trans"])


def test_demo_template_matches_reference(cuda, orc, demo):
    m, r = demo
    N = int(r["N"])
    pid = PD.InitializeDeformTemplate(torch.from_numpy(m["target_V"]), torch.from_numpy(m["target_F"]), 0, N)
    scale, trans = PD.GetTransform(pid)
    assert scale == float(r["scale"]) and np.array_equal(trans, r["trans"])
    Tn = _target_normalized(orc, m, r)
    diag = float(np.linalg.norm(Tn.max(0) - Tn.min(0)))
    grid = PD.GetDistanceField(pid).reshape(-1).cpu().numpy().astype(np.float64)
    err = np.abs(grid - r["grid"].astype(np.float64)).max()
    assert err <= DF_TOL_REL_DIAG * diag, err
    V = torch.from_numpy(m["source_V"].copy()).to(cuda)
    PD.NormalizeByTemplate(V, pid)
    assert np.array_equal(V.cpu().numpy().view(np.uint32), r["source_normalized"].view(np.uint32))
    PD.ReleaseTemplate(pid)


def test_demo_losses_bit_exact_on_reference_grid(cuda, demo):
    m, r = demo
    N = int(r["N"])
    grid = torch.from_numpy(r["grid"]).to(cuda)
    s = L.stream_ptr()
    Vn = torch.from_numpy(r["source_normalized"].copy())
    F = torch.from_numpy(m["source_F"]).to(cuda)
    # the rest offsets come from the normalised source (rigid_loss_layer.py:38)
    pid = PD.InitializeDeformTemplate(torch.from_numpy(m["target_V"]), torch.from_numpy(m["target_F"]), 0, 8)
    PD.StoreRigidityInformation(Vn.to(cuda), F, pid)
    for tag, V in (("at_source", Vn), ("at_perturbed", _perturbed(Vn, r))):
        Vg = V.to(cuda)
        n = Vg.shape[0]
        loss = torch.empty(n, dtype=torch.float32, device=cuda)
        grad = torch.empty((n, 3), dtype=torch.float32, device=cuda)
        L.call("mo_dfloss_forward", L.ptr(Vg), n, L.ptr(grid), N, L.MO_LAYOUT_LINEAR, L.ptr(loss), s)
        L.call("mo_dfloss_backward", L.ptr(Vg), n, L.ptr(grid), N, L.MO_LAYOUT_LINEAR, L.ptr(grad), s)
        assert _sha(loss) == str(r["df_forward_" + tag]), tag
        assert _sha(grad) == str(r["df_backward_" + tag]), tag
        assert _sha(PD.RigidEdgeLoss_forward(Vg, F, pid)) == str(r["rigid_forward_" + tag]), tag
        assert _sha(PD.RigidEdgeLoss_backward(Vg, F, pid)) == str(r["rigid_backward_" + tag]), tag
    PD.ReleaseTemplate(pid)


def test_demo_rigid_fit_chamfer(cuda, orc, demo):
    m, r = demo
    steps = int(r["loop_steps"])
    Tn = _target_normalized(orc, m, r)
    tF = m["target_F"]
    sF = m["source_F"]
    c_ref = metrics.chamfer(r["loop_final_normalized"], sF, Tn, tF, samples=20000)
    # rigid_deform.py:25-39 verbatim over the GPU layers
    src_V = torch.from_numpy(m["source_V"].copy()).to(cuda)
    src_F = torch.from_numpy(sF).to(cuda)
    rigid_deform = layers.RigidLossLayer(src_V, src_F, torch.from_numpy(m["target_V"]), torch.from_numpy(tF))
    param_id = rigid_deform.param_id
    src_V = torch.nn.Parameter(src_V)
    optimizer = torch.optim.Adam([src_V], lr=1e-3)
    first = None
    for it in range(steps):
        optimizer.zero_grad()
        loss = rigid_deform(src_V, src_F)
        loss.backward()
        optimizer.step()
        if it == 0:
            first = loss.item()
    c_plain = metrics.chamfer(src_V.detach().cpu().numpy(), sF, Tn, tF, samples=20000)
    # the first loss: the same terms, summed in another order than torch's CPU sum
    assert abs(first - r["loop_losses_every_100"][0]) <= 1e-5 * abs(r["loop_losses_every_100"][0])
    # the fused loop from the same normalised source
    V = torch.from_numpy(r["source_normalized"].copy()).to(cuda)
    out, _ = fused.fused_fit(int(param_id), V, steps)
    c_fused = metrics.chamfer(out.cpu().numpy(), sF, Tn, tF, samples=20000)
    assert abs(c_plain - c_ref) <= CHAMFER_TOL, (c_plain, c_ref)
    assert abs(c_fused - c_ref) <= CHAMFER_TOL, (c_fused, c_ref)
    PD.ReleaseTemplate(int(param_id))


def _cad_invariants(out):
    V, F, E, s2g, GV, GE = out
    nv, ng = V.shape[0], GV.shape[0]
    assert F.min() >= 0 and F.max() < nv and E.min() >= 0 and E.max() < nv
    assert s2g.shape == (nv, 1) and s2g.min() >= 0 and s2g.max() < ng
    assert np.bincount(s2g[:, 0], minlength=ng).min() >= 1  # every graph node represents a vertex
    assert GE.min() >= 0 and GE.max() < ng and (GE[:, 0] < GE[:, 1]).all()
    assert np.isfinite(V).all() and np.isfinite(GV).all()
    # remeshed edges are at most 3x the 0.02 subdivision length (mesh_tensor.cc:111)
    e = np.linalg.norm(V[F[:, [1, 2, 0]]].astype(np.float64) - V[F].astype(np.float64), axis=2)
    assert e.max() <= 0.06 + 1e-6


def test_demo_cad_pipeline_and_fit(cuda, orc, demo):
    m, _ = demo
    steps = 300
    src = cadmesh.load_cad_mesh_arrays(m["cad_source_V64"], m["cad_source_F"])
    tar = cadmesh.load_cad_mesh_arrays(m["cad_target_V64"], m["cad_target_F"])
    _cad_invariants(src)
    _cad_invariants(tar)
    _, _, _, _, graph_V, graph_E = src
    tar_V, tar_F, _, _, graph_V_tar, _ = tar
    rigidity = 1.0
    # cad_deform2.py:34-57 on the GPU layers (without the early stop)
    gV = torch.from_numpy(graph_V).to(cuda)
    gE = torch.from_numpy(graph_E).to(cuda)
    graph_deform = layers.GraphLossLayer(gV, gE, torch.from_numpy(tar_V), torch.from_numpy(tar_F), rigidity)
    pid = int(graph_deform.param_id)
    reverse_deform = layers.ReverseLossLayer()
    gV0 = gV.detach().cpu().clone()  # the normalised graph the fit starts from
    P = torch.nn.Parameter(gV)
    opt = torch.optim.Adam([P], lr=1e-3)
    gT = torch.from_numpy(graph_V_tar.copy()).to(cuda)
    PD.NormalizeByTemplate(gT, pid)
    for _ in range(steps):
        opt.zero_grad()
        loss = graph_deform(P, gE) / P.shape[0] + reverse_deform(P, gT) / gT.shape[0]
        loss.backward()
        opt.step()
    # the same loop on the oracle (CPU, same grid): graph loss + reverse loss
    opid = orc.InitializeDeformTemplate(tar_V, tar_F, 0, 64, grid=PD.GetDistanceField(pid).cpu().numpy())
    Eo = torch.from_numpy(graph_E)
    orc.StoreGraphInformation(gV0, Eo, opid)
    gTo = gT.cpu()
    Vo = torch.nn.Parameter(gV0.clone())
    opt_o = torch.optim.Adam([Vo], lr=1e-3)
    r2 = rigidity * rigidity
    for _ in range(steps):
        opt_o.zero_grad()
        with torch.no_grad():
            _, g = orc.graph_loss_grad(Vo.data, Eo, opid, r2)
        lr_, _ = orc.reverse_loss(Vo, gTo)
        (lr_ / gTo.shape[0]).backward()
        with torch.no_grad():
            Vo.grad += g / Vo.shape[0]
        opt_o.step()
    sc, tr = orc.normalize_params(tar_V)
    Tn = orc.normalized_double(tar_V, sc, tr)
    empty = np.zeros((0, 3), np.int32)
    c_gpu = metrics.chamfer(P.detach().cpu().numpy(), empty, Tn, tar_F, samples=20000)
    c_orc = metrics.chamfer(Vo.detach().numpy(), empty, Tn, tar_F, samples=20000)
    c_start = metrics.chamfer(gV0.numpy(), empty, Tn, tar_F, samples=20000)
    assert c_gpu < c_start  # the fit moved the graph toward the target
    assert abs(c_gpu - c_orc) <= CHAMFER_TOL, (c_gpu, c_orc)
    PD.ReleaseTemplate(pid)
