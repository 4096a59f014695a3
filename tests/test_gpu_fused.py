"""Fused optimiser step on the GPU.

* The total gradient of a fused step equals the oracle's
  RigidLossFunction / GraphLossFunction gradient bit for bit
  (rigid_loss_layer.py:20-27, graph_loss_layer.py:33-43).
* Positions after several steps equal the oracle loop with the op-by-op
  Adam restatement bit for bit, and match the oracle gradients driven by
  torch.optim.Adam on the CPU within 1e-6 (torch's CPU kernels round some
  lanes differently).
* The loss of each step matches the layer loss within rtol 1e-5.
* A pair stepped alone and inside a mix of other pairs gives bit-identical
  results (the serving invariance).
"""
import numpy as np
import pytest
import torch

from meshode_gb300 import fused
from meshode_gb300 import meshgen
from meshode_gb300 import pyDeform as PD

pytestmark = pytest.mark.gpu


def _pair(cuda, orc, level=3, N=32, seed=1, graph=False):
    rng = np.random.Generator(np.random.PCG64(seed))
    V, F = meshgen.icosphere(level)
    T = meshgen.displace(V, rng).astype(np.float32)
    V = V.astype(np.float32)
    F = F.astype(np.int32)
    Tt, Ft = torch.from_numpy(T), torch.from_numpy(F)
    pid = PD.InitializeDeformTemplate(Tt, Ft, 0, N)
    Vs = torch.from_numpy(V.copy())
    PD.NormalizeByTemplate(Vs, pid)
    if graph:
        E = torch.from_numpy(meshgen.edges_from_faces(F))
        PD.StoreGraphInformation(Vs, E, pid)
        idx = E
    else:
        PD.StoreRigidityInformation(Vs, Ft, pid)
        idx = Ft
    # the oracle gets the GPU grid and the same normalised source
    opid = orc.InitializeDeformTemplate(T, F, 0, N, grid=PD.GetDistanceField(pid).cpu().numpy())
    if graph:
        orc.StoreGraphInformation(Vs, idx, opid)
    else:
        orc.StoreRigidityInformation(Vs, idx, opid)
    return pid, opid, Vs, idx


def test_fused_gradient_bitexact_rigid(cuda, orc):
    pid, opid, Vs, F = _pair(cuda, orc)
    pr = fused.pair_from_template(pid, Vs, steps=1, debug_grad=True)
    runner = fused.StepGroupRunner(cuda, 1, pr.ntiles, group_steps=1, use_graph=False)
    runner.upload([pr], [0])
    runner.run_group()
    g = pr.grad_dbg.view(-1, 3).cpu().numpy()
    ref = orc.rigid_grad(Vs, F, opid).numpy()
    assert np.array_equal(g, ref), int((g != ref).sum())


def test_fused_gradient_bitexact_graph_mask(cuda, orc):
    pid, opid, Vs, E = _pair(cuda, orc, graph=True)
    rig2 = float(torch.tensor(0.7 * 0.7, dtype=torch.float32))
    thresh = float(np.float32(0.5 * 0.03 * 0.03))
    pr = fused.pair_from_template(pid, Vs, steps=1, debug_grad=True, w_edge=rig2, mask_thresh=thresh)
    runner = fused.StepGroupRunner(cuda, 1, pr.ntiles, group_steps=1, use_graph=False)
    runner.upload([pr], [0])
    runner.run_group()
    g = pr.grad_dbg.view(-1, 3).cpu().numpy()
    loss, ref = orc.graph_loss_grad(Vs, E, opid, 0.7 * 0.7)
    assert np.array_equal(g, ref.numpy()), int((g != ref.numpy()).sum())
    L = runner.pair_losses(1)[0, 0].item()
    assert abs(L - float(loss)) <= 1e-5 * abs(float(loss)) + 1e-9


def test_fused_trajectory_bitexact_vs_exact_adam(cuda, orc):
    """40 fused steps equal the oracle loop with the op-by-op Adam
    restatement bit for bit (gradients and update both exact)."""
    pid, opid, Vs, F = _pair(cuda, orc)
    out, _ = fused.fused_fit(pid, Vs, 40, group_steps=8)
    ref, _ = orc.rigid_fit(Vs, F, opid, 40, adam="exact")
    assert torch.equal(out.cpu(), ref), (out.cpu() - ref).abs().max().item()


@pytest.mark.parametrize("use_graph", [False, True])
def test_fused_steps_vs_cpu_adam(cuda, orc, use_graph):
    pid, opid, Vs, F = _pair(cuda, orc)
    K = 30
    out, losses = fused.fused_fit(pid, Vs, K, group_steps=8, use_graph=use_graph, record_loss=True)
    ref, ref_losses = orc.rigid_fit(Vs, F, opid, K, loss_every=1)
    err = (out.cpu() - ref).abs().max().item()
    assert err <= 1e-6, err
    rl = np.asarray(ref_losses)
    gl = losses.cpu().numpy()
    assert np.allclose(gl, rl, rtol=1e-5, atol=1e-9), np.abs(gl - rl).max()


def test_alone_vs_mix_bitexact(cuda, orc):
    pairs_cfg = [(3, 32, 1), (2, 16, 2), (4, 48, 3)]
    built = [_pair(cuda, orc, level=l, N=n, seed=s) for (l, n, s) in pairs_cfg]
    K = 20
    alone = []
    for pid, _, Vs, _ in built:
        out, _ = fused.fused_fit(pid, Vs, K, group_steps=5)
        alone.append(out.cpu())
    prs = [fused.pair_from_template(pid, Vs, steps=K) for pid, _, Vs, _ in built]
    # staggered: the second pair joins later and the third has fewer steps
    prs[2].steps = K - 7
    max_tiles = sum(p.ntiles for p in prs)
    runner = fused.StepGroupRunner(cuda, 3, max_tiles, group_steps=5)
    active = [prs[0], prs[2]]
    for g in range(8):
        if g == 1:
            active.append(prs[1])
        active = [p for p in active if not p.done]
        if not active:
            break
        runner.upload(active, [p.t for p in active])
        runner.run_group()
        for p in active:
            p.t = min(p.steps, p.t + runner.S)
    assert all(p.done for p in prs)
    assert torch.equal(prs[0].positions().cpu(), alone[0])
    assert torch.equal(prs[1].positions().cpu(), alone[1])
    # the third pair ran fewer steps: compare against its own alone run
    out3, _ = fused.fused_fit(built[2][0], built[2][2], K - 7, group_steps=5)
    assert torch.equal(prs[2].positions().cpu(), out3.cpu())


def _cad_pair(cuda, orc, level=3, N=32, seed=4):
    rng = np.random.Generator(np.random.PCG64(seed))
    V, F = meshgen.icosphere(level)
    T = meshgen.displace(V, rng).astype(np.float32)
    V = V.astype(np.float32)
    F = F.astype(np.int32)
    E = meshgen.edges_from_faces(F)[::3]
    Tt, Ft, Et = torch.from_numpy(T), torch.from_numpy(F), torch.from_numpy(np.ascontiguousarray(E))
    pid = PD.InitializeDeformTemplate(Tt, Ft, 0, N)
    Vs = torch.from_numpy(V.copy())
    PD.NormalizeByTemplate(Vs, pid)
    PD.StoreCadInformation(Vs, Ft, Et, pid)
    opid = orc.InitializeDeformTemplate(T, F, 0, N, grid=PD.GetDistanceField(pid).cpu().numpy())
    orc.StoreCadInformation(Vs, Ft, Et, opid)
    return pid, opid, Vs, Ft, Et


def test_weighted_fused_step_bitexact_cad(cuda, orc):
    """The weighted fused step (mo_fused_step_weighted: per-edge weights of
    StoreCadInformation, E's edges then F's half-edges) against the oracle's
    CadLossFunction loop (cad_loss_layer.py:9-31, cad_layer.cc:152-223) with
    the op-by-op Adam: the first gradient and 30 steps bit for bit; the
    unweighted step on the same pair differs (the weights are used)."""
    pid, opid, Vs, F, E = _cad_pair(cuda, orc)
    # start away from the rest pose, so that the edge residuals (and the
    # weights) are not zero in the first step
    rng = np.random.Generator(np.random.PCG64(12))
    V0 = (Vs + torch.from_numpy(rng.normal(0, 0.01, Vs.shape).astype(np.float32))).contiguous()
    pr = fused.pair_from_template(pid, V0, steps=1, debug_grad=True)
    assert pr.sell_w is not None
    runner = fused.StepGroupRunner(cuda, 1, pr.ntiles, group_steps=1, use_graph=False, weighted=True)
    runner.upload([pr], [0])
    runner.run_group()
    g = pr.grad_dbg.view(-1, 3).cpu().numpy()
    ref = (orc.DistanceFieldLoss_backward(V0, opid) + orc.CadEdgeLoss_backward(V0, F, E, opid)).numpy()
    assert np.array_equal(g, ref), int((g != ref).sum())
    out, _ = fused.fused_fit(pid, V0, 30, group_steps=8)
    want = orc.cad_fit(V0, F, E, opid, 30, adam="exact")
    assert torch.equal(out.cpu(), want), (out.cpu() - want).abs().max().item()
    pr2 = fused.pair_from_template(pid, V0, steps=1, debug_grad=True)
    plain = fused.StepGroupRunner(cuda, 1, pr2.ntiles, group_steps=1, use_graph=False)
    plain.upload([pr2], [0])
    plain.run_group()
    assert not np.array_equal(pr2.grad_dbg.view(-1, 3).cpu().numpy(), ref)
