"""Rigid / graph edge losses on the GPU against the oracle's serial loops.

Reference: src/interface/rigid_layer.cc:11-133 and graph_layer.cc:11-135.  The
backward pass is a per-vertex reduction over a CSR sorted in half-edge order,
so it must reproduce the reference's serial scatter bit for bit.
"""
import numpy as np
import pytest
import torch

from meshode_gb300 import _lib as L
from meshode_gb300 import meshgen
from meshode_gb300 import pyDeform as PD

pytestmark = pytest.mark.gpu


def _template(cuda, N=16):
    V, F = meshgen.icosphere(1)
    return PD.InitializeDeformTemplate(torch.from_numpy(V.astype(np.float32)), torch.from_numpy(F.astype(np.int32)),
                                       0, N)


def _same(a, b):
    a = np.asarray(a, np.float32)
    b = np.asarray(b, np.float32)
    eq = (a == b) | (np.isnan(a) & np.isnan(b))
    return bool(eq.all()), int((~eq).sum())


@pytest.mark.parametrize("level", [1, 3])
def test_rigid_edges_bitexact(cuda, orc, level):
    rng = np.random.Generator(np.random.PCG64(level))
    V, F = meshgen.icosphere(level)
    V0 = (V * 0.3 + 0.5).astype(np.float32)
    F = F.astype(np.int32)
    pid = _template(cuda)
    Vt = torch.from_numpy(V0)
    Ft = torch.from_numpy(F)
    PD.StoreRigidityInformation(Vt, Ft, pid)
    off = orc.edge_offsets(V0, F, 0)
    ok, _ = _same(PD.GetParams(pid).edge.offsets.cpu().numpy(), off)
    assert ok
    V1 = (V0 + rng.normal(scale=0.01, size=V0.shape)).astype(np.float32)
    for dev in ("cpu", cuda):
        Vx = torch.from_numpy(V1).to(dev)
        Fx = Ft.to(dev)
        f = PD.RigidEdgeLoss_forward(Vx, Fx, pid).cpu().numpy()
        b = PD.RigidEdgeLoss_backward(Vx, Fx, pid).cpu().numpy()
        ok, n = _same(f, orc.edge_forward(V1, F, 0, off))
        assert ok, n
        ok, n = _same(b, orc.edge_backward(V1, F, 0, off))
        assert ok, n
    # the combined entry point (no weights) gives the two calls' results
    st = PD.GetParams(pid).edge
    Vx = torch.from_numpy(V1).to(cuda)
    loss = torch.empty(st.nh, 3, dtype=torch.float32, device=cuda)
    grad = torch.empty(Vx.shape[0], 3, dtype=torch.float32, device=cuda)
    L.call("mo_edge_fwd_bwd", L.ptr(Vx), Vx.shape[0], L.ptr(st.idx), F.shape[0], L.MO_EDGES_FACES, L.ptr(st.csr),
           L.ptr(st.offsets), None, L.ptr(loss), L.ptr(grad), L.stream_ptr())
    assert torch.equal(loss, PD.RigidEdgeLoss_forward(Vx, Ft.to(cuda), pid))
    assert torch.equal(grad, PD.RigidEdgeLoss_backward(Vx, Ft.to(cuda), pid))


def test_graph_edges_degenerate_and_duplicates(cuda, orc):
    rng = np.random.Generator(np.random.PCG64(7))
    nv = 500
    V0 = rng.uniform(0, 1, size=(nv, 3)).astype(np.float32)
    E = rng.integers(0, nv, size=(3000, 2)).astype(np.int32)
    E[:50, 1] = E[:50, 0]          # degenerate v0 == v1
    E[50:100] = E[100:150]         # duplicates
    E[150:200] = E[200:250][:, ::-1]  # reversed duplicates
    E = np.ascontiguousarray(E)
    pid = _template(cuda)
    PD.StoreGraphInformation(torch.from_numpy(V0), torch.from_numpy(E), pid)
    off = orc.edge_offsets(V0, E, 1)
    V1 = (V0 + rng.normal(scale=0.05, size=V0.shape)).astype(np.float32)
    Vx = torch.from_numpy(V1).to(cuda)
    Ex = torch.from_numpy(E).to(cuda)
    ok, n = _same(PD.GraphEdgeLoss_forward(Vx, Ex, pid).cpu().numpy(), orc.edge_forward(V1, E, 1, off))
    assert ok, n
    ok, n = _same(PD.GraphEdgeLoss_backward(Vx, Ex, pid).cpu().numpy(), orc.edge_backward(V1, E, 1, off))
    assert ok, n


def test_isolated_vertices_and_high_degree(cuda, orc):
    # a fan: vertex 0 connected to 2000 others (a long CSR row), plus isolated vertices
    nv = 2100
    rng = np.random.Generator(np.random.PCG64(9))
    V0 = rng.uniform(0, 1, size=(nv, 3)).astype(np.float32)
    F = np.stack([np.zeros(1999), np.arange(1, 2000), np.arange(2, 2001)], 1).astype(np.int32)
    pid = _template(cuda)
    PD.StoreRigidityInformation(torch.from_numpy(V0), torch.from_numpy(F), pid)
    off = orc.edge_offsets(V0, F, 0)
    V1 = (V0 + rng.normal(scale=0.02, size=V0.shape)).astype(np.float32)
    b = PD.RigidEdgeLoss_backward(torch.from_numpy(V1).to(cuda), torch.from_numpy(F).to(cuda), pid).cpu().numpy()
    ok, n = _same(b, orc.edge_backward(V1, F, 0, off))
    assert ok, n
    assert np.all(b[2001:] == 0)


def test_bad_index_raises(cuda):
    V0 = np.zeros((10, 3), np.float32)
    F = np.array([[0, 1, 2], [3, 4, 10]], np.int32)
    pid = _template(cuda)
    with pytest.raises(RuntimeError):
        PD.StoreRigidityInformation(torch.from_numpy(V0), torch.from_numpy(F), pid)
    F2 = np.array([[0, 1, -1]], np.int32)
    with pytest.raises(RuntimeError):
        PD.StoreRigidityInformation(torch.from_numpy(V0), torch.from_numpy(F2), pid)


def test_empty_edges(cuda):
    V0 = np.zeros((4, 3), np.float32)
    F = np.zeros((0, 3), np.int32)
    pid = _template(cuda)
    PD.StoreRigidityInformation(torch.from_numpy(V0), torch.from_numpy(F), pid)
    out = PD.RigidEdgeLoss_forward(torch.from_numpy(V0).to(cuda), torch.from_numpy(F).to(cuda), pid)
    assert out.shape == (0, 3)
    g = PD.RigidEdgeLoss_backward(torch.from_numpy(V0).to(cuda), torch.from_numpy(F).to(cuda), pid)
    assert torch.all(g == 0)


@pytest.mark.parametrize("level", [1, 3])
def test_cad_edges_bitexact(cuda, orc, level):
    """StoreCadInformation / CadEdgeLoss_forward/_backward
    (src/interface/cad_layer.cc:11-223): E's edges then F's half-edges with
    weights 2e-2/(|off|+1e-8); forward ((r*w)^2), backward (serial scatter of
    r*w^2) bit for bit against the oracle, from CPU and CUDA tensors, with
    duplicated and degenerate (v0 == v1, zero offset) edges in E."""
    rng = np.random.Generator(np.random.PCG64(10 + level))
    V, F = meshgen.icosphere(level)
    V0 = (V * 0.3 + 0.5).astype(np.float32)
    F = F.astype(np.int32)
    E = meshgen.edges_from_faces(F)[::2]
    E = np.concatenate([E, E[:5], np.array([[0, 0], [1, 1]], np.int32)]).astype(np.int32)
    pid = _template(cuda)
    Vt, Ft, Et = torch.from_numpy(V0), torch.from_numpy(F), torch.from_numpy(E)
    PD.StoreCadInformation(Vt, Ft, Et, pid)
    opid = orc.InitializeDeformTemplate(np.zeros((3, 3), np.float32), np.array([[0, 1, 2]], np.int32), 0, 2,
                                        grid=np.zeros(8, np.float32))
    orc.StoreCadInformation(V0, F, E, opid)
    st = PD.GetParams(pid).edge
    assert _same(st.offsets.cpu().numpy(), orc.GetParams(opid).edge_offset)[0]
    assert _same(st.weights.cpu().numpy(), orc.GetParams(opid).edge_lambda)[0]
    V1 = (V0 + rng.normal(scale=0.01, size=V0.shape)).astype(np.float32)
    for dev in ("cpu", cuda):
        Vx = torch.from_numpy(V1).to(dev)
        f = PD.CadEdgeLoss_forward(Vx, Ft.to(dev), Et.to(dev), pid).cpu().numpy()
        b = PD.CadEdgeLoss_backward(Vx, Ft.to(dev), Et.to(dev), pid).cpu().numpy()
        ok, n = _same(f, orc.CadEdgeLoss_forward(V1, F, E, opid).numpy())
        assert ok, n
        ok, n = _same(b, orc.CadEdgeLoss_backward(V1, F, E, opid).numpy())
        assert ok, n
    with pytest.raises(RuntimeError):
        PD.RigidEdgeLoss_forward(torch.from_numpy(V1), Ft, pid)  # the template holds CAD edges now
    # the combined entry point gives the two calls' results
    Vx = torch.from_numpy(V1).to(cuda)
    _, st_, Vd, lst, csr = PD._cad_state(pid, Vx, Ft.to(cuda), Et.to(cuda))
    loss = torch.empty(st_.nh, 3, dtype=torch.float32, device=cuda)
    grad = torch.empty(Vd.shape[0], 3, dtype=torch.float32, device=cuda)
    L.call("mo_edge_fwd_bwd", L.ptr(Vd), Vd.shape[0], L.ptr(lst), st_.nh, L.MO_EDGES_LIST, L.ptr(csr),
           L.ptr(st_.offsets), L.ptr(st_.weights), L.ptr(loss), L.ptr(grad), L.stream_ptr())
    assert torch.equal(loss, PD.CadEdgeLoss_forward(Vx, Ft.to(cuda), Et.to(cuda), pid))
    assert torch.equal(grad, PD.CadEdgeLoss_backward(Vx, Ft.to(cuda), Et.to(cuda), pid))
