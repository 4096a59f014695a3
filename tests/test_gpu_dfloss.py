"""DistanceFieldLoss forward/backward on the GPU against the oracle, bit for bit.

Reference: src/interface/distance_layer.cc:8-81 with
UniformGrid::DistanceFloat (src/lib/uniformgrid.cc:85-150).  The GPU grid is
handed to the oracle so the comparison isolates the lookup and its jet
derivative; both must agree exactly (integer-equal bit patterns).
"""
import numpy as np
import pytest
import torch

from meshode_gb300 import _lib as L
from meshode_gb300 import meshgen
from meshode_gb300 import pyDeform as PD

pytestmark = pytest.mark.gpu


def _template(N, level=3, seed=11):
    rng = np.random.Generator(np.random.PCG64(seed))
    V, F = meshgen.icosphere(level)
    T = meshgen.displace(V, rng).astype(np.float32)
    pid = PD.InitializeDeformTemplate(torch.from_numpy(T), torch.from_numpy(F.astype(np.int32)), 0, N)
    return pid


def _probe_points(N, n=20000, seed=3):
    rng = np.random.Generator(np.random.PCG64(seed))
    P = rng.uniform(-0.15, 1.15, size=(n, 3)).astype(np.float32)
    # near the surface region as well
    Q = rng.uniform(0.2, 0.8, size=(n, 3)).astype(np.float32)
    edge = []
    # exactly on the far slab p*N == N-1 (no penalty term on that axis)
    edge.append([(N - 1) / N, 0.5, 0.5])
    edge.append([0.5, (N - 1) / N, 0.2])
    # truncation toward zero: (-1/N, 0) maps to cell 0 and extrapolates
    edge.append([-0.4 / N, 0.3, 0.6])
    edge.append([0.3, -0.9 / N, -0.2 / N])
    # beyond N on one axis, below zero on another
    edge.append([1.3, -0.2, 0.5])
    edge.append([1.0, 1.0, 1.0])
    edge.append([0.0, 0.0, 0.0])
    # grid nodes exactly
    for k in range(0, N, max(1, N // 7)):
        edge.append([k / N, (k // 2) / N, (N - 2 - k // 3) / N])
    # huge magnitudes (x86 integer-indefinite truncation) and NaN
    edge.append([3.0e9, 0.5, 0.5])
    edge.append([-3.0e9, 0.5, 0.5])
    edge.append([np.nan, 0.5, 0.5])
    E = np.asarray(edge, np.float32)
    return np.concatenate([P, Q, E], 0)


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def _same(a, b):
    """Bit equality, treating every NaN as equal and +0 == -0."""
    a = np.asarray(a, np.float32)
    b = np.asarray(b, np.float32)
    both_nan = np.isnan(a) & np.isnan(b)
    eq = (a == b) | both_nan
    return bool(eq.all()), int((~eq).sum())


@pytest.mark.parametrize("N", [16, 63, 64])
@pytest.mark.parametrize("layout", [L.MO_LAYOUT_LINEAR, L.MO_LAYOUT_CELL, L.MO_LAYOUT_BRICK4])
def test_dfloss_bitexact(cuda, orc, N, layout):
    pid = _template(N)
    grid = PD.GetDistanceField(pid).cpu().numpy().reshape(-1)
    P = _probe_points(N)
    PD.GetParams(pid).layout = layout
    if layout == L.MO_LAYOUT_LINEAR:
        PD.GetParams(pid).grid = PD.GetParams(pid).grid_linear
    else:
        nb = L.lib().mo_grid_bytes(N, layout)
        g = torch.empty(nb // 4, dtype=torch.float32, device=cuda)
        L.call("mo_grid_relayout", L.ptr(PD.GetParams(pid).grid_linear), N, layout, L.ptr(g), L.stream_ptr())
        PD.GetParams(pid).grid = g
    Vt = torch.from_numpy(P).to(cuda)
    lf = PD.DistanceFieldLoss_forward(Vt, pid).cpu().numpy()
    lb = PD.DistanceFieldLoss_backward(Vt, pid).cpu().numpy()
    of = orc.dfloss_forward(P, grid, N)
    ob = orc.dfloss_backward(P, grid, N)
    ok, nbad = _same(lf, of)
    assert ok, "forward mismatches: %d" % nbad
    ok, nbad = _same(lb, ob)
    assert ok, "backward mismatches: %d" % nbad


def test_dfloss_cpu_tensor_roundtrip(cuda, orc):
    N = 32
    pid = _template(N)
    grid = PD.GetDistanceField(pid).cpu().numpy().reshape(-1)
    P = _probe_points(N, n=1000)
    out = PD.DistanceFieldLoss_forward(torch.from_numpy(P), pid)
    assert out.device.type == "cpu" and out.dtype == torch.float32 and out.shape == (P.shape[0],)
    ok, _ = _same(out.numpy(), orc.dfloss_forward(P, grid, N))
    assert ok


def test_dfloss_fwd_bwd_mask(cuda, orc):
    N = 32
    pid = _template(N)
    grid = PD.GetDistanceField(pid).cpu().numpy().reshape(-1)
    P = _probe_points(N, n=5000)
    thresh = float(np.float32(0.5 * 0.03 * 0.03))
    loss, grad = PD.DistanceFieldLoss_fwd_bwd(torch.from_numpy(P).to(cuda), pid, mask_thresh=thresh)
    of = orc.dfloss_forward(P, grid, N)
    ob = orc.dfloss_backward(P, grid, N)
    mask = ((of * np.float32(0.5)) < np.float32(thresh)).astype(np.float32)[:, None]
    ok, _ = _same(loss.cpu().numpy(), of)
    assert ok
    ok, nbad = _same(grad.cpu().numpy(), ob * mask)
    assert ok, nbad


def test_dfloss_empty_and_errors(cuda):
    pid = _template(16, level=1)
    out = PD.DistanceFieldLoss_forward(torch.zeros(0, 3, device=cuda), pid)
    assert out.shape == (0,)
    with pytest.raises(RuntimeError):
        PD.DistanceFieldLoss_forward(torch.zeros(5, 3, dtype=torch.float64, device=cuda), pid)
    with pytest.raises(RuntimeError):
        PD.DistanceFieldLoss_forward(torch.zeros(5, 2, device=cuda), pid)
    with pytest.raises(RuntimeError):
        PD.DistanceFieldLoss_forward(torch.zeros(5, 3, device=cuda), 10 ** 6)
