"""The loss-preserving distance-field band (MoDfOptions.band,
mo_df_loss_band) on the GPU.

* Grid: voxels below the band hold exactly the exact build's value, every
  other voxel holds the band; in the two lowest layers along each axis the
  band is band + 13/N.  The same for both methods and every packet shape.
* DistanceFieldLoss forward and backward (UniformGrid::DistanceFloat through
  the jet, uniformgrid.cc:85-150) from the banded grid equal, bit for bit,
  those from the exact grid at points everywhere: inside the cube, near the
  surface, on the 0.2 cutoff, in the extrapolation slab (-1/N, 0) of each
  axis, in the penalty region; in every grid layout.
"""
import ctypes

import numpy as np
import pytest
import torch

from meshode_gb300 import _lib as L
from meshode_gb300 import meshgen
from meshode_gb300._lib import call, ptr, stream_ptr

pytestmark = pytest.mark.gpu


def _targets():
    rng = np.random.Generator(np.random.PCG64(7))
    V, F = meshgen.icosphere(3)
    sphere = (meshgen.displace(V, rng).astype(np.float32), F.astype(np.int32))
    # a small sphere next to a large one: deep interior and wide far field
    V2, F2 = meshgen.icosphere(2)
    both = (np.concatenate([V * 0.9, V2 * 0.15 + np.array([1.6, 0.3, -0.2])]).astype(np.float32),
            np.concatenate([F, F2 + len(V)]).astype(np.int32))
    # an open, noisy plane strip (CAD-like)
    g = np.linspace(0, 1, 24)
    X, Y = np.meshgrid(g, g * 0.4)
    P = np.stack([X.ravel(), Y.ravel(), 0.02 * rng.standard_normal(X.size)], 1).astype(np.float32)
    idx = np.arange(24 * 24).reshape(24, 24)
    Fp = np.concatenate([np.stack([idx[:-1, :-1].ravel(), idx[:-1, 1:].ravel(), idx[1:, :-1].ravel()], 1),
                         np.stack([idx[1:, :-1].ravel(), idx[:-1, 1:].ravel(), idx[1:, 1:].ravel()], 1)])
    plane = (P, Fp.astype(np.int32))
    return {"sphere": sphere, "two": both, "plane": plane}


def _build(V, F, N, method, packet, band):
    dev = torch.device("cuda")
    Vd = torch.from_numpy(V).to(dev)
    Fd = torch.from_numpy(F).to(dev)
    bbox = torch.empty(6, dtype=torch.int32, device=dev)
    prm = torch.empty(4, dtype=torch.float64, device=dev)
    s = stream_ptr()
    call("mo_bbox", ptr(Vd), Vd.shape[0], ptr(bbox), s)
    call("mo_norm_params", ptr(bbox), ptr(prm), s)
    grid = torch.empty(N ** 3, dtype=torch.float32, device=dev)
    opt = L.MoDfOptions(method, packet, band)
    call("mo_df_build_ex", ptr(Vd), Vd.shape[0], ptr(Fd), Fd.shape[0], N, ptr(prm), ctypes.byref(opt), None, 0,
         ptr(grid), None, s)
    return grid, prm


def _low_layers(N):
    z, y, x = np.meshgrid(np.arange(N), np.arange(N), np.arange(N), indexing="ij")
    return ((x <= 1) | (y <= 1) | (z <= 1)).reshape(-1)


@pytest.mark.parametrize("name", ["sphere", "two", "plane"])
@pytest.mark.parametrize("N", [16, 33, 64])
def test_band_grid(cuda, name, N):
    V, F = _targets()[name]
    band = L.lib().mo_df_loss_band(N)
    assert abs(band - (0.2 + 3 ** 0.5 / N + 1e-3)) < 1e-6
    exact, _ = _build(V, F, N, L.MO_DF_LBVH, L.MO_PACKET_4x4x2, 0.0)
    exact = exact.cpu().numpy()
    low = _low_layers(N)
    wide = np.float32(band) + np.float32(13.0) / np.float32(N)
    keep = (low & (exact < wide)) | (~low & (exact < np.float32(band)))
    assert (~keep).any() and keep.any()
    for method, packets in ((L.MO_DF_BRUTE, [L.MO_PACKET_4x4x2]),
                            (L.MO_DF_LBVH, [L.MO_PACKET_4x4x2, L.MO_PACKET_8x4x1, L.MO_PACKET_4x2x4,
                                            L.MO_PACKET_2x4x4, L.MO_PACKET_8x2x2, L.MO_PACKET_4x4x4,
                                            L.MO_PACKET_2x4x8, L.MO_PACKET_8x4x2, L.MO_PACKET_4x4x2_TRI2,
                                            L.MO_PACKET_2x4x4_TRI2])):
        for packet in packets:
            g, _ = _build(V, F, N, method, packet, band)
            g = g.cpu().numpy()
            assert np.array_equal(g[keep], exact[keep]), (method, packet)
            assert np.all(g[~keep & ~low] == np.float32(band)), (method, packet)
            assert np.all(g[~keep & low] == wide), (method, packet)


def _probes(N, Vn, n=40000, seed=5):
    rng = np.random.Generator(np.random.PCG64(seed))
    pts = [rng.uniform(-0.15, 1.15, size=(n, 3))]
    # near the surface, and on shells around the 0.2 cutoff distance
    k = rng.integers(0, len(Vn), size=n)
    d = rng.standard_normal((n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    for r in (0.0, 0.02, 0.19, 0.2, 0.21, 0.2 + 1.0 / N, 0.25):
        pts.append(Vn[k] + d * r * rng.uniform(0.97, 1.03, size=(n, 1)))
    # the extrapolation slab (-1/N, 0) of each axis, alone and combined
    for axes in ((0,), (1,), (2,), (0, 1), (0, 2), (1, 2), (0, 1, 2)):
        P = rng.uniform(0.0, 1.0, size=(n // 4, 3))
        for a in axes:
            P[:, a] = -rng.uniform(0.0, 1.0, size=n // 4) / N
        pts.append(P)
    # grid nodes and cell centres
    c = rng.integers(0, N, size=(n // 4, 3))
    pts.append(c / N)
    pts.append((c + 0.5) / N)
    return np.ascontiguousarray(np.concatenate(pts).astype(np.float32))


def _loss(P, grid, N, layout):
    dev = torch.device("cuda")
    s = stream_ptr()
    if layout != L.MO_LAYOUT_LINEAR:
        g = torch.empty(L.lib().mo_grid_bytes(N, layout) // 4, dtype=torch.float32, device=dev)
        call("mo_grid_relayout", ptr(grid), N, layout, ptr(g), s)
        grid = g
    Pd = torch.from_numpy(P).to(dev)
    loss = torch.empty(len(P), dtype=torch.float32, device=dev)
    grad = torch.empty(len(P), 3, dtype=torch.float32, device=dev)
    call("mo_dfloss_fwd_bwd", ptr(Pd), len(P), ptr(grid), N, layout, ptr(loss), ptr(grad), 0, 0.0, s)
    return loss.cpu().numpy(), grad.cpu().numpy()


def _same(a, b):
    eq = (a == b) | (np.isnan(a) & np.isnan(b))
    return bool(eq.all()), int((~eq).sum())


@pytest.mark.parametrize("name", ["sphere", "two", "plane"])
@pytest.mark.parametrize("N", [16, 33, 64])
def test_band_preserves_dfloss(cuda, orc, name, N):
    V, F = _targets()[name]
    band = L.lib().mo_df_loss_band(N)
    exact, prm = _build(V, F, N, L.MO_DF_AUTO, L.MO_PACKET_4x4x2, 0.0)
    banded, _ = _build(V, F, N, L.MO_DF_AUTO, L.MO_PACKET_4x4x2, band)
    assert not torch.equal(exact, banded)
    sc, tr = orc.normalize_params(V)
    P = _probes(N, orc.normalized_double(V, sc, tr))
    for layout in (L.MO_LAYOUT_LINEAR, L.MO_LAYOUT_CELL, L.MO_LAYOUT_BRICK4):
        le, ge = _loss(P, exact, N, layout)
        lb, gb = _loss(P, banded, N, layout)
        ok, nbad = _same(le, lb)
        assert ok, ("loss", layout, nbad)
        ok, nbad = _same(ge, gb)
        assert ok, ("grad", layout, nbad)
        # the probes reach every branch: nonzero losses, cutoff zeros, penalties
        assert (le > 0).sum() > 1000 and (le == 0).sum() > 1000


def test_band_argument_checks(cuda):
    V, F = _targets()["sphere"]
    with pytest.raises(RuntimeError, match="band"):
        _build(V, F, 16, L.MO_DF_LBVH, L.MO_PACKET_4x4x2, -1.0)
    assert L.lib().mo_df_loss_band(1) == 0.0
