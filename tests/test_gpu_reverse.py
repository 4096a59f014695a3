"""Reverse (target -> source) nearest-point loss on the GPU
(src/python/layers/reverse_loss_layer.py:14-25).

* Nearest indices equal scipy's cKDTree's, and the distances its float64
  distances within 2 ulp (the library evaluates the squared sum without
  fused multiply-adds; a SciPy build may fuse them), on random clouds, mesh
  vertices and clustered points; exact ties (duplicate source points) go to
  the lowest index at the same distance.
* The loss matches the reference expression on the CPU (torch autograd over
  the cKDTree indices) within 1e-6 relative, and the gradient matches it bit
  for bit, for upstream gradients 1 and 1/n.
* Bad input raises; one source point and zero targets work.
"""
import ctypes

import numpy as np
import pytest
import torch

from meshode_gb300 import _lib as L
from meshode_gb300 import layers, meshgen

pytestmark = pytest.mark.gpu


def _nn(P, Q):
    dev = torch.device("cuda")
    Pd = torch.from_numpy(np.ascontiguousarray(P, np.float32)).to(dev)
    Qd = torch.from_numpy(np.ascontiguousarray(Q, np.float32)).to(dev)
    idx = torch.empty(len(Q), dtype=torch.int32, device=dev)
    d2 = torch.empty(len(Q), dtype=torch.float64, device=dev)
    L.call("mo_nn_query", L.ptr(Pd), len(P), L.ptr(Qd), len(Q), L.ptr(idx), L.ptr(d2), None, 0, L.stream_ptr())
    return idx.cpu().numpy(), d2.cpu().numpy()


def _clouds():
    rng = np.random.Generator(np.random.PCG64(31))
    out = {"uniform": (rng.uniform(-1, 1, (5000, 3)), rng.uniform(-1.2, 1.2, (7000, 3)))}
    V, F = meshgen.icosphere(4)
    T = meshgen.displace(V, rng)
    out["mesh"] = (V * 0.9, T)
    centers = rng.uniform(-5, 5, (20, 3))
    P = np.concatenate([c + 0.01 * rng.standard_normal((300, 3)) for c in centers])
    Q = np.concatenate([c + 0.02 * rng.standard_normal((200, 3)) for c in centers] + [rng.uniform(-6, 6, (500, 3))])
    out["clusters"] = (P, Q)
    return {k: (np.asarray(a, np.float32), np.asarray(b, np.float32)) for k, (a, b) in out.items()}


@pytest.mark.parametrize("name", ["uniform", "mesh", "clusters"])
def test_nn_matches_ckdtree(cuda, name):
    from scipy.spatial import cKDTree
    P, Q = _clouds()[name]
    dd, ii = cKDTree(P).query(Q, k=1)
    idx, d2 = _nn(P, Q)
    assert np.array_equal(idx, ii)
    assert np.allclose(np.sqrt(d2), dd, rtol=4.5e-16, atol=0)


def test_nn_ties_lowest_index(cuda):
    from scipy.spatial import cKDTree
    rng = np.random.Generator(np.random.PCG64(2))
    base = rng.uniform(0, 1, (400, 3)).astype(np.float32)
    P = np.concatenate([base, base[::-1], base[:50]])  # every point at least twice
    Q = np.concatenate([base[:100], rng.uniform(0, 1, (300, 3)).astype(np.float32)])
    idx, d2 = _nn(P, Q)
    dd, ii = cKDTree(P).query(Q, k=1)
    assert np.allclose(np.sqrt(d2), dd, rtol=4.5e-16, atol=0)
    # the lowest index among the points at that exact distance
    D = ((P[None, :, :].astype(np.float64) - Q[:, None, :].astype(np.float64)) ** 2).sum(-1)
    low = np.array([np.flatnonzero(D[q] == D[q].min()).min() for q in range(len(Q))])
    assert np.array_equal(idx, low)


@pytest.mark.parametrize("scale", [1.0, "1/n"])
@pytest.mark.parametrize("name", ["uniform", "mesh", "clusters"])
def test_reverse_loss_and_grad(cuda, orc, name, scale):
    P, Q = _clouds()[name]
    src_c = torch.from_numpy(P.copy()).requires_grad_(True)
    tar_c = torch.from_numpy(Q.copy())
    k = 1.0 if scale == 1.0 else 1.0 / len(Q)
    ref_loss, _ = orc.reverse_loss(src_c, tar_c)
    (ref_loss * k).backward()
    src_g = torch.from_numpy(P.copy()).cuda().requires_grad_(True)
    loss = layers.ReverseLossLayer()(src_g, torch.from_numpy(Q.copy()).cuda())
    assert loss.device.type == "cuda" and loss.dtype == torch.float32
    assert abs(float(loss) - float(ref_loss)) <= 1e-6 * abs(float(ref_loss))
    (loss * k).backward()
    assert torch.equal(src_g.grad.cpu(), src_c.grad)


def test_reverse_loss_cpu_tensors(cuda, orc):
    P, Q = _clouds()["mesh"]
    src = torch.from_numpy(P.copy()).requires_grad_(True)
    loss = layers.ReverseLossLayer()(src, torch.from_numpy(Q.copy()))
    assert loss.device.type == "cpu"
    loss.backward()
    ref_src = torch.from_numpy(P.copy()).requires_grad_(True)
    ref, _ = orc.reverse_loss(ref_src, torch.from_numpy(Q.copy()))
    ref.backward()
    assert torch.equal(src.grad, ref_src.grad)


def test_nn_edge_cases_and_errors(cuda):
    P = np.array([[0.5, 0.5, 0.5]], np.float32)
    Q = np.random.Generator(np.random.PCG64(1)).uniform(0, 1, (37, 3)).astype(np.float32)
    idx, d2 = _nn(P, Q)
    assert (idx == 0).all()
    idx, _ = _nn(Q, Q[:0].reshape(0, 3))
    assert idx.shape == (0,)
    Qn = Q.copy()
    Qn[3, 1] = np.nan
    with pytest.raises(RuntimeError, match="non-finite"):
        _nn(Q, Qn)
    # out-of-range indices into the loss are reported, not read
    dev = torch.device("cuda")
    S = torch.from_numpy(Q).to(dev)
    bad = torch.tensor([0, 5, 37], dtype=torch.int32, device=dev)
    nb = L.lib().mo_reverse_loss_scratch_bytes(37, 3)
    scratch = torch.empty(nb, dtype=torch.uint8, device=dev)
    loss = torch.empty(1, dtype=torch.float64, device=dev)
    with pytest.raises(RuntimeError, match="out of range"):
        L.call("mo_reverse_loss_forward", L.ptr(S), 37, L.ptr(S[:3].contiguous()), 3, L.ptr(bad), L.ptr(loss),
               L.ptr(scratch), nb, None, L.stream_ptr())
