"""SolveLinear on the GPU (src/interface/linear_layer.cc:5-79): conjugate
gradients in double against the oracle's direct sparse solve of the same
system assembled as the reference does (src/lib/linear.cc), for
LinearEstimation (graph cells + face springs + extra edges) and
LinearEstimationWithRot (per-vertex rotations and scales).  Tolerance: 1e-6
of the mesh's bounding-box diagonal (the result is float32; both solvers are
double)."""
import numpy as np
import pytest
import torch

from meshode_gb300 import meshgen
from meshode_gb300 import pyDeform as PD

pytestmark = pytest.mark.gpu


def _problem(level=3, seed=3, cell=0.25):
    rng = np.random.Generator(np.random.PCG64(seed))
    V, F = meshgen.icosphere(level)
    V = (0.4 * V + 0.5).astype(np.float32)
    # graph nodes: vertices grouped by a coarse voxel grid, nodes at the
    # groups' centroids moved by a rotation, a scale and noise
    key = np.floor(V / cell).astype(np.int64)
    _, ref = np.unique(key[:, 0] * 10000 + key[:, 1] * 100 + key[:, 2], return_inverse=True)
    ng = int(ref.max()) + 1
    cent = np.stack([V[ref == g].mean(0) for g in range(ng)])
    th = 0.2
    Rz = np.array([[np.cos(th), -np.sin(th), 0], [np.sin(th), np.cos(th), 0], [0, 0, 1]])
    G = ((cent - 0.5) @ Rz.T * 1.1 + 0.5 + 0.01 * rng.standard_normal(cent.shape)).astype(np.float32)
    # extra edges between random near vertices
    i = rng.integers(0, len(V), 200)
    d = ((V[i][:, None, :] - V[None, :, :]) ** 2).sum(-1)
    d[np.arange(200), i] = np.inf
    j = d.argmin(1)
    E = np.stack([i, j], 1).astype(np.int32)
    return V, F.astype(np.int32), E, ref.astype(np.int32), G


def _diag(V):
    return float(np.linalg.norm(V.max(0) - V.min(0)))


@pytest.mark.parametrize("rigidity", [1.0, 0.1])
def test_linear_estimation(cuda, orc, rigidity):
    V, F, E, ref, G = _problem()
    ref_out = orc.solve_linear(V, F, E, ref, G, rigidity, with_rot=0)
    Vt = torch.from_numpy(V.copy()).cuda()
    it, res = PD.SolveLinear(Vt, torch.from_numpy(F), torch.from_numpy(E), torch.from_numpy(ref),
                             torch.from_numpy(G), rigidity, 0)
    assert res <= 1e-13 and it > 0
    err = np.abs(Vt.cpu().numpy() - ref_out).max()
    assert err <= 1e-6 * _diag(V), (err, it)


@pytest.mark.parametrize("rigidity", [1.0, 3.0])
def test_linear_estimation_with_rot(cuda, orc, rigidity):
    rng = np.random.Generator(np.random.PCG64(8))
    V, F = meshgen.icosphere(3)
    V = (0.4 * V + 0.5).astype(np.float32)
    # targets: a twist about z, a scale and a little noise
    c = V - 0.5
    ang = 0.8 * c[:, 2:3]
    T = np.concatenate([c[:, :1] * np.cos(ang) - c[:, 1:2] * np.sin(ang),
                        c[:, :1] * np.sin(ang) + c[:, 1:2] * np.cos(ang), c[:, 2:3]], 1) * 1.2 + 0.5
    T = (T + 0.003 * rng.standard_normal(T.shape)).astype(np.float32)
    ref_out = orc.solve_linear(V, F, None, None, T, rigidity, with_rot=1)
    Vt = torch.from_numpy(V.copy())  # a CPU tensor, updated in place
    it, res = PD.SolveLinear(Vt, torch.from_numpy(F.astype(np.int32)), None, None, torch.from_numpy(T), rigidity, 1)
    assert res <= 1e-13
    err = np.abs(Vt.numpy() - ref_out).max()
    assert err <= 1e-6 * _diag(V), (err, it)


def test_solve_linear_errors(cuda):
    V, F, E, ref, G = _problem(level=2)
    bad = ref.copy()
    bad[3] = len(G) + 5
    with pytest.raises(RuntimeError, match="reference index"):
        PD.SolveLinear(torch.from_numpy(V.copy()).cuda(), torch.from_numpy(F), torch.from_numpy(E),
                       torch.from_numpy(bad), torch.from_numpy(G), 1.0, 0)
    Eb = E.copy()
    Eb[0, 1] = len(V)
    with pytest.raises(RuntimeError, match="out of range"):
        PD.SolveLinear(torch.from_numpy(V.copy()).cuda(), torch.from_numpy(F), torch.from_numpy(Eb),
                       torch.from_numpy(ref), torch.from_numpy(G), 1.0, 0)
    with pytest.raises(RuntimeError, match="did not reach"):
        PD.SolveLinear(torch.from_numpy(V.copy()).cuda(), torch.from_numpy(F), torch.from_numpy(E),
                       torch.from_numpy(ref), torch.from_numpy(G), 1.0, 0, tol=1e-30, max_iter=40)
