"""The velocity-field ODE deformation: the fused MLP kernels' checkpointed
RK4 adjoint against an FP64 reference.

The FP64 reference is the same model written with torch float64 autograd on
the CPU: the MLP, 20 classic RK4 steps, the distance lookup restated from
UniformGrid::distance<double> (src/lib/uniformgrid.cc:18-83: truncation
toward zero, the out-of-box penalty without the N-1 slab, the 0.2 cutoff) on
the GPU grid, and the rigidity term with the fp32 rest offsets.  It is
itself checked against FP64 central differences (h = 1e-6).  The GPU fp32
gradients of every parameter must lie within 1e-5 of the FP64 gradient's
scale (max |g64|), the tolerance the configuration states.  Widths 16 and 64 run zero-padded
in the 256-wide kernels; 256 is the configuration's own width, checked on
a small source here and at full size (50k vertices, 128^3) against FP64
autograd on the GPU.
"""
import numpy as np
import pytest
import torch

from meshode_gb300 import meshgen, neuralode
from meshode_gb300 import pyDeform as PD

pytestmark = pytest.mark.gpu


def _lookup64(grid, N, P):
    """UniformGrid::distance<double> on a [z][y][x] grid, differentiable in P."""
    s = P * N
    idx = torch.trunc(s).long()
    out = ((idx < 0) | (idx >= N - 1)).any(1)
    Cf = float(N - 1 - 1e-3)
    pen = torch.where(idx < 0, -s, torch.where(idx >= N, s - Cf, torch.zeros_like(s))).sum(1)
    i = idx.clamp(0, N - 2)
    w = s - i.double()
    res = torch.zeros(P.shape[0], dtype=torch.float64, device=P.device)
    for dz in (0, 1):
        for dy in (0, 1):
            for dx in (0, 1):
                wt = (w[:, 0] if dx else 1 - w[:, 0]) * (w[:, 1] if dy else 1 - w[:, 1]) * \
                     (w[:, 2] if dz else 1 - w[:, 2])
                res = res + wt * grid[i[:, 2] + dz, i[:, 1] + dy, i[:, 0] + dx]
    res = torch.where(res > 0.2, torch.zeros_like(res), res)
    return torch.where(out, pen, res)


def _model64(params, x0, steps, grid, N, F, off, r2):
    W1, b1, W2, b2, W3, b3, W4, b4 = params
    sp = torch.nn.functional.softplus

    def f(x):
        return sp(sp(sp(x @ W1.t() + b1) @ W2.t() + b2) @ W3.t() + b3) @ W4.t() + b4

    h = 1.0 / steps
    x = x0
    for _ in range(steps):
        k1 = f(x)
        k2 = f(x + h / 2 * k1)
        k3 = f(x + h / 2 * k2)
        k4 = f(x + h * k3)
        x = x + h / 6 * (k1 + 2 * k2 + 2 * k3 + k4)
    d = _lookup64(grid, N, x)
    v0 = x[F[:, [0, 1, 2]].reshape(-1)]
    v1 = x[F[:, [1, 2, 0]].reshape(-1)]
    r = v1 - v0 - off
    return 0.5 * (d * d).sum() + r2 * 0.5 * (r * r).sum()


@pytest.fixture(scope="module")
def problem(cuda):
    rng = np.random.Generator(np.random.PCG64(4))
    Vs, Fs = meshgen.icosphere(2)
    Vt, Ft = meshgen.icosphere(3)
    Vt = meshgen.displace(Vt, rng)
    src_V = torch.from_numpy((Vs * 0.8).astype(np.float32))
    src_F = torch.from_numpy(Fs.astype(np.int32))
    return src_V, src_F, torch.from_numpy(Vt.astype(np.float32)), torch.from_numpy(Ft.astype(np.int32))


@pytest.mark.parametrize("hidden", [16, 64, 256])
def test_adjoint_vs_fp64(problem, hidden):
    src_V, src_F, tar_V, tar_F = problem
    N, steps = 32, 20
    dfm = neuralode.NeuralODEDeformer(src_V, src_F, tar_V, tar_F, grid_resolution=N, rigidity=0.1, hidden=hidden,
                                      steps=steps, seed=4)
    # scale the last layer up so that the flow moves the mesh noticeably
    with torch.no_grad():
        dfm.params[6].mul_(20.0)
    loss = dfm.loss()
    loss.backward()
    g32 = [p.grad.detach().double().cpu() for p in dfm.params]
    grid = PD.GetDistanceField(dfm.pid).double().cpu()
    x0 = dfm.x0.double().cpu()
    F = src_F.long()
    off = PD.GetParams(dfm.pid).edge.offsets.double().cpu()
    p64 = [p.detach().double().cpu().requires_grad_(True) for p in dfm.params]
    L64 = _model64(p64, x0, steps, grid, N, F, off, dfm.rigidity2)
    L64.backward()
    assert abs(float(loss) - float(L64)) <= 1e-5 * abs(float(L64)) + 1e-9
    for name, a, b in zip(neuralode.PARAM_NAMES, g32, p64):
        scale = b.grad.abs().max().item()
        err = (a - b.grad).abs().max().item()
        assert err <= 1e-5 * max(scale, 1e-12), (name, err, scale)
    # the FP64 reference against central differences (h = 1e-6)
    if hidden == 256:
        return  # the FP64 reference is pinned by central differences at the smaller widths
    rng = np.random.Generator(np.random.PCG64(1))
    for pi in (0, 2, 5, 6, 7):
        P = p64[pi]
        for flat in rng.choice(P.numel(), size=3, replace=False):
            with torch.no_grad():
                q = [t.detach().clone() for t in p64]
                q[pi].view(-1)[flat] += 1e-6
                lp = _model64(q, x0, steps, grid, N, F, off, dfm.rigidity2)
                q[pi].view(-1)[flat] -= 2e-6
                lm = _model64(q, x0, steps, grid, N, F, off, dfm.rigidity2)
            fd = float(lp - lm) / 2e-6
            ad = float(P.grad.view(-1)[flat])
            assert abs(fd - ad) <= 1e-5 * max(abs(ad), P.grad.abs().max().item()) + 1e-7, (pi, flat, fd, ad)


def test_fit_decreases_loss(problem):
    src_V, src_F, tar_V, tar_F = problem
    dfm = neuralode.NeuralODEDeformer(src_V, src_F, tar_V, tar_F, grid_resolution=32, rigidity=0.1, hidden=64,
                                      steps=10, seed=4, lr=1e-3)
    l0 = float(dfm.step())
    for _ in range(30):
        l1 = float(dfm.step())
    assert l1 < l0


def test_stored_activations_give_the_same_gradients(cuda):
    """store_activations=True skips the adjoint's recompute; the gradients
    and the updated parameters are the checkpointed mode's, bit for bit."""
    rng = np.random.Generator(np.random.PCG64(9))
    Vs, Fs = meshgen.icosphere(3)
    Vt, Ft = meshgen.icosphere(4)
    Vt = meshgen.displace(Vt, rng)
    args = (torch.from_numpy((Vs * 0.8).astype(np.float32)), torch.from_numpy(Fs.astype(np.int32)),
            torch.from_numpy(Vt.astype(np.float32)), torch.from_numpy(Ft.astype(np.int32)))
    runs = []
    for store in (False, True):
        d = neuralode.NeuralODEDeformer(*args, grid_resolution=32, rigidity=0.1, hidden=64, steps=5, seed=4,
                                        store_activations=store)
        losses = [d.step() for _ in range(3)]
        runs.append((losses, [p.detach().clone() for p in d.params]))
    (la, pa), (lb, pb) = runs
    assert all(torch.equal(x, y) for x, y in zip(la, lb))
    assert all(torch.equal(x, y) for x, y in zip(pa, pb))



def test_config4_full_size_vs_fp64_on_gpu(cuda):
    """The ODE configuration at full size: a 50k-vertex source, the 256-wide
    MLP, 20 RK4 steps, a 128^3 grid, rigidity 0.1.  The fused kernels'
    gradients of every parameter against the same model in float64 torch
    autograd on the GPU, within 1e-5 of each gradient's scale."""
    rng = np.random.Generator(np.random.PCG64(4))
    Vs, Fs = meshgen.cubesphere_for_vertices(50_000)
    Vt, Ft = meshgen.icosphere(6)
    Vt = meshgen.displace(Vt, rng)
    dfm = neuralode.NeuralODEDeformer(torch.from_numpy((Vs * 0.8).astype(np.float32)),
                                      torch.from_numpy(Fs.astype(np.int32)), torch.from_numpy(Vt.astype(np.float32)),
                                      torch.from_numpy(Ft.astype(np.int32)), grid_resolution=128, rigidity=0.1,
                                      hidden=256, steps=20, seed=4)
    with torch.no_grad():
        dfm.params[6].mul_(20.0)
    loss = dfm.loss()
    loss.backward()
    g32 = [p.grad.detach().double() for p in dfm.params]
    N = 128
    grid = PD.GetDistanceField(dfm.pid).double()
    F = dfm.F.long()
    off = PD.GetParams(dfm.pid).edge.offsets.double()
    p64 = [p.detach().double().requires_grad_(True) for p in dfm.params]
    L64 = _model64(p64, dfm.x0.double(), 20, grid, N, F, off, dfm.rigidity2)
    L64.backward()
    assert abs(float(loss) - float(L64)) <= 1e-5 * abs(float(L64)) + 1e-9
    for name, a, b in zip(neuralode.PARAM_NAMES, g32, p64):
        scale = b.grad.abs().max().item()
        err = (a - b.grad).abs().max().item()
        assert err <= 1e-5 * max(scale, 1e-12), (name, err, scale)
