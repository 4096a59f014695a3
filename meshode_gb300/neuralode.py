"""Velocity-field ODE deformation with a checkpointed RK4 adjoint.

The reference's NeuralODE variant (src/python/layers/neuralode_fast.py:7-64,
driven by src/python/cad_neural_deform2.py:51-86) deforms the source by
integrating a learned velocity field with torchdiffeq's RK4 and fits it with
the graph/DF losses, back-propagating through the stored RK4 graph.  Here:

* the velocity field is an MLP 3 -> m -> m -> m -> 3 with softplus
  (m = 256, Xavier-uniform weights from ``torch.manual_seed(seed)``, zero
  biases), autonomous (no time input);
* x(1) = RK4(x(0)) with ``steps`` fixed steps over t in [0, 1];
* the fit loss at t = 1 is the GPU DistanceFieldLoss (0.5 sum d^2) plus
  rigidity^2 * RigidEdgeLoss (0.5 sum |r|^2) over the source faces;
* the backward pass is a checkpointed adjoint: only the state at the start
  of every RK4 step is kept; each step's four stage activations are
  recomputed and back-propagated in reverse, accumulating the parameter
  gradients (``store_activations=True`` keeps every stage's activations
  from the forward instead: plain autograd's memory, no recompute, the same
  gradients bit for bit).

The m x m layers are cuBLAS fp32 GEMMs (TF32 must be off:
``torch.backends.cuda.matmul.allow_tf32 = False``, torch's default); the
3-wide layers, bias + softplus epilogues, RK4 stage updates and the backward
gates are libmeshode kernels (mo_mlp_*, mo_bias_softplus, mo_softplus_bwd).
"""
import math

import torch
from torch.autograd import Function

from . import _lib as L
from . import pyDeform as PD
from ._lib import call, ptr, stream_ptr

PARAM_NAMES = ("W1", "b1", "W2", "b2", "W3", "b3", "W4", "b4")


def init_params(hidden=256, seed=4, device="cuda"):
    """Xavier-uniform weights (torch.manual_seed(seed)), zero biases."""
    torch.manual_seed(seed)
    shapes = [(hidden, 3), (hidden, hidden), (hidden, hidden), (3, hidden)]
    out = []
    for shp in shapes:
        W = torch.empty(shp, dtype=torch.float32)
        torch.nn.init.xavier_uniform_(W)
        out += [W.to(device), torch.zeros(shp[0], dtype=torch.float32, device=device)]
    return out


class _Stage:
    __slots__ = ("u", "z1", "h1", "z2", "h2", "z3", "h3")


def _stage(params, u, x, a, w, init_acc, unext, acc, store):
    """One MLP evaluation k = f(u) fused with the RK4 update
    unext = x + a*k, acc = (init ? x : acc) + w*k."""
    W1, b1, W2, b2, W3, b3, W4, b4 = params
    n, m = u.shape[0], W1.shape[0]
    s = stream_ptr()
    z1 = torch.empty(n, m, dtype=torch.float32, device=u.device) if store else None
    h1 = torch.empty(n, m, dtype=torch.float32, device=u.device)
    call("mo_mlp_in", ptr(u), n, ptr(W1), ptr(b1), m, ptr(z1), ptr(h1), s)
    z2 = torch.matmul(h1, W2.t())
    h2 = torch.empty_like(z2)
    call("mo_bias_softplus", ptr(z2), n, m, ptr(b2), ptr(h2), s)
    z3 = torch.matmul(h2, W3.t())
    h3 = torch.empty_like(z3)
    call("mo_bias_softplus", ptr(z3), n, m, ptr(b3), ptr(h3), s)
    call("mo_mlp_out_rk4", ptr(h3), n, m, ptr(W4), ptr(b4), ptr(x), float(a), float(w), int(init_acc), None,
         ptr(unext), ptr(acc), s)
    if not store:
        return None
    st = _Stage()
    st.u, st.z1, st.h1, st.z2, st.h2, st.z3, st.h3 = u, z1, h1, z2, h2, z3, h3
    return st


def _rk4_step(params, x, h, store=False):
    """One classic RK4 step; returns (x_next, [4 stage records] or None)."""
    acc = torch.empty_like(x)
    u2, u3, u4 = torch.empty_like(x), torch.empty_like(x), torch.empty_like(x)
    s1 = _stage(params, x, x, h / 2, h / 6, 1, u2, acc, store)
    s2 = _stage(params, u2, x, h / 2, h / 3, 0, u3, acc, store)
    s3 = _stage(params, u3, x, h, h / 3, 0, u4, acc, store)
    s4 = _stage(params, u4, x, 0.0, h / 6, 0, None, acc, store)
    return acc, ([s1, s2, s3, s4] if store else None)


def _vjp(params, grads, st, g_out):
    """Back-propagate g_out = dL/dk through one MLP evaluation; accumulates
    the parameter gradients into `grads`, returns dL/du."""
    W1, b1, W2, b2, W3, b3, W4, b4 = params
    dW1, db1, dW2, db2, dW3, db3, dW4, db4 = grads
    n, m = st.u.shape[0], W1.shape[0]
    s = stream_ptr()
    dW4.addmm_(g_out.t(), st.h3)
    db4.add_(g_out.sum(0))
    g_z3 = torch.empty(n, m, dtype=torch.float32, device=g_out.device)
    call("mo_mlp_out_bwd", ptr(g_out), n, m, ptr(W4), ptr(st.z3), ptr(g_z3), s)
    dW3.addmm_(g_z3.t(), st.h2)
    db3.add_(g_z3.sum(0))
    g_z2 = torch.matmul(g_z3, W3)
    call("mo_softplus_bwd", ptr(g_z2), ptr(st.z2), n * m, s)
    dW2.addmm_(g_z2.t(), st.h1)
    db2.add_(g_z2.sum(0))
    g_z1 = torch.matmul(g_z2, W2)
    call("mo_softplus_bwd", ptr(g_z1), ptr(st.z1), n * m, s)
    dW1.addmm_(g_z1.t(), st.u)
    db1.add_(g_z1.sum(0))
    g_u = torch.empty(n, 3, dtype=torch.float32, device=g_out.device)
    call("mo_mlp_in_bwd", ptr(g_z1), n, m, ptr(W1), ptr(g_u), 0, s)
    return g_u


class ODEFlow(Function):
    """x(1) = RK4^steps(x(0)) under the velocity MLP, with an adjoint
    backward.  store=False: checkpointed (states at step starts kept, each
    step's stage activations recomputed in the backward: one step's
    activations in memory); store=True: every stage's activations kept from
    the forward (the memory of plain autograd, no recompute).  Both give the
    same gradients bit for bit (the recompute repeats the same kernels)."""

    @staticmethod
    def forward(ctx, x0, steps, store, W1, b1, W2, b2, W3, b3, W4, b4):
        params = [t.detach().contiguous() for t in (W1, b1, W2, b2, W3, b3, W4, b4)]
        steps = int(steps)
        h = 1.0 / steps
        x = x0.detach().contiguous()
        ckpt = torch.empty(steps, x.shape[0], 3, dtype=torch.float32, device=x.device)
        ctx.stages = [] if store else None
        for k in range(steps):
            ckpt[k].copy_(x)
            x, st = _rk4_step(params, x, h, store=bool(store))
            if store:
                ctx.stages.append(st)
        ctx.save_for_backward(ckpt, *params)
        ctx.steps = steps
        return x

    @staticmethod
    def backward(ctx, a_out):
        ckpt, *params = ctx.saved_tensors
        steps = ctx.steps
        h = 1.0 / steps
        grads = [torch.zeros_like(p) for p in params]
        a = a_out.contiguous().float()
        for k in reversed(range(steps)):
            if ctx.stages is not None:
                st = ctx.stages[k]
                ctx.stages[k] = None  # freed as the backward passes it
            else:
                _, st = _rk4_step(params, ckpt[k], h, store=True)
            dk4 = a * (h / 6)
            g4 = _vjp(params, grads, st[3], dk4)
            dx = a + g4
            g3 = _vjp(params, grads, st[2], a * (h / 3) + h * g4)
            dx += g3
            g2 = _vjp(params, grads, st[1], a * (h / 3) + (h / 2) * g3)
            dx += g2
            g1 = _vjp(params, grads, st[0], a * (h / 6) + (h / 2) * g2)
            dx += g1
            a = dx
        ctx.stages = None
        return (a, None, None) + tuple(grads)


class FitLossFunction(Function):
    """0.5 sum d(x)^2 + rigidity^2 * 0.5 sum |r|^2 of the deformed source
    (the GraphLoss2Function objective, src/python/layers/graph_loss2_layer.py:
    9-41, with the source faces' half-edges as the edge set)."""

    @staticmethod
    def forward(ctx, X, F, pid, rigidity2):
        lossD, gD = PD.DistanceFieldLoss_fwd_bwd(X, pid)
        lossR = PD.RigidEdgeLoss_forward(X, F, pid)
        gR = PD.RigidEdgeLoss_backward(X, F, pid)
        ctx.save_for_backward(gD, gR)
        ctx.r2 = float(rigidity2)
        return lossD.double().sum() * 0.5 + lossR.double().sum() * 0.5 * ctx.r2

    @staticmethod
    def backward(ctx, grad_h):
        gD, gR = ctx.saved_tensors
        return grad_h.float() * (gD + gR * ctx.r2), None, None, None


class NeuralODEDeformer:
    """The velocity-field fit: source normalised by the target template, the
    MLP parameters are the optimisation variables (torch.optim.Adam)."""

    def __init__(self, src_V, src_F, tar_V, tar_F, grid_resolution=128, rigidity=0.1, hidden=256, steps=20,
                 seed=4, lr=1e-3, store_activations=False):
        L.require_cuda()
        if torch.backends.cuda.matmul.allow_tf32:
            raise RuntimeError("TF32 matmul is enabled; the ODE fit needs fp32 GEMMs "
                               "(torch.backends.cuda.matmul.allow_tf32 = False)")
        dev = torch.device("cuda", torch.cuda.current_device())
        self.pid = PD.InitializeDeformTemplate(tar_V, tar_F, 0, grid_resolution)
        self.x0 = src_V.detach().to(dev).float().contiguous().clone()
        PD.NormalizeByTemplate(self.x0, self.pid)
        self.F = src_F.detach().to(dev).contiguous()
        PD.StoreRigidityInformation(self.x0, self.F, self.pid)
        self.rigidity2 = float(torch.tensor(rigidity * rigidity, dtype=torch.float32))
        self.steps = int(steps)
        # False: checkpointed adjoint (low memory); True: activations kept (faster)
        self.store_activations = bool(store_activations)
        self.params = [p.requires_grad_(True) for p in init_params(hidden, seed, dev)]
        self.opt = torch.optim.Adam(self.params, lr=lr)

    def deformed(self):
        return ODEFlow.apply(self.x0, self.steps, self.store_activations, *self.params)

    def loss(self):
        return FitLossFunction.apply(self.deformed(), self.F, self.pid, self.rigidity2)

    def step(self):
        self.opt.zero_grad()
        L_ = self.loss()
        L_.backward()
        self.opt.step()
        return L_.detach()
