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

Every evaluation of the MLP is one fused libmeshode kernel (mo_mlp_fwd:
the four layers of a 64-vertex tile with its activations kept on chip, and
the RK4 stage update), its vector-Jacobian product another (mo_mlp_bwd), and
the 256x256 weight gradients a split-K kernel over the four stages of a step
(mo_mlp_wgrad); all FP32 (packed FFMA2), no library GEMM.
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


MLP_WIDTH = 256  # the fused kernels' hidden width; narrower MLPs run zero-padded


class _Packed:
    """The parameters as the fused kernels take them: zero-padded to the
    kernels' width (exact: a padded unit's pre-activation and outgoing
    weights are 0), with W2 and W3 also transposed for the forward."""

    def __init__(self, params):
        W1, b1, W2, b2, W3, b3, W4, b4 = [p.detach() for p in params]
        m = W1.shape[0]
        M = L.lib().mo_mlp_width()
        if m > M:
            raise RuntimeError("hidden width %d exceeds the fused kernels' %d" % (m, M))
        self.m, self.M = m, M
        dev = W1.device

        def pad(t, shape):
            out = torch.zeros(shape, dtype=torch.float32, device=dev)
            out[tuple(slice(0, k) for k in t.shape)] = t
            return out

        self.W1, self.b1 = pad(W1, (M, 3)), pad(b1, (M,))
        self.W2, self.b2 = pad(W2, (M, M)), pad(b2, (M,))
        self.W3, self.b3 = pad(W3, (M, M)), pad(b3, (M,))
        self.W4, self.b4 = pad(W4, (3, M)), b4.contiguous().float()
        self.W2T = torch.empty_like(self.W2)
        self.W3T = torch.empty_like(self.W3)
        s = stream_ptr()
        call("mo_mlp_transpose", ptr(self.W2), ptr(self.W2T), s)
        call("mo_mlp_transpose", ptr(self.W3), ptr(self.W3T), s)

    def grads(self):
        M = self.M
        return [torch.zeros(sh, dtype=torch.float32, device=self.W1.device)
                for sh in ((M, 3), (M,), (M, M), (M,), (M, M), (M,), (3, M), (3,))]

    def unpad(self, g):
        m = self.m
        return [g[0][:m].contiguous(), g[1][:m].contiguous(), g[2][:m, :m].contiguous(), g[3][:m].contiguous(),
                g[4][:m, :m].contiguous(), g[5][:m].contiguous(), g[6][:, :m].contiguous(), g[7]]


def _fwd(P, u, x, a, w, init_acc, unext, acc, store=None, astride=0):
    """One fused MLP evaluation k = f(u) with the RK4 update
    unext = x + a*k, acc = (init ? x : acc) + w*k (mo_mlp_fwd); store: the
    stage's Z1 H1 Z2 H2 Z3 H3 at stride astride."""
    call("mo_mlp_fwd", ptr(u), ptr(x), u.shape[0], ptr(P.W1), ptr(P.b1), ptr(P.W2T), ptr(P.b2), ptr(P.W3T),
         ptr(P.b3), ptr(P.W4), ptr(P.b4), float(a), float(w), int(init_acc), ptr(unext), ptr(acc), ptr(store),
         int(astride), stream_ptr())


class _StepStore:
    """The activations of one RK4 step's four evaluations:
    act [6][4][n][M] (Z1 H1 Z2 H2 Z3 H3 of stages 1..4) and the stage
    inputs u2..u4."""

    def __init__(self, n, M, dev):
        self.n, self.M = n, M
        self.act = torch.empty(6 * 4 * n * M, dtype=torch.float32, device=dev)
        self.u = [None, torch.empty(n, 3, dtype=torch.float32, device=dev),
                  torch.empty(n, 3, dtype=torch.float32, device=dev), torch.empty(n, 3, dtype=torch.float32, device=dev)]

    def stage(self, s):
        return self.act[s * self.n * self.M:], 4 * self.n * self.M

    def array(self, a):
        """Array a (0 Z1, 1 H1, 2 Z2, 3 H2, 4 Z3, 5 H3) of all four stages, [4n, M]."""
        return self.act[a * 4 * self.n * self.M:(a + 1) * 4 * self.n * self.M]


def _rk4_step(P, x, h, st=None):
    """One classic RK4 step of the fused evaluations; with st, the stages'
    activations and inputs are kept there.  Returns x_next."""
    acc = torch.empty_like(x)
    if st is None:
        u2, u3, u4 = torch.empty_like(x), torch.empty_like(x), torch.empty_like(x)
    else:
        u2, u3, u4 = st.u[1], st.u[2], st.u[3]
    ss = [st.stage(k) if st is not None else (None, 0) for k in range(4)]
    _fwd(P, x, x, h / 2, h / 6, 1, u2, acc, *ss[0])
    _fwd(P, u2, x, h / 2, h / 3, 0, u3, acc, *ss[1])
    _fwd(P, u3, x, h, h / 3, 0, u4, acc, *ss[2])
    _fwd(P, u4, x, 0.0, h / 6, 0, None, acc, *ss[3])
    return acc


class _Backward:
    """Work buffers of the adjoint: the stage gradients g_z3, g_z2 of the
    four evaluations of a step ([2][4][n][M]), the per-warp partial rows of
    the small gradients and the split partials of the weight gradients."""

    def __init__(self, n, M, dev):
        lib = L.lib()
        self.n, self.M = n, M
        self.tiles = int(lib.mo_mlp_tiles(n))
        self.pw = int(lib.mo_mlp_partial_floats())
        self.gz = torch.empty(2 * 4 * n * M, dtype=torch.float32, device=dev)
        self.partial = torch.empty(4 * self.tiles * 8 * self.pw, dtype=torch.float32, device=dev)
        self.splits = max(1, min(2 * torch.cuda.get_device_properties(dev).multi_processor_count // 4,
                                 (4 * n) // 256))
        self.wpart = torch.empty(int(lib.mo_mlp_wgrad_partial_bytes(self.splits)) // 4, dtype=torch.float32,
                                 device=dev)
        self.gu = [torch.empty(n, 3, dtype=torch.float32, device=dev) for _ in range(4)]
        self.red = torch.empty(int(lib.mo_mlp_partial_reduce_bytes()) // 4, dtype=torch.float32, device=dev)

    def stage_vjp(self, P, st, s, u, gk):
        """dL/du of evaluation s (0..3) of the step for dL/dk = gk."""
        n, M = self.n, self.M
        act, astride = st.stage(s)
        gz3 = self.gz[s * n * M:]
        gz2 = self.gz[(4 + s) * n * M:]
        part = self.partial[s * self.tiles * 8 * self.pw:]
        call("mo_mlp_bwd", ptr(gk), ptr(u), n, ptr(P.W1), ptr(P.W2), ptr(P.W3), ptr(P.W4), ptr(act), int(astride),
             ptr(gz3), ptr(gz2), ptr(self.gu[s]), ptr(part), stream_ptr())
        return self.gu[s]

    def weights(self, st, grads, stream=None):
        """The parameter gradients of the step's four evaluations, added to
        grads (on `stream`, default the current one)."""
        n, M = self.n, self.M
        dW1, db1, dW2, db2, dW3, db3, dW4, db4 = grads
        s = stream_ptr(stream)
        call("mo_mlp_partial_reduce", ptr(self.partial), 4 * self.tiles * 8, ptr(self.red), ptr(dW4), ptr(db4),
             ptr(db3), ptr(db2), ptr(db1), ptr(dW1), s)
        call("mo_mlp_wgrad", ptr(self.gz), ptr(st.array(3)), 4 * n, self.splits, ptr(self.wpart), ptr(dW3), s)
        call("mo_mlp_wgrad", ptr(self.gz[4 * n * M:]), ptr(st.array(1)), 4 * n, self.splits, ptr(self.wpart),
             ptr(dW2), s)


class ODEFlow(Function):
    """x(1) = RK4^steps(x(0)) under the velocity MLP, with an adjoint
    backward on the fused kernels.  store=False: checkpointed (states at
    step starts kept, each step's stage activations recomputed in the
    backward: one step's activations in memory); store=True: every step's
    activations kept from the forward (no recompute).  Both give the same
    gradients bit for bit (the recompute repeats the same kernels)."""

    @staticmethod
    def forward(ctx, x0, steps, store, W1, b1, W2, b2, W3, b3, W4, b4):
        P = _Packed((W1, b1, W2, b2, W3, b3, W4, b4))
        steps = int(steps)
        h = 1.0 / steps
        x = x0.detach().contiguous().float()
        n = x.shape[0]
        ckpt = torch.empty(steps, n, 3, dtype=torch.float32, device=x.device)
        ctx.stores = [] if store else None
        for k in range(steps):
            ckpt[k].copy_(x)
            st = _StepStore(n, P.M, x.device) if store else None
            x = _rk4_step(P, x, h, st)
            if store:
                ctx.stores.append(st)
        ctx.P = P
        ctx.save_for_backward(ckpt)
        ctx.steps = steps
        return x

    @staticmethod
    def backward(ctx, a_out):
        (ckpt,) = ctx.saved_tensors
        P = ctx.P
        steps = ctx.steps
        h = 1.0 / steps
        n = ckpt.shape[1]
        grads = P.grads()
        a = a_out.contiguous().float()
        dev = a.device
        main = torch.cuda.current_stream(dev)
        # The weight gradients of step k (reads of its activations and stage
        # gradients, adds into grads) run on a side stream while the main
        # stream recomputes and back-propagates step k-1 into the other of
        # two buffer sets; they fill the tail waves of those launches.  All
        # additions into grads are on the side stream, in step order.
        side = torch.cuda.Stream(device=dev)
        Bs = [_Backward(n, P.M, dev), _Backward(n, P.M, dev)]
        works = [None, None] if ctx.stores is not None else [_StepStore(n, P.M, dev), _StepStore(n, P.M, dev)]
        done = [None, None]   # side-stream event after the last use of each buffer set
        held = [None, None]   # stored activations kept alive until the side stream is past them
        for k in reversed(range(steps)):
            j = k & 1
            if done[j] is not None:
                main.wait_event(done[j])
            B = Bs[j]
            xk = ckpt[k]
            if ctx.stores is not None:
                st = ctx.stores[k]
                ctx.stores[k] = None
                held[j] = st  # freed once its weight gradients have run
            else:
                st = works[j]
                _rk4_step(P, xk, h, st)
            us = [xk, st.u[1], st.u[2], st.u[3]]
            dk4 = a * (h / 6)
            g4 = B.stage_vjp(P, st, 3, us[3], dk4)
            dx = a + g4
            g3 = B.stage_vjp(P, st, 2, us[2], a * (h / 3) + h * g4)
            dx += g3
            g2 = B.stage_vjp(P, st, 1, us[1], a * (h / 3) + (h / 2) * g3)
            dx += g2
            g1 = B.stage_vjp(P, st, 0, us[0], a * (h / 6) + (h / 2) * g2)
            dx += g1
            ready = torch.cuda.Event()
            ready.record(main)
            side.wait_event(ready)
            B.weights(st, grads, stream=side)
            done[j] = torch.cuda.Event()
            done[j].record(side)
            a = dx
        main.wait_stream(side)
        held = None
        ctx.stores = None
        ctx.P = None
        return (a, None, None) + tuple(P.unpad(grads))


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
