"""torch.autograd.Function layers over the GPU pyDeform (drop-in for the
reference's src/python/layers/rigid_loss_layer.py and graph_loss_layer.py).

The forward and backward passes call the hand-written kernels through
``meshode_gb300.pyDeform``; loss values and gradients stay on the GPU (the
reference copied V to the host and back on every call,
graph_loss_layer.py:15,23,36,42).
"""
import torch
from torch import nn
from torch.autograd import Function

from . import pyDeform


class RigidLossFunction(Function):
    """rigid_loss_layer.py:7-27: 0.5*sum d^2 + 0.5*sum r^2, backward
    grad_h*(gD + gR)."""

    @staticmethod
    def forward(ctx, src_V, src_F, param_id):
        pid = int(param_id)
        lossD = pyDeform.DistanceFieldLoss_forward(src_V, pid) * 0.5
        lossR = pyDeform.RigidEdgeLoss_forward(src_V, src_F, pid) * 0.5
        ctx.save_for_backward(src_V)
        ctx.src_F = src_F
        ctx.pid = pid
        return lossD.sum() + lossR.sum()

    @staticmethod
    def backward(ctx, grad_h):
        (src_V,) = ctx.saved_tensors
        gD = pyDeform.DistanceFieldLoss_backward(src_V, ctx.pid)
        gR = pyDeform.RigidEdgeLoss_backward(src_V, ctx.src_F, ctx.pid)
        return grad_h * (gD + gR), None, None


class RigidLossLayer(nn.Module):
    """rigid_loss_layer.py:30-41: builds the target template (grid
    ``grid_resolution``, 64 in the reference), normalises src_V in place and
    stores the rigidity information."""

    def __init__(self, src_V, src_F, tar_V, tar_F, grid_resolution=64):
        super().__init__()
        self.param_id = torch.tensor(pyDeform.InitializeDeformTemplate(tar_V, tar_F, 0, grid_resolution))
        pyDeform.NormalizeByTemplate(src_V, int(self.param_id))
        pyDeform.StoreRigidityInformation(src_V, src_F, int(self.param_id))

    def forward(self, src_V, src_F):
        return RigidLossFunction.apply(src_V, src_F, int(self.param_id))


def Finalize(src_V, param_id):
    """rigid_loss_layer.py:43-44."""
    pyDeform.DenormalizeByTemplate(src_V, int(param_id))


class GraphLossFunction(Function):
    """graph_loss_layer.py:9-43: 0.5*sum d^2 + rigidity^2 * 0.5*sum r^2; the
    DF gradient is zeroed where 0.5*d^2 >= 0.5*0.03*0.03."""

    MASK = 0.5 * 0.03 * 0.03

    @staticmethod
    def forward(ctx, src_V, src_E, rigidity2, param_id):
        pid = int(param_id)
        r2 = float(rigidity2)
        lossD, gD = pyDeform.DistanceFieldLoss_fwd_bwd(src_V, pid, mask_thresh=GraphLossFunction.MASK)
        lossD = lossD * 0.5
        lossR = pyDeform.GraphEdgeLoss_forward(src_V, src_E, pid) * 0.5
        ctx.save_for_backward(src_V, gD)
        ctx.src_E = src_E
        ctx.pid = pid
        ctx.r2 = r2
        return lossD.sum() + lossR.sum() * r2

    @staticmethod
    def backward(ctx, grad_h):
        src_V, gD = ctx.saved_tensors
        gR = pyDeform.GraphEdgeLoss_backward(src_V, ctx.src_E, ctx.pid)
        return grad_h * (gD + gR * ctx.r2), None, None, None


class GraphLossLayer(nn.Module):
    """graph_loss_layer.py:46-57."""

    def __init__(self, src_V, src_E, tar_V, tar_F, rigidity, d=None, grid_resolution=64):
        super().__init__()
        self.param_id = torch.tensor(pyDeform.InitializeDeformTemplate(tar_V, tar_F, 0, grid_resolution))
        pyDeform.NormalizeByTemplate(src_V, int(self.param_id))
        pyDeform.StoreGraphInformation(src_V, src_E, int(self.param_id))
        # torch.tensor(rigidity * rigidity) is float32 in the reference
        self.rigidity2 = float(torch.tensor(rigidity * rigidity, dtype=torch.float32))

    def forward(self, src_V, src_E):
        return GraphLossFunction.apply(src_V, src_E, self.rigidity2, int(self.param_id))


def GraphFinalize(src_V, src_F, src_E, src_to_graph, graph_V, rigidity, param_id):
    """graph_loss_layer.py:62-66 (the module's second Finalize): propagate the
    fitted graph back to the full mesh with SolveLinear (LinearEstimation) in
    the template's normalised frame, in place on src_V."""
    pid = int(param_id)
    pyDeform.NormalizeByTemplate(src_V, pid)
    pyDeform.SolveLinear(src_V, src_F, src_E, src_to_graph, graph_V, rigidity, 0)
    pyDeform.DenormalizeByTemplate(src_V, pid)


class ReverseLossFunction(Function):
    """reverse_loss_layer.py:14-25: ii = nearest source vertex of every
    target vertex (cKDTree in the reference, an LBVH query here), loss =
    0.5 * sum |src_V[ii] - tar_V|^2.  The indices are constants of the
    forward pass; the backward is torch's CPU autograd of that expression,
    bit for bit.  The work runs on the GPU; the loss and the gradient come
    back on src_V's device."""

    @staticmethod
    def forward(ctx, src_V, tar_V):
        from . import _lib as L
        L.require_cuda()
        dev = torch.device("cuda", torch.cuda.current_device())
        S = src_V.detach().to(dev, torch.float32).contiguous()
        T = tar_V.detach().to(dev, torch.float32).contiguous()
        if S.dim() != 2 or S.shape[1] != 3 or T.dim() != 2 or T.shape[1] != 3:
            raise RuntimeError("ReverseLossLayer expects [n,3] source and target vertices")
        ns, nt = int(S.shape[0]), int(T.shape[0])
        s = L.stream_ptr()
        idx = torch.empty(nt, dtype=torch.int32, device=dev)
        L.call("mo_nn_query", L.ptr(S), ns, L.ptr(T), nt, L.ptr(idx), None, None, 0, s)
        nb = L.lib().mo_reverse_loss_scratch_bytes(ns, nt)
        scratch = torch.empty(max(int(nb), 1), dtype=torch.uint8, device=dev)
        loss = torch.empty(1, dtype=torch.float64, device=dev)
        L.call("mo_reverse_loss_forward", L.ptr(S), ns, L.ptr(T), nt, L.ptr(idx), L.ptr(loss), L.ptr(scratch), nb,
               None, s)
        ctx.save_for_backward(S, T, idx)
        ctx.src_device = src_V.device
        return loss.to(torch.float32).reshape(()).to(src_V.device)

    @staticmethod
    def backward(ctx, grad):
        from . import _lib as L
        S, T, idx = ctx.saved_tensors
        ns, nt = int(S.shape[0]), int(T.shape[0])
        g = grad.detach().to(S.device, torch.float32).reshape(1).contiguous()
        gs = torch.empty_like(S)
        nb = L.lib().mo_reverse_loss_scratch_bytes(ns, nt)
        scratch = torch.empty(max(int(nb), 1), dtype=torch.uint8, device=S.device)
        st = torch.zeros(1, dtype=torch.int32, device=S.device)  # the forward checked the indices
        L.call("mo_reverse_loss_backward", L.ptr(S), ns, L.ptr(T), nt, L.ptr(idx), L.ptr(g), L.ptr(gs),
               L.ptr(scratch), nb, L.ptr(st), L.stream_ptr())
        return gs.to(ctx.src_device), None


class ReverseLossLayer(nn.Module):
    """reverse_loss_layer.py:10-25.  `device` is accepted for the reference's
    signature; the result is on src_V's device."""

    def forward(self, src_V, tar_V, device=None):
        return ReverseLossFunction.apply(src_V, tar_V)
