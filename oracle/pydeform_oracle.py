"""CPU oracle with the reference's ``pyDeform`` interface (test infrastructure).

This module is the oracle ``meshode_gb300.pyDeform`` is tested against: it
restates the reference's pybind11 module (src/interface/pydeform.cc:14-39) on
CPU float32 tensors, calling the C restatement in ``meshode_oracle.c`` through
ctypes.  Only tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import it.

Parity status: pinned against the reference's own sources compiled in
``oracle/_ref`` (``tests/test_ref_pin.py``); see the header of
meshode_oracle.c for what remains unpinned.
"""
import ctypes
import os

import numpy as np
import torch

from . import build as _build

_lib = None


def lib():
    """Load (building if needed) the oracle shared library."""
    global _lib
    if _lib is None:
        path = _build.build()
        L = ctypes.CDLL(path)
        P = ctypes.c_void_p
        i64 = ctypes.c_int64
        L.orc_distance_float.restype = ctypes.c_float
        L.orc_distance_float.argtypes = [P, ctypes.c_int, P]
        L.orc_distance_jet.argtypes = [P, ctypes.c_int, P, P]
        L.orc_dfloss_forward.argtypes = [P, i64, P, ctypes.c_int, P]
        L.orc_dfloss_backward.argtypes = [P, i64, P, ctypes.c_int, P]
        L.orc_edge_offsets.argtypes = [P, P, i64, ctypes.c_int, P]
        L.orc_edge_forward.argtypes = [P, P, i64, ctypes.c_int, P, P]
        L.orc_edge_backward.argtypes = [P, i64, P, i64, ctypes.c_int, P, P]
        L.orc_edge_cad_list.argtypes = [P, i64, P, i64, P]
        L.orc_edge_cad_weights.argtypes = [P, i64, P]
        L.orc_edge_forward_w.argtypes = [P, P, i64, ctypes.c_int, P, P, P]
        L.orc_edge_backward_w.argtypes = [P, i64, P, i64, ctypes.c_int, P, P, P]
        L.orc_normalize_params.argtypes = [P, i64, P, P]
        L.orc_normalize_double.argtypes = [P, i64, ctypes.c_double, P, P]
        L.orc_normalize_by_template.argtypes = [P, i64, ctypes.c_double, P]
        L.orc_denormalize_by_template.argtypes = [P, i64, ctypes.c_double, P]
        L.orc_point_tri_dist2.restype = ctypes.c_double
        L.orc_point_tri_dist2.argtypes = [P, P, P, P]
        L.orc_df_bruteforce.argtypes = [P, P, i64, ctypes.c_int, P, i64, P]
        L.orc_df_bvh.restype = ctypes.c_int
        L.orc_df_bvh.argtypes = [P, P, i64, ctypes.c_int, P, i64, P, ctypes.c_int]
        L.orc_df_bvh_timed.restype = ctypes.c_int
        L.orc_df_bvh_timed.argtypes = [P, P, i64, ctypes.c_int, P, i64, P, ctypes.c_int, P]
        L.orc_morton_codes.argtypes = [P, P, i64, P]
        L.orc_sort_codes.argtypes = [P, i64, P, P]
        L.orc_karras.argtypes = [P, ctypes.c_int, P, P]
        L.orc_trunc_i32.restype = ctypes.c_int
        L.orc_trunc_i32.argtypes = [ctypes.c_float]
        F = ctypes.c_float
        L.orc_adam_step.argtypes = [P, P, P, P, i64, F, F, F, F, F, F]
        _lib = L
    return _lib


def _p(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


def _f32(t):
    a = t.detach().cpu().numpy() if isinstance(t, torch.Tensor) else np.asarray(t)
    return np.ascontiguousarray(a, dtype=np.float32)


def _i32(t):
    a = t.detach().cpu().numpy() if isinstance(t, torch.Tensor) else np.asarray(t)
    return np.ascontiguousarray(a, dtype=np.int32)


# --------------------------------------------------------------------------
# Raw numpy-level helpers
# --------------------------------------------------------------------------
def normalize_params(V):
    """Mesh::Normalize (src/lib/mesh.cc:66-96): (scale, trans[3]) in double."""
    V = _f32(V)
    scale = np.zeros(1, np.float64)
    trans = np.zeros(3, np.float64)
    lib().orc_normalize_params(_p(V), V.shape[0], _p(scale), _p(trans))
    return float(scale[0]), trans


def normalized_double(V, scale, trans):
    """Normalised target vertices in double (mesh.cc:83-85)."""
    V = _f32(V)
    out = np.empty(V.shape, np.float64)
    tr = np.ascontiguousarray(trans, np.float64)
    lib().orc_normalize_double(_p(V), V.shape[0], scale, _p(tr), _p(out))
    return out


def df_build(Vn64, F, N, voxels=None, method="bvh", threads=0):
    """Unsigned DF of a normalised target (mesh.cc:106-152) in FP64.

    Returns sqrt(min squared distance) for every voxel (flattened [z][y][x])
    or for the given voxel indices.
    """
    Vn64 = np.ascontiguousarray(Vn64, np.float64)
    F = _i32(F)
    if voxels is None:
        nvox = N ** 3
        vox = None
    else:
        vox = np.ascontiguousarray(voxels, np.int64)
        nvox = vox.shape[0]
    out = np.empty(nvox, np.float64)
    if method == "brute":
        lib().orc_df_bruteforce(_p(Vn64), _p(F), F.shape[0], N, _p(vox), nvox, _p(out))
    else:
        rc = lib().orc_df_bvh(_p(Vn64), _p(F), F.shape[0], N, _p(vox), nvox, _p(out), threads)
        if rc != 0:
            raise RuntimeError("orc_df_bvh failed: %d" % rc)
    return out


def df_build_timed(Vn64, F, N, voxels=None, threads=0):
    """df_build through the AABB tree with its phases timed inside the
    library: (values, seconds of the serial tree build, seconds of the voxel
    queries)."""
    Vn64 = np.ascontiguousarray(Vn64, np.float64)
    F = _i32(F)
    vox = None if voxels is None else np.ascontiguousarray(voxels, np.int64)
    nvox = N ** 3 if vox is None else vox.shape[0]
    out = np.empty(max(nvox, 1), np.float64)
    t = np.zeros(2, np.float64)
    rc = lib().orc_df_bvh_timed(_p(Vn64), _p(F), F.shape[0], N, _p(vox), nvox, _p(out), threads, _p(t))
    if rc != 0:
        raise RuntimeError("orc_df_bvh_timed failed: %d" % rc)
    return out[:nvox], float(t[0]), float(t[1])


def distance_float(grid, N, p):
    g = np.ascontiguousarray(grid, np.float32)
    pp = np.ascontiguousarray(p, np.float32)
    return lib().orc_distance_float(_p(g), N, _p(pp))


def distance_jet(grid, N, p):
    g = np.ascontiguousarray(grid, np.float32)
    pp = np.ascontiguousarray(p, np.float32)
    out = np.zeros(4, np.float32)
    lib().orc_distance_jet(_p(g), N, _p(pp), _p(out))
    return out


def dfloss_forward(V, grid, N):
    V = _f32(V); g = np.ascontiguousarray(grid, np.float32)
    L = np.empty(V.shape[0], np.float32)
    lib().orc_dfloss_forward(_p(V), V.shape[0], _p(g), N, _p(L))
    return L


def dfloss_backward(V, grid, N):
    V = _f32(V); g = np.ascontiguousarray(grid, np.float32)
    Gd = np.empty((V.shape[0], 3), np.float32)
    lib().orc_dfloss_backward(_p(V), V.shape[0], _p(g), N, _p(Gd))
    return Gd


def edge_count(idx, kind):
    return idx.shape[0] * 3 if kind == 0 else idx.shape[0]


def edge_offsets(V, idx, kind):
    V = _f32(V); idx = _i32(idx)
    nh = edge_count(idx, kind)
    off = np.empty((nh, 3), np.float32)
    lib().orc_edge_offsets(_p(V), _p(idx), nh, kind, _p(off))
    return off


def edge_forward(V, idx, kind, off):
    V = _f32(V); idx = _i32(idx); off = _f32(off)
    nh = edge_count(idx, kind)
    L = np.empty((nh, 3), np.float32)
    lib().orc_edge_forward(_p(V), _p(idx), nh, kind, _p(off), _p(L))
    return L


def edge_backward(V, idx, kind, off):
    V = _f32(V); idx = _i32(idx); off = _f32(off)
    nh = edge_count(idx, kind)
    Gd = np.empty((V.shape[0], 3), np.float32)
    lib().orc_edge_backward(_p(V), V.shape[0], _p(idx), nh, kind, _p(off), _p(Gd))
    return Gd


def cad_edge_list(F, E):
    """E's edges then F's half-edges, the CAD loss's edge set (cad_layer.cc:33-67)."""
    F = _i32(F); E = _i32(E)
    out = np.empty((E.shape[0] + 3 * F.shape[0], 2), np.int32)
    lib().orc_edge_cad_list(_p(E), E.shape[0], _p(F), F.shape[0], _p(out))
    return out


def cad_edge_weights(off):
    off = _f32(off)
    lam = np.empty(off.shape[0], np.float32)
    lib().orc_edge_cad_weights(_p(off), off.shape[0], _p(lam))
    return lam


def edge_forward_w(V, idx, kind, off, w):
    V = _f32(V); idx = _i32(idx); off = _f32(off); w = _f32(w)
    nh = edge_count(idx, kind)
    L = np.empty((nh, 3), np.float32)
    lib().orc_edge_forward_w(_p(V), _p(idx), nh, kind, _p(off), _p(w), _p(L))
    return L


def edge_backward_w(V, idx, kind, off, w):
    V = _f32(V); idx = _i32(idx); off = _f32(off); w = _f32(w)
    nh = edge_count(idx, kind)
    Gd = np.empty((V.shape[0], 3), np.float32)
    lib().orc_edge_backward_w(_p(V), V.shape[0], _p(idx), nh, kind, _p(off), _p(w), _p(Gd))
    return Gd


def morton_codes(Vn32, F):
    Vn32 = _f32(Vn32); F = _i32(F)
    codes = np.empty(F.shape[0], np.uint32)
    lib().orc_morton_codes(_p(Vn32), _p(F), F.shape[0], _p(codes))
    return codes


def sort_codes(codes):
    codes = np.ascontiguousarray(codes, np.uint32)
    sc = np.empty_like(codes)
    perm = np.empty(codes.shape[0], np.int32)
    lib().orc_sort_codes(_p(codes), codes.shape[0], _p(sc), _p(perm))
    return sc, perm


def karras(sorted_codes):
    k = np.ascontiguousarray(sorted_codes, np.uint32)
    n = k.shape[0]
    left = np.zeros(max(n - 1, 0), np.int32)
    right = np.zeros(max(n - 1, 0), np.int32)
    if n > 1:
        lib().orc_karras(_p(k), n, _p(left), _p(right))
    return left, right


# --------------------------------------------------------------------------
# OBJ I/O with the reference's quirks (src/lib/mesh.cc:14-64)
# --------------------------------------------------------------------------
def read_obj(path):
    """Mesh::ReadOBJ: 'v x y z' parsed as double, 'f a b c' keeps the leading
    digits of each token (a/b/c -> a), 1-based; reading stops at the first line
    of 256 or more characters (std::istream::getline with a 256-byte buffer)."""
    V, F = [], []
    with open(path, "rb") as fh:
        for raw in fh:
            line = raw.rstrip(b"\n")
            if len(line) >= 256:
                break
            toks = line.split()
            if not toks:
                continue
            if toks[0] == b"v":
                V.append([float(t) for t in toks[1:4]])
            elif toks[0] == b"f":
                f = []
                for t in toks[1:4]:
                    i = 0
                    for ch in t:
                        if ch == ord("/"):
                            break
                        i = i * 10 + (ch - 48)
                    f.append(i - 1)
                F.append(f)
    return np.asarray(V, np.float64).reshape(-1, 3), np.asarray(F, np.int64).reshape(-1, 3)


def write_obj(path, V, F):
    """Mesh::WriteOBJ (mesh.cc:46-64): default ostream precision (%g)."""
    V = np.asarray(V, np.float64)
    F = np.asarray(F, np.int64)
    with open(path, "w") as fh:
        for v in V:
            fh.write("v %g %g %g\n" % (v[0], v[1], v[2]))
        for f in F:
            fh.write("f %d %d %d\n" % (f[0] + 1, f[1] + 1, f[2] + 1))


# --------------------------------------------------------------------------
# pyDeform-compatible module surface (src/interface/pydeform.cc:14-39)
# --------------------------------------------------------------------------
class _Params:
    def __init__(self):
        self.scale = 1.0
        self.trans = np.zeros(3)
        self.N = 0
        self.grid = None          # float32 [N^3], [z][y][x]
        self.Vn64 = None
        self.F = None
        self.edge_offset = None   # float32 [H,3]


_params = []


def GetParams(pid):
    return _params[pid]


def LoadMesh(path):
    """mesh_tensor.cc:87-100: raw (un-normalised) float32 V and int32 F."""
    V, F = read_obj(path)
    return [torch.from_numpy(V.astype(np.float32)), torch.from_numpy(F.astype(np.int32))]


def SaveMesh(path, V, F):
    write_obj(path, _f32(V).astype(np.float64), _i32(F))


def InitializeDeformTemplate(V, F, symmetry, N, df_method="bvh", grid=None):
    """deform_params.cc:16-40.  ``symmetry`` is accepted and, as in the
    reference, has no effect (it is applied to an empty mesh)."""
    p = _Params()
    p.scale, p.trans = normalize_params(V)
    p.N = int(N)
    p.F = _i32(F)
    p.Vn64 = normalized_double(V, p.scale, p.trans)
    if grid is not None:
        p.grid = np.ascontiguousarray(grid, np.float32).reshape(-1)
    else:
        p.grid = df_build(p.Vn64, p.F, p.N, method=df_method).astype(np.float32)
    _params.append(p)
    return len(_params) - 1


def ReleaseTemplate(pid):
    """Drop a template's state (the handle stays unused).  The reference
    never frees its templates (deform_params.cc:7-14); this is for long
    measuring loops that create many."""
    _params[pid] = None


def NormalizeByTemplate(V, pid):
    p = _params[pid]
    a = V.detach().numpy() if isinstance(V, torch.Tensor) else V
    assert a.dtype == np.float32 and a.flags.c_contiguous
    lib().orc_normalize_by_template(_p(a), a.shape[0], p.scale, _p(np.ascontiguousarray(p.trans)))


def DenormalizeByTemplate(V, pid):
    p = _params[pid]
    a = V.detach().numpy() if isinstance(V, torch.Tensor) else V
    assert a.dtype == np.float32 and a.flags.c_contiguous
    lib().orc_denormalize_by_template(_p(a), a.shape[0], p.scale, _p(np.ascontiguousarray(p.trans)))


def StoreRigidityInformation(V, F, pid):
    _params[pid].edge_offset = edge_offsets(V, F, 0)


def StoreGraphInformation(V, E, pid):
    _params[pid].edge_offset = edge_offsets(V, E, 1)


def StoreCadInformation(V, F, E, pid):
    """cad_layer.cc:11-77: rest offsets and weights of E's edges then F's
    half-edges."""
    lst = cad_edge_list(F, E)
    p = _params[pid]
    p.edge_offset = edge_offsets(V, lst, 1)
    p.edge_lambda = cad_edge_weights(p.edge_offset)


def CadEdgeLoss_forward(V, F, E, pid):
    p = _params[pid]
    return torch.from_numpy(edge_forward_w(V, cad_edge_list(F, E), 1, p.edge_offset, p.edge_lambda))


def CadEdgeLoss_backward(V, F, E, pid):
    p = _params[pid]
    return torch.from_numpy(edge_backward_w(V, cad_edge_list(F, E), 1, p.edge_offset, p.edge_lambda))


def DistanceFieldLoss_forward(V, pid):
    p = _params[pid]
    return torch.from_numpy(dfloss_forward(V, p.grid, p.N))


def DistanceFieldLoss_backward(V, pid):
    p = _params[pid]
    return torch.from_numpy(dfloss_backward(V, p.grid, p.N))


def RigidEdgeLoss_forward(V, F, pid):
    return torch.from_numpy(edge_forward(V, F, 0, _params[pid].edge_offset))


def RigidEdgeLoss_backward(V, F, pid):
    return torch.from_numpy(edge_backward(V, F, 0, _params[pid].edge_offset))


def GraphEdgeLoss_forward(V, E, pid):
    return torch.from_numpy(edge_forward(V, E, 1, _params[pid].edge_offset))


def GraphEdgeLoss_backward(V, E, pid):
    return torch.from_numpy(edge_backward(V, E, 1, _params[pid].edge_offset))


# --------------------------------------------------------------------------
# The plain CPU optimiser loop (src/python/rigid_deform.py:28-41 with
# RigidLossFunction from src/python/layers/rigid_loss_layer.py:7-27).
# --------------------------------------------------------------------------
def rigid_loss(V, F, pid):
    """RigidLossFunction.forward: 0.5*sum(d^2) + 0.5*sum(r^2)."""
    lossD = DistanceFieldLoss_forward(V, pid) * 0.5
    lossR = RigidEdgeLoss_forward(V, F, pid) * 0.5
    return lossD.sum() + lossR.sum()


def rigid_grad(V, F, pid, grad_h=1.0):
    """RigidLossFunction.backward: grad_h*(gD + gR)."""
    gD = DistanceFieldLoss_backward(V, pid)
    gR = RigidEdgeLoss_backward(V, F, pid)
    return grad_h * (gD + gR)


def graph_loss_grad(V, E, pid, rigidity2):
    """GraphLossFunction (src/python/layers/graph_loss_layer.py:9-43):
    loss = 0.5*sum(d^2) + rigidity2*0.5*sum(r^2); DF gradient masked where
    0.5*d^2 >= 0.5*0.03*0.03."""
    lossD = DistanceFieldLoss_forward(V, pid) * 0.5
    lossR = GraphEdgeLoss_forward(V, E, pid) * 0.5
    mask = (lossD < (0.5 * 0.03 * 0.03)).view(-1, 1).expand(-1, 3)
    loss = lossD.sum() + lossR.sum() * float(torch.tensor(rigidity2).item())
    gD = DistanceFieldLoss_backward(V, pid)
    gR = GraphEdgeLoss_backward(V, E, pid)
    gD = gD * mask
    r2 = float(torch.tensor(rigidity2, dtype=torch.float32).item())
    return loss, gD + gR * r2


class ExactAdam:
    """torch.optim.Adam([V], lr) (betas 0.9/0.999, eps 1e-8) with the update
    restated in C, one IEEE rounding per tensor op (orc_adam_step); the bias
    corrections are computed in Python double exactly as adam.py does."""

    def __init__(self, V, lr=1e-3, betas=(0.9, 0.999), eps=1e-8):
        self.V = V
        self.lr, self.b1, self.b2, self.eps = float(lr), float(betas[0]), float(betas[1]), float(eps)
        self.m = np.zeros(V.numel(), np.float32)
        self.v = np.zeros(V.numel(), np.float32)
        self.t = 0

    def step(self, grad):
        self.t += 1
        step = float(self.t)
        step_size = self.lr / (1 - self.b1 ** step)
        bc2s = (1 - self.b2 ** step) ** 0.5
        p = self.V.detach().numpy().reshape(-1)
        g = np.ascontiguousarray(grad.detach().numpy().reshape(-1), np.float32)
        lib().orc_adam_step(_p(p), _p(g), _p(self.m), _p(self.v), p.size, 1 - self.b1, self.b2, 1 - self.b2,
                             self.eps, step_size, bc2s)


def _optimizer(V, lr, adam):
    if adam == "torch":
        return torch.optim.Adam([V], lr=lr)
    if adam == "exact":
        return ExactAdam(V, lr=lr)
    raise ValueError("adam must be 'torch' or 'exact'")


def _adam_step(opt, V, g):
    if isinstance(opt, ExactAdam):
        opt.step(g)
    else:
        opt.zero_grad()
        V.grad = g
        opt.step()


def rigid_fit(src_V, src_F, pid, steps, lr=1e-3, loss_every=0, threads=None, adam="torch"):
    """Adam loop of rigid_deform.py:32-41 on CPU, returns (V, losses).
    adam="torch": torch.optim.Adam on the CPU; "exact": ExactAdam."""
    if threads is not None:
        torch.set_num_threads(threads)
    V = torch.nn.Parameter(src_V.clone())
    opt = _optimizer(V, lr, adam)
    losses = []
    for it in range(steps):
        with torch.no_grad():
            if loss_every and it % loss_every == 0:
                losses.append(float(rigid_loss(V.data, src_F, pid)))
            g = rigid_grad(V.data, src_F, pid)
            _adam_step(opt, V, g)
    return V.detach(), losses


def graph_fit(src_V, src_E, pid, steps, rigidity2, lr=1e-3, adam="torch"):
    """The CAD loop (src/python/cad_deform.py:30-37) with GraphLossFunction
    (graph_loss_layer.py:9-43) and Adam on the CPU (adam as in rigid_fit)."""
    V = torch.nn.Parameter(src_V.clone())
    opt = _optimizer(V, lr, adam)
    for _ in range(steps):
        with torch.no_grad():
            _, g = graph_loss_grad(V.data, src_E, pid, rigidity2)
            _adam_step(opt, V, g)
    return V.detach()


def cad_fit(src_V, src_F, src_E, pid, steps, lr=1e-3, adam="exact"):
    """The CadLossFunction loop (src/python/layers/cad_loss_layer.py:9-31:
    grad_h * (DistanceFieldLoss_backward + CadEdgeLoss_backward), grad_h = 1)
    with Adam on the CPU (adam as in rigid_fit)."""
    V = torch.nn.Parameter(src_V.clone())
    opt = _optimizer(V, lr, adam)
    for _ in range(steps):
        with torch.no_grad():
            g = 1.0 * (DistanceFieldLoss_backward(V.data, pid) + CadEdgeLoss_backward(V.data, src_F, src_E, pid))
            _adam_step(opt, V, g)
    return V.detach()


def reverse_loss(src_V, tar_V):
    """ReverseLossLayer.forward (src/python/layers/reverse_loss_layer.py:14-25)
    on the CPU: cKDTree 1-NN of every target vertex among the source
    vertices, then 0.5 * sum |src_V[ii] - tar_V|^2 with torch autograd.
    (The reference passes n_jobs=4, which SciPy no longer accepts; the
    neighbours do not depend on the thread count.)  Returns (loss, ii)."""
    from scipy.spatial import cKDTree
    tree = cKDTree(src_V.detach().cpu().numpy())
    _, ii = tree.query(tar_V.detach().cpu().numpy(), k=1)
    src_c = src_V[torch.from_numpy(ii)]
    loss = src_c - tar_V
    loss = 0.5 * (loss * loss).sum()
    return loss, ii


def inverse_fit(src_V, src_F, tar_V, pid, steps, lr=1e-3):
    """The loop of src/python/inverse_deform.py:26-38 on the CPU (without its
    early stop): RigidLossFunction (oracle gradient) * 10 + ReverseLossLayer
    (cKDTree + torch autograd), torch.optim.Adam.  src_V and tar_V are
    normalised by the template already.  Returns the fitted vertices."""
    V = torch.nn.Parameter(src_V.clone())
    opt = torch.optim.Adam([V], lr=lr)
    for _ in range(steps):
        opt.zero_grad()
        loss_r, _ = reverse_loss(V, tar_V)
        loss_r.backward()
        with torch.no_grad():
            V.grad += rigid_grad(V.data, src_F, pid) * 10
        opt.step()
    return V.detach()


def solve_linear(V, F, E, ref, G, rigidity, with_rot=0):
    """SolveLinear (src/interface/linear_layer.cc:5-79) on the CPU: the
    system of LinearEstimation (src/lib/linear.cc:10-112) or
    LinearEstimationWithRot (linear.cc:114-230) assembled entry by entry as
    the reference does (duplicates summed), solved directly in double
    (scipy.sparse.linalg.spsolve instead of Eigen's SimplicialLDLT: the same
    solution up to rounding).  Returns the new float32 vertices."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spl
    V = np.asarray(V, np.float32).astype(np.float64)
    F = np.asarray(F, np.int64).reshape(-1, 3)
    G = np.asarray(G, np.float32).astype(np.float64)
    n = V.shape[0]
    rows, cols, vals = [], [], []
    B = np.zeros((n, 3))
    face_edges = np.stack([F[:, [0, 1, 2]].reshape(-1), F[:, [1, 2, 0]].reshape(-1)], 1)
    if not with_rot:
        ref = np.asarray(ref, np.int64)
        E = np.asarray(E, np.int64).reshape(-1, 2)
        for g in range(G.shape[0]):
            cell = np.flatnonzero(ref == g)
            if cell.size == 0:
                continue
            w = 1.0 / cell.size
            jj, kk = np.meshgrid(cell, cell, indexing="ij")
            rows.append(jj.reshape(-1)); cols.append(kk.reshape(-1)); vals.append(np.full(jj.size, w * w))
            B[cell] += w * G[g]
        rows.append(np.arange(n)); cols.append(np.arange(n)); vals.append(np.full(n, 1e-6))
        B += 1e-6 * G[ref]
        edges = np.concatenate([face_edges, E])
        a, b = edges[:, 0], edges[:, 1]
        reg = rigidity * 2e-2 / (np.linalg.norm(V[a] - V[b], axis=1) + 1e-8)
        reg = reg * reg
        rows += [a, a, b, b]; cols += [a, b, a, b]; vals += [reg, -reg, -reg, reg]
        np.add.at(B, a, reg[:, None] * (V[a] - V[b]))
        np.add.at(B, b, reg[:, None] * (V[b] - V[a]))
    else:
        links = [set() for _ in range(n)]
        for a, b in face_edges:
            links[a].add(b)
            links[b].add(a)
        R = np.zeros((n, 3, 3))
        scale = np.zeros(n)
        for i in range(n):
            M = np.zeros((3, 3))
            lo = lc = 0.0
            for p in sorted(links[i]):
                d1 = V[p] - V[i]
                d2 = G[p] - G[i]
                lo += np.linalg.norm(d1)
                lc += np.linalg.norm(d2)
                M += np.outer(d2, d1)
            scale[i] = lc / (lo + 1e-8)
            U, _, Vt = np.linalg.svd(M)
            R[i] = U @ Vt
        rows.append(np.arange(n)); cols.append(np.arange(n)); vals.append(np.ones(n))
        B += G
        for j in (0, 1):
            a, b = face_edges[:, j], face_edges[:, 1 - j]
            off = V[b] - V[a]
            reg = 1.0 * 2e-2 / np.linalg.norm(off, axis=1) * rigidity
            off = scale[a, None] * np.einsum("nij,nj->ni", R[a], off)
            rows += [a, a, b, b]; cols += [a, b, a, b]; vals += [reg, -reg, -reg, reg]
            np.add.at(B, a, -reg[:, None] * off)
            np.add.at(B, b, reg[:, None] * off)
    A = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(n, n))
    X = spl.spsolve(A.tocsc(), B)
    return X.astype(np.float32)
