"""Drop-in GPU replacement for the reference's ``pyDeform`` extension module.

Same function names, argument order, meaning and results as the pybind11
module registered in src/interface/pydeform.cc:14-39; every computation runs
in libmeshode.so on the current CUDA device.  Differences from the reference,
all additive:

* Inputs are validated (dtype float32 / int32, shapes, index ranges) and a
  RuntimeError is raised where the reference read raw storage
  (distance_layer.cc:21, rigid_layer.cc:24-25 ...) with undefined behaviour.
* Tensors may live on the CPU or on the GPU.  Results are returned on the
  device of the vertex tensor (the reference always returned CPU tensors, and
  so does this module for CPU inputs).
* Template handles are ints into a process-global list, as in
  deform_params.cc:7-14; ``ReleaseTemplate`` frees one's device memory.

``LoadCadMesh`` (the reference's CGAL remeshing) is restated on the CPU in
``cadmesh``; ``SolveLinear`` runs in libmeshode.so (matrix-free conjugate
gradients in double).
"""
import ctypes

import numpy as np
import torch

from . import _lib as L
from . import objio
from ._lib import call, ptr, stream_ptr

DEFAULT_LAYOUT = L.MO_LAYOUT_CELL


class _EdgeState:
    def __init__(self, kind, idx_dev, nh, offsets):
        self.kind = kind
        self.idx = idx_dev
        self.nh = nh
        self.offsets = offsets      # float32 [nh,3] on the device
        self.csr_cache = {}         # key -> (idx_dev, csr buffer)
        self.csr = None             # CSR of the index tensor given at Store time
        self.rest = None            # the vertices the rest offsets were taken from
        self.weights = None         # float32 [nh] per-edge weights (CadEdgeLoss)


class DeformParams:
    """Per-target state: transform, distance grid and edge rest offsets
    (the reference's DeformParams, src/interface/deform_params.h:7-34)."""

    def __init__(self):
        self.device = None
        self.N = 0
        self.layout = DEFAULT_LAYOUT
        self.params = None          # cuda float64 [4] = scale, tx, ty, tz
        self.grid_linear = None     # cuda float32 [N^3]
        self.grid = None            # cuda float32 in `layout`
        self.edge = None
        self._host_params = None

    @property
    def scale(self):
        return float(self.host_params()[0])

    @property
    def trans(self):
        return self.host_params()[1:].copy()

    def host_params(self):
        if self._host_params is None:
            self._host_params = self.params.cpu().numpy()
        return self._host_params


_g_params = []


def GetParams(param_id):
    try:
        p = _g_params[int(param_id)]
    except (IndexError, ValueError, TypeError):
        raise RuntimeError("invalid template id %r" % (param_id,))
    if p is None:
        raise RuntimeError("template %d was released" % int(param_id))
    return p


def ReleaseTemplate(param_id):
    """Free a template's device memory (an addition; the reference never frees)."""
    GetParams(param_id)
    _g_params[int(param_id)] = None


# ---------------------------------------------------------------------------
# validation helpers
# ---------------------------------------------------------------------------
def _cuda_device():
    L.require_cuda()
    return torch.device("cuda", torch.cuda.current_device())


def _check_vertices(V, name="V"):
    if not isinstance(V, torch.Tensor):
        raise RuntimeError("%s must be a torch.Tensor" % name)
    if V.dtype != torch.float32:
        raise RuntimeError("%s must be float32, got %s" % (name, V.dtype))
    if V.dim() != 2 or V.shape[1] != 3:
        raise RuntimeError("%s must have shape [n,3], got %s" % (name, tuple(V.shape)))


def _check_indices(I, cols, name):
    if not isinstance(I, torch.Tensor):
        raise RuntimeError("%s must be a torch.Tensor" % name)
    if I.dtype != torch.int32:
        raise RuntimeError("%s must be int32, got %s" % (name, I.dtype))
    if I.dim() != 2 or I.shape[1] != cols:
        raise RuntimeError("%s must have shape [m,%d], got %s" % (name, cols, tuple(I.shape)))


def _on_device(t, dev):
    return t.detach().to(dev, non_blocking=False).contiguous()


def _out(t, like):
    return t if like.is_cuda else t.cpu()


# ---------------------------------------------------------------------------
# mesh I/O (src/interface/mesh_tensor.cc:87-100, 180-186)
# ---------------------------------------------------------------------------
def LoadMesh(filename):
    """Raw (un-normalised) float32 V [n,3] and int32 F [m,3] CPU tensors."""
    V, F = objio.read_obj(filename)
    return [torch.from_numpy(V.astype(np.float32)), torch.from_numpy(F.astype(np.int32))]


def SaveMesh(filename, tensorV, tensorF):
    _check_vertices(tensorV)
    _check_indices(tensorF, 3, "F")
    objio.write_obj(filename, tensorV.detach().cpu().numpy().astype(np.float64), tensorF.detach().cpu().numpy())


def LoadCadMesh(filename):
    """mesh_tensor.cc:102-178: [V f32 [n,3], F i32 [m,3], E i32 [k,2]
    (geometry neighbour pairs), src_to_graph i32 [n,1], graph V f32 [g,3],
    graph E i32 [q,2]] as CPU tensors -- the CAD model remeshed at 0.02 with
    its representative graph (restated with SciPy's Delaunay; see cadmesh)."""
    from . import cadmesh
    return [torch.from_numpy(np.ascontiguousarray(a)) for a in cadmesh.load_cad_mesh(filename)]


def SolveLinear(tensorV, tensorF, tensorE, tensorRef, tensorGraphV, rigidity, with_rot=0, tol=1e-13,
                max_iter=200000):
    """In place on tensorV (linear_layer.cc:5-79): with_rot 0, LinearEstimation
    (linear.cc:10-112) -- each vertex pulled to its graph node's position
    (tensorRef [n] int32 into tensorGraphV [g,3]) through the cell means,
    rigidity springs on the faces' half-edges and on tensorE; with_rot 1,
    LinearEstimationWithRot (linear.cc:114-230) -- tensorGraphV [n,3] the
    per-vertex targets, springs carrying each vertex's rotation and scale.
    Solved in double by preconditioned conjugate gradients on the GPU
    (relative residual <= tol); returns (iterations, relative residual)."""
    _check_vertices(tensorV)
    _check_indices(tensorF, 3, "F")
    _check_vertices(tensorGraphV, "GraphV")
    dev = _cuda_device()
    nv = int(tensorV.shape[0])
    with_rot = 1 if with_rot else 0
    F = _on_device(tensorF, dev)
    G = _on_device(tensorGraphV, dev)
    if with_rot:
        if int(G.shape[0]) != nv:
            raise RuntimeError("SolveLinear with_rot needs one target per vertex")
        E = ref = None
        ne = 0
    else:
        _check_indices(tensorE, 2, "E")
        # LoadCadMesh returns the references as [n,1]; [n] is accepted too
        if not isinstance(tensorRef, torch.Tensor) or tensorRef.dtype != torch.int32 or tensorRef.numel() != nv \
                or not (tensorRef.dim() == 1 or (tensorRef.dim() == 2 and tensorRef.shape[1] == 1)):
            raise RuntimeError("references must be an int32 tensor [n] or [n,1]")
        E = _on_device(tensorE, dev)
        ref = _on_device(tensorRef.reshape(-1), dev)
        ne = int(E.shape[0])
    work = tensorV if (tensorV.is_cuda and tensorV.is_contiguous()) else _on_device(tensorV, dev)
    it = ctypes.c_int()
    res = ctypes.c_double()
    call("mo_solve_linear", ptr(work), nv, ptr(F), int(F.shape[0]), ptr(E), ne, ptr(ref), ptr(G),
         int(G.shape[0]), float(rigidity), with_rot, float(tol), int(max_iter), None, 0, ctypes.byref(it),
         ctypes.byref(res), stream_ptr())
    if work is not tensorV:
        with torch.no_grad():
            tensorV.copy_(work)
    return it.value, res.value


def _cad_edges(state, tensorF, tensorE, nv, dev):
    """(device edge list, validated CSR) of the CAD loss's edge set -- E's
    edges then F's half-edges (cad_layer.cc:33-67) -- cached by the identity
    and version of F and E."""
    key = ("cad", _idx_key(tensorF, nv), _idx_key(tensorE, nv))
    hit = state.csr_cache.get(key)
    if hit is not None:
        return hit
    Fd = _on_device(tensorF, dev)
    Ed = _on_device(tensorE, dev)
    nh = Ed.shape[0] + 3 * Fd.shape[0]
    lst = torch.empty(nh, 2, dtype=torch.int32, device=dev)
    call("mo_edge_cad_list", ptr(Ed), Ed.shape[0], ptr(Fd), Fd.shape[0], ptr(lst), stream_ptr())
    nbytes = L.lib().mo_edge_csr_bytes(nv, nh, L.MO_EDGES_LIST)
    csr = torch.empty((nbytes + 3) // 4, dtype=torch.int32, device=dev)
    call("mo_edge_csr_build", ptr(lst), nh, L.MO_EDGES_LIST, nv, ptr(csr), nbytes, None, stream_ptr())
    if len(state.csr_cache) > 8:
        state.csr_cache.clear()
    state.csr_cache[key] = (lst, csr)
    return state.csr_cache[key]


def StoreCadInformation(tensorV, tensorF, tensorE, param_id):
    """Rest offsets and weights 2e-2/(|off|+1e-8) of E's edges then F's
    half-edges (cad_layer.cc:11-77)."""
    _check_vertices(tensorV)
    _check_indices(tensorF, 3, "F")
    _check_indices(tensorE, 2, "E")
    p = GetParams(param_id)
    Vd = _on_device(tensorV, p.device)
    nh = tensorE.shape[0] + 3 * tensorF.shape[0]
    off = torch.empty(nh, 3, dtype=torch.float32, device=p.device)
    state = _EdgeState(L.MO_EDGES_LIST, None, nh, off)
    lst, state.csr = _cad_edges(state, tensorF, tensorE, Vd.shape[0], p.device)
    state.idx = lst
    s = stream_ptr()
    call("mo_edge_offsets", ptr(Vd), Vd.shape[0], ptr(lst), nh, L.MO_EDGES_LIST, ptr(off), s)
    state.weights = torch.empty(nh, dtype=torch.float32, device=p.device)
    call("mo_edge_cad_weights", ptr(off), nh, ptr(state.weights), s)
    state.rest = Vd.clone()
    p.edge = state


def _cad_state(param_id, tensorV, tensorF, tensorE):
    _check_vertices(tensorV)
    _check_indices(tensorF, 3, "F")
    _check_indices(tensorE, 2, "E")
    p = GetParams(param_id)
    st = p.edge
    if st is None or st.weights is None:
        raise RuntimeError("template %d has no CAD edge information; call StoreCadInformation first"
                           % int(param_id))
    nh = tensorE.shape[0] + 3 * tensorF.shape[0]
    if nh != st.nh:
        raise RuntimeError("edge set has %d edges but the stored rest offsets have %d" % (nh, st.nh))
    Vd = _on_device(tensorV, p.device)
    lst, csr = _cad_edges(st, tensorF, tensorE, Vd.shape[0], p.device)
    return p, st, Vd, lst, csr


def CadEdgeLoss_forward(tensorV, tensorF, tensorE, param_id):
    """[E+3F,3] weighted squared residual components (cad_layer.cc:79-150)."""
    p, st, Vd, lst, _ = _cad_state(param_id, tensorV, tensorF, tensorE)
    out = torch.empty(st.nh, 3, dtype=torch.float32, device=p.device)
    call("mo_edge_forward_w", ptr(Vd), Vd.shape[0], ptr(lst), st.nh, L.MO_EDGES_LIST, ptr(st.offsets),
         ptr(st.weights), ptr(out), stream_ptr())
    return _out(out, tensorV)


def CadEdgeLoss_backward(tensorV, tensorF, tensorE, param_id):
    """[V,3] scatter of the residuals times the squared weights
    (cad_layer.cc:152-223)."""
    p, st, Vd, _, csr = _cad_state(param_id, tensorV, tensorF, tensorE)
    out = torch.empty(Vd.shape[0], 3, dtype=torch.float32, device=p.device)
    call("mo_edge_backward_w", ptr(Vd), Vd.shape[0], ptr(csr), st.nh, ptr(st.offsets), ptr(st.weights), ptr(out),
         stream_ptr())
    return _out(out, tensorV)


# ---------------------------------------------------------------------------
# template (deform_params.cc:16-40)
# ---------------------------------------------------------------------------
def InitializeDeformTemplate(tensorV, tensorF, symmetry, grid_resolution, layout=None, df_method=L.MO_DF_AUTO):
    """Normalise a copy of the target, build its distance field, return a
    handle.  ``symmetry`` is accepted and, as in the reference
    (deform_params.cc:28-33 reflects an empty mesh), has no effect."""
    _check_vertices(tensorV, "V")
    _check_indices(tensorF, 3, "F")
    N = int(grid_resolution)
    if N < 2:
        raise RuntimeError("grid resolution must be >= 2, got %d" % N)
    if tensorV.shape[0] == 0 or tensorF.shape[0] == 0:
        raise RuntimeError("target mesh must have vertices and faces")
    dev = _cuda_device()
    p = DeformParams()
    p.device = dev
    p.N = N
    p.layout = DEFAULT_LAYOUT if layout is None else int(layout)
    s = stream_ptr()
    Vd = _on_device(tensorV, dev)
    Fd = _on_device(tensorF, dev)
    bbox = torch.empty(6, dtype=torch.int32, device=dev)
    p.params = torch.empty(4, dtype=torch.float64, device=dev)
    call("mo_bbox", ptr(Vd), Vd.shape[0], ptr(bbox), s)
    call("mo_norm_params", ptr(bbox), ptr(p.params), s)
    nbytes = L.lib().mo_df_build_scratch_bytes(Vd.shape[0], Fd.shape[0], N, int(df_method))
    scratch = torch.empty(int(nbytes), dtype=torch.uint8, device=dev)
    p.grid_linear = torch.empty(N * N * N, dtype=torch.float32, device=dev)
    call("mo_df_build", ptr(Vd), Vd.shape[0], ptr(Fd), Fd.shape[0], N, ptr(p.params), int(df_method),
         ptr(scratch), nbytes, ptr(p.grid_linear), None, s)
    del scratch
    if p.layout == L.MO_LAYOUT_LINEAR:
        p.grid = p.grid_linear
    else:
        nb = L.lib().mo_grid_bytes(N, p.layout)
        if nb == 0:
            raise RuntimeError("unknown grid layout %d" % p.layout)
        p.grid = torch.empty(nb // 4, dtype=torch.float32, device=dev)
        call("mo_grid_relayout", ptr(p.grid_linear), N, p.layout, ptr(p.grid), s)
    _g_params.append(p)
    return len(_g_params) - 1


def GetDistanceField(param_id):
    """The template's distance grid, float32 [N,N,N] indexed [z][y][x]."""
    p = GetParams(param_id)
    return p.grid_linear.view(p.N, p.N, p.N)


def GetTransform(param_id):
    """(scale, trans[3]) of the template normalisation (Mesh::GetScale/GetTranslation)."""
    p = GetParams(param_id)
    return p.scale, p.trans


def _normalize_inplace(tensorV, param_id, inverse):
    _check_vertices(tensorV)
    p = GetParams(param_id)
    if tensorV.shape[0] == 0:
        return
    s = stream_ptr()
    if tensorV.is_cuda and tensorV.is_contiguous():
        call("mo_normalize", ptr(tensorV), tensorV.shape[0], ptr(p.params), inverse, s)
        return
    work = _on_device(tensorV, p.device)
    call("mo_normalize", ptr(work), work.shape[0], ptr(p.params), inverse, s)
    with torch.no_grad():
        tensorV.copy_(work)


def NormalizeByTemplate(tensorV, param_id):
    """In place: v = (v - trans)/scale with the target's transform (normalize.cc:5-24)."""
    _normalize_inplace(tensorV, param_id, 0)


def DenormalizeByTemplate(tensorV, param_id):
    """In place: v = v*scale + trans (normalize.cc:26-45)."""
    _normalize_inplace(tensorV, param_id, 1)


# ---------------------------------------------------------------------------
# DistanceFieldLoss (distance_layer.cc:8-81)
# ---------------------------------------------------------------------------
def DistanceFieldLoss_forward(tensorV, param_id):
    _check_vertices(tensorV)
    p = GetParams(param_id)
    Vd = _on_device(tensorV, p.device)
    out = torch.empty(Vd.shape[0], dtype=torch.float32, device=p.device)
    call("mo_dfloss_forward", ptr(Vd), Vd.shape[0], ptr(p.grid), p.N, p.layout, ptr(out), stream_ptr())
    return _out(out, tensorV)


def DistanceFieldLoss_backward(tensorV, param_id):
    _check_vertices(tensorV)
    p = GetParams(param_id)
    Vd = _on_device(tensorV, p.device)
    out = torch.empty(Vd.shape[0], 3, dtype=torch.float32, device=p.device)
    call("mo_dfloss_backward", ptr(Vd), Vd.shape[0], ptr(p.grid), p.N, p.layout, ptr(out), stream_ptr())
    return _out(out, tensorV)


def DistanceFieldLoss_fwd_bwd(tensorV, param_id, mask_thresh=None):
    """Both outputs in one pass (an addition); ``mask_thresh`` applies the
    GraphLossFunction gradient mask (0.5*d^2 < mask_thresh)."""
    _check_vertices(tensorV)
    p = GetParams(param_id)
    Vd = _on_device(tensorV, p.device)
    loss = torch.empty(Vd.shape[0], dtype=torch.float32, device=p.device)
    grad = torch.empty(Vd.shape[0], 3, dtype=torch.float32, device=p.device)
    use_mask = 0 if mask_thresh is None else 1
    call("mo_dfloss_fwd_bwd", ptr(Vd), Vd.shape[0], ptr(p.grid), p.N, p.layout, ptr(loss), ptr(grad), use_mask,
         float(mask_thresh or 0.0), stream_ptr())
    return _out(loss, tensorV), _out(grad, tensorV)


# ---------------------------------------------------------------------------
# edge losses (rigid_layer.cc, graph_layer.cc)
# ---------------------------------------------------------------------------
def _store_edges(tensorV, idx, param_id, kind):
    _check_vertices(tensorV)
    _check_indices(idx, 3 if kind == L.MO_EDGES_FACES else 2, "F" if kind == L.MO_EDGES_FACES else "E")
    p = GetParams(param_id)
    Vd = _on_device(tensorV, p.device)
    Id = _on_device(idx, p.device)
    nh = int(L.lib().mo_edge_count(Id.shape[0], kind))
    off = torch.empty(nh, 3, dtype=torch.float32, device=p.device)
    s = stream_ptr()
    state = _EdgeState(kind, Id, nh, off)
    # validates the indices against the vertex count (raises on a bad index)
    _, state.csr = _csr_for(state, idx, Id, Vd.shape[0], p.device)
    call("mo_edge_offsets", ptr(Vd), Vd.shape[0], ptr(Id), Id.shape[0], kind, ptr(off), s)
    # a copy: for a contiguous CUDA input Vd aliases the caller's tensor,
    # which the caller's optimiser then moves
    state.rest = Vd.clone()
    p.edge = state


def _idx_key(idx, nv):
    return (idx.device.type, idx.data_ptr(), idx._version, tuple(idx.shape), int(nv))


def _csr_for(state, idx, idx_dev, nv, dev):
    """(device copy of idx, validated CSR) for this index tensor, cached by
    tensor identity and version so a loop passing the same F each step pays
    for the copy and the CSR build once."""
    key = _idx_key(idx, nv)
    hit = state.csr_cache.get(key)
    if hit is not None:
        return hit
    if idx_dev is None:
        idx_dev = _on_device(idx, dev)
    nbytes = L.lib().mo_edge_csr_bytes(nv, idx_dev.shape[0], state.kind)
    csr = torch.empty((nbytes + 3) // 4, dtype=torch.int32, device=dev)
    call("mo_edge_csr_build", ptr(idx_dev), idx_dev.shape[0], state.kind, nv, ptr(csr), nbytes, None, stream_ptr())
    if len(state.csr_cache) > 8:
        state.csr_cache.clear()
    state.csr_cache[key] = (idx_dev, csr)
    return state.csr_cache[key]


def _edge_state(param_id, kind, idx):
    p = GetParams(param_id)
    st = p.edge
    if st is None or st.kind != kind or st.weights is not None:
        raise RuntimeError("template %d has no %s information; call %s first" % (
            int(param_id), "rigidity" if kind == L.MO_EDGES_FACES else "graph",
            "StoreRigidityInformation" if kind == L.MO_EDGES_FACES else "StoreGraphInformation"))
    nh = int(L.lib().mo_edge_count(idx.shape[0], kind))
    if nh != st.nh:
        raise RuntimeError("edge list has %d half-edges but the stored rest offsets have %d" % (nh, st.nh))
    return p, st


def _edge_forward(tensorV, idx, param_id, kind):
    _check_vertices(tensorV)
    _check_indices(idx, 3 if kind == L.MO_EDGES_FACES else 2, "F" if kind == L.MO_EDGES_FACES else "E")
    p, st = _edge_state(param_id, kind, idx)
    Vd = _on_device(tensorV, p.device)
    idx_dev, _ = _csr_for(st, idx, None, Vd.shape[0], p.device)
    out = torch.empty(st.nh, 3, dtype=torch.float32, device=p.device)
    call("mo_edge_forward", ptr(Vd), Vd.shape[0], ptr(idx_dev), idx_dev.shape[0], kind, ptr(st.offsets), ptr(out),
         stream_ptr())
    return _out(out, tensorV)


def _edge_backward(tensorV, idx, param_id, kind):
    _check_vertices(tensorV)
    _check_indices(idx, 3 if kind == L.MO_EDGES_FACES else 2, "F" if kind == L.MO_EDGES_FACES else "E")
    p, st = _edge_state(param_id, kind, idx)
    Vd = _on_device(tensorV, p.device)
    _, csr = _csr_for(st, idx, None, Vd.shape[0], p.device)
    out = torch.empty(Vd.shape[0], 3, dtype=torch.float32, device=p.device)
    call("mo_edge_backward", ptr(Vd), Vd.shape[0], ptr(csr), st.nh, ptr(st.offsets), ptr(out), stream_ptr())
    return _out(out, tensorV)


def StoreRigidityInformation(tensorV, tensorF, param_id):
    """Rest offsets v1 - v0 of the 3F half-edges (rigid_layer.cc:11-46)."""
    _store_edges(tensorV, tensorF, param_id, L.MO_EDGES_FACES)


def RigidEdgeLoss_forward(tensorV, tensorF, param_id):
    """[3F,3] squared residual components (rigid_layer.cc:48-89)."""
    return _edge_forward(tensorV, tensorF, param_id, L.MO_EDGES_FACES)


def RigidEdgeLoss_backward(tensorV, tensorF, param_id):
    """[V,3] residual scatter (rigid_layer.cc:91-133)."""
    return _edge_backward(tensorV, tensorF, param_id, L.MO_EDGES_FACES)


def StoreGraphInformation(tensorV, tensorE, param_id):
    """Rest offsets of an explicit edge list (graph_layer.cc:11-45)."""
    _store_edges(tensorV, tensorE, param_id, L.MO_EDGES_LIST)


def GraphEdgeLoss_forward(tensorV, tensorE, param_id):
    return _edge_forward(tensorV, tensorE, param_id, L.MO_EDGES_LIST)


def GraphEdgeLoss_backward(tensorV, tensorE, param_id):
    return _edge_backward(tensorV, tensorE, param_id, L.MO_EDGES_LIST)
