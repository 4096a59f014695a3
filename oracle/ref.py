"""The reference's own ``pyDeform`` functions, from oracle/_ref (test
infrastructure: only tests and fixture generators use this module).

``oracle/build_ref.py`` compiles the reference's C++ loops unchanged
(uniformgrid.cc, mesh.cc, deform_params.cc, mesh_tensor.cc,
distance_layer.cc, rigid_layer.cc, graph_layer.cc, cad_layer.cc,
normalize.cc) against stand-ins for Eigen, ceres::Jet, torch and libigl.
This module exposes them with the names, arguments and results of the
pybind11 module registered in src/interface/pydeform.cc:14-39, on CPU torch
tensors, so that the reference's Python layers
(src/python/layers/*_loss_layer.py) can run on it unchanged: install it as
``sys.modules["pyDeform"]`` (``install_as_pydeform``).

Like the reference, the functions read and write the tensors' memory
directly; the tensors must be contiguous CPU tensors of the reference's
dtypes (float32 vertices, int32 faces and edges).

``LoadCadMesh`` (CGAL remeshing) and ``SolveLinear`` (Eigen's sparse
Cholesky) are not compiled: they raise.
"""
import ctypes
import os
import sys

import numpy as np
import torch

from . import build_ref

_LIB = None


def available():
    return build_ref.available()


def lib():
    global _LIB
    if _LIB is None:
        path = build_ref.build()
        if path is None:
            raise RuntimeError("oracle/_ref needs the reference's sources, which are not mounted here")
        L = ctypes.CDLL(path)
        L.ref_last_error.restype = ctypes.c_char_p
        _LIB = L
    return _LIB


def _call(name, *args):
    rc = getattr(lib(), name)(*args)
    if rc != 0:
        raise RuntimeError("%s: %s" % (name, lib().ref_last_error().decode()))


def _i64(x):
    return ctypes.c_int64(int(x))


def _ptr(t, dtype):
    if not isinstance(t, torch.Tensor):
        raise TypeError("expected a torch.Tensor")
    if t.device.type != "cpu" or t.dtype != dtype or not t.is_contiguous():
        raise RuntimeError("oracle/_ref takes contiguous CPU %s tensors (got %s %s)" % (dtype, t.device, t.dtype))
    return ctypes.c_void_p(t.data_ptr())


def _f(t):
    return _ptr(t, torch.float32)


def _i(t):
    return _ptr(t, torch.int32)


def _pid(param_id):
    return ctypes.c_int(int(param_id))


def LoadMesh(filename):
    nv, nf = ctypes.c_int64(), ctypes.c_int64()
    _call("ref_load_mesh_counts", filename.encode(), ctypes.byref(nv), ctypes.byref(nf))
    V = torch.zeros((nv.value, 3), dtype=torch.float32)
    F = torch.zeros((nf.value, 3), dtype=torch.int32)
    _call("ref_load_mesh", filename.encode(), _f(V), _i(F))
    return [V, F]


def SaveMesh(filename, tensorV, tensorF):
    _call("ref_save_mesh", filename.encode(), _f(tensorV), _i64(tensorV.shape[0]), _i(tensorF),
          _i64(tensorF.shape[0]))


def LoadCadMesh(filename):
    raise NotImplementedError("LoadCadMesh's remeshing needs CGAL, which the reference does not vendor")


def SolveLinear(*args, **kwargs):
    raise NotImplementedError("SolveLinear needs Eigen's sparse Cholesky and is not part of oracle/_ref")


def InitializeDeformTemplate(tensorV, tensorF, symmetry, grid_resolution):
    out = ctypes.c_int()
    _call("ref_init_template", _f(tensorV), _i64(tensorV.shape[0]), _i(tensorF), _i64(tensorF.shape[0]),
          ctypes.c_int(int(symmetry)), ctypes.c_int(int(grid_resolution)), ctypes.byref(out))
    return out.value


def NormalizeByTemplate(tensorV, param_id):
    _call("ref_normalize", _f(tensorV), _i64(tensorV.shape[0]), _pid(param_id))


def DenormalizeByTemplate(tensorV, param_id):
    _call("ref_denormalize", _f(tensorV), _i64(tensorV.shape[0]), _pid(param_id))


def DistanceFieldLoss_forward(tensorV, param_id):
    out = torch.zeros(tensorV.shape[0], dtype=torch.float32)
    _call("ref_df_forward", _f(tensorV), _i64(tensorV.shape[0]), _pid(param_id), _f(out))
    return out


def DistanceFieldLoss_backward(tensorV, param_id):
    out = torch.zeros((tensorV.shape[0], 3), dtype=torch.float32)
    _call("ref_df_backward", _f(tensorV), _i64(tensorV.shape[0]), _pid(param_id), _f(out))
    return out


def StoreRigidityInformation(tensorV, tensorF, param_id):
    _call("ref_store_rigidity", _f(tensorV), _i64(tensorV.shape[0]), _i(tensorF), _i64(tensorF.shape[0]),
          _pid(param_id))


def RigidEdgeLoss_forward(tensorV, tensorF, param_id):
    out = torch.zeros((3 * tensorF.shape[0], 3), dtype=torch.float32)
    _call("ref_rigid_forward", _f(tensorV), _i64(tensorV.shape[0]), _i(tensorF), _i64(tensorF.shape[0]),
          _pid(param_id), _f(out))
    return out


def RigidEdgeLoss_backward(tensorV, tensorF, param_id):
    out = torch.zeros((tensorV.shape[0], 3), dtype=torch.float32)
    _call("ref_rigid_backward", _f(tensorV), _i64(tensorV.shape[0]), _i(tensorF), _i64(tensorF.shape[0]),
          _pid(param_id), _f(out))
    return out


def StoreGraphInformation(tensorV, tensorE, param_id):
    _call("ref_store_graph", _f(tensorV), _i64(tensorV.shape[0]), _i(tensorE), _i64(tensorE.shape[0]),
          _pid(param_id))


def GraphEdgeLoss_forward(tensorV, tensorE, param_id):
    out = torch.zeros((tensorE.shape[0], 3), dtype=torch.float32)
    _call("ref_graph_forward", _f(tensorV), _i64(tensorV.shape[0]), _i(tensorE), _i64(tensorE.shape[0]),
          _pid(param_id), _f(out))
    return out


def GraphEdgeLoss_backward(tensorV, tensorE, param_id):
    out = torch.zeros((tensorV.shape[0], 3), dtype=torch.float32)
    _call("ref_graph_backward", _f(tensorV), _i64(tensorV.shape[0]), _i(tensorE), _i64(tensorE.shape[0]),
          _pid(param_id), _f(out))
    return out


def StoreCadInformation(tensorV, tensorF, tensorE, param_id):
    _call("ref_store_cad", _f(tensorV), _i64(tensorV.shape[0]), _i(tensorF), _i64(tensorF.shape[0]), _i(tensorE),
          _i64(tensorE.shape[0]), _pid(param_id))


def CadEdgeLoss_forward(tensorV, tensorF, tensorE, param_id):
    out = torch.zeros((tensorE.shape[0] + 3 * tensorF.shape[0], 3), dtype=torch.float32)
    _call("ref_cad_forward", _f(tensorV), _i64(tensorV.shape[0]), _i(tensorF), _i64(tensorF.shape[0]), _i(tensorE),
          _i64(tensorE.shape[0]), _pid(param_id), _f(out))
    return out


def CadEdgeLoss_backward(tensorV, tensorF, tensorE, param_id):
    out = torch.zeros((tensorV.shape[0], 3), dtype=torch.float32)
    _call("ref_cad_backward", _f(tensorV), _i64(tensorV.shape[0]), _i(tensorF), _i64(tensorF.shape[0]), _i(tensorE),
          _i64(tensorE.shape[0]), _pid(param_id), _f(out))
    return out


# ---- access to the reference's stored state (not part of pyDeform) ----

def template_grid(param_id, N):
    """The template's UniformGrid as double [N^3], [z][y][x]."""
    out = np.zeros(N ** 3, np.float64)
    _call("ref_template_grid", _pid(param_id), out.ctypes.data_as(ctypes.c_void_p))
    return out


def template_transform(param_id):
    """(scale, trans[3]) in double, as Mesh::Normalize left them."""
    out = np.zeros(4, np.float64)
    _call("ref_template_transform", _pid(param_id), out.ctypes.data_as(ctypes.c_void_p))
    return float(out[0]), out[1:].copy()


def template_edges(param_id, n_edges):
    """The stored rest offsets [n,3] and weights [n] (weights: the CAD layer's)."""
    off = np.zeros((n_edges, 3), np.float32)
    lam = np.zeros(n_edges, np.float32)
    _call("ref_template_edges", _pid(param_id), off.ctypes.data_as(ctypes.c_void_p),
          lam.ctypes.data_as(ctypes.c_void_p))
    return off, lam


def grid_template(grid, N):
    """A template whose UniformGrid holds the given [z][y][x] values."""
    g = np.ascontiguousarray(grid, np.float64).reshape(-1)
    assert g.size == N ** 3
    out = ctypes.c_int()
    _call("ref_grid_template", g.ctypes.data_as(ctypes.c_void_p), ctypes.c_int(N), ctypes.byref(out))
    return out.value


def cad_clean(filename):
    """Mesh::ReadOBJ + RemoveDegenerated + MergeDuplex (the first steps of
    LoadCadMesh, mesh_tensor.cc:105-107): double vertices, int32 faces."""
    nv, nf = ctypes.c_int64(), ctypes.c_int64()
    _call("ref_cad_clean_counts", filename.encode(), ctypes.byref(nv), ctypes.byref(nf))
    V = np.zeros((nv.value, 3), np.float64)
    F = np.zeros((nf.value, 3), np.int32)
    _call("ref_cad_clean", filename.encode(), V.ctypes.data_as(ctypes.c_void_p), F.ctypes.data_as(ctypes.c_void_p))
    return V, F


def install_as_pydeform():
    """Make ``import pyDeform`` resolve to this module (so the reference's
    Python layers run on the reference's C++ loops)."""
    sys.modules["pyDeform"] = sys.modules[__name__]


def reference_path(*parts):
    return os.path.join(build_ref.REF_ROOT, *parts)
