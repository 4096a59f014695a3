"""The oracle pinned to the reference's own source text (CPU, no GPU).

oracle/_ref is the reference's pyDeform loops compiled unchanged from the
reference tree (uniformgrid.cc, mesh.cc, deform_params.cc, mesh_tensor.cc,
distance_layer.cc, rigid_layer.cc, graph_layer.cc, cad_layer.cc,
normalize.cc) against stand-ins for its un-vendored dependencies (Eigen,
ceres::Jet, torch, and libigl's point-mesh distance, which is the oracle's
FP64 tree).  These tests check the oracle's C restatement, the host-side
readers and the committed reference fixtures against it, bit for bit, on
the reference's own demo meshes (data/source.obj, target.obj,
cad-source.obj, cad-target.obj) and on probes at every branch of
UniformGrid::DistanceFloat (uniformgrid.cc:85-150).

They run only where the reference is mounted (the library is built from
its sources); elsewhere they skip.
"""
import hashlib
import os

import numpy as np
import pytest
import torch

from meshode_gb300 import meshops, objio
from oracle import ref as R

pytestmark = pytest.mark.skipif(not R.available(), reason="the reference's sources are not mounted")

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _data(name):
    return R.reference_path("data", name)


def _bits_equal(a, b):
    """Equal bit patterns, except that any NaN equals any NaN (the payload
    and sign of a NaN made by an invalid operation differ between x86, Arm
    and the GPU)."""
    a = np.ascontiguousarray(np.asarray(a))
    b = np.ascontiguousarray(np.asarray(b))
    if a.shape != b.shape or a.dtype != b.dtype:
        return False
    if a.dtype.kind != "f":
        return a.tobytes() == b.tobytes()
    na, nb = np.isnan(a), np.isnan(b)
    if not np.array_equal(na, nb):
        return False
    return a[~na].tobytes() == b[~nb].tobytes()


@pytest.fixture(scope="module")
def meshes():
    out = {}
    for name in ("source.obj", "target.obj", "cad-source.obj", "cad-target.obj"):
        out[name] = R.LoadMesh(_data(name))
    return out


def test_load_mesh_counts_and_reader(meshes):
    """pyDeform.LoadMesh (mesh_tensor.cc:87-100 over Mesh::ReadOBJ,
    mesh.cc:14-44) on the demo meshes: the counts of the files, and the
    host reader returns the same arrays bit for bit (including the
    ``f a//n`` records of the CAD meshes)."""
    from meshode_gb300 import pyDeform as PD
    counts = {"source.obj": (21542, 43100), "target.obj": (14762, 29532),
              "cad-source.obj": (2856, 11436), "cad-target.obj": (70, 272)}
    for name, (nv, nf) in counts.items():
        V, F = meshes[name]
        assert (V.shape[0], F.shape[0]) == (nv, nf), name
        V2, F2 = PD.LoadMesh(_data(name))
        assert _bits_equal(V.numpy(), V2.numpy()), name
        assert _bits_equal(F.numpy(), F2.numpy()), name


def test_committed_fixture_is_the_reference_output(meshes):
    """tests/golden/ref_demo_meshes.npz holds LoadMesh's output for the demo
    meshes (so that GPU tests can use them where the reference is not
    mounted); it must equal the reference's LoadMesh and name the files'
    SHA-256."""
    z = np.load(os.path.join(GOLDEN, "ref_demo_meshes.npz"))
    for name in ("source.obj", "target.obj", "cad-source.obj", "cad-target.obj"):
        key = name.replace(".obj", "").replace("-", "_")
        V, F = meshes[name]
        assert _bits_equal(z[key + "_V"], V.numpy()), name
        assert _bits_equal(z[key + "_F"], F.numpy()), name
        sha = hashlib.sha256(open(_data(name), "rb").read()).hexdigest()
        assert str(z[key + "_sha256"]) == sha, name


def test_template_transform_and_grid(orc, meshes):
    """InitializeDeformTemplate (deform_params.cc:16-40): Mesh::Normalize's
    scale and translation bit for bit; the distance grid (mesh.cc:106-152)
    equals the oracle's FP64 grid bit for bit (both take the same FP64
    point-triangle distance; the reference adds the sampling, the sqrt and
    the [z][y][x] storage)."""
    T, TF = meshes["target.obj"]
    N = 32
    pid = R.InitializeDeformTemplate(T, TF, 0, N)
    scale, trans = R.template_transform(pid)
    oscale, otrans = orc.normalize_params(T.numpy())
    assert scale == oscale and _bits_equal(trans, otrans)
    grid = R.template_grid(pid, N)
    Tn = orc.normalized_double(T.numpy(), oscale, otrans)
    assert _bits_equal(grid, orc.df_build(Tn, TF.numpy(), N))


def _probes(N, rng, n=4000):
    """Points at every branch of DistanceFloat: inside, on cell faces, in the
    (-1/N, 0) truncation slab, in the N-1 slab that adds no penalty, beyond
    it, far outside, NaN."""
    P = [rng.uniform(-0.3, 1.3, (n, 3))]
    P.append(rng.uniform(-1.0 / N, 0, (n // 4, 3)))
    P.append(rng.uniform((N - 1) / N, 1.0, (n // 4, 3)))
    P.append(rng.integers(0, N, (n // 4, 3)) / N)
    P.append(rng.uniform(-3e9, 3e9, (32, 3)))
    q = rng.uniform(0, 1, (16, 3))
    q[::2, 0] = np.nan
    P.append(q)
    mix = rng.uniform(0, 1, (n // 4, 3))
    pick = rng.integers(0, 3, n // 4)
    mix[np.arange(n // 4), pick] = rng.choice([-0.5 / N, (N - 1) / N, (N - 0.5) / N, 1.0 + 1e-3], n // 4)
    P.append(mix)
    return np.ascontiguousarray(np.concatenate(P).astype(np.float32))


@pytest.mark.parametrize("N", [8, 32])
def test_distance_float_every_branch(orc, N):
    """DistanceFieldLoss_forward/_backward (distance_layer.cc:8-81) over
    UniformGrid::DistanceFloat<float> and <Jet<float,3>>, on a random grid
    whose values straddle the 0.2 cutoff: the oracle equals the reference
    bit for bit (NaN for NaN)."""
    rng = np.random.Generator(np.random.PCG64(N))
    grid = rng.uniform(0.0, 0.35, N ** 3)
    pid = R.grid_template(grid, N)
    opid = orc.InitializeDeformTemplate(np.zeros((3, 3), np.float32), np.array([[0, 1, 2]], np.int32), 0, N,
                                        grid=grid.astype(np.float32))
    P = torch.from_numpy(_probes(N, rng))
    assert _bits_equal(R.DistanceFieldLoss_forward(P, pid).numpy(), orc.DistanceFieldLoss_forward(P, opid).numpy())
    assert _bits_equal(R.DistanceFieldLoss_backward(P, pid).numpy(),
                       orc.DistanceFieldLoss_backward(P, opid).numpy())


def test_demo_pair_losses_and_normalisation(orc, meshes):
    """source.obj -> target.obj as rigid_deform.py sets it up: the
    normalisation in place, DistanceFieldLoss and RigidEdgeLoss forward and
    backward at the normalised source and at a perturbed copy, and the
    denormalisation: the oracle equals the reference bit for bit."""
    (S, SF), (T, TF) = meshes["source.obj"], meshes["target.obj"]
    N = 64
    pid = R.InitializeDeformTemplate(T, TF, 0, N)
    grid = R.template_grid(pid, N)
    opid = orc.InitializeDeformTemplate(T.numpy(), TF.numpy(), 0, N, grid=grid.astype(np.float32))
    Vr, Vo = S.clone(), S.clone()
    R.NormalizeByTemplate(Vr, pid)
    orc.NormalizeByTemplate(Vo, opid)
    assert _bits_equal(Vr.numpy(), Vo.numpy())
    R.StoreRigidityInformation(Vr, SF, pid)
    orc.StoreRigidityInformation(Vo, SF, opid)
    off, _ = R.template_edges(pid, 3 * SF.shape[0])
    assert _bits_equal(off, np.asarray(orc.GetParams(opid).edge_offset, np.float32).reshape(-1, 3))
    rng = np.random.Generator(np.random.PCG64(7))
    for V in (Vr, Vr + torch.from_numpy(rng.normal(0, 0.01, Vr.shape).astype(np.float32))):
        V = V.contiguous()
        assert _bits_equal(R.DistanceFieldLoss_forward(V, pid).numpy(), orc.DistanceFieldLoss_forward(V, opid).numpy())
        assert _bits_equal(R.DistanceFieldLoss_backward(V, pid).numpy(),
                           orc.DistanceFieldLoss_backward(V, opid).numpy())
        assert _bits_equal(R.RigidEdgeLoss_forward(V, SF, pid).numpy(),
                           orc.RigidEdgeLoss_forward(V, SF, opid).numpy())
        assert _bits_equal(R.RigidEdgeLoss_backward(V, SF, pid).numpy(),
                           orc.RigidEdgeLoss_backward(V, SF, opid).numpy())
    R.DenormalizeByTemplate(Vr, pid)
    orc.DenormalizeByTemplate(Vo, opid)
    assert _bits_equal(Vr.numpy(), Vo.numpy())


def test_graph_edges(orc, meshes):
    """StoreGraphInformation / GraphEdgeLoss_forward/_backward
    (graph_layer.cc:11-135) on the CAD source's unique edges."""
    V, F = meshes["cad-source.obj"]
    Fn = F.numpy()
    E = np.unique(np.sort(np.concatenate([Fn[:, [0, 1]], Fn[:, [1, 2]], Fn[:, [2, 0]]]), axis=1), axis=0)
    E = torch.from_numpy(np.ascontiguousarray(E.astype(np.int32)))
    pid = R.grid_template(np.zeros(8), 2)
    opid = orc.InitializeDeformTemplate(np.zeros((3, 3), np.float32), np.array([[0, 1, 2]], np.int32), 0, 2,
                                        grid=np.zeros(8, np.float32))
    R.StoreGraphInformation(V, E, pid)
    orc.StoreGraphInformation(V, E, opid)
    rng = np.random.Generator(np.random.PCG64(8))
    W = (V + torch.from_numpy(rng.normal(0, 0.05, V.shape).astype(np.float32))).contiguous()
    assert _bits_equal(R.GraphEdgeLoss_forward(W, E, pid).numpy(), orc.GraphEdgeLoss_forward(W, E, opid).numpy())
    assert _bits_equal(R.GraphEdgeLoss_backward(W, E, pid).numpy(), orc.GraphEdgeLoss_backward(W, E, opid).numpy())


def test_cad_cleaning_steps():
    """Mesh::RemoveDegenerated + MergeDuplex (mesh.cc:181-232, 320-333), the
    first steps of LoadCadMesh, on the CAD demo meshes: the host
    restatement in meshops gives the reference's vertices and faces."""
    for name in ("cad-source.obj", "cad-target.obj"):
        Vr, Fr = R.cad_clean(_data(name))
        V, F = objio.read_obj(_data(name))
        V, F = meshops.remove_degenerated(V, F)
        V2, F2 = meshops.merge_duplex(V, F)
        assert _bits_equal(np.asarray(V2, np.float64), Vr), name
        assert _bits_equal(np.asarray(F2, np.int32), Fr), name


def test_rigid_loop_matches_reference_layers(orc, meshes):
    """The reference's RigidLossLayer (src/python/layers/rigid_loss_layer.py)
    and the loop of rigid_deform.py:28-39, run over the reference's C++
    loops, against the oracle's loop (orc.rigid_fit, torch CPU Adam) on the
    demo pair: identical positions after 20 steps."""
    import importlib.util
    import sys
    (S, SF), (T, TF) = meshes["source.obj"], meshes["target.obj"]
    saved = sys.modules.get("pyDeform")
    R.install_as_pydeform()
    try:
        spec = importlib.util.spec_from_file_location(
            "ref_rigid_loss_layer", R.reference_path("src", "python", "layers", "rigid_loss_layer.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        src_V = S.clone()
        layer = mod.RigidLossLayer(src_V, SF, T, TF)
        pid = int(layer.param_id)
        src_V = torch.nn.Parameter(src_V)
        opt = torch.optim.Adam([src_V], lr=1e-3)
        for _ in range(20):
            opt.zero_grad()
            loss = layer(src_V, SF)
            loss.backward()
            opt.step()
    finally:
        if saved is None:
            sys.modules.pop("pyDeform", None)
        else:
            sys.modules["pyDeform"] = saved
    grid = R.template_grid(pid, 64)
    opid = orc.InitializeDeformTemplate(T.numpy(), TF.numpy(), 0, 64, grid=grid.astype(np.float32))
    Vo = S.clone()
    orc.NormalizeByTemplate(Vo, opid)
    orc.StoreRigidityInformation(Vo, SF, opid)
    out, _ = orc.rigid_fit(Vo, SF, opid, 20)
    assert _bits_equal(src_V.detach().numpy(), out.numpy())


def test_cad_edges(orc, meshes):
    """StoreCadInformation / CadEdgeLoss_forward/_backward
    (cad_layer.cc:11-223): E's edges then F's half-edges, the weights
    2e-2/(|off|+1e-8), the weighted residuals and their serial scatter, on
    the CAD source with its unique edges as E."""
    V, F = meshes["cad-source.obj"]
    Fn = F.numpy()
    E = np.unique(np.sort(np.concatenate([Fn[:, [0, 1]], Fn[:, [1, 2]]]), axis=1), axis=0)
    E = torch.from_numpy(np.ascontiguousarray(E[::3].astype(np.int32)))
    pid = R.grid_template(np.zeros(8), 2)
    opid = orc.InitializeDeformTemplate(np.zeros((3, 3), np.float32), np.array([[0, 1, 2]], np.int32), 0, 2,
                                        grid=np.zeros(8, np.float32))
    R.StoreCadInformation(V, F, E, pid)
    orc.StoreCadInformation(V, F, E, opid)
    nh = E.shape[0] + 3 * F.shape[0]
    off, lam = R.template_edges(pid, nh)
    assert _bits_equal(off, orc.GetParams(opid).edge_offset)
    assert _bits_equal(lam, orc.GetParams(opid).edge_lambda)
    rng = np.random.Generator(np.random.PCG64(9))
    W = (V + torch.from_numpy(rng.normal(0, 0.02, V.shape).astype(np.float32))).contiguous()
    assert _bits_equal(R.CadEdgeLoss_forward(W, F, E, pid).numpy(), orc.CadEdgeLoss_forward(W, F, E, opid).numpy())
    assert _bits_equal(R.CadEdgeLoss_backward(W, F, E, pid).numpy(),
                       orc.CadEdgeLoss_backward(W, F, E, opid).numpy())
