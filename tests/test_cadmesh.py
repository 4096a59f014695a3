"""LoadCadMesh restated (src/interface/mesh_tensor.cc:102-178,
src/lib/subdivision.cc:28-399) on small CAD models, CPU only: the remeshed
faces cover the original faces with edges <= 3 * 0.02, new vertices lie on
the original faces, the neighbour pairs include every mesh edge, the graph
references every vertex to the cluster of int(v/0.01) whose mean it holds,
and the graph edges join different clusters; the output is deterministic."""
import numpy as np
import pytest
import torch

from meshode_gb300 import cadmesh, meshgen, objio
from meshode_gb300 import pyDeform as PD


def _box(c, s):
    V, F = meshgen._box(np.asarray(c, float), np.asarray(s, float))
    return V.astype(np.float64), F.astype(np.int64)


def test_subdivide_box():
    V, F = _box([0.1, 0.2, 0.3], [0.1, 0.07, 0.05])
    Vs, Fs = cadmesh.subdivide(V, F, 0.02)
    assert np.array_equal(Vs[:len(V)], V)
    L = np.linalg.norm(Vs[Fs[:, [0, 1, 2]]] - Vs[Fs[:, [1, 2, 0]]], axis=2)
    assert L.max() <= 3 * 0.02 + 1e-12
    # every new vertex lies on the box surface
    lo, hi = V.min(0), V.max(0)
    on = np.isclose(Vs, lo, atol=1e-9) | np.isclose(Vs, hi, atol=1e-9)
    assert on.any(1).all()
    # the remeshed area equals the box's
    def area(V_, F_):
        return 0.5 * np.linalg.norm(np.cross(V_[F_[:, 1]] - V_[F_[:, 0]], V_[F_[:, 2]] - V_[F_[:, 0]]), axis=1).sum()
    assert area(Vs, Fs) == pytest.approx(area(V, F), rel=1e-9)
    # consistent orientation: remeshed normals agree with the original faces'
    n0 = np.cross(V[F[:, 1]] - V[F[:, 0]], V[F[:, 2]] - V[F[:, 0]]).sum(0)
    n1 = np.cross(Vs[Fs[:, 1]] - Vs[Fs[:, 0]], Vs[Fs[:, 2]] - Vs[Fs[:, 0]]).sum(0)
    assert np.allclose(n0, n1, atol=1e-12)


def test_neighbors_and_graph():
    V, F = _box([0.0, 0.0, 0.0], [0.06, 0.05, 0.04])
    Vs, Fs = cadmesh.subdivide(V, F, 0.02)
    E = cadmesh.geometry_neighbors(Vs, Fs, 1.5e-2)
    assert (E[:, 0] < E[:, 1]).all()
    assert len(np.unique(E, axis=0)) == len(E)
    fe = {tuple(sorted(e)) for f in Fs.tolist() for e in ((f[0], f[1]), (f[1], f[2]), (f[2], f[0]))}
    assert fe <= {tuple(e) for e in E.tolist()}
    ref, GV, GE = cadmesh.representative_graph(Vs, Fs, E, 1e-2)
    keys = np.trunc(Vs / 1e-2).astype(np.int64)
    for g in range(len(GV)):
        members = np.flatnonzero(ref == g)
        assert len(np.unique(keys[members], axis=0)) == 1
        assert np.allclose(GV[g], Vs[members].mean(0))
    assert (GE[:, 0] < GE[:, 1]).all() and (ref[E[:, 0]] != ref[E[:, 1]]).sum() > 0


def test_delaunay3d_edges_degenerate():
    P = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0], [0.4, 0.6, 0]], float)
    E = cadmesh.delaunay3d_edges(P)
    assert len(E) == 8  # planar: 4 sides + 4 spokes to the interior point
    P = np.array([[0, 0, 0], [2, 0, 0], [1, 0, 0]], float)
    assert sorted(map(tuple, cadmesh.delaunay3d_edges(P).tolist())) in ([(0, 2), (1, 2)], [(0, 2), (2, 1)])
    P = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], float)
    assert len(cadmesh.delaunay3d_edges(P)) == 6


def test_load_cad_mesh_file(tmp_path):
    V1, F1 = _box([0.0, 0.0, 0.0], [0.05, 0.05, 0.05])
    V2, F2 = _box([0.2, 0.0, 0.0], [0.04, 0.03, 0.02])
    V = np.concatenate([V1, V2])
    F = np.concatenate([F1, F2 + len(V1)])
    objio.write_obj(str(tmp_path / "cad.obj"), V, F)
    out = PD.LoadCadMesh(str(tmp_path / "cad.obj"))
    assert [t.dtype for t in out] == [torch.float32, torch.int32, torch.int32, torch.int32, torch.float32,
                                      torch.int32]
    Vs, Fs, E, ref, GV, GE = out
    assert ref.shape == (Vs.shape[0], 1) and int(ref.max()) == GV.shape[0] - 1
    assert int(Fs.max()) < Vs.shape[0] and int(E.max()) < Vs.shape[0] and int(GE.max()) < GV.shape[0]
    again = PD.LoadCadMesh(str(tmp_path / "cad.obj"))
    assert all(torch.equal(a, b) for a, b in zip(out, again))
