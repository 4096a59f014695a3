"""Iso-surface extraction (meshode_gb300.isosurface, the role of
Mesh::FromDistanceField, mesh.cc:154-179) on the CPU.

* A radial field's level set is a closed, consistently oriented sphere of the
  right radius (every edge in two faces, Euler characteristic 2, normals
  toward increasing values).
* The reference's call (level 0 of an unsigned distance field) is empty.
* A level above 0 of a target's distance field is a closed surface around it.
"""
import numpy as np

from meshode_gb300 import isosurface, meshgen


def _closed(V, F):
    e = np.sort(np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]]), axis=1)
    _, counts = np.unique(e, axis=0, return_counts=True)
    return bool(np.all(counts == 2)), len(V) - len(counts) + len(F)


def test_sphere_level_set():
    N = 40
    z, y, x = np.meshgrid(np.arange(N), np.arange(N), np.arange(N), indexing="ij")
    c = np.array([0.47, 0.52, 0.5])
    g = np.sqrt((x / N - c[0]) ** 2 + (y / N - c[1]) ** 2 + (z / N - c[2]) ** 2).astype(np.float32)
    V, F = isosurface.from_distance_field(g, level=0.3)
    assert len(F) > 1000
    r = np.linalg.norm(V - c, axis=1)
    assert np.abs(r - 0.3).max() < 0.5 / N  # linear interpolation of a curved field
    closed, euler = _closed(V, F)
    assert closed and euler == 2
    # outward: toward increasing distance from the centre
    P = V[F]
    n = np.cross(P[:, 1] - P[:, 0], P[:, 2] - P[:, 0])
    assert np.all((n * (P.mean(1) - c)).sum(1) > 0)


def test_reference_level_zero_is_empty():
    g = np.random.Generator(np.random.PCG64(0)).uniform(0.01, 1.0, size=16 ** 3).astype(np.float32)
    V, F = isosurface.from_distance_field(g)
    assert V.shape == (0, 3) and F.shape == (0, 3)


def test_offset_surface_of_a_target(orc):
    V, F = meshgen.icosphere(2)
    sc, tr = orc.normalize_params(V.astype(np.float32))
    Vn = orc.normalized_double(V.astype(np.float32), sc, tr)
    N = 24
    grid = orc.df_build(Vn, F.astype(np.int32), N, method="bvh")
    Vs, Fs = isosurface.from_distance_field(grid, level=2.0 / N)
    assert len(Fs) > 1000
    # an inner and an outer shell; the outer one reaches past the grid's far
    # faces (the target spans [0.05, 0.959], the grid [0, 23/24]), so the
    # only open edges lie on the grid boundary
    e = np.sort(np.concatenate([Fs[:, [0, 1]], Fs[:, [1, 2]], Fs[:, [2, 0]]]), axis=1)
    ue, counts = np.unique(e, axis=0, return_counts=True)
    assert set(np.unique(counts).tolist()) <= {1, 2}
    ends = Vs[ue[counts == 1]].reshape(-1, 3)
    on_face = (np.abs(ends) < 1e-9) | (np.abs(ends - (N - 1) / N) < 1e-9)
    assert len(ends) > 0 and on_face.any(1).all()
