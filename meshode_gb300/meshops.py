"""Host-side mesh utilities used by the command-line front ends.

Restated from the reference's Mesh class (src/lib/mesh.cc):
* ``reflection_symmetrize`` -- Mesh::ReflectionSymmetrize (mesh.cc:234-246):
  append the mirror image x -> -x of every vertex and a copy of every face.
* ``remove_degenerated`` -- Mesh::RemoveDegenerated (mesh.cc:320-333): drop
  faces whose cross product has zero norm.
* ``merge_duplex`` -- Mesh::MergeDuplex (mesh.cc:181-232): merge vertices whose
  coordinates truncated at 1e-6 (int(v*1e6)) coincide, keep the first, remap
  faces, then drop faces with a repeated corner and faces whose sorted corner
  triple was already seen.
* ``subdivide_to`` -- midpoint subdivision until the mesh has at least the
  requested number of vertices (the meaning given here to MESH_RESOLUTION,
  which the reference parses but never uses: src/app/rigid_deform.cc:36-37).
All work in float64 like the reference's Mesh.
"""
import numpy as np


def reflection_symmetrize(V, F):
    V = np.asarray(V, np.float64)
    F = np.asarray(F, np.int64)
    Vr = V * np.array([-1.0, 1.0, 1.0])
    return np.concatenate([V, Vr], 0), np.concatenate([F, F + V.shape[0]], 0)


def remove_degenerated(V, F):
    V = np.asarray(V, np.float64)
    F = np.asarray(F, np.int64)
    n = np.cross(V[F[:, 1]] - V[F[:, 0]], V[F[:, 2]] - V[F[:, 0]])
    return V, F[np.linalg.norm(n, axis=1) > 0]


def _trunc_int(x):
    # double -> int conversion of the key (truncation toward zero)
    return np.trunc(x).astype(np.int64)


def merge_duplex(V, F):
    V = np.asarray(V, np.float64)
    F = np.asarray(F, np.int64)
    keys = _trunc_int(V * 1e6)
    seen = {}
    shrink = np.empty(V.shape[0], np.int64)
    keep = []
    for i, k in enumerate(map(tuple, keys)):
        j = seen.get(k)
        if j is None:
            j = len(keep)
            seen[k] = j
            keep.append(i)
        shrink[i] = j
    V2 = V[keep]
    F2 = shrink[F]
    out, faces = [], set()
    for f in F2:
        a, b, c = int(f[0]), int(f[1]), int(f[2])
        if a == b or b == c or c == a:
            continue
        k = tuple(sorted((a, b, c)))
        if k in faces:
            continue
        faces.add(k)
        out.append((a, b, c))
    return V2, np.asarray(out, np.int64).reshape(-1, 3)


def _midpoint_subdivide(V, F):
    e = np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]], 0)
    e.sort(axis=1)
    key = e[:, 0] * (V.shape[0] + 1) + e[:, 1]
    uniq, inv = np.unique(key, return_inverse=True)
    a, b = uniq // (V.shape[0] + 1), uniq % (V.shape[0] + 1)
    mid = 0.5 * (V[a] + V[b])
    nf = F.shape[0]
    m01, m12, m20 = V.shape[0] + inv[:nf], V.shape[0] + inv[nf:2 * nf], V.shape[0] + inv[2 * nf:]
    F2 = np.concatenate([np.stack([F[:, 0], m01, m20], 1), np.stack([F[:, 1], m12, m01], 1),
                         np.stack([F[:, 2], m20, m12], 1), np.stack([m01, m12, m20], 1)], 0)
    return np.concatenate([V, mid], 0), F2


def subdivide_to(V, F, min_vertices, max_rounds=8):
    V = np.asarray(V, np.float64)
    F = np.asarray(F, np.int64)
    for _ in range(max_rounds):
        if V.shape[0] >= min_vertices or F.shape[0] == 0:
            break
        V, F = _midpoint_subdivide(V, F)
    return V, F
