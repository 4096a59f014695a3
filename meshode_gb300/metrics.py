"""Evaluation metric: symmetric Chamfer distance (CPU, FP64).

The reference defines no Chamfer metric.  Here it is the symmetric mean
nearest-neighbour Euclidean distance between two point sets, each made of the
mesh's vertices plus ``samples`` area-uniform surface samples (numpy PCG64,
``seed``), computed with scipy's cKDTree (the tool the reference uses for its
reverse loss, src/python/layers/reverse_loss_layer.py:18) in the coordinates
given (the target-normalised unit cube for the benchmark).
"""
import numpy as np


def surface_samples(V, F, n, seed=0):
    V = np.asarray(V, np.float64)
    F = np.asarray(F, np.int64)
    if n <= 0 or F.shape[0] == 0:
        return np.zeros((0, 3))
    a, b, c = V[F[:, 0]], V[F[:, 1]], V[F[:, 2]]
    area = 0.5 * np.linalg.norm(np.cross(b - a, c - a), axis=1)
    tot = area.sum()
    rng = np.random.Generator(np.random.PCG64(seed))
    p = area / tot if tot > 0 else np.full(F.shape[0], 1.0 / F.shape[0])
    idx = rng.choice(F.shape[0], size=n, p=p)
    u = rng.uniform(size=n)
    v = rng.uniform(size=n)
    flip = u + v > 1
    u[flip], v[flip] = 1 - u[flip], 1 - v[flip]
    return a[idx] + u[:, None] * (b[idx] - a[idx]) + v[:, None] * (c[idx] - a[idx])


def point_set(V, F, samples=100_000, seed=0):
    V = np.asarray(V, np.float64)
    return np.concatenate([V, surface_samples(V, F, samples, seed)], 0)


def chamfer(VA, FA, VB, FB, samples=100_000, seed=0):
    """Symmetric mean nearest-neighbour distance between two meshes."""
    from scipy.spatial import cKDTree
    A = point_set(VA, FA, samples, seed)
    B = point_set(VB, FB, samples, seed)
    da, _ = cKDTree(B).query(A, k=1, workers=-1)
    db, _ = cKDTree(A).query(B, k=1, workers=-1)
    return 0.5 * (float(da.mean()) + float(db.mean()))
