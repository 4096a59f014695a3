"""Seeded synthetic meshes with the shapes of the benchmark workloads.

The reference ships only four demo OBJ files and the 3,265-pair download set
is unavailable offline, so the workloads are generated:

* ``icosphere(level)``: 10*4^L + 2 vertices, 20*4^L triangles.
* ``cubesphere(n)``: a subdivided cube projected to the unit sphere,
  6*n^2 + 2 vertices, 12*n^2 triangles (any size between icosphere levels).
* ``displace(V, rng)``: radial displacement r = 1 + 0.15*sum_k s_k(theta, phi),
  s_k = a_k*sin(m_k*theta + alpha_k)*cos(n_k*phi + beta_k), 8 terms,
  m_k, n_k in [1, 6], phases ~U[0, 2pi), a_k = 1/8; then anisotropic scale
  (1.2, 0.9, 0.8) and a rotation about a random axis by an angle ~U[0, 20 deg].
* ``rigid_pair_ico5`` (the plain rigid-deform workload): icosphere level 5 source,
  displaced level-5 target, numpy PCG64(seed=1).
* ``large_pair``: displaced icosphere level 8 target (1,310,720 triangles),
  a ~200k-vertex cube-sphere source with a per-vertex Gaussian
  perturbation (sigma 0.02), PCG64(seed=3).
* ``serving_requests``: the 512-request stream: source vertices log-uniform in
  [2k, 100k], target triangles log-uniform in [5k, 500k], grid 64 or 128
  (50/50), Poisson arrivals at 200 requests/s, PCG64(seed=5).
* ``cad_pair``: 40 seeded boxes and cylinders (12-256 triangles each) as the
  source, the same primitives jittered by +-20% plus a 2k-triangle noisy plane
  as the target, PCG64(seed=2).
"""
import math

import numpy as np


# ---------------------------------------------------------------------------
# base shapes
# ---------------------------------------------------------------------------
def _subdivide(V, F):
    """Split every triangle into four with shared, deduplicated midpoints."""
    e = np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]], 0)
    e.sort(axis=1)
    key = e[:, 0].astype(np.int64) * (V.shape[0] + 1) + e[:, 1]
    uniq, inv = np.unique(key, return_inverse=True)
    a = (uniq // (V.shape[0] + 1)).astype(np.int64)
    b = (uniq % (V.shape[0] + 1)).astype(np.int64)
    mid = 0.5 * (V[a] + V[b])
    mid /= np.linalg.norm(mid, axis=1, keepdims=True)
    nf = F.shape[0]
    m01 = V.shape[0] + inv[:nf]
    m12 = V.shape[0] + inv[nf:2 * nf]
    m20 = V.shape[0] + inv[2 * nf:]
    V2 = np.concatenate([V, mid], 0)
    F2 = np.concatenate([
        np.stack([F[:, 0], m01, m20], 1),
        np.stack([F[:, 1], m12, m01], 1),
        np.stack([F[:, 2], m20, m12], 1),
        np.stack([m01, m12, m20], 1)], 0)
    return V2, F2


def icosphere(level):
    """Unit icosphere: returns (V float64 [n,3], F int64 [m,3])."""
    t = (1.0 + 5 ** 0.5) / 2.0
    V = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0],
                  [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], np.float64)
    V /= np.linalg.norm(V, axis=1, keepdims=True)
    F = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
                  [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
                  [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
                  [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], np.int64)
    for _ in range(level):
        V, F = _subdivide(V, F)
    return V, F


def cubesphere(n):
    """Cube with n x n quads per face projected to the unit sphere."""
    n = max(int(n), 1)
    s = np.linspace(-1.0, 1.0, n + 1)
    U, W = np.meshgrid(s, s, indexing="ij")
    faces_pts = []
    for axis in range(3):
        for sign in (-1.0, 1.0):
            P = np.zeros((n + 1, n + 1, 3))
            P[..., axis] = sign
            P[..., (axis + 1) % 3] = U
            P[..., (axis + 2) % 3] = W * sign
            faces_pts.append(P.reshape(-1, 3))
    allp = np.concatenate(faces_pts, 0)
    q = np.round((allp + 1.0) * n).astype(np.int64)
    key = (q[:, 0] * (2 * n + 1) + q[:, 1]) * (2 * n + 1) + q[:, 2]
    uniq, first, inv = np.unique(key, return_index=True, return_inverse=True)
    V = allp[first]
    V = V / np.linalg.norm(V, axis=1, keepdims=True)
    ii, jj = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    ii = ii.reshape(-1); jj = jj.reshape(-1)
    Fs = []
    stride = (n + 1) * (n + 1)
    for f in range(6):
        base = f * stride
        a = base + ii * (n + 1) + jj
        b = a + (n + 1)
        c = b + 1
        d = a + 1
        Fs.append(np.stack([a, b, c], 1))
        Fs.append(np.stack([a, c, d], 1))
    F = inv[np.concatenate(Fs, 0)]
    return V, F.astype(np.int64)


def _rotation(axis, angle):
    axis = axis / np.linalg.norm(axis)
    x, y, z = axis
    c, s = math.cos(angle), math.sin(angle)
    C = 1 - c
    return np.array([[c + x * x * C, x * y * C - z * s, x * z * C + y * s],
                     [y * x * C + z * s, c + y * y * C, y * z * C - x * s],
                     [z * x * C - y * s, z * y * C + x * s, c + z * z * C]])


def displace(V, rng, amp=0.15, terms=8):
    """Radial sinusoidal displacement + anisotropic scale + random rotation."""
    r = np.linalg.norm(V, axis=1)
    theta = np.arccos(np.clip(V[:, 2] / r, -1, 1))
    phi = np.arctan2(V[:, 1], V[:, 0])
    m = rng.integers(1, 7, size=terms)
    nn = rng.integers(1, 7, size=terms)
    al = rng.uniform(0, 2 * np.pi, size=terms)
    be = rng.uniform(0, 2 * np.pi, size=terms)
    a = np.full(terms, 1.0 / terms)
    s = np.zeros_like(r)
    for k in range(terms):
        s += a[k] * np.sin(m[k] * theta + al[k]) * np.cos(nn[k] * phi + be[k])
    rad = 1.0 + amp * s
    out = V / r[:, None] * rad[:, None]
    out = out * np.array([1.2, 0.9, 0.8])
    axis = rng.normal(size=3)
    angle = math.radians(rng.uniform(0, 20))
    return out @ _rotation(axis, angle).T


def _as32(V, F):
    return np.ascontiguousarray(V, np.float32), np.ascontiguousarray(F, np.int32)


# ---------------------------------------------------------------------------
# workloads
# ---------------------------------------------------------------------------
def rigid_pair_ico5(seed=1):
    """Plain rigid deform: ico-5 source (10,242 v / 20,480 f) -> displaced ico-5."""
    rng = np.random.Generator(np.random.PCG64(seed))
    V, F = icosphere(5)
    T = displace(V, rng)
    return _as32(V, F) + _as32(T, F)


def cubesphere_for_vertices(nv):
    n = max(2, int(round(math.sqrt(max(nv - 2, 6) / 6.0))))
    return cubesphere(n)


def cubesphere_for_triangles(nt):
    n = max(2, int(round(math.sqrt(max(nt, 12) / 12.0))))
    return cubesphere(n)


def large_pair(seed=3, target_level=8, source_vertices=200_000, sigma=0.02):
    """Large-scale build and loss: ico-8 target (1.31M tris), 200k-vertex source."""
    rng = np.random.Generator(np.random.PCG64(seed))
    Vt, Ft = icosphere(target_level)
    Vt = displace(Vt, rng)
    Vs, Fs = cubesphere_for_vertices(source_vertices)
    Vs = Vs + rng.normal(scale=sigma, size=Vs.shape)
    return _as32(Vs, Fs) + _as32(Vt, Ft)


def serving_requests(n=512, seed=5, rate=200.0, steps=500,
                     v_range=(2_000, 100_000), t_range=(5_000, 500_000), grids=(64, 128)):
    """The mixed request stream; returns a list of dicts (meshes generated lazily
    by ``request_meshes``)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    nv = np.exp(rng.uniform(math.log(v_range[0]), math.log(v_range[1]), size=n))
    nt = np.exp(rng.uniform(math.log(t_range[0]), math.log(t_range[1]), size=n))
    Ns = rng.choice(np.asarray(grids), size=n)
    gaps = rng.exponential(1.0 / rate, size=n)
    arrivals = np.cumsum(gaps) - gaps[0]
    seeds = rng.integers(0, 2 ** 31 - 1, size=n)
    return [dict(id=i, nv=int(nv[i]), nt=int(nt[i]), N=int(Ns[i]), arrival=float(arrivals[i]),
                 seed=int(seeds[i]), steps=int(steps)) for i in range(n)]


def request_meshes(req):
    """(srcV, srcF, tarV, tarF) float32/int32 for one serving request."""
    rng = np.random.Generator(np.random.PCG64(req["seed"]))
    Vs, Fs = cubesphere_for_vertices(req["nv"])
    Vt, Ft = cubesphere_for_triangles(req["nt"])
    Vt = displace(Vt, rng)
    return _as32(Vs, Fs) + _as32(Vt, Ft)


def _box(center, size):
    c = np.asarray(center); s = np.asarray(size) / 2
    V = np.array([[x, y, z] for x in (-1, 1) for y in (-1, 1) for z in (-1, 1)], np.float64) * s + c
    F = np.array([[0, 1, 3], [0, 3, 2], [4, 6, 7], [4, 7, 5], [0, 4, 5], [0, 5, 1],
                  [2, 3, 7], [2, 7, 6], [0, 2, 6], [0, 6, 4], [1, 5, 7], [1, 7, 3]], np.int64)
    return V, F


def _cylinder(center, radius, height, k):
    ang = np.arange(k) * 2 * np.pi / k
    ring = np.stack([np.cos(ang) * radius, np.sin(ang) * radius, np.zeros(k)], 1)
    bot = ring + np.asarray(center) + [0, 0, -height / 2]
    top = ring + np.asarray(center) + [0, 0, height / 2]
    cb = np.asarray(center) + [0, 0, -height / 2]
    ct = np.asarray(center) + [0, 0, height / 2]
    V = np.concatenate([bot, top, cb[None], ct[None]], 0)
    F = []
    for i in range(k):
        j = (i + 1) % k
        F += [[i, j, k + j], [i, k + j, k + i], [2 * k, j, i], [2 * k + 1, k + i, k + j]]
    return V, np.asarray(F, np.int64)


def _merge(parts):
    Vs, Fs, off = [], [], 0
    for V, F in parts:
        Vs.append(V); Fs.append(F + off); off += V.shape[0]
    return np.concatenate(Vs, 0), np.concatenate(Fs, 0)


def cad_pair(seed=2, n_prims=40, plane_tris=2000):
    """CAD-style non-watertight pair (disconnected boxes and cylinders)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    src, tar = [], []
    for _ in range(n_prims):
        c = rng.uniform(-1, 1, size=3)
        if rng.uniform() < 0.5:
            s = rng.uniform(0.1, 0.4, size=3)
            src.append(_box(c, s))
            tar.append(_box(c + rng.uniform(-0.2, 0.2, 3) * s, s * rng.uniform(0.8, 1.2, 3)))
        else:
            k = int(rng.integers(3, 65))
            r, h = rng.uniform(0.05, 0.2), rng.uniform(0.1, 0.5)
            src.append(_cylinder(c, r, h, k))
            tar.append(_cylinder(c + rng.uniform(-0.2, 0.2, 3) * r, r * rng.uniform(0.8, 1.2),
                                 h * rng.uniform(0.8, 1.2), k))
    g = int(round(math.sqrt(plane_tris / 2)))
    xs = np.linspace(-1.2, 1.2, g + 1)
    X, Y = np.meshgrid(xs, xs, indexing="ij")
    Z = -1.2 + rng.normal(scale=0.01, size=X.shape)
    PV = np.stack([X, Y, Z], -1).reshape(-1, 3)
    ii, jj = np.meshgrid(np.arange(g), np.arange(g), indexing="ij")
    a = (ii * (g + 1) + jj).reshape(-1)
    PF = np.concatenate([np.stack([a, a + g + 1, a + g + 2], 1), np.stack([a, a + g + 2, a + 1], 1)], 0)
    tar.append((PV, PF))
    Vs, Fs = _merge(src)
    Vt, Ft = _merge(tar)
    return _as32(Vs, Fs) + _as32(Vt, Ft)


def edges_from_faces(F):
    """Undirected unique edge list of a triangle mesh, int32 [E,2] (i < j)."""
    e = np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]], 0).astype(np.int64)
    e.sort(axis=1)
    e = np.unique(e, axis=0)
    return np.ascontiguousarray(e, np.int32)
