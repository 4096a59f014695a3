"""Generate tests/golden/meshode_golden.npz.

The reference ships no golden vectors and cannot be built here, so these
fixtures come from a second, independent restatement of the reference's
arithmetic, written here in numpy scalar float32 operations (one rounding per
operation, no fused multiply-add) and numpy float64:

* UniformGrid::DistanceFloat<float> and <ceres::Jet<float,3>>
  (src/lib/uniformgrid.cc:85-150) -- a small dual-number class;
* DistanceFieldLoss_forward/_backward (src/interface/distance_layer.cc:8-81);
* StoreRigidityInformation / RigidEdgeLoss_forward / _backward
  (src/interface/rigid_layer.cc:11-133), serial loops;
* Mesh::Normalize and NormalizeByTemplate (src/lib/mesh.cc:66-96,
  src/interface/normalize.cc:5-45);
* the unsigned distance field of Mesh::ConstructDistanceField
  (mesh.cc:106-152) by FP64 brute force with Ericson's closest-point-on-
  triangle regions (a different formulation from the oracle's).

tests/test_golden.py checks the C oracle against these values (bit for bit
for the float32 paths, 1e-12 for the FP64 distance field).  Run from the
repository root: python tests/golden/gen_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
f32 = np.float32


def trunc_x86(v):
    """int(float) with x86-64 cvttss2si semantics."""
    v = float(v)
    if v != v or not (-2147483648.0 <= v < 2147483648.0):
        return -2147483648
    return int(v)


class Dual:
    """Forward-mode dual number with 3 float32 derivative slots."""

    def __init__(self, a, v=(0.0, 0.0, 0.0)):
        self.a = f32(a)
        self.v = [f32(x) for x in v]

    def __add__(self, o):
        return Dual(self.a + o.a, [x + y for x, y in zip(self.v, o.v)])

    def __sub__(self, o):
        return Dual(self.a - o.a, [x - y for x, y in zip(self.v, o.v)])

    def __neg__(self):
        return Dual(-self.a, [-x for x in self.v])

    def __mul__(self, o):
        return Dual(self.a * o.a, [self.a * y + x * o.a for x, y in zip(self.v, o.v)])


def grid_at(g, N, z, y, x):
    return f32(g[(z * N + y) * N + x])


def distance(g, N, p, jet):
    """DistanceFloat<T> with T = float (jet=False) or Jet<float,3>."""
    if jet:
        P = [Dual(p[k], [1.0 if j == k else 0.0 for j in range(3)]) for k in range(3)]
        C = lambda x: Dual(x)  # noqa: E731
    else:
        P = [f32(x) for x in p]
        C = f32
    Nf = f32(N)
    av = lambda q: q.a if jet else q  # noqa: E731
    px = trunc_x86(av(P[0]) * Nf)
    py = trunc_x86(av(P[1]) * Nf)
    pz = trunc_x86(av(P[2]) * Nf)
    if px < 0 or py < 0 or pz < 0 or px >= N - 1 or py >= N - 1 or pz >= N - 1:
        K = C(f32((N - 1) - 1e-3))
        NN = C(Nf)
        l = C(f32(0.0))
        for q, pi in ((P[0], px), (P[1], py), (P[2], pz)):
            if pi < 0:
                l = l + (-q) * NN
            elif pi >= N:
                l = l + (q * NN - K)
        return l
    NN = C(Nf)
    wx = P[0] * NN - C(f32(px))
    wy = P[1] * NN - C(f32(py))
    wz = P[2] * NN - C(f32(pz))
    one = C(f32(1.0))
    ox, oy, oz = one - wx, one - wy, one - wz
    corners = [
        (ox, oy, oz, 0, 0, 0), (wx, oy, oz, 0, 0, 1), (ox, wy, oz, 0, 1, 0), (wx, wy, oz, 0, 1, 1),
        (ox, oy, wz, 1, 0, 0), (wx, oy, wz, 1, 0, 1), (ox, wy, wz, 1, 1, 0), (wx, wy, wz, 1, 1, 1)]
    res = None
    for fx, fy, fz, dz, dy, dx in corners:
        w = fx * fy * fz * C(grid_at(g, N, pz + dz, py + dy, px + dx))
        res = w if res is None else res + w
    if av(res) > f32(0.2):
        return C(f32(0.0))
    return res


def point_tri_d2_ericson(p, a, b, c):
    """Closest point on a triangle by Voronoi regions (Ericson, Real-Time
    Collision Detection 5.1.5), FP64; degenerate triangles fall back to their
    segments."""
    def seg(p, a, b):
        ab = b - a
        l2 = ab @ ab
        t = 0.0 if l2 == 0 else min(1.0, max(0.0, (p - a) @ ab / l2))
        q = a + t * ab
        return (p - q) @ (p - q)
    n = np.cross(b - a, c - a)
    if n @ n == 0.0:
        return min(seg(p, a, b), seg(p, b, c), seg(p, c, a))
    ab, ac, ap = b - a, c - a, p - a
    d1, d2 = ab @ ap, ac @ ap
    if d1 <= 0 and d2 <= 0:
        q = a
    else:
        bp = p - b
        d3, d4 = ab @ bp, ac @ bp
        if d3 >= 0 and d4 <= d3:
            q = b
        else:
            vc = d1 * d4 - d3 * d2
            if vc <= 0 and d1 >= 0 and d3 <= 0:
                q = a + d1 / (d1 - d3) * ab
            else:
                cp = p - c
                d5, d6 = ab @ cp, ac @ cp
                if d6 >= 0 and d5 <= d6:
                    q = c
                else:
                    vb = d5 * d2 - d1 * d6
                    if vb <= 0 and d2 >= 0 and d6 <= 0:
                        q = a + d2 / (d2 - d6) * ac
                    else:
                        va = d3 * d6 - d5 * d4
                        if va <= 0 and (d4 - d3) >= 0 and (d5 - d6) >= 0:
                            q = b + (d4 - d3) / ((d4 - d3) + (d5 - d6)) * (c - b)
                        else:
                            den = 1.0 / (va + vb + vc)
                            q = a + ab * (vb * den) + ac * (vc * den)
    return float((p - q) @ (p - q))


def icosphere1():
    t = (1.0 + 5 ** 0.5) / 2.0
    V = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], np.float64)
    V /= np.linalg.norm(V, axis=1, keepdims=True)
    F = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4], [11, 10, 2],
                  [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5],
                  [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], np.int64)
    return V, F


def main():
    rng = np.random.Generator(np.random.PCG64(2024))
    V, F = icosphere1()
    # target: anisotropic, shifted, plus one degenerate face (repeated vertex)
    T = (V * np.array([1.3, 0.8, 0.6]) + np.array([0.2, -0.1, 0.4])).astype(np.float32)
    TF = np.concatenate([F, [[0, 0, 5]]]).astype(np.int32)
    # Mesh::Normalize in double over float input
    Td = T.astype(np.float64)
    mn, mx = Td.min(0), Td.max(0)
    ext = mx - mn
    scale = max(ext[0], max(ext[1], ext[2])) * 1.1
    trans = mn - 0.05 * scale
    Tn = (Td - trans) / scale
    N = 8
    grid64 = np.empty(N ** 3)
    for idx in range(N ** 3):
        k, j, i = idx % N, (idx // N) % N, idx // (N * N)
        p = np.array([k / N, j / N, i / N])
        grid64[idx] = np.sqrt(min(point_tri_d2_ericson(p, Tn[f[0]], Tn[f[1]], Tn[f[2]]) for f in TF))
    grid = grid64.astype(np.float32)
    # probe points: both branches, the N-1 slab, truncation toward zero, far
    P = list(rng.uniform(-0.2, 1.2, size=(48, 3)))
    P += [[(N - 1) / N, 0.5, 0.5], [-0.3 / N, 0.4, 0.6], [0.5, 1.4, -0.1], [0.0, 0.0, 0.0], [0.999, 0.3, 0.2],
          [3.0e9, 0.5, 0.5]]
    P = np.asarray(P, np.float32)
    d = np.asarray([distance(grid, N, p, False) for p in P], np.float32)
    jets = [distance(grid, N, p, True) for p in P]
    jet = np.asarray([[j.a] + j.v for j in jets], np.float32)
    loss_fwd = d * d
    loss_bwd = np.asarray([[f32(f32(j.a * v + v * j.a) * f32(0.5)) for v in j.v] for j in jets], np.float32)
    # source mesh normalised by the target (normalize.cc:13-23)
    S = (V * 0.9 + rng.normal(scale=0.05, size=V.shape)).astype(np.float32)
    Sn = ((S.astype(np.float64) - trans) / scale).astype(np.float32)
    SF = F.astype(np.int32)
    off = np.zeros((3 * len(SF), 3), np.float32)
    for f in range(len(SF)):
        for j in range(3):
            v0, v1 = SF[f, j], SF[f, (j + 1) % 3]
            for c in range(3):
                off[3 * f + j, c] = f32(Sn[v1, c] - Sn[v0, c])
    S1 = (Sn + rng.normal(scale=0.01, size=Sn.shape)).astype(np.float32)
    efwd = np.zeros((3 * len(SF), 3), np.float32)
    ebwd = np.zeros((len(S1), 3), np.float32)
    for f in range(len(SF)):
        for j in range(3):
            v0, v1 = SF[f, j], SF[f, (j + 1) % 3]
            for c in range(3):
                r = f32(f32(S1[v1, c] - S1[v0, c]) - off[3 * f + j, c])
                efwd[3 * f + j, c] = f32(r * r)
                ebwd[v0, c] = f32(ebwd[v0, c] - r)
                ebwd[v1, c] = f32(ebwd[v1, c] + r)
    np.savez_compressed(os.path.join(HERE, "meshode_golden.npz"),
                        target_V=T, target_F=TF, N=np.int64(N), scale=np.float64(scale), trans=trans,
                        grid64=grid64, grid=grid, probes=P, distance=d, jet=jet, dfloss_fwd=loss_fwd,
                        dfloss_bwd=loss_bwd, source_V=S, source_Vn=Sn, source_F=SF, edge_offsets=off,
                        source_V1=S1, edge_fwd=efwd, edge_bwd=ebwd)
    print("wrote", os.path.join(HERE, "meshode_golden.npz"))


if __name__ == "__main__":
    sys.exit(main())
