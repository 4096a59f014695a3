"""Iso-surface of a distance grid (the role of Mesh::FromDistanceField,
src/lib/mesh.cc:154-179).

The reference samples the grid at integer points (x, y, z) = (k, j, i),
extracts the level set with marching cubes and divides the vertices by N,
so the mesh lives in the target-normalised unit cube.  It always uses level
0, which for an unsigned distance field is empty: a point is inside when its
value is below the level, and no distance is below 0.  This restatement
takes the level as an argument (0 by default, as the reference), splits
every cell into six tetrahedra around its main diagonal and triangulates
each tetrahedron by its sign pattern (marching tetrahedra); a vertex sits on
a grid edge at the linear zero crossing and is shared by every triangle
that uses that edge, so the surface is watertight wherever it does not meet
the grid boundary, and triangles face toward increasing values.  The
triangulation differs from libigl's marching-cubes tables, as any two
marching schemes do; both interpolate the same crossings on the grid edges
they share.  CPU, numpy; the grid is the `[z][y][x]` float32 array of
`pyDeform.GetDistanceField` (any N).
"""
import numpy as np

# cell corner c = (bx, by, bz) -> index bx + 2 by + 4 bz
_CORNER = np.array([[c & 1, (c >> 1) & 1, (c >> 2) & 1] for c in range(8)], dtype=np.int64)
# six tetrahedra sharing the diagonal 0-7, each a monotone corner path 0 -> 7
_TETS = np.array([[0, 1, 3, 7], [0, 1, 5, 7], [0, 2, 3, 7], [0, 2, 6, 7], [0, 4, 5, 7], [0, 4, 6, 7]],
                 dtype=np.int64)


def from_distance_field(grid, level=0.0):
    """Vertices float64 [m, 3] (unit cube) and faces int64 [f, 3] of the
    level set {value = level} of `grid` (N^3 values, [z][y][x]); empty for an
    unsigned field at level 0, as the reference's call."""
    g = np.asarray(grid, dtype=np.float64)
    N = int(round(g.size ** (1.0 / 3.0)))
    if N < 2 or N ** 3 != g.size:
        raise ValueError("grid must hold N^3 values with N >= 2")
    g = g.reshape(N, N, N)  # [z][y][x]
    level = float(level)
    inside = g < level
    M = N - 1
    # cells with both signs among their corners
    any_in = np.zeros((M, M, M), dtype=bool)
    all_in = np.ones((M, M, M), dtype=bool)
    for bx, by, bz in _CORNER:
        s = inside[bz:bz + M, by:by + M, bx:bx + M]
        any_in |= s
        all_in &= s
    zz, yy, xx = np.nonzero(any_in & ~all_in)
    if len(xx) == 0:
        return np.zeros((0, 3)), np.zeros((0, 3), dtype=np.int64)
    base = np.stack([xx, yy, zz], 1)  # (x, y, z) of corner 0
    corners = base[:, None, :] + _CORNER[None, :, :]  # [cells, 8, 3]
    # tetrahedra [t, 4, 3] of the mixed cells
    tets = corners[:, _TETS, :].reshape(-1, 4, 3)
    val = g[tets[..., 2], tets[..., 1], tets[..., 0]]
    tin = val < level
    cnt = tin.sum(1)
    keep = (cnt > 0) & (cnt < 4)
    tets, val, tin, cnt = tets[keep], val[keep], tin[keep], cnt[keep]
    lin = (tets[..., 2] * N + tets[..., 1]) * N + tets[..., 0]  # grid point ids [t, 4]

    edge_key, edge_pts = [], []
    tris = []

    def edge(a, b, rows):
        """Crossing on edge (a, b) of tets `rows`: global key, point."""
        ia, ib = lin[rows, a], lin[rows, b]
        va, vb = val[rows, a], val[rows, b]
        t = (level - va) / (vb - va)
        p = tets[rows, a] + t[:, None] * (tets[rows, b] - tets[rows, a])
        key = np.minimum(ia, ib) * (N ** 3) + np.maximum(ia, ib)
        return key, p

    def add(keys_pts, rows):
        """One triangle per row from three (key, point) crossings."""
        ks = np.stack([k for k, _ in keys_pts], 1)
        ps = np.stack([p for _, p in keys_pts], 1)
        edge_key.append(ks.ravel())
        edge_pts.append(ps.reshape(-1, 3))
        tris.append((rows, ps))

    # one corner on its own side (1 inside or 3 inside): one triangle
    for lone_inside in (True, False):
        rows = np.nonzero(cnt == (1 if lone_inside else 3))[0]
        if len(rows) == 0:
            continue
        side = tin[rows] if lone_inside else ~tin[rows]
        lone = np.argmax(side, 1)
        others = np.array([[j for j in range(4) if j != c] for c in range(4)])[lone]
        add([edge_col(lone, others[:, k], rows, edge) for k in range(3)], rows)
    # two and two: a quad, two triangles
    rows = np.nonzero(cnt == 2)[0]
    if len(rows):
        order = np.argsort(~tin[rows], axis=1, kind="stable")  # inside corners first
        a0, a1, b0, b1 = order[:, 0], order[:, 1], order[:, 2], order[:, 3]
        e00 = edge_col(a0, b0, rows, edge)
        e01 = edge_col(a0, b1, rows, edge)
        e11 = edge_col(a1, b1, rows, edge)
        e10 = edge_col(a1, b0, rows, edge)
        add([e00, e01, e11], rows)
        add([e00, e11, e10], rows)

    keys = np.concatenate(edge_key)
    pts = np.concatenate(edge_pts)
    uniq, first, inv = np.unique(keys, return_index=True, return_inverse=True)
    V = pts[first] / N
    F = inv.reshape(-1, 3).astype(np.int64)
    # orient every triangle toward increasing values (outward from `inside`)
    rows_all = np.concatenate([r for r, _ in tris])
    tin_all = tin[rows_all]
    tet_all = tets[rows_all].astype(np.float64)
    cin_mean = (tet_all * tin_all[..., None]).sum(1) / tin_all.sum(1, keepdims=True)
    cout_mean = (tet_all * ~tin_all[..., None]).sum(1) / (~tin_all).sum(1, keepdims=True)
    up = cout_mean - cin_mean
    P = V[F] * N
    nrm = np.cross(P[:, 1] - P[:, 0], P[:, 2] - P[:, 0])
    flip = (nrm * up).sum(1) < 0
    F[flip] = F[flip][:, ::-1]
    # drop triangles collapsed by a crossing at a grid point
    good = (F[:, 0] != F[:, 1]) & (F[:, 1] != F[:, 2]) & (F[:, 0] != F[:, 2])
    return V, F[good]


def edge_col(a, b, rows, edge):
    """The crossing on the edge between per-row tet corners a[r] and b[r]."""
    out_k = np.empty(len(rows), dtype=np.int64)
    out_p = np.empty((len(rows), 3))
    for ca in range(4):
        for cb in range(4):
            sel = (a == ca) & (b == cb)
            if sel.any():
                k, p = edge(ca, cb, rows[sel])
                out_k[sel] = k
                out_p[sel] = p
    return out_k, out_p
