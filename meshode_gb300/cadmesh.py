"""LoadCadMesh (src/interface/mesh_tensor.cc:102-178): CAD remeshing and the
representative graph, restated on the CPU with numpy and SciPy's Qhull.

The reference reads the OBJ, drops degenerate faces (Mesh::RemoveDegenerated),
merges duplicate vertices (Mesh::MergeDuplex), then (src/lib/subdivision.cc):

* Subdivide (:28-129) at 0.02: faces grouped by edge-connected component;
  every edge split into int(|e|/0.02 + 1) equal segments; every face
  re-triangulated (DelaunaySubdivision, :131-250) from its edge points --
  pushed onto a radius-1e3 arc so the boundary stays convex -- and the
  points of the face-plane lattice of spacing 0.02 strictly inside it, by a
  2D Delaunay triangulation (CGAL in the reference), keeping triangles whose
  edges are at most 3 * 0.02;
* ComputeGeometryNeighbors (:252-341) at 0.015: every vertex hashed into the
  eight cells int((v + d)/0.015) (d in {0, 0.015}^3); each cell's vertices
  joined by the edges of their 3D Delaunay triangulation (two vertices: one
  edge), plus the mesh edges;
* ComputeRepresentativeGraph (:343-399) at 0.01: vertices clustered by
  int(v/0.01); graph vertices the cluster means in key order; graph edges
  the neighbour pairs and mesh edges between different clusters.

CGAL is not available, so the triangulations are Qhull's (scipy.spatial
.Delaunay); lattice points are co-circular, where both libraries pick one of
several valid triangulations, and CGAL's lower-dimensional triangulations
(coplanar or collinear cells) are reproduced by triangulating in the
points' plane or chaining them along their line.  The vertex, face and edge
sets therefore match the reference's construction, but individual diagonals
may differ: parity unpinned, compared through the Chamfer distance of the
final deformation.  Degenerate-key collisions of the reference's 1e-7
point lookup (near-duplicate points) are not reproduced.
"""
import numpy as np

from . import meshops, objio

SUBDIV_LEN = 2e-2
NEIGHBOR_STEP = 1.5e-2
GRAPH_STEP = 1e-2
_POINT_NINE = float(np.float32(0.999999))  # the reference's 0.999999f


def _trunc_key(P, step):
    """int(v / step) per component (C++ truncation toward zero)."""
    return np.trunc(P / step).astype(np.int64)


def _face_components(F):
    """Connected components of faces sharing an edge, labelled in order of
    their lowest face index (subdivision.cc:37-82)."""
    from scipy.sparse import coo_matrix
    from scipy.sparse.csgraph import connected_components
    m = len(F)
    if m == 0:
        return np.zeros(0, np.int64)
    a = F[:, [0, 1, 2]].reshape(-1)
    b = F[:, [1, 2, 0]].reshape(-1)
    key = np.minimum(a, b).astype(np.int64) * (int(F.max()) + 1) + np.maximum(a, b)
    face = np.repeat(np.arange(m), 3)
    order = np.argsort(key, kind="stable")
    ks, fs = key[order], face[order]
    same = ks[1:] == ks[:-1]
    rows, cols = fs[:-1][same], fs[1:][same]
    G = coo_matrix((np.ones(len(rows)), (rows, cols)), shape=(m, m))
    _, labels = connected_components(G, directed=False)
    # relabel by first appearance so labels follow the lowest face index
    first = {}
    out = np.empty(m, np.int64)
    for i, l in enumerate(labels):
        out[i] = first.setdefault(l, len(first))
    return out


def _delaunay2d(P):
    """Triangles (counter-clockwise) of the 2D Delaunay triangulation."""
    from scipy.spatial import Delaunay
    if len(P) < 3:
        return np.zeros((0, 3), np.int64)
    try:
        return Delaunay(P).simplices.astype(np.int64)
    except Exception:  # all points collinear: no triangle
        return np.zeros((0, 3), np.int64)


def _chain(P):
    """Edges between consecutive points along their common line."""
    d = P - P.mean(0)
    u = np.linalg.svd(d, full_matrices=False)[2][0]
    o = np.argsort(d @ u, kind="stable")
    return np.stack([o[:-1], o[1:]], 1)


def delaunay3d_edges(P):
    """Finite edges of the 3D Delaunay triangulation of P, falling back to the
    2D triangulation in the points' plane or the chain along their line when
    they are coplanar or collinear (what a 3D Delaunay library builds then)."""
    from scipy.spatial import Delaunay
    n = len(P)
    if n < 2:
        return np.zeros((0, 2), np.int64)
    if n == 2:
        return np.array([[0, 1]], np.int64)
    d = P - P.mean(0)
    s = np.linalg.svd(d, compute_uv=False)
    scale = max(s[0], 1e-300)
    rank = int((s > 1e-9 * scale).sum())
    if rank == 0:
        return np.zeros((0, 2), np.int64)
    if rank == 1:
        return _chain(P)
    if rank == 3 and n >= 4:
        try:
            T = Delaunay(P).simplices.astype(np.int64)
            e = np.concatenate([T[:, [i, j]] for i in range(4) for j in range(i + 1, 4)])
            e.sort(1)
            return np.unique(e, axis=0)
        except Exception:
            pass
    _, _, vt = np.linalg.svd(d, full_matrices=False)
    Q = d @ vt[:2].T
    T = _delaunay2d(Q)
    if len(T) == 0:
        return _chain(P)
    e = np.concatenate([T[:, [0, 1]], T[:, [1, 2]], T[:, [2, 0]]])
    e.sort(1)
    return np.unique(e, axis=0)


def _edges3(V, M):
    """Delaunay edges of 3-point cells: the triangle, or the chain when
    collinear."""
    A, B, C = V[M[:, 0]], V[M[:, 1]], V[M[:, 2]]
    cr = np.linalg.norm(np.cross(B - A, C - A), axis=1)
    sc = np.maximum(np.maximum(np.linalg.norm(B - A, axis=1), np.linalg.norm(C - A, axis=1)), 1e-300)
    tri = cr > 1e-9 * sc * sc
    out = [np.concatenate([M[tri][:, [0, 1]], M[tri][:, [1, 2]], M[tri][:, [0, 2]]])]
    for ids in M[~tri]:
        P = V[ids]
        if np.ptp(P, axis=0).max() > 0:
            out.append(ids[_chain(P)])
    return np.concatenate(out) if out else np.zeros((0, 2), np.int64)


def _edges4(V, M):
    """Delaunay edges of 4-point cells: the tetrahedron's six; when coplanar,
    the edges of the planar Delaunay triangulation of the points projected
    on their plane; when collinear, the chain."""
    P = V[M]                                   # [c,4,3]
    D = P[:, 1:] - P[:, :1]
    vol = np.abs(np.einsum("ci,ci->c", D[:, 0], np.cross(D[:, 1], D[:, 2])))
    sc = np.maximum(np.linalg.norm(D, axis=2).max(1), 1e-300)
    tet = vol > 1e-9 * sc ** 3
    all6 = [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)]
    out = [np.concatenate([M[tet][:, list(e)] for e in all6])] if tet.any() else []
    for ids, Q in zip(M[~tet], P[~tet]):
        d = Q - Q.mean(0)
        u, sv, vt = np.linalg.svd(d, full_matrices=False)
        if sv[1] <= 1e-9 * max(sv[0], 1e-300):
            if sv[0] > 0:
                out.append(ids[_chain(Q)])
            continue
        X = d @ vt[:2].T                           # 2D coordinates
        T = _delaunay2d(X)
        if len(T) == 0:
            continue
        e = np.concatenate([T[:, [0, 1]], T[:, [1, 2]], T[:, [2, 0]]])
        e.sort(1)
        out.append(ids[np.unique(e, axis=0)])
    return np.concatenate(out) if out else np.zeros((0, 2), np.int64)


def _barycentric_inside(ax, ay, bx, by, cx, cy, px, py):
    """subdivision.cc:442-460: strictly inside by barycentric coordinates."""
    def area2(ax_, ay_, bx_, by_, cx_, cy_):
        return (cx_ - ax_) * (by_ - ay_) - (bx_ - ax_) * (cy_ - ay_)
    beta_tri = area2(ax, ay, px, py, cx, cy)
    gamma_tri = area2(ax, ay, bx, by, px, py)
    tri_inv = 1.0 / area2(ax, ay, bx, by, cx, cy)
    beta = beta_tri * tri_inv
    gamma = gamma_tri * tri_inv
    alpha = 1.0 - beta - gamma
    return (alpha > 0) & (alpha < 1) & (beta > 0) & (beta < 1) & (gamma > 0) & (gamma < 1)


def _delaunay_subdivision(bidx, V, newF, face, len_thres):
    """subdivision.cc:131-250 for one face; appends lattice points to V (a
    list) and triangles to newF."""
    v0, v1, v2 = (np.asarray(V[face[k]], np.float64) for k in range(3))
    n = np.cross(v1 - v0, v2 - v0)
    n = n / np.linalg.norm(n)
    merged = {}  # insertion-ordered set of the boundary points
    for i in range(3):
        x = np.asarray(V[face[i]], np.float64)
        y = np.asarray(V[face[(i + 1) % 3]], np.float64)
        dr = np.cross(n, y - x)
        dr = dr / np.linalg.norm(dr)
        c = (y + x) * 0.5 + 1e3 * dr
        rad = np.linalg.norm(c - x)
        for p in bidx[i]:
            diff = np.asarray(V[p], np.float64) - c
            merged[p] = diff / np.linalg.norm(diff) * rad + c
    vind = list(merged.keys())
    pts = [merged[p] for p in vind]
    # the reference's axis choice (it only ever picks axis 0 or 1)
    min_axis = 0
    for i in (1, 2):
        if abs(n[i]) < abs(n[min_axis]):
            min_axis = 1
    tx = np.zeros(3)
    tx[min_axis] = 1.0
    tx = np.cross(tx, n)
    tx = tx / np.linalg.norm(tx)
    ty = np.cross(n, tx)
    v1x, v1y = (v1 - v0) @ tx / len_thres, (v1 - v0) @ ty / len_thres
    v2x, v2y = (v2 - v0) @ tx / len_thres, (v2 - v0) @ ty / len_thres
    minX, minY = int(min(0.0, v1x, v2x)), int(min(0.0, v1y, v2y))
    maxX, maxY = int(max(0.0, v1x, v2x) + _POINT_NINE), int(max(0.0, v1y, v2y) + _POINT_NINE)
    if maxX >= minX and maxY >= minY:
        py, px = np.meshgrid(np.arange(minY, maxY + 1, dtype=np.float64),
                             np.arange(minX, maxX + 1, dtype=np.float64), indexing="ij")
        px, py = px.reshape(-1), py.reshape(-1)
        inside = _barycentric_inside(0.0, 0.0, v1x, v1y, v2x, v2y, px, py)
        for qx, qy in zip(px[inside], py[inside]):
            p = v0 + tx * (qx * len_thres) + ty * (qy * len_thres)
            vind.append(len(V))
            V.append(p)
            pts.append(p)
    P = np.asarray(pts)
    Q = np.stack([(P - v0) @ tx, (P - v0) @ ty], 1)
    T = _delaunay2d(Q)
    if len(T) == 0:
        return
    vind = np.asarray(vind, np.int64)
    G = vind[T]
    X = np.stack([np.asarray(V[k], np.float64) for k in G.reshape(-1)]).reshape(-1, 3, 3)
    L = np.stack([np.linalg.norm(X[:, 0] - X[:, 1], axis=1), np.linalg.norm(X[:, 1] - X[:, 2], axis=1),
                  np.linalg.norm(X[:, 0] - X[:, 2], axis=1)], 1)
    keep = ~(L > 3 * len_thres).any(1)
    newF.extend(G[keep].tolist())


def subdivide(V, F, len_thres=SUBDIV_LEN):
    """Subdivision::Subdivide (subdivision.cc:28-129): returns (V, F) of the
    remeshed model, float64 / int64."""
    V = [np.asarray(v, np.float64) for v in np.asarray(V, np.float64)]
    F = np.asarray(F, np.int64).reshape(-1, 3)
    labels = _face_components(F)
    order = np.lexsort((np.arange(len(F)), labels))
    split = {}
    newF = []
    for fi in order:
        face = F[fi]
        bidx = []
        for j in range(3):
            a, b = int(face[j]), int(face[(j + 1) % 3])
            key = (min(a, b), max(a, b))
            if key not in split:
                diff = V[b] - V[a]
                num = int(np.linalg.norm(diff) / len_thres + 1)
                diff = diff / float(num)
                ids = [a]
                for k in range(1, num):
                    ids.append(len(V))
                    V.append(V[a] + diff * k)
                ids.append(b)
                split[key] = ids
            bidx.append(split[key])
        _delaunay_subdivision(bidx, V, newF, face, len_thres)
    return np.asarray(V, np.float64).reshape(-1, 3), np.asarray(newF, np.int64).reshape(-1, 3)


def _face_edges(F):
    e = np.stack([F[:, [0, 1, 2]].reshape(-1), F[:, [1, 2, 0]].reshape(-1)], 1)
    e.sort(1)
    return e[e[:, 0] != e[:, 1]]


def geometry_neighbors(V, F, thres=NEIGHBOR_STEP):
    """Subdivision::ComputeGeometryNeighbors (subdivision.cc:252-341): sorted
    unique vertex pairs (i < j), int64 [k,2]."""
    V = np.asarray(V, np.float64)
    n = len(V)
    offs = np.array([[0, 0, 0], [0, 0, 1], [0, 1, 0], [0, 1, 1], [1, 0, 0], [1, 0, 1], [1, 1, 0], [1, 1, 1]],
                    np.float64) * thres
    K = _trunc_key(V[:, None, :] + offs[None], thres).reshape(-1, 3)
    vid = np.repeat(np.arange(n), 8)
    # unique (cell, vertex) incidences grouped by cell
    _, cell = np.unique(K, axis=0, return_inverse=True)
    cell = cell.reshape(-1)
    inc = np.unique(np.stack([cell, vid], 1), axis=0)
    starts = np.flatnonzero(np.r_[True, inc[1:, 0] != inc[:-1, 0]])
    ends = np.r_[starts[1:], len(inc)]
    sizes = ends - starts
    two = inc[starts[sizes == 2]][:, 1], inc[starts[sizes == 2] + 1][:, 1]
    pairs = [np.stack(two, 1)]
    for k in np.unique(sizes[sizes >= 3]):
        sel = starts[sizes == k]
        M = inc[sel[:, None] + np.arange(k)[None, :], 1]
        M = np.unique(M, axis=0)  # overlapping windows repeat member sets
        if k == 3:
            pairs.append(_edges3(V, M))
        elif k == 4:
            pairs.append(_edges4(V, M))
        else:
            for ids in M:
                E = delaunay3d_edges(V[ids])
                if len(E):
                    pairs.append(ids[E])
    pairs.append(_face_edges(np.asarray(F, np.int64)))
    P = np.concatenate(pairs).astype(np.int64)
    P.sort(1)
    P = P[P[:, 0] != P[:, 1]]
    return np.unique(P, axis=0)


def representative_graph(V, F, pairs, thres=GRAPH_STEP):
    """Subdivision::ComputeRepresentativeGraph (subdivision.cc:343-399):
    (references [n], graph vertices [g,3] float64, graph edges [q,2])."""
    V = np.asarray(V, np.float64)
    K = _trunc_key(V, thres)
    _, ref = np.unique(K, axis=0, return_inverse=True)  # keys in std::map (lexicographic) order
    ref = ref.reshape(-1)
    g = int(ref.max()) + 1 if len(ref) else 0
    GV = np.zeros((g, 3))
    np.add.at(GV, ref, V)
    GV /= np.bincount(ref, minlength=g)[:, None]
    E = np.concatenate([ref[np.asarray(pairs, np.int64)].reshape(-1, 2),
                        ref[_face_edges(np.asarray(F, np.int64))].reshape(-1, 2)])
    E.sort(1)
    E = E[E[:, 0] != E[:, 1]]
    return ref, GV, np.unique(E, axis=0)


def load_cad_mesh_arrays(V, F):
    """The LoadCadMesh pipeline on arrays: (V, F, E, src_to_graph [n,1],
    graph V, graph E) as numpy arrays (float32 / int32)."""
    V, F = meshops.remove_degenerated(np.asarray(V, np.float64), np.asarray(F, np.int64))
    V, F = meshops.merge_duplex(V, F)
    Vs, Fs = subdivide(V, F, SUBDIV_LEN)
    E = geometry_neighbors(Vs, Fs, NEIGHBOR_STEP)
    ref, GV, GE = representative_graph(Vs, Fs, E, GRAPH_STEP)
    return (Vs.astype(np.float32), Fs.astype(np.int32), E.astype(np.int32), ref.astype(np.int32).reshape(-1, 1),
            GV.astype(np.float32), GE.astype(np.int32))


def load_cad_mesh(filename):
    V, F = objio.read_obj(filename)
    return load_cad_mesh_arrays(V, F)
