"""Known-answer and property tests of the CPU oracle (no GPU).

* point-triangle distance in the vertex, edge and face regions and for
  degenerate triangles;
* the trilinear lookup reproduces a linear field, and every branch of
  UniformGrid::DistanceFloat (src/lib/uniformgrid.cc:85-150): below zero,
  beyond N, the N-1 slab without a term, truncation toward zero, the 0.2
  cutoff;
* the jet derivative agrees with FP64 finite differences (h = 1e-6) of an FP64
  restatement of the same trilinear formula;
* the edge backward equals the gradient of 0.5*sum r^2 (FP64 FD);
* the Karras tree is a valid binary tree over the sorted leaves;
* the Adam step table equals torch.optim.Adam's bias corrections.
"""
import numpy as np
import pytest
import torch


def _d2(orc, p, a, b, c):
    f = lambda x: np.ascontiguousarray(x, np.float64)  # noqa: E731
    return orc.lib().orc_point_tri_dist2(orc._p(f(p)), orc._p(f(a)), orc._p(f(b)), orc._p(f(c)))


def test_point_triangle_regions(orc):
    a, b, c = np.array([0., 0, 0]), np.array([1., 0, 0]), np.array([0., 1, 0])
    assert _d2(orc, [0.2, 0.2, 0.5], a, b, c) == pytest.approx(0.25)          # face
    assert _d2(orc, [-1.0, -1.0, 0.0], a, b, c) == pytest.approx(2.0)         # vertex a
    assert _d2(orc, [2.0, 0.0, 1.0], a, b, c) == pytest.approx(2.0)           # vertex b
    assert _d2(orc, [0.5, -1.0, 0.0], a, b, c) == pytest.approx(1.0)          # edge ab
    assert _d2(orc, [1.0, 1.0, 0.0], a, b, c) == pytest.approx(0.5)           # edge bc
    assert _d2(orc, [0.3, 0.3, 0.0], a, b, c) == 0.0                          # on the face
    # degenerate: collinear and a point
    assert _d2(orc, [0.5, 1.0, 0.0], a, b, np.array([2., 0, 0])) == pytest.approx(1.0)
    assert _d2(orc, [0.0, 3.0, 4.0], a, a, a) == pytest.approx(25.0)


def test_timed_df_build_matches_untimed(orc):
    """The timed AABB-tree build (used for bounded CPU timings) returns the
    untimed build's values, on the whole grid and on a z-slab sample, with
    non-negative phase times."""
    from meshode_gb300 import meshgen
    V, F = meshgen.icosphere(2)
    Vn = 0.5 + 0.4 * np.asarray(V, np.float64)
    N = 12
    whole = orc.df_build(Vn, F, N)
    vals, t_tree, t_query = orc.df_build_timed(Vn, F, N)
    assert np.array_equal(vals, whole) and t_tree >= 0.0 and t_query >= 0.0
    zs = np.arange(1, N, 4)
    vox = (zs[:, None] * N * N + np.arange(N * N)[None, :]).ravel().astype(np.int64)
    part, _, _ = orc.df_build_timed(Vn, F, N, voxels=vox)
    assert np.array_equal(part, whole[vox])
    empty, _, _ = orc.df_build_timed(Vn, F, N, voxels=np.zeros(0, np.int64))
    assert empty.shape == (0,)


def test_trilinear_reproduces_linear_field(orc):
    N = 16
    z, y, x = np.meshgrid(np.arange(N), np.arange(N), np.arange(N), indexing="ij")
    grid = (0.01 + 0.002 * x + 0.001 * y + 0.003 * z).astype(np.float32).reshape(-1)
    rng = np.random.Generator(np.random.PCG64(0))
    for p in rng.uniform(0.0, (N - 1.5) / N, size=(200, 3)):
        p = p.astype(np.float32)
        exact = 0.01 + (0.002 * p[0] + 0.001 * p[1] + 0.003 * p[2]) * N
        assert orc.distance_float(grid, N, p) == pytest.approx(exact, abs=2e-6)
        j = orc.distance_jet(grid, N, p)
        assert j[1:] == pytest.approx(np.array([0.002, 0.001, 0.003]) * N, rel=2e-4)


def test_lookup_branches(orc):
    N = 8
    grid = np.full(N ** 3, 0.05, np.float32)
    Cf = np.float32((N - 1) - 1e-3)
    # below zero on x: penalty -x*N, derivative -N
    v = orc.distance_jet(grid, N, np.float32([-0.5, 0.5, 0.5]))
    assert v[0] == np.float32(0.5) * np.float32(N) and v[1] == -N and v[2] == 0 and v[3] == 0
    # beyond N on y and below zero on z: two terms
    p = np.float32([0.5, 1.25, -0.25])
    v = orc.distance_jet(grid, N, p)
    assert v[0] == np.float32(np.float32(p[1] * np.float32(N)) - Cf) + np.float32(-p[2] * np.float32(N))
    assert (v[2], v[3]) == (N, -N)
    # on the N-1 slab (p*N == N-1): out of range, but no term for that axis
    v = orc.distance_jet(grid, N, np.float32([(N - 1) / N, 0.5, 0.5]))
    assert v[0] == 0 and v[1] == 0
    # truncation toward zero: p in (-1/N, 0) is in range and extrapolates
    v = orc.distance_float(grid, N, np.float32([-0.5 / N, 0.5, 0.5]))
    assert v == pytest.approx(0.05, abs=1e-7)
    # the 0.2 cutoff: a grid of 0.3 returns exactly 0 with zero derivative
    big = np.full(N ** 3, 0.3, np.float32)
    v = orc.distance_jet(big, N, np.float32([0.5, 0.5, 0.5]))
    assert list(v) == [0, 0, 0, 0]
    # x86 integer-indefinite truncation for huge or NaN inputs
    assert orc.lib().orc_trunc_i32(3.0e9) == -2 ** 31
    assert orc.lib().orc_trunc_i32(float("nan")) == -2 ** 31
    assert orc.lib().orc_trunc_i32(-2.5) == -2


def _trilinear64(grid, N, p):
    s = np.asarray(p, np.float64) * N
    i = np.floor(s).astype(int)
    w = s - i
    g = grid.reshape(N, N, N).astype(np.float64)
    r = 0.0
    for dz in (0, 1):
        for dy in (0, 1):
            for dx in (0, 1):
                wt = (w[0] if dx else 1 - w[0]) * (w[1] if dy else 1 - w[1]) * (w[2] if dz else 1 - w[2])
                r += wt * g[i[2] + dz, i[1] + dy, i[0] + dx]
    return r


def test_jet_matches_fp64_finite_differences(orc):
    N = 16
    rng = np.random.Generator(np.random.PCG64(1))
    grid = rng.uniform(0.0, 0.15, size=N ** 3).astype(np.float32)
    h = 1e-6
    for p in rng.uniform(0.1, 0.85, size=(100, 3)):
        p32 = p.astype(np.float32)
        s = p32.astype(np.float64) * N
        frac = s - np.floor(s)
        if np.any(frac < 1e-3) or np.any(frac > 1 - 1e-3):
            continue  # too close to a cell face for a one-sided difference
        j = orc.distance_jet(grid, N, p32)
        if j[0] == 0:
            continue  # beyond the 0.2 cutoff
        for k in range(3):
            e = np.zeros(3)
            e[k] = h
            fd = (_trilinear64(grid, N, p32.astype(np.float64) + e) -
                  _trilinear64(grid, N, p32.astype(np.float64) - e)) / (2 * h)
            assert j[1 + k] == pytest.approx(fd, rel=1e-4, abs=1e-4)


def test_edge_backward_is_gradient(orc):
    rng = np.random.Generator(np.random.PCG64(2))
    V0 = rng.uniform(size=(30, 3)).astype(np.float32)
    F = rng.integers(0, 30, size=(40, 3)).astype(np.int32)
    off = orc.edge_offsets(V0, F, 0)
    V = (V0 + rng.normal(scale=0.05, size=V0.shape)).astype(np.float32)
    g = orc.edge_backward(V, F, 0, off)

    def loss(Vd):
        r = []
        for f in range(len(F)):
            for j in range(3):
                v0, v1 = F[f, j], F[f, (j + 1) % 3]
                r.append(Vd[v1] - Vd[v0] - off[3 * f + j].astype(np.float64))
        r = np.asarray(r)
        return 0.5 * (r * r).sum()

    Vd = V.astype(np.float64)
    for i in rng.choice(30, size=8, replace=False):
        for k in range(3):
            e = np.zeros_like(Vd)
            e[i, k] = 1e-6
            fd = (loss(Vd + e) - loss(Vd - e)) / 2e-6
            assert g[i, k] == pytest.approx(fd, abs=1e-4)


def test_karras_tree_is_valid(orc):
    rng = np.random.Generator(np.random.PCG64(3))
    for n in (2, 3, 17, 1000):
        codes = np.sort(rng.integers(0, 2 ** 30, size=n).astype(np.uint32))
        codes[n // 3: n // 3 + 5] = codes[n // 3]  # duplicates
        codes = np.sort(codes)
        left, right = orc.karras(codes)
        seen_leaf = np.zeros(n, int)
        seen_int = np.zeros(n - 1, int)
        stack = [0]
        while stack:
            x = stack.pop()
            seen_int[x] += 1
            for c in (left[x], right[x]):
                if c < 0:
                    seen_leaf[~c] += 1
                else:
                    stack.append(c)
        assert (seen_leaf == 1).all() and (seen_int == 1).all()


def test_adam_table_matches_torch():
    from meshode_gb300 import fused
    tab = fused.adam_table(50, 1e-3, 0.9, 0.999, "cpu").numpy()
    p = torch.nn.Parameter(torch.zeros(1))
    opt = torch.optim.Adam([p], lr=1e-3)
    for t in range(1, 51):
        p.grad = torch.ones(1)
        opt.step()
        st = opt.state[p]["step"].item()
        bc1 = 1 - 0.9 ** st
        bc2 = 1 - 0.999 ** st
        assert tab[t - 1, 0] == np.float32(1e-3 / bc1)
        assert tab[t - 1, 1] == np.float32(bc2 ** 0.5)


def _f32_round(x):
    """Correctly rounded float32 of an exact rational (ties to even)."""
    from fractions import Fraction
    f = np.float32(float(x))
    best = None
    for c in (np.nextafter(f, np.float32(-np.inf)), f, np.nextafter(f, np.float32(np.inf))):
        d = abs(Fraction(float(c)) - x)
        if best is None or d < best[0] or (d == best[0] and int(np.float32(c).view(np.uint32)) % 2 == 0):
            best = (d, c)
    return np.float32(best[1])


def test_exact_adam_definition_and_torch(orc):
    """orc_adam_step is torch's _single_tensor_adam op sequence with one
    rounding per op (checked against exact rational arithmetic), and stays
    within a few ulps of torch.optim.Adam on the CPU over many steps."""
    import torch
    from fractions import Fraction as Fr
    rng = np.random.Generator(np.random.PCG64(12))
    n = 37
    V0 = rng.standard_normal(n).astype(np.float32)
    grads = [rng.standard_normal(n).astype(np.float32) * np.float32(10.0 ** rng.integers(-3, 2))
             for _ in range(60)]
    Vt = torch.nn.Parameter(torch.from_numpy(V0.copy()))
    opt = torch.optim.Adam([Vt], lr=1e-3)
    Ve = torch.nn.Parameter(torch.from_numpy(V0.copy()))
    ex = orc.ExactAdam(Ve, lr=1e-3)
    # first step against the definition, element by element
    p, m, v = V0.copy(), np.zeros(n, np.float32), np.zeros(n, np.float32)
    g = grads[0]
    step_size = np.float32(1e-3 / (1 - 0.9 ** 1.0))
    bc2s = np.float32((1 - 0.999 ** 1.0) ** 0.5)
    omb1, b2, omb2, eps = np.float32(1 - 0.9), np.float32(0.999), np.float32(1 - 0.999), np.float32(1e-8)
    for i in range(n):
        m[i] = _f32_round(Fr(float(omb1)) * Fr(float(np.float32(g[i] - m[i]))) + Fr(float(m[i])))
        v[i] = np.float32(v[i] * b2) + np.float32(np.float32(omb2 * g[i]) * g[i])
        denom = np.float32(np.float32(np.sqrt(v[i])) / bc2s) + eps
        q = np.float32(m[i] / denom)
        p[i] = _f32_round(Fr(-float(step_size)) * Fr(float(q)) + Fr(float(p[i])))
    ex.step(torch.from_numpy(g))
    assert np.array_equal(Ve.detach().numpy(), p)
    for g in grads[1:]:
        ex.step(torch.from_numpy(g))
    for g in grads:
        opt.zero_grad()
        Vt.grad = torch.from_numpy(g.copy())
        opt.step()
    diff = np.abs(Ve.detach().numpy() - Vt.detach().numpy()).max()
    assert diff <= 1e-6, diff


def test_reverse_loss_known_answer(orc):
    """Two source points, two targets: each target's nearest source point and
    the loss 0.5*sum of squared offsets, with its autograd gradient."""
    src = torch.tensor([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0]], requires_grad=True)
    tar = torch.tensor([[0.875, 0.0, 0.0], [0.25, 0.0, 0.0], [0.75, 0.5, 0.0]])
    loss, ii = orc.reverse_loss(src, tar)
    assert list(ii) == [1, 0, 1]
    assert float(loss) == pytest.approx(0.5 * (0.125 ** 2 + 0.25 ** 2 + 0.25 ** 2 + 0.5 ** 2))
    loss.backward()
    assert torch.equal(src.grad, torch.tensor([[-0.25, 0.0, 0.0], [0.125 + 0.25, -0.5, 0.0]]))


def test_solve_linear_known_answer(orc):
    """Two vertices, one face-less edge, each its own graph node: the system
    ((w^2 + 1e-6) I + reg L) x = (w + 1e-6) G + reg L V has the closed form
    below (w = 1)."""
    V = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0]], np.float32)
    G = np.array([[0.0, 0.5, 0.0], [2.0, 0.5, 0.0]], np.float32)
    F = np.zeros((0, 3), np.int32)
    E = np.array([[0, 1]], np.int32)
    ref = np.array([0, 1], np.int32)
    X = orc.solve_linear(V, F, E, ref, G, 1.0, with_rot=0).astype(np.float64)
    reg = (0.02 / (1.0 + 1e-8)) ** 2
    a = 1.0 + 1e-6
    # symmetric system per coordinate: [[a+reg, -reg], [-reg, a+reg]] x = b
    for c in range(3):
        b0 = a * G[0, c] + reg * (V[0, c] - V[1, c])
        b1 = a * G[1, c] + reg * (V[1, c] - V[0, c])
        det = (a + reg) ** 2 - reg ** 2
        x0 = ((a + reg) * b0 + reg * b1) / det
        x1 = (reg * b0 + (a + reg) * b1) / det
        assert X[0, c] == pytest.approx(x0, abs=1e-7) and X[1, c] == pytest.approx(x1, abs=1e-7)
