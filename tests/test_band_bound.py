"""The bound behind the distance-field band of the two lowest layers (CPU).

A lookup with a coordinate in (-1/N, 0) extrapolates from cell 0 of that
axis (UniformGrid::DistanceFloat, uniformgrid.cc:85-150: the cell index
truncates toward zero and the weight is the coordinate times N).  With corner
values 1/N apart differing by at most h = 1/N (distances and their clamps are
1-Lipschitz), the extrapolated trilinear value is at least the smallest
corner minus 13h: each extrapolated axis lowers the value by at most the
spread of its two inputs and at most triples the spread along the next axis
(h, then 3h, then 9h).  This is why the low layers can store
min(d, band + 13/N) without changing any loss.  Checked here in float32 with
the jet's product order, on random corner sets and on the extreme ones.
"""
import itertools

import numpy as np


def _trilinear(c, wx, wy, wz):
    """DistanceFloat's value: sum over corners k = (bz<<2)|(by<<1)|bx of
    ((fx*fy)*fz)*c[k], accumulated in k order, all in float32."""
    f32 = np.float32
    ox, oy, oz = f32(1) - wx, f32(1) - wy, f32(1) - wz
    ra = None
    for k in range(8):
        bx, by, bz = k & 1, (k >> 1) & 1, (k >> 2) & 1
        fx = wx if bx else ox
        fy = wy if by else oy
        fz = wz if bz else oz
        w = f32(f32(f32(fx * fy) * fz) * c[..., k])
        ra = w if ra is None else f32(ra + w)
    return ra


def _lipschitz_corners(rng, n, h):
    """n corner sets (8 values, k = (z<<2)|(y<<1)|x) whose values at adjacent
    corners differ by at most h: values d(p) = |p - q| for a random point q,
    which is 1-Lipschitz, scaled to corners h apart."""
    q = rng.uniform(-4, 4, size=(n, 3))
    base = rng.uniform(0.0, 2.0, size=(n, 1))
    c = np.empty((n, 8))
    for k in range(8):
        p = np.array([k & 1, (k >> 1) & 1, (k >> 2) & 1], dtype=np.float64)
        c[:, k] = np.linalg.norm(p[None, :] - q, axis=1)
    return (base + c * h).astype(np.float32)


def test_extrapolation_stays_above_min_minus_13h():
    rng = np.random.Generator(np.random.PCG64(11))
    for N in (16, 64, 128, 256):
        h = 1.0 / N
        n = 20000
        c = _lipschitz_corners(rng, n, h)
        lo = c.min(axis=1)
        for axes in ((0,), (1,), (2,), (0, 1), (0, 2), (1, 2), (0, 1, 2)):
            w = rng.uniform(0.0, 1.0, size=(3, n)).astype(np.float32)
            for a in axes:  # coordinates in (-1/N, 0): weights in (-1, 0)
                w[a] = -rng.uniform(0.0, 1.0, size=n).astype(np.float32)
            v = _trilinear(c, w[0], w[1], w[2])
            margin = len(axes) and {1: 1, 2: 4, 3: 13}[len(axes)]
            assert np.all(v >= lo - np.float32(margin * h) - np.float32(1e-6)), (N, axes)


def test_extreme_corner_sets_meet_the_bound():
    """Corner sets at the edge of the Lipschitz condition and weights near
    -1 come close to the bound without crossing it."""
    h = np.float32(1.0 / 64)
    worst = np.float32(0)
    for bits in itertools.product((0, 1), repeat=8):
        c = np.array([1.0 + h * b for b in bits], dtype=np.float32)
        # only sets whose adjacent corners differ by at most h
        ok = all(abs(c[k] - c[k ^ m]) <= h + 1e-7 for k in range(8) for m in (1, 2, 4))
        if not ok:
            continue
        for wx, wy, wz in itertools.product((-0.999, -0.5, 0.0, 0.5), repeat=3):
            v = _trilinear(c, np.float32(wx), np.float32(wy), np.float32(wz))
            drop = c.min() - v
            assert drop <= np.float32(13) * h + np.float32(1e-6)
            worst = max(worst, drop)
    assert worst > h  # extrapolation does go below the smallest corner
