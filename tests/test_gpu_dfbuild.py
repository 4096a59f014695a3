"""Distance-field build on the GPU against the FP64 oracle, and the LBVH
stages bit for bit against the CPU build of the same Morton codes.

Reference: Mesh::Normalize (src/lib/mesh.cc:66-96) and
Mesh::ConstructDistanceField (mesh.cc:106-152).  Tolerance: fp32 error at or
below 1e-5 of the normalised target's bounding-box diagonal.
"""
import numpy as np
import pytest
import torch

from meshode_gb300 import _lib as L
from meshode_gb300 import meshgen
from meshode_gb300 import pyDeform as PD

pytestmark = pytest.mark.gpu

TOL_REL_DIAG = 1e-5


def _target(level, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    V, F = meshgen.icosphere(level)
    return meshgen.displace(V, rng).astype(np.float32), F.astype(np.int32)


def _diag(Vn64):
    return float(np.linalg.norm(Vn64.max(0) - Vn64.min(0)))


@pytest.mark.parametrize("method", [L.MO_DF_BRUTE, L.MO_DF_LBVH])
@pytest.mark.parametrize("level,N", [(0, 8), (2, 24), (3, 32), (0, 7), (1, 13)])
def test_df_vs_fp64(cuda, orc, method, level, N):
    """Both methods against the FP64 oracle, including grids whose size is
    not a multiple of the voxel packets (partial packets at the far faces)."""
    V, F = _target(level, seed=level + 1)
    pid = PD.InitializeDeformTemplate(torch.from_numpy(V), torch.from_numpy(F), 0, N, df_method=method)
    g = PD.GetDistanceField(pid).cpu().numpy().reshape(-1).astype(np.float64)
    scale, trans = orc.normalize_params(V)
    s2, t2 = PD.GetTransform(pid)
    assert s2 == scale and np.array_equal(t2, trans)
    Vn = orc.normalized_double(V, scale, trans)
    ref = orc.df_build(Vn, F, N, method="brute")
    err = np.abs(g - ref).max()
    assert err <= TOL_REL_DIAG * _diag(Vn), (err, _diag(Vn))
    other = L.MO_DF_LBVH if method == L.MO_DF_BRUTE else L.MO_DF_BRUTE
    pid2 = PD.InitializeDeformTemplate(torch.from_numpy(V), torch.from_numpy(F), 0, N, df_method=other)
    assert torch.equal(PD.GetDistanceField(pid), PD.GetDistanceField(pid2))  # the two methods, bit for bit
    PD.ReleaseTemplate(pid2)


def test_df_lbvh_large_subsampled(cuda, orc):
    # ico-5 target (20,480 triangles) at 64^3, checked on 1% of the voxels
    V, F = _target(5, seed=1)
    N = 64
    pid = PD.InitializeDeformTemplate(torch.from_numpy(V), torch.from_numpy(F), 0, N, df_method=L.MO_DF_LBVH)
    g = PD.GetDistanceField(pid).cpu().numpy().reshape(-1).astype(np.float64)
    scale, trans = orc.normalize_params(V)
    Vn = orc.normalized_double(V, scale, trans)
    rng = np.random.Generator(np.random.PCG64(3))
    vox = rng.choice(N ** 3, size=N ** 3 // 100, replace=False).astype(np.int64)
    ref = orc.df_build(Vn, F, N, voxels=vox, method="bvh")
    err = np.abs(g[vox] - ref).max()
    assert err <= TOL_REL_DIAG * _diag(Vn), err


def test_df_degenerate_and_single_triangle(cuda, orc):
    # one triangle; then a mesh with a zero-area (collinear) and a repeated-vertex face
    V = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0.5, 0.5, 1], [2, 0, 0]], np.float32)
    for F in (np.array([[0, 1, 2]], np.int32),
              np.array([[0, 1, 2], [0, 1, 4], [3, 3, 3], [0, 3, 1]], np.int32)):
        for method in (L.MO_DF_BRUTE, L.MO_DF_LBVH):
            N = 12
            pid = PD.InitializeDeformTemplate(torch.from_numpy(V), torch.from_numpy(F), 0, N, df_method=method)
            g = PD.GetDistanceField(pid).cpu().numpy().reshape(-1).astype(np.float64)
            scale, trans = orc.normalize_params(V)
            Vn = orc.normalized_double(V, scale, trans)
            ref = orc.df_build(Vn, F, N, method="brute")
            assert np.abs(g - ref).max() <= TOL_REL_DIAG * _diag(Vn)


def test_df_bad_face_index_raises(cuda):
    V = np.random.rand(10, 3).astype(np.float32)
    F = np.array([[0, 1, 2], [3, 4, 99]], np.int32)
    for method in (L.MO_DF_BRUTE, L.MO_DF_LBVH):
        with pytest.raises(RuntimeError):
            PD.InitializeDeformTemplate(torch.from_numpy(V), torch.from_numpy(F), 0, 8, df_method=method)


@pytest.mark.parametrize("level", [0, 2, 4, 6])
def test_lbvh_bitexact(cuda, orc, level):
    V, F = _target(level, seed=5)
    if level == 6:  # duplicate codes: many tiny triangles share Morton cells
        pass
    dev = cuda
    Vd = torch.from_numpy(V).to(dev)
    Fd = torch.from_numpy(F).to(dev)
    nf = F.shape[0]
    bbox = torch.empty(6, dtype=torch.int32, device=dev)
    prm = torch.empty(4, dtype=torch.float64, device=dev)
    s = L.stream_ptr()
    L.call("mo_bbox", L.ptr(Vd), V.shape[0], L.ptr(bbox), s)
    L.call("mo_norm_params", L.ptr(bbox), L.ptr(prm), s)
    codes = torch.empty(nf, dtype=torch.int32, device=dev)
    order = torch.empty(nf, dtype=torch.int32, device=dev)
    left = torch.empty(max(nf - 1, 1), dtype=torch.int32, device=dev)
    right = torch.empty(max(nf - 1, 1), dtype=torch.int32, device=dev)
    box = torch.empty(6, dtype=torch.float32, device=dev)
    L.call("mo_lbvh_build", L.ptr(Vd), V.shape[0], L.ptr(Fd), nf, L.ptr(prm), None, 0, L.ptr(codes), L.ptr(order),
           L.ptr(left), L.ptr(right), L.ptr(box), s)
    scale, trans = orc.normalize_params(V)
    Vn32 = orc.normalized_double(V, scale, trans).astype(np.float32)
    oc = orc.morton_codes(Vn32, F)
    sc, perm = orc.sort_codes(oc)
    ol, orr = orc.karras(sc)
    assert np.array_equal(codes.cpu().numpy().view(np.uint32), sc)
    assert np.array_equal(order.cpu().numpy(), perm)
    if nf > 1:
        assert np.array_equal(left.cpu().numpy()[:nf - 1], ol)
        assert np.array_equal(right.cpu().numpy()[:nf - 1], orr)
        tri = Vn32[F]
        assert np.array_equal(box.cpu().numpy()[:3], tri.reshape(-1, 3).min(0))
        assert np.array_equal(box.cpu().numpy()[3:], tri.reshape(-1, 3).max(0))
