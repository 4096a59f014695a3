"""The allocation-free distance-field build, mo_df_build_noalloc.

It serves callers that cannot allocate device memory while they run (a plugin
inside a host runtime that owns the device memory pool, a real-time loop that
forbids allocation after start-up): its scratch is one fixed device array
inside libmeshode.so instead of caller or library allocations.

Two calls in a row through the C ABI, on two different targets (the second
takes the other build method, so it runs over what the first left in the
shared array), each compared with the regular entry point mo_df_build given
caller scratch.  Both take the same method and kernels on the same input, so
the grids must be equal bit for bit: a stale value left in the shared array
would show up here even if it moved a distance by one ulp.  Each grid is
also compared once with the FP64 oracle, within the distance-field tolerance
of the other GPU tests (1e-5 of the normalised target's bounding-box
diagonal).  A target too large for the fixed array is refused with
MO_ERR_SCRATCH.

The file is named so that pytest collects it last.
"""
import numpy as np
import pytest
import torch

from meshode_gb300 import _lib as L
from meshode_gb300 import meshgen
from oracle import pydeform_oracle as orc

pytestmark = pytest.mark.gpu

TOL_REL_DIAG = 1e-5


def _target(level, seed, dev):
    rng = np.random.Generator(np.random.PCG64(seed))
    V, F = meshgen.icosphere(level)
    T = meshgen.displace(V, rng).astype(np.float32)
    return torch.from_numpy(T).to(dev), torch.from_numpy(F.astype(np.int32)).to(dev)


def _params(V):
    s = L.stream_ptr()
    bbox = torch.empty(6, dtype=torch.int32, device=V.device)
    prm = torch.empty(4, dtype=torch.float64, device=V.device)
    L.call("mo_bbox", L.ptr(V), V.shape[0], L.ptr(bbox), s)
    L.call("mo_norm_params", L.ptr(bbox), L.ptr(prm), s)
    return prm


def _regular(V, F, N, prm):
    lib = L.lib()
    method = lib.mo_df_method_for(F.shape[0], N)
    nb = lib.mo_df_build_scratch_bytes(V.shape[0], F.shape[0], N, method)
    scratch = torch.empty(int(nb), dtype=torch.uint8, device=V.device)
    grid = torch.empty(N ** 3, dtype=torch.float32, device=V.device)
    L.call("mo_df_build", L.ptr(V), V.shape[0], L.ptr(F), F.shape[0], N, L.ptr(prm), method, L.ptr(scratch), nb,
           L.ptr(grid), None, L.stream_ptr())
    return grid


def _diag(V, prm):
    p = prm.cpu().numpy()
    Vn = (V.cpu().numpy().astype(np.float64) - p[1:]) / p[0]
    return float(np.linalg.norm(Vn.max(0) - Vn.min(0)))


def test_noalloc_matches_regular_build_twice(cuda):
    lib = L.lib()
    cases = [(4, 3, 48), (2, 4, 32)]  # (icosphere level, seed, N): LBVH first, then brute force
    methods = []
    grids = []
    inputs = []
    for level, seed, N in cases:
        V, F = _target(level, seed, cuda)
        prm = _params(V)
        methods.append(lib.mo_df_method_for(F.shape[0], N))
        grid = torch.full((N ** 3,), float("nan"), dtype=torch.float32, device=cuda)
        L.call("mo_df_build_noalloc", L.ptr(V), V.shape[0], L.ptr(F), F.shape[0], N, L.ptr(prm), L.ptr(grid),
               L.stream_ptr())
        grids.append(grid)
        inputs.append((V, F, N, prm))
    assert methods == [L.MO_DF_LBVH, L.MO_DF_BRUTE]
    for grid, (V, F, N, prm) in zip(grids, inputs):
        ref = _regular(V, F, N, prm)
        torch.cuda.synchronize()
        assert torch.isfinite(grid).all()
        assert torch.equal(grid, ref)
        p = prm.cpu().numpy()
        Vn = orc.normalized_double(V.cpu().numpy(), float(p[0]), p[1:])
        exact = orc.df_build(Vn, F.cpu().numpy(), N)
        err = np.abs(grid.cpu().numpy().astype(np.float64) - exact).max()
        assert err <= TOL_REL_DIAG * _diag(V, prm), err


def test_noalloc_rejects_targets_beyond_its_array(cuda):
    lib = L.lib()
    V, F = _target(6, 5, cuda)  # 81,920 triangles: more scratch than the fixed array
    N = 64
    method = lib.mo_df_method_for(F.shape[0], N)
    assert lib.mo_df_build_scratch_bytes(V.shape[0], F.shape[0], N, method) > lib.mo_df_noalloc_scratch_capacity()
    prm = _params(V)
    grid = torch.empty(N ** 3, dtype=torch.float32, device=cuda)
    rc = lib.mo_df_build_noalloc(L.ptr(V), V.shape[0], L.ptr(F), F.shape[0], N, L.ptr(prm), L.ptr(grid),
                                 L.stream_ptr())
    assert rc == L.MO_ERR_SCRATCH
    assert b"fixed" in lib.mo_last_error()
