"""On-demand distance field (mo_df_tree_build, mo_df_lazy_seed/fill and the
pool's MO_DF_ON_DEMAND mode) on the GPU.

* The cells a fill writes hold exactly the full build's values (banded and
  exact grids; N 64 and 128; positions inside, on the faces of and outside the
  unit cube), and the cell bits are set for exactly the cells the positions
  read.
* A pool filling grids on demand returns the same results and losses, bit for
  bit, as a pool that builds every grid at admission, on requests of the
  serving stream's shapes.
"""
import ctypes

import numpy as np
import pytest
import torch

from meshode_gb300 import _lib as L
from meshode_gb300 import meshgen, pool, serving
from meshode_gb300._lib import call, ptr, stream_ptr

pytestmark = pytest.mark.gpu


def _target(seed, n_tris):
    spec = meshgen.serving_requests(n=1, seed=seed, t_range=(n_tris, n_tris + 1), v_range=(500, 600))[0]
    _, _, Vt, Ft = meshgen.request_meshes(spec)
    return torch.from_numpy(Vt).cuda(), torch.from_numpy(Ft).cuda()


def _cells_of(P, N):
    """Cells df_eval reads for float4 positions P (the kernel's own rule)."""
    s = P[:, :3] * np.float32(N)
    c = np.trunc(s).astype(np.int64)
    ok = np.all((s > -1.0) & (c >= 0) & (c < N - 1), axis=1)
    c = c[ok]
    M = N - 1
    return np.unique((c[:, 2] * M + c[:, 1]) * M + c[:, 0])


@pytest.mark.parametrize("N,band_kind,seed", [(64, "loss", 1), (128, "loss", 2), (64, "exact", 3)])
def test_lazy_fill_matches_full_build(cuda, N, band_kind, seed):
    lib = L.lib()
    V, F = _target(seed, 20000)
    nv, nf = V.shape[0], F.shape[0]
    s = stream_ptr()
    bbox = torch.empty(6, dtype=torch.int32, device=cuda)
    params = torch.empty(4, dtype=torch.float64, device=cuda)
    call("mo_bbox", ptr(V), nv, ptr(bbox), s)
    call("mo_norm_params", ptr(bbox), ptr(params), s)
    band = lib.mo_df_loss_band(N) if band_kind == "loss" else 0.0
    # full build, relaid out into cell records
    opt = L.MoDfOptions(L.MO_DF_LBVH, L.MO_PACKET_4x4x2, band)
    sb = lib.mo_df_build_scratch_bytes(nv, nf, N, L.MO_DF_LBVH)
    scratch = torch.empty(sb, dtype=torch.uint8, device=cuda)
    glin = torch.empty(N ** 3, dtype=torch.float32, device=cuda)
    status = torch.zeros(4, dtype=torch.int32, device=cuda)
    call("mo_df_build_ex", ptr(V), nv, ptr(F), nf, N, ptr(params), ctypes.byref(opt), ptr(scratch), sb, ptr(glin),
         ptr(status), s)
    full = torch.empty(lib.mo_grid_bytes(N, L.MO_LAYOUT_CELL) // 4, dtype=torch.float32, device=cuda)
    call("mo_grid_relayout", ptr(glin), N, L.MO_LAYOUT_CELL, ptr(full), s)
    # the tree alone, then the cells of some positions
    tsb = lib.mo_df_tree_scratch_bytes(nv, nf)
    tscratch = torch.empty(tsb, dtype=torch.uint8, device=cuda)
    tree = torch.empty(lib.mo_df_tree_bytes(nf) // 4, dtype=torch.float32, device=cuda)
    call("mo_df_tree_build", ptr(V), nv, ptr(F), nf, ptr(params), ptr(tscratch), tsb, ptr(tree), ptr(status[1:2]), s)
    lin = torch.full((N ** 3,), float("nan"), dtype=torch.float32, device=cuda)
    grid = torch.full_like(full, float("nan"))
    bits = torch.zeros(lib.mo_df_lazy_bytes(N) // 4, dtype=torch.int32, device=cuda)
    cell_words = ((N - 1) ** 3 + 31) // 32
    pr = L.MoPair()
    pr.grid, pr.N, pr.layout = ptr(grid), N, L.MO_LAYOUT_CELL
    pr.df_tree, pr.df_lin = ptr(tree), ptr(lin)
    pr.df_cells, pr.df_packets = ptr(bits), ptr(bits[cell_words:])
    pr.df_status, pr.df_ntri, pr.df_band = ptr(status[2:3]), nf, band
    pair_dev = torch.frombuffer(bytearray(bytes(pr)), dtype=torch.uint8).to(cuda)
    rng = np.random.default_rng(seed)
    n = 3000
    P = np.zeros((n, 4), np.float32)
    P[:, :3] = rng.uniform(-0.05, 1.05, size=(n, 3)).astype(np.float32)
    P[:40, 0] = 0.0                               # on the x = 0 face
    P[40:80, 1] = np.float32((N - 1) / N)          # on the far face
    P[80:120, 2] = np.float32(-0.5 / N)            # within a voxel below: extrapolates from layer 0
    P[120:160, 2] = np.float32(-1.5 / N)           # further below: no cell
    Pd = torch.from_numpy(P).cuda()
    queue = torch.empty(2 * n, dtype=torch.int32, device=cuda)
    pqueue = torch.empty(16 * n, dtype=torch.int32, device=cuda)
    count = torch.zeros(2, dtype=torch.int32, device=cuda)
    call("mo_df_lazy_seed", ptr(pair_dev), 0, ptr(Pd), n, ptr(queue), ptr(pqueue), ptr(count), n, s)
    totals = torch.zeros(2, dtype=torch.int64, device=cuda)
    call("mo_df_lazy_fill", ptr(pair_dev), ptr(queue), ptr(pqueue), ptr(count), n, ptr(totals), s)
    torch.cuda.synchronize()
    assert totals.tolist() == count.tolist()
    assert status.tolist() == [0, 0, 0, 0]
    want = _cells_of(P, N)
    got = np.sort(queue[: 2 * int(count[0].item())].view(-1, 2)[:, 1].cpu().numpy())
    assert np.array_equal(got, want)
    # the packets queued: those of the cells' corners, each once
    M = N - 1
    cx, cy, cz = want % M, (want // M) % M, want // (M * M)
    b4 = (N + 3) // 4
    pks = set()
    for j in range(8):
        x, y, z = cx + (j & 1), cy + ((j >> 1) & 1), cz + (j >> 2)
        pks.update(((z // 2 * b4 + y // 4) * b4 + x // 4).tolist())
    gotp = pqueue[: 2 * int(count[1].item())].view(-1, 2)[:, 1].cpu().numpy()
    assert len(gotp) == len(set(gotp.tolist())) and set(gotp.tolist()) == pks
    b = bits[:cell_words].cpu().numpy().view(np.uint32)
    set_cells = np.nonzero(np.unpackbits(b.view(np.uint8), bitorder="little")[: (N - 1) ** 3])[0]
    assert np.array_equal(set_cells, want)
    g = grid.view(-1, 8)[torch.from_numpy(want).cuda()]
    f = full.view(-1, 8)[torch.from_numpy(want).cuda()]
    assert torch.equal(g.view(torch.int32), f.view(torch.int32))
    # a second fill of the same cells finds them queued and changes nothing
    count.zero_()
    call("mo_df_lazy_seed", ptr(pair_dev), 0, ptr(Pd), n, ptr(queue), ptr(pqueue), ptr(count), n, s)
    call("mo_df_lazy_fill", ptr(pair_dev), ptr(queue), ptr(pqueue), ptr(count), n, None, s)
    assert count.tolist() == [0, 0]


def test_lazy_arguments_are_checked(cuda):
    lib = L.lib()
    assert lib.mo_df_lazy_bytes(1) == 0 and lib.mo_df_lazy_bytes(L.MO_DF_LAZY_MAX_N + 1) == 0
    assert lib.mo_df_lazy_bytes(64) == 4 * ((63 ** 3 + 31) // 32 + (16 * 16 * 32 + 31) // 32)
    assert lib.mo_df_tree_bytes(0) == 0 and lib.mo_df_tree_bytes(10) == 16 * (56 + 8 * 9)  # 50 triangle float4 padded to 56
    assert lib.mo_df_lazy_fill(None, None, None, None, 0, None, None) == L.MO_ERR_INVALID
    assert lib.mo_df_tree_build(None, 0, None, 0, None, None, 0, None, None, None) == L.MO_ERR_INVALID


def _fresh(reqs):
    return [serving.Request(r.id, r.srcV, r.srcF, r.tarV, r.tarF, N=r.N, steps=r.steps) for r in reqs]


def test_on_demand_pool_matches_full_grids(cuda):
    # the serving stream's shapes (grids 64 and 128), shortened fits
    specs = meshgen.serving_requests(n=10, seed=5, steps=150)
    meshes = [meshgen.request_meshes(s) for s in specs]
    base = serving.requests_from_meshes(meshes, specs, device=None, pin=True)
    full = _fresh(base)
    Pf = pool.NativePool(group_steps=10, df_mode=L.MO_DF_FULL)
    Pf.run(full)
    assert Pf.stats().fill_launches_per_step == 0
    Pf.close()
    lazy = _fresh(base)
    Pl = pool.NativePool(group_steps=10, df_mode=L.MO_DF_ON_DEMAND)
    Pl.run(lazy)
    st = Pl.stats()
    assert st.fill_launches_per_step == 2 and st.failed == 0
    cells, packets = Pl.fill_totals()
    assert 0 < packets and 0 < cells
    Pl.close()
    for a, b in zip(full, lazy):
        assert a.error is None and b.error is None
        assert torch.equal(a.out, b.out)
        assert torch.equal(a.out_normalized, b.out_normalized)
        assert a.loss == b.loss
