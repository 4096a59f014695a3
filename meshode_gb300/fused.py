"""Device-resident deformation pairs and CUDA-graph groups of fused steps.

A *pair* is one source mesh being fitted to one target distance field.  Its
whole optimiser state lives in HBM: float4 positions (ping-pong), Adam
moments, the sliced-ELL edge records (rest offsets in the reference's
half-edge order) and a pointer to the target grid.  One ``mo_fused_step``
launch advances every active pair by one Adam step; a *group* of S launches
is captured once as a CUDA graph and replayed, with the pair and tile tables
re-uploaded between groups (all kernel inputs are read from device memory,
so the graph stays valid as pairs come and go).
"""
import ctypes
import math

import numpy as np
import torch

from . import _lib as L
from ._lib import call, ptr, stream_ptr

PAIR_BYTES = ctypes.sizeof(L.MoPair)
TILE_BYTES = ctypes.sizeof(L.MoTile)
SLICES_PER_TILE = 8
# int32 word offsets of the per-group fields inside a MoPair row
_OFF_T0 = L.MoPair.t0.offset // 4
_OFF_TILE0 = L.MoPair.tile0.offset // 4
_OFF_NTILES = L.MoPair.ntiles.offset // 4

_adam_tables = {}


def adam_table(tmax, lr, b1, b2, device):
    """float32 [tmax, 2]: (lr/(1-b1^t), sqrt(1-b2^t)) for t = 1..tmax,
    computed in Python double exactly as torch.optim.Adam does each step."""
    key = (int(tmax), float(lr), float(b1), float(b2), str(device))
    tab = _adam_tables.get(key)
    if tab is None:
        rows = np.empty((tmax, 2), np.float32)
        for t in range(1, tmax + 1):
            step = float(t)
            bc1 = 1 - b1 ** step
            bc2 = 1 - b2 ** step
            rows[t - 1, 0] = lr / bc1
            rows[t - 1, 1] = bc2 ** 0.5
        tab = torch.from_numpy(rows).to(device)
        _adam_tables[key] = tab
    return tab


class Pair:
    """Optimiser state of one deformation pair on the device."""

    def __init__(self, grid, N, layout, V, csr, nh, rest, steps, lr=1e-3, betas=(0.9, 0.999), eps=1e-8,
                 w_edge=1.0, mask_thresh=None, grad_scale=1.0, debug_grad=False, stream=None, slice_ptr=None,
                 nrec=None, slices_per_tile=SLICES_PER_TILE, edge_w=None):
        """V: normalised source vertices, float32 [nv,3] on the device (the
        optimiser's start).  csr/nh: the edge CSR buffer and half-edge count.
        rest: float32 [nv,3] positions the rest offsets were taken from (the V
        given to StoreRigidityInformation).  When slice_ptr/nrec are given, the
        sliced-ELL plan was already made.  edge_w: optional float32 [nh]
        per-edge weights (CadEdgeLoss); the pair then needs the weighted step
        (StepGroupRunner(weighted=True))."""
        dev = V.device
        s = stream_ptr(stream)
        self.device = dev
        self.grid = grid
        self.N = int(N)
        self.layout = int(layout)
        if self.layout == L.MO_LAYOUT_BRICK4 and self.N > 1280:
            raise RuntimeError("the brick layout supports grids up to 1280^3")
        if not 1 <= int(slices_per_tile) <= L.MO_TILE_WARPS:
            raise RuntimeError("slices per tile must be in [1, %d]" % L.MO_TILE_WARPS)
        self.slices_per_tile = int(slices_per_tile)
        self.nv = int(V.shape[0])
        self.nslices = (self.nv + 31) // 32
        self.steps = int(steps)
        self.t = 0
        self.lr = float(lr)
        self.b1, self.b2 = float(betas[0]), float(betas[1])
        self.eps = float(eps)
        self.w_edge = float(w_edge)
        self.mask_thresh = mask_thresh
        self.grad_scale = float(grad_scale)
        self.pos = torch.zeros(2, self.nv, 4, dtype=torch.float32, device=dev)
        call("mo_pack_pos", ptr(V), self.nv, ptr(self.pos[0]), s)
        self.rest = torch.empty(self.nv, 4, dtype=torch.float32, device=dev)
        call("mo_pack_pos", ptr(rest.contiguous()), self.nv, ptr(self.rest), s)
        self.m = torch.zeros(self.nv * 3, dtype=torch.float32, device=dev)
        self.v = torch.zeros(self.nv * 3, dtype=torch.float32, device=dev)
        if slice_ptr is None:
            slice_ptr = torch.empty(self.nslices + 1, dtype=torch.int32, device=dev)
            call("mo_sell_plan", ptr(csr), self.nv, nh, ptr(slice_ptr), s)
            nrec = int(slice_ptr[self.nslices].item())
        self.slice_ptr = slice_ptr
        self.nrec = int(nrec)
        self.sell = torch.empty(max(self.nrec, 1), dtype=torch.int32, device=dev)
        call("mo_sell_fill", ptr(csr), self.nv, nh, ptr(self.slice_ptr), ptr(self.sell), s)
        self.sell_w = None
        if edge_w is not None:
            self.sell_w = torch.empty(max(self.nrec, 1), dtype=torch.float32, device=dev)
            call("mo_sell_fill_w", ptr(csr), self.nv, nh, ptr(self.slice_ptr), ptr(edge_w.contiguous()),
                 ptr(self.sell_w), s)
        self.grad_dbg = torch.zeros(self.nv * 3, dtype=torch.float32, device=dev) if debug_grad else None
        self.adam_tab = adam_table(max(self.steps, 1), self.lr, self.b1, self.b2, dev)
        self.loss_history = []
        self._row = None
        self._row_steps = None
        self._tiles = None

    def nbytes(self):
        return (self.pos.numel() + self.rest.numel() + self.m.numel() + self.v.numel() + self.sell.numel()) * 4 + \
            self.slice_ptr.numel() * 4

    @property
    def done(self):
        return self.t >= self.steps

    def positions(self):
        """Current positions as float32 [nv,3] (a view-free copy)."""
        return self.pos[self.t & 1, :, :3].contiguous()

    @property
    def ntiles(self):
        return tiles_for(self.nslices, self.slices_per_tile)

    def row(self):
        """This pair's MoPair bytes (t0, tile0 and ntiles are set per group)."""
        if self._row is None or self._row_steps != self.steps:
            self._row = np.frombuffer(bytes(self.struct(0, 0, 0)), np.uint8).copy()
            self._row_steps = self.steps
        return self._row

    def tile_rows(self):
        """int32 [ntiles, 4] = (pair, first slice, slices, 0) with pair = 0."""
        if self._tiles is None:
            nt, spt = self.ntiles, self.slices_per_tile
            t = np.zeros((nt, 4), np.int32)
            t[:, 1] = np.arange(nt) * spt
            t[:, 2] = np.minimum(spt, self.nslices - t[:, 1])
            self._tiles = t
        return self._tiles

    def struct(self, t0, tile0, ntiles):
        p = L.MoPair()
        p.grid = self.grid.data_ptr()
        p.slice_ptr = self.slice_ptr.data_ptr()
        p.sell = self.sell.data_ptr()
        p.rest = self.rest.data_ptr()
        p.pos0 = self.pos[0].data_ptr()
        p.pos1 = self.pos[1].data_ptr()
        p.adam_m = self.m.data_ptr()
        p.adam_v = self.v.data_ptr()
        p.adam_tab = self.adam_tab.data_ptr()
        p.grad_dbg = self.grad_dbg.data_ptr() if self.grad_dbg is not None else None
        p.sell_w = self.sell_w.data_ptr() if self.sell_w is not None else None
        p.N, p.layout, p.nv, p.nslices = self.N, self.layout, self.nv, self.nslices
        p.w_edge = self.w_edge
        p.mask_thresh = float(self.mask_thresh) if self.mask_thresh is not None else 0.0
        p.use_mask = 1 if self.mask_thresh is not None else 0
        p.grad_scale = self.grad_scale
        p.one_minus_b1 = 1 - self.b1
        p.b2 = self.b2
        p.one_minus_b2 = 1 - self.b2
        p.eps = self.eps
        p.t0 = int(t0)
        p.t_end = self.steps
        p.tile0, p.ntiles = int(tile0), int(ntiles)
        return p


def tiles_for(nslices, slices_per_tile=SLICES_PER_TILE):
    return (nslices + slices_per_tile - 1) // slices_per_tile


class StepGroupRunner:
    """Runs groups of S fused steps over a set of pairs (graph-captured)."""

    def __init__(self, device, max_pairs, max_tiles, group_steps=25, use_graph=True, weighted=False):
        self.device = device
        self.weighted = bool(weighted)  # pairs with per-edge weights: mo_fused_step_weighted
        self.max_pairs = int(max_pairs)
        self.max_tiles = int(max_tiles)
        self.S = int(group_steps)
        self.use_graph = use_graph
        self.pairs_dev = torch.zeros(self.max_pairs * PAIR_BYTES, dtype=torch.uint8, device=device)
        self.tiles_dev = torch.zeros(self.max_tiles * TILE_BYTES, dtype=torch.uint8, device=device)
        self.ntiles_dev = torch.zeros(1, dtype=torch.int32, device=device)
        self.tile_loss = torch.zeros(self.S * self.max_tiles * L.MO_TILE_WARPS, dtype=torch.float32, device=device)
        self.pair_loss = torch.zeros(self.S * self.max_pairs, dtype=torch.float64, device=device)
        nbytes = self.max_pairs * PAIR_BYTES + self.max_tiles * TILE_BYTES + 4
        self._staging = [torch.zeros(nbytes, dtype=torch.uint8).pin_memory() for _ in range(2)]
        self._staging_ev = [None, None]
        self._slot = 0
        self._tiles_key = None
        self.graph = None
        self.npairs = 0
        self.ntiles = 0
        self.launches = 0  # fused-step kernel launches issued

    def _launch_group(self):
        s = stream_ptr()
        step = "mo_fused_step_weighted" if self.weighted else "mo_fused_step"
        for k in range(self.S):
            call(step, ptr(self.pairs_dev), ptr(self.tiles_dev), ptr(self.ntiles_dev), self.max_tiles, k,
                 ptr(self.tile_loss), 0, s)

    def upload(self, pairs, t0s):
        """Write the pair and tile tables for the next group (async H2D).
        Each pair's table row and tile rows are built once and cached; the
        tile table is only re-sent when the list of active pairs changed."""
        n = len(pairs)
        if n > self.max_pairs:
            raise RuntimeError("too many pairs for this runner (%d > %d)" % (n, self.max_pairs))
        nts = np.fromiter((p.ntiles for p in pairs), np.int64, count=n)
        total = int(nts.sum()) if n else 0
        if total > self.max_tiles:
            raise RuntimeError("too many tiles for this runner (%d > %d)" % (total, self.max_tiles))
        key = tuple(id(p) for p in pairs)
        send_tiles = key != self._tiles_key
        slot = self._slot
        self._slot ^= 1
        ev = self._staging_ev[slot]
        if ev is not None:
            ev.synchronize()
        buf = self._staging[slot]
        view = buf.numpy()
        pb = n * PAIR_BYTES
        if n:
            tab = view[:pb].reshape(n, PAIR_BYTES)
            for i, p in enumerate(pairs):
                tab[i] = p.row()
            ints = tab.view(np.int32)
            tile0 = np.concatenate([[0], np.cumsum(nts)[:-1]])
            ints[:, _OFF_T0] = np.asarray(t0s, np.int32)
            ints[:, _OFF_TILE0] = tile0
            ints[:, _OFF_NTILES] = nts
            self.pairs_dev[:pb].copy_(buf[:pb], non_blocking=True)
        tb = total * TILE_BYTES
        t_off = self.max_pairs * PAIR_BYTES
        nt_off = t_off + self.max_tiles * TILE_BYTES
        if send_tiles:
            if total:
                tiles = view[t_off:t_off + tb].view(np.int32).reshape(total, 4)
                tiles[:] = np.concatenate([p.tile_rows() for p in pairs])
                tiles[:, 0] = np.repeat(np.arange(n, dtype=np.int32), nts)
                self.tiles_dev[:tb].copy_(buf[t_off:t_off + tb], non_blocking=True)
            view[nt_off:nt_off + 4].view(np.int32)[0] = total
            self.ntiles_dev.view(torch.uint8).copy_(buf[nt_off:nt_off + 4], non_blocking=True)
            self._tiles_key = key
        ev = torch.cuda.Event()
        ev.record()
        self._staging_ev[slot] = ev
        self.npairs = n
        self.ntiles = total

    def run_group(self):
        """Launch S fused steps (graph replay when enabled)."""
        if self.use_graph:
            if self.graph is None:
                # warm-up (occupancy query, module load) and capture both run
                # with an empty tile table, so neither advances any pair
                saved = self.ntiles_dev.clone()
                self.ntiles_dev.zero_()
                self._launch_group()
                torch.cuda.synchronize(self.device)
                g = torch.cuda.CUDAGraph()
                with torch.cuda.graph(g):
                    self._launch_group()
                torch.cuda.synchronize(self.device)
                self.ntiles_dev.copy_(saved)
                self.graph = g
            self.graph.replay()
        else:
            self._launch_group()
        self.launches += self.S

    def pair_losses(self, nlaunch=None):
        """float64 [nlaunch, npairs] losses of the last group (device tensor)."""
        n = self.S if nlaunch is None else int(nlaunch)
        call("mo_pair_loss", ptr(self.pairs_dev), self.npairs, self.max_tiles, n, ptr(self.tile_loss),
             ptr(self.pair_loss), stream_ptr())
        return self.pair_loss[:n * self.npairs].view(n, self.npairs)


def pair_from_template(pid, src_V_norm, steps, lr=1e-3, w_edge=1.0, mask_thresh=None, debug_grad=False, **kw):
    """Pair state from a pyDeform template whose edge information is stored.
    src_V_norm: normalised source vertices (float32 [nv,3], any device)."""
    from . import pyDeform
    p = pyDeform.GetParams(pid)
    st = p.edge
    if st is None:
        raise RuntimeError("template %d has no stored edge information" % int(pid))
    V = src_V_norm.detach().to(p.device).contiguous()
    return Pair(p.grid, p.N, p.layout, V, st.csr, st.nh, st.rest, steps, lr=lr, w_edge=w_edge,
                mask_thresh=mask_thresh, debug_grad=debug_grad, edge_w=st.weights, **kw)


def fused_fit(pid, src_V_norm, steps, lr=1e-3, group_steps=25, use_graph=True, w_edge=1.0, mask_thresh=None,
              record_loss=False):
    """Fit one pair with the fused step (the GPU-native form of the
    reference's plain Adam loop, rigid_deform.py:34-41; with the template's
    CAD edges (StoreCadInformation), the CadLossFunction objective,
    cad_loss_layer.py:9-31, on the weighted step).  Returns
    (final normalised positions [nv,3] on the device, per-step losses or None)."""
    pr = pair_from_template(pid, src_V_norm, steps, lr=lr, w_edge=w_edge, mask_thresh=mask_thresh)
    runner = StepGroupRunner(pr.device, 1, pr.ntiles, group_steps=group_steps, use_graph=use_graph,
                             weighted=pr.sell_w is not None)
    losses = []
    while not pr.done:
        runner.upload([pr], [pr.t])
        runner.run_group()
        n = min(runner.S, pr.steps - pr.t)
        if record_loss:
            losses.append(runner.pair_losses(n)[:, 0].clone())
        pr.t += n
    out = pr.positions()
    return out, (torch.cat(losses) if record_loss else None)
