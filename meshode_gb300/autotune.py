"""Autotuner for the serving loop: per size bucket, the fastest

* distance-field build: method (shared-memory brute force or LBVH) and the
  LBVH traversal packet shape (the 32 voxels a warp walks the tree with:
  4x4x2, 8x4x1, 4x2x4, 2x4x4, 8x2x2), timed with the loss-preserving band
  the serving builds use;
* fused-step configuration: grid brick layout (linear [z][y][x], 2x2x2
  overlapping cell bricks of 32 B, or 4x4x4 bricks of 256 B) and tile width
  (32-vertex slices per tile, 1-8).

Threads per vertex is fixed at one: a vertex's edge gradient is summed in
the reference's serial scatter order, which a split across threads would
reorder.  None of the knobs changes a result; only the speed.

Buckets: grid resolution N exactly, target triangles by power of two
(DF build); N and source vertices by power of two (step).  Each candidate is
timed with CUDA events on a synthetic mesh of the bucket's size (cube-sphere
source, displaced cube-sphere target).  Results are kept in memory and in a
JSON cache keyed by the GPU name (default meshode_gb300/_tune/autotune.json).
"""
import ctypes
import json
import math
import os

import numpy as np
import torch

from . import _lib as L
from . import meshgen
from ._lib import call, ptr, stream_ptr

PACKETS = {"4x4x2": L.MO_PACKET_4x4x2, "8x4x1": L.MO_PACKET_8x4x1, "4x2x4": L.MO_PACKET_4x2x4,
           "2x4x4": L.MO_PACKET_2x4x4, "8x2x2": L.MO_PACKET_8x2x2,
           "4x4x4": L.MO_PACKET_4x4x4, "2x4x8": L.MO_PACKET_2x4x8, "8x4x2": L.MO_PACKET_8x4x2,
           "4x4x2t": L.MO_PACKET_4x4x2_TRI2, "2x4x4t": L.MO_PACKET_2x4x4_TRI2}
LAYOUTS = {"linear": L.MO_LAYOUT_LINEAR, "cell": L.MO_LAYOUT_CELL, "brick4": L.MO_LAYOUT_BRICK4}
TILE_WIDTHS = (4, 8)
DEFAULT_CACHE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_tune", "autotune.json")


def t_bucket(ntri):
    return int(max(0, math.floor(math.log2(max(ntri, 1)))))


def v_bucket(nv):
    return int(max(0, math.floor(math.log2(max(nv, 1)))))


class Autotuner:
    def __init__(self, cache_path=DEFAULT_CACHE, reps=2, timer=None):
        self.cache_path = cache_path
        self.reps = int(reps)
        self.timer = timer  # optional callable(candidate_fn) -> ms, for tests
        self.device_name = torch.cuda.get_device_name() if torch.cuda.is_available() else "cpu"
        self.table = {"df": {}, "step": {}}
        self._load()

    # -- cache -------------------------------------------------------------
    def _load(self):
        if self.cache_path and os.path.exists(self.cache_path):
            try:
                data = json.load(open(self.cache_path))
                self.table = data.get(self.device_name, self.table)
            except (OSError, ValueError):
                pass

    def save(self):
        if not self.cache_path:
            return
        os.makedirs(os.path.dirname(self.cache_path), exist_ok=True)
        data = {}
        if os.path.exists(self.cache_path):
            try:
                data = json.load(open(self.cache_path))
            except (OSError, ValueError):
                data = {}
        data[self.device_name] = self.table
        tmp = self.cache_path + ".tmp"
        with open(tmp, "w") as fh:
            json.dump(data, fh, indent=1, sort_keys=True)
        os.replace(tmp, self.cache_path)

    # -- timing ------------------------------------------------------------
    def _time(self, fn):
        if self.timer is not None:
            return float(self.timer(fn))
        fn()
        torch.cuda.synchronize()
        best = float("inf")
        for _ in range(self.reps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            torch.cuda.synchronize()
            best = min(best, e0.elapsed_time(e1))
        return best

    # -- DF build ------------------------------------------------------------
    def df_options(self, N, ntri):
        """(method, packet) for a build of an N^3 grid over `ntri` triangles."""
        key = "%d/%d" % (N, t_bucket(ntri))
        hit = self.table["df"].get(key)
        if hit is None:
            hit = self._tune_df(N, 2 ** t_bucket(ntri))
            self.table["df"][key] = hit
        return hit["method"], hit["packet"]

    def _tune_df(self, N, ntri):
        dev = torch.device("cuda")
        rng = np.random.Generator(np.random.PCG64(ntri))
        Vt, Ft = meshgen.cubesphere_for_triangles(ntri)
        Vt = meshgen.displace(Vt, rng).astype(np.float32)
        Vd = torch.from_numpy(Vt).to(dev)
        Fd = torch.from_numpy(Ft.astype(np.int32)).to(dev)
        lib = L.lib()
        s = stream_ptr()
        bbox = torch.empty(6, dtype=torch.int32, device=dev)
        prm = torch.empty(4, dtype=torch.float64, device=dev)
        call("mo_bbox", ptr(Vd), Vd.shape[0], ptr(bbox), s)
        call("mo_norm_params", ptr(bbox), ptr(prm), s)
        grid = torch.empty(N ** 3, dtype=torch.float32, device=dev)
        nb = max(lib.mo_df_build_scratch_bytes(Vd.shape[0], Fd.shape[0], N, m) for m in (L.MO_DF_BRUTE, L.MO_DF_LBVH))
        scratch = torch.empty(int(nb), dtype=torch.uint8, device=dev)
        band = lib.mo_df_loss_band(N)  # the serving builds' band
        cands = [(L.MO_DF_LBVH, p) for p in PACKETS.values()]
        if Fd.shape[0] * float(N) ** 3 <= 2e9:
            cands.append((L.MO_DF_BRUTE, L.MO_PACKET_4x4x2))
        results = {}
        for method, packet in cands:
            opt = L.MoDfOptions(method, packet, band)

            def run(opt=opt):
                call("mo_df_build_ex", ptr(Vd), Vd.shape[0], ptr(Fd), Fd.shape[0], N, ptr(prm),
                     ctypes.byref(opt), ptr(scratch), nb, ptr(grid), None, s)
            results[(method, packet)] = self._time(run)
        (method, packet), ms = min(results.items(), key=lambda kv: kv[1])
        return {"method": int(method), "packet": int(packet), "ms": float(ms), "ntri": int(Fd.shape[0]),
                "candidates": {"%d/%d" % k: float(v) for k, v in results.items()}}

    # -- fused step ------------------------------------------------------------
    def step_options(self, N, nv):
        """(layout, slices_per_tile) for pairs of ~nv vertices on an N^3 grid."""
        key = "%d/%d" % (N, v_bucket(nv))
        hit = self.table["step"].get(key)
        if hit is None:
            hit = self._tune_step(N, 2 ** v_bucket(nv))
            self.table["step"][key] = hit
        return hit["layout"], hit["slices_per_tile"]

    def _tune_step(self, N, nv, npairs=None):
        from . import fused
        from . import pyDeform as PD
        dev = torch.device("cuda")
        npairs = npairs or max(1, min(64, (1 << 21) // max(nv, 1)))
        rng = np.random.Generator(np.random.PCG64(nv))
        Vs, Fs = meshgen.cubesphere_for_vertices(nv)
        Vt, Ft = meshgen.cubesphere_for_triangles(4 * nv)
        Vt = meshgen.displace(Vt, rng).astype(np.float32)
        pid = PD.InitializeDeformTemplate(torch.from_numpy(Vt), torch.from_numpy(Ft.astype(np.int32)), 0, N,
                                          layout=L.MO_LAYOUT_LINEAR)
        P = PD.GetParams(pid)
        grids = {L.MO_LAYOUT_LINEAR: P.grid_linear}
        for lay in (L.MO_LAYOUT_CELL, L.MO_LAYOUT_BRICK4):
            g = torch.empty(L.lib().mo_grid_bytes(N, lay) // 4, dtype=torch.float32, device=dev)
            call("mo_grid_relayout", ptr(P.grid_linear), N, lay, ptr(g), stream_ptr())
            grids[lay] = g
        V = torch.from_numpy(Vs.astype(np.float32)).to(dev)
        PD.NormalizeByTemplate(V, pid)
        PD.StoreRigidityInformation(V, torch.from_numpy(Fs.astype(np.int32)).to(dev), pid)
        st = P.edge
        results = {}
        for lay, grid in grids.items():
            for spt in TILE_WIDTHS:
                prs = [fused.Pair(grid, N, lay, V, st.csr, st.nh, st.rest, 100000, slices_per_tile=spt)
                       for _ in range(npairs)]
                runner = fused.StepGroupRunner(dev, npairs, sum(p.ntiles for p in prs), group_steps=10)
                runner.upload(prs, [0] * npairs)

                def run(runner=runner, prs=prs):
                    runner.upload(prs, [0] * len(prs))
                    runner.run_group()
                results[(lay, spt)] = self._time(run)
                del prs, runner
        PD.ReleaseTemplate(pid)
        (lay, spt), ms = min(results.items(), key=lambda kv: kv[1])
        return {"layout": int(lay), "slices_per_tile": int(spt), "ms_per_group": float(ms), "nv": int(V.shape[0]),
                "pairs": int(npairs), "candidates": {"%d/%d" % k: float(v) for k, v in results.items()}}

    def tune_for(self, requests):
        """Tune every bucket the requests touch (call before timing)."""
        for r in requests:
            self.df_options(r.N, int(r.tarF.shape[0]))
            self.step_options(r.N, int(r.srcV.shape[0]))
        self.save()
        return self.table
