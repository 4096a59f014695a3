"""Continuous-batching serving loop for deformation requests.

A request is one (source mesh, target mesh, grid resolution, step count)
fit, i.e. one run of the reference's rigid_deform loop
(src/python/rigid_deform.py:25-44): normalise by the target, build the
target's distance field, store the rigidity information, run ``steps`` Adam
steps of DistanceFieldLoss + RigidEdgeLoss, denormalise.

Requests that arrive while others are on the GPU are admitted as memory and
slots free up:

* admission is by HBM bytes (grid, mesh copies, edge records, Adam state and
  the transient distance-field build scratch) against a budget;
* each admitted request is prepared on a side stream (H2D copies, DF build,
  CSR and sliced-ELL records) while the step stream keeps stepping the
  already-active pairs, so the two overlap on the device;
* every group of S optimiser steps of all active pairs is one replay of a
  captured CUDA graph of S persistent fused-step launches;
* a pair whose last step ran in a group is retired right after it: its
  positions are denormalised (Finalize) and copied out, and its memory is
  released for the next admission.

Each pair's arithmetic depends only on its own state, so a result is the
same, bit for bit, whether the request ran alone or in any mix.
"""
import collections
import ctypes
import gc
import time

import numpy as np
import torch

from . import _lib as L
from . import fused
from ._lib import call, ptr, stream_ptr


class Request:
    """One deformation request.  Meshes may be CPU (pinned for async copies)
    or CUDA tensors: srcV float32 [n,3], srcF int32 [m,3], tarV float32
    [k,3], tarF int32 [l,3]."""

    def __init__(self, rid, srcV, srcF, tarV, tarF, N=64, steps=500, lr=1e-3, w_edge=1.0, arrival=0.0):
        self.id = rid
        self.srcV, self.srcF, self.tarV, self.tarF = srcV, srcF, tarV, tarF
        self.N = int(N)
        self.steps = int(steps)
        self.lr = float(lr)
        self.w_edge = float(w_edge)
        self.arrival = float(arrival)
        # results
        self.out = None            # denormalised fitted vertices [n,3]
        self.out_normalized = None  # fitted vertices in the target-normalised frame (device)
        self.error = None
        self.t_arrive = None
        self.t_admit = None
        self.t_active = None
        self.t_done = None

    @property
    def latency(self):
        return None if self.t_done is None else self.t_done - self.t_arrive


def estimate_bytes(nv, nf_src, nv_tar, nf_tar, N, layout=L.MO_LAYOUT_CELL, df_mode=L.MO_DF_FULL):
    """Peak device bytes one request holds from admission to retirement
    (the grid counted in the largest layout); df_mode MO_DF_ON_DEMAND adds
    the native pool's traversal tree, cell bits and seeding queue."""
    lib = L.lib()
    nh = 3 * nf_src
    grid = max(lib.mo_grid_bytes(N, lay) for lay in (L.MO_LAYOUT_CELL, L.MO_LAYOUT_BRICK4, layout)) + 4 * N ** 3
    scratch = lib.mo_df_build_scratch_bytes(nv_tar, nf_tar, N, L.MO_DF_AUTO)
    if df_mode == L.MO_DF_ON_DEMAND:
        grid += lib.mo_df_tree_bytes(nf_tar) + lib.mo_df_lazy_bytes(N) + ctypes.sizeof(L.MoPair) + 72 * nv + 256
        scratch = lib.mo_df_tree_scratch_bytes(nv_tar, nf_tar)
    meshes = 12 * (nv + nf_src + nv_tar + nf_tar)
    edges = lib.mo_edge_csr_bytes(nv, nf_src, L.MO_EDGES_FACES)
    sell = 4 * (2 * nh + 32 * ((nv + 31) // 32) * 4)
    state = 48 * nv + 24 * nv + 4 * ((nv + 31) // 32 + 1) + 12 * nv
    return int(grid + scratch + meshes + edges + sell + state + (1 << 16))


class _Job:
    __slots__ = ("req", "bytes", "phase", "ev", "host", "nv", "nh", "Vd", "Fd", "params", "grid", "csr", "off",
                 "slice_ptr", "status", "pair", "out_dev", "out_host", "stream", "layout", "spt")

    def __init__(self, req, nbytes):
        self.req = req
        self.bytes = nbytes
        self.phase = 0
        self.ev = None
        self.pair = None
        self.out_dev = self.out_host = None


class ServingEngine:
    def __init__(self, device=None, hbm_budget_bytes=None, max_pairs=512, max_tiles=None, group_steps=25,
                 layout=L.MO_LAYOUT_CELL, use_graph=True, max_building=8, results_to_host=True, lr=1e-3,
                 build_streams=2, autotuner=None, df_band=-1.0):
        L.require_cuda()
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        free, total = torch.cuda.mem_get_info(self.device)
        self.budget = int(hbm_budget_bytes) if hbm_budget_bytes else int(free * 0.6)
        self.layout = int(layout)
        self.max_pairs = int(max_pairs)
        if max_tiles is None:
            max_tiles = 1 << 17
        self.runner = fused.StepGroupRunner(self.device, self.max_pairs, int(max_tiles), group_steps=group_steps,
                                            use_graph=use_graph)
        # builds alternate between side streams so one build's set-up kernels
        # and tail overlap another's traversal
        self.build_streams = [torch.cuda.Stream(self.device) for _ in range(max(1, int(build_streams)))]
        self._next_build = 0
        self.step_stream = torch.cuda.current_stream(self.device)
        self.max_building = int(max_building)
        # per-request DF build options and step layout / tile width
        self.autotuner = autotuner
        # DF band: < 0 the loss-preserving band of mo_df_loss_band, 0 exact
        self.df_band = float(df_band)
        self.results_to_host = bool(results_to_host)
        self.in_use = 0
        self.peak_in_use = 0
        self.group_time_s = 0.0
        self.group_bytes = 0.0
        self.groups = 0
        self._timing = []

    # ------------------------------------------------------------------
    def _to_dev(self, t, copy=False):
        if copy and t.is_cuda:
            out = torch.empty_like(t, memory_format=torch.contiguous_format)
            out.copy_(t, non_blocking=True)
            return out
        return t.to(self.device, non_blocking=True).contiguous()

    def _phase_a(self, job):
        """Copies, DF build, normalisation, edge offsets, CSR, ELL plan."""
        req = job.req
        lib = L.lib()
        job.stream = self.build_streams[self._next_build % len(self.build_streams)]
        self._next_build += 1
        with torch.cuda.stream(job.stream):
            s = stream_ptr(job.stream)
            Vd = self._to_dev(req.srcV, copy=True)  # normalised in place below
            Fd = self._to_dev(req.srcF)
            Td = self._to_dev(req.tarV)
            TFd = self._to_dev(req.tarF)
            nv, nf = Vd.shape[0], Fd.shape[0]
            job.status = torch.zeros(4, dtype=torch.int32, device=self.device)
            bbox = torch.empty(6, dtype=torch.int32, device=self.device)
            job.params = torch.empty(4, dtype=torch.float64, device=self.device)
            call("mo_bbox", ptr(Td), Td.shape[0], ptr(bbox), s)
            call("mo_norm_params", ptr(bbox), ptr(job.params), s)
            N = req.N
            if self.autotuner is not None:
                method, packet = self.autotuner.df_options(N, TFd.shape[0])
                job.layout, job.spt = self.autotuner.step_options(N, nv)
            else:
                method, packet = L.MO_DF_AUTO, L.MO_PACKET_4x4x2
                job.layout, job.spt = self.layout, fused.SLICES_PER_TILE
            band = lib.mo_df_loss_band(N) if self.df_band < 0 else self.df_band
            opt = L.MoDfOptions(method, packet, band)
            nb = lib.mo_df_build_scratch_bytes(Td.shape[0], TFd.shape[0], N, method)
            scratch = torch.empty(int(nb), dtype=torch.uint8, device=self.device)
            glin = torch.empty(N ** 3, dtype=torch.float32, device=self.device)
            call("mo_df_build_ex", ptr(Td), Td.shape[0], ptr(TFd), TFd.shape[0], N, ptr(job.params),
                 ctypes.byref(opt), ptr(scratch), nb, ptr(glin), ptr(job.status[0:1]), s)
            del scratch
            if job.layout == L.MO_LAYOUT_LINEAR:
                job.grid = glin
            else:
                job.grid = torch.empty(lib.mo_grid_bytes(N, job.layout) // 4, dtype=torch.float32,
                                       device=self.device)
                call("mo_grid_relayout", ptr(glin), N, job.layout, ptr(job.grid), s)
                del glin
            del Td, TFd
            call("mo_normalize", ptr(Vd), nv, ptr(job.params), 0, s)
            nh = 3 * nf
            cb = lib.mo_edge_csr_bytes(nv, nf, L.MO_EDGES_FACES)
            job.csr = torch.empty((cb + 3) // 4, dtype=torch.int32, device=self.device)
            call("mo_edge_csr_build", ptr(Fd), nf, L.MO_EDGES_FACES, nv, ptr(job.csr), cb, ptr(job.status[1:2]), s)
            nsl = (nv + 31) // 32
            job.slice_ptr = torch.empty(nsl + 1, dtype=torch.int32, device=self.device)
            call("mo_sell_plan", ptr(job.csr), nv, nh, ptr(job.slice_ptr), s)
            job.status[2:3].copy_(job.slice_ptr[nsl:nsl + 1])
            job.host = torch.empty(4, dtype=torch.int32).pin_memory()
            job.host.copy_(job.status, non_blocking=True)
            job.Vd, job.Fd, job.nv, job.nh = Vd, Fd, nv, nh
            job.ev = torch.cuda.Event()
            job.ev.record(job.stream)
        job.phase = 1

    def _phase_b(self, job):
        """Validate the build, then the sliced-ELL records and optimiser state."""
        st = job.host.tolist()
        if st[0] or st[1]:
            job.req.error = "invalid mesh (DF status %d, edge status %d)" % (st[0], st[1])
            return False
        req = job.req
        with torch.cuda.stream(job.stream):
            # the rest offsets are taken from the normalised source itself
            job.pair = fused.Pair(job.grid, req.N, job.layout, job.Vd, job.csr, job.nh, job.Vd, req.steps,
                                  lr=req.lr, w_edge=req.w_edge, stream=job.stream, slice_ptr=job.slice_ptr,
                                  nrec=st[2], slices_per_tile=job.spt)
            job.csr = job.off = job.Fd = job.Vd = None
            for t in (job.grid, job.pair.pos, job.pair.rest, job.pair.m, job.pair.v, job.pair.sell,
                      job.pair.slice_ptr, job.params):
                t.record_stream(self.step_stream)
            job.ev = torch.cuda.Event()
            job.ev.record(job.stream)
        job.phase = 2
        return True

    def _retire(self, job):
        """Finalize (denormalise) and copy out the fitted positions."""
        req = job.req
        pr = job.pair
        s = stream_ptr(self.step_stream)
        out = torch.empty(pr.nv, 3, dtype=torch.float32, device=self.device)
        call("mo_unpack_pos", ptr(pr.pos[pr.t & 1]), pr.nv, ptr(out), s)
        req.out_normalized = out.clone()
        call("mo_normalize", ptr(out), pr.nv, ptr(job.params), 1, s)
        if self.results_to_host:
            host = torch.empty(pr.nv, 3, dtype=torch.float32).pin_memory()
            host.copy_(out, non_blocking=True)
            job.out_host = host
        job.out_dev = out
        job.ev = torch.cuda.Event()
        job.ev.record(self.step_stream)
        job.phase = 4

    def _release(self, job):
        self.in_use -= job.bytes
        job.pair = None
        job.grid = job.params = job.status = job.slice_ptr = None

    # ------------------------------------------------------------------
    def run(self, requests, realtime=False, measure_groups=True):
        """Serve ``requests`` to completion.  With realtime=True a request
        becomes visible at its ``arrival`` time (seconds after the start);
        otherwise all are queued at the start.  Returns the wall time (s).
        The garbage collector is held off while serving (a full collection
        stalls the loop for tens of ms)."""
        gc_on = gc.isenabled()
        gc.disable()
        try:
            return self._serve(requests, realtime, measure_groups)
        finally:
            if gc_on:
                gc.enable()

    def _serve(self, requests, realtime, measure_groups):
        lib = L.lib()
        future = collections.deque(sorted(requests, key=lambda r: r.arrival))
        pending = collections.deque()
        building, active, retiring = [], [], []
        ndone = 0
        total = len(requests)
        # the Adam tables are shared: make them before any admission
        for r in requests:
            fused.adam_table(max(r.steps, 1), r.lr, 0.9, 0.999, self.device)
        torch.cuda.synchronize(self.device)
        t0 = time.perf_counter()
        S = self.runner.S
        while ndone < total:
            now = time.perf_counter()
            while future and (not realtime or future[0].arrival <= now - t0):
                r = future.popleft()
                r.t_arrive = t0 + r.arrival if realtime else t0
                pending.append(r)
            # admission (FIFO, by HBM bytes and slots)
            while pending and len(building) < self.max_building and \
                    len(active) + len(building) + len(retiring) < self.max_pairs:
                r = pending[0]
                nb = estimate_bytes(r.srcV.shape[0], r.srcF.shape[0], r.tarV.shape[0], r.tarF.shape[0], r.N,
                                    self.layout)
                if self.in_use + nb > self.budget and (active or building or retiring):
                    break
                pending.popleft()
                job = _Job(r, nb)
                self.in_use += nb
                self.peak_in_use = max(self.peak_in_use, self.in_use)
                r.t_admit = time.perf_counter()
                try:
                    self._phase_a(job)
                except Exception as e:  # bad input: fail this request only
                    r.error = str(e)
                    r.t_done = time.perf_counter()
                    self._release(job)
                    ndone += 1
                    continue
                building.append(job)
            # advance builds
            still = []
            for job in building:
                if job.ev.query():
                    if job.phase == 1:
                        if not self._phase_b(job):
                            job.req.t_done = time.perf_counter()
                            self._release(job)
                            ndone += 1
                            continue
                        still.append(job)
                    else:
                        self.step_stream.wait_event(job.ev)
                        job.phase = 3
                        job.req.t_active = time.perf_counter()
                        active.append(job)
                else:
                    still.append(job)
            building = still
            # one group of S steps over every active pair
            if active:
                self.runner.upload([j.pair for j in active], [j.pair.t for j in active])
                if measure_groups:
                    e0 = torch.cuda.Event(enable_timing=True)
                    e1 = torch.cuda.Event(enable_timing=True)
                    e0.record(self.step_stream)
                self.runner.run_group()
                if measure_groups:
                    e1.record(self.step_stream)
                    nbytes = 0
                    for j in active:
                        p = j.pair
                        k = min(S, p.steps - p.t)
                        nbytes += k * (104 * p.nv + 44 * (j.nh))
                    self._timing.append((e0, e1, nbytes))
                remaining = []
                for j in active:
                    j.pair.t = min(j.pair.steps, j.pair.t + S)
                    if j.pair.done:
                        self._retire(j)
                        retiring.append(j)
                    else:
                        remaining.append(j)
                active = remaining
                self.groups += 1
            # completed retirements
            still = []
            for job in retiring:
                if job.ev.query():
                    r = job.req
                    r.t_done = time.perf_counter()
                    r.out = job.out_host if self.results_to_host else job.out_dev
                    self._release(job)
                    ndone += 1
                else:
                    still.append(job)
            retiring = still
            if not active and ndone < total:
                # nothing to step: wait briefly for a build or an arrival
                if building:
                    building[0].ev.synchronize()
                elif retiring:
                    retiring[0].ev.synchronize()
                elif future and realtime:
                    time.sleep(max(0.0, min(1e-3, future[0].arrival - (time.perf_counter() - t0))))
        torch.cuda.synchronize(self.device)
        wall = time.perf_counter() - t0
        for e0, e1, nb in self._timing:
            self.group_time_s += e0.elapsed_time(e1) * 1e-3
            self.group_bytes += nb
        self._timing = []
        return wall

    def prepare(self, requests):
        """Admit and build every request without stepping (for steady-state
        measurements of the fused step); returns the jobs."""
        for r in requests:
            fused.adam_table(max(r.steps, 1), r.lr, 0.9, 0.999, self.device)
        jobs = []
        for r in requests:
            j = _Job(r, 0)
            self._phase_a(j)
            jobs.append(j)
        torch.cuda.synchronize(self.device)
        for j in jobs:
            if not self._phase_b(j):
                raise RuntimeError("request %s failed: %s" % (j.req.id, j.req.error))
        torch.cuda.synchronize(self.device)
        return jobs

    def steady_state(self, jobs, groups=2):
        """Time `groups` step groups with every prepared pair active: returns
        (seconds per step, algorithmic bytes per step, vertices)."""
        pairs = [j.pair for j in jobs]
        if sum(p.ntiles for p in pairs) > self.runner.max_tiles:
            raise RuntimeError("too many tiles for one group")
        self.runner.upload(pairs, [0] * len(pairs))
        self.runner.run_group()  # warm-up (and graph capture)
        torch.cuda.synchronize(self.device)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(self.step_stream)
        for g in range(groups):
            self.runner.upload(pairs, [self.runner.S * (g + 1)] * len(pairs))
            self.runner.run_group()
        e1.record(self.step_stream)
        torch.cuda.synchronize(self.device)
        t = e0.elapsed_time(e1) * 1e-3 / (groups * self.runner.S)
        nbytes = sum(104 * p.nv + 44 * j.nh for p, j in zip(pairs, jobs))
        return t, nbytes, sum(p.nv for p in pairs)

    def step_roofline(self):
        """(algorithmic GB/s of the fused steps, their total seconds)."""
        if self.group_time_s <= 0:
            return 0.0, 0.0
        return self.group_bytes / self.group_time_s / 1e9, self.group_time_s


def requests_from_meshes(meshes, specs, device=None, pin=True):
    """Build Request objects from (srcV, srcF, tarV, tarF) numpy tuples and
    spec dicts (id, N, steps, arrival).  With device set, the meshes are placed
    on that device (inputs resident in HBM); else they are pinned host tensors."""
    out = []
    for (Vs, Fs, Vt, Ft), sp in zip(meshes, specs):
        ts = [torch.from_numpy(np.ascontiguousarray(a)) for a in (Vs, Fs, Vt, Ft)]
        if device is not None:
            ts = [t.to(device) for t in ts]
        elif pin:
            ts = [t.pin_memory() for t in ts]
        out.append(Request(sp["id"], *ts, N=sp["N"], steps=sp["steps"], arrival=sp.get("arrival", 0.0)))
    return out
