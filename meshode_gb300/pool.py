"""Python face of the native serving pool (``mo_pool_*`` in libmeshode.so).

``NativePool.run`` serves a list of :class:`serving.Request` exactly like
``serving.ServingEngine.run`` -- same admission by HBM bytes, side-stream
builds, CUDA-graph groups of fused steps and retirement -- but the whole
loop (bookkeeping, table uploads, graph replays, stream-ordered allocation)
runs in C++ inside the library; Python only submits requests as they arrive
and collects finished ones.  A request's result is bit-identical to the
Python engine's and to the request run alone.
"""
import ctypes
import gc
import time

import torch

from . import _lib as L
from ._lib import check


class NativePool:
    def __init__(self, device=None, hbm_budget_bytes=None, max_pairs=512, max_tiles=None, group_steps=25,
                 layout=L.MO_LAYOUT_CELL, use_graph=True, max_building=16, results_to_host=True, build_streams=6,
                 slices_per_tile=L.MO_TILE_WARPS, autotuner=None, df_band=-1.0, step_grid=0,
                 df_mode=L.MO_DF_FULL):
        L.require_cuda()
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        self.lib = L.lib()
        self.cfg = L.MoPoolConfig(
            hbm_budget_bytes=int(hbm_budget_bytes or 0), max_pairs=int(max_pairs),
            max_tiles=int(max_tiles if max_tiles is not None else 1 << 17), group_steps=int(group_steps),
            use_graph=1 if use_graph else 0, max_building=int(max_building), build_streams=int(build_streams),
            layout=int(layout), slices_per_tile=int(slices_per_tile), step_grid=int(step_grid),
            df_mode=int(df_mode))
        # MO_DF_ON_DEMAND: grids are filled cell by cell as the vertices reach
        # them (cell layout); MO_DF_FULL: every grid is built at admission
        self.df_mode = int(df_mode)
        self.S = int(group_steps)
        self.layout = int(layout)
        self.autotuner = autotuner
        # DF band: < 0 the loss-preserving band of mo_df_loss_band, 0 exact
        self.df_band = float(df_band)
        self.results_to_host = bool(results_to_host)
        self._h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            check(self.lib.mo_pool_create(ctypes.byref(self.cfg), ctypes.byref(self._h)), "mo_pool_create")
        self.group_time_s = 0.0
        self.group_bytes = 0.0
        self._keep = {}

    # ------------------------------------------------------------------
    def close(self):
        if self._h is not None and self._h.value:
            self.lib.mo_pool_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def trim(self, keep_bytes=0):
        """Give the device memory the pool keeps for reuse back to the device."""
        check(self.lib.mo_pool_trim(self._h, int(keep_bytes)), "mo_pool_trim")

    def stats(self):
        st = L.MoPoolStats()
        check(self.lib.mo_pool_stats(self._h, ctypes.byref(st)), "mo_pool_stats")
        return st

    @property
    def launches(self):
        """Kernels of the step groups issued: mo_fused_step launches (a graph
        replay counts its S launches) and the on-demand fills after them."""
        st = self.stats()
        return int(st.fused_launches) * (1 + int(st.fill_launches_per_step))

    def fill_totals(self):
        """On-demand grids: (cells written, voxel packets computed) so far."""
        out = (ctypes.c_int64 * 2)()
        check(self.lib.mo_pool_fill_totals(self._h, out), "mo_pool_fill_totals")
        return int(out[0]), int(out[1])

    @property
    def peak_in_use(self):
        return int(self.stats().peak_bytes)

    # ------------------------------------------------------------------
    def _request(self, r):
        tensors = [r.srcV, r.srcF, r.tarV, r.tarF]
        on_dev = [t.is_cuda for t in tensors]
        if any(on_dev) and not all(on_dev):
            tensors = [t.to(self.device) for t in tensors]
            on_dev = [True] * 4
        tensors = [t.contiguous() for t in tensors]
        for t, dt in zip(tensors, (torch.float32, torch.int32, torch.float32, torch.int32)):
            if t.dtype != dt or t.dim() != 2 or t.shape[1] != 3:
                raise RuntimeError("request %s: meshes must be float32/int32 [n,3] tensors" % r.id)
        layout, spt = self.layout, 0
        method, packet = L.MO_DF_AUTO, L.MO_PACKET_4x4x2
        if self.autotuner is not None:
            method, packet = self.autotuner.df_options(r.N, int(tensors[3].shape[0]))
            layout, spt = self.autotuner.step_options(r.N, int(tensors[0].shape[0]))
        # result buffers the pool fills as the request retires
        nv = int(tensors[0].shape[0])
        if self.results_to_host:
            out = torch.empty(nv, 3, dtype=torch.float32, pin_memory=True)
        else:
            out = torch.empty(nv, 3, dtype=torch.float32, device=self.device)
        normed = torch.empty(nv, 3, dtype=torch.float32, device=self.device)
        q = L.MoRequest(
            srcV=tensors[0].data_ptr(), srcF=tensors[1].data_ptr(), tarV=tensors[2].data_ptr(),
            tarF=tensors[3].data_ptr(), nv=nv, nf=tensors[1].shape[0], ntv=tensors[2].shape[0],
            ntf=tensors[3].shape[0], inputs_on_host=0 if on_dev[0] else 1, N=r.N, steps=r.steps,
            w_edge=r.w_edge, lr=r.lr, layout=layout, slices_per_tile=spt, df_method=method, df_packet=packet,
            df_band=self.df_band, out_on_host=1 if self.results_to_host else 0, V_out=out.data_ptr(),
            V_normalized_out=normed.data_ptr())
        return q, tensors + [out, normed]

    def _submit(self, r):
        q, keep = self._request(r)
        rid = ctypes.c_int64()
        check(self.lib.mo_pool_submit(self._h, ctypes.byref(q), ctypes.byref(rid)), "mo_pool_submit")
        self._keep[rid.value] = (r, keep)
        return rid.value

    def _collect(self):
        ids = (ctypes.c_int64 * 64)()
        n = ctypes.c_int()
        st = ctypes.c_int32()
        loss = ctypes.c_double()
        done = 0
        while True:
            check(self.lib.mo_pool_completed(self._h, ids, 64, ctypes.byref(n)), "mo_pool_completed")
            for k in range(n.value):
                pid = ids[k]
                r, keep = self._keep.pop(pid)
                check(self.lib.mo_pool_state(self._h, pid, ctypes.byref(st)), "mo_pool_state")
                if st.value == L.MO_REQ_FAILED:
                    buf = ctypes.create_string_buffer(256)
                    self.lib.mo_pool_error(self._h, pid, buf, 256)
                    r.error = buf.value.decode()
                else:
                    out, normed = keep[4], keep[5]
                    check(self.lib.mo_pool_result(self._h, pid, None, None, 0, ctypes.byref(loss)),
                          "mo_pool_result")
                    r.out = out
                    r.out_normalized = normed
                    r.loss = loss.value
                r.t_done = time.perf_counter()
                check(self.lib.mo_pool_release(self._h, pid), "mo_pool_release")
                done += 1
            if n.value < 64:
                return done

    def run(self, requests, realtime=False, measure_groups=True):
        """Serve ``requests`` to completion (see ServingEngine.run); returns
        the wall time in seconds."""
        check(self.lib.mo_pool_set_timing(self._h, 1 if measure_groups else 0), "mo_pool_set_timing")
        future = sorted(requests, key=lambda r: r.arrival)
        for r in requests:
            r.out = r.out_normalized = r.error = None
        # device inputs written on torch's stream must be complete before the
        # pool's own streams read them
        torch.cuda.current_stream(self.device).synchronize()
        total = len(requests)
        nfin = ctypes.c_int64()
        # the garbage collector is held off while the loop serves: a full
        # collection over the requests' objects stalls it for tens of ms
        gc_on = gc.isenabled()
        gc.disable()
        try:
            wall = self._serve(future, total, realtime, nfin)
        finally:
            if gc_on:
                gc.enable()
        self._accumulate_groups()
        return wall

    def _serve(self, future, total, realtime, nfin):
        ndone = 0
        i = 0
        t0 = time.perf_counter()
        while ndone < total:
            now = time.perf_counter()
            while i < len(future) and (not realtime or future[i].arrival <= now - t0):
                r = future[i]
                r.t_arrive = t0 + r.arrival if realtime else t0
                r.t_admit = now
                try:
                    self._submit(r)
                except RuntimeError as e:  # rejected on the host: fail this request only
                    r.error = str(e)
                    r.t_done = time.perf_counter()
                    ndone += 1
                i += 1
            st = self.stats()
            idle = st.active == 0 and st.building == 0 and st.retiring == 0 and st.queued == 0
            if idle and i < len(future):
                time.sleep(max(0.0, min(1e-3, future[i].arrival - (time.perf_counter() - t0))))
                continue
            check(self.lib.mo_pool_progress(self._h, 1, ctypes.byref(nfin)), "mo_pool_progress")
            ndone += self._collect()
        torch.cuda.synchronize(self.device)
        return time.perf_counter() - t0

    def _accumulate_groups(self):
        ms, nb = ctypes.c_double(), ctypes.c_double()
        check(self.lib.mo_pool_group_time(self._h, ctypes.byref(ms), ctypes.byref(nb)), "mo_pool_group_time")
        self.group_time_s += ms.value * 1e-3
        self.group_bytes += nb.value

    def step_roofline(self):
        """(algorithmic GB/s of the fused steps, their total seconds)."""
        if self.group_time_s <= 0:
            return 0.0, 0.0
        return self.group_bytes / self.group_time_s / 1e9, self.group_time_s

    def steady_state(self, requests, groups=2):
        """Build every request, then time `groups` step groups with all of them
        active: returns (seconds per step, algorithmic bytes per step,
        vertices).  The requests need more than (groups+1)*S steps."""
        for r in requests:
            if r.steps <= (groups + 1) * self.S:
                raise RuntimeError("steady_state needs requests longer than %d steps" % ((groups + 1) * self.S))
        torch.cuda.current_stream(self.device).synchronize()
        check(self.lib.mo_pool_set_hold(self._h, 1), "mo_pool_set_hold")
        ids = [self._submit(r) for r in requests]
        check(self.lib.mo_pool_wait(self._h), "mo_pool_wait")
        st = self.stats()
        if st.active != len(requests):
            raise RuntimeError("steady_state: %d of %d requests active (failed %d; raise max_pairs/max_tiles?)"
                               % (st.active, len(requests), st.failed))
        check(self.lib.mo_pool_set_timing(self._h, 0), "mo_pool_set_timing")
        check(self.lib.mo_pool_run_groups(self._h, 1), "mo_pool_run_groups")  # warm-up (graph capture)
        check(self.lib.mo_pool_set_timing(self._h, 1), "mo_pool_set_timing")
        ms, nb = ctypes.c_double(), ctypes.c_double()
        check(self.lib.mo_pool_group_time(self._h, ctypes.byref(ms), ctypes.byref(nb)), "mo_pool_group_time")
        check(self.lib.mo_pool_run_groups(self._h, groups), "mo_pool_run_groups")
        check(self.lib.mo_pool_group_time(self._h, ctypes.byref(ms), ctypes.byref(nb)), "mo_pool_group_time")
        check(self.lib.mo_pool_set_hold(self._h, 0), "mo_pool_set_hold")
        steps = groups * self.S
        nv = sum(int(r.srcV.shape[0]) for r in requests)
        # the pool is left with unfinished requests: it is only good for closing
        del ids
        return ms.value * 1e-3 / steps, nb.value / steps, nv
