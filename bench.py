#!/usr/bin/env python
"""Headline benchmark: the mixed 512-request deformation serving stream.

Workload (synthetic, seeded; the reference publishes no benchmark data):
512 requests, source vertices log-uniform in [2k, 100k] (cube-spheres),
target triangles log-uniform in [5k, 500k] (displaced cube-spheres), grid 64^3
or 128^3 (50/50), 500 Adam steps each (lr 1e-3), numpy PCG64(seed=5); each
request is one run of the reference's rigid_deform loop (normalise by the
target, build its distance field, DistanceFieldLoss + RigidEdgeLoss + Adam,
denormalise).

One bench step = the whole 512-request stream served to completion by the
continuous-batching engine, all requests offered at the start (saturating
load).  ``value`` = pair-solves/s with the meshes already resident in HBM;
``e2e`` = the same through the public API with pinned host meshes copied in
and fitted meshes copied out inside the timed region.  Also reported: p50/p95/
p99 latency under Poisson arrivals at 200 requests/s, the plain one-pair-at-
a-time GPU loop (the reference loop over the GPU pyDeform + torch.optim.Adam)
and the CPU path (the oracle restatement of pyDeform + torch CPU Adam) on
bounded samples, and the fused step's HBM roofline.

``--impl reference`` times the reference's CPU implementation of the path
(the oracle port; the reference itself cannot be built here) on the host
cores, one bounded sample of the stream per step.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402
import torch  # noqa: E402

METRIC = "pair-solves/s (batched serving, 512-request mixed stream)"
# DRAM bytes (read + write) per vertex of one k_fused_step launch, from an ncu
# capture of the kernel with 64 pairs of the stream active
# (dram__bytes_read.sum + dram__bytes_write.sum over the launch's vertices);
# the traffic grows in proportion to the vertices stepped.
TRAFFIC_BYTES_PER_VERTEX = (229.997312e6 + 44.046080e6) / 1638986
UNIT = "pair-solves/s"
WORKLOAD = "serving-stream-512 (V logU[2k,100k], T logU[5k,500k], N 64|128, 500 steps)"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--requests", type=int, default=512)
    ap.add_argument("--req-steps", type=int, default=500)
    ap.add_argument("--group-steps", type=int, default=10)
    ap.add_argument("--plain-sample", type=int, default=6)
    ap.add_argument("--cpu-sample-s", type=float, default=20.0)
    ap.add_argument("--no-extras", action="store_true", help="skip latency/plain/cpu legs")
    ap.add_argument("--no-autotune", action="store_true", help="fixed kernel choices instead of tuned ones")
    ap.add_argument("--step-grid", type=int, default=0, help="CTAs per fused-step launch (0: all resident)")
    ap.add_argument("--df-mode", default="full", choices=["on-demand", "full"],
                    help="grids filled cell by cell as vertices reach them, or built whole at admission")
    ap.add_argument("--build-streams", type=int, default=6)
    ap.add_argument("--max-building", type=int, default=32)
    ap.add_argument("--engine", default="native", choices=["native", "python"],
                    help="serving loop: the C++ pool behind mo_pool_* or the Python engine")
    return ap.parse_args()


# ---------------------------------------------------------------------------
# distributed plumbing (replicas: each rank serves its own stream)
# ---------------------------------------------------------------------------
def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    elif torch.cuda.is_available():
        torch.cuda.set_device(0)
    return world, rank


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world):
    if world <= 1:
        return x
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------------------
# clocks sampled with nvidia-smi during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.fh.close()
        sm, smax, power, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax.append(float(p[2]))
                power.append(float(p[3]))
            except ValueError:
                continue
            for name, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        os.unlink(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)), "power_w_max": float(max(power)),
                "samples": len(sm), "reasons": sorted(reasons)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        d = json.load(open(path))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ---------------------------------------------------------------------------
# workload
# ---------------------------------------------------------------------------
def make_stream(args, seed):
    from meshode_gb300 import meshgen
    specs = meshgen.serving_requests(n=args.requests, seed=seed, steps=args.req_steps)
    meshes = [meshgen.request_meshes(s) for s in specs]
    return specs, meshes


def cpu_strata(specs):
    """The stream's requests grouped for the CPU baseline: grid size (64,
    128) x source vertices (the stream's terciles) x target triangles (below
    / above the stream's median): 12 strata, {key: [request ids]}."""
    nv = np.array([s["nv"] for s in specs], np.float64)
    nt = np.array([s["nt"] for s in specs], np.float64)
    v_edges = np.quantile(nv, [1.0 / 3.0, 2.0 / 3.0])
    t_med = float(np.median(nt))
    out = {}
    for i, s in enumerate(specs):
        key = (int(s["N"]), int(np.searchsorted(v_edges, nv[i], side="right")), int(nt[i] > t_med))
        out.setdefault(key, []).append(i)
    return out


def cpu_sample_ids(specs, seed=7):
    """One seeded request from every stratum (cpu_strata), in stratum order."""
    rng = np.random.Generator(np.random.PCG64(seed))
    strata = cpu_strata(specs)
    return [int(rng.choice(strata[k])) for k in sorted(strata)]


def stream_mean_seconds(specs, seconds):
    """Stream-weighted mean CPU seconds per request from per-request times
    {id: [s, ...]} of sampled requests: each stratum's mean, weighted by its
    share of the stream's requests (a stratum with no timed request takes the
    mean of the timed ones)."""
    strata = cpu_strata(specs)
    timed = {i: float(np.mean(v)) for i, v in seconds.items() if v}
    overall = float(np.mean(list(timed.values())))
    est = 0.0
    for ids in strata.values():
        t = [timed[i] for i in ids if i in timed]
        est += len(ids) / len(specs) * (float(np.mean(t)) if t else overall)
    return est


def cpu_request_model(specs, meshes, i, threads, loop_steps=50, voxel_stride=1):
    """CPU seconds of one request on the oracle port, measured in two parts
    and scaled: the FP64 distance-field build (its serial AABB-tree build
    timed whole; its voxel queries on every voxel_stride-th z-slab, from a
    per-request offset, scaled to all N^3 voxels) and loop_steps of the
    rigid_deform loop (the restated pyDeform losses + torch.optim.Adam on the
    CPU, scaled to the request's steps; every step costs the same).  Returns
    (seconds, df seconds, loop seconds)."""
    from oracle import pydeform_oracle as orc
    torch.set_num_threads(threads)
    Vs, Fs, Vt, Ft = meshes[i]
    N = specs[i]["N"]
    sc, tr = orc.normalize_params(Vt)
    Tn = orc.normalized_double(Vt, sc, tr)
    vox = None
    if voxel_stride > 1:
        zs = np.arange(i % voxel_stride, N, voxel_stride)
        vox = (zs[:, None] * (N * N) + np.arange(N * N)[None, :]).ravel().astype(np.int64)
    grid, t_tree, t_query = orc.df_build_timed(Tn, Ft, N, voxels=vox, threads=threads)
    t_df = t_tree + t_query * (1 if vox is None else N ** 3 / vox.shape[0])
    if vox is not None:
        grid = np.zeros(N ** 3)  # the loop's speed does not depend on the values
    pid = orc.InitializeDeformTemplate(Vt, Ft, 0, N, grid=grid.astype(np.float32))
    V = torch.from_numpy(Vs.copy())
    orc.NormalizeByTemplate(V, pid)
    Ft_ = torch.from_numpy(Fs)
    orc.StoreRigidityInformation(V, Ft_, pid)
    orc.rigid_fit(V, Ft_, pid, 3)  # warm-up: the first optimiser steps of a process take ~1 s more
    t0 = time.perf_counter()
    orc.rigid_fit(V, Ft_, pid, loop_steps)
    t_loop = (time.perf_counter() - t0) * specs[i]["steps"] / loop_steps
    orc.ReleaseTemplate(pid)
    return t_df + t_loop, t_df, t_loop


def run_cpu_port(specs, meshes, ids, threads):
    """The oracle restatement of the reference's CPU path for the listed
    requests: FP64 DF through an AABB tree, then the rigid_deform loop with
    the restated pyDeform losses and torch.optim.Adam on the CPU."""
    from oracle import pydeform_oracle as orc
    torch.set_num_threads(threads)
    t0 = time.perf_counter()
    outs = []
    for i in ids:
        Vs, Fs, Vt, Ft = meshes[i]
        pid = orc.InitializeDeformTemplate(Vt, Ft, 0, specs[i]["N"])
        V = torch.from_numpy(Vs.copy())
        orc.NormalizeByTemplate(V, pid)
        Ft_ = torch.from_numpy(Fs)
        orc.StoreRigidityInformation(V, Ft_, pid)
        out, _ = orc.rigid_fit(V, Ft_, pid, specs[i]["steps"])
        outs.append(out)
        orc.ReleaseTemplate(pid)
    return time.perf_counter() - t0, outs


def run_plain_gpu(specs, meshes, ids):
    """The reference's loop verbatim (rigid_deform.py:25-41) over the GPU
    pyDeform, one pair at a time, torch.optim.Adam on CUDA."""
    from meshode_gb300 import layers
    dev = torch.device("cuda")

    def fit(i, steps):
        Vs, Fs, Vt, Ft = meshes[i]
        src_V = torch.from_numpy(Vs).to(dev)
        src_F = torch.from_numpy(Fs).to(dev)
        layer = layers.RigidLossLayer(src_V, src_F, torch.from_numpy(Vt).to(dev), torch.from_numpy(Ft).to(dev),
                                      grid_resolution=specs[i]["N"])
        P = torch.nn.Parameter(src_V)
        opt = torch.optim.Adam([P], lr=1e-3)
        for _ in range(steps):
            opt.zero_grad()
            loss = layer(P, src_F)
            loss.backward()
            opt.step()
        return P.detach().clone()

    # untimed warm-up: the first use of torch's optimiser kernels in a fresh
    # process can take seconds (library pages read from disk)
    fit(ids[0], 3)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    outs = [fit(i, specs[i]["steps"]) for i in ids]
    torch.cuda.synchronize()
    return time.perf_counter() - t0, outs


def df_build_times(specs, meshes, ids):
    """Warm, isolated DF builds (bbox, normalisation, LBVH/brute build, cell
    relayout) of the listed requests: CUDA-event ms each."""
    from meshode_gb300 import pyDeform as PD
    dev = torch.device("cuda")
    out = []
    for i in ids:
        Vs, Fs, Vt, Ft = meshes[i]
        Vd, Fd = torch.from_numpy(Vt).to(dev), torch.from_numpy(Ft).to(dev)
        PD.ReleaseTemplate(PD.InitializeDeformTemplate(Vd, Fd, 0, specs[i]["N"]))
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        pid = PD.InitializeDeformTemplate(Vd, Fd, 0, specs[i]["N"])
        e1.record()
        torch.cuda.synchronize()
        PD.ReleaseTemplate(pid)
        out.append((specs[i]["N"], Ft.shape[0], e0.elapsed_time(e1)))
    return out


# FP32 operations of one warp-lane evaluation in the traversal
# (mo_df_trav.cuh): a child's oriented-box distance (obb_d2: 3 subtractions,
# three 3-term dot products with fused multiply-adds, 3 subtractions, 3
# squares and 2 additions = 26, FMA = 2) and a full point-triangle test
# (tri_d2, non-degenerate path: 55; a test cut short by the plane-distance
# cull costs 9).  A node visit evaluates both children's boxes.
BOX_FLOPS = 26
TRI_FLOPS = 55


def df_roofline(specs, meshes, ids, tuner, sm_mhz):
    """The DF traversal of the stream's builds against the FP32 SIMT peak:
    for each listed request, the build as the serving pool runs it (the
    loss-preserving band, the tuned method and packet shape), its node
    visits and point-triangle tests counted per voxel by one counting build
    (mo_df_build_count, untimed), and its time with CUDA events (warm); the
    walk's time is the build's minus the tree-only build's (mo_df_tree_build).
    FLOPs = visits * 2 * BOX_FLOPS + tests * TRI_FLOPS (an upper bound on the
    tests' share: culled tests cost less)."""
    import ctypes
    from meshode_gb300 import _lib as L
    from meshode_gb300._lib import call, ptr, stream_ptr
    dev = torch.device("cuda")
    lib = L.lib()
    s = stream_ptr()
    tot = {"visits": 0, "tests": 0, "build_ms": 0.0, "tree_ms": 0.0, "voxels": 0}
    rows = []
    for i in ids:
        _, _, Vt, Ft = meshes[i]
        N = specs[i]["N"]
        Vd, Fd = torch.from_numpy(Vt).to(dev), torch.from_numpy(Ft).to(dev)
        bbox = torch.empty(6, dtype=torch.int32, device=dev)
        prm = torch.empty(4, dtype=torch.float64, device=dev)
        call("mo_bbox", ptr(Vd), Vd.shape[0], ptr(bbox), s)
        call("mo_norm_params", ptr(bbox), ptr(prm), s)
        method, packet = tuner.df_options(N, Fd.shape[0]) if tuner is not None else (L.MO_DF_AUTO, 0)
        if method == L.MO_DF_AUTO:
            method = lib.mo_df_method_for(Fd.shape[0], N)
        opt = L.MoDfOptions(method, packet, lib.mo_df_loss_band(N))
        nb = lib.mo_df_build_scratch_bytes(Vd.shape[0], Fd.shape[0], N, method)
        scratch = torch.empty(int(nb), dtype=torch.uint8, device=dev)
        grid = torch.empty(N ** 3, dtype=torch.float32, device=dev)
        counts = torch.zeros(2, dtype=torch.int64, device=dev)
        args = (ptr(Vd), Vd.shape[0], ptr(Fd), Fd.shape[0], N, ptr(prm), ctypes.byref(opt), ptr(scratch), nb,
                ptr(grid), None)
        call("mo_df_build_count", *args, ptr(counts), s)
        call("mo_df_build_ex", *args, s)
        ms, _ = _gpu_ms(lambda: call("mo_df_build_ex", *args, s))
        tree_ms = 0.0
        if method == L.MO_DF_LBVH:
            tb = lib.mo_df_tree_bytes(Fd.shape[0])
            tsb = lib.mo_df_tree_scratch_bytes(Vd.shape[0], Fd.shape[0])
            tree = torch.empty(int(tb), dtype=torch.uint8, device=dev)
            tscr = torch.empty(int(tsb), dtype=torch.uint8, device=dev)
            st = torch.zeros(1, dtype=torch.int32, device=dev)
            targs = (ptr(Vd), Vd.shape[0], ptr(Fd), Fd.shape[0], ptr(prm), ptr(tscr), tsb, ptr(tree), ptr(st), s)
            call("mo_df_tree_build", *targs)
            tree_ms, _ = _gpu_ms(lambda: call("mo_df_tree_build", *targs))
        c = counts.cpu().tolist()
        tot["visits"] += c[0]
        tot["tests"] += c[1]
        tot["build_ms"] += ms
        tot["tree_ms"] += tree_ms
        tot["voxels"] += N ** 3
        rows.append({"request": i, "N": N, "tris": int(Fd.shape[0]), "method": int(method), "packet": int(packet),
                     "build_ms": round(ms, 4), "tree_ms": round(tree_ms, 4), "node_visits": c[0], "tri_tests": c[1]})
    walk_s = (tot["build_ms"] - tot["tree_ms"]) * 1e-3
    flops = tot["visits"] * 2 * BOX_FLOPS + tot["tests"] * TRI_FLOPS
    peak = 152 * 128 * 2 * sm_mhz * 1e6
    return {"kernel": "k_df_lbvh / k_df_lbvh2 / k_df_brute (the nearest-triangle walk of each build)",
            "builds": len(ids), "voxels": tot["voxels"], "build_ms_total": tot["build_ms"],
            "tree_ms_total": tot["tree_ms"], "walk_ms_total": walk_s * 1e3,
            "node_visits_per_voxel": tot["visits"] / tot["voxels"], "tri_tests_per_voxel": tot["tests"] / tot["voxels"],
            "box_tests_per_s": 2 * tot["visits"] / walk_s, "tri_tests_per_s": tot["tests"] / walk_s,
            "fp32_flops_per_s": flops / walk_s, "fp32_peak_flops_per_s": peak, "fp32_frac": flops / walk_s / peak,
            "peak_note": "152 SMs x 128 FP32 lanes x 2 (FMA) x %.0f MHz (median SM clock sampled in the timed "
                         "region)" % sm_mhz,
            "flops_note": "visits x 2 x %d + tests x %d per voxel lane (an upper bound)" % (BOX_FLOPS, TRI_FLOPS),
            "per_build": rows}


def df_brute_roofline(sm_mhz):
    """The brute-force DF build (k_df_brute: every voxel against every
    triangle, triangles staged through shared memory) on the ico-5 workload's
    target (20,480 triangles) at 64^3, exact grid (no band): point-triangle
    pair tests per second against the FP32 SIMT peak, beside the LBVH build
    of the same grid (the method the library picks at this size)."""
    import ctypes
    from meshode_gb300 import _lib as L, meshgen
    from meshode_gb300._lib import call, ptr, stream_ptr
    dev = torch.device("cuda")
    lib = L.lib()
    s = stream_ptr()
    _, _, Vt, Ft = meshgen.rigid_pair_ico5(seed=1)
    N = 64
    Vd, Fd = torch.from_numpy(Vt).to(dev), torch.from_numpy(Ft).to(dev)
    bbox = torch.empty(6, dtype=torch.int32, device=dev)
    prm = torch.empty(4, dtype=torch.float64, device=dev)
    call("mo_bbox", ptr(Vd), Vd.shape[0], ptr(bbox), s)
    call("mo_norm_params", ptr(bbox), ptr(prm), s)
    out = {}
    grids = {}
    for name, method in (("brute", L.MO_DF_BRUTE), ("lbvh", L.MO_DF_LBVH)):
        opt = L.MoDfOptions(method, L.MO_PACKET_4x4x2, 0.0)
        nb = lib.mo_df_build_scratch_bytes(Vd.shape[0], Fd.shape[0], N, method)
        scratch = torch.empty(int(nb), dtype=torch.uint8, device=dev)
        grid = torch.empty(N ** 3, dtype=torch.float32, device=dev)
        args = (ptr(Vd), Vd.shape[0], ptr(Fd), Fd.shape[0], N, ptr(prm), ctypes.byref(opt), ptr(scratch), nb,
                ptr(grid), None, s)
        call("mo_df_build_ex", *args)
        out[name + "_ms"], _ = _gpu_ms(lambda: call("mo_df_build_ex", *args), reps=3)
        grids[name] = grid
    tests = float(N ** 3) * Fd.shape[0]
    rate = tests / (out["brute_ms"] * 1e-3)
    peak = 152 * 128 * 2 * sm_mhz * 1e6
    out.update({"kernel": "k_df_brute", "N": N, "target_tris": int(Fd.shape[0]), "pair_tests": tests,
                "pair_tests_per_s": rate, "fp32_flops_per_s": rate * TRI_FLOPS, "fp32_peak_flops_per_s": peak,
                "fp32_frac": rate * TRI_FLOPS / peak,
                "grids_equal": bool(torch.equal(grids["brute"], grids["lbvh"])),
                "note": "whole build timed (normalisation and triangle records included, < 1%%); FLOPs = tests x "
                        "%d (a full test; the plane-distance cull makes most cheaper, so an upper bound)"
                        % TRI_FLOPS})
    return out


def large_config(threads):
    """The large-scale configuration: displaced ico-8 target (1,310,720
    triangles) at 256^3, a 200k-vertex source: DF build ms (GPU; CPU oracle
    extrapolated from a 0.2% voxel sample) and the fused step's steady state."""
    from meshode_gb300 import fused, meshgen
    from meshode_gb300 import pyDeform as PD
    from oracle import pydeform_oracle as orc  # oracle: CPU baseline only
    dev = torch.device("cuda")
    Vs, Fs, Vt, Ft = meshgen.large_pair(seed=3)
    N = 256
    Vd, Fd = torch.from_numpy(Vt).to(dev), torch.from_numpy(Ft).to(dev)
    PD.ReleaseTemplate(PD.InitializeDeformTemplate(Vd, Fd, 0, N))
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    pid = PD.InitializeDeformTemplate(Vd, Fd, 0, N)
    e1.record()
    torch.cuda.synchronize()
    gpu_ms = e0.elapsed_time(e1)
    # DF parity on a voxel sample against the FP64 oracle
    grid = PD.GetDistanceField(pid).reshape(-1)
    sc, tr = orc.normalize_params(Vt)
    Tn = orc.normalized_double(Vt, sc, tr)
    rng = np.random.Generator(np.random.PCG64(3))
    vox = rng.choice(N ** 3, size=N ** 3 // 500, replace=False).astype(np.int64)
    t0 = time.perf_counter()
    ref = orc.df_build(Tn, Ft, N, voxels=vox, method="bvh", threads=threads)
    cpu_s = time.perf_counter() - t0
    err = float(np.abs(grid[torch.from_numpy(vox).to(dev)].double().cpu().numpy() - ref).max())
    diag = float(np.linalg.norm(Tn.max(0) - Tn.min(0)))
    # fused step on the 200k-vertex source
    V = torch.from_numpy(Vs.copy()).to(dev)
    PD.NormalizeByTemplate(V, pid)
    PD.StoreRigidityInformation(V, torch.from_numpy(Fs).to(dev), pid)
    pr = fused.pair_from_template(pid, V, steps=100000)
    runner = fused.StepGroupRunner(dev, 1, pr.ntiles, group_steps=25)
    runner.upload([pr], [0])
    runner.run_group()
    torch.cuda.synchronize()
    e0.record()
    for g in range(4):
        runner.upload([pr], [25 * (g + 1)])
        runner.run_group()
    e1.record()
    torch.cuda.synchronize()
    step_ms = e0.elapsed_time(e1) / 100
    nh = 3 * Fs.shape[0]
    nbytes = 104 * pr.nv + 44 * nh
    PD.ReleaseTemplate(pid)
    return {"target_tris": int(Ft.shape[0]), "N": N, "source_vertices": int(Vs.shape[0]), "half_edges": nh,
            "df_build_ms": gpu_ms,
            "df_max_abs_err_over_diag_vs_fp64": err / diag, "df_check_voxels": int(vox.shape[0]),
            "cpu_df_build_ms_extrapolated": cpu_s * 1e3 * (N ** 3 / vox.shape[0]), "cpu_threads": threads,
            "step_ms": step_ms, "step_algorithmic_gbs": nbytes / (step_ms * 1e-3) / 1e9}


def _gpu_ms(fn, reps=1):
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        out = fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps, out


def pair_config(name, Vs, Fs, Vt, Ft, N, steps, graph=None, threads=1, cpu_steps=100):
    """One deformation pair measured five ways: the GPU DF build (warm), the
    plain GPU loop (the reference's loop over the GPU layers, torch Adam on
    CUDA), the fused loop, the CPU oracle loop at one thread and at all
    threads (cpu_steps steps, per-step time), and the final Chamfer of each
    fit against the CPU oracle loop run to the same step count.  graph =
    (E, rigidity) selects the CAD loss (GraphLossLayer semantics: edge
    weight rigidity^2, DF gradient masked where d >= 0.03)."""
    from meshode_gb300 import fused, layers, metrics
    from meshode_gb300 import pyDeform as PD
    from oracle import pydeform_oracle as orc  # oracle: CPU baseline and Chamfer reference
    dev = torch.device("cuda")
    Vtd, Ftd = torch.from_numpy(Vt).to(dev), torch.from_numpy(Ft).to(dev)
    PD.ReleaseTemplate(PD.InitializeDeformTemplate(Vtd, Ftd, 0, N))
    df_ms, pid = _gpu_ms(lambda: PD.InitializeDeformTemplate(Vtd, Ftd, 0, N))
    src = torch.from_numpy(Vs.copy()).to(dev)
    Fd = torch.from_numpy(Fs).to(dev)
    if graph is None:
        layer = layers.RigidLossLayer(src, Fd, Vtd, Ftd, grid_resolution=N)
        idx = Fd
        r2 = 1.0
        mask = None
    else:
        E, rigidity = graph
        idx = torch.from_numpy(E).to(dev)
        layer = layers.GraphLossLayer(src, idx, Vtd, Ftd, rigidity, grid_resolution=N)
        r2 = layer.rigidity2
        mask = float(np.float32(0.5 * 0.03 * 0.03))
    lid = int(layer.param_id)
    x0 = src.clone()  # normalised by the layer
    P = torch.nn.Parameter(src)
    opt = torch.optim.Adam([P], lr=1e-3)

    def plain(k):
        for _ in range(k):
            opt.zero_grad()
            layer(P, idx).backward()
            opt.step()

    plain(3)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    plain(steps - 3)
    torch.cuda.synchronize()
    plain_ms = (time.perf_counter() - t0) * 1e3 / (steps - 3)
    # warm-up fit: the process's first graph capture and launches cost ~0.9 s once
    fused.fused_fit(lid, x0, 50, w_edge=r2, mask_thresh=mask)
    fused_ms, (out, _) = _gpu_ms(lambda: fused.fused_fit(lid, x0, steps, w_edge=r2, mask_thresh=mask))
    # CPU oracle loop: same normalised source, the GPU grid
    opid = orc.InitializeDeformTemplate(Vt, Ft, 0, N, grid=PD.GetDistanceField(lid).cpu().numpy())
    xc = x0.cpu()
    if graph is None:
        orc.StoreRigidityInformation(xc, torch.from_numpy(Fs), opid)
        fit = lambda k, th: orc.rigid_fit(xc, torch.from_numpy(Fs), opid, k, threads=th)[0]  # noqa: E731
    else:
        Et = torch.from_numpy(graph[0])
        orc.StoreGraphInformation(xc, Et, opid)

        def fit(k, th):
            torch.set_num_threads(th)
            return orc.graph_fit(xc, Et, opid, k, r2)
    cpu = {}
    for label, th in (("one_thread", 1), ("all_threads", threads)):
        fit(3, th)
        t0 = time.perf_counter()
        fit(cpu_steps, th)
        cpu[label] = {"ms_per_step": (time.perf_counter() - t0) * 1e3 / cpu_steps, "cores": th}
    ref = fit(steps, threads)
    torch.set_num_threads(threads)
    sc, tr = orc.normalize_params(Vt)
    Tn = orc.normalized_double(Vt, sc, tr)
    c_ref = metrics.chamfer(ref.numpy(), Fs, Tn, Ft, samples=20000)
    c_plain = metrics.chamfer(P.detach().cpu().numpy(), Fs, Tn, Ft, samples=20000)
    c_fused = metrics.chamfer(out.cpu().numpy(), Fs, Tn, Ft, samples=20000)
    PD.ReleaseTemplate(pid)
    PD.ReleaseTemplate(lid)
    return {"workload": name, "source_vertices": int(Vs.shape[0]), "target_tris": int(Ft.shape[0]), "N": N,
            "steps": steps, "df_build_ms": df_ms, "plain_gpu_ms_per_step": plain_ms,
            "fused_ms_per_step": fused_ms / steps, "cpu_ms_per_step": cpu,
            "chamfer": {"cpu_oracle": c_ref, "plain_gpu": c_plain, "fused": c_fused,
                        "plain_minus_cpu": c_plain - c_ref, "fused_minus_cpu": c_fused - c_ref}}


def config1(threads):
    """Plain rigid deform: ico-5 source -> displaced ico-5 target, 64^3,
    1000 Adam steps."""
    from meshode_gb300 import meshgen
    Vs, Fs, Vt, Ft = meshgen.rigid_pair_ico5(seed=1)
    return pair_config("ico5 -> displaced ico5, 64^3, lambda 1", Vs, Fs, Vt, Ft, 64, 1000, threads=threads)


def config2(threads):
    """CAD-style non-watertight deform: 40 seeded boxes and cylinders against
    their jittered copies plus a 2k-triangle noisy plane, 128^3, rigidity 1,
    the source resampled to 5000+ vertices, 1000 steps."""
    from meshode_gb300 import meshgen, meshops
    Vs, Fs, Vt, Ft = meshgen.cad_pair(seed=2)
    Vs, Fs = meshops.subdivide_to(Vs, Fs, 5000)
    Vs, Fs = Vs.astype(np.float32), Fs.astype(np.int32)
    E = meshgen.edges_from_faces(Fs)
    return pair_config("CAD 40 primitives + plane, 128^3, rigidity 1, MESH_RESOLUTION 5000", Vs, Fs, Vt, Ft, 128,
                       1000, graph=(E, 1.0), threads=threads)


def reverse_config():
    """The reverse (target -> source) nearest-point loss of inverse_deform.py
    and cad_deform2.py, forward + backward per call: the GPU layer against the
    reference's CPU path (cKDTree with 4 query threads, as its n_jobs=4, and
    torch CPU autograd), at three sizes of a displaced-sphere pair.  The
    indices are checked equal and the gradients bit-identical on the way."""
    import time as _t
    from meshode_gb300 import layers, meshgen
    out = []
    for n in (10_000, 50_000, 200_000):
        rng = np.random.Generator(np.random.PCG64(n))
        Vs, _ = meshgen.cubesphere_for_vertices(n)
        Vt, _ = meshgen.cubesphere_for_vertices(n)
        Vt = meshgen.displace(Vt, rng)
        S = torch.from_numpy((Vs * 0.9).astype(np.float32))
        T = torch.from_numpy(Vt.astype(np.float32))
        Sg = S.cuda().requires_grad_(True)
        Tg = T.cuda()
        lay = layers.ReverseLossLayer()
        for _ in range(3):
            Sg.grad = None
            lay(Sg, Tg).backward()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        reps = 10
        e0.record()
        for _ in range(reps):
            Sg.grad = None
            lay(Sg, Tg).backward()
        e1.record()
        torch.cuda.synchronize()
        gpu_ms = e0.elapsed_time(e1) / reps
        Sc = S.clone().requires_grad_(True)
        from scipy.spatial import cKDTree
        t0 = _t.perf_counter()
        tree = cKDTree(Sc.detach().numpy())
        _, ii = tree.query(T.numpy(), k=1, workers=4)
        lc = Sc[torch.from_numpy(ii)] - T
        (0.5 * (lc * lc).sum()).backward()
        cpu_ms = (_t.perf_counter() - t0) * 1e3
        # the gradient's definition: per source vertex, the matched rows
        # (g*l + g*l, g = 0.5) added from zero in target order -- torch's CPU
        # index_put_ accumulation on x86; other builds may associate a vertex
        # with three or more matches differently
        l = (S.numpy()[ii] - T.numpy()).astype(np.float32)
        gl = (np.float32(0.5) * l).astype(np.float32)
        serial = np.zeros(S.shape, np.float32)
        np.add.at(serial, ii, (gl + gl).astype(np.float32))
        ours = Sg.grad.cpu()
        out.append({"source_vertices": int(S.shape[0]), "target_vertices": int(T.shape[0]),
                    "gpu_ms_fwd_bwd": gpu_ms, "cpu_ms_fwd_bwd": cpu_ms, "cpu_threads": 4,
                    "grad_bitexact_vs_serial_sum": bool(np.array_equal(ours.numpy(), serial)),
                    "grad_rows_differing_from_this_torch": int((ours != Sc.grad).any(1).sum())})
    return out


def solve_linear_config():
    """SolveLinear's LinearEstimation (the CAD pipeline's final propagation,
    graph_loss_layer.py:62-66) on a 40,962-vertex mesh with 1,000+ graph
    cells, 200 extra edges, rigidity 1: the GPU conjugate-gradient solve
    against the oracle's direct sparse solve (CPU, double) of the same
    system, with their largest difference."""
    import time as _t
    from meshode_gb300 import meshgen
    from meshode_gb300 import pyDeform as PD
    from oracle import pydeform_oracle as orc  # oracle: the CPU path
    rng = np.random.Generator(np.random.PCG64(11))
    V, F = meshgen.icosphere(6)
    V = (0.4 * V + 0.5).astype(np.float32)
    key = np.floor(V / 0.06).astype(np.int64)
    _, ref = np.unique(key[:, 0] * 10000 + key[:, 1] * 100 + key[:, 2], return_inverse=True)
    ng = int(ref.max()) + 1
    cent = np.zeros((ng, 3))
    np.add.at(cent, ref, V)
    cent /= np.bincount(ref, minlength=ng)[:, None]
    G = ((cent - 0.5) * 1.1 + 0.5 + 0.005 * rng.standard_normal(cent.shape)).astype(np.float32)
    i = rng.integers(0, len(V), 200)
    j = (i + 1) % len(V)
    E = np.stack([i, j], 1).astype(np.int32)
    args = (torch.from_numpy(F.astype(np.int32)), torch.from_numpy(E), torch.from_numpy(ref.astype(np.int32)),
            torch.from_numpy(G), 1.0, 0)
    Vt = torch.from_numpy(V.copy()).cuda()
    PD.SolveLinear(Vt, *args)  # warm-up
    Vt = torch.from_numpy(V.copy()).cuda()
    torch.cuda.synchronize()
    t0 = _t.perf_counter()
    it, res = PD.SolveLinear(Vt, *args)
    gpu_ms = (_t.perf_counter() - t0) * 1e3
    t0 = _t.perf_counter()
    X = orc.solve_linear(V, F, E, ref, G, 1.0, 0)
    cpu_ms = (_t.perf_counter() - t0) * 1e3
    diag = float(np.linalg.norm(V.max(0) - V.min(0)))
    return {"vertices": int(len(V)), "graph_cells": ng, "cg_iterations": int(it), "rel_residual": float(res),
            "gpu_ms": gpu_ms, "oracle_direct_solve_ms": cpu_ms,
            "max_abs_diff_over_diag": float(np.abs(Vt.cpu().numpy() - X).max() / diag),
            "note": "GPU: Jacobi-PCG in double to relative residual 1e-13 (wall time incl. set-up); "
                    "oracle: assembly in numpy + scipy spsolve, single thread"}


def ode_config():
    """The velocity-field ODE configuration: 50k-vertex source, MLP
    3->256->256->256->3 (softplus, Xavier seed 4), 20 RK4 steps, 128^3 grid,
    rigidity 0.1: ms per optimiser iteration (forward flow + fit loss +
    checkpointed adjoint + Adam) against torch autograd through the same
    fp32 model (all activations stored)."""
    from meshode_gb300 import meshgen, neuralode
    rng = np.random.Generator(np.random.PCG64(4))
    Vs, Fs = meshgen.cubesphere_for_vertices(50_000)
    Vt, Ft = meshgen.icosphere(6)
    Vt = meshgen.displace(Vt, rng)
    src_V = torch.from_numpy((Vs * 0.8).astype(np.float32))
    dfm = neuralode.NeuralODEDeformer(src_V, torch.from_numpy(Fs.astype(np.int32)),
                                      torch.from_numpy(Vt.astype(np.float32)), torch.from_numpy(Ft.astype(np.int32)),
                                      grid_resolution=128, rigidity=0.1, hidden=256, steps=20, seed=4)
    for _ in range(2):
        dfm.step()
    torch.cuda.synchronize()
    base = torch.cuda.memory_allocated()
    torch.cuda.reset_peak_memory_stats()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(3):
        dfm.step()
    e1.record()
    torch.cuda.synchronize()
    ours = e0.elapsed_time(e1) / 3
    ours_mem = torch.cuda.max_memory_allocated() - base
    # torch autograd through the same model (stores every activation)
    W = [p.detach().clone().requires_grad_(True) for p in dfm.params]
    sp = torch.nn.functional.softplus

    def f(x):
        return sp(sp(sp(x @ W[0].t() + W[1]) @ W[2].t() + W[3]) @ W[4].t() + W[5]) @ W[6].t() + W[7]

    def torch_iter():
        x = dfm.x0
        hh = 1.0 / 20
        for _ in range(20):
            k1 = f(x)
            k2 = f(x + hh / 2 * k1)
            k3 = f(x + hh / 2 * k2)
            k4 = f(x + hh * k3)
            x = x + hh / 6 * (k1 + 2 * k2 + 2 * k3 + k4)
        neuralode.FitLossFunction.apply(x, dfm.F, dfm.pid, dfm.rigidity2).backward()

    torch_iter()
    torch.cuda.synchronize()
    base = torch.cuda.memory_allocated()
    torch.cuda.reset_peak_memory_stats()
    e0.record()
    for _ in range(3):
        torch_iter()
    e1.record()
    torch.cuda.synchronize()
    plain = e0.elapsed_time(e1) / 3
    plain_mem = torch.cuda.max_memory_allocated() - base
    # the same fit keeping every stage's activations (no recompute)
    dfm.store_activations = True
    dfm.step()
    torch.cuda.synchronize()
    base = torch.cuda.memory_allocated()
    torch.cuda.reset_peak_memory_stats()
    e0.record()
    for _ in range(3):
        dfm.step()
    e1.record()
    torch.cuda.synchronize()
    stored = e0.elapsed_time(e1) / 3
    stored_mem = torch.cuda.max_memory_allocated() - base
    n = dfm.x0.shape[0]
    eval_flops = 2 * n * (3 * 256 + 2 * 256 * 256 + 256 * 3)
    # 80 evaluations forward, 80 recomputed and 80 back-propagated (~2x) in the adjoint
    flops = eval_flops * (80 + 80 + 2 * 80)
    return {"source_vertices": n, "hidden": 256, "rk4_steps": 20, "N": 128,
            "ms_per_iteration": ours, "peak_extra_mem_gb": ours_mem / 1e9,
            "stored_activations_ms_per_iteration": stored, "stored_activations_peak_extra_mem_gb": stored_mem / 1e9,
            "torch_autograd_ms_per_iteration": plain, "torch_autograd_peak_extra_mem_gb": plain_mem / 1e9,
            "tflops": flops / (ours * 1e-3) / 1e12,
            "fp32_peak_tflops": 152 * 128 * 2 * 2.07e9 / 1e12,
            "kernels": "mo_mlp_fwd (fused 4-layer evaluation + RK4 update per 64-vertex tile), mo_mlp_bwd "
                       "(fused vector-Jacobian product), mo_mlp_wgrad (split-K 256x256 weight gradients): "
                       "FP32 SIMT with packed FFMA2, no library GEMM",
            "note": "checkpointed adjoint: recomputes each RK4 step's activations (4/3 of the FLOPs) to hold "
                    "one step's activations instead of all 80 stage evaluations'; stored_activations: the same "
                    "fit keeping them (same gradients bit for bit); torch_autograd: the same fp32 model through "
                    "torch (cuBLAS) autograd, every activation stored"}


# ---------------------------------------------------------------------------
REF_VOXEL_STRIDE = 4  # the reference arm's DF queries: every 4th z-slab, scaled


def reference_arm(args, world, rank):
    """CPU implementation of the path (oracle port), all host threads.  Each
    step is one bounded pass over the stratified sample, one seeded request
    of every stratum: each request's cost from cpu_request_model (its FP64
    DF build, the tree whole and the voxel queries on every
    REF_VOXEL_STRIDE-th z-slab scaled to the grid, plus 50 of its Adam steps
    scaled to all of them); value = 1 / the stream-weighted mean seconds per
    request over all steps, so every step already covers every stratum."""
    if rank != 0:
        return
    specs, meshes = make_stream(argparse.Namespace(requests=args.requests, req_steps=args.req_steps), 5)
    ids = cpu_sample_ids(specs)
    threads = os.cpu_count() or 1
    from oracle import build as ob
    ob.build()
    cheapest = min(ids, key=lambda i: specs[i]["nv"])
    for _ in range(args.warmup):
        run_cpu_port(specs, meshes, [cheapest], threads)
    per = {i: [] for i in ids}
    times = []
    for k in range(args.steps):
        t0 = time.perf_counter()
        for i in ids:
            tot, _, _ = cpu_request_model(specs, meshes, i, threads, voxel_stride=REF_VOXEL_STRIDE)
            per[i].append(tot)
        times.append(time.perf_counter() - t0)
    torch.set_num_threads(threads)
    est = stream_mean_seconds(specs, per)
    value = 1.0 / est
    sample = ("every step one bounded pass over one seeded request of each of %d strata (grid 64|128 x "
              "source-vertex tercile x target-triangle half): each request's FP64 DF build (tree whole, voxel "
              "queries on every %dth z-slab scaled to the grid) and 50 of its %d Adam steps (scaled); value = 1 / "
              "the stream-weighted mean seconds per request" % (len(ids), REF_VOXEL_STRIDE, args.req_steps))
    print(json.dumps({
        "metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": float(np.mean(times)) * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "sample": sample},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "per_request_s": {str(i): [round(t, 4) for t in v] for i, v in per.items() if v},
        "stream_mean_s_per_request": est,
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def cpu_baseline_model(specs, meshes, threads):
    """The ours-arm CPU baseline on the same stratified sample as the
    reference arm, bounded: every sampled request's cost from
    cpu_request_model, at all host threads and at one thread (the
    reference's serial pyDeform; its DF queries on every 16th z-slab)."""
    ids = cpu_sample_ids(specs)
    out = {}
    for label, th, stride in (("all_threads", threads, 1), ("one_thread", 1, 16)):
        per = {}
        parts = {}
        t0 = time.perf_counter()
        for i in ids:
            tot, tdf, tloop = cpu_request_model(specs, meshes, i, th, voxel_stride=stride)
            per[i] = [tot]
            parts[str(i)] = {"s": round(tot, 4), "df_s": round(tdf, 4), "loop_s": round(tloop, 4)}
        est = stream_mean_seconds(specs, per)
        out[label] = {"value": 1.0 / est, "unit": UNIT, "cores": th, "stream_mean_s_per_request": est,
                      "per_request": parts, "wall_s": time.perf_counter() - t0}
    torch.set_num_threads(threads)
    return ids, out


def ours_arm(args, world, rank):
    from meshode_gb300 import _lib as L
    from meshode_gb300 import metrics, serving
    from meshode_gb300 import build as B
    B.build()
    L.require_cuda()
    dev = torch.device("cuda", torch.cuda.current_device())
    specs, meshes = make_stream(args, 5 + rank)
    lib = L.lib()
    req_dev = serving.requests_from_meshes(meshes, specs, device=dev)
    req_host = serving.requests_from_meshes(meshes, specs, device=None, pin=True)
    h2d = sum(sum(a.nbytes for a in m) for m in meshes)
    d2h = sum(m[0].nbytes for m in meshes)
    torch.cuda.synchronize()

    def fresh(reqs):
        return [serving.Request(r.id, r.srcV, r.srcF, r.tarV, r.tarF, N=r.N, steps=r.steps, arrival=r.arrival)
                for r in reqs]

    # per-bucket kernel choices, tuned once before anything is timed
    from meshode_gb300 import autotune
    tuner = None if args.no_autotune else autotune.Autotuner()
    if tuner is not None:
        tuner.tune_for(req_dev)
    from meshode_gb300 import pool

    # one HBM budget for every engine of this run, fixed before any of them
    # holds memory (a native pool keeps freed blocks until trimmed; torch's
    # caching allocator keeps them for the Python engine)
    budget = int(torch.cuda.mem_get_info(dev)[0] * 0.6)

    df_mode = L.MO_DF_ON_DEMAND if args.df_mode == "on-demand" else L.MO_DF_FULL

    def make_engine(results_to_host, max_pairs=512, mode=None):
        if args.engine == "native":
            return pool.NativePool(device=dev, group_steps=args.group_steps, results_to_host=results_to_host,
                                   autotuner=tuner, max_pairs=max_pairs, hbm_budget_bytes=budget,
                                   build_streams=args.build_streams, max_building=args.max_building,
                                   step_grid=args.step_grid, df_mode=df_mode if mode is None else mode)
        return serving.ServingEngine(device=dev, group_steps=args.group_steps, results_to_host=results_to_host,
                                     autotuner=tuner, max_pairs=max_pairs, hbm_budget_bytes=budget,
                                     build_streams=args.build_streams, max_building=args.max_building)

    def fused_launches(eng):
        if args.engine == "native":
            return eng.launches  # every mo_fused_step launch, graph replays included
        return eng.runner.launches if eng.runner.use_graph else 0

    engine = make_engine(False)
    for _ in range(args.warmup):
        engine.run(fresh(req_dev))
    engine.group_time_s = engine.group_bytes = 0.0
    # ---- timed: device-resident inputs ----
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    barrier(world)
    torch.cuda.synchronize()
    n0 = lib.mo_launch_count()
    g0 = fused_launches(engine)
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record()
    last = None
    for _ in range(args.steps):
        last = fresh(req_dev)
        engine.run(last)
    ev1.record()
    torch.cuda.synchronize()
    barrier(world)
    clk = clocks.stop()
    t_dev = ev0.elapsed_time(ev1) * 1e-3
    # direct launches counted by the library, plus the fused steps replayed from graphs
    launches = (lib.mo_launch_count() - n0) + (fused_launches(engine) - g0)
    t_max = max_over_ranks(t_dev, world)
    value = world * args.requests * args.steps / t_max
    achieved, step_s = engine.step_roofline()
    # ---- timed: end to end through host buffers ----
    if args.engine == "native":
        engine.trim()
    engine_h = make_engine(True)
    engine_h.run(fresh(req_host))  # warm-up of this engine (graph capture)
    barrier(world)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        engine_h.run(fresh(req_host))
    e1.record()
    torch.cuda.synchronize()
    barrier(world)
    t_e2e = max_over_ranks(e0.elapsed_time(e1) * 1e-3, world)
    if args.engine == "native":
        engine_h.close()
    e2e_value = world * args.requests * args.steps / t_e2e
    if rank != 0:
        return
    extras = {}
    if not args.no_extras:
        # latency under Poisson arrivals at 200 requests/s: three runs, the
        # median one (by p99) reported, every run's p99 listed (a single run
        # can catch a host stall of tens of ms)
        runs = []
        for _ in range(3):
            lat_reqs = fresh(req_dev)
            engine.run(lat_reqs, realtime=True)
            lats = np.asarray([r.latency for r in lat_reqs]) * 1e3
            runs.append([float(np.percentile(lats, q)) for q in (50, 95, 99)])
        runs.sort(key=lambda x: x[2])
        p50, p95, p99 = runs[1]
        extras["latency_ms"] = {"p50": p50, "p95": p95, "p99": p99, "arrivals": "poisson 200 req/s",
                                "runs_p99": [r[2] for r in runs], "reported": "median of 3 runs by p99"}
        extras["saturated_latency_ms_p99"] = float(np.percentile(
            np.asarray([r.latency for r in last]) * 1e3, 99))
        if args.engine == "native" and df_mode == L.MO_DF_ON_DEMAND:
            # the same stream with every grid built whole at admission: its
            # throughput, and the results compared bit for bit
            full_eng = make_engine(False, mode=L.MO_DF_FULL)
            full_eng.run(fresh(req_dev))
            torch.cuda.synchronize()
            f0 = torch.cuda.Event(enable_timing=True)
            f1 = torch.cuda.Event(enable_timing=True)
            f0.record()
            full_reqs = fresh(req_dev)
            full_eng.run(full_reqs)
            f1.record()
            torch.cuda.synchronize()
            full_eng.close()
            same = all(torch.equal(a.out, b.out) and a.loss == b.loss for a, b in zip(last, full_reqs))
            extras["full_grid"] = {"value": args.requests / (f0.elapsed_time(f1) * 1e-3), "unit": UNIT,
                                   "results_bitexact_vs_on_demand": bool(same),
                                   "note": "every grid built whole at admission (one timed pass)"}
        # plain one-pair-at-a-time GPU loop on a bounded sample
        ids = list(range(min(args.plain_sample, len(specs))))
        t_plain, plain_out = run_plain_gpu(specs, meshes, ids)
        plain_rate = len(ids) / t_plain
        extras["plain_gpu"] = {"value": plain_rate, "unit": UNIT, "sample": "requests %s, sequential" % ids,
                               "batched_over_plain": value / plain_rate}
        # matched Chamfer on the sample (target-normalised unit cube)
        diffs = []
        for j, i in enumerate(ids):
            Vs, Fs, Vt, Ft = meshes[i]
            from oracle import pydeform_oracle as orc  # oracle: Chamfer reference only
            sc, tr = orc.normalize_params(Vt)
            Tn = orc.normalized_double(Vt, sc, tr)
            a = last[i].out_normalized.cpu().numpy()
            b = plain_out[j].cpu().numpy()
            ca = metrics.chamfer(a, Fs, Tn, Ft, samples=20000)
            cb = metrics.chamfer(b, Fs, Tn, Ft, samples=20000)
            diffs.append(abs(ca - cb))
        extras["chamfer_vs_plain_max_abs_diff"] = float(max(diffs))
        # CPU path: the reference arm's stratified sample, bounded
        threads = os.cpu_count() or 1
        cids, cpu_model = cpu_baseline_model(specs, meshes, threads)
        cpu_rate = cpu_model["all_threads"]["value"]
        # matched Chamfer: the cheapest sampled request run whole on the CPU
        i = min(cids, key=lambda j: specs[j]["nv"])
        _, cpu_out = run_cpu_port(specs, meshes, [i], threads)
        sc, tr = orc.normalize_params(meshes[i][2])
        Tn = orc.normalized_double(meshes[i][2], sc, tr)
        c_cpu = metrics.chamfer(cpu_out[0].numpy(), meshes[i][1], Tn, meshes[i][3], samples=20000)
        c_gpu = metrics.chamfer(last[i].out_normalized.cpu().numpy(), meshes[i][1], Tn, meshes[i][3], samples=20000)
        extras["chamfer_vs_cpu_abs_diff"] = abs(c_cpu - c_gpu)
        extras["cpu_one_thread"] = cpu_model["one_thread"]
        cpu_baseline = {"value": cpu_rate, "unit": UNIT, "cores": threads, "kind": "port",
                        "sample": ("requests %s, one per stratum (grid x source-vertex tercile x target-triangle "
                                   "half) as in the reference arm; each request's FP64 DF build timed whole and "
                                   "50 of its %d Adam steps timed and scaled; value = 1 / the stream-weighted mean "
                                   "seconds per request" % (cids, args.req_steps)),
                        "per_request": cpu_model["all_threads"]["per_request"],
                        "stream_mean_s_per_request": cpu_model["all_threads"]["stream_mean_s_per_request"]}
        # DF build ms: a 48-request sample of the stream, and the large configuration
        dfs = df_build_times(specs, meshes, list(range(min(48, len(specs)))))
        by_n = {}
        for n_, t_, ms in dfs:
            by_n.setdefault(str(n_), []).append(ms)
        extras["roofline_df"] = df_roofline(specs, meshes, list(range(min(48, len(specs)))), tuner,
                                            float(clk.get("sm_mhz") or 2070.0))
        extras["df_build_ms"] = {
            "stream_sample_mean": float(np.mean([d[2] for d in dfs])),
            "by_grid": {k: {"mean": float(np.mean(v)), "p50": float(np.median(v)), "max": float(max(v)),
                            "n": len(v)} for k, v in by_n.items()},
            # B_df = 4 N^3 (grid write) + 36 T (triangle read) per build
            "algorithmic_gbs_mean": float(np.mean([(4.0 * n_ ** 3 + 36.0 * t_) / (ms * 1e-3) / 1e9
                                                   for n_, t_, ms in dfs])),
            "bytes_formula": "4*N^3 + 36*T per build (grid write + triangle read)",
            "note": "warm, one build at a time: bbox + normalisation + LBVH or brute force + cell relayout; "
                    "the builds are bound by the traversal's latency (roofline_df), not by these bytes"}
        extras["roofline_df_brute"] = df_brute_roofline(float(clk.get("sm_mhz") or 2070.0))
        extras["config1"] = config1(threads)
        extras["config2"] = config2(threads)
        extras["large_config"] = large_config(threads)
        extras["ode_config"] = ode_config()
        extras["reverse_loss"] = reverse_config()
        extras["solve_linear"] = solve_linear_config()
    else:
        cpu_baseline = None
    peak, peak_kind = measured_peaks()
    # steady state of the fused step: every request of the stream active at
    # once (long runs so no pair finishes inside the measured groups)
    ss_reqs = fresh(req_dev)
    for r in ss_reqs:
        r.steps = 100000
    # full grids here: the groups time the fused step alone, with no fills
    ss_engine = make_engine(False, max_pairs=len(ss_reqs) + 1, mode=L.MO_DF_FULL)
    if args.engine == "native":
        engine.close()
        t_ss, bytes_ss, nv_ss = ss_engine.steady_state(ss_reqs, groups=2)
        ss_engine.close()
    else:
        ss_jobs = ss_engine.prepare(ss_reqs)
        t_ss, bytes_ss, nv_ss = ss_engine.steady_state(ss_jobs, groups=2)
        del ss_jobs
    del ss_engine
    achieved_ss = bytes_ss / t_ss / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_max / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "requests": args.requests, "req_steps": args.req_steps,
                   "group_steps": args.group_steps, "parallelism": "replicas" if world > 1 else "single",
                   "engine": "mo_pool (C ABI)" if args.engine == "native" else "python",
                   "build_streams": args.build_streams, "max_building": args.max_building,
                   "step_grid": args.step_grid,
                   "df": ("on-demand cells (traversal tree at admission, a cell's corners when a vertex "
                          "first reaches it)" if df_mode == L.MO_DF_ON_DEMAND else "full grid at admission"),
                   "l2": "inputs larger than L2 (~1.3 GB meshes, ~20 GB grids per stream)"},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "roofline": {"bound": "hbm", "kernel": "k_fused_step", "achieved": achieved_ss, "peak": peak,
                     "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved_ss / peak,
                     "traffic": (TRAFFIC_BYTES_PER_VERTEX * nv_ss) if TRAFFIC_BYTES_PER_VERTEX else None,
                     # measured DRAM bytes over the launch time: the neighbour
                     # gathers the formula counts are mostly served from L1/L2
                     "traffic_gbs": TRAFFIC_BYTES_PER_VERTEX * nv_ss / t_ss / 1e9,
                     "traffic_frac": TRAFFIC_BYTES_PER_VERTEX * nv_ss / t_ss / 1e9 / peak,
                     "algorithmic_bytes_per_launch": bytes_ss, "ms_per_launch": t_ss * 1e3,
                     "launch": "all %d pairs of the stream active (%d vertices)" % (len(ss_reqs), nv_ss),
                     "bytes_formula": "104*V + 44*H per pair-step",
                     "in_serving": {"achieved": achieved, "step_seconds": step_s,
                                    "note": "same kernel timed inside the timed streams, sharing the GPU "
                                            "with the concurrent DF builds"}},
        "cpu_baseline": cpu_baseline,
        "gpu_launches": int(launches),
        "autotune": None if tuner is None else {
            "df": {k: "%s/%s" % ({1: "brute", 2: "lbvh"}.get(v["method"], v["method"]),
                                 [n for n, c in autotune.PACKETS.items() if c == v["packet"]][0])
                   for k, v in sorted(tuner.table["df"].items())},
            "step": {k: "%s/%d" % ([n for n, c in autotune.LAYOUTS.items() if c == v["layout"]][0],
                                   v["slices_per_tile"]) for k, v in sorted(tuner.table["step"].items())},
            "keys": "df: N/log2(triangles); step: N/log2(vertices)"},
        "clocks": clk,
    }
    line.update(extras)
    print(json.dumps(line))


def main():
    args = parse()
    world, rank = dist_setup(args)
    if args.impl == "reference":
        reference_arm(args, world, rank)
    else:
        ours_arm(args, world, rank)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
