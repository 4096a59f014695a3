"""Small, fixed workloads for profiling single kernels with ncu.

    python -m meshode_gb300.profiling step --pairs 64 --groups 1 [--engine python]
        the first `pairs` requests of the serving stream prepared and stepped
        together by the native pool (or the Python engine): `groups` x 25
        launches of k_fused_step with every pair active (plus one warm-up
        group);
    python -m meshode_gb300.profiling df --request 1 --repeat 2 [--band] [--packet 4x2x4]
        the distance-field build of one request of the stream, `repeat` times
        (--band: with the loss-preserving band the serving builds use).

Each prints one line with the CUDA-event timing of the measured launches.
"""
import argparse
import ctypes
import sys

import torch

from . import _lib as L
from . import build as B
from . import autotune, meshgen, pool, serving


def _stream(n, seed=5):
    specs = meshgen.serving_requests(n=512, seed=seed)[:n]
    return specs, [meshgen.request_meshes(s) for s in specs]


def step(args):
    specs, meshes = _stream(args.pairs)
    dev = torch.device("cuda")
    reqs = serving.requests_from_meshes(meshes, specs, device=dev)
    for r in reqs:
        r.steps = 100000
    if args.engine == "native":
        eng = pool.NativePool(group_steps=25, results_to_host=False, max_pairs=max(len(reqs), 1))
        t, nbytes, nv = eng.steady_state(reqs, groups=args.groups)
        eng.close()
    else:
        eng = serving.ServingEngine(group_steps=25, results_to_host=False)
        t, nbytes, nv = eng.steady_state(eng.prepare(reqs), groups=args.groups)
    print("k_fused_step: %d pairs, %d vertices, %.4f ms/launch, %.1f GB/s algorithmic (104V+44H)"
          % (len(reqs), nv, t * 1e3, nbytes / t / 1e9))


def df(args):
    specs, meshes = _stream(args.request + 1)
    s = specs[args.request]
    Vs, Fs, Vt, Ft = meshes[args.request]
    dev = torch.device("cuda")
    Vd = torch.from_numpy(Vt).to(dev)
    Fd = torch.from_numpy(Ft).to(dev)
    method = {"auto": L.MO_DF_AUTO, "brute": L.MO_DF_BRUTE, "lbvh": L.MO_DF_LBVH}[args.method]
    from . import autotune
    N = s["N"]
    lib = L.lib()
    band = lib.mo_df_loss_band(N) if args.band else 0.0
    opt = L.MoDfOptions(method, autotune.PACKETS[args.packet], band)
    st = L.stream_ptr()
    bbox = torch.empty(6, dtype=torch.int32, device=dev)
    prm = torch.empty(4, dtype=torch.float64, device=dev)
    L.call("mo_bbox", L.ptr(Vd), Vd.shape[0], L.ptr(bbox), st)
    L.call("mo_norm_params", L.ptr(bbox), L.ptr(prm), st)
    nb = lib.mo_df_build_scratch_bytes(Vd.shape[0], Fd.shape[0], N, method)
    scratch = torch.empty(int(nb), dtype=torch.uint8, device=dev)
    grid = torch.empty(N ** 3, dtype=torch.float32, device=dev)
    times = []
    for _ in range(args.repeat):
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        L.call("mo_df_build_ex", L.ptr(Vd), Vd.shape[0], L.ptr(Fd), Fd.shape[0], N, L.ptr(prm),
               ctypes.byref(opt), L.ptr(scratch), nb, L.ptr(grid), None, st)
        e1.record()
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    print("df build: request %d, N=%d, %d triangles, band %.4f, packet %s, ms per build %s"
          % (args.request, N, Ft.shape[0], band, args.packet, ", ".join("%.2f" % t for t in times)))


def main(argv=None):
    ap = argparse.ArgumentParser(prog="python -m meshode_gb300.profiling")
    sub = ap.add_subparsers(dest="cmd", required=True)
    a = sub.add_parser("step")
    a.add_argument("--pairs", type=int, default=64)
    a.add_argument("--groups", type=int, default=1)
    a.add_argument("--engine", default="native", choices=["native", "python"],
                   help="the native pool (mo_pool_*) or the Python engine over the same kernels")
    b = sub.add_parser("df")
    b.add_argument("--request", type=int, default=1)
    b.add_argument("--repeat", type=int, default=2)
    b.add_argument("--method", default="auto", choices=["auto", "brute", "lbvh"])
    b.add_argument("--band", action="store_true")
    b.add_argument("--packet", default="4x4x2", choices=list(autotune.PACKETS))
    args = ap.parse_args(argv)
    B.build()
    L.require_cuda()
    {"step": step, "df": df}[args.cmd](args)


if __name__ == "__main__":
    sys.exit(main())
