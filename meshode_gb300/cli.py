"""Command-line front ends with the reference's argument surface.

    python -m meshode_gb300.cli rigid_deform source.obj reference.obj output.obj \\
        [GRID_RESOLUTION=64] [MESH_RESOLUTION=5000] [lambda=1] [symmetry=0]
    python -m meshode_gb300.cli cad_deform cad.obj reference.obj output.obj \\
        [GRID_RESOLUTION=64] [MESH_RESOLUTION=5000] [lambda=1] [symmetry=0] [flow_output]
    python -m meshode_gb300.cli inverse_deform source.obj reference.obj output.obj

Positional arguments, defaults and their order follow src/app/rigid_deform.cc:
13-41 and src/app/cad_deform.cc:22-61 (with fewer than four arguments the
usage line is printed and the program exits 0, as there).  The solve is the
GPU Adam loop over the fused step instead of the reference's Ceres
Levenberg-Marquardt: same objective (0.5*sum d^2 + lambda^2 * 0.5*sum r^2,
the Ceres edge residual being lambda*(p1 - p2 - v)), ``--steps`` Adam steps at
``--lr``.  Differences, by necessity:
* rigid_deform: as the reference, MESH_RESOLUTION is parsed and unused.
* cad_deform: the reference remeshes the CAD model with CGAL and optimises a
  representative graph (subdivision.cc); here the model is cleaned like the
  reference (RemoveDegenerated, MergeDuplex), midpoint-subdivided to at least
  MESH_RESOLUTION vertices, and its mesh edges are the graph, fitted with the
  GraphLossFunction objective (rigidity = lambda, DF gradient mask d < 0.03).
  With flow_output, snapshots every ``--flow-every`` steps are written in the
  reference's flow format (cad_deform.cc:90-114).
* inverse_deform: the reference's Python script (src/python/inverse_deform.py):
  RigidLossLayer (64^3 grid) plus ReverseLossLayer, loss = 10*rigid +
  reverse, torch Adam (lr 1e-3) for up to ``--steps`` (10000) iterations,
  stopping when the loss printed every 100 iterations rises, then Finalize.
  The layers run on the GPU kernels (the reverse loss's nearest-point query
  included) and so does Adam.
"""
import argparse
import sys

import numpy as np
import torch

from . import fused, layers, meshops, objio
from . import pyDeform as PD

RIGID_USAGE = ("./rigid_deform source.obj reference.obj output.obj [GRID_RESOLUTION=64] "
               "[MESH_RESOLUTION=5000] [lambda=1] [symmetry=0]")
INVERSE_USAGE = "inverse_deform.py source.obj reference.obj output.obj"
CAD_USAGE = ("./cad_deform cad.obj reference.obj output.obj [GRID_RESOLUTION=64] [MESH_RESOLUTION=5000] "
             "[lambda=1] [symmetry=0] [flow_output=filename]")


def _positional(argv, n_min):
    """The reference's sscanf-style optional positionals (absent -> default)."""
    return argv + [None] * max(0, n_min - len(argv))


def _load(path):
    V, F = objio.read_obj(path)
    return V, F


def _fit(src_V, src_F, tar_V, tar_F, N, lam, steps, lr, graph=False, flow_every=0, log=print):
    dev = torch.device("cuda", torch.cuda.current_device())
    tV = torch.from_numpy(np.ascontiguousarray(tar_V, np.float32)).to(dev)
    tF = torch.from_numpy(np.ascontiguousarray(tar_F, np.int32)).to(dev)
    pid = PD.InitializeDeformTemplate(tV, tF, 0, N)
    V = torch.from_numpy(np.ascontiguousarray(src_V, np.float32)).to(dev)
    PD.NormalizeByTemplate(V, pid)
    F = torch.from_numpy(np.ascontiguousarray(src_F, np.int32)).to(dev)
    w = float(np.float32(lam * lam))
    if graph:
        from . import meshgen
        E = torch.from_numpy(meshgen.edges_from_faces(np.asarray(src_F))).to(dev)
        PD.StoreGraphInformation(V, E, pid)
        mask = float(np.float32(0.5 * 0.03 * 0.03))
    else:
        PD.StoreRigidityInformation(V, F, pid)
        mask = None
    pr = fused.pair_from_template(pid, V, steps, lr=lr, w_edge=w, mask_thresh=mask)
    group = 25 if not flow_every else max(1, min(25, flow_every))
    runner = fused.StepGroupRunner(dev, 1, pr.ntiles, group_steps=group)
    flow = []
    while not pr.done:
        runner.upload([pr], [pr.t])
        runner.run_group()
        n = min(runner.S, pr.steps - pr.t)
        losses = runner.pair_losses(n)[:, 0].cpu().numpy()
        for k in range(n):
            if (pr.t + k) % 100 == 0:
                log("iter=%d loss=%.6f" % (pr.t + k, losses[k]))
        pr.t += n
        if flow_every and (pr.t % flow_every == 0 or pr.done):
            snap = pr.positions()
            PD.DenormalizeByTemplate(snap, pid)
            flow.append(snap.cpu().numpy().astype(np.float64))
    out = pr.positions()
    PD.DenormalizeByTemplate(out, pid)
    PD.ReleaseTemplate(pid)
    return out.cpu().numpy().astype(np.float64), flow


def _write_flow(path, V0, flow):
    """cad_deform.cc:98-114: per vertex its snapshots as 'v' lines joined by 'l'."""
    snaps = [V0] + flow
    with open(path, "w") as fh:
        top = 1
        for i in range(V0.shape[0]):
            for s in snaps:
                fh.write("v %g %g %g\n" % tuple(s[i]))
            for j in range(len(snaps) - 1):
                fh.write("l %d %d\n" % (top + j, top + j + 1))
            top += len(snaps)


def rigid_deform(argv, steps=1000, lr=1e-3):
    if len(argv) < 4:  # argc < 5 in rigid_deform.cc:13
        print(RIGID_USAGE)
        return 0
    src, ref, out, grid, mesh_res, lam, sym = _positional(argv, 7)[:7]
    N = int(grid) if grid is not None else 64
    _ = int(mesh_res) if mesh_res is not None else 5000  # parsed, unused (rigid_deform.cc:36-37)
    lam = float(lam) if lam is not None else 1.0
    sym = int(sym) if sym is not None else 0
    sV, sF = _load(src)
    rV, rF = _load(ref)
    if sym:
        rV, rF = meshops.reflection_symmetrize(rV, rF)
    print("Source:\t\tNum vertices: %d\tNum faces: %d" % (sV.shape[0], sF.shape[0]))
    print("Reference:\tNum vertices: %d\tNum faces: %d\n" % (rV.shape[0], rF.shape[0]))
    V, _ = _fit(sV, sF, rV, rF, N, lam, steps, lr)
    print("Deformed")
    objio.write_obj(out, V, sF)
    return 0


def cad_deform(argv, steps=1000, lr=1e-3, flow_every=50):
    if len(argv) < 4:  # argc < 5 in cad_deform.cc:22
        print(CAD_USAGE)
        return 0
    cad, ref, out, grid, mesh_res, lam, sym, flow_file = _positional(argv, 8)[:8]
    N = int(grid) if grid is not None else 64
    mres = int(mesh_res) if mesh_res is not None else 5000
    lam = float(lam) if lam is not None else 1.0
    sym = int(sym) if sym is not None else 0
    cV, cF = _load(cad)
    rV, rF = _load(ref)
    if sym:
        rV, rF = meshops.reflection_symmetrize(rV, rF)
    cV, cF = meshops.remove_degenerated(cV, cF)
    cV, cF = meshops.merge_duplex(cV, cF)
    cV, cF = meshops.subdivide_to(cV, cF, mres)
    print("Source:\t\tNum vertices: %d\tNum faces: %d" % (cV.shape[0], cF.shape[0]))
    print("Reference:\tNum vertices: %d\tNum faces: %d\n" % (rV.shape[0], rF.shape[0]))
    V, flow = _fit(cV, cF, rV, rF, N, lam, steps, lr, graph=True, flow_every=flow_every if flow_file else 0)
    if flow_file:
        _write_flow(flow_file, cV, flow)
    print("Deformed")
    objio.write_obj(out, V, cF)
    return 0


def inverse_fit(src_V, src_F, tar_V, tar_F, steps=10000, lr=1e-3, log=print):
    """inverse_deform.py:17-45 on the GPU; returns the fitted source vertices
    in the source's coordinates and the iterations run."""
    dev = torch.device("cuda", torch.cuda.current_device())
    sV = torch.from_numpy(np.ascontiguousarray(src_V, np.float32)).to(dev)
    sF = torch.from_numpy(np.ascontiguousarray(src_F, np.int32)).to(dev)
    tV = torch.from_numpy(np.ascontiguousarray(tar_V, np.float32)).to(dev)
    tF = torch.from_numpy(np.ascontiguousarray(tar_F, np.int32)).to(dev)
    rigid = layers.RigidLossLayer(sV, sF, tV, tF)
    reverse = layers.ReverseLossLayer()
    pid = int(rigid.param_id)
    P = torch.nn.Parameter(sV)
    opt = torch.optim.Adam([P], lr=lr)
    PD.NormalizeByTemplate(tV, pid)
    prev = 1e30
    it = 0
    for it in range(steps):
        opt.zero_grad()
        loss_src2tar = rigid(P, sF)
        loss_tar2src = reverse(P, tV)
        loss = loss_src2tar * 10 + loss_tar2src
        loss.backward()
        opt.step()
        if it % 100 == 0:
            lv = loss.item()
            log("iter=%d loss=%.6f loss_tar2src=%.6f" % (it, lv, np.sqrt(loss_tar2src.item() / tV.shape[0])))
            if lv > prev:
                break
            prev = lv
    out = P.detach().clone()
    layers.Finalize(out, pid)
    PD.ReleaseTemplate(pid)
    return out.cpu().numpy().astype(np.float64), it + 1


def inverse_deform(argv, steps=10000, lr=1e-3):
    if len(argv) < 3:
        print(INVERSE_USAGE)
        return 0
    src, ref, out = argv[:3]
    sV, sF = _load(src)
    rV, rF = _load(ref)
    V, _ = inverse_fit(sV, sF, rV, rF, steps=steps, lr=lr)
    objio.write_obj(out, V, sF)
    return 0


def main(argv=None):
    argv = list(sys.argv[1:] if argv is None else argv)
    ap = argparse.ArgumentParser(prog="python -m meshode_gb300.cli", add_help=True)
    ap.add_argument("program", choices=["rigid_deform", "cad_deform", "inverse_deform"])
    ap.add_argument("--steps", type=int, default=None,
                    help="Adam steps (rigid/cad: 1000; inverse: at most 10000)")
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--flow-every", type=int, default=50)
    ap.add_argument("args", nargs="*")
    a = ap.parse_intermixed_args(argv)
    if a.program == "rigid_deform":
        return rigid_deform(a.args, steps=a.steps or 1000, lr=a.lr)
    if a.program == "inverse_deform":
        return inverse_deform(a.args, steps=a.steps or 10000, lr=a.lr)
    return cad_deform(a.args, steps=a.steps or 1000, lr=a.lr, flow_every=a.flow_every)


if __name__ == "__main__":
    sys.exit(main())
