"""Command-line front ends with the reference's argument surface.

    python -m meshode_gb300.cli rigid_deform source.obj reference.obj output.obj \\
        [GRID_RESOLUTION=64] [MESH_RESOLUTION=5000] [lambda=1] [symmetry=0]
    python -m meshode_gb300.cli cad_deform cad.obj reference.obj output.obj \\
        [GRID_RESOLUTION=64] [MESH_RESOLUTION=5000] [lambda=1] [symmetry=0] [flow_output]
    python -m meshode_gb300.cli inverse_deform source.obj reference.obj output.obj
    python -m meshode_gb300.cli cad_deform2 --source cad.obj --target cad-ref.obj --output out.obj [--rigidity 1]

Positional arguments, defaults and their order follow src/app/rigid_deform.cc:
13-41 and src/app/cad_deform.cc:22-61 (with fewer than four arguments the
usage line is printed and the program exits 0, as there).  The solve is the
GPU Adam loop over the fused step instead of the reference's Ceres
Levenberg-Marquardt: same objective (0.5*sum d^2 + lambda^2 * 0.5*sum r^2,
the Ceres edge residual being lambda*(p1 - p2 - v)), ``--steps`` Adam steps at
``--lr``.  Differences, by necessity:
* rigid_deform: as the reference, MESH_RESOLUTION is parsed and unused.
* cad_deform: as the reference, the CAD model is cleaned (RemoveDegenerated,
  MergeDuplex), remeshed at 0.02 with its geometry neighbours and its
  representative graph (Subdivision, restated in cadmesh with SciPy's
  Delaunay); the graph is fitted (DeformGraph's objective: 0.5*sum d^2 +
  lambda^2 * 0.5*sum r^2 over the graph edges) and SolveLinear (rigidity 2,
  Subdivision::LinearSolve) carries the fit to every remeshed vertex.  With
  flow_output every remeshed vertex is fitted instead (DeformSubdivision,
  with the neighbour pairs as uniformly weighted edges where the reference
  uses its length-adaptive edge loss) and snapshots every ``--flow-every``
  steps are written in the reference's flow format (cad_deform.cc:90-114).
  MESH_RESOLUTION is parsed and unused, as in the reference.
* cad_deform2: the Python script src/python/cad_deform2.py (its own
  --source/--target/--output/--rigidity options).
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

from . import cadmesh, fused, layers, meshops, objio
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


def _fit(src_V, src_F, tar_V, tar_F, N, lam, steps, lr, edges=None, mask=False, flow_every=0, log=print,
         keep=False):
    """The fused GPU Adam loop: source normalised by the target's template,
    edges = the faces' half-edges (StoreRigidityInformation) or an explicit
    list (StoreGraphInformation), edge weight lam^2, the d < 0.03 DF mask
    when `mask`.  Returns the fitted vertices denormalised (float64 numpy)
    and the flow snapshots; with keep=True, the normalised device tensor, the
    snapshots and the template id instead (the caller releases it)."""
    dev = torch.device("cuda", torch.cuda.current_device())
    tV = torch.from_numpy(np.ascontiguousarray(tar_V, np.float32)).to(dev)
    tF = torch.from_numpy(np.ascontiguousarray(tar_F, np.int32)).to(dev)
    pid = PD.InitializeDeformTemplate(tV, tF, 0, N)
    V = torch.from_numpy(np.ascontiguousarray(src_V, np.float32)).to(dev)
    PD.NormalizeByTemplate(V, pid)
    w = float(np.float32(lam * lam))
    if edges is not None:
        E = torch.from_numpy(np.ascontiguousarray(edges, np.int32)).to(dev)
        PD.StoreGraphInformation(V, E, pid)
    else:
        F = torch.from_numpy(np.ascontiguousarray(src_F, np.int32)).to(dev)
        PD.StoreRigidityInformation(V, F, pid)
    mask = float(np.float32(0.5 * 0.03 * 0.03)) if mask else None
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
    if keep:
        return out, flow, pid
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
    print("Source:\t\tNum vertices: %d\tNum faces: %d" % (cV.shape[0], cF.shape[0]))
    print("Reference:\tNum vertices: %d\tNum faces: %d\n" % (rV.shape[0], rF.shape[0]))
    # Subdivision (cad_deform.cc:46-49): remesh at 0.02, neighbours, graph
    Vs = Fs = E = ref_ = GV = GE = None
    Vs, Fs = cadmesh.subdivide(cV, cF, cadmesh.SUBDIV_LEN)
    E = cadmesh.geometry_neighbors(Vs, Fs, cadmesh.NEIGHBOR_STEP)
    if not flow_file:
        # Deformer::DeformGraph: the representative graph fitted (distance +
        # lambda * edge residuals), then Subdivision::LinearSolve propagates
        # it to every remeshed vertex (LinearEstimation, rigidity 2)
        ref_, GV, GE = cadmesh.representative_graph(Vs, Fs, E, cadmesh.GRAPH_STEP)
        G, _, pid = _fit(GV, None, rV, rF, N, lam, steps, lr, edges=GE, keep=True)
        dev = G.device
        V = torch.from_numpy(Vs.astype(np.float32)).to(dev)
        PD.NormalizeByTemplate(V, pid)
        PD.SolveLinear(V, torch.from_numpy(Fs.astype(np.int32)), torch.from_numpy(E.astype(np.int32)),
                       torch.from_numpy(ref_.astype(np.int32)), G, 2.0, 0)
        PD.DenormalizeByTemplate(V, pid)
        PD.ReleaseTemplate(pid)
        Vout = V.cpu().numpy().astype(np.float64)
    else:
        # Deformer::DeformSubdivision: every remeshed vertex fitted, edges the
        # neighbour pairs (which include the mesh edges), flow snapshots
        Vout, flow = _fit(Vs, Fs, rV, rF, N, lam, steps, lr, edges=E, flow_every=flow_every)
        _write_flow(flow_file, Vs, flow)
    print("Deformed")
    objio.write_obj(out, Vout, Fs)
    return 0


def cad_deform2(argv, steps=10000, lr=1e-3, log=print):
    """src/python/cad_deform2.py: both models through LoadCadMesh; the
    source's representative graph fitted with GraphLossLayer + the reverse
    loss against the target's graph (each divided by its vertex count), torch
    Adam, stopping when neither loss improves by 1e-6 between the reports
    every 100 iterations; then the graph Finalize (SolveLinear, rigidity 1)
    and SaveMesh of the remeshed source."""
    ap = argparse.ArgumentParser(prog="cad_deform2")
    ap.add_argument("--source", default="../data/cad-source.obj")
    ap.add_argument("--target", default="../data/cad-target.obj")
    ap.add_argument("--output", default="./cad-output.obj")
    ap.add_argument("--rigidity", default="1")
    a = ap.parse_args(argv)
    rigidity = float(a.rigidity)
    src_V, src_F, src_E, src_to_graph, graph_V, graph_E = PD.LoadCadMesh(a.source)
    tar_V, tar_F, _, _, graph_V_tar, _ = PD.LoadCadMesh(a.target)
    dev = torch.device("cuda", torch.cuda.current_device())
    graph_V = graph_V.to(dev)
    graph_E = graph_E.to(dev)
    graph_deform = layers.GraphLossLayer(graph_V, graph_E, tar_V, tar_F, rigidity)
    param_id = graph_deform.param_id
    reverse_deform = layers.ReverseLossLayer()
    graph_V = torch.nn.Parameter(graph_V)
    optimizer = torch.optim.Adam([graph_V], lr=lr)
    graph_V_tar = graph_V_tar.to(dev)
    PD.NormalizeByTemplate(graph_V_tar, int(param_id))
    prev_src, prev_tar = 1e30, 1e30
    for it in range(steps):
        optimizer.zero_grad()
        loss_src2tar = graph_deform(graph_V, graph_E)
        loss_tar2src = reverse_deform(graph_V, graph_V_tar)
        loss = loss_src2tar / graph_V.shape[0] + loss_tar2src / graph_V_tar.shape[0]
        loss.backward()
        optimizer.step()
        if it % 100 == 0:
            cur_src = float(np.sqrt(loss_src2tar.item() / graph_V.shape[0]))
            cur_tar = float(np.sqrt(loss_tar2src.item() / graph_V_tar.shape[0]))
            log("iter=%d, loss_src2tar=%.6f loss_tar2src=%.6f" % (it, cur_src, cur_tar))
            if prev_src - cur_src < 1e-6 and prev_tar - cur_tar < 1e-6:
                break
            prev_src, prev_tar = cur_src, cur_tar
    layers.GraphFinalize(src_V, src_F, src_E, src_to_graph, graph_V.detach(), 1, param_id)
    PD.SaveMesh(a.output, src_V, src_F)
    PD.ReleaseTemplate(int(param_id))
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
    ap.add_argument("program", choices=["rigid_deform", "cad_deform", "inverse_deform", "cad_deform2"])
    ap.add_argument("--steps", type=int, default=None,
                    help="Adam steps (rigid/cad: 1000; inverse: at most 10000)")
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--flow-every", type=int, default=50)
    ap.add_argument("args", nargs="*")
    if argv and argv[0] == "cad_deform2":  # the script's own --source/--target/--output/--rigidity
        rest = argv[1:]
        steps = 10000
        if "--steps" in rest:
            k = rest.index("--steps")
            steps = int(rest[k + 1])
            rest = rest[:k] + rest[k + 2:]
        return cad_deform2(rest, steps=steps)
    a = ap.parse_intermixed_args(argv)
    if a.program == "rigid_deform":
        return rigid_deform(a.args, steps=a.steps or 1000, lr=a.lr)
    if a.program == "inverse_deform":
        return inverse_deform(a.args, steps=a.steps or 10000, lr=a.lr)
    return cad_deform(a.args, steps=a.steps or 1000, lr=a.lr, flow_every=a.flow_every)


if __name__ == "__main__":
    sys.exit(main())
