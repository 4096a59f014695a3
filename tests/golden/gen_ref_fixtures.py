"""Generate the reference fixtures of tests/golden from the reference itself.

Run from the repository root where the reference is mounted:
    python tests/golden/gen_ref_fixtures.py

Everything here comes from oracle/_ref -- the reference's pyDeform C++ loops
compiled unchanged (see oracle/build_ref.py) -- and from the reference's own
Python layer src/python/layers/rigid_loss_layer.py, imported unchanged with
``pyDeform`` bound to oracle/_ref:

ref_demo_meshes.npz
    LoadMesh (mesh_tensor.cc:87-100) of the four demo meshes of data/
    (float32 V, int32 F, and each file's SHA-256), plus Mesh::ReadOBJ's double
    vertices of the CAD meshes (LoadCadMesh keeps them in double).
ref_demo_rigid.npz
    The demo pair source.obj -> target.obj set up as rigid_deform.py:25-30
    does (64^3 grid): the target transform, the reference's grid (as the
    float32 values DistanceFloat reads), the normalised source, SHA-256
    digests of DistanceFieldLoss and RigidEdgeLoss forward/backward at the
    normalised source and at a seeded perturbation of it, and the loop of
    rigid_deform.py:32-39 (torch.optim.Adam, lr 1e-3) for 1000 steps: the
    loss every 100 steps and the final normalised positions.

The GPU tests read only these files (the reference is not mounted where
they run).
"""
import hashlib
import importlib.util
import os
import sys
import time

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from meshode_gb300 import objio  # noqa: E402
from oracle import ref as R  # noqa: E402

N = 64
STEPS = 1000
PERTURB_SEED = 11
PERTURB_SIGMA = 0.01


def sha(t):
    a = t.detach().numpy() if isinstance(t, torch.Tensor) else np.asarray(t)
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def perturbed(Vn):
    rng = np.random.Generator(np.random.PCG64(PERTURB_SEED))
    return (Vn + torch.from_numpy(rng.normal(0, PERTURB_SIGMA, Vn.shape).astype(np.float32))).contiguous()


def demo_meshes():
    out = {}
    for name in ("source.obj", "target.obj", "cad-source.obj", "cad-target.obj"):
        key = name.replace(".obj", "").replace("-", "_")
        path = R.reference_path("data", name)
        V, F = R.LoadMesh(path)
        out[key + "_V"] = V.numpy()
        out[key + "_F"] = F.numpy()
        out[key + "_sha256"] = np.array(hashlib.sha256(open(path, "rb").read()).hexdigest())
        if name.startswith("cad"):
            Vd, Fd = objio.read_obj(path)
            assert np.array_equal(Vd.astype(np.float32), V.numpy()) and np.array_equal(Fd, F.numpy())
            out[key + "_V64"] = Vd
    np.savez_compressed(os.path.join(HERE, "ref_demo_meshes.npz"), **out)
    return out


def reference_layer():
    R.install_as_pydeform()
    spec = importlib.util.spec_from_file_location(
        "ref_rigid_loss_layer", R.reference_path("src", "python", "layers", "rigid_loss_layer.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def demo_rigid(meshes):
    src_V = torch.from_numpy(meshes["source_V"].copy())
    src_F = torch.from_numpy(meshes["source_F"].copy())
    tar_V = torch.from_numpy(meshes["target_V"].copy())
    tar_F = torch.from_numpy(meshes["target_F"].copy())
    mod = reference_layer()
    # rigid_deform.py:28-30 (the layer normalises src_V in place; grid 64,
    # rigid_loss_layer.py:35)
    rigid_deform = mod.RigidLossLayer(src_V, src_F, tar_V, tar_F)
    pid = int(rigid_deform.param_id)
    scale, trans = R.template_transform(pid)
    grid = R.template_grid(pid, N).astype(np.float32)
    out = {"N": np.int32(N), "scale": np.float64(scale), "trans": trans, "grid": grid,
           "source_normalized": src_V.numpy().copy()}
    Vp = perturbed(src_V)
    for tag, V in (("at_source", src_V), ("at_perturbed", Vp)):
        out["df_forward_" + tag] = np.array(sha(R.DistanceFieldLoss_forward(V, pid)))
        out["df_backward_" + tag] = np.array(sha(R.DistanceFieldLoss_backward(V, pid)))
        out["rigid_forward_" + tag] = np.array(sha(R.RigidEdgeLoss_forward(V, src_F, pid)))
        out["rigid_backward_" + tag] = np.array(sha(R.RigidEdgeLoss_backward(V, src_F, pid)))
    # rigid_deform.py:31-39
    src_V = torch.nn.Parameter(src_V)
    optimizer = torch.optim.Adam([src_V], lr=1e-3)
    losses = []
    t0 = time.time()
    for it in range(STEPS):
        optimizer.zero_grad()
        loss = rigid_deform(src_V, src_F)
        loss.backward()
        optimizer.step()
        if it % 100 == 0:
            losses.append(loss.item())
    print("reference loop: %d steps in %.1f s" % (STEPS, time.time() - t0))
    out["loop_steps"] = np.int32(STEPS)
    out["loop_losses_every_100"] = np.array(losses, np.float64)
    out["loop_final_normalized"] = src_V.detach().numpy().copy()
    out["perturb"] = np.array([PERTURB_SEED, PERTURB_SIGMA])
    np.savez_compressed(os.path.join(HERE, "ref_demo_rigid.npz"), **out)


if __name__ == "__main__":
    torch.set_num_threads(1)
    m = demo_meshes()
    demo_rigid(m)
    for f in ("ref_demo_meshes.npz", "ref_demo_rigid.npz"):
        print(f, os.path.getsize(os.path.join(HERE, f)))
