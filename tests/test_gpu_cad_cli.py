"""The CAD-style graph deformation (40 disconnected boxes and cylinders
against their jittered copies plus a noisy plane, 128^3 grid, rigidity 1,
source resampled to >= 5000 vertices) and the command-line front ends.

GraphLossFunction semantics (src/python/layers/graph_loss_layer.py:9-43): the
fused GPU loop against the oracle loop (CPU, same grid, op-by-op Adam) bit
for bit after 30 steps and within the Chamfer bar after 300; the plain GPU GraphLossLayer loop
(torch Adam on CUDA) within the Chamfer bar.
"""
import numpy as np
import pytest
import torch

from meshode_gb300 import cli, fused, layers, meshgen, meshops, metrics, objio
from meshode_gb300 import pyDeform as PD

pytestmark = pytest.mark.gpu

MASK = float(np.float32(0.5 * 0.03 * 0.03))


@pytest.fixture(scope="module")
def cad(cuda, orc):
    Vs, Fs, Vt, Ft = meshgen.cad_pair(seed=2)
    Vs, Fs = meshops.subdivide_to(Vs, Fs, 5000)
    Vs = Vs.astype(np.float32)
    Fs = Fs.astype(np.int32)
    E = meshgen.edges_from_faces(Fs)
    N = 128
    pid = PD.InitializeDeformTemplate(torch.from_numpy(Vt), torch.from_numpy(Ft), 0, N)
    V = torch.from_numpy(Vs.copy()).to(cuda)
    PD.NormalizeByTemplate(V, pid)
    PD.StoreGraphInformation(V, torch.from_numpy(E).to(cuda), pid)
    opid = orc.InitializeDeformTemplate(Vt, Ft, 0, N, grid=PD.GetDistanceField(pid).cpu().numpy())
    Vc = V.cpu()
    orc.StoreGraphInformation(Vc, torch.from_numpy(E), opid)
    sc, tr = orc.normalize_params(Vt)
    return dict(Vs=Vs, Fs=Fs, Vt=Vt, Ft=Ft, E=E, pid=pid, opid=opid, V=V, Vc=Vc,
                Tn=orc.normalized_double(Vt, sc, tr))


def test_cad_fused_vs_oracle(orc, cad):
    """Bit-identical 30-step trajectory against the oracle loop with the
    op-by-op Adam restatement (torch's CPU Adam differs by about an ulp per
    step, which the d < 0.03 mask can amplify at a vertex on its edge)."""
    r2 = float(torch.tensor(1.0 * 1.0, dtype=torch.float32))
    out, _ = fused.fused_fit(cad["pid"], cad["V"], 30, group_steps=10, w_edge=r2, mask_thresh=MASK)
    ref = orc.graph_fit(cad["Vc"], torch.from_numpy(cad["E"]), cad["opid"], 30, r2, adam="exact")
    assert torch.equal(out.cpu(), ref), (out.cpu() - ref).abs().max().item()


def test_cad_chamfer_300_steps(orc, cad):
    steps = 300
    r2 = 1.0
    out, _ = fused.fused_fit(cad["pid"], cad["V"], steps, w_edge=r2, mask_thresh=MASK)
    ref = orc.graph_fit(cad["Vc"], torch.from_numpy(cad["E"]), cad["opid"], steps, r2)
    c_gpu = metrics.chamfer(out.cpu().numpy(), cad["Fs"], cad["Tn"], cad["Ft"], samples=20000)
    c_ref = metrics.chamfer(ref.numpy(), cad["Fs"], cad["Tn"], cad["Ft"], samples=20000)
    assert abs(c_gpu - c_ref) <= 1e-4
    # the plain GPU loop: GraphLossLayer + torch.optim.Adam on CUDA
    src = torch.from_numpy(cad["Vs"].copy()).cuda()
    E = torch.from_numpy(cad["E"]).cuda()
    layer = layers.GraphLossLayer(src, E, torch.from_numpy(cad["Vt"]), torch.from_numpy(cad["Ft"]), 1.0,
                                  grid_resolution=128)
    P = torch.nn.Parameter(src)
    opt = torch.optim.Adam([P], lr=1e-3)
    for _ in range(steps):
        opt.zero_grad()
        layer(P, E).backward()
        opt.step()
    c_plain = metrics.chamfer(P.detach().cpu().numpy(), cad["Fs"], cad["Tn"], cad["Ft"], samples=20000)
    assert abs(c_plain - c_ref) <= 1e-4


def test_cli_rigid_and_cad(cuda, tmp_path):
    rng = np.random.Generator(np.random.PCG64(4))
    V, F = meshgen.icosphere(3)
    T = meshgen.displace(V, rng)
    objio.write_obj(str(tmp_path / "src.obj"), V, F)
    objio.write_obj(str(tmp_path / "ref.obj"), T, F)
    out = tmp_path / "out.obj"
    assert cli.main(["rigid_deform", "--steps", "60", str(tmp_path / "src.obj"), str(tmp_path / "ref.obj"),
                     str(out), "32", "5000", "1", "1"]) == 0
    V2, F2 = objio.read_obj(str(out))
    assert V2.shape == V.shape and np.array_equal(F2, F) and np.isfinite(V2).all()
    Vc, Fc, Vr, Fr = meshgen.cad_pair(seed=2, n_prims=6, plane_tris=200)
    objio.write_obj(str(tmp_path / "cad.obj"), Vc, Fc)
    objio.write_obj(str(tmp_path / "cref.obj"), Vr, Fr)
    flow = tmp_path / "flow.obj"
    assert cli.main(["cad_deform", "--steps", "40", "--flow-every", "20", str(tmp_path / "cad.obj"),
                     str(tmp_path / "cref.obj"), str(tmp_path / "cout.obj"), "32", "500", "1", "0", str(flow)]) == 0
    Vo, Fo = objio.read_obj(str(tmp_path / "cout.obj"))
    lines = flow.read_text().splitlines()
    nv = Vo.shape[0]
    assert sum(1 for l in lines if l.startswith("v ")) == nv * 3      # start + 2 snapshots
    assert sum(1 for l in lines if l.startswith("l ")) == nv * 2


def test_cad_deform_graph_and_linear_solve(cuda, tmp_path):
    """cad_deform without flow output: the remeshed model's representative
    graph fitted on the GPU, then SolveLinear carries the fit to every
    remeshed vertex; the result moves toward the target."""
    from meshode_gb300 import cadmesh
    Vc, Fc, Vr, Fr = meshgen.cad_pair(seed=4, n_prims=5, plane_tris=200)
    objio.write_obj(str(tmp_path / "cad.obj"), Vc, Fc)
    objio.write_obj(str(tmp_path / "cref.obj"), Vr, Fr)
    assert cli.main(["cad_deform", "--steps", "300", str(tmp_path / "cad.obj"), str(tmp_path / "cref.obj"),
                     str(tmp_path / "cout.obj"), "64"]) == 0
    Vo, Fo = objio.read_obj(str(tmp_path / "cout.obj"))
    Vf, Ff = objio.read_obj(str(tmp_path / "cad.obj"))  # the model as the program reads it
    V0, F0 = cadmesh.subdivide(*meshops.merge_duplex(*meshops.remove_degenerated(Vf, Ff)))
    assert Vo.shape == V0.shape and np.array_equal(Fo, F0) and np.isfinite(Vo).all()
    before = metrics.chamfer(V0, F0, Vr.astype(np.float64), Fr, samples=5000)
    after = metrics.chamfer(Vo, Fo, Vr.astype(np.float64), Fr, samples=5000)
    assert after < before, (before, after)


def test_cad_deform2_script(cuda, tmp_path):
    """src/python/cad_deform2.py through the CLI: LoadCadMesh on both models,
    graph loss + reverse loss, the graph Finalize (SolveLinear)."""
    Vc, Fc, Vr, Fr = meshgen.cad_pair(seed=6, n_prims=4, plane_tris=200)
    objio.write_obj(str(tmp_path / "cad.obj"), Vc, Fc)
    objio.write_obj(str(tmp_path / "cref.obj"), Vr, Fr)
    out = tmp_path / "cad-output.obj"
    assert cli.main(["cad_deform2", "--source", str(tmp_path / "cad.obj"), "--target", str(tmp_path / "cref.obj"),
                     "--output", str(out), "--rigidity", "1", "--steps", "300"]) == 0
    src = PD.LoadCadMesh(str(tmp_path / "cad.obj"))
    Vo, Fo = objio.read_obj(str(out))
    assert Vo.shape == tuple(src[0].shape) and np.array_equal(Fo, src[1].numpy()) and np.isfinite(Vo).all()
    before = metrics.chamfer(src[0].numpy().astype(np.float64), Fo, Vr.astype(np.float64), Fr, samples=5000)
    after = metrics.chamfer(Vo, Fo, Vr.astype(np.float64), Fr, samples=5000)
    assert after < before, (before, after)
