"""The C oracle against the golden fixtures of tests/golden/gen_golden.py (an
independent numpy restatement of the reference's arithmetic).  CPU only."""
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "meshode_golden.npz")


@pytest.fixture(scope="module")
def g():
    return dict(np.load(GOLDEN))


def _bits_equal(a, b):
    a = np.asarray(a, np.float32)
    b = np.asarray(b, np.float32)
    return bool((((a == b) | (np.isnan(a) & np.isnan(b)))).all())


def test_normalisation(orc, g):
    scale, trans = orc.normalize_params(g["target_V"])
    assert scale == float(g["scale"])
    assert np.array_equal(trans, g["trans"])
    S = np.array(g["source_V"], copy=True)
    orc.lib().orc_normalize_by_template(orc._p(S), S.shape[0], scale, orc._p(np.ascontiguousarray(trans)))
    assert np.array_equal(S, g["source_Vn"])


@pytest.mark.parametrize("method", ["brute", "bvh"])
def test_distance_field_fp64(orc, g, method):
    scale, trans = orc.normalize_params(g["target_V"])
    Vn = orc.normalized_double(g["target_V"], scale, trans)
    grid = orc.df_build(Vn, g["target_F"], int(g["N"]), method=method)
    assert np.abs(grid - g["grid64"]).max() <= 1e-12


def test_distance_lookup_and_jet(orc, g):
    N = int(g["N"])
    for p, d, j in zip(g["probes"], g["distance"], g["jet"]):
        assert _bits_equal(orc.distance_float(g["grid"], N, p), d)
        assert _bits_equal(orc.distance_jet(g["grid"], N, p), j)


def test_dfloss(orc, g):
    N = int(g["N"])
    assert _bits_equal(orc.dfloss_forward(g["probes"], g["grid"], N), g["dfloss_fwd"])
    assert _bits_equal(orc.dfloss_backward(g["probes"], g["grid"], N), g["dfloss_bwd"])


def test_edges(orc, g):
    off = orc.edge_offsets(g["source_Vn"], g["source_F"], 0)
    assert _bits_equal(off, g["edge_offsets"])
    assert _bits_equal(orc.edge_forward(g["source_V1"], g["source_F"], 0, off), g["edge_fwd"])
    assert _bits_equal(orc.edge_backward(g["source_V1"], g["source_F"], 0, off), g["edge_bwd"])
