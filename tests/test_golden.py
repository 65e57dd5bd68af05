"""Committed golden fixtures (tests/golden/*.npz, written by make_golden.py):
the oracle must reproduce them on this host, and the GPU path through the C
ABI must reproduce them bit for bit."""
import glob
import os

import numpy as np
import pytest

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FIXTURES = sorted(glob.glob(os.path.join(HERE, "blast*.npz")))  # SPH runs (make_golden.py)
STATE = ["x", "y", "vx", "vy", "u", "ax", "ay", "udot", "rho", "c", "h"]


def _load(path):
    return dict(np.load(path))


@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p) for p in FIXTURES])
@pytest.mark.parametrize("mode", ["tree", "exact"])
def test_oracle_reproduces_fixture(oracle, path, mode):
    g = _load(path)
    n, k = int(g["n"]), int(g["k"])
    p = oracle.make_params(n, k, knn_mode=oracle.KNN_TREE if mode == "tree" else oracle.KNN_EXACT,
                           alpha=float(g["alpha"]), beta=float(g["beta"]), dth=float(g["dth"]))
    s = oracle.OracleSim(p, g["x0"], g["y0"], None, None, g["u0"])
    s.step(int(g["steps"]))
    st = s.state()
    for key in STATE:
        assert np.array_equal(st[key], g["out_" + key]), key
    ids, dist, img = s.neighbours()
    assert np.array_equal(ids, g["ids"]) and np.array_equal(img, g["img"]) and np.array_equal(dist, g["dist"])


@pytest.mark.gpu
@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p) for p in FIXTURES])
def test_gpu_reproduces_fixture(gpu, path):
    from sphugo_gb300 import sim as S
    g = _load(path)
    n, k = int(g["n"]), int(g["k"])
    conf = S.SphConfig(DeltaTHalf=float(g["dth"]), Gamma=5.0 / 3.0, ParticleMass=1.0 / n,
                       HorPeriodicity=(0.0, 1.0), VertPeriodicity=(0.0, 1.0), NeighbourCount=k,
                       ViscosityAlpha=float(g["alpha"]), ViscosityBeta=float(g["beta"]))
    sim = S.Simulation(conf, g["x0"], g["y0"], None, None, g["u0"])
    sim.Step(int(g["steps"]))
    st = sim.state()
    st.update(sim.derived())
    for key in STATE:
        assert np.array_equal(st[key], g["out_" + key]), key
    ids, dist, img = sim.neighbours()
    assert np.array_equal(ids, g["ids"]) and np.array_equal(img, g["img"]) and np.array_equal(dist, g["dist"])


def test_colour_ramp_matches_the_reference_image(oracle, sphlib):
    """ParaRamp of the frames against the colours in the reference's own
    doc/customColorMaps.png (output of examples/color-ramp/color-ramp.go),
    fixture made by tests/golden/make_ramp_golden.py."""
    import ctypes as C

    ref = np.load(os.path.join(HERE, "color_ramps_ref.npz"))["para"]
    assert np.array_equal(oracle.para_ramp(), ref)
    lut = np.zeros(1024, np.uint8)
    assert sphlib.sph_para_ramp(lut.ctypes.data_as(C.POINTER(C.c_uint8))) == 0
    lut = lut.reshape(256, 4)
    assert np.array_equal(lut[:, :3], ref) and np.all(lut[:, 3] == 255)
