"""GPU frames (sph_render) and point sources (sph_append) against the CPU
oracle. Frames are compared byte for byte; runs with sources bit for bit."""
import copy
import ctypes as C

import numpy as np
import pytest

from sphugo_gb300 import _lib as L
from sphugo_gb300 import ics
from sphugo_gb300 import sim as S
from test_gpu_parity import assert_bitwise, pair

pytestmark = pytest.mark.gpu


def gpu_frame_inputs(g):
    st, der = g.state(), g.derived()
    return st["x"], st["y"], der["rho"]


@pytest.mark.parametrize("n,w,h", [(3000, 1280, 720), (800, 333, 211)])
def test_frame_matches_painter_with_draw_keys(gpu, oracle, n, w, h):
    conf = ics.periodic_config(n, 32, 1e-4)
    g = S.Simulation(conf, *ics.uniform_blast(n, 11))
    z = np.random.default_rng(n).choice(2**62, size=n, replace=False).astype(np.int64)
    g.SetDrawKeys(z)
    g.Step(3)
    img = g.Frame(w, h)
    x, y, rho = gpu_frame_inputs(g)
    ref = oracle.render(x, y, rho, conf.ParticleMass, oracle.draw_order(z), w, h)
    assert img.shape == (h, w, 4)
    assert np.array_equal(img, ref), f"{np.sum(np.any(img != ref, axis=2))} pixels differ"
    assert len(np.unique(img.reshape(-1, 4), axis=0)) > 3  # disks of several colours


def test_frame_default_order_and_unevaluated_state(gpu, oracle):
    n = 1500
    conf = ics.periodic_config(n, 32, 1e-4)
    g = S.Simulation(conf, *ics.uniform_blast(n, 12))
    x0, y0 = g.state()["x"], g.state()["y"]
    img0 = g.Frame(640, 360)  # before any evaluation: every density counts as 0
    ref0 = oracle.render(x0, y0, np.zeros(n), conf.ParticleMass, np.arange(n), 640, 360)
    assert np.array_equal(img0, ref0)
    g.Step(2)
    x, y, rho = gpu_frame_inputs(g)
    ref = oracle.render(x, y, rho, conf.ParticleMass, np.arange(n), 640, 360)  # caller order
    assert np.array_equal(g.Frame(640, 360), ref)


def spawn(lib, src, t, seed):
    probe = L.SphPointSource.from_buffer_copy(src)
    m = int(lib.sph_point_source_spawn(C.byref(probe), t, 0, None, None, None, None, None, None))
    arrs = [np.zeros(max(m, 0)) for _ in range(5)]
    z = np.zeros(max(m, 0), np.int64)
    if m > 0:
        lib.sph_point_source_spawn(C.byref(src), t, seed, *[L.dptr(a) for a in arrs], L.i64ptr(z))
    return arrs, z


def test_point_sources_append_particles_like_the_reference(gpu, oracle):
    n = 2500
    conf = ics.periodic_config(n, 32, 1e-3)
    conf.Sources = [S.PointSource(S.Vec2(0.3, 0.4), 3000.0, 0.0), S.PointSource(S.Vec2(0.72, 0.61), 1700.0, 0.0)]
    arrs = ics.uniform_blast(n, 5)
    g, o = pair(oracle, conf, arrs)
    srcs = [L.SphPointSource((C.c_double * 2)(s.origin.X, s.origin.Y), s.rate, s.LastSpwned)
            for s in copy.deepcopy(conf.Sources)]
    keys = []
    for step in range(7):
        t = float(step) * conf.DeltaTHalf * 2
        for i, src in enumerate(srcs):
            (x, y, vx, vy, u), z = spawn(gpu, src, t, S._source_seed(step, i))
            if len(x):
                o.append(x, y, vx, vy, u)
                keys.append(z)
        o.step(1)
        g.Step(1)
    assert g.n == o.n > n + 20
    assert g.Config.Sources[0].LastSpwned == srcs[0].last_spawned
    assert_bitwise(g, o)
    # the appended particles' draw keys order the frame
    zall = np.concatenate([np.arange(n, dtype=np.int64) * 0 - np.arange(n)] + keys)
    x, y, rho = gpu_frame_inputs(g)
    ref = oracle.render(x, y, rho, conf.ParticleMass, oracle.draw_order(zall), 400, 300)
    assert np.array_equal(g.Frame(400, 300), ref)


def test_append_rejects_ensembles_and_grows_capacity(gpu):
    confs, arrays = ics.make_ensemble(nsims=2, seed=5)
    e = S.Ensemble(confs, arrays)
    x = np.array([0.5])
    with pytest.raises(L.SphError):
        L.check(gpu.sph_append(e._h, 1, L.dptr(x), L.dptr(x), None, None, None, None))
    n = 500
    g = S.Simulation(ics.periodic_config(n, 16, 1e-4), *ics.uniform_blast(n, 2))
    g.Step(1)
    rng = np.random.default_rng(0)
    for _ in range(4):  # several reallocations
        m = 300
        xs, ys = rng.random(m), rng.random(m)
        L.check(gpu.sph_append(g._h, m, L.dptr(xs), L.dptr(ys), None, None, None, None))
        g.n += m
        g.Step(1)
    assert g.n == n + 1200 and np.all(np.isfinite(g.derived()["rho"]))
