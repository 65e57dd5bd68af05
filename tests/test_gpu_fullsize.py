"""GPU parity at the benchmark workloads' full sizes, through the C ABI:

  * the stress workload (N = 16,777,216, k = 64): one force evaluation of
    both arithmetic forms against the oracle's exact evaluation of the same
    state: neighbour sets bit-exact in both forms, the FP64 form bit-exact in
    every array, the mixed form within its stated tolerances;
  * the clustered workload (N = 4,194,304, k = 32): one force evaluation of
    the FP64 form against the oracle, bit for bit; and at the
    end of the mixed form's full 50-step run both forms evaluate its final
    state: sets bit-exact, mixed errors within the stated tolerances;
  * the 256-simulation ensemble in the mixed form, simulation by simulation
    against the oracle; and in the FP64 form over its full 100 steps.

Tolerances (the stated ones): neighbour ids, images and NNDists bit-exact;
SPH_PREC_FP64 bit-exact; SPH_PREC_MIXED density 1e-5 relative, acceleration
and du/dt 1e-4 normalised per particle by the sum of neighbour-term
magnitudes.
"""
import numpy as np
import pytest

from sphugo_gb300 import ics
from sphugo_gb300 import sim as S

from test_gpu_parity import STATE, normalised_errors, oracle_params

pytestmark = pytest.mark.gpu

RHO_TOL, ACC_TOL, UDOT_TOL = 1e-5, 1e-4, 1e-4


def _moving(n, seed):
    rng = np.random.default_rng(seed)
    return rng.normal(0, 0.3, n), rng.normal(0, 0.3, n)


def test_stress_full_size_both_forms_against_oracle(gpu, oracle):
    """N = 16,777,216, k = 64: 99 % of the particles in a 0.1 x 0.1 square, a
    hot disc at its centre; random velocities so that viscosity and du/dt
    terms appear."""
    n, k = 1 << 24, 64
    x, y, _, _, u = ics.stress(n, 4)
    vx, vy = _moving(n, 4)
    conf = ics.periodic_config(n, k, 1e-6, "Exact")
    o = oracle.OracleSim(oracle_params(oracle, conf, n), x, y, vx, vy, u)
    o.forces()
    os_ = o.state()
    an, un = o.norms()
    oi, od, om = o.neighbours()
    o.close()
    for form in ("Exact", "Mixed"):
        g = S.Simulation(ics.periodic_config(n, k, 1e-6, form), x, y, vx, vy, u)
        g.Autotune()  # the stress case's binning level (the automatic one overfills its dense cells)
        g.CalculateForces()
        gi, gd, gm = g.neighbours()
        assert np.array_equal(gi, oi), f"{form}: ids differ for {np.sum(np.any(gi != oi, axis=1))} particles"
        assert np.array_equal(gm, om), form
        assert np.array_equal(gd, od), form
        del gi, gd, gm
        gs, gder = g.state(), g.derived()
        g.close()
        assert np.array_equal(gder["h"], os_["h"]), form
        if form == "Exact":
            for key in STATE:
                assert np.array_equal(gs[key], os_[key]), key
            for key in ("rho", "c"):
                assert np.array_equal(gder[key], os_[key]), key
        else:
            r, a, ud = normalised_errors(gs, gder, os_, an, un)
            assert r.max() <= RHO_TOL, r.max()
            assert a.max() <= ACC_TOL, a.max()
            assert ud.max() <= UDOT_TOL, ud.max()


def test_clustered_full_size_fp64_against_oracle(gpu, oracle):
    """The clustered workload at the benchmark's size (N = 4,194,304, k = 32,
    seed 3) with random velocities: one force evaluation of the FP64 form
    against the oracle's exact evaluation, every array bit for bit."""
    n = 1 << 22
    x, y, _, _, u = ics.clustered(n, 3)
    vx, vy = _moving(n, 3)
    conf = ics.periodic_config(n, 32, 1e-5, "Exact")
    o = oracle.OracleSim(oracle_params(oracle, conf, n), x, y, vx, vy, u)
    g = S.Simulation(conf, x, y, vx, vy, u)
    g.Autotune()
    o.forces()
    g.CalculateForces()
    os_, gs, gder = o.state(), g.state(), g.derived()
    oi, od, om = o.neighbours()
    gi, gd, gm = g.neighbours()
    assert np.array_equal(gi, oi), np.sum(np.any(gi != oi, axis=1))
    assert np.array_equal(gm, om) and np.array_equal(gd, od)
    del oi, od, om, gi, gd, gm
    for key in STATE:
        assert np.array_equal(gs[key], os_[key]), key
    for key in ("rho", "c", "h"):
        assert np.array_equal(gder[key], os_[key]), key
    o.close()
    g.close()


def test_clustered_mixed_errors_after_full_run(gpu):
    """The clustered workload's full mixed run (N = 4,194,304, k = 32,
    dt = 1e-5, 50 steps); both forms then evaluate the forces of its final
    state: sets bit-exact and the mixed errors within the stated tolerances,
    normalised by the FP64 evaluation's own neighbour-term sums (which equal
    the oracle's bit for bit)."""
    n = 1 << 22
    arrs = ics.clustered(n, 3)
    m = S.Simulation(ics.periodic_config(n, 32, 1e-5, "Mixed"), *arrs)
    m.Step(50)
    st = m.state()
    m.close()
    out = {}
    for form in ("Exact", "Mixed"):
        g = S.Simulation(ics.periodic_config(n, 32, 1e-5, form), st["x"], st["y"], st["vx"], st["vy"], st["u"])
        g.set_state(*(st[c] for c in STATE))
        g.CalculateForces()
        out[form] = (g.state(), g.derived(), g.neighbours(), g.error_norms() if form == "Exact" else None)
        g.close()
    (es, ed, en, (an, un)), (ms, md, mn, _) = out["Exact"], out["Mixed"]
    for a, b in zip(en, mn):
        assert np.array_equal(a, b)
    fp64 = dict(es)
    fp64.update(ed)
    r, a, ud = normalised_errors(ms, md, fp64, an, un)
    assert r.max() <= RHO_TOL, r.max()
    assert a.max() <= ACC_TOL, a.max()
    assert ud.max() <= UDOT_TOL, ud.max()


def test_mixed_ensemble_full_size_against_oracle(gpu, oracle):
    """The 256-simulation ensemble (3.83M particles) in the mixed form, one
    force evaluation on moving initial states: every simulation's neighbour
    sets bit-exact and its rho, a and du/dt within the stated tolerances of
    the oracle's evaluation of that simulation alone."""
    confs, arrays = ics.make_ensemble(precision="Mixed")
    moving = []
    for s, (x, y, _, _, u) in enumerate(arrays):
        vx, vy = _moving(len(x), 500 + s)
        moving.append((x, y, vx, vy, u))
    e = S.Ensemble(confs, moving)
    e.CalculateForces()
    est, eder = e.state(), e.derived()
    eids, edist, eimg = e.neighbours()
    off = e.offsets
    worst = [0.0, 0.0, 0.0]
    for s in range(len(confs)):
        n = off[s + 1] - off[s]
        o = oracle.OracleSim(oracle_params(oracle, confs[s], n), *moving[s])
        o.forces()
        os_ = o.state()
        an, un = o.norms()
        oi, od, om = o.neighbours()
        o.close()
        sl = slice(off[s], off[s + 1])
        assert np.array_equal(eids[sl] - off[s], oi), s
        assert np.array_equal(eimg[sl], om), s
        assert np.array_equal(edist[sl], od), s
        assert np.array_equal(eder["h"][sl], os_["h"]), s
        r, a, ud = normalised_errors({k: v[sl] for k, v in est.items()}, {k: v[sl] for k, v in eder.items()},
                                     os_, an, un)
        worst = [max(worst[0], r.max()), max(worst[1], a.max()), max(worst[2], ud.max())]
    assert worst[0] <= RHO_TOL and worst[1] <= ACC_TOL and worst[2] <= UDOT_TOL, worst


def test_fp64_ensemble_full_run_against_oracle(gpu, oracle):
    """The 256-simulation ensemble in the FP64 form over its full 100 steps
    (one graph per step); sixteen of its simulations, spread over the size
    range, run alone in the oracle for the same 100 steps: bit for bit."""
    confs, arrays = ics.make_ensemble(precision="Exact")
    e = S.Ensemble(confs, arrays)
    e.Step(100)
    est, eder = e.state(), e.derived()
    off = e.offsets
    sizes = np.diff(off)
    picks = np.argsort(sizes)[np.linspace(0, len(sizes) - 1, 16).astype(int)]
    for s in picks:
        n = int(sizes[s])
        o = oracle.OracleSim(oracle_params(oracle, confs[s], n), *arrays[s])
        o.step(100)
        os_ = o.state()
        o.close()
        sl = slice(off[s], off[s + 1])
        for key in STATE:
            assert np.array_equal(est[key][sl], os_[key]), (int(s), key)
        assert np.array_equal(eder["rho"][sl], os_["rho"]), int(s)
