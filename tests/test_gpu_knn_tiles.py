"""The neighbour search's tile shapes against the per-query search, through the
C ABI: block tiles of eight and four warps (256 / 128 consecutive queries
sharing one tile) and one tile per warp (32 queries). Every shape must return
the same exact neighbour sets as the per-query search (and so as the oracle,
which the parity tests pin); in the FP64 form every result is identical bit
for bit. The workloads cover periodic images at the box edges, open
boundaries, boxes far from the origin, clustered and strongly non-uniform
particles, every list shape (k = 16, 32, 37, 64) and ensembles whose tiles
straddle several simulations."""
import numpy as np
import pytest

from sphugo_gb300 import _lib as L
from sphugo_gb300 import ics
from sphugo_gb300 import sim as S

pytestmark = pytest.mark.gpu


def _inputs(kind, n, seed):
    if kind == "clustered":
        return ics.clustered(n, seed)
    if kind == "stress":
        return ics.stress(n, seed)
    return ics.uniform_blast(n, seed)


def _conf(n, k, precision, kind):
    # the stress workload packs 99 % of the particles into 1 % of the box: at
    # the automatic level its cells hold hundreds, more than any tile holds,
    # so it is binned three levels finer (as the tuner would)
    level = 0
    if kind == "stress":
        level = int(np.floor(0.5 * np.log2(n / 2.0) + 0.5)) + 3
    conf = ics.periodic_config(n, k, 1e-5, precision, grid_level=level)
    if kind == "open":
        conf.HorPeriodicity = conf.VertPeriodicity = S.OPEN
    return conf


def _run(kind, n, k, precision, tiles, shift=1000.0):
    x, y, vx, vy, u = _inputs("blast" if kind in ("blast", "open", "far") else kind, n, 7)
    conf = _conf(n, k, precision, kind)
    if kind == "far":
        conf.HorPeriodicity = (shift, shift + 1.0)
        conf.VertPeriodicity = (shift, shift + 1.0)
        x, y = x + shift, y + shift
    rng = np.random.default_rng(5)
    vx, vy = rng.normal(0, 0.3, n), rng.normal(0, 0.3, n)
    s = S.Simulation(conf, x, y, vx, vy, u)
    s.SetSearch(tiles)
    # the first evaluation has no previous smoothing lengths (per-query search
    # everywhere); the second, on the same state, runs the tiles
    s.CalculateForces()
    s.CalculateForces()
    out = (s.neighbours(), s.derived(), s.state(), s.search_stats())
    s.close()
    return out


CASES = [("blast", 40_000, 32), ("blast", 40_000, 16), ("blast", 30_000, 37), ("clustered", 60_000, 32),
         ("stress", 60_000, 64), ("open", 30_000, 32), ("far", 30_000, 32), ("blast", 30_000, 64)]


@pytest.mark.parametrize("kind,n,k", CASES)
@pytest.mark.parametrize("precision", ["Exact", "Mixed"])
def test_tile_shapes_match_per_query_search(gpu, kind, n, k, precision):
    ref = _run(kind, n, k, precision, 0)
    shapes = [8, 4, 2] if k <= 37 else [4, 2]
    for tiles in shapes:
        got = _run(kind, n, k, precision, tiles)
        (gi, gd, gm), (ri, rd, rm) = got[0], ref[0]
        assert np.array_equal(gi, ri), (tiles, np.sum(np.any(gi != ri, axis=1)))
        assert np.array_equal(gm, rm) and np.array_equal(gd, rd), tiles
        if precision == "Exact":
            for key in ("rho", "c", "h"):
                assert np.array_equal(got[1][key], ref[1][key]), (tiles, key)
            for key in ("ax", "ay", "udot"):
                assert np.array_equal(got[2][key], ref[2][key]), (tiles, key)
        else:
            assert np.array_equal(got[1]["h"], ref[1]["h"])
            assert np.allclose(got[1]["rho"], ref[1]["rho"], rtol=1e-5, atol=0)
        q, d = got[3]
        assert q == n
        if k != 37:  # k = 37 fills 37 of the 40 list entries: many lists overflow to the per-query search
            assert d < 0.25 * n, (tiles, d)  # most queries settled by the tiles


def test_block_tiles_settle_most_queries(gpu):
    """On the uniform blast (N = 200,000, k = 32) the block tiles leave only a
    few per cent of the queries to the per-query search."""
    for tiles in (8, 4):
        _, _, _, (q, d) = _run("blast", 200_000, 32, "Mixed", tiles)
        assert d < 0.05 * q, (tiles, d)


def test_block_tiles_straddle_ensemble_members(gpu):
    """Ensembles of small simulations: block tiles of 256 queries span several
    simulations (one pass per simulation); the results equal the per-query
    search's bit for bit over several steps."""
    _, arrays = ics.make_ensemble(nsims=20, seed=4, precision="Exact")
    confs = [ics.periodic_config(len(a[0]), 32, 1e-4, "Exact") for a in arrays]
    runs = []
    for tiles in (0, 8, 4, 2):
        e = S.Ensemble(confs, arrays)
        e.SetSearch(tiles)
        e.Step(4)
        runs.append((e.state(), e.search_stats()))
        e.close()
    ref = runs[0][0]
    for st, (q, d) in runs[1:]:
        for key in ref:
            assert np.array_equal(st[key], ref[key]), key
        assert d < 0.3 * q


def test_search_shape_arguments(gpu):
    x, y, vx, vy, u = ics.uniform_blast(3000, 3)
    s = S.Simulation(ics.periodic_config(3000, 64, 1e-4, "Exact"), x, y, vx, vy, u)
    with pytest.raises(L.SphError):
        s.SetSearch(8)  # k = 64 lists are too long for eight-warp tiles
    s.SetSearch(4)
    with pytest.raises(L.SphError):
        s.SetSearch(3)
