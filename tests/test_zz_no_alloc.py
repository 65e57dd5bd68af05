"""sph_density_noalloc: the allocation-free entry point for callers that cannot
call cudaMalloc. Its neighbour lists and densities must equal those of the
regular entry points (sph_create + sph_forces) bit for bit, on two calls in a
row through the shared static scratch. Kept in its own file, collected last."""
import ctypes as C

import numpy as np
import pytest

from sphugo_gb300 import _lib as L
from sphugo_gb300 import ics
from sphugo_gb300 import sim as S

pytestmark = pytest.mark.gpu


def _noalloc(lib, conf, x, y):
    import torch

    n, k = len(x), conf.NeighbourCount
    dev = torch.device("cuda", 0)
    dx = torch.from_numpy(np.ascontiguousarray(x)).to(dev)
    dy = torch.from_numpy(np.ascontiguousarray(y)).to(dev)
    ids = torch.full((n * k,), -1, dtype=torch.int64, device=dev)
    dist = torch.zeros(n * k, dtype=torch.float64, device=dev)
    rho = torch.zeros(n, dtype=torch.float64, device=dev)
    h = torch.zeros(n, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    p = conf.params()
    L.check(lib.sph_density_noalloc(C.byref(p), dx.data_ptr(), dy.data_ptr(), n, ids.data_ptr(),
                                    dist.data_ptr(), rho.data_ptr(), h.data_ptr(), None))
    return (ids.cpu().numpy().reshape(n, k), dist.cpu().numpy().reshape(n, k), rho.cpu().numpy(),
            h.cpu().numpy())


def _regular(conf, x, y):
    sim = S.Simulation(conf, x, y)
    sim.CalculateForces()
    ids, dist, _ = sim.neighbours()
    d = sim.derived()
    sim.close()
    return ids, dist, d["rho"], d["h"]


@pytest.mark.parametrize("periodic", [True, False])
def test_noalloc_matches_regular_entry_points_twice(gpu, periodic):
    # two calls in a row, the second smaller than the first: the shared
    # scratch still holds the first call's arrays
    for n, seed in ((6000, 21), (2500, 22)):
        x, y, *_ = ics.uniform_blast(n, seed)
        conf = ics.periodic_config(n, 32, 1e-4)
        if not periodic:
            conf.HorPeriodicity = conf.VertPeriodicity = S.OPEN
        got = _noalloc(gpu, conf, x, y)
        want = _regular(conf, x, y)
        for g, w, name in zip(got, want, ("ids", "dist", "rho", "h")):
            assert np.array_equal(g, w), name


def test_noalloc_rejects_sizes_beyond_its_scratch(gpu):
    n = L.NOALLOC_MAX_N + 1
    conf = ics.periodic_config(n, 32, 1e-4)
    p = conf.params()
    rc = gpu.sph_density_noalloc(C.byref(p), 1, 1, n, None, None, None, None, None)
    assert rc == L.SPH_ERR_ARG and "at most" in L.last_error()
    conf = ics.periodic_config(100, 33, 1e-4)
    p = conf.params()
    assert gpu.sph_density_noalloc(C.byref(p), 1, 1, 100, None, None, None, None, None) == L.SPH_ERR_ARG


def test_noalloc_launch_shape_follows_k(gpu):
    """A call with k = 16 after calls with k = 32 (the search's list shape and
    launch shape differ by k): still equal to the regular entry points."""
    n = 3000
    x, y, *_ = ics.uniform_blast(n, 23)
    for k in (32, 16, 32):
        conf = ics.periodic_config(n, k, 1e-4)
        got = _noalloc(gpu, conf, x, y)
        want = _regular(conf, x, y)
        for g, w, name in zip(got, want, ("ids", "dist", "rho", "h")):
            assert np.array_equal(g, w), (k, name)
