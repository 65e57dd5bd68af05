"""GPU behaviour of the measurement entry points and of stepping semantics."""
import ctypes as C

import numpy as np
import pytest

from sphugo_gb300 import _lib as L
from sphugo_gb300 import ics
from sphugo_gb300 import sim as S

pytestmark = pytest.mark.gpu


def _sim(n=20_000, precision="Exact"):
    conf = ics.periodic_config(n, 32, 1e-4, precision)
    return S.Simulation(conf, *ics.uniform_blast(n, 3))


def test_timed_and_profiled_steps(gpu):
    a, b = _sim(), _sim()
    ms = C.c_double()
    L.check(gpu.sph_step_timed(a._h, 4, C.byref(ms)))
    assert ms.value > 0 and a.CurrentStep == 4
    stages = np.zeros(L.NUM_STAGES)
    L.check(gpu.sph_step_profiled(b._h, 4, L.dptr(stages)))
    assert b.CurrentStep == 4 and np.all(stages > 0)
    # the profiled graph advances the same trajectory
    sa, sb = a.state(), b.state()
    for k in sa:
        assert np.array_equal(sa[k], sb[k])
    assert gpu.sph_kernels_per_step(a._h) >= 7


def test_probe_peaks(gpu):
    d, f = C.c_double(), C.c_double()
    L.check(gpu.sph_probe_peaks(C.byref(d), C.byref(f)))
    assert 0.1 < d.value < 20 and f.value > 10 * d.value


@pytest.mark.parametrize("precision", ["Fast", "Mixed"])
def test_forms_share_neighbour_lists(gpu, precision):
    a, b = _sim(8000), _sim(8000, precision)
    a.CalculateForces()
    b.CalculateForces()
    ia, da, ma = a.neighbours()
    ib, db, mb = b.neighbours()
    assert np.array_equal(ia, ib) and np.array_equal(ma, mb) and np.array_equal(da, db)
    assert np.array_equal(a.derived()["h"], b.derived()["h"])
