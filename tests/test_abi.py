"""C-ABI checks that need no GPU: the library loads, exports every function
include/sphgpu.h declares, and its host-only entry points behave."""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    src = open(os.path.join(ROOT, "include", "sphgpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^[A-Za-z_][\w\s\*]*?\b(sph_\w+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_library_exports_every_declared_function(sphlib):
    names = header_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(sphlib, n)]
    assert not missing, missing
    from sphugo_gb300 import _lib as L
    assert sorted(L.EXPORTS) == names


def test_abi_version_and_defaults(sphlib):
    from sphugo_gb300 import _lib as L
    assert sphlib.sph_abi_version() == 1
    p = sphlib.sph_default_params()
    # sim/config-parser.go:131-149 MakeConfig
    assert p.k == 32 and p.gamma == 1.66666 and p.mass == 1.0 and p.dth == 0.001
    assert p.hor[0] == -L.DBL_MAX and p.hor[1] == L.DBL_MAX
    assert (p.alpha, p.beta, p.etasq) == (0.75, 1.5, 0.01)


def test_struct_layout_matches_header(sphlib, tmp_path):
    """ctypes mirrors of the ABI structs have the C compiler's sizes and offsets."""
    import subprocess
    from sphugo_gb300 import _lib as L
    src = tmp_path / "layout.c"
    src.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "sphgpu.h"\n'
        'int main(void){printf("%zu %zu %zu %zu %zu %zu\\n", sizeof(sph_params), offsetof(sph_params, gamma),'
        ' offsetof(sph_params, alpha), sizeof(sph_config), offsetof(sph_config, start),'
        ' offsetof(sph_config, sources)); return 0;}\n')
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    want = [C.sizeof(L.SphParams), L.SphParams.gamma.offset, L.SphParams.alpha.offset,
            C.sizeof(L.SphConfig), L.SphConfig.start.offset, L.SphConfig.sources.offset]
    assert got == want


def test_create_without_gpu_fails_cleanly(sphlib):
    from sphugo_gb300 import _lib as L
    n = C.c_int32(0)
    if sphlib.sph_device_count(C.byref(n)) == 0 and n.value > 0:
        pytest.skip("a GPU is visible")
    p = sphlib.sph_default_params()
    h = C.c_void_p()
    rc = sphlib.sph_create(C.byref(p), 100, C.byref(h))
    assert rc == L.SPH_ERR_CUDA and not h.value
    assert "device" in L.last_error().lower() or "cuda" in L.last_error().lower()


def test_argument_checks_precede_device_use(sphlib):
    from sphugo_gb300 import _lib as L
    p = sphlib.sph_default_params()
    h = C.c_void_p()
    assert sphlib.sph_create(C.byref(p), 10, C.byref(h)) == L.SPH_ERR_ARG  # n < k+1
    assert "k+1" in L.last_error()
    p.hor[1] = 1.0  # open low bound with a finite high one: sim/nearest-neighbour.go:43-45 panics
    assert sphlib.sph_create(C.byref(p), 100, C.byref(h)) == L.SPH_ERR_ARG
    p = sphlib.sph_default_params()
    p.k = 0
    assert sphlib.sph_create(C.byref(p), 100, C.byref(h)) == L.SPH_ERR_ARG
    ptr = C.c_void_p()
    assert sphlib.sph_host_alloc(0, C.byref(ptr)) == L.SPH_ERR_ARG
    assert sphlib.sph_host_alloc(64, None) == L.SPH_ERR_ARG
    assert sphlib.sph_host_free(None) == L.SPH_ERR_ARG


def test_uniform_blast_ic_is_deterministic_and_uniform(sphlib):
    from sphugo_gb300 import ics
    a = ics.uniform_blast(100_000, 1)
    b = ics.uniform_blast(100_000, 1)
    c = ics.uniform_blast(100_000, 2)
    for u, v in zip(a, b):
        assert np.array_equal(u, v)
    assert not np.array_equal(a[0], c[0])
    x, y, vx, vy, u = a
    assert 0 <= x.min() and x.max() < 1 and abs(x.mean() - 0.5) < 0.005
    assert np.all(vx == 0) and np.all(vy == 0)
    inside = (x - 0.5) ** 2 + (y - 0.5) ** 2 < 0.01
    assert np.array_equal(u == 10.0, inside) and abs(inside.mean() - np.pi * 0.01) < 0.002


def test_splitmix_first_values(sphlib):
    # SplitMix64 with seed 0: first output 0xe220a8397b1dcdaf (published reference value)
    from sphugo_gb300 import ics
    x, y, *_ = ics.uniform_blast(1, 0)
    assert x[0] == (0xE220A8397B1DCDAF >> 11) * 2.0 ** -53


def test_clustered_and_stress_ics(sphlib):
    from sphugo_gb300 import ics
    x, y, _, _, u = ics.clustered(200_000, 3)
    assert x.min() >= 0 and x.max() < 1 and y.min() >= 0 and y.max() < 1
    assert set(np.unique(u)) == {1.0, 10.0}
    # a Gaussian core holds 1 - e^{-1/2} of its blob
    assert abs((u == 10.0).mean() - 0.8 * (1 - np.exp(-0.5))) < 0.01
    x, y, _, _, u = ics.stress(100_000, 4)
    span = np.percentile(x, 99.4) - np.percentile(x, 0.6)
    assert span < 0.11
    assert (u == 100.0).sum() > 0


def test_ensemble_sizes(sphlib):
    from sphugo_gb300 import ics
    counts, ub = ics.ensemble_sizes(256, 5)
    assert counts.min() >= 1000 and counts.max() <= 65536
    assert 5 <= ub.min() and ub.max() <= 50
    lc = np.log(counts)
    assert abs(lc.mean() - 0.5 * (np.log(1000) + np.log(65536))) < 0.3


def test_oracle_workloads_equal_the_library_generators(sphlib, oracle):
    """The benchmark's CPU arms build their inputs with the oracle's copy of
    the recipes (no GPU library loaded): the arrays must be the library's,
    bit for bit."""
    from sphugo_gb300 import ics
    cases = [(ics.uniform_blast, oracle.uniform_blast, (50_000, 2)),
             (ics.uniform_blast, oracle.uniform_blast, (7_000, 1005, 1.0, 23.5, 0.1)),
             (ics.clustered, oracle.clustered, (60_000, 3)),
             (ics.stress, oracle.stress, (40_000, 4))]
    for lib_fn, orc_fn, args in cases:
        for a, b in zip(lib_fn(*args), orc_fn(*args)):
            assert np.array_equal(a, b), (lib_fn.__name__, args)
    c1, u1 = ics.ensemble_sizes(256, 5)
    c2, u2 = oracle.ensemble_sizes(256, 5)
    assert np.array_equal(c1, c2) and np.array_equal(u1, u2)
