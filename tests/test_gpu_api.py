"""GPU behaviour of the measurement entry points and of stepping semantics."""
import ctypes as C

import numpy as np
import pytest

from sphugo_gb300 import _lib as L
from sphugo_gb300 import ics
from sphugo_gb300 import sim as S

pytestmark = pytest.mark.gpu


def _sim(n=20_000, precision="Exact", k=32):
    conf = ics.periodic_config(n, k, 1e-4, precision)
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
    d, f, dv, sq = C.c_double(), C.c_double(), C.c_double(), C.c_double()
    L.check(gpu.sph_probe_peaks(C.byref(d), C.byref(f), C.byref(dv), C.byref(sq)))
    assert 0.1 < d.value < 20 and f.value > 10 * d.value
    assert 1.0 < dv.value < 100 and 1.0 < sq.value < 100
    L.check(gpu.sph_probe_peaks(C.byref(d), None, None, None))


@pytest.mark.parametrize("precision", ["Fast", "Mixed"])
def test_forms_share_neighbour_lists(gpu, precision):
    a, b = _sim(8000), _sim(8000, precision)
    a.CalculateForces()
    b.CalculateForces()
    ia, da, ma = a.neighbours()
    ib, db, mb = b.neighbours()
    assert np.array_equal(ia, ib) and np.array_equal(ma, mb) and np.array_equal(da, db)
    assert np.array_equal(a.derived()["h"], b.derived()["h"])


@pytest.mark.parametrize("precision", ["Exact", "Mixed"])
def test_autotune_keeps_results_and_caches(gpu, tmp_path, monkeypatch, precision):
    monkeypatch.setenv("SPHGPU_TUNE_CACHE", str(tmp_path / "tune.txt"))
    a, b = _sim(12_000, precision), _sim(12_000, precision)
    rep = a.Autotune(use_cache=False)
    assert rep["cached"] is False and rep["trials"] >= 12 and rep["level_delta"] in (-1, 0, 1)
    assert a.CurrentStep == 0
    if precision == "Exact":  # exact sets and orders: tuning changes only speed
        a.Step(3)
        b.Step(3)
        sa, sb = a.state(), b.state()
        for k in sa:
            assert np.array_equal(sa[k], sb[k]), k
    else:  # exact sets; the FP32 sums may follow the search's visiting order
        a.CalculateForces()
        b.CalculateForces()
        ia, da, _ = a.neighbours()
        ib, db, _ = b.neighbours()
        assert np.array_equal(ia, ib) and np.array_equal(da, db)
        ra, rb = a.derived()["rho"], b.derived()["rho"]
        assert np.allclose(ra, rb, rtol=1e-6, atol=0)
    c = _sim(12_000, precision)
    rep2 = c.Autotune(use_cache=True)
    assert rep2["cached"] is True and rep2["theta"] == rep["theta"] and rep2["level_delta"] == rep["level_delta"]
    assert rep2["block_warps"] == rep["block_warps"] and rep2["tiles"] == rep["tiles"]
    assert (tmp_path / "tune.txt").read_text().count("sphgpu-tune-v3") == 1


@pytest.mark.parametrize("precision", ["Exact", "Mixed"])
def test_checkpoint_resume_is_bitwise(gpu, tmp_path, precision):
    a = _sim(9000, precision)
    a.Step(6)
    b = _sim(9000, precision)
    b.Step(3)
    ck = tmp_path / "state.ck"
    b.Save(ck)
    c = _sim(9000, precision)
    c.Load(ck)
    assert c.CurrentStep == 3
    c.Step(3)
    sa, sc = a.state(), c.state()
    for k in sa:
        assert np.array_equal(sa[k], sc[k]), k


def test_checkpoint_rejects_other_parameters(gpu, tmp_path):
    a = _sim(3000)
    a.Step(1)
    a.Save(tmp_path / "s.ck")
    b = _sim(3000, "Mixed")
    with pytest.raises(L.SphError) as e:
        b.Load(tmp_path / "s.ck")
    assert e.value.code == L.SPH_ERR_ARG


def test_state_round_trip_through_pinned_host_allocations(gpu):
    """sph_set_state / sph_get_state from and to memory of sph_host_alloc:
    the state read back equals the state written, bit for bit."""
    import numpy as np
    n = 20_000
    x, y, vx, vy, u = ics.uniform_blast(n, 5)
    s = S.Simulation(ics.periodic_config(n, 32, 1e-4, "Exact"), x, y, vx, vy, u)
    s.Step(2)
    st = s.state()
    keys = ["x", "y", "vx", "vy", "u", "ax", "ay", "udot"]
    raw = []
    try:
        for _ in keys:
            p = C.c_void_p()
            L.check(gpu.sph_host_alloc(8 * n, C.byref(p)))
            raw.append(p)
        bufs = [np.ctypeslib.as_array(C.cast(p, C.POINTER(C.c_double)), shape=(n,)) for p in raw]
        for b, k in zip(bufs, keys):
            b[:] = st[k] * 1.0
        bufs[2][:] += 0.25  # a changed velocity must arrive
        L.check(gpu.sph_set_state(s._h, *[L.dptr(b) for b in bufs]))
        for b in bufs:
            b[:] = 0.0
        L.check(gpu.sph_get_state(s._h, *[L.dptr(b) for b in bufs]))
        for b, k in zip(bufs, keys):
            want = st[k] + (0.25 if k == "vx" else 0.0)
            assert np.array_equal(b, want), k
        del bufs
    finally:
        for p in raw:
            gpu.sph_host_free(p)
        s.close()


def test_division_sequences_are_correctly_rounded(gpu):
    """The FP64 form replaces some IEEE divisions by FMA sequences that must
    return the same bits (division by 3; a shared reciprocal with a Markstein
    correction). Checked against the hardware division on 2e8 operand pairs,
    half of them next to rounding midpoints."""
    bad = C.c_int64(-1)
    L.check(gpu.sph_selftest_division(200_000_000, 12345, C.byref(bad)))
    assert bad.value == 0


def test_integer_pipe_fp64_operations_match_the_hardware(gpu):
    """The FP64 kernels compute some multiplications, additions,
    subtractions, divisions, square roots and float-pair splits with integer
    instructions; each must return the hardware instruction's bits. 12 x 2^31
    results over random bit patterns, nearby and extreme exponents, exact
    ties, near cancellation, perfect squares and their neighbours, quotients
    next to rounding boundaries, and special values."""
    bad = C.c_int64(-1)
    L.check(gpu.sph_selftest_fp64emu(1 << 31, 2024, C.byref(bad)))
    assert bad.value == 0
    L.check(gpu.sph_selftest_fp64emu(1 << 28, 7, C.byref(bad)))
    assert bad.value == 0


@pytest.mark.parametrize("precision,k", [("Exact", 32), ("Mixed", 32), ("Exact", 16), ("Mixed", 16),
                                         ("Exact", 64), ("Mixed", 64)])
def test_group_tiles_match_per_query_search(gpu, precision, k):
    """The group-tile search (default) and the per-query search return the
    same exact neighbour sets; in the FP64 form every result is identical.
    k = 16, 32 and 64 take the three list shapes of the tile kernel (24- and
    40-entry sorting networks, the 81-key insertion chain)."""
    a, b = _sim(30_000, precision, k), _sim(30_000, precision, k)
    b.SetSearch(False)
    if precision == "Exact":
        a.Step(5)
        b.Step(5)
        sa, sb = a.state(), b.state()
        for key in sa:
            assert np.array_equal(sa[key], sb[key]), key
    else:
        # the first evaluation has no previous smoothing lengths (per-query
        # search in both); the second, on the same positions, runs the tiles in a
        for _ in range(2):
            a.CalculateForces()
            b.CalculateForces()
        ia, da, ma = a.neighbours()
        ib, db, mb = b.neighbours()
        assert np.array_equal(ia, ib) and np.array_equal(da, db) and np.array_equal(ma, mb)
        assert np.allclose(a.derived()["rho"], b.derived()["rho"], rtol=1e-5, atol=0)  # the mixed tolerance
    qa, dfa = a.search_stats()
    qb, dfb = b.search_stats()
    assert qa == qb == 30_000 and dfb == qb
    assert dfa < 0.3 * qa  # most queries settled by the tiles


def test_group_tiles_cover_ensemble_boundaries_and_images(gpu):
    """Groups that straddle two simulations of an ensemble, and tiles that
    reach across the periodic boundary, give the same results as the per-query
    search."""
    confs, arrays = ics.make_ensemble(nsims=12, seed=3, precision="Exact")
    e1, e2 = S.Ensemble(confs, arrays), S.Ensemble(confs, arrays)
    e2.SetSearch(False)
    e1.Step(4)
    e2.Step(4)
    s1, s2 = e1.state(), e2.state()
    for key in s1:
        assert np.array_equal(s1[key], s2[key]), key
    q, d = e1.search_stats()
    assert d < q


def test_truncated_checkpoint_leaves_the_state(gpu, tmp_path):
    a = _sim(4000)
    a.Step(2)
    a.Save(tmp_path / "s.ck")
    data = (tmp_path / "s.ck").read_bytes()
    (tmp_path / "t.ck").write_bytes(data[: len(data) // 2])
    b = _sim(4000)
    b.Step(1)
    before = b.state()
    with pytest.raises(L.SphError):
        b.Load(tmp_path / "t.ck")
    after = b.state()
    assert b.CurrentStep == 1
    for key in before:
        assert np.array_equal(before[key], after[key]), key


def test_memory_bytes_counts_the_handle(gpu):
    """The device memory a handle reports covers at least its state and
    neighbour lists, stays far below the device, and grows when particles are
    appended past the allocated capacity."""
    a = _sim(20_000)
    mb = a.memory_bytes()
    assert 20_000 * (32 * 4 + 2 * 100) < mb < 1 << 31
    x = np.random.default_rng(1).random(40_000)
    y = np.ascontiguousarray(x[::-1])
    L.check(gpu.sph_append(a._h, x.size, L.dptr(x), L.dptr(y), None, None, None, None))
    assert a.memory_bytes() > mb


def _fnv1a(data: bytes) -> int:
    h = 1469598103934665603
    for b in data:
        h = ((h ^ b) * 1099511628211) & 0xFFFFFFFFFFFFFFFF
    return h


def test_checkpoint_payload_is_checked_before_upload(gpu, tmp_path):
    """A corrupt payload (hash mismatch) and a payload whose particle ids are
    not a permutation (hash made to match) are both refused with
    SPH_ERR_ARG, and the handle keeps its state: the kernels index the
    caller's order by id, so a bad id must never reach the device."""
    import struct
    n = 3000
    a = _sim(n)
    a.Step(2)
    a.Save(tmp_path / "s.ck")
    data = bytearray((tmp_path / "s.ck").read_bytes())
    hdr = 72  # header bytes; the payload hash is its last field
    id_off = hdr + 4 * 16 * n + 3 * 8 * n
    assert len(data) == hdr + 4 * 16 * n + 3 * 8 * n + 4 * n + 4 * n
    b = _sim(n)
    b.Step(1)
    before = b.state()
    bad = bytearray(data)
    bad[hdr + 5] ^= 0x40  # a position bit, hash left as written
    (tmp_path / "c.ck").write_bytes(bytes(bad))
    for case, mutate in (("out of range", lambda ids: ids.__setitem__(0, n + 5)),
                         ("duplicate", lambda ids: ids.__setitem__(0, ids[1])),
                         ("negative", lambda ids: ids.__setitem__(7, -1))):
        bad = bytearray(data)
        ids = np.frombuffer(bytes(bad[id_off:id_off + 4 * n]), np.int32).copy()
        mutate(ids)
        bad[id_off:id_off + 4 * n] = ids.tobytes()
        bad[hdr - 8:hdr] = struct.pack("<Q", _fnv1a(bytes(bad[hdr:])))
        (tmp_path / f"{case}.ck").write_bytes(bytes(bad))
    for name in ["c.ck", "out of range.ck", "duplicate.ck", "negative.ck"]:
        with pytest.raises(L.SphError) as e:
            b.Load(tmp_path / name)
        assert e.value.code == L.SPH_ERR_ARG, name
    assert "hash" in L.last_error() or "permutation" in L.last_error()
    after = b.state()
    assert b.CurrentStep == 1
    for key in before:
        assert np.array_equal(before[key], after[key]), key
    # the untouched file still loads
    b.Load(tmp_path / "s.ck")
    assert b.CurrentStep == 2
