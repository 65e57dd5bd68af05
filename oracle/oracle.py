"""ctypes wrapper of the CPU oracle (TEST INFRASTRUCTURE).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import
this module; the product package never does. The C source it loads restates
the reference's hot path (bbeni/sphugo ``sim/core.go``,
``sim/nearest-neighbour.go``, ``sim/sph.go``); see ``sph_oracle.h`` for the
per-function citations and for what is and is not pinned.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liborc.so")
SRC = os.path.join(HERE, "sph_oracle.c")
SOURCES = [SRC, os.path.join(HERE, "workloads.c")]

KERNEL_MONAHAN = 0
KERNEL_WENDLAND = 1
KNN_TREE = 0
KNN_EXACT = 1
DBL_MAX = sys.float_info.max


def build(force: bool = False) -> str:
    """Compiles the oracle with contraction off (a*b+c stays two roundings)."""
    os.makedirs(os.path.dirname(LIB_PATH), exist_ok=True)
    deps = SOURCES + [os.path.join(HERE, "sph_oracle.h")]
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < max(map(os.path.getmtime, deps)):
        cmd = ["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC",
               "-shared", "-o", LIB_PATH, *SOURCES, "-lm"]
        subprocess.run(cmd, check=True)
    return LIB_PATH


class Params(C.Structure):
    _fields_ = [
        ("n", C.c_int32), ("k", C.c_int32), ("kernel", C.c_int32), ("knn_mode", C.c_int32),
        ("threads", C.c_int32), ("pad_", C.c_int32),
        ("gamma", C.c_double), ("mass", C.c_double), ("dth", C.c_double),
        ("accel", C.c_double * 2), ("hor", C.c_double * 2), ("vert", C.c_double * 2),
        ("refl", C.c_double * 4),
        ("alpha", C.c_double), ("beta", C.c_double), ("etasq", C.c_double),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
        i64p = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
        i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
        L.orc_create.restype = C.c_void_p
        L.orc_create.argtypes = [C.POINTER(Params), dp, dp, dp, dp, dp]
        L.orc_destroy.argtypes = [C.c_void_p]
        L.orc_set_knn_mode.argtypes = [C.c_void_p, C.c_int]
        L.orc_set_check_tree.argtypes = [C.c_void_p, C.c_int]
        L.orc_tree_exact_mismatches.argtypes = [C.c_void_p]
        L.orc_tree_exact_mismatches.restype = C.c_int64
        L.orc_step.argtypes = [C.c_void_p, C.c_int]
        L.orc_forces.argtypes = [C.c_void_p]
        L.orc_current_step.argtypes = [C.c_void_p]
        L.orc_get_state.argtypes = [C.c_void_p] + [dp] * 11
        L.orc_get_pred.argtypes = [C.c_void_p, dp, dp, dp]
        L.orc_get_neighbours.argtypes = [C.c_void_p, i64p, dp, i32p]
        L.orc_get_norms.argtypes = [C.c_void_p, dp, dp]
        L.orc_diagnostics.argtypes = [C.c_void_p, dp]
        L.orc_partition.argtypes = [dp, dp, C.c_int, C.c_int, C.c_double]
        L.orc_tree_count_outside.argtypes = [dp, dp, C.c_int]
        L.orc_hypot.argtypes = [C.c_double, C.c_double]
        L.orc_hypot.restype = C.c_double
        for f in (L.orc_knn_exact, L.orc_knn_brute):
            f.argtypes = [C.POINTER(Params), dp, dp, i64p, dp, i32p]
        for f in (L.orc_kernel_f, L.orc_kernel_df):
            f.argtypes = [C.c_int, C.c_double]
            f.restype = C.c_double
        L.orc_append.argtypes = [C.c_void_p, C.c_int, dp, dp, dp, dp, dp]
        L.orc_draw_order.argtypes = [C.c_int64, i64p, i64p]
        u8p = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")
        L.orc_render.argtypes = [C.c_int64, dp, dp, dp, C.c_double, i64p, C.c_int, C.c_int, u8p]
        L.orc_para_ramp.argtypes = [C.c_int, u8p]
        for f in (L.orc_kernel_fpref, L.orc_kernel_dfpref):
            f.argtypes = [C.c_int]
            f.restype = C.c_double
        L.orc_ic_uniform_blast.argtypes = [C.c_int64, C.c_uint64, C.c_double, C.c_double, C.c_double] + [dp] * 5
        L.orc_ic_clustered.argtypes = [C.c_int64, C.c_uint64, C.c_int32, C.c_double, C.c_double, C.c_double,
                                       C.c_double, C.c_double] + [dp] * 5
        L.orc_ic_stress.argtypes = [C.c_int64, C.c_uint64, C.c_double, C.c_double, C.c_double, C.c_double,
                                    C.c_double] + [dp] * 5
        L.orc_ic_ensemble.argtypes = [C.c_int32, C.c_uint64, C.c_int64, C.c_int64, C.c_double, C.c_double,
                                      i64p, dp]
        _lib = L
    return _lib


def make_params(n, k=32, *, kernel=KERNEL_MONAHAN, knn_mode=KNN_EXACT, threads=0,
                gamma=5.0 / 3.0, mass=None, dth=5e-5, accel=(0.0, 0.0),
                hor=(0.0, 1.0), vert=(0.0, 1.0),
                refl=(-DBL_MAX, DBL_MAX, -DBL_MAX, DBL_MAX),
                alpha=0.75, beta=1.5, etasq=0.01) -> Params:
    p = Params()
    p.n, p.k, p.kernel, p.knn_mode, p.threads = n, k, kernel, knn_mode, threads
    p.gamma = gamma
    p.mass = (1.0 / n) if mass is None else mass
    p.dth = dth
    p.accel[:] = accel
    p.hor[:] = hor
    p.vert[:] = vert
    p.refl[:] = refl
    p.alpha, p.beta, p.etasq = alpha, beta, etasq
    return p


def _c(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class OracleSim:
    """One simulation held by the C oracle (arrays in original particle order)."""

    def __init__(self, params: Params, x, y, vx=None, vy=None, u=None):
        n = params.n
        self.params = params
        self.n, self.k = n, params.k
        z = np.zeros(n)
        self._h = lib().orc_create(C.byref(params), _c(x), _c(y),
                                   _c(z if vx is None else vx), _c(z if vy is None else vy),
                                   _c(z if u is None else u))
        if not self._h:
            raise ValueError("orc_create failed")

    def close(self):
        if self._h:
            lib().orc_destroy(self._h)
            self._h = None

    __del__ = close

    def step(self, n=1):
        rc = lib().orc_step(self._h, n)
        if rc:
            raise RuntimeError(f"oracle step failed: status {rc}")

    def append(self, x, y, vx=None, vy=None, u=None):
        """Particles spawned during the run (sim/sph.go:71-85)."""
        m = len(x)
        z = np.zeros(m)
        rc = lib().orc_append(self._h, m, _c(x), _c(y), _c(z if vx is None else vx), _c(z if vy is None else vy),
                              _c(z if u is None else u))
        if rc:
            raise RuntimeError(f"oracle append failed: status {rc}")
        self.n += m
        self.params.n = self.n

    def forces(self):
        rc = lib().orc_forces(self._h)
        if rc:
            raise RuntimeError(f"oracle forces failed: status {rc}")

    def set_knn_mode(self, mode):
        lib().orc_set_knn_mode(self._h, mode)

    def set_check_tree(self, on=True):
        lib().orc_set_check_tree(self._h, 1 if on else 0)

    def tree_mismatches(self):
        return int(lib().orc_tree_exact_mismatches(self._h))

    @property
    def current_step(self):
        return int(lib().orc_current_step(self._h))

    def state(self):
        n = self.n
        names = ["x", "y", "vx", "vy", "u", "ax", "ay", "udot", "rho", "c", "h"]
        arrs = [np.empty(n) for _ in names]
        lib().orc_get_state(self._h, *arrs)
        return dict(zip(names, arrs))

    def pred(self):
        a = [np.empty(self.n) for _ in range(3)]
        lib().orc_get_pred(self._h, *a)
        return dict(zip(["vpx", "vpy", "upred"], a))

    def neighbours(self):
        """(ids, dist, img), each (n, k), slot 0 = farthest as in the reference."""
        n, k = self.n, self.k
        ids = np.empty(n * k, dtype=np.int64)
        d = np.empty(n * k)
        img = np.empty(n * k, dtype=np.int32)
        lib().orc_get_neighbours(self._h, ids, d, img)
        return ids.reshape(n, k), d.reshape(n, k), img.reshape(n, k)

    def norms(self):
        a, u = np.empty(self.n), np.empty(self.n)
        lib().orc_get_norms(self._h, a, u)
        return a, u

    def diagnostics(self):
        out = np.empty(3)
        lib().orc_diagnostics(self._h, out)
        return out


def draw_order(z):
    """Painting order of sim/animator.go:65-70 (QuickSort by -Z)."""
    z = np.ascontiguousarray(z, np.int64)
    order = np.empty(len(z), np.int64)
    lib().orc_draw_order(len(z), z, order)
    return order


def para_ramp():
    """gx.ParaRamp for every index: (256, 3) bytes."""
    out = np.empty((256, 3), np.uint8)
    for i in range(256):
        lib().orc_para_ramp(i, out[i])
    return out


def render(x, y, rho, mass, order, width=1280, height=720):
    """sim/animator.go:55-103 CurrentFrame as (height, width, 4) NRGBA bytes."""
    out = np.empty((height, width, 4), np.uint8)
    lib().orc_render(len(x), _c(x), _c(y), _c(rho), float(mass), np.ascontiguousarray(order, np.int64),
                     width, height, out)
    return out


def knn_exact(params: Params, x, y, brute=False):
    """Exact kNN, slot 0 = nearest; returns (ids, d2, img) each (n, k)."""
    n, k = params.n, params.k
    ids = np.empty(n * k, dtype=np.int64)
    d2 = np.empty(n * k)
    img = np.empty(n * k, dtype=np.int32)
    f = lib().orc_knn_brute if brute else lib().orc_knn_exact
    rc = f(C.byref(params), _c(x), _c(y), ids, d2, img)
    if rc:
        raise RuntimeError(f"oracle knn failed: status {rc}")
    return ids.reshape(n, k), d2.reshape(n, k), img.reshape(n, k)


def partition(xs, ys, orientation, middle):
    """sim/core.go:126 Partition; returns (len(a), len(b), xs, ys)."""
    xs, ys = _c(xs).copy(), _c(ys).copy()
    a = lib().orc_partition(xs, ys, len(xs), orientation, middle)
    return a, len(xs) - a, xs, ys


def tree_count_outside(x, y):
    return int(lib().orc_tree_count_outside(_c(x), _c(y), len(x)))


def hypot(p, q):
    return lib().orc_hypot(p, q)


# ---- seeded synthetic workloads (workloads.c), the same arrays as the
# library's sph_ic_* generators


def _ic(fn, n, *args):
    a = [np.empty(n) for _ in range(5)]
    rc = fn(n, *args, *a)
    if rc:
        raise ValueError(f"initial-condition recipe rejected its arguments (status {rc})")
    return a


def uniform_blast(n, seed, u_bg=1.0, u_blast=10.0, r_blast=0.1):
    return _ic(lib().orc_ic_uniform_blast, n, seed, u_bg, u_blast, r_blast)


def clustered(n, seed, nblobs=64, sig_min=0.005, sig_max=0.05, f_bg=0.2, u_bg=1.0, u_core=10.0):
    return _ic(lib().orc_ic_clustered, n, seed, nblobs, sig_min, sig_max, f_bg, u_bg, u_core)


def stress(n, seed, side=0.1, f_in=0.99, u_bg=1.0, u_hot=100.0, r_hot=0.01):
    return _ic(lib().orc_ic_stress, n, seed, side, f_in, u_bg, u_hot, r_hot)


def ensemble_sizes(nsims, seed, nmin=1000, nmax=65536, ublo=5.0, ubhi=50.0):
    counts = np.empty(nsims, np.int64)
    ub = np.empty(nsims)
    rc = lib().orc_ic_ensemble(nsims, seed, nmin, nmax, ublo, ubhi, counts, ub)
    if rc:
        raise ValueError(f"ensemble recipe rejected its arguments (status {rc})")
    return counts, ub
