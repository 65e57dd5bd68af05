"""ctypes binding of libsphgpu.so (the C ABI declared in include/sphgpu.h).

The shared library is built in-tree by ``sphugo_gb300.build``; loading fails
loudly when it is missing -- there is no CPU fallback behind this module.
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libsphgpu.so")
DBL_MAX = sys.float_info.max

SPH_OK = 0
SPH_ERR_ARG = -1
SPH_ERR_CUDA = -2
SPH_ERR_NOMEM = -3
SPH_ERR_KNN = -4
SPH_ERR_SENTINEL = -5
SPH_ERR_RANGE = -6
SPH_ERR_CONFIG = -7
SPH_ERR_STATE = -8

KERNEL_MONAHAN = 0
KERNEL_WENDLAND = 1
PREC_FP64 = 0
PREC_MIXED = 1
PREC_FP64_FAST = 2

# every entry point include/sphgpu.h declares
EXPORTS = [
    "sph_default_params", "sph_abi_version", "sph_last_error", "sph_device_count",
    "sph_create", "sph_ens_create", "sph_destroy", "sph_upload", "sph_set_state",
    "sph_get_state", "sph_get_derived", "sph_error_norms", "sph_memory_bytes", "sph_get_neighbours", "sph_step",
    "sph_step_async", "sph_forces",
    "sph_synchronize", "sph_current_step", "sph_num_particles", "sph_host_register",
    "sph_host_unregister", "sph_host_alloc", "sph_host_free", "sph_diagnostics", "sph_ic_uniform_blast", "sph_ic_clustered",
    "sph_ic_stress", "sph_ic_ensemble", "sph_config_default", "sph_config_load",
    "sph_config_start_count", "sph_config_spawn", "sph_point_source_spawn",
    "sph_step_timed", "sph_step_profiled", "sph_kernels_per_step", "sph_set_search", "sph_search_stats",
    "sph_probe_peaks", "sph_append", "sph_set_draw_keys", "sph_render", "sph_para_ramp",
    "sph_density_noalloc", "sph_autotune", "sph_save", "sph_load", "sph_selftest_division", "sph_selftest_fp64emu",
]
NOALLOC_MAX_N = 8192
NOALLOC_MAX_K = 32
NUM_STAGES = 6
STAGES = ["bin", "scan", "permute", "knn", "density", "force_integrate"]


class SphParams(C.Structure):
    _fields_ = [
        ("k", C.c_int32), ("kernel", C.c_int32), ("precision", C.c_int32),
        ("grid_level", C.c_int32),
        ("gamma", C.c_double), ("mass", C.c_double), ("dth", C.c_double),
        ("accel", C.c_double * 2), ("hor", C.c_double * 2), ("vert", C.c_double * 2),
        ("refl", C.c_double * 4),
        ("alpha", C.c_double), ("beta", C.c_double), ("etasq", C.c_double),
    ]


MAX_SPAWNERS = 64


class SphRectSpawner(C.Structure):
    _fields_ = [("upper_left", C.c_double * 2), ("lower_right", C.c_double * 2), ("n", C.c_int64)]


class SphPointSource(C.Structure):
    _fields_ = [("origin", C.c_double * 2), ("rate", C.c_double), ("last_spawned", C.c_double)]


class SphConfig(C.Structure):
    _fields_ = [
        ("params", SphParams), ("nsteps", C.c_int32), ("nstart", C.c_int32),
        ("nsources", C.c_int32), ("pad_", C.c_int32), ("viewport", C.c_double * 4),
        ("start", SphRectSpawner * MAX_SPAWNERS), ("sources", SphPointSource * MAX_SPAWNERS),
    ]


class SphError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


_lib = None


def load() -> C.CDLL:
    """Loads the in-tree library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: build it with `python -m sphugo_gb300.build`")
    L = C.CDLL(LIB_PATH)
    vp = C.c_void_p
    dp = C.POINTER(C.c_double)
    i64p = C.POINTER(C.c_int64)
    i32p = C.POINTER(C.c_int32)
    L.sph_default_params.restype = SphParams
    L.sph_default_params.argtypes = []
    L.sph_abi_version.restype = C.c_int32
    L.sph_last_error.restype = C.c_char_p
    L.sph_device_count.argtypes = [i32p]
    L.sph_create.argtypes = [C.POINTER(SphParams), C.c_int64, C.POINTER(vp)]
    L.sph_ens_create.argtypes = [C.POINTER(SphParams), i64p, C.c_int32, C.POINTER(vp)]
    L.sph_destroy.argtypes = [vp]
    L.sph_upload.argtypes = [vp] + [dp] * 5
    L.sph_set_state.argtypes = [vp] + [dp] * 8
    L.sph_get_state.argtypes = [vp] + [dp] * 8
    L.sph_get_derived.argtypes = [vp] + [dp] * 3
    L.sph_error_norms.argtypes = [vp] + [dp] * 2
    L.sph_memory_bytes.argtypes = [vp, i64p]
    L.sph_get_neighbours.argtypes = [vp, i64p, dp, i32p]
    L.sph_step.argtypes = [vp, C.c_int32]
    L.sph_step_async.argtypes = [vp, C.c_int32]
    L.sph_forces.argtypes = [vp]
    L.sph_synchronize.argtypes = [vp]
    L.sph_current_step.argtypes = [vp]
    L.sph_current_step.restype = C.c_int32
    L.sph_num_particles.argtypes = [vp]
    L.sph_num_particles.restype = C.c_int64
    L.sph_host_register.argtypes = [vp, C.c_int64]
    L.sph_host_unregister.argtypes = [vp]
    L.sph_host_alloc.argtypes = [C.c_int64, C.POINTER(vp)]
    L.sph_host_free.argtypes = [vp]
    L.sph_diagnostics.argtypes = [vp, C.c_int32, dp]
    L.sph_ic_uniform_blast.argtypes = [C.c_int64, C.c_uint64, C.c_double, C.c_double, C.c_double] + [dp] * 5
    L.sph_ic_clustered.argtypes = [C.c_int64, C.c_uint64, C.c_int32, C.c_double, C.c_double, C.c_double,
                                   C.c_double, C.c_double] + [dp] * 5
    L.sph_ic_stress.argtypes = [C.c_int64, C.c_uint64, C.c_double, C.c_double, C.c_double, C.c_double,
                                C.c_double] + [dp] * 5
    L.sph_ic_ensemble.argtypes = [C.c_int32, C.c_uint64, C.c_int64, C.c_int64, C.c_double, C.c_double,
                                  i64p, dp]
    L.sph_config_default.argtypes = [C.POINTER(SphConfig)]
    L.sph_config_load.argtypes = [C.c_char_p, C.POINTER(SphConfig), C.c_char_p, C.c_int32]
    L.sph_config_start_count.argtypes = [C.POINTER(SphConfig)]
    L.sph_config_start_count.restype = C.c_int64
    L.sph_config_spawn.argtypes = [C.POINTER(SphConfig)] + [dp] * 5 + [C.POINTER(C.c_int64)]
    L.sph_point_source_spawn.argtypes = [C.POINTER(SphPointSource), C.c_double, C.c_uint64] + [dp] * 5 + [C.POINTER(C.c_int64)]
    L.sph_point_source_spawn.restype = C.c_int64
    L.sph_step_timed.argtypes = [vp, C.c_int32, dp]
    L.sph_step_profiled.argtypes = [vp, C.c_int32, dp]
    L.sph_kernels_per_step.argtypes = [vp]
    L.sph_kernels_per_step.restype = C.c_int32
    L.sph_set_search.argtypes = [vp, C.c_int32]
    L.sph_append.argtypes = [vp, C.c_int64, dp, dp, dp, dp, dp, C.POINTER(C.c_int64)]
    L.sph_set_draw_keys.argtypes = [vp, C.POINTER(C.c_int64)]
    L.sph_render.argtypes = [vp, C.c_int32, C.c_int32, C.POINTER(C.c_uint8)]
    L.sph_para_ramp.argtypes = [C.POINTER(C.c_uint8)]
    L.sph_search_stats.argtypes = [vp, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
    L.sph_probe_peaks.argtypes = [dp, dp, dp, dp]
    L.sph_autotune.argtypes = [vp, C.c_int32, C.c_char_p, C.c_int32]
    L.sph_save.argtypes = [vp, C.c_char_p]
    L.sph_selftest_division.argtypes = [C.c_int64, C.c_uint64, i64p]
    L.sph_selftest_fp64emu.argtypes = [C.c_int64, C.c_uint64, i64p]
    L.sph_load.argtypes = [vp, C.c_char_p]
    L.sph_density_noalloc.argtypes = [C.POINTER(SphParams), vp, vp, C.c_int32, vp, vp, vp, vp, vp]
    _lib = L
    return L


def last_error() -> str:
    return load().sph_last_error().decode(errors="replace")


def check(rc: int) -> None:
    if rc != SPH_OK:
        raise SphError(rc, last_error())


def dptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"], "need contiguous float64"
    return a.ctypes.data_as(C.POINTER(C.c_double))


def i64ptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype == np.int64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.POINTER(C.c_int64))


def i32ptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype == np.int32 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.POINTER(C.c_int32))
