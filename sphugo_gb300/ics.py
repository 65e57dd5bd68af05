"""Seeded synthetic workloads (initial conditions and physics settings).

The generators run on the host inside libsphgpu.so (SplitMix64 streams); these
wrappers return numpy arrays plus the matching SphConfig.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import _lib as L
from .sim import SphConfig


def uniform_blast(n: int, seed: int, u_bg=1.0, u_blast=10.0, r_blast=0.1):
    a = [np.empty(n) for _ in range(5)]
    L.check(L.load().sph_ic_uniform_blast(n, seed, u_bg, u_blast, r_blast, *[L.dptr(x) for x in a]))
    return a


def clustered(n: int, seed: int, nblobs=64, sig_min=0.005, sig_max=0.05, f_bg=0.2, u_bg=1.0, u_core=10.0):
    a = [np.empty(n) for _ in range(5)]
    L.check(L.load().sph_ic_clustered(n, seed, nblobs, sig_min, sig_max, f_bg, u_bg, u_core,
                                      *[L.dptr(x) for x in a]))
    return a


def stress(n: int, seed: int, side=0.1, f_in=0.99, u_bg=1.0, u_hot=100.0, r_hot=0.01):
    a = [np.empty(n) for _ in range(5)]
    L.check(L.load().sph_ic_stress(n, seed, side, f_in, u_bg, u_hot, r_hot, *[L.dptr(x) for x in a]))
    return a


def ensemble_sizes(nsims: int, seed: int, nmin=1000, nmax=65536, ublo=5.0, ubhi=50.0):
    counts = np.empty(nsims, np.int64)
    ub = np.empty(nsims)
    L.check(L.load().sph_ic_ensemble(nsims, seed, nmin, nmax, ublo, ubhi, L.i64ptr(counts), L.dptr(ub)))
    return counts, ub


def periodic_config(n: int, k: int = 32, dt: float = 1e-4, precision: str = "Exact", alpha=1.0, beta=2.0,
                    gamma=5.0 / 3.0, grid_level: int = 0, nsteps: int = 100) -> SphConfig:
    """The blast-wave physics of the workloads: unit periodic box, m = 1/N."""
    return SphConfig(NSteps=nsteps, DeltaTHalf=dt / 2, Gamma=gamma, ParticleMass=1.0 / n,
                     HorPeriodicity=(0.0, 1.0), VertPeriodicity=(0.0, 1.0), NeighbourCount=k,
                     ViscosityAlpha=alpha, ViscosityBeta=beta, Precision=precision, GridLevel=grid_level)


@dataclass
class Workload:
    name: str
    n: int
    k: int
    steps: int
    dt: float
    seed: int
    kind: str  # blast | clustered | stress


# the five synthetic workloads (sizes, seeds and step counts)
SMALL_BLAST = Workload("uniform-blast N=10000 k=32", 10_000, 32, 100, 1e-4, 1, "blast")
SCALE_BLAST = Workload("uniform-blast N=1048576 k=32", 1_048_576, 32, 200, 2e-5, 2, "blast")
CLUSTERED = Workload("clustered 64 blobs N=4194304 k=32", 4_194_304, 32, 50, 1e-5, 3, "clustered")
STRESS = Workload("stress 99% in 0.1^2 N=16777216 k=64", 16_777_216, 64, 20, 1e-6, 4, "stress")
ENSEMBLE_SIMS, ENSEMBLE_SEED = 256, 5


def make(w: Workload, precision="Exact", n: int | None = None, grid_level: int = 0):
    n = w.n if n is None else n
    if w.kind == "blast":
        arrs = uniform_blast(n, w.seed)
    elif w.kind == "clustered":
        arrs = clustered(n, w.seed)
    else:
        arrs = stress(n, w.seed)
    return periodic_config(n, w.k, w.dt, precision, grid_level=grid_level, nsteps=w.steps), arrs


def make_ensemble(nsims=ENSEMBLE_SIMS, seed=ENSEMBLE_SEED, precision="Exact", k=32, dt=1e-4):
    counts, ub = ensemble_sizes(nsims, seed)
    confs, arrays = [], []
    for s in range(nsims):
        n = int(counts[s])
        confs.append(periodic_config(n, k, dt, precision))
        arrays.append(uniform_blast(n, 1000 + s, 1.0, float(ub[s]), 0.1))
    return confs, arrays
