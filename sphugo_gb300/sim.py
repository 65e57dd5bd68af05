"""Host-side mirror of the reference's Go package ``sim`` (bbeni/sphugo).

Same names, argument meaning and error behaviour as ``sim/sph.go`` and
``sim/config-parser.go``; every call goes through the C ABI of
``include/sphgpu.h`` (libsphgpu.so) and the particle state stays on the GPU
between calls. Where Go returns ``(value, error)`` these functions return the
same pair; where Go panics they raise.
"""
from __future__ import annotations

import ctypes as C
import logging
from dataclasses import dataclass, field

import numpy as np

from . import _lib as L

log = logging.getLogger("sphugo_gb300")

DBL_MAX = L.DBL_MAX
OPEN = (-DBL_MAX, DBL_MAX)


@dataclass
class Vec2:
    X: float = 0.0
    Y: float = 0.0


@dataclass
class Reflections:
    L: float = -DBL_MAX
    R: float = DBL_MAX
    U: float = -DBL_MAX
    D: float = DBL_MAX


@dataclass
class UniformRectSpawner:
    """sim/config-parser.go:37-41; Spawn reseeds its generator per call."""
    UpperLeft: Vec2 = field(default_factory=Vec2)
    LowerRight: Vec2 = field(default_factory=lambda: Vec2(1.0, 1.0))
    NParticles: int = 1000


@dataclass
class PointSource:
    """sim/config-parser.go:43-47."""
    origin: Vec2 = field(default_factory=Vec2)
    rate: float = 0.0
    LastSpwned: float = 0.0


def MakeUniformRectSpawner() -> UniformRectSpawner:
    """sim/config-parser.go:50-55."""
    return UniformRectSpawner()


@dataclass
class SphConfig:
    """sim/config-parser.go:111-128 plus the constants the reference hard-codes."""
    NSteps: int = 10000
    DeltaTHalf: float = 0.001
    Gamma: float = 1.66666
    ParticleMass: float = 1.0
    Acceleration: Vec2 = field(default_factory=Vec2)
    Kernel: str = "Monahan"
    HorPeriodicity: tuple = OPEN
    VertPeriodicity: tuple = OPEN
    Reflections: Reflections = field(default_factory=Reflections)
    Sources: list = field(default_factory=list)
    Start: list = field(default_factory=list)
    Viewport: tuple = ((0.0, 0.0), (1.0, 1.0))
    # not expressible in the reference (NN_SIZE, sim/sph.go:379-383 constants)
    NeighbourCount: int = 32
    ViscosityAlpha: float = 0.75
    ViscosityBeta: float = 1.5
    ViscosityEtaSq: float = 0.01
    Precision: str = "Exact"   # Exact (bitwise FP64) | Fast (FP64) | Mixed
    GridLevel: int = 0

    def params(self) -> L.SphParams:
        p = L.load().sph_default_params()
        p.k = int(self.NeighbourCount)
        p.kernel = {"Monahan": L.KERNEL_MONAHAN, "Wendtland": L.KERNEL_WENDLAND}[self.Kernel]
        p.precision = {"Exact": L.PREC_FP64, "Fast": L.PREC_FP64_FAST, "Mixed": L.PREC_MIXED}[self.Precision]
        p.grid_level = int(self.GridLevel)
        p.gamma, p.mass, p.dth = self.Gamma, self.ParticleMass, self.DeltaTHalf
        p.accel[:] = (self.Acceleration.X, self.Acceleration.Y)
        p.hor[:] = tuple(self.HorPeriodicity)
        p.vert[:] = tuple(self.VertPeriodicity)
        r = self.Reflections
        p.refl[:] = (r.L, r.R, r.U, r.D)
        p.alpha, p.beta, p.etasq = self.ViscosityAlpha, self.ViscosityBeta, self.ViscosityEtaSq
        return p

    def to_c(self) -> L.SphConfig:
        c = L.SphConfig()
        L.load().sph_config_default(C.byref(c))
        c.params = self.params()
        c.nsteps = int(self.NSteps)
        c.viewport[:] = (*self.Viewport[0], *self.Viewport[1])
        if len(self.Start) > L.MAX_SPAWNERS or len(self.Sources) > L.MAX_SPAWNERS:
            raise ValueError("too many spawners")
        c.nstart = len(self.Start)
        for i, s in enumerate(self.Start):
            c.start[i].upper_left[:] = (s.UpperLeft.X, s.UpperLeft.Y)
            c.start[i].lower_right[:] = (s.LowerRight.X, s.LowerRight.Y)
            c.start[i].n = int(s.NParticles)
        c.nsources = len(self.Sources)
        for i, s in enumerate(self.Sources):
            c.sources[i].origin[:] = (s.origin.X, s.origin.Y)
            c.sources[i].rate = s.rate
            c.sources[i].last_spawned = s.LastSpwned
        return c

    @classmethod
    def from_c(cls, c: L.SphConfig) -> "SphConfig":
        p = c.params
        cfg = cls(
            NSteps=c.nsteps, DeltaTHalf=p.dth, Gamma=p.gamma, ParticleMass=p.mass,
            Acceleration=Vec2(p.accel[0], p.accel[1]),
            Kernel="Wendtland" if p.kernel == L.KERNEL_WENDLAND else "Monahan",
            HorPeriodicity=(p.hor[0], p.hor[1]), VertPeriodicity=(p.vert[0], p.vert[1]),
            Reflections=Reflections(*p.refl),
            Viewport=((c.viewport[0], c.viewport[1]), (c.viewport[2], c.viewport[3])),
            NeighbourCount=p.k, ViscosityAlpha=p.alpha, ViscosityBeta=p.beta, ViscosityEtaSq=p.etasq,
            Precision={L.PREC_FP64: "Exact", L.PREC_FP64_FAST: "Fast", L.PREC_MIXED: "Mixed"}[p.precision],
            GridLevel=p.grid_level,
        )
        for i in range(c.nstart):
            s = c.start[i]
            cfg.Start.append(UniformRectSpawner(Vec2(*s.upper_left), Vec2(*s.lower_right), int(s.n)))
        for i in range(c.nsources):
            s = c.sources[i]
            cfg.Sources.append(PointSource(Vec2(*s.origin), s.rate, s.last_spawned))
        return cfg



def _set_search(h, tiles):
    """True / 1: tiles of the default shape; 2: one tile per warp; 4 or 8:
    block tiles of that many warps; False / 0: per-query search."""
    L.check(L.load().sph_set_search(h, int(tiles)))


def _search_stats(h) -> tuple:
    q, d = C.c_int64(), C.c_int64()
    L.check(L.load().sph_search_stats(h, C.byref(q), C.byref(d)))
    return q.value, d.value

def _autotune(h, use_cache: bool) -> dict:
    import json
    buf = C.create_string_buffer(1024)
    L.check(L.load().sph_autotune(h, 1 if use_cache else 0, buf, len(buf)))
    return json.loads(buf.value.decode())


class ConfigError(Exception):
    """The error value of MakeConfigFromFile (reference message format)."""


def MakeConfig() -> SphConfig:
    """sim/config-parser.go:131-149."""
    return SphConfig()


def MakeConfigFromFile(path: str):
    """sim/config-parser.go:151-167: returns (SphConfig, error-or-None)."""
    c = L.SphConfig()
    buf = C.create_string_buffer(2048)
    rc = L.load().sph_config_load(path.encode(), C.byref(c), buf, len(buf))
    if rc != L.SPH_OK:
        return MakeConfig(), ConfigError(buf.value.decode(errors="replace"))
    return SphConfig.from_c(c), None


def spawn_start(conf: SphConfig, with_keys: bool = False):
    """Spawn(0) of every [[Start]] spawner: (x, y, vx, vy, u) arrays, and the
    draw keys Z (Particle.Z) as a sixth array when with_keys."""
    c = conf.to_c()
    n = int(L.load().sph_config_start_count(C.byref(c)))
    arrs = [np.zeros(n) for _ in range(5)]
    z = np.zeros(n, np.int64)
    L.check(L.load().sph_config_spawn(C.byref(c), *[L.dptr(a) for a in arrs], L.i64ptr(z)))
    return (*arrs, z) if with_keys else arrs


def _source_seed(step: int, index: int) -> int:
    """Generator seed of source `index` at step `step` (deterministic runs)."""
    return (0x5EED5EED00000000 + (step << 8) + index) & 0xFFFFFFFFFFFFFFFF


class Simulation:
    """sim/sph.go:14-21. Particle state lives on the GPU; accessors copy out."""

    def __init__(self, conf: SphConfig, x, y, vx=None, vy=None, u=None):
        self.Config = conf
        lib = L.load()
        x = np.ascontiguousarray(x, np.float64)
        y = np.ascontiguousarray(y, np.float64)
        n = len(x)
        if n == 0:
            raise RuntimeError("int Run(): Simulation not initialized!")  # sim/sph.go:93
        self.n = n
        self.k = int(conf.NeighbourCount)
        h = C.c_void_p()
        p = conf.params()
        L.check(lib.sph_create(C.byref(p), n, C.byref(h)))
        self._h = h
        z = np.zeros(n)
        f = lambda a: np.ascontiguousarray(z if a is None else a, np.float64)
        L.check(lib.sph_upload(h, L.dptr(x), L.dptr(y), L.dptr(f(vx)), L.dptr(f(vy)), L.dptr(f(u))))

    def close(self):
        if getattr(self, "_h", None):
            L.load().sph_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def CurrentStep(self) -> int:
        return int(L.load().sph_current_step(self._h))

    def Step(self, nsteps: int = 1):
        """sim/sph.go:64 (one call of Step per requested step). With point
        sources, each step first appends what they spawn at t = step * dt
        (sim/sph.go:71-85)."""
        if not self.Config.Sources:
            L.check(L.load().sph_step(self._h, int(nsteps)))
            return
        for _ in range(int(nsteps)):
            self._spawn_sources()
            L.check(L.load().sph_step(self._h, 1))

    def _spawn_sources(self):
        lib = L.load()
        step = self.CurrentStep
        t = float(step) * self.Config.DeltaTHalf * 2
        for i, src in enumerate(self.Config.Sources):
            cs = L.SphPointSource((C.c_double * 2)(src.origin.X, src.origin.Y), src.rate, src.LastSpwned)
            probe = L.SphPointSource.from_buffer_copy(cs)
            cnt = int(lib.sph_point_source_spawn(C.byref(probe), t, 0, None, None, None, None, None, None))
            if cnt <= 0:
                continue
            x, y, vx, vy, u = (np.zeros(cnt) for _ in range(5))
            z = np.zeros(cnt, np.int64)
            got = int(lib.sph_point_source_spawn(C.byref(cs), t, _source_seed(step, i), L.dptr(x), L.dptr(y),
                                                 L.dptr(vx), L.dptr(vy), L.dptr(u), L.i64ptr(z)))
            src.LastSpwned = cs.last_spawned
            L.check(lib.sph_append(self._h, got, L.dptr(x), L.dptr(y), L.dptr(vx), L.dptr(vy), L.dptr(u),
                                   L.i64ptr(z)))
            self.n += got

    def SetDrawKeys(self, z):
        """Particle.Z per particle (caller order) for Frame(); None = caller order."""
        if z is None:
            L.check(L.load().sph_set_draw_keys(self._h, None))
        else:
            zz = np.ascontiguousarray(z, np.int64)
            if len(zz) != self.n:
                raise ValueError("one draw key per particle")
            L.check(L.load().sph_set_draw_keys(self._h, L.i64ptr(zz)))

    def Frame(self, width: int = 1280, height: int = 720) -> np.ndarray:
        """sim/animator.go:55-103 CurrentFrame: (height, width, 4) NRGBA bytes."""
        out = np.empty((height, width, 4), np.uint8)
        L.check(L.load().sph_render(self._h, width, height, out.ctypes.data_as(C.POINTER(C.c_uint8))))
        return out

    def FrameToPNG(self, path: str, width: int = 1280, height: int = 720):
        """sim/animator.go:121-138 FrameToPNG for the current state."""
        write_png(path, self.Frame(width, height))

    def Run(self):
        """sim/sph.go:56-61."""
        for step in range(self.Config.NSteps):
            self.Step()
            log.info("Calculated step %d/%d", step, self.Config.NSteps)

    def CalculateForces(self):
        """sim/sph.go:403-435."""
        L.check(L.load().sph_forces(self._h))

    def Autotune(self, use_cache: bool = True) -> dict:
        """Picks the neighbour search's launch shape for this workload (before the first step)."""
        return _autotune(self._h, use_cache)

    def SetSearch(self, tiles=True):
        """Neighbour search path: True / 1 tiles of the default shape, 8 or 4
        block tiles of that many warps, 2 one tile per warp, False / 0 the
        per-query search; every path returns the same neighbour sets."""
        _set_search(self._h, tiles)

    def search_stats(self) -> tuple:
        """(queries, deferred to the per-query search) of the last force evaluation."""
        return _search_stats(self._h)

    def Save(self, path: str):
        """Checkpoint of the whole integrator state (resumes bit for bit)."""
        L.check(L.load().sph_save(self._h, str(path).encode()))

    def Load(self, path: str):
        L.check(L.load().sph_load(self._h, str(path).encode()))

    def _diag(self, sim=-1):
        out = np.zeros(4)
        L.check(L.load().sph_diagnostics(self._h, sim, L.dptr(out)))
        return out

    def TotalEnergy(self) -> float:
        return float(self._diag()[0])

    def TotalDensity(self) -> float:
        return float(self._diag()[1])

    def TotalMomentum(self) -> float:
        """As the reference computes it: |v| of the last particle (sim/sph.go:457-463)."""
        return float(self._diag()[2])

    def SumSpeed(self) -> float:
        return float(self._diag()[3])

    # ---- data access (Root.Particles fields), arrays in the caller's order
    def state(self) -> dict:
        names = ["x", "y", "vx", "vy", "u", "ax", "ay", "udot"]
        arrs = [np.empty(self.n) for _ in names]
        L.check(L.load().sph_get_state(self._h, *[L.dptr(a) for a in arrs]))
        return dict(zip(names, arrs))

    def set_state(self, x, y, vx, vy, u, ax, ay, udot):
        c = lambda a: np.ascontiguousarray(a, np.float64)
        L.check(L.load().sph_set_state(self._h, *[L.dptr(c(a)) for a in (x, y, vx, vy, u, ax, ay, udot)]))

    def derived(self) -> dict:
        arrs = [np.empty(self.n) for _ in range(3)]
        L.check(L.load().sph_get_derived(self._h, *[L.dptr(a) for a in arrs]))
        return dict(zip(["rho", "c", "h"], arrs))

    def memory_bytes(self) -> int:
        """Device memory this simulation holds (bytes)."""
        b = C.c_int64()
        L.check(L.load().sph_memory_bytes(self._h, C.byref(b)))
        return b.value

    def error_norms(self):
        """(anorm, unorm): per particle, the sums of the magnitudes of its
        neighbour terms in the acceleration and du/dt of the last evaluation
        (FP64 form only); the normalisers of the mixed form's errors."""
        a = np.empty(self.n)
        u = np.empty(self.n)
        L.check(L.load().sph_error_norms(self._h, L.dptr(a), L.dptr(u)))
        return a, u

    def neighbours(self):
        """(ids, NNDists, image codes), each (n, k); slot 0 = farthest."""
        n, k = self.n, self.k
        ids = np.empty(n * k, np.int64)
        d = np.empty(n * k)
        img = np.empty(n * k, np.int32)
        L.check(L.load().sph_get_neighbours(self._h, L.i64ptr(ids), L.dptr(d), L.i32ptr(img)))
        return ids.reshape(n, k), d.reshape(n, k), img.reshape(n, k)


def MakeSimulationFromConf(conf: SphConfig) -> Simulation:
    """sim/sph.go:41-54: spawns the [[Start]] particles and builds the simulation."""
    x, y, vx, vy, u, z = spawn_start(conf, with_keys=True)
    sim = Simulation(conf, x, y, vx, vy, u)
    sim.SetDrawKeys(z)
    return sim


def write_png(path: str, rgba: np.ndarray):
    """8-bit RGBA PNG (what image/png writes for an opaque NRGBA image holds
    the same pixels)."""
    import struct
    import zlib
    h, w = rgba.shape[:2]
    raw = b"".join(b"\x00" + rgba[r].tobytes() for r in range(h))

    def chunk(tag, data):
        return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)

    with open(path, "wb") as f:
        f.write(b"\x89PNG\r\n\x1a\n")
        f.write(chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 0)))
        f.write(chunk(b"IDAT", zlib.compress(raw, 6)))
        f.write(chunk(b"IEND", b""))


def MakeSimulation() -> Simulation:
    """sim/sph.go:23-30: default config with one default UniformRect spawner."""
    conf = MakeConfig()
    conf.Start = [MakeUniformRectSpawner()]
    return MakeSimulationFromConf(conf)


def MakeSimulationFromConfig(path: str):
    """sim/sph.go:32-39: returns (Simulation, error-or-None)."""
    conf, err = MakeConfigFromFile(path)
    if err is not None:
        return MakeSimulation(), err
    return MakeSimulationFromConf(conf), None


class Ensemble:
    """Independent simulations advanced together (one graph per step)."""

    def __init__(self, confs: list, arrays: list):
        lib = L.load()
        self.confs = confs
        counts = np.array([len(a[0]) for a in arrays], np.int64)
        self.counts = counts
        self.offsets = np.concatenate([[0], np.cumsum(counts)])
        self.n = int(counts.sum())
        self.k = int(confs[0].NeighbourCount)
        ps = (L.SphParams * len(confs))(*[c.params() for c in confs])
        h = C.c_void_p()
        L.check(lib.sph_ens_create(ps, L.i64ptr(counts), len(confs), C.byref(h)))
        self._h = h
        cat = [np.ascontiguousarray(np.concatenate([a[i] for a in arrays]), np.float64) for i in range(5)]
        L.check(lib.sph_upload(h, *[L.dptr(a) for a in cat]))

    def close(self):
        if getattr(self, "_h", None):
            L.load().sph_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def Step(self, nsteps: int = 1):
        L.check(L.load().sph_step(self._h, int(nsteps)))

    def CalculateForces(self):
        """Every simulation's CalculateForces (sim/sph.go:403) on its current
        state, without integrating."""
        L.check(L.load().sph_forces(self._h))

    def error_norms(self):
        """Per-particle normalisers of the mixed form's error statements (FP64 ensembles)."""
        a, u = np.empty(self.n), np.empty(self.n)
        L.check(L.load().sph_error_norms(self._h, L.dptr(a), L.dptr(u)))
        return a, u

    def Autotune(self, use_cache: bool = True) -> dict:
        return _autotune(self._h, use_cache)

    def SetSearch(self, tiles=True):
        _set_search(self._h, tiles)

    def search_stats(self) -> tuple:
        return _search_stats(self._h)

    def memory_bytes(self) -> int:
        """Device memory the ensemble holds (bytes)."""
        b = C.c_int64()
        L.check(L.load().sph_memory_bytes(self._h, C.byref(b)))
        return b.value

    def state(self) -> dict:
        names = ["x", "y", "vx", "vy", "u", "ax", "ay", "udot"]
        arrs = [np.empty(self.n) for _ in names]
        L.check(L.load().sph_get_state(self._h, *[L.dptr(a) for a in arrs]))
        return dict(zip(names, arrs))

    def derived(self) -> dict:
        arrs = [np.empty(self.n) for _ in range(3)]
        L.check(L.load().sph_get_derived(self._h, *[L.dptr(a) for a in arrs]))
        return dict(zip(["rho", "c", "h"], arrs))

    def neighbours(self):
        n, k = self.n, self.k
        ids = np.empty(n * k, np.int64)
        d = np.empty(n * k)
        img = np.empty(n * k, np.int32)
        L.check(L.load().sph_get_neighbours(self._h, L.i64ptr(ids), L.dptr(d), L.i32ptr(img)))
        return ids.reshape(n, k), d.reshape(n, k), img.reshape(n, k)

    def diagnostics(self, sim: int = -1):
        out = np.zeros(4)
        L.check(L.load().sph_diagnostics(self._h, sim, L.dptr(out)))
        return out
