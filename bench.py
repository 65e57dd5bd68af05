#!/usr/bin/env python3
"""Particle-steps/s of sphugo's 2D SPH step on GB300.

Headline workload (the configuration the metric is quoted on): N = 4,194,304
particles drawn from a seeded mixture of 64 Gaussian blobs (centres uniform in
the periodic unit box, sigma log-uniform in [0.005, 0.05]) plus a 20 %
uniform background, u = 10 within one sigma of a blob centre (else 1), zero
velocities, k = 32, Monahan kernel, gamma 5/3, alpha 1, beta 2, dt = 1e-5;
the workload's full run is 50 steps.

`value` is the plain FP64 drop-in (SPH_PREC_FP64, bit-exact with the
reference's arithmetic), timed with CUDA events on the library's stream over K
steps after W warm-up steps, inputs resident in HBM (state and neighbour lists
of several GB, larger than L2). `e2e` times the same steps through the public
C ABI with the whole state copied host->device and back every step from pinned
host buffers. `mixed` is the mixed form (FP32 relative-coordinate Kahan sums,
FP64 kNN decisions, smoothing lengths and integrator) on the same workload:
its rate, its ratio to the FP64 form, and the max / RMS relative errors of
rho, a and du/dt against the FP64 form, stated after five steps and after the
workload's full 50-step run. `forms` adds the uniform blast at N = 1,048,576,
the 256-simulation ensemble and the N = 16,777,216, k = 64 stress case.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

`--impl reference` times the reference's algorithm on the host cores: the
oracle's restatement of the reference's tree search and step (no GPU library
is loaded), on the same workload, config and metric.

Under torchrun (N > 1) every rank advances its own replica (a single
simulation does not shard without a halo exchange): value = all ranks'
particle-steps / the slowest rank's time.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# the headline workload: clustered blobs, N = 2^22, k = 32, dt = 1e-5, seed 3, 50-step run
HEAD_KIND, HEAD_N, HEAD_K, HEAD_DT, HEAD_SEED, HEAD_RUN = "clustered", 4_194_304, 32, 1e-5, 3, 50
METRIC = "particle-steps/s on 1 GB300: mixed/batched vs plain FP64 GPU at stated rel. error"
TOLERANCES = {"neighbour_sets": "bit-exact", "fp64": "bit-exact", "fp64_fast": 1e-12,
              "mixed_rho": 1e-5, "mixed_accel_normalised": 1e-4, "mixed_udot_normalised": 1e-4}
FORM_NAMES = {"Exact": "SPH_PREC_FP64 (bit-exact)", "Fast": "SPH_PREC_FP64_FAST (FMA, <=1e-12)",
              "Mixed": "SPH_PREC_MIXED (FP32 relative-coordinate Kahan sums, FP64 kNN decisions/h/integrator)"}
HBM_FALLBACK_GBS = 6800.0


def head_config(n):
    """The workload's `config`, identical in both arms."""
    return {"workload": f"clustered 64 blobs + 20% background N={n} k={HEAD_K} periodic unit box dt={HEAD_DT}",
            "n": n, "k": HEAD_K, "parallelism": "replicas",
            "l2": "inputs larger than L2 (state and neighbour lists of several GB)"}


def auto_level(n):
    """The library's automatic binning level (one to four particles per finest cell)."""
    lv = math.floor(0.5 * math.log2(max(n, 2) / 2.0) + 0.5)
    return int(min(max(lv, 1), 14))


# Algorithmic work per particle and force evaluation. Streaming stages count
# HBM bytes. FP64 stages count the FP64 operations of the reference's own
# formulas in FMA issue slots: an add, multiply or compare is one slot, a
# correctly rounded division or square root costs `div` / `sqrt` slots as
# priced by the device probe in the same run (the FP64 pipe's real cost of
# those operations). Work the GPU form does beyond the formulas (recomputing
# distances, reciprocals shared by two quotients) is not counted.
#   density (sim/sph.go:306-323, :423-429, and the kNN's FP64 squared
#     distance and final square root of each kept neighbour,
#     sim/nearest-neighbour.go:64-80): per neighbour d2 = ((p+o)-q)^2 7 ops,
#     sqrt, div (q = d/h), kernel F (4 ops for q < 0.5, 3 + one division by 3
#     otherwise), 1 add, and the force's dF(q) (4 ops for q < 0.5, 2
#     otherwise; evaluated here and handed over); per particle h = sqrt,
#     rho (3 + div), c (3 + sqrt), cA (2 + div).
#   force (sim/sph.go:327-401 plus the leapfrog update :121-193):
#     per neighbour vAB 2, rAB 4, dot 3,
#     (Pi + cA) + cB 2, x/y terms 2 x (2 + div + 1), du/dt term 2; per
#     approaching pair (dot < 0) cAB, rhoAB, hAB 6, r2 3, mu 2 + div,
#     Pi 5 + div; per particle the prefactor 3 + div, outputs 6, integrator 12.
# The FP64 density and force compute part of their FP64 operations with
# integer instructions, bit-identical to the hardware's (sph_selftest_fp64emu
# checks every one against __dmul_rn, __ddiv_rn and __dsqrt_rn), so that the
# integer pipes work beside the FP64 unit, which issues two lanes per SM per
# clock. Their achieved FP64-slot rate can therefore exceed the FP64 unit's
# own issue ceiling (frac > 1).
FP64_NOTE = ("the density computes its multiplications, square roots and divisions, the force its "
             "multiplications and divisions, with integer instructions beside the FP64 unit (bit-identical "
             "to the hardware instructions; sph_selftest_fp64emu), so frac can exceed 1 against the FP64 "
             "unit's issue ceiling; ncu on the clustered workload at N = 1,048,576: force FP64 pipe 67 %, "
             "ALU pipe 52 %, issue slots 56 % busy; density 72 %, 62 %, 63 %")


def algorithmic(k, div, sqrt, lo_frac, visc_frac):
    kern_f = lo_frac * 4 + (1 - lo_frac) * (3 + div)
    kern_df = lo_frac * 4 + (1 - lo_frac) * 2
    dens = k * (7 + sqrt + div + kern_f + kern_df + 1) + sqrt + (3 + div) + (3 + sqrt) + (2 + div)
    force = k * (2 + 4 + 3 + 2 + 2 * (3 + div) + 2) + k * visc_frac * (6 + 3 + 2 + div + 5 + div) \
        + (3 + div) + 6 + 12
    return {
        "bin": {"bytes": 32 + 8},
        "scan": {"bytes": None},  # per cell: 16 B, filled in below
        "permute": {"bytes": 76 + 8 + 4 + 92},
        "knn": {"bytes": 16 + 4 * k + 8},
        "density": {"fp64_slots": dens, "bytes": 16 + 8 * k + 4 * k + 56},
        "force_integrate": {"fp64_slots": force, "bytes": 80 + 4 * k + 8 * k},
    }


def pair_statistics(sim, dth):
    """Fraction of neighbour pairs with q < 0.5 and of approaching pairs
    (v_AB . r_AB < 0, with VPred = Vel + VDot dth), which set the taken
    branches of the kernel functions and of the viscosity term."""
    import numpy as np
    st = sim.state()
    ids, dist, img = sim.neighbours()
    h = dist[:, :1]
    lo = float(np.mean(dist < 0.5 * h))
    vpx, vpy = st["vx"] + st["ax"] * dth, st["vy"] + st["ay"] * dth
    L = 1.0
    ia, ib = img // 3 - 1, img % 3 - 1
    rx = (st["x"][ids] - ia * L) - st["x"][:, None]
    ry = (st["y"][ids] - ib * L) - st["y"][:, None]
    dot = (vpx[ids] - vpx[:, None]) * rx + (vpy[ids] - vpy[:, None]) * ry
    return lo, float(np.mean(dot < 0))


def env_rank():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


class Dist:
    """Barrier and max-over-ranks for torchrun launches (gloo, CPU tensors)."""

    def __init__(self):
        self.rank, self.world, self.local = env_rank()
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, v: float) -> float:
        if not self.pg:
            return v
        import torch
        t = torch.tensor([v], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


def max_over_ranks(values):
    """Reduction the timed region uses (max over ranks)."""
    return max(values)


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 50 ms; the summary
    keeps the samples taken inside the marked timed region (the nearest ones
    when the region is shorter than the sampling interval)."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []  # (arrival time, line)
        self.t0 = self.t1 = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except OSError:
            self.proc = None
            return
        deadline = time.time() + 5.0  # sampling is running before the timed region starts
        while not self.lines and time.time() < deadline and self.proc.poll() is None:
            time.sleep(0.01)

    def mark_start(self):
        self.t0 = time.time()

    def mark_end(self):
        self.t1 = time.time()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.time(), line.strip()))

    def stop(self):
        if self.proc:
            time.sleep(0.1)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        lines = self.lines
        if self.t0 is not None and self.t1 is not None and lines:
            inside = [x for x in lines if self.t0 <= x[0] <= self.t1 + 0.05]
            if not inside:  # shorter than the interval: the samples nearest the region
                mid = 0.5 * (self.t0 + self.t1)
                inside = sorted(lines, key=lambda x: abs(x[0] - mid))[:2]
            lines = inside
        for _, ln in lines:
            f = [v.strip() for v in ln.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx = max(mx, float(f[1]))
            except ValueError:
                continue
            for nm, v in zip(names, f[3:7]):
                if v.lower() in ("active", "1", "yes"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def ncu_entry(stage, form, kind):
    """The committed ncu capture of a stage's kernel (profiles/ncu_traffic.json):
    key stage/form/workload kind; None when there is none."""
    try:
        with open(os.path.join(ROOT, "profiles", "ncu_traffic.json")) as f:
            return json.load(f).get(f"{stage}/{form.lower()}/{kind}")
    except (OSError, ValueError):
        return None


def ncu_traffic(stage, form, kind, n):
    """DRAM bytes per launch of a stage at n particles: the capture's own
    figure scaled by particle count (the stages stream per-particle data and
    gather neighbours from L2, so traffic grows in proportion), and a note of
    where the figure comes from."""
    ent = ncu_entry(stage, form, kind)
    if not ent or not ent.get("dram_bytes_per_launch"):
        return None, None
    scale = n / ent["n"]
    note = (f"ncu dram__bytes_read.sum + dram__bytes_write.sum of {ent['kernel']} on the {kind} workload at "
            f"N={ent['n']} (commit {ent.get('commit', '?')}, profiles/ncu_traffic.json), x{scale:g} for N={n}")
    return ent["dram_bytes_per_launch"] * scale, note


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def hbm_peak():
    """Measured HBM copy bandwidth (GB/s) and its source."""
    p = measured_peaks()
    for key in ("hbm_gbs", "hbm_GBps", "hbm_copy_gbs"):
        if isinstance(p.get(key), (int, float)) and p[key] > 0:
            return float(p[key]), "MEASURED_PEAKS.json " + key
    return HBM_FALLBACK_GBS, "fallback (MEASURED_PEAKS.json absent): 6.8 TB/s, an earlier GB300 copy measurement"


def library_inputs(kind, n, seed):
    from sphugo_gb300 import ics
    return {"clustered": ics.clustered, "stress": ics.stress, "blast": ics.uniform_blast}[kind](n, seed)


def make_sim(kind, n, k, dt, seed, form, tune=True, level=0):
    """A workload's simulation, autotuned (the tuner caches its choice)."""
    from sphugo_gb300 import ics
    from sphugo_gb300 import sim as S
    sim = S.Simulation(ics.periodic_config(n, k, dt, form, grid_level=level), *library_inputs(kind, n, seed))
    sim.tune_report = sim.Autotune() if tune else None
    return sim


def timed(sim, steps):
    from sphugo_gb300 import _lib as L
    ms = C.c_double(0)
    L.check(L.load().sph_step_timed(sim._h, steps, C.byref(ms)))
    return ms.value


def profile(sim, steps=3):
    from sphugo_gb300 import _lib as L
    import numpy as np
    out = np.zeros(L.NUM_STAGES)
    L.check(L.load().sph_step_profiled(sim._h, steps, L.dptr(out)))
    return dict(zip(L.STAGES, out.tolist()))


def ensemble_case(form, steps, nsims):
    """256 independent simulations: one graph per ensemble step, against the
    same simulations as separate handles (each on its own stream). Two
    baselines: every handle's step enqueued back to back with one wait per
    ensemble step (sph_step_async, then sph_synchronize on each), and the
    plain blocking sph_step per handle."""
    from sphugo_gb300 import _lib as L
    from sphugo_gb300 import ics
    from sphugo_gb300 import sim as S
    lib = L.load()
    confs, arrays = ics.make_ensemble(nsims=nsims, precision=form)
    ntot = sum(len(a[0]) for a in arrays)
    e = S.Ensemble(confs, arrays)
    tune = e.Autotune()
    e.Step(2)
    ms = timed(e, steps)
    e.close()
    sims = [S.Simulation(c, *a) for c, a in zip(confs, arrays)]
    for s in sims:
        s.Autotune()  # cached per size class, as the ensemble's own choice
        s.Step(2)
    t0 = time.perf_counter()
    for _ in range(steps):
        for s in sims:
            L.check(lib.sph_step_async(s._h, 1))
        for s in sims:
            L.check(lib.sph_synchronize(s._h))
    sep_async = time.perf_counter() - t0
    t0 = time.perf_counter()
    for _ in range(steps):
        for s in sims:
            s.Step(1)
    sep_sync = time.perf_counter() - t0
    for s in sims:
        s.close()
    graph = ntot * steps / (ms / 1e3)
    one = ntot * steps / sep_async
    return {"n_total": ntot, "sims": nsims, "graph": graph, "one_by_one": one, "ratio": graph / one,
            "one_by_one_blocking": ntot * steps / sep_sync, "ratio_vs_blocking": graph * sep_sync / (ntot * steps),
            "tune": tune,
            "baseline": "each simulation its own handle and stream, every handle's step enqueued back to back, "
                        "one wait per ensemble step"}


def errors_on_state(st, n, k, dt):
    """Max and RMS relative errors of the mixed form against the FP64 form
    (which equals the oracle bit for bit) when both evaluate the forces of
    the same state once; every particle. rho error relative to rho; |a| and
    du/dt errors over the particle's sum of the magnitudes of its neighbour
    terms (a zero sum demands a zero error)."""
    import numpy as np
    from sphugo_gb300 import ics
    from sphugo_gb300 import sim as S
    out = {}
    for form in ("Exact", "Mixed"):
        s = S.Simulation(ics.periodic_config(n, k, dt, form), st["x"], st["y"], st["vx"], st["vy"], st["u"])
        s.Autotune()  # the cached choice of the timed run
        s.set_state(*(st[c] for c in ("x", "y", "vx", "vy", "u", "ax", "ay", "udot")))
        s.CalculateForces()
        out[form] = (s.state(), s.derived(), s.error_norms() if form == "Exact" else None)
        s.close()
    (es, ed, (an, un)), (ms, md, _) = out["Exact"], out["Mixed"]

    def ratio(err, norm):
        r = np.where(norm > 0, err / np.where(norm > 0, norm, 1.0), np.where(err == 0, 0.0, np.inf))
        return {"max": float(r.max()), "rms": float(np.sqrt(np.mean(r * r)))}
    return {
        "rho": ratio(np.abs(md["rho"] - ed["rho"]), np.abs(ed["rho"])),
        "accel_normalised": ratio(np.hypot(ms["ax"] - es["ax"], ms["ay"] - es["ay"]), an),
        "udot_normalised": ratio(np.abs(ms["udot"] - es["udot"]), un),
    }


def mixed_errors(kind, n, k, dt, seed, fp64_steps=5, run_steps=None):
    """The mixed form's stated errors on a workload: on the FP64 form's state
    after `fp64_steps` steps (particles moving: viscosity and du/dt terms
    active), and, with `run_steps`, on the mixed form's own state at the end
    of the workload's full run."""
    from sphugo_gb300 import ics
    from sphugo_gb300 import sim as S
    arrays = library_inputs(kind, n, seed)
    res = {}
    s = S.Simulation(ics.periodic_config(n, k, dt, "Exact"), *arrays)
    s.Autotune()
    s.Step(fp64_steps)
    st = s.state()
    s.close()
    res["after_fp64_steps"] = errors_on_state(st, n, k, dt)
    res["after_fp64_steps"]["sample"] = (f"all {n} particles, one force evaluation of both forms on the FP64 "
                                         f"form's state after {fp64_steps} steps")
    if run_steps:
        m = S.Simulation(ics.periodic_config(n, k, dt, "Mixed"), *arrays)
        m.Autotune()
        m.Step(run_steps)
        st = m.state()
        m.close()
        res["after_full_run"] = errors_on_state(st, n, k, dt)
        res["after_full_run"]["sample"] = (f"all {n} particles, one force evaluation of both forms on the mixed "
                                           f"form's state at the end of its full {run_steps}-step run")
    return res


def workload_case(kind, n, k, dt, seed, form, steps):
    sim = make_sim(kind, n, k, dt, seed, form)
    sim.Step(2)
    ms = timed(sim, steps)
    st = profile(sim, 2)
    hbm = sim.memory_bytes()
    nq, nd = sim.search_stats()
    sim.close()
    return {"value": n * steps / (ms / 1e3), "ms_per_step": ms / steps, "stages_ms": st, "tune": sim.tune_report,
            "hbm_bytes": hbm, "search_deferred": nd}


def e2e_run(sim, steps):
    """set_state from pinned host arrays + step + get_state, every step. The
    arrays live in pinned memory from sph_host_alloc, as a caller keeping its
    per-step state for the library would hold them."""
    import numpy as np
    from sphugo_gb300 import _lib as L
    lib = L.load()
    n = sim.n
    raw = []
    for _ in range(8):
        p = C.c_void_p()
        L.check(lib.sph_host_alloc(8 * n, C.byref(p)))
        raw.append(p)
    bufs = [np.ctypeslib.as_array(C.cast(p, C.POINTER(C.c_double)), shape=(n,)) for p in raw]
    try:
        st = sim.state()
        for b, k in zip(bufs, ["x", "y", "vx", "vy", "u", "ax", "ay", "udot"]):
            b[:] = st[k]
        ptrs = [L.dptr(b) for b in bufs]
        t0 = time.perf_counter()
        for _ in range(steps):
            L.check(lib.sph_set_state(sim._h, *ptrs))
            L.check(lib.sph_step(sim._h, 1))
            L.check(lib.sph_get_state(sim._h, *ptrs))
        dt = time.perf_counter() - t0
    finally:
        del bufs
        for p in raw:
            lib.sph_host_free(p)
    return dt, 8 * 8 * n, 8 * 8 * n


def cpu_tree_run(n, steps, threads, warm):
    """The oracle's faithful restatement of the reference's Step (tree build,
    tree kNN with the sorted queue, density, force, leapfrog) on host cores,
    on the headline workload built by the oracle's own copy of the recipe
    (no GPU library is loaded). Returns seconds for `steps` regular steps
    after `warm` warm-up steps (step 0 evaluates the forces twice)."""
    from oracle import oracle as O
    x, y, vx, vy, u = O.clustered(n, HEAD_SEED)
    s = O.OracleSim(O.make_params(n, HEAD_K, knn_mode=O.KNN_TREE, threads=threads, alpha=1.0, beta=2.0,
                                  dth=HEAD_DT / 2), x, y, vx, vy, u)
    s.step(warm)
    t0 = time.perf_counter()
    s.step(steps)
    secs = time.perf_counter() - t0
    s.close()
    return secs


def run_reference(args, dist):
    """--impl reference: the reference's CPU algorithm (oracle port, all cores)."""
    if dist.rank != 0:
        return 0
    threads = os.cpu_count() or 1
    n = args.n or HEAD_N
    warm = max(1, args.warmup)
    steps = max(1, args.steps)
    secs = cpu_tree_run(n, steps, threads, warm)
    v = n * steps / secs
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "particle-steps/s", "n_gpus": args.gpus,
        "steps": steps, "warmup": warm, "ms_per_step": 1e3 * secs / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded SplitMix64 clustered blobs)",
        "config": head_config(n), "form": "the reference's tree search and step, FP64 (oracle restatement)",
        "cpu_baseline": {"value": v, "unit": "particle-steps/s", "cores": threads, "kind": "port",
                         "sample": f"{steps} full steps of the N={n} workload after {warm} warm-up steps, "
                                   f"OpenMP over the per-particle loops"},
        "e2e": {"value": v, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=0, help="override the particle count (testing only)")
    ap.add_argument("--no-extras", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--form", default="exact", choices=["exact", "fast", "mixed"],
                    help="arithmetic form of the headline run (profiling only; default exact)")
    ap.add_argument("--no-mixed", action="store_true", help="skip the mixed form's line (profiling only)")
    ap.add_argument("--no-tune", action="store_true",
                    help="no autotuning: default search shape at the binning level --level (profiling only)")
    ap.add_argument("--level", type=int, default=0, help="binning level with --no-tune (0: automatic)")
    args = ap.parse_args()
    dist = Dist()
    try:
        if args.impl == "reference":
            return run_reference(args, dist)
        return run_ours(args, dist)
    finally:
        dist.close()


def stage_rooflines(stages, work, n, form, level, slot_peak, hbm):
    roof = {}
    for st, t in stages.items():
        w = work[st]
        entry = {"ms": t}
        if "fp64_slots" in w and form != "Mixed":
            entry.update(bound="fp64", unit="G FP64-slot/s", achieved=w["fp64_slots"] * n / (t * 1e-3) / 1e9,
                         peak=slot_peak)
        else:
            b = w["bytes"] * n if w["bytes"] else 16 * 4 ** level
            entry.update(bound="hbm", unit="GB/s", achieved=b / (t * 1e-3) / 1e9, peak=hbm)
        entry["frac"] = entry["achieved"] / entry["peak"]
        if st == "knn":
            # no HBM or FP roofline binds the search: it is issue- and latency-bound
            entry["binding"] = "instruction issue / shared-memory and L2 latency"
        if entry["bound"] == "fp64":
            entry["binding"] = "FP64 unit and integer pipes together (see roofline.fp64_note)"
        roof[st] = entry
    return roof


def run_ours(args, dist):
    from sphugo_gb300 import _lib as L
    from sphugo_gb300 import build
    build.build()
    lib = L.load()
    n = args.n or HEAD_N
    K, W = max(1, args.steps), max(3, args.warmup)
    fp64_pk, fp32_pk, div_cost, sqrt_cost = C.c_double(0), C.c_double(0), C.c_double(0), C.c_double(0)
    L.check(lib.sph_probe_peaks(C.byref(fp64_pk), C.byref(fp32_pk), C.byref(div_cost), C.byref(sqrt_cost)))
    hbm, hbm_src = hbm_peak()
    slot_peak = fp64_pk.value / 2 * 1e3  # G FP64 FMA issue slots per second

    form = {"exact": "Exact", "fast": "Fast", "mixed": "Mixed"}[args.form]
    sim = make_sim(HEAD_KIND, n, HEAD_K, HEAD_DT, HEAD_SEED + 1000 * dist.rank, form, tune=not args.no_tune,
                   level=args.level if args.no_tune else 0)
    tune_report = sim.tune_report
    sim.Step(W)
    kernels = int(lib.sph_kernels_per_step(sim._h))
    clk = ClockSampler(dist.local)
    clk.start()
    dist.barrier()
    clk.mark_start()
    ms = timed(sim, K)
    clk.mark_end()
    dist.barrier()
    clocks = clk.stop()
    ms_max = dist.max(ms)
    value = n * K * dist.world / (ms_max / 1e3)

    stages = profile(sim, 3)
    nq, ndef = sim.search_stats()
    hbm_bytes = sim.memory_bytes()
    lo_frac, visc_frac = pair_statistics(sim, HEAD_DT / 2)
    work = algorithmic(HEAD_K, div_cost.value, sqrt_cost.value, lo_frac, visc_frac)
    level = args.level if args.no_tune and args.level else auto_level(n) + int((tune_report or {}).get("level_delta", 0))
    roof = stage_rooflines(stages, work, n, form, level, slot_peak, hbm)
    dom = max(stages, key=stages.get)
    d = roof[dom]
    traffic, traffic_note = ncu_traffic(dom, form, HEAD_KIND, n)
    roofline = {"kernel": dom, "bound": d["bound"], "achieved": d["achieved"], "peak": d["peak"],
                "unit": d["unit"], "frac": d["frac"], "traffic": traffic,
                "traffic_unit": "bytes per launch", "traffic_source": traffic_note,
                "peak_source": ("FP64 FMA issue rate from the device probe run by this bench (2 flops per slot; "
                                "MEASURED_PEAKS.json has no FP64 figure)" if d["bound"] == "fp64" else hbm_src),
                "fp64_costs": {"div_slots": div_cost.value, "sqrt_slots": sqrt_cost.value,
                               "q_below_half": lo_frac, "approaching_pairs": visc_frac},
                "stages": roof}
    if d["bound"] == "fp64":
        roofline["fp64_note"] = FP64_NOTE

    e2e_steps = max(3, K // 2)
    dt, h2d, d2h = e2e_run(sim, e2e_steps)
    e2e = {"value": n * e2e_steps / dt, "unit": "particle-steps/s", "h2d_bytes_per_step": h2d,
           "d2h_bytes_per_step": d2h}
    sim.close()

    mixed = None
    if dist.rank == 0 and form == "Exact" and not args.no_mixed:
        sm = make_sim(HEAD_KIND, n, HEAD_K, HEAD_DT, HEAD_SEED, "Mixed")
        sm.Step(W)
        t = timed(sm, K)
        mstages = profile(sm, 3)
        mixed = {"value": n * K / (t / 1e3), "ms_per_step": t / K, "stages_ms": mstages,
                 "roofline_stages": stage_rooflines(mstages, work, n, "Mixed", level, slot_peak, hbm),
                 "tune": sm.tune_report, "search_deferred": sm.search_stats()[1], "hbm_bytes": sm.memory_bytes()}
        sm.close()
        mixed["mixed_vs_fp64"] = mixed["value"] / value * dist.world
        mixed["errors_vs_fp64"] = mixed_errors(HEAD_KIND, n, HEAD_K, HEAD_DT, HEAD_SEED, 5, HEAD_RUN)

    extras = {}
    if not args.no_extras and dist.rank == 0:
        blast = {f.lower(): workload_case("blast", 1_048_576, 32, 2e-5, 2, f, 20) for f in ("Exact", "Fast", "Mixed")}
        blast["mixed_vs_fp64"] = blast["mixed"]["value"] / blast["exact"]["value"]
        blast["mixed"]["errors_vs_fp64"] = mixed_errors("blast", 1_048_576, 32, 2e-5, 2)
        extras["uniform_blast_N1048576_k32"] = blast
        extras["ensemble_256"] = {f.lower(): ensemble_case(f, 5, 256) for f in ("Exact", "Mixed")}
        stress = {f.lower(): workload_case("stress", 16_777_216, 64, 1e-6, 4, f, 3) for f in ("Exact", "Mixed")}
        stress["mixed_vs_fp64"] = stress["mixed"]["value"] / stress["exact"]["value"]
        stress["mixed"]["errors_vs_fp64"] = mixed_errors("stress", 16_777_216, 64, 1e-6, 4)
        extras["stress_N16777216_k64"] = stress

    cpu = None
    if not args.no_cpu and dist.rank == 0:
        threads = os.cpu_count() or 1
        secs = cpu_tree_run(n, 2, threads, 1)
        cpu = {"value": n * 2 / secs, "unit": "particle-steps/s", "cores": threads, "kind": "port",
               "sample": f"2 regular steps of the same workload (N={n}) through the oracle's restatement of the "
                         f"reference's tree search and step, after step 0"}

    if dist.rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": dist.world, "steps": K,
            "warmup": W, "ms_per_step": ms_max / K, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if form != "Mixed" else "f32+f64",
            "data": "synthetic (seeded SplitMix64 clustered blobs)",
            "config": head_config(n), "form": FORM_NAMES[form],
            "clocks": clocks, "e2e": e2e, "gpu_launches": kernels * K, "kernels_per_step": kernels,
            "roofline": roofline, "cpu_baseline": cpu, "mixed": mixed,
            "mixed_vs_fp64": mixed["mixed_vs_fp64"] if mixed else None, "tolerances": TOLERANCES,
            "peaks_probe": {"fp64_tflops": fp64_pk.value, "fp32_tflops": fp32_pk.value,
                            "fp64_div_slots": div_cost.value, "fp64_sqrt_slots": sqrt_cost.value,
                            "hbm_gbs": hbm, "hbm_source": hbm_src},
            "forms": extras, "tune": tune_report, "hbm_bytes": hbm_bytes,
            "search": {"queries": nq, "deferred_to_per_query": ndef,
                       "path": "group tiles + per-query for deferred" if ndef < nq else "per-query"},
        }
        print(json.dumps(line), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
