#!/usr/bin/env python3
"""Particle-steps/s of sphugo's 2D SPH step on GB300.

Workload (the plain-FP64-at-scale case): N = 1,048,576 particles uniform in the
periodic unit box, blast u = 10 inside r < 0.1 (else 1), k = 32, Monahan
kernel, gamma 5/3, alpha 1, beta 2, dt = 2e-5, seeded SplitMix64 inputs.
`value` is the plain FP64 drop-in (SPH_PREC_FP64, bit-exact with the
reference's arithmetic) timed with CUDA events on the library's stream over K
steps after W warm-up steps, inputs resident in HBM (state > 1 GB, larger than
L2). `e2e` times the same steps through the public C ABI with the whole state
copied host->device and back every step from pinned host buffers. Extra
lines of the JSON report the FP64-fast and mixed forms and the 256-simulation
ensemble, each against the stated tolerances that the test-suite enforces.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Under torchrun (N > 1) every rank advances its own replica (a single
simulation does not shard without a halo exchange): value = all ranks'
particle-steps / the slowest rank's time.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_DEFAULT = 1_048_576
K_NEIGH = 32
DT = 2e-5
SEED = 2
METRIC = "particle-steps/s on 1 GB300: mixed/batched vs plain FP64 GPU at stated rel. error"
TOLERANCES = {"neighbour_sets": "bit-exact", "fp64": "bit-exact", "fp64_fast": 1e-12,
              "mixed_rho": 1e-5, "mixed_accel_normalised": 1e-4, "mixed_udot_normalised": 1e-4}

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


def ncu_traffic(kernel, form, n):
    """DRAM bytes per launch of a stage's kernel from the committed ncu
    summary (profiles/ncu_traffic.json), for the same form and size."""
    try:
        with open(os.path.join(ROOT, "profiles", "ncu_traffic.json")) as f:
            tab = json.load(f)
    except (OSError, ValueError):
        return None
    ent = tab.get(f"{kernel}/{form.lower()}/{n}")
    return ent.get("dram_bytes_per_launch") if ent else None


def ncu_field(stage, form, n, field):
    """Another figure of the committed ncu summary for a stage (or None)."""
    try:
        with open(os.path.join(ROOT, "profiles", "ncu_traffic.json")) as f:
            ent = json.load(f).get(f"{stage}/{form.lower()}/{n}")
    except (OSError, ValueError):
        return None
    return ent.get(field) if ent else None


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except OSError:
        return {}


def make_sim(n, precision, seed, tune=True):
    """The workload's simulation, autotuned (the tuner caches its choice)."""
    from sphugo_gb300 import ics
    from sphugo_gb300 import sim as S
    conf = ics.periodic_config(n, K_NEIGH, DT, precision)
    arrs = ics.uniform_blast(n, seed)
    sim = S.Simulation(conf, *arrs)
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
    """256 independent simulations: one graph per ensemble step vs one by one."""
    from sphugo_gb300 import ics
    from sphugo_gb300 import sim as S
    confs, arrays = ics.make_ensemble(nsims=nsims, precision=form)
    ntot = sum(len(a[0]) for a in arrays)
    e = S.Ensemble(confs, arrays)
    e.Step(2)
    ms = timed(e, steps)
    e.close()
    sims = [S.Simulation(c, *a) for c, a in zip(confs, arrays)]
    for s in sims:
        s.Step(2)
    t0 = time.perf_counter()
    for _ in range(steps):
        for s in sims:
            s.Step(1)
    sep = time.perf_counter() - t0
    for s in sims:
        s.close()
    graph = ntot * steps / (ms / 1e3)
    one = ntot * steps / sep
    return {"n_total": ntot, "sims": nsims, "graph": graph, "one_by_one": one, "ratio": graph / one}


def workload_case(kind, n, k, dt, seed, form, steps, grid_level=0):
    from sphugo_gb300 import ics
    from sphugo_gb300 import sim as S
    arrs = {"clustered": ics.clustered, "stress": ics.stress}[kind](n, seed)
    conf = ics.periodic_config(n, k, dt, form, grid_level=grid_level)
    sim = S.Simulation(conf, *arrs)
    tune = sim.Autotune()
    sim.Step(2)
    ms = timed(sim, steps)
    st = profile(sim, 2)
    hbm = sim.memory_bytes()
    sim.close()
    return {"value": n * steps / (ms / 1e3), "ms_per_step": ms / steps, "stages_ms": st, "tune": tune,
            "hbm_bytes": hbm}


def mixed_errors(arrays, n, k, dt):
    """Max and RMS relative errors of the mixed form against the FP64 form
    (which equals the oracle bit for bit) on identical inputs: the FP64 form
    runs five steps (so that particles move: viscosity and du/dt terms), then
    both forms take that state and evaluate the forces once; every particle.
    rho error relative to rho; |a| and du/dt errors over the particle's sum of
    the magnitudes of its neighbour terms (a zero sum demands a zero error)."""
    import numpy as np
    from sphugo_gb300 import ics
    from sphugo_gb300 import sim as S
    sims = {}
    for form in ("Exact", "Mixed"):
        s = S.Simulation(ics.periodic_config(n, k, dt, form), *arrays)
        s.Autotune()  # the cached choice of the timed run
        sims[form] = s
    sims["Exact"].Step(5)
    st = sims["Exact"].state()
    for s in sims.values():
        s.set_state(*(st[c] for c in ("x", "y", "vx", "vy", "u", "ax", "ay", "udot")))
        s.CalculateForces()
    e, m = sims["Exact"], sims["Mixed"]
    es, ed, (an, un) = e.state(), e.derived(), e.error_norms()
    ms, md = m.state(), m.derived()
    for s in sims.values():
        s.close()

    def ratio(err, norm):
        out = np.where(norm > 0, err / np.where(norm > 0, norm, 1.0), np.where(err == 0, 0.0, np.inf))
        return {"max": float(out.max()), "rms": float(np.sqrt(np.mean(out * out)))}
    return {
        "rho": ratio(np.abs(md["rho"] - ed["rho"]), np.abs(ed["rho"])),
        "accel_normalised": ratio(np.hypot(ms["ax"] - es["ax"], ms["ay"] - es["ay"]), an),
        "udot_normalised": ratio(np.abs(ms["udot"] - es["udot"]), un),
        "sample": f"all {n} particles, one force evaluation of both forms on the FP64 form's state after 5 steps",
    }


def e2e_run(sim, steps):
    """set_state from pinned host arrays + step + get_state, every step."""
    import numpy as np
    from sphugo_gb300 import _lib as L
    lib = L.load()
    n = sim.n
    bufs = [np.empty(n) for _ in range(8)]
    for b in bufs:
        L.check(lib.sph_host_register(b.ctypes.data, b.nbytes))
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
        for b in bufs:
            lib.sph_host_unregister(b.ctypes.data)
    return dt, 8 * 8 * n, 8 * 8 * n


def cpu_baseline(n, steps, threads, warm=1):
    """The oracle's faithful tree path (restating the reference's Step) on host cores."""
    from oracle import oracle as O
    from sphugo_gb300 import ics
    x, y, vx, vy, u = ics.uniform_blast(n, SEED)
    s = O.OracleSim(O.make_params(n, K_NEIGH, knn_mode=O.KNN_TREE, threads=threads, alpha=1.0, beta=2.0,
                                  dth=DT / 2), x, y, vx, vy, u)
    s.step(warm)  # step 0 evaluates forces twice; time regular steps only
    t0 = time.perf_counter()
    s.step(steps)
    return time.perf_counter() - t0


def run_reference(args, dist):
    """--impl reference: the reference's CPU algorithm (oracle port, all cores)."""
    if dist.rank != 0:
        return 0
    threads = os.cpu_count() or 1
    n = args.n or N_DEFAULT
    warm = max(1, args.warmup)
    steps = max(1, args.steps)
    secs = cpu_baseline(n, steps, threads, warm=warm)
    v = n * steps / secs
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "particle-steps/s", "n_gpus": args.gpus,
        "steps": steps, "warmup": warm, "ms_per_step": 1e3 * secs / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded SplitMix64)",
        "config": {"workload": f"uniform-blast N={n} k={K_NEIGH} periodic unit box dt={DT}",
                   "n": n, "k": K_NEIGH, "form": "reference tree search, FP64"},
        "cpu_baseline": {"value": v, "unit": "particle-steps/s", "cores": threads, "kind": "port",
                         "sample": f"{steps} full steps of N={n} after {warm} warm-up steps"},
        "e2e": {"value": v, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=60)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=0, help="override the particle count (testing only)")
    ap.add_argument("--no-extras", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--form", default="exact", choices=["exact", "fast", "mixed"],
                    help="arithmetic form of the headline run (profiling only; default exact)")
    args = ap.parse_args()
    dist = Dist()
    try:
        if args.impl == "reference":
            return run_reference(args, dist)
        return run_ours(args, dist)
    finally:
        dist.close()


def run_ours(args, dist):
    from sphugo_gb300 import _lib as L
    from sphugo_gb300 import build
    build.build()
    lib = L.load()
    n = args.n or N_DEFAULT
    K, W = max(1, args.steps), max(3, args.warmup)
    fp64_pk, fp32_pk, div_cost, sqrt_cost = C.c_double(0), C.c_double(0), C.c_double(0), C.c_double(0)
    L.check(lib.sph_probe_peaks(C.byref(fp64_pk), C.byref(fp32_pk), C.byref(div_cost), C.byref(sqrt_cost)))

    form = {"exact": "Exact", "fast": "Fast", "mixed": "Mixed"}[args.form]
    form_name = {"Exact": "SPH_PREC_FP64 (bit-exact)", "Fast": "SPH_PREC_FP64_FAST (FMA, <=1e-12)",
                 "Mixed": "SPH_PREC_MIXED (FP32 relative-coordinate Kahan sums, FP64 kNN decisions/h/integrator)"}[form]
    head_form = form
    sim = make_sim(n, form, SEED + 1000 * dist.rank)
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
    lo_frac, visc_frac = pair_statistics(sim, DT / 2)
    work = algorithmic(K_NEIGH, div_cost.value, sqrt_cost.value, lo_frac, visc_frac)
    ncells = 4 ** 10  # auto level for N = 2^20
    peaks = measured_peaks()
    hbm_peak = peaks.get("hbm_gbs")
    slot_peak = fp64_pk.value / 2 * 1e3  # G FP64 FMA issue slots per second
    roof = {}
    for st, t in stages.items():
        w = work[st]
        entry = {"ms": t}
        if "fp64_slots" in w and form != "Mixed":
            entry.update(bound="fp64", unit="G FP64-slot/s", achieved=w["fp64_slots"] * n / (t * 1e-3) / 1e9,
                         peak=slot_peak)
        else:
            b = w["bytes"] * n if w["bytes"] else 16 * ncells
            entry.update(bound="hbm", unit="GB/s", achieved=b / (t * 1e-3) / 1e9, peak=hbm_peak)
        if entry.get("peak"):
            entry["frac"] = entry["achieved"] / entry["peak"]
        if st == "knn":
            # no HBM or FP roofline binds the search: it is issue- and latency-bound
            entry["binding"] = "instruction issue / shared-memory latency"
            issue = ncu_field("knn", form, n, "issue_active_frac")
            if issue is not None:
                entry["ncu_issue_active_frac"] = issue
        roof[st] = entry
    dom = max(stages, key=stages.get)
    d = roof[dom]
    traffic = ncu_traffic(dom, form, n)
    roofline = {"kernel": dom, "bound": d["bound"], "achieved": d["achieved"], "peak": d["peak"],
                "unit": d["unit"], "frac": d.get("frac"), "traffic": traffic,
                "traffic_unit": "bytes per launch (ncu dram__bytes_read.sum + dram__bytes_write.sum)",
                "peak_source": ("FP64 FMA issue rate from the device probe run by this bench (2 flops per slot; "
                                "MEASURED_PEAKS.json has no FP64 figure)" if d["bound"] == "fp64"
                                else "MEASURED_PEAKS.json hbm_gbs"),
                "fp64_costs": {"div_slots": div_cost.value, "sqrt_slots": sqrt_cost.value,
                               "q_below_half": lo_frac, "approaching_pairs": visc_frac},
                "stages": roof}

    dt, h2d, d2h = e2e_run(sim, max(3, K // 2))
    e2e = {"value": n * max(3, K // 2) / dt, "unit": "particle-steps/s", "h2d_bytes_per_step": h2d,
           "d2h_bytes_per_step": d2h}
    sim.close()

    extras = {}
    if not args.no_extras and dist.rank == 0:
        from sphugo_gb300 import ics
        for form in ("Fast", "Mixed"):
            s2 = make_sim(n, form, SEED)
            s2.Step(W)
            t = timed(s2, K)
            extras[{"Fast": "fp64_fast", "Mixed": "mixed"}[form]] = {
                "value": n * K / (t / 1e3), "ms_per_step": t / K, "stages_ms": profile(s2, 3),
                "tune": s2.tune_report, "search_deferred": s2.search_stats()[1], "hbm_bytes": s2.memory_bytes()}
            s2.close()
        extras["mixed_vs_fp64"] = extras["mixed"]["value"] / value * dist.world
        extras["mixed"]["errors_vs_fp64"] = mixed_errors(ics.uniform_blast(n, SEED), n, K_NEIGH, DT)
        ens = {}
        for form in ("Exact", "Mixed"):
            ens[form.lower()] = ensemble_case(form, 5, 256)
        extras["ensemble_256"] = ens
        clu = {f.lower(): workload_case("clustered", 4_194_304, 32, 1e-5, 3, f, 5) for f in ("Exact", "Mixed")}
        clu["mixed_vs_fp64"] = clu["mixed"]["value"] / clu["exact"]["value"]
        clu["mixed"]["errors_vs_fp64"] = mixed_errors(ics.clustered(4_194_304, 3), 4_194_304, 32, 1e-5)
        extras["clustered_N4194304_k32"] = clu
        stress = {f.lower(): workload_case("stress", 16_777_216, 64, 1e-6, 4, f, 3) for f in ("Exact", "Mixed")}
        stress["mixed_vs_fp64"] = stress["mixed"]["value"] / stress["exact"]["value"]
        stress["mixed"]["errors_vs_fp64"] = mixed_errors(ics.stress(16_777_216, 4), 16_777_216, 64, 1e-6)
        extras["stress_N16777216_k64"] = stress

    cpu = None
    if not args.no_cpu and dist.rank == 0:
        threads = os.cpu_count() or 1
        ncpu = n
        secs = cpu_baseline(ncpu, 2, threads)
        cpu = {"value": ncpu * 2 / secs, "unit": "particle-steps/s", "cores": threads, "kind": "port",
               "sample": f"2 regular steps of the same workload (N={ncpu}) through the oracle's tree path"}

    if dist.rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": dist.world, "steps": K,
            "warmup": W, "ms_per_step": ms_max / K, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if head_form != "Mixed" else "f32+f64", "data": "synthetic (seeded SplitMix64 uniform blast)",
            "config": {"workload": f"uniform-blast N={n} k={K_NEIGH} periodic unit box dt={DT}, {head_form.lower()} form",
                       "n": n, "k": K_NEIGH, "form": form_name, "parallelism": "replicas",
                       "l2": "inputs larger than L2 (state + neighbour lists > 1 GB)"},
            "clocks": clocks, "e2e": e2e, "gpu_launches": kernels * K, "kernels_per_step": kernels,
            "roofline": roofline, "cpu_baseline": cpu, "tolerances": TOLERANCES,
            "peaks_probe": {"fp64_tflops": fp64_pk.value, "fp32_tflops": fp32_pk.value,
                            "fp64_div_slots": div_cost.value, "fp64_sqrt_slots": sqrt_cost.value}, "forms": extras,
            "tune": tune_report, "hbm_bytes": hbm_bytes,
            "search": {"queries": nq, "deferred_to_per_query": ndef,
                       "path": "group tiles + per-query for deferred" if ndef < nq else "per-query"},
        }
        print(json.dumps(line), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
