/*
 * sphgpu.h -- C ABI of the GB300-native SPH step (libsphgpu.so).
 *
 * This is the drop-in boundary under the Go package sim of bbeni/sphugo: each
 * entry point replaces one piece of the reference's Go API (cited per
 * function, paths within that project). A cgo shim binds these directly; the
 * library owns all device memory, keeps particle state resident in HBM between
 * calls and copies the caller's host arrays in and out, so the caller keeps
 * ownership of its buffers. Every function returns an int status (0 = ok,
 * negative = error class) and leaves a message for sph_last_error().
 * Plain pointers and sizes only; nothing here depends on a GPU being present
 * until a handle is created.
 */
#ifndef SPHGPU_H
#define SPHGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SPHGPU_ABI_VERSION 1

/* status codes */
#define SPH_OK 0
#define SPH_ERR_ARG -1        /* invalid argument (the reference would panic or misbehave) */
#define SPH_ERR_CUDA -2       /* CUDA runtime error / no device */
#define SPH_ERR_NOMEM -3      /* device allocation failed */
#define SPH_ERR_KNN -4        /* neighbour search failed (see sph_last_error) */
#define SPH_ERR_SENTINEL -5   /* a k-th neighbour lies beyond the reference's 0.4 queue sentinel */
#define SPH_ERR_RANGE -6      /* q = r/h outside [0,1] or non-finite state */
#define SPH_ERR_CONFIG -7     /* .sph-config parse / validation error */
#define SPH_ERR_STATE -8      /* call out of order (e.g. step before upload) */

/* kernels: sim/sph.go:258 Monahan2D, sim/sph.go:284 Wendtland2D */
#define SPH_KERNEL_MONAHAN 0
#define SPH_KERNEL_WENDLAND 1

/* arithmetic form of density and force */
#define SPH_PREC_FP64 0       /* plain FP64 drop-in: the reference's operation order, bit for bit */
#define SPH_PREC_MIXED 1      /* FP32 relative-coordinate sums with compensation; FP64 kNN decisions, h and integrator */
#define SPH_PREC_FP64_FAST 2  /* FP64 with contraction and per-particle reciprocals (within 1e-12 of SPH_PREC_FP64);
                               * on GB300 slower than SPH_PREC_FP64, whose kernels move part of their FP64
                               * work to the integer pipes */

/* Simulation parameters: the fields of SphConfig that the step reads
 * (sim/config-parser.go:111-128) plus the constants the reference hard-codes
 * (NN_SIZE sim/core.go:14; alpha, beta, etaSq sim/sph.go:379-383). */
typedef struct sph_params {
    int32_t k;           /* neighbours per particle (NN_SIZE), 1..128 */
    int32_t kernel;      /* SPH_KERNEL_* (SphConfig.Kernel) */
    int32_t precision;   /* SPH_PREC_* */
    int32_t grid_level;  /* finest binning level (cells per axis = 2^level); 0 = automatic */
    double gamma;        /* SphConfig.Gamma */
    double mass;         /* SphConfig.ParticleMass */
    double dth;          /* SphConfig.DeltaTHalf */
    double accel[2];     /* SphConfig.Acceleration */
    double hor[2];       /* SphConfig.HorPeriodicity; {-DBL_MAX, DBL_MAX} = open */
    double vert[2];      /* SphConfig.VertPeriodicity */
    double refl[4];      /* SphConfig.Reflections L, R, U, D */
    double alpha, beta, etasq; /* artificial viscosity (reference: 0.75, 1.5, 0.01) */
} sph_params;

typedef struct sph_handle sph_handle;

/* Defaults of sim/config-parser.go:131-149 MakeConfig (open bounds, gamma
 * 1.66666, mass 1, DeltaTHalf 0.001, Monahan) with k = 32 and the
 * reference's viscosity constants. */
sph_params sph_default_params(void);

/* Library / device info. */
int32_t sph_abi_version(void);
const char *sph_last_error(void);           /* thread-local message of the last failure */
int sph_device_count(int32_t *count);

/* ---- lifetime ---- */
/* One simulation of n particles. Replaces sim/sph.go:41 MakeSimulationFromConf
 * (the particles themselves come with sph_upload). */
int sph_create(const sph_params *p, int64_t n, sph_handle **out);
/* An ensemble of nsims independent simulations advanced together, each with
 * its own parameters and particle count; particle arrays passed to the other
 * calls are the concatenation of the simulations in order. k and precision
 * must agree across the ensemble. No reference counterpart (the reference
 * runs one Simulation per process). */
int sph_ens_create(const sph_params *params, const int64_t *counts, int32_t nsims, sph_handle **out);
int sph_destroy(sph_handle *h);

/* ---- state transfer (host arrays in the caller's particle order) ---- */
/* Sets positions, velocities and specific internal energies and resets the
 * step counter to 0, as building Root.Particles does (sim/sph.go:41-53).
 * vx, vy, u may be NULL (zero). */
int sph_upload(sph_handle *h, const double *x, const double *y, const double *vx,
               const double *vy, const double *u);
/* Replaces the full integrator state (including the last accelerations and
 * du/dt that the next drift reads) without touching the step counter, for a
 * caller that owns the state on the host between steps. */
int sph_set_state(sph_handle *h, const double *x, const double *y, const double *vx,
                  const double *vy, const double *u, const double *ax, const double *ay,
                  const double *udot);
/* Particle.Pos, Vel, E, VDot, EDot; any pointer may be NULL. */
int sph_get_state(sph_handle *h, double *x, double *y, double *vx, double *vy, double *u,
                  double *ax, double *ay, double *udot);
/* Particle.Rho, C and NNDists[0] (the smoothing length) of the last force
 * evaluation; any pointer may be NULL. */
int sph_get_derived(sph_handle *h, double *rho, double *c, double *hsml);
/* Per particle (caller order), the sums of the magnitudes of its neighbour
 * terms of the last force evaluation: |r_AB| |(Pi + cA + cB) dF / r| |f| for the
 * acceleration and |v_AB . r_AB dF| |cA m| for du/dt (sim/sph.go:343-398), the
 * normalisers of the mixed form's error statements. SPH_PREC_FP64 handles
 * only; any pointer may be NULL. No reference counterpart. */
int sph_error_norms(sph_handle *h, double *anorm, double *unorm);
/* Device memory the handle holds, in bytes: state and evaluation arrays,
 * neighbour lists, cell tables and scratch (not the on-demand export buffer of
 * sph_get_neighbours). No reference counterpart. */
int sph_memory_bytes(sph_handle *h, int64_t *bytes);
/* Particle.NearestNeighbours / NNDists in the reference layout
 * (sim/core.go:36-38): n*k entries, slot 0 = the farthest neighbour; ids are
 * particle indices in the caller's order; dist may be NULL; img (may be
 * NULL) is the periodic image code (i+1)*3+(j+1) of the offset (i*dX, j*dY)
 * used by sim/nearest-neighbour.go:57-61. */
int sph_get_neighbours(sph_handle *h, int64_t *ids, double *dist, int32_t *img);

/* ---- stepping ---- */
/* sim/sph.go:64 (*Simulation).Step, nsteps times; step 0 performs the extra
 * force evaluation of sim/sph.go:89-103. Runs as captured CUDA graphs. */
int sph_step(sph_handle *h, int32_t nsteps);
/* sim/sph.go:403 CalculateForces on the current positions and predicted
 * velocities / energies (without integrating). */
int sph_forces(sph_handle *h);
/* sph_step without the wait: enqueues nsteps steps on the handle's stream
 * and returns. Device-side errors of those steps (kNN, sentinel, range) are
 * reported by the next sph_synchronize, sph_step or sph_forces. Lets a caller
 * that drives many handles keep them all queued (Step itself blocks,
 * sim/sph.go:64-198). No reference counterpart. */
int sph_step_async(sph_handle *h, int32_t nsteps);
/* Waits for the handle's queued work and reports any device-side error it
 * raised (the status sph_step would have returned). */
int sph_synchronize(sph_handle *h);
int32_t sph_current_step(const sph_handle *h);
int64_t sph_num_particles(const sph_handle *h);

/* ---- checkpoint / resume (no reference counterpart) ----
 * sph_save writes a versioned binary file: a header (sizes, step counter,
 * binning level, a hash of the parameters and simulation sizes) and the
 * integrator state in the device's storage order, so that a run resumed with
 * sph_load on a handle created with the same parameters continues bit for
 * bit in every arithmetic form. */
int sph_save(sph_handle *h, const char *path);
int sph_load(sph_handle *h, const char *path);

/* Append particles to a single simulation, as Step does with the particles
 * its sources spawn (sim/sph.go:71-85: Spawn(t) then append to
 * Root.Particles). They take caller indices n .. n+count-1, zero
 * acceleration and du/dt, and join the binning at the next evaluation; the
 * arrays grow like a Go slice (x1.5) and the step graphs are captured again.
 * vx, vy, u may be NULL (zero); z (may be NULL) gives their draw keys
 * (Particle.Z) for sph_render. */
int sph_append(sph_handle *h, int64_t count, const double *x, const double *y, const double *vx,
               const double *vy, const double *u, const int64_t *z);

/* ---- frames (sim/animator.go:55-103 CurrentFrame, gx/graphics.go) ----
 * Draw keys per caller index (Particle.Z; n values, NULL = caller order):
 * disks are painted in descending Z (the reference sorts by -Z), ties by
 * caller index, so the smallest Z ends on top. */
int sph_set_draw_keys(sph_handle *h, const int64_t *z);
/* gx.ParaRamp (gx/graphics.go:156-164) for every index 0..255 as NRGBA bytes
 * (1024 bytes): the colour table the frames use. No device needed. */
int sph_para_ramp(uint8_t *rgba);
/* Renders the current state into rgba (width*height*4 bytes, NRGBA, row y =
 * Pos.Y*height from the top): black background, a disk of radius 4 pixels per
 * particle at (Pos.X*width, Pos.Y*height) with the reference's float32 pixel
 * test, coloured by ParaRamp(min(rho/(m N 10)*256, 255)) from the densities
 * of the last force evaluation (0 for particles that have none yet). The
 * reference's canvas is 1280 x 720. Single simulations only. */
int sph_render(sph_handle *h, int32_t width, int32_t height, uint8_t *rgba);

/* ---- measurement (no reference counterpart) ---- */
#define SPH_NUM_STAGES 6   /* bin (incl. prep/bbox), scan, permute, knn, density, force+integrate */
/* sph_step with the device time between CUDA events recorded on the
 * handle's stream before the first and after the last step, in ms. */
int sph_step_timed(sph_handle *h, int32_t nsteps, double *ms);
/* nsteps steps (step 0's extra evaluation excluded from the timing) through
 * a graph that carries event nodes between the stages; stage_ms receives the
 * per-step mean device time of each stage. */
int sph_step_profiled(sph_handle *h, int32_t nsteps, double stage_ms[SPH_NUM_STAGES]);
/* Kernel launches of one regular step (graph kernel nodes). */
int32_t sph_kernels_per_step(sph_handle *h);
/* Neighbour search path (no reference counterpart): tiles of candidate
 * records in shared memory scanned by one thread per query, the queries they
 * cannot settle finished by the per-query search. 1 (default) = the default
 * tile shape for k (block tiles of 8 warps = 256 consecutive particles for
 * k <= 37, of 4 warps for k <= 80, else one tile per warp); 4 or 8 = block
 * tiles of that many warps; 2 = one tile per warp (32 particles); 0 =
 * per-query search for every particle. The neighbour sets and every FP64
 * result are identical on every path; the mixed form's FP32 sums may differ
 * in the last bits (they follow the list order). SPH_ERR_ARG for a shape
 * that k does not allow. */
int sph_set_search(sph_handle *h, int32_t tiles);
/* Queries of the last force evaluation and how many of them the group-tile
 * search left to the per-query search (all of them with tiles off). */
int sph_search_stats(sph_handle *h, int64_t *queries, int64_t *deferred);
/* Autotuner (no reference counterpart): on a freshly uploaded state (before
 * the first step) it times forces-only evaluations over a small grid of the
 * neighbour search's shape (search path and tile shape: block tiles of 8 or
 * 4 warps, one tile per warp, or the per-query search; cell side / search
 * radius factor, automatic binning level -1..+1, or -1..+2 for clustered
 * data), keeps the fastest, restores the
 * uploaded state and caches the choice per (particle count in half octaves,
 * k, arithmetic form, single/ensemble, distribution class from the spread of
 * smoothing lengths) in the text file named by SPHGPU_TUNE_CACHE (default
 * $HOME/.cache/sphgpu/tune.txt). With use_cache the cached choice is applied
 * without timing. Results do not depend on the choice; only speed does.
 * report (may be NULL) receives a one-line JSON summary. */
int sph_autotune(sph_handle *h, int32_t use_cache, char *report, int32_t report_len);
/* Arithmetic throughput probe on the current device: FP64 FMA and FP32 FMA
 * in TFLOP/s (2 flops per FMA), from independent FMA chains, and the cost of
 * one correctly rounded FP64 division and square root in FP64 FMA issue
 * slots (time per operation / time per FMA, at full occupancy). Any output
 * pointer may be NULL. */
int sph_probe_peaks(double *fp64_tflops, double *fp32_tflops, double *div_cost, double *sqrt_cost);

/* ---- allocation-free neighbour search and density ----
 * No counterpart in the reference. For callers that cannot call cudaMalloc
 * (a host framework that owns the device memory pool, or a latency-critical
 * loop where an allocation may synchronise the device): the exact periodic
 * kNN and density of one small particle set (the SPH_PREC_FP64 arithmetic of
 * a force evaluation), with every intermediate array in a static device
 * scratch area of about 8 MB that each GPU loading this library holds until
 * the process exits. x, y (n each) and the outputs are device-accessible
 * pointers; any output may be NULL: nbr_ids / nbr_dist (n*k, slot 0 =
 * farthest, as sph_get_neighbours), rho and hsml (n). stream is a
 * cudaStream_t (NULL = the default stream); the call is synchronous: it
 * returns after its work on that stream is done (it reads its status back
 * and waits), so it cannot be captured in a CUDA graph. n <= SPH_NOALLOC_MAX_N and k <= SPH_NOALLOC_MAX_K,
 * else SPH_ERR_ARG. The first call on a device looks up the scratch's device
 * address and sets kernel attributes, so make it before any stream capture.
 * All calls share the scratch: calls that overlap on the GPU (other threads
 * or streams) race, so serialise them. p->precision and p->grid_level are
 * ignored (the binning level follows n, at most 2^7 cells per axis). */
#define SPH_NOALLOC_MAX_N 8192
#define SPH_NOALLOC_MAX_K 32
int sph_density_noalloc(const sph_params *p, const double *x, const double *y, int32_t n, int64_t *nbr_ids,
                        double *nbr_dist, double *rho, double *hsml, void *stream);

/* Self-check (no reference counterpart): runs the library's FMA-based
 * correctly rounded divisions (a shared reciprocal with one Markstein
 * correction, and division by 3) against the hardware division on n seeded
 * operand pairs, half of them built to lie next to rounding midpoints, and
 * reports the number of results that differ (0 expected). */
int sph_selftest_division(int64_t n, uint64_t seed, int64_t *mismatches);

/* Self-check (no reference counterpart): runs the library's binary64
 * multiplication, addition, subtraction, division and square root, its
 * 1 - x for x in [1/2, 1] and its binary64 -> (float, float) splits, computed
 * with integer instructions (which the FP64 kernels use beside the hardware
 * FP64 unit) against the hardware instructions on 12 n results from n seeded
 * operand pairs (random bits, nearby and extreme exponents, exact ties, near
 * cancellation, perfect squares and their neighbours, quotients next to
 * rounding boundaries, zeros, subnormals,
 * infinities and NaNs) and reports the number of results that differ in any
 * bit (NaN against NaN counts as equal; 0 expected). */
int sph_selftest_fp64emu(int64_t n, uint64_t seed, int64_t *mismatches);

/* Page-locks (pins) caller memory so that transfers from / to it run at
 * full link speed; no reference counterpart. */
int sph_host_register(void *ptr, int64_t bytes);
int sph_host_unregister(void *ptr);

/* Allocates / frees pinned host memory owned by the CUDA driver: the
 * fastest source and destination for sph_set_state / sph_get_state (on a
 * GB300 with Grace, 211 GB/s host->device against 128-180 GB/s from
 * registered malloc memory, 256 MB copies); no reference counterpart. */
int sph_host_alloc(int64_t bytes, void **ptr);
int sph_host_free(void *ptr);

/* ---- diagnostics (sim/sph.go:441-463) ----
 * out[0] = TotalEnergy (sum E), out[1] = TotalDensity (sum rho),
 * out[2] = TotalMomentum as the reference computes it (the norm of the last
 * particle's velocity: its loop assigns instead of adding),
 * out[3] = sum of |v| (the intended total). For an ensemble, sim selects one
 * simulation (-1 = all particles). */
int sph_diagnostics(sph_handle *h, int32_t sim, double out[4]);

/* ---- synthetic initial conditions (host only; no GPU needed) ----
 * SplitMix64 stream, 53-bit uniform doubles in [0,1). */
/* Uniform positions in [0,1)^2, v = 0, u = u_blast inside the disc of
 * radius r_blast about (0.5,0.5), u_bg elsewhere. */
int sph_ic_uniform_blast(int64_t n, uint64_t seed, double u_bg, double u_blast, double r_blast,
                         double *x, double *y, double *vx, double *vy, double *u);
/* nblobs Gaussian blobs (centres U[0,1)^2, sigma log-uniform in
 * [sig_min, sig_max], wrapped periodically) holding (1-f_bg) of the
 * particles in equal shares, plus f_bg uniform background; u = u_core inside
 * sigma of the own blob centre, u_bg elsewhere. */
int sph_ic_clustered(int64_t n, uint64_t seed, int32_t nblobs, double sig_min, double sig_max,
                     double f_bg, double u_bg, double u_core,
                     double *x, double *y, double *vx, double *vy, double *u);
/* f_in of the particles uniform in a side x side square at a uniform random
 * offset in [0, 1-side)^2, the rest uniform outside it; u = u_hot within
 * r_hot of the square centre, u_bg elsewhere. */
int sph_ic_stress(int64_t n, uint64_t seed, double side, double f_in, double u_bg, double u_hot,
                  double r_hot, double *x, double *y, double *vx, double *vy, double *u);
/* Ensemble sizes log-uniform in [nmin, nmax] and per-simulation blast
 * energies uniform in [ublo, ubhi]. */
int sph_ic_ensemble(int32_t nsims, uint64_t seed, int64_t nmin, int64_t nmax, double ublo,
                    double ubhi, int64_t *counts, double *u_blast);

/* ---- .sph-config setup (sim/config-parser.go) ---- */
#define SPH_CONFIG_MAX_SPAWNERS 64

/* [[Start]] [UniformRect] (sim/config-parser.go:37-41) */
typedef struct sph_rect_spawner {
    double upper_left[2];
    double lower_right[2];
    int64_t n;
} sph_rect_spawner;

/* [[Sources]] [Point] (sim/config-parser.go:43-47) */
typedef struct sph_point_source {
    double origin[2];
    double rate;
    double last_spawned;
} sph_point_source;

/* SphConfig (sim/config-parser.go:111-128) with the fields this library adds
 * (k, viscosity constants, precision, grid level) inside params. */
typedef struct sph_config {
    sph_params params;
    int32_t nsteps;                  /* NSteps */
    int32_t nstart;                  /* number of start spawners */
    int32_t nsources;                /* number of point sources */
    int32_t pad_;
    double viewport[4];              /* Viewport UpperLeft (x,y), LowerRight (x,y) */
    sph_rect_spawner start[SPH_CONFIG_MAX_SPAWNERS];
    sph_point_source sources[SPH_CONFIG_MAX_SPAWNERS];
} sph_config;

/* sim/config-parser.go:131 MakeConfig defaults. */
void sph_config_default(sph_config *out);
/* sim/config-parser.go:151 MakeConfigFromFile: tokenises and validates a
 * .sph-config file with the reference's grammar; on failure returns
 * SPH_ERR_CONFIG, writes the reference-format message
 * "file:line:col: ConfigParseError|ConfigMakeError: ..." into err and resets
 * *out to the defaults. Extra keys under [[Simulation]] [Config]:
 * NeighbourCount (int), ViscosityAlpha, ViscosityBeta, ViscosityEtaSq
 * (float), Precision (a word: Exact = SPH_PREC_FP64, Fast =
 * SPH_PREC_FP64_FAST, Mixed = SPH_PREC_MIXED), GridLevel (int). */
int sph_config_load(const char *path, sph_config *out, char *err, int32_t errlen);
/* Total particles of all start spawners. */
int64_t sph_config_start_count(const sph_config *cfg);
/* UniformRectSpawner.Spawn(0) of every start spawner in order
 * (sim/config-parser.go:58-80): the generator is reseeded with 12345678 at
 * each spawner, as the reference reseeds math/rand; E = 0.01, v = 0.
 * Arrays hold sph_config_start_count() entries; vx, vy, u may be NULL. */
int sph_config_spawn(const sph_config *cfg, double *x, double *y, double *vx, double *vy, double *u,
                     int64_t *z);
/* PointSource.Spawn(t) (sim/config-parser.go:82-102): returns how many
 * particles the source emits at time t (int(deltaT / cooldown)), advances its
 * last_spawned clock, and when x/y are not NULL fills them (origin +- 0.01
 * uniform, seeded by seed) with u = 0.002, v = 0 and draw keys z (may be
 * NULL). */
int64_t sph_point_source_spawn(sph_point_source *src, double t, uint64_t seed, double *x, double *y,
                               double *vx, double *vy, double *u, int64_t *z);

#ifdef __cplusplus
}
#endif
#endif
