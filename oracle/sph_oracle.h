/*
 * sph_oracle.h -- CPU oracle for the sphugo 2D SPH step (TEST INFRASTRUCTURE).
 *
 * This library is the correctness checker and the CPU baseline only. It is
 * loaded by the test-suite, by __graft_entry__.smoke() and by bench.py's CPU
 * baseline leg; nothing in the product (sphugo_gb300/) links or calls it.
 *
 * It restates, in plain C compiled with -ffp-contract=off, the reference's
 * algorithm (bbeni/sphugo, package sim):
 *   - Partition / Treebuild / BoundingSpheres        sim/core.go:126-312
 *   - periodic kNN with the sorted insertion queue    sim/nearest-neighbour.go:28-165
 *   - Monahan2D / Wendtland2D kernels                 sim/sph.go:258-304
 *   - Density2D                                       sim/sph.go:306-323
 *   - sound speed                                     sim/sph.go:421-429
 *   - AccelerationAndEDot2D                           sim/sph.go:327-401
 *   - Step (leapfrog, periodic wrap, reflections)     sim/sph.go:64-198
 *   - TotalEnergy / TotalDensity / TotalMomentum      sim/sph.go:441-463
 *   - sources appending particles during a run        sim/sph.go:71-85
 *   - the animator's frame (QuickSort by -Z, disks,   sim/animator.go:55-103,
 *     ParaRamp)                                       sim/heap.go:229-268,
 *                                                     gx/graphics.go:90-164
 * and adds an independent exact kNN (grid search, ties broken by
 * (squared distance, particle id, image code)) that defines the neighbour
 * sets the GPU path must reproduce bit for bit.
 *
 * Pinning: the Partition restatement is checked against the thirteen cases of
 * the reference's sim/partition_test.go, the sphere builder against the
 * containment property of sim/bounding-sphere_test.go, and the frame's colour
 * ramp against the reference's own output image doc/customColorMaps.png. The reference has no
 * tests or vectors for kNN, density, force or the integrator and its Go
 * toolchain is not available, so those restatements are pinned only by
 * analytic known-answer tests and by the agreement of the two independent kNN
 * restatements (tree and exact): physics parity against a reference run is
 * unpinned.
 */
#ifndef SPH_ORACLE_H
#define SPH_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_KERNEL_MONAHAN = 0, ORC_KERNEL_WENDLAND = 1 };
enum { ORC_KNN_TREE = 0, ORC_KNN_EXACT = 1 };

typedef struct {
    int32_t n;            /* particles */
    int32_t k;            /* neighbours per particle (NN_SIZE in the reference) */
    int32_t kernel;       /* ORC_KERNEL_* */
    int32_t knn_mode;     /* ORC_KNN_* */
    int32_t threads;      /* OpenMP threads, 0 = runtime default */
    int32_t pad_;
    double gamma, mass, dth;       /* Gamma, ParticleMass, DeltaTHalf */
    double accel[2];               /* Acceleration */
    double hor[2], vert[2];        /* HorPeriodicity / VertPeriodicity, +-DBL_MAX = open */
    double refl[4];                /* Reflections L, R, U, D */
    double alpha, beta, etasq;     /* viscosity constants (reference: 0.75, 1.5, 0.01) */
} orc_params;

typedef struct orc_sim orc_sim;

/* Status codes (0 = ok). */
enum {
    ORC_OK = 0,
    ORC_ERR_ARG = -1,
    ORC_ERR_SENTINEL = -2,   /* a k-th neighbour lies beyond the 0.4 queue sentinel */
    ORC_ERR_Q_RANGE = -3,    /* q = r/h outside [0,1] (the reference panics) */
    ORC_ERR_OPEN_MIX = -4,   /* open and periodic bound on one axis (reference panics) */
};

orc_sim *orc_create(const orc_params *p, const double *x, const double *y,
                    const double *vx, const double *vy, const double *u);
void orc_destroy(orc_sim *s);
int orc_set_knn_mode(orc_sim *s, int mode);
int orc_step(orc_sim *s, int nsteps);
int orc_forces(orc_sim *s);              /* CalculateForces with the stored predictions */
int orc_current_step(const orc_sim *s);

/* Per-particle state in the caller's original order (index = particle id). */
void orc_get_state(const orc_sim *s, double *x, double *y, double *vx, double *vy,
                   double *u, double *ax, double *ay, double *udot,
                   double *rho, double *c, double *h);
void orc_get_pred(const orc_sim *s, double *vpx, double *vpy, double *upred);
/* Neighbour lists in the reference layout: slot 0 is the farthest (NNDists[0]).
 * ids: original particle ids (n*k), dist: NNDists after the square root,
 * img: image code (i+1)*3+(j+1) of the offset (i*dX, j*dY). Any may be NULL. */
void orc_get_neighbours(const orc_sim *s, int64_t *ids, double *dist, int32_t *img);
/* Error normalisers of the last force evaluation (original order):
 * anorm = m*DFPref/h^3 * sum_j |rAB_j| * |(Pi+cA+cB) dW/r_j|,
 * unorm = |cA| * m * sum_j |dot_j * dW_j|. */
void orc_get_norms(const orc_sim *s, double *anorm, double *unorm);
/* TotalEnergy, TotalDensity, TotalMomentum (the last keeps the reference's
 * assignment: the norm of the last particle's velocity in array order). */
void orc_diagnostics(const orc_sim *s, double out[3]);
/* Number of particles whose tree-search neighbour set differed from the exact
 * set in the last evaluation that ran both (ORC_KNN_TREE with checking on). */
int64_t orc_tree_exact_mismatches(const orc_sim *s);
void orc_set_check_tree(orc_sim *s, int on);

/* ---- standalone pieces used by known-answer tests ---- */
/* sim/core.go:126 Partition on positions (reorders xs/ys in place); returns len(a). */
int orc_partition(double *xs, double *ys, int n, int orientation, double middle);
/* Builds the tree over (x,y) with root bounds [0,1]^2 as MakeCells does and
 * returns the number of particles not inside ANY node's bounding sphere
 * (sim/bounding-sphere_test.go:7-24 property). */
int orc_tree_count_outside(const double *x, const double *y, int n);
/* Go's math.Hypot (pure-Go scaled form). */
double orc_hypot(double p, double q);
/* Exact kNN of positions alone (no physics); ids ascending by (d2,id,img) per
 * particle i.e. slot 0 is the NEAREST here; d2 is the reference-rounded
 * squared distance. Returns status. */
int orc_knn_exact(const orc_params *p, const double *x, const double *y,
                  int64_t *ids, double *d2, int32_t *img);
int orc_knn_brute(const orc_params *p, const double *x, const double *y,
                  int64_t *ids, double *d2, int32_t *img);
/* Kernel values F, DF and prefactors, for unit tests. */
double orc_kernel_f(int kernel, double q);
double orc_kernel_df(int kernel, double q);
double orc_kernel_fpref(int kernel);
double orc_kernel_dfpref(int kernel);

/* Particles spawned during a run (sim/sph.go:71-85), appended with ids n.. */
int orc_append(orc_sim *s, int n_new, const double *x, const double *y, const double *vx,
               const double *vy, const double *u);

/* Frames (sim/animator.go:55-103): draw order by the reference's QuickSort
 * on -Z (sim/heap.go:229-268), and the painted NRGBA canvas. */
void orc_draw_order(int64_t n, const int64_t *z, int64_t *order);
void orc_para_ramp(int index, uint8_t *rgb);  /* gx/graphics.go:156-164 */
void orc_render(int64_t n, const double *x, const double *y, const double *rho, double mass,
                const int64_t *order, int W, int H, uint8_t *rgba);

/* Seeded synthetic initial conditions (workloads.c); value for value the
 * library's sph_ic_* generators, so that the CPU baseline builds its inputs
 * without the GPU library. */
int orc_ic_uniform_blast(int64_t n, uint64_t seed, double u_bg, double u_blast, double r_blast, double *x,
                         double *y, double *vx, double *vy, double *u);
int orc_ic_clustered(int64_t n, uint64_t seed, int32_t nblobs, double sig_min, double sig_max, double f_bg,
                     double u_bg, double u_core, double *x, double *y, double *vx, double *vy, double *u);
int orc_ic_stress(int64_t n, uint64_t seed, double side, double f_in, double u_bg, double u_hot, double r_hot,
                  double *x, double *y, double *vx, double *vy, double *u);
int orc_ic_ensemble(int32_t nsims, uint64_t seed, int64_t nmin, int64_t nmax, double ublo, double ubhi,
                    int64_t *counts, double *u_blast);

#ifdef __cplusplus
}
#endif
#endif
