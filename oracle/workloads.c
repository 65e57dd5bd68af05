/*
 * workloads.c -- the seeded synthetic initial conditions, restated for the
 * oracle (TEST INFRASTRUCTURE).
 *
 * The CPU baseline and the reference arm of the benchmark build their inputs
 * here, so that they never load the GPU library. The recipes match the
 * library's generators (sph_ic_* in include/sphgpu.h) value for value; a CPU
 * test compares the two. The reference seeds Go's math/rand with 12345678
 * (sim/config-parser.go:58-80, sim/core.go:76-91); that stream is not
 * available here, so both sides use SplitMix64 (Steele, Lea and Flood, 2014:
 * a Weyl sequence with increment 0x9E3779B97F4A7C15 and the variant-13
 * finaliser), the top 53 bits scaled to a double in [0, 1).
 *
 * Recipes (positions in the periodic unit square, zero velocities):
 *   blast      i.i.d. uniform; u = u_blast within r_blast of (0.5, 0.5)
 *   clustered  nblobs Gaussian blobs (centre uniform, sigma log-uniform in
 *              [sig_min, sig_max], Box-Muller offsets, wrapped) holding
 *              1 - f_bg of the particles in equal shares, then a uniform
 *              background; u = u_core within one sigma of the blob centre
 *   stress     f_in of the particles uniform in a side x side square at a
 *              uniform offset in [0, 1 - side)^2, the rest uniform outside
 *              it (rejection); u = u_hot within r_hot of the square's centre
 *   ensemble   per simulation a count log-uniform in [nmin, nmax] (rounded,
 *              clamped) and a blast energy uniform in [ublo, ubhi]
 */
#include <math.h>
#include <stdint.h>

#include "sph_oracle.h"

typedef struct {
    uint64_t s;
} wl_rng;

static uint64_t wl_next(wl_rng *r) {
    uint64_t z = (r->s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static double wl_uniform(wl_rng *r) { return (double)(wl_next(r) >> 11) * 0x1.0p-53; }

static void wl_still(int64_t n, double *vx, double *vy) {
    for (int64_t i = 0; i < n; i++) {
        if (vx) vx[i] = 0.0;
        if (vy) vy[i] = 0.0;
    }
}

int orc_ic_uniform_blast(int64_t n, uint64_t seed, double u_bg, double u_blast, double r_blast, double *x,
                         double *y, double *vx, double *vy, double *u) {
    if (n < 0 || !x || !y) return ORC_ERR_ARG;
    wl_rng r = {seed};
    const double r2 = r_blast * r_blast;
    for (int64_t i = 0; i < n; i++) {
        const double px = wl_uniform(&r), py = wl_uniform(&r);
        x[i] = px;
        y[i] = py;
        const double ex = px - 0.5, ey = py - 0.5;
        if (u) u[i] = ex * ex + ey * ey < r2 ? u_blast : u_bg;
    }
    wl_still(n, vx, vy);
    return ORC_OK;
}

int orc_ic_clustered(int64_t n, uint64_t seed, int32_t nblobs, double sig_min, double sig_max, double f_bg,
                     double u_bg, double u_core, double *x, double *y, double *vx, double *vy, double *u) {
    if (n < 0 || nblobs < 1 || !x || !y || !(sig_min > 0) || !(sig_max >= sig_min) || !(f_bg >= 0 && f_bg <= 1))
        return ORC_ERR_ARG;
    wl_rng r = {seed};
    const int64_t background = llround((double)n * f_bg);
    const int64_t in_blobs = n - background;
    const double lmin = log(sig_min), lspan = log(sig_max) - lmin;
    int64_t i = 0;
    for (int32_t b = 0; b < nblobs; b++) {
        const double cx = wl_uniform(&r), cy = wl_uniform(&r);
        const double sigma = exp(lmin + wl_uniform(&r) * lspan);
        const int64_t share = in_blobs / nblobs + (b < in_blobs % nblobs ? 1 : 0);
        for (int64_t c = 0; c < share; c++, i++) {
            const double a = wl_uniform(&r), t = wl_uniform(&r);
            const double rad = sqrt(-2.0 * log(1.0 - a)); /* offset in units of sigma */
            const double ang = 6.283185307179586 * t;
            double px = cx + sigma * rad * cos(ang);
            double py = cy + sigma * rad * sin(ang);
            px -= floor(px);
            py -= floor(py);
            x[i] = px < 1.0 ? px : 0.0;
            y[i] = py < 1.0 ? py : 0.0;
            if (u) u[i] = rad < 1.0 ? u_core : u_bg;
        }
    }
    for (; i < n; i++) {
        x[i] = wl_uniform(&r);
        y[i] = wl_uniform(&r);
        if (u) u[i] = u_bg;
    }
    wl_still(n, vx, vy);
    return ORC_OK;
}

int orc_ic_stress(int64_t n, uint64_t seed, double side, double f_in, double u_bg, double u_hot, double r_hot,
                  double *x, double *y, double *vx, double *vy, double *u) {
    if (n < 0 || !x || !y || !(side > 0 && side < 1) || !(f_in >= 0 && f_in <= 1)) return ORC_ERR_ARG;
    wl_rng r = {seed};
    const double x0 = wl_uniform(&r) * (1.0 - side), y0 = wl_uniform(&r) * (1.0 - side);
    const double hx = x0 + 0.5 * side, hy = y0 + 0.5 * side;
    const int64_t inside = llround((double)n * f_in);
    const double r2 = r_hot * r_hot;
    for (int64_t i = 0; i < n; i++) {
        double px, py;
        if (i < inside) {
            px = x0 + side * wl_uniform(&r);
            py = y0 + side * wl_uniform(&r);
        } else {
            do {
                px = wl_uniform(&r);
                py = wl_uniform(&r);
            } while (px >= x0 && px < x0 + side && py >= y0 && py < y0 + side);
        }
        x[i] = px;
        y[i] = py;
        const double ex = px - hx, ey = py - hy;
        if (u) u[i] = ex * ex + ey * ey < r2 ? u_hot : u_bg;
    }
    wl_still(n, vx, vy);
    return ORC_OK;
}

int orc_ic_ensemble(int32_t nsims, uint64_t seed, int64_t nmin, int64_t nmax, double ublo, double ubhi,
                    int64_t *counts, double *u_blast) {
    if (nsims < 1 || nmin < 1 || nmax < nmin || !counts) return ORC_ERR_ARG;
    wl_rng r = {seed};
    const double lmin = log((double)nmin), lspan = log((double)nmax) - lmin;
    for (int32_t s = 0; s < nsims; s++) {
        const int64_t c = llround(exp(lmin + wl_uniform(&r) * lspan));
        counts[s] = c < nmin ? nmin : (c > nmax ? nmax : c);
        const double ub = ublo + wl_uniform(&r) * (ubhi - ublo);
        if (u_blast) u_blast[s] = ub;
    }
    return ORC_OK;
}
