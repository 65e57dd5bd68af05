// ic.cpp -- seeded synthetic initial conditions (host only).
//
// The reference seeds Go's math/rand with 12345678 on every spawn
// (sim/config-parser.go:58-80); that generator's stream is not reproduced
// here. These recipes use SplitMix64 (Steele, Lea and Flood, 2014: a Weyl
// sequence with increment 0x9E3779B97F4A7C15 followed by the variant-13
// 64-bit finaliser) and map the top 53 bits to a double in [0,1). Compiled
// with -ffp-contract=off so that x86 and Arm hosts produce the same arrays
// from the same seed (the clustered recipe also calls libm's log/exp/sin/cos,
// whose last bit may differ between platforms).
#include <cmath>
#include <cstdint>

#include "../../include/sphgpu.h"

namespace {

struct SplitMix64 {
    uint64_t s;
    explicit SplitMix64(uint64_t seed) : s(seed) {}
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uni() { return (double)(next() >> 11) * 0x1.0p-53; }
};

void zero_vel(int64_t n, double *vx, double *vy) {
    for (int64_t i = 0; i < n; i++) {
        if (vx) vx[i] = 0.0;
        if (vy) vy[i] = 0.0;
    }
}

}  // namespace

extern "C" {

int sph_ic_uniform_blast(int64_t n, uint64_t seed, double u_bg, double u_blast, double r_blast, double *x,
                         double *y, double *vx, double *vy, double *u) {
    if (n < 0 || !x || !y) return SPH_ERR_ARG;
    SplitMix64 r(seed);
    const double rr = r_blast * r_blast;
    for (int64_t i = 0; i < n; i++) {
        x[i] = r.uni();
        y[i] = r.uni();
        double dx = x[i] - 0.5, dy = y[i] - 0.5;
        if (u) u[i] = (dx * dx + dy * dy < rr) ? u_blast : u_bg;
    }
    zero_vel(n, vx, vy);
    return SPH_OK;
}

int sph_ic_clustered(int64_t n, uint64_t seed, int32_t nblobs, double sig_min, double sig_max, double f_bg,
                     double u_bg, double u_core, double *x, double *y, double *vx, double *vy, double *u) {
    if (n < 0 || nblobs < 1 || !x || !y || !(sig_min > 0) || !(sig_max >= sig_min) || !(f_bg >= 0 && f_bg <= 1))
        return SPH_ERR_ARG;
    SplitMix64 r(seed);
    const int64_t nbg = (int64_t)std::llround((double)n * f_bg);
    const int64_t nblob = n - nbg;
    const double l0 = std::log(sig_min), l1 = std::log(sig_max);
    const double two_pi = 6.283185307179586;
    int64_t i = 0;
    for (int32_t b = 0; b < nblobs; b++) {
        const double cx = r.uni(), cy = r.uni();
        const double sig = std::exp(l0 + r.uni() * (l1 - l0));
        const int64_t cnt = nblob / nblobs + (b < nblob % nblobs ? 1 : 0);
        for (int64_t c = 0; c < cnt; c++, i++) {
            // Box-Muller: radius sqrt(-2 ln(1-u1)) is the offset in units of sigma
            const double u1 = r.uni(), u2 = r.uni();
            const double rad = std::sqrt(-2.0 * std::log(1.0 - u1));
            const double th = two_pi * u2;
            double px = cx + sig * rad * std::cos(th);
            double py = cy + sig * rad * std::sin(th);
            px -= std::floor(px);
            py -= std::floor(py);
            x[i] = px < 1.0 ? px : 0.0;
            y[i] = py < 1.0 ? py : 0.0;
            if (u) u[i] = rad < 1.0 ? u_core : u_bg;
        }
    }
    for (; i < n; i++) {
        x[i] = r.uni();
        y[i] = r.uni();
        if (u) u[i] = u_bg;
    }
    zero_vel(n, vx, vy);
    return SPH_OK;
}

int sph_ic_stress(int64_t n, uint64_t seed, double side, double f_in, double u_bg, double u_hot, double r_hot,
                  double *x, double *y, double *vx, double *vy, double *u) {
    if (n < 0 || !x || !y || !(side > 0 && side < 1) || !(f_in >= 0 && f_in <= 1)) return SPH_ERR_ARG;
    SplitMix64 r(seed);
    const double ox = r.uni() * (1.0 - side), oy = r.uni() * (1.0 - side);
    const double cx = ox + 0.5 * side, cy = oy + 0.5 * side;
    const int64_t nin = (int64_t)std::llround((double)n * f_in);
    const double rr = r_hot * r_hot;
    for (int64_t i = 0; i < n; i++) {
        double px, py;
        if (i < nin) {
            px = ox + side * r.uni();
            py = oy + side * r.uni();
        } else {
            do {
                px = r.uni();
                py = r.uni();
            } while (px >= ox && px < ox + side && py >= oy && py < oy + side);
        }
        x[i] = px;
        y[i] = py;
        const double dx = px - cx, dy = py - cy;
        if (u) u[i] = (dx * dx + dy * dy < rr) ? u_hot : u_bg;
    }
    zero_vel(n, vx, vy);
    return SPH_OK;
}

int sph_ic_ensemble(int32_t nsims, uint64_t seed, int64_t nmin, int64_t nmax, double ublo, double ubhi,
                    int64_t *counts, double *u_blast) {
    if (nsims < 1 || nmin < 1 || nmax < nmin || !counts) return SPH_ERR_ARG;
    SplitMix64 r(seed);
    const double l0 = std::log((double)nmin), l1 = std::log((double)nmax);
    for (int32_t s = 0; s < nsims; s++) {
        int64_t c = (int64_t)std::llround(std::exp(l0 + r.uni() * (l1 - l0)));
        counts[s] = c < nmin ? nmin : (c > nmax ? nmax : c);
        const double ub = ublo + r.uni() * (ubhi - ublo);
        if (u_blast) u_blast[s] = ub;
    }
    return SPH_OK;
}

}  // extern "C"
