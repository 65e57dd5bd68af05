// common.cuh -- device data layout and helpers shared by the SPH kernels.
//
// Particle state lives in HBM as structure-of-arrays, in cell (Morton) order
// of the last binning. Two particle-array sets ping-pong each step:
//   state A --(bin + permute, drift1)--> sorted B --(kNN + density)--> derived D
//   B + D --(force, kick, drift2, wrap, reflect)--> state A (same order as B)
// so A always holds the integrator state in the order of the latest binning
// and `id` maps each slot back to the caller's particle index.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/sphgpu.h"
#include "fp64emu.cuh"

namespace sphgpu {

constexpr int kMaxLevel = 14;          // finest grid: 2^14 cells per axis
constexpr int kImgBits = 4;            // nbr code = (slot index << kCodeShift) | image code
constexpr int kCodeShift = 5;          // bit 4 is a scratch flag inside the kNN kernel
constexpr uint32_t kCodeFlag = 16u;
constexpr int64_t kMaxParticles = (int64_t)1 << 27;

// internal precision modes (SPH_PREC_* of the ABI map onto these)
enum Mode { MODE_EXACT64 = 0, MODE_FAST64 = 1, MODE_MIXED = 2 };

// integration mode of a force evaluation
enum Pred { PRED_DRIFT = 0, PRED_INIT = 1, PRED_KEEP = 2 };

// device error flags (OR-ed into a word the host reads after each call)
enum Flags : unsigned {
    FLAG_KNN_ATTEMPTS = 1u,   // search radius did not converge
    FLAG_KNN_FEW = 2u,        // fewer than k candidates exist
    FLAG_SENTINEL = 4u,       // k-th squared distance >= 0.4 (reference sentinel)
    FLAG_Q_RANGE = 8u,        // q outside [0,1] / non-finite
    FLAG_NONFINITE = 16u,     // non-finite position
};

// Per-simulation constants (device copy). Grid fields of open axes are
// rewritten on the device every binning from the particles' bounding box.
struct SimDev {
    int64_t off, n;        // particle range in the flattened arrays
    int64_t cell_off;      // first cell of this simulation's table
    int32_t level;         // finest level (2^level cells per axis)
    int32_t kernel;
    int32_t periodic[2];
    double lo[2];          // grid origin
    double L[2];           // grid extent
    double s[2], inv_s[2]; // finest cell side and its inverse
    double per_lo[2], per_hi[2]; // HorPeriodicity / VertPeriodicity
    double dimg[2];        // image shifts dX, dY (0 on open axes)
    double gamma, mass, dth;
    double accel[2];
    double refl[4];
    double alpha, beta, etasq;
    double fpref, dfpref;
    float overshoot;       // max distance of a particle outside [lo, lo+L) (periodic axes)
    float tol;             // absolute slack of the FP32 cell tests
    // FP32 copies used per query (no FP64 instruction in the search's hot path)
    float fs[2];           // finest cell side
    float fdtc[2];         // dth / finest cell side (the binning's drift in cell units)
    float fimg_h[2], fimg_l[2]; // image shifts as float pairs (hi, lo)
    float flmax;           // max(L)
    float fmag;            // bound on |p + offset| of any particle image (the reference rounds it)
    // FP32 copies of the constants the mixed form's sums use
    float falpha, fbeta, fetasq, fgamma, fgg1, ffm, fdfm, fmass;
    unsigned long long bbox[4]; // open axes: ordered-key min x, max x, min y, max y
};

struct PArrays {
    double2 *pos, *vel, *vp, *acc;
    double *u, *up, *udot;
    int32_t *id;
    float *hprev;
    float4 *rec;    // (x hi, y hi, x lo, y lo): position relative to the grid origin as float pairs
    float4 *vrec;   // (vx hi, vy hi, vx lo, vy lo) of the predicted velocity (mixed path)
};

struct Derived {
    double *rho, *c, *h;
    double4 *der;   // FP64 modes: (c, rho, h, c^2/(gamma rho))
    float4 *derf;   // mixed:      (c, rho, h, c^2/(gamma rho))
    int32_t *nbr;   // n*k neighbour codes, slot 0 = nearest
    double2 *dist;  // FP64 modes: n*k squared distance from the search, then
                    // (NNDists, NNDists/h) [bit-exact form] or (NNDists, 1/NNDists) [fast form]
    float *d2f;     // mixed: n*k FP32 squared distances
    int32_t *defer;  // queries the group-tile search leaves to the per-query search (n)
    int32_t *ndefer; // their count; ndefer[1]: queries to re-rank, stored from the end of defer
};

struct Tables {
    int32_t *key, *rank;   // per particle (rank becomes the destination slot)
    int32_t *tmp;          // per particle: source indices grouped by cell
    int32_t *count;        // per cell (zero between binnings)
    int32_t *start;        // per cell + 1
    int32_t *partial;      // scan block sums
    int64_t ncells;
};

struct Ctx {
    const SimDev *sims;
    SimDev *sims_rw;
    const int64_t *offs;   // nsims + 1 particle offsets
    const int32_t *simidx; // per slot: its simulation (slot ranges never change); NULL for one simulation
    int nsims;
    int64_t n;
    int k;
    unsigned *flags;
};

// ---------------------------------------------------------------- helpers
// The simulation owning slot i: binning keeps every simulation inside its own
// slot range, so a static per-slot index answers with one load.
__device__ __forceinline__ int sim_of(const Ctx &c, int64_t i) { return c.simidx ? __ldg(c.simidx + i) : 0; }

__device__ __forceinline__ uint32_t part1by1(uint32_t x) {
    x &= 0x0000ffffu;
    x = (x | (x << 8)) & 0x00ff00ffu;
    x = (x | (x << 4)) & 0x0f0f0f0fu;
    x = (x | (x << 2)) & 0x33333333u;
    x = (x | (x << 1)) & 0x55555555u;
    return x;
}
__device__ __forceinline__ uint32_t morton2(uint32_t cx, uint32_t cy) {
    return part1by1(cx) | (part1by1(cy) << 1);
}

// FP32 fields of a SimDev from its FP64 grid fields
__host__ __device__ inline void simdev_floats(SimDev &S) {
    for (int a = 0; a < 2; a++) {
        S.fs[a] = (float)S.s[a];
        S.fdtc[a] = (float)(S.dth * S.inv_s[a]);
        S.fimg_h[a] = (float)S.dimg[a];
        S.fimg_l[a] = (float)(S.dimg[a] - (double)S.fimg_h[a]);
    }
    S.flmax = (float)(S.L[0] > S.L[1] ? S.L[0] : S.L[1]);
    double mag = 0.0;
    for (int a = 0; a < 2; a++) {
        const double lo = S.lo[a] < 0 ? -S.lo[a] : S.lo[a], hi = S.lo[a] + S.L[a] < 0 ? -(S.lo[a] + S.L[a]) : S.lo[a] + S.L[a];
        const double m = (lo > hi ? lo : hi) + S.L[a] + (S.dimg[a] < 0 ? -S.dimg[a] : S.dimg[a]);
        mag = m > mag ? m : mag;
    }
    S.fmag = (float)mag;
    S.falpha = (float)S.alpha;
    S.fbeta = (float)S.beta;
    S.fetasq = (float)S.etasq;
    S.fgamma = (float)S.gamma;
    S.fgg1 = (float)(S.gamma * (S.gamma - 1.0));
    S.ffm = (float)(S.fpref * S.mass);
    S.fdfm = (float)(S.mass * S.dfpref);
    S.fmass = (float)S.mass;
}

// order-preserving 64-bit key of a double (for atomic min/max)
__device__ __forceinline__ unsigned long long dkey(double d) {
    unsigned long long b = (unsigned long long)__double_as_longlong(d);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__host__ __device__ inline double dkey_inv(unsigned long long k) {
    unsigned long long b = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)b);
#else
    double d;
    __builtin_memcpy(&d, &b, 8);
    return d;
#endif
}

// double -> (hi, lo) float pair
__device__ __forceinline__ void split_df(double v, float &hi, float &lo) {
    emu_split_df(v, hi, lo);  // hi = RN_float(v), lo = RN_float(v - hi), on the integer pipes
}

// The drift of sim/sph.go:108-117 (no contraction: two roundings each).
__device__ __forceinline__ void predict(const SimDev &S, int mode, double2 pos, double2 vel,
                                        double2 acc, double u, double udot, double2 vp_old,
                                        double up_old, double2 &p, double2 &vp, double &up) {
    if (mode == PRED_DRIFT) {
        double dth = S.dth;
        p.x = __dadd_rn(pos.x, emu_mul(vel.x, dth));
        p.y = __dadd_rn(pos.y, emu_mul(vel.y, dth));
        vp.x = __dadd_rn(vel.x, emu_mul(acc.x, dth));
        vp.y = __dadd_rn(vel.y, emu_mul(acc.y, dth));
        up = __dadd_rn(u, emu_mul(udot, dth));
    } else if (mode == PRED_INIT) {
        p = pos; vp = vel; up = u;
    } else {
        p = pos; vp = vp_old; up = up_old;
    }
}

// ------------------------------------------------------------- launchers
struct Launch {
    int sms;
    cudaStream_t stream;
};

void launch_prep(const Ctx &c, const Launch &L, bool any_open);
void launch_bbox(const Ctx &c, const Launch &L, const PArrays &A, int pred);
void launch_grid(const Ctx &c, const Launch &L);
void launch_bin(const Ctx &c, const Launch &L, const PArrays &A, const Tables &T, int pred);
void launch_scan(const Ctx &c, const Launch &L, const Tables &T);
void launch_stable(const Ctx &c, const Launch &L, const Tables &T);
void launch_permute(const Ctx &c, const Launch &L, const PArrays &A, const PArrays &B,
                    const Tables &T, int pred, bool mixed);

struct KnnTune {
    int block;      // threads per block
    int cap;        // list capacity per query
    float theta;    // cell side >= theta * search radius
    float hgrow;    // radius guess = hgrow * previous h
    int blocks_per_sm; // resident blocks per SM at this block size / capacity
    int tile;          // 1: group tiles first, per-query search for the deferred queries
    int tile_blocks_per_sm;
    int block_warps;   // tiles shared by the warps of a block (4 or 8 warps; 0: one tile per warp)
};
void knn_init_attrs();
void launch_knn(const Ctx &c, const Launch &L, const PArrays &B, const Derived &D,
                const Tables &T, int mode, const KnnTune &tune);
// tune: the search's shape (NULL: a search without tiles); when the block
// tiles computed the settled queries' densities, only the deferred are done
void launch_density(const Ctx &c, const Launch &L, const PArrays &B, const Derived &D, int mode,
                    const KnnTune *tune);
void force_init_attrs(int k);
void launch_force(const Ctx &c, const Launch &L, const PArrays &B, const PArrays &A,
                  const Derived &D, int mode, bool integrate);
void launch_error_norms(const Ctx &c, const Launch &L, const PArrays &B, const Derived &D, double *anorm,
                        double *unorm);

void launch_gather_state(const Ctx &c, const Launch &L, const PArrays &A, double *x, double *y,
                         double *vx, double *vy, double *u, double *ax, double *ay, double *udot);
void launch_scatter_state(const Ctx &c, const Launch &L, const PArrays &A, const double *x,
                          const double *y, const double *vx, const double *vy, const double *u,
                          const double *ax, const double *ay, const double *udot, bool have_acc);
void launch_append(const Launch &L, const PArrays &A, int64_t n0, int64_t count, const double *buf);
void launch_gather_derived(const Ctx &c, const Launch &L, const PArrays &A, const Derived &D,
                           double *rho, double *cs, double *h);
void launch_gather_neighbours(const Ctx &c, const Launch &L, const PArrays &A, const PArrays &B,
                              const Derived &D, int64_t *ids, double *dist, int32_t *img, bool exact_stored);
void launch_diagnostics(const Ctx &c, const Launch &L, const PArrays &A, const Derived &D,
                        int64_t lo, int64_t hi, double *scratch);
int knn_occupancy_blocks(int block, int cap, int mode);
int knn_tile_occupancy_blocks(int k, int mode);
int probe_peaks(double *fp64_tflops, double *fp32_tflops, double *div_cost, double *sqrt_cost);
int div_selftest(int64_t n, uint64_t seed, long long *mismatches);
int emu_selftest(int64_t n, uint64_t seed, long long *mismatches);
// message returned by sph_last_error() on this thread
void set_last_error(const std::string &msg);

}  // namespace sphgpu
