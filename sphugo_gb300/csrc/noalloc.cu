// noalloc.cu -- exact neighbour search and density for a small particle set
// without any device allocation.
//
// Some callers cannot call cudaMalloc: a host framework that owns the whole
// device memory pool and forbids other allocations, or a latency-critical
// loop where an allocation (which may synchronise the device) is not allowed.
// sph_density_noalloc serves them with the same kernel chain as a force
// evaluation of the FP64 form (bin, scan, permute, kNN + density) but keeps
// every intermediate array in one file-scope static device array of
// kScratchBytes (about 7.7 MB, held by every GPU that loads the library until
// the process exits). The caller passes device-accessible inputs and outputs.
#include <cfloat>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include "common.cuh"

namespace sphgpu {
namespace {

constexpr int kNoAllocMaxN = SPH_NOALLOC_MAX_N;
constexpr int kNoAllocMaxK = SPH_NOALLOC_MAX_K;
constexpr int kNoAllocMaxLevel = 7;  // 2^7 x 2^7 cells
constexpr int64_t kNoAllocCells = (int64_t)1 << (2 * kNoAllocMaxLevel);

constexpr size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

// per-array byte sizes at the maximum size
constexpr size_t kN = kNoAllocMaxN, kNK = (size_t)kNoAllocMaxN * kNoAllocMaxK;
constexpr size_t kPArraysBytes = 4 * align256(16 * kN) + 3 * align256(8 * kN) + align256(4 * kN) +
                                 align256(4 * kN) + align256(16 * kN);
constexpr size_t kScratchBytes =
    2 * kPArraysBytes +                                                        // A, B
    3 * align256(8 * kN) + align256(32 * kN) + align256(4 * kNK) + align256(16 * kNK) +  // D
    3 * align256(4 * kN) + align256(4 * kNoAllocCells) + align256(4 * (kNoAllocCells + 1)) +
    align256(4 * (kNoAllocCells / 4096 + 2)) +                               // T
    align256(sizeof(SimDev)) + align256(2 * sizeof(int64_t)) + align256(sizeof(unsigned));

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

struct DeviceSetup {
    bool done = false;
    unsigned char *ptr = nullptr;  // device address of g_noalloc_scratch
    int sms = 0;
    int blocks_per_sm[kNoAllocMaxK + 1] = {};  // search launch shape by k (0: not measured yet)
};
std::mutex g_setup_mu;
DeviceSetup g_setup[64];

int nfail(int code, const std::string &m) {
    set_last_error(m);
    return code;
}

struct Carve {
    unsigned char *p;
    template <typename T>
    T *take(size_t count) {
        T *r = (T *)p;
        p += align256(count * sizeof(T));
        return r;
    }
};

void carve_parrays(Carve &c, PArrays &P) {
    P.pos = c.take<double2>(kN);
    P.vel = c.take<double2>(kN);
    P.vp = c.take<double2>(kN);
    P.acc = c.take<double2>(kN);
    P.u = c.take<double>(kN);
    P.up = c.take<double>(kN);
    P.udot = c.take<double>(kN);
    P.id = c.take<int32_t>(kN);
    P.hprev = c.take<float>(kN);
    P.rec = c.take<float4>(kN);
    P.vrec = nullptr;
}

// writes the simulation constants, offsets and the error word into scratch
__global__ void k_noalloc_init(SimDev S, SimDev *sims, int64_t *offs, unsigned *flags) {
    sims[0] = S;
    offs[0] = 0;
    offs[1] = S.n;
    flags[0] = 0u;
}

const double kMonahanPref = 0x1.5d3b3e3583243p+3;  // 6*40/(pi*7), sim/sph.go:266
const double kWendFPref = 0x1.1d34a60108f72p+1;    // 4*7/(pi*4), sim/sph.go:293
const double kWendDFPref = 0x1.1d34a60108f72p+2;   // 8*7/(pi*4), sim/sph.go:303

}  // namespace
}  // namespace sphgpu

using namespace sphgpu;

extern "C" int sph_density_noalloc(const sph_params *p, const double *x, const double *y, int32_t n,
                                   int64_t *nbr_ids, double *nbr_dist, double *rho, double *hsml,
                                   void *stream) {
    if (!p || !x || !y) return nfail(SPH_ERR_ARG, "sph_density_noalloc: params, x and y are required");
    if (n > kNoAllocMaxN || p->k > kNoAllocMaxK)
        return nfail(SPH_ERR_ARG, "sph_density_noalloc: at most " + std::to_string(kNoAllocMaxN) +
                                      " particles and k <= " + std::to_string(kNoAllocMaxK) +
                                      " fit its static scratch");
    if (p->k < 1 || n < p->k + 1) return nfail(SPH_ERR_ARG, "sph_density_noalloc: need 1 <= k and n >= k+1");
    if (p->kernel != SPH_KERNEL_MONAHAN && p->kernel != SPH_KERNEL_WENDLAND)
        return nfail(SPH_ERR_ARG, "sph_density_noalloc: unknown kernel");
    const double *axes[2] = {p->hor, p->vert};
    for (int a = 0; a < 2; a++) {
        if (axes[a][0] == -DBL_MAX ? axes[a][1] != DBL_MAX
                                   : !(axes[a][1] > axes[a][0]) || !std::isfinite(axes[a][1] - axes[a][0]))
            return nfail(SPH_ERR_ARG, "sph_density_noalloc: bad periodic bounds");
    }
    if (!std::isfinite(p->dth) || !std::isfinite(p->gamma) || !std::isfinite(p->mass))
        return nfail(SPH_ERR_ARG, "sph_density_noalloc: non-finite parameter");
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        cudaGetLastError();
        return nfail(SPH_ERR_CUDA, "sph_density_noalloc: no current CUDA device");
    }
    // One-time set-up per device (first call on that device; make it before
    // any stream capture): the symbol's device address, kernel attributes and
    // the launch shape of the neighbour search.
    DeviceSetup ds;
    {
        std::lock_guard<std::mutex> lk(g_setup_mu);
        if (!g_setup[dev].done) {
            void *ptr = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
            if (e != cudaSuccess || !ptr)
                return nfail(SPH_ERR_CUDA, std::string("sph_density_noalloc: cudaGetSymbolAddress: ") +
                                               cudaGetErrorString(e));
            knn_init_attrs();
            g_setup[dev].ptr = (unsigned char *)ptr;
            cudaDeviceGetAttribute(&g_setup[dev].sms, cudaDevAttrMultiProcessorCount, dev);
            g_setup[dev].done = true;
        }
        // the search's resident blocks per SM depend on k (its list shape)
        if (!g_setup[dev].blocks_per_sm[p->k])
            g_setup[dev].blocks_per_sm[p->k] = std::max(1, knn_occupancy_blocks(128, p->k + 16, MODE_EXACT64));
        ds = g_setup[dev];
    }
    cudaStream_t st = (cudaStream_t)stream;

    // carve the scratch
    Carve cv{ds.ptr};
    PArrays A{}, B{};
    carve_parrays(cv, A);
    carve_parrays(cv, B);
    Derived D{};
    D.rho = cv.take<double>(kN);
    D.c = cv.take<double>(kN);
    D.h = cv.take<double>(kN);
    D.der = cv.take<double4>(kN);
    D.nbr = cv.take<int32_t>(kNK);
    D.dist = cv.take<double2>(kNK);
    D.derf = nullptr;
    Tables T{};
    T.key = cv.take<int32_t>(kN);
    T.rank = cv.take<int32_t>(kN);
    T.tmp = cv.take<int32_t>(kN);
    T.count = cv.take<int32_t>(kNoAllocCells);
    T.start = cv.take<int32_t>(kNoAllocCells + 1);
    T.partial = cv.take<int32_t>(kNoAllocCells / 4096 + 2);
    SimDev *d_sims = cv.take<SimDev>(1);
    int64_t *d_offs = cv.take<int64_t>(2);
    unsigned *d_flags = cv.take<unsigned>(1);
    if ((size_t)(cv.p - ds.ptr) > kScratchBytes)
        return nfail(SPH_ERR_ARG, "sph_density_noalloc: internal scratch layout exceeds the static array");

    // constants of this call: the automatic binning level for n, capped to
    // the scratch's cell table (p->grid_level is not used)
    SimDev S;
    memset(&S, 0, sizeof S);
    double l = std::floor(0.5 * std::log2(std::max<double>((double)n, 2.0) / 2.0) + 0.5);
    S.level = (int)std::min<double>(std::max<double>(l, 1.0), kNoAllocMaxLevel);
    S.n = n;
    S.kernel = p->kernel;
    const int G = 1 << S.level;
    for (int a = 0; a < 2; a++) {
        S.per_lo[a] = axes[a][0];
        S.per_hi[a] = axes[a][1];
        S.periodic[a] = axes[a][0] != -DBL_MAX;
        S.lo[a] = S.periodic[a] ? axes[a][0] : 0.0;
        S.L[a] = S.periodic[a] ? axes[a][1] - axes[a][0] : 1.0;
        S.dimg[a] = S.periodic[a] ? axes[a][1] - axes[a][0] : 0.0;
        S.s[a] = S.L[a] / G;
        S.inv_s[a] = G / S.L[a];
    }
    S.gamma = p->gamma;
    S.mass = p->mass;
    S.dth = p->dth;
    S.alpha = p->alpha;
    S.beta = p->beta;
    S.etasq = p->etasq;
    S.fpref = p->kernel == SPH_KERNEL_WENDLAND ? kWendFPref : kMonahanPref;
    S.dfpref = p->kernel == SPH_KERNEL_WENDLAND ? kWendDFPref : kMonahanPref;
    S.tol = (float)(std::max(S.L[0], S.L[1]) * 4.0e-7);
    simdev_floats(S);
    T.ncells = (int64_t)1 << (2 * S.level);
    const bool any_open = !S.periodic[0] || !S.periodic[1];

    Ctx c;
    c.sims = d_sims;
    c.sims_rw = d_sims;
    c.offs = d_offs;
    c.simidx = nullptr;
    c.nsims = 1;
    c.n = n;
    c.k = p->k;
    c.flags = d_flags;
    Launch L{ds.sms, st};
    KnnTune tune{128, p->k + 16, 0.5f, 1.04f, ds.blocks_per_sm[p->k]};

    // the array keeps the previous call's contents: clear what starts at zero
    if (cudaMemsetAsync(T.count, 0, T.ncells * sizeof(int32_t), st) != cudaSuccess)
        return nfail(SPH_ERR_CUDA, "sph_density_noalloc: clearing the cell table failed");
    k_noalloc_init<<<1, 1, 0, st>>>(S, d_sims, d_offs, d_flags);
    launch_scatter_state(c, L, A, x, y, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, false);
    launch_prep(c, L, any_open);
    if (any_open) {
        launch_bbox(c, L, A, PRED_INIT);
        launch_grid(c, L);
    }
    launch_bin(c, L, A, T, PRED_INIT);
    launch_scan(c, L, T);
    launch_stable(c, L, T);
    launch_permute(c, L, A, B, T, PRED_INIT, false);
    launch_knn(c, L, B, D, T, MODE_EXACT64, tune);
    launch_density(c, L, B, D, MODE_EXACT64, nullptr);
    if (nbr_ids || nbr_dist) launch_gather_neighbours(c, L, B, B, D, nbr_ids, nbr_dist, nullptr, true);
    if (rho || hsml) launch_gather_derived(c, L, B, D, rho, nullptr, hsml);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return nfail(SPH_ERR_CUDA, std::string("sph_density_noalloc: ") + cudaGetErrorString(e));
    unsigned f = 0;
    e = cudaMemcpyAsync(&f, d_flags, sizeof f, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return nfail(SPH_ERR_CUDA, std::string("sph_density_noalloc: ") + cudaGetErrorString(e));
    if (f & FLAG_SENTINEL) return nfail(SPH_ERR_SENTINEL, "sph_density_noalloc: a k-th neighbour lies beyond the 0.4 sentinel");
    if (f & (FLAG_KNN_FEW | FLAG_KNN_ATTEMPTS)) return nfail(SPH_ERR_KNN, "sph_density_noalloc: neighbour search failed");
    if (f) return nfail(SPH_ERR_RANGE, "sph_density_noalloc: non-finite input");
    return SPH_OK;
}
