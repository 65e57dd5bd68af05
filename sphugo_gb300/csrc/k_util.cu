// k_util.cu -- state transfer between the caller's particle order and the
// cell order kept on the device, neighbour-list export in the reference's
// layout, and the diagnostics of sim/sph.go:441-463.
#include "physics.cuh"
#include "fp64emu.cuh"

namespace sphgpu {

#define GRID_STRIDE(i, n) \
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (n); i += (int64_t)gridDim.x * blockDim.x)

static int grid_for(const Launch &L, int64_t n, int block) {
    int64_t need = (n + block - 1) / block;
    int64_t cap = (int64_t)L.sms * 16;
    int g = (int)(need < cap ? need : cap);
    return g < 1 ? 1 : g;
}

__global__ void k_gather_state(Ctx c, PArrays A, double *x, double *y, double *vx, double *vy,
                               double *u, double *ax, double *ay, double *udot) {
    GRID_STRIDE(i, c.n) {
        int32_t id = A.id[i];
        double2 p = A.pos[i], v = A.vel[i], a = A.acc[i];
        if (x) x[id] = p.x;
        if (y) y[id] = p.y;
        if (vx) vx[id] = v.x;
        if (vy) vy[id] = v.y;
        if (u) u[id] = A.u[i];
        if (ax) ax[id] = a.x;
        if (ay) ay[id] = a.y;
        if (udot) udot[id] = A.udot[i];
    }
}

void launch_gather_state(const Ctx &c, const Launch &L, const PArrays &A, double *x, double *y,
                         double *vx, double *vy, double *u, double *ax, double *ay, double *udot) {
    k_gather_state<<<grid_for(L, c.n, 256), 256, 0, L.stream>>>(c, A, x, y, vx, vy, u, ax, ay, udot);
}

// have_acc = 0: fresh upload, slot i holds particle i and the integrator
// history (accelerations, predictions, radius guess) starts from zero.
// have_acc = 1: replace the state of every particle in its current slot.
__global__ void k_scatter_state(Ctx c, PArrays A, const double *x, const double *y, const double *vx,
                                const double *vy, const double *u, const double *ax, const double *ay,
                                const double *udot, int have_acc) {
    GRID_STRIDE(i, c.n) {
        int32_t id;
        if (have_acc) {
            id = A.id[i];
        } else {
            id = (int32_t)i;
            A.id[i] = id;
            A.hprev[i] = 0.f;
        }
        double2 v = make_double2(vx ? vx[id] : 0.0, vy ? vy[id] : 0.0);
        double e = u ? u[id] : 0.0;
        A.pos[i] = make_double2(x[id], y[id]);
        A.vel[i] = v;
        A.u[i] = e;
        if (have_acc) {
            A.acc[i] = make_double2(ax ? ax[id] : 0.0, ay ? ay[id] : 0.0);
            A.udot[i] = udot ? udot[id] : 0.0;
        } else {
            A.acc[i] = make_double2(0.0, 0.0);
            A.udot[i] = 0.0;
        }
        A.vp[i] = v;
        A.up[i] = e;
    }
}

// New particles at slots n0 .. n0+count-1 (their caller indices): state from
// buf (x, y, vx, vy, u blocks of count values), no integrator history.
__global__ void k_append(PArrays A, int64_t n0, int64_t count, const double *buf) {
    GRID_STRIDE(i, count) {
        const int64_t s = n0 + i;
        const double2 v = make_double2(buf[2 * count + i], buf[3 * count + i]);
        const double e = buf[4 * count + i];
        A.pos[s] = make_double2(buf[i], buf[count + i]);
        A.vel[s] = v;
        A.vp[s] = v;
        A.acc[s] = make_double2(0.0, 0.0);
        A.u[s] = e;
        A.up[s] = e;
        A.udot[s] = 0.0;
        A.id[s] = (int32_t)s;
        A.hprev[s] = 0.f;
    }
}

void launch_append(const Launch &L, const PArrays &A, int64_t n0, int64_t count, const double *buf) {
    k_append<<<grid_for(L, count, 256), 256, 0, L.stream>>>(A, n0, count, buf);
}

void launch_scatter_state(const Ctx &c, const Launch &L, const PArrays &A, const double *x,
                          const double *y, const double *vx, const double *vy, const double *u,
                          const double *ax, const double *ay, const double *udot, bool have_acc) {
    k_scatter_state<<<grid_for(L, c.n, 256), 256, 0, L.stream>>>(c, A, x, y, vx, vy, u, ax, ay, udot,
                                                                 have_acc ? 1 : 0);
}

__global__ void k_gather_derived(Ctx c, PArrays A, Derived D, double *rho, double *cs, double *h) {
    GRID_STRIDE(i, c.n) {
        int32_t id = A.id[i];
        if (rho) rho[id] = D.rho[i];
        if (cs) cs[id] = D.c[i];
        if (h) h[id] = D.h[i];
    }
}

void launch_gather_derived(const Ctx &c, const Launch &L, const PArrays &A, const Derived &D,
                           double *rho, double *cs, double *h) {
    k_gather_derived<<<grid_for(L, c.n, 256), 256, 0, L.stream>>>(c, A, D, rho, cs, h);
}

// Reference layout: slot 0 = farthest (sim/nearest-neighbour.go:139-153 keeps
// NNDists descending); dist = sqrt of the reference's squared distance. Lists
// are re-sorted here by (squared distance, particle id, image code): the
// mixed form stores its neighbour set unordered.
constexpr int kMaxK = 128;

__global__ void k_gather_nbrs(Ctx c, PArrays B, Derived D, int64_t *ids, double *dist, int32_t *img) {
    const int k = c.k;
    GRID_STRIDE(i, c.n) {
        const int s = sim_of(c, i);
        const SimDev &S = c.sims[s];
        const int64_t idq = B.id[i];
        const double2 P = B.pos[i];
        double d2[kMaxK];
        uint32_t cd[kMaxK];
        for (int e = 0; e < k; e++) {
            const uint32_t code = (uint32_t)D.nbr[i * k + e];
            double ox, oy;
            img_shift(S, code & 15u, ox, oy);
            const double2 Q = B.pos[code >> kCodeShift];
            const double v = dist_sq_ref(P.x, P.y, ox, oy, Q.x, Q.y);
            int f = e - 1;
            while (f >= 0) {
                bool gt = d2[f] > v;
                if (d2[f] == v) {
                    const int32_t ia = B.id[cd[f] >> kCodeShift], ib = B.id[code >> kCodeShift];
                    gt = ia != ib ? ia > ib : (cd[f] & 15u) > (code & 15u);
                }
                if (!gt) break;
                d2[f + 1] = d2[f];
                cd[f + 1] = cd[f];
                f--;
            }
            d2[f + 1] = v;
            cd[f + 1] = code;
        }
        for (int e = 0; e < k; e++) {
            const int64_t o = idq * k + (k - 1 - e);
            if (ids) ids[o] = B.id[cd[e] >> kCodeShift];
            if (img) img[o] = (int32_t)(cd[e] & 15u);
            if (dist) dist[o] = __dsqrt_rn(d2[e]);
        }
    }
}

void launch_gather_neighbours(const Ctx &c, const Launch &L, const PArrays &, const PArrays &B,
                              const Derived &D, int64_t *ids, double *dist, int32_t *img, bool) {
    k_gather_nbrs<<<grid_for(L, c.n, 128), 128, 0, L.stream>>>(c, B, D, ids, dist, img);
}

// ---- diagnostics: deterministic sums over the caller's particle order.
// scratch layout: e[n], r[n], v[n] in id order, then block partials.
constexpr int kRedBlock = 256;

__global__ void k_diag_scatter(Ctx c, PArrays A, Derived D, double *scr) {
    GRID_STRIDE(i, c.n) {
        int32_t id = A.id[i];
        double2 v = A.vel[i];
        scr[id] = A.u[i];
        scr[c.n + id] = D.rho[i];
        // Vec2.Norm (sim/linear-algebra.go:54-56): sqrt(x*x + y*y), two roundings
        scr[2 * c.n + id] = __dsqrt_rn(__dadd_rn(__dmul_rn(v.x, v.x), __dmul_rn(v.y, v.y)));
    }
}

__device__ __forceinline__ double block_sum(double v, double *sh) {
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) sh[w] = v;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x == 0)
        for (int i = 0; i < (int)(blockDim.x >> 5); i++) r += sh[i];
    __syncthreads();
    return r;
}

// one block per (quantity, chunk); fixed chunking makes the sum order fixed
__global__ void k_diag_reduce(const double *scr, int64_t n, int64_t lo, int64_t hi, double *part) {
    __shared__ double sh[32];
    const int qn = blockIdx.y;
    const int64_t chunk = (hi - lo + gridDim.x - 1) / gridDim.x;
    const int64_t b0 = lo + blockIdx.x * chunk, b1 = min(hi, b0 + chunk);
    double v = 0.0;
    for (int64_t i = b0 + threadIdx.x; i < b1; i += blockDim.x) v += scr[qn * n + i];
    double r = block_sum(v, sh);
    if (threadIdx.x == 0) part[qn * gridDim.x + blockIdx.x] = r;
}

__global__ void k_diag_final(const double *scr, int64_t n, int64_t hi, const double *part, int nb,
                             double *out4) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double s[3] = {0.0, 0.0, 0.0};
    for (int q = 0; q < 3; q++)
        for (int b = 0; b < nb; b++) s[q] += part[q * nb + b];
    out4[0] = s[0];
    out4[1] = s[1];
    out4[2] = hi > 0 ? scr[2 * n + hi - 1] : 0.0;  // the reference's assignment: last particle only
    out4[3] = s[2];
}

void launch_diagnostics(const Ctx &c, const Launch &L, const PArrays &A, const Derived &D, int64_t lo,
                        int64_t hi, double *scratch) {
    // scratch: 3n doubles in id order, 3*nb block partials, then 4 outputs
    const int nb = 64;
    double *part = scratch + 3 * c.n;
    double *out4 = part + 3 * nb;
    k_diag_scatter<<<grid_for(L, c.n, 256), 256, 0, L.stream>>>(c, A, D, scratch);
    dim3 g(nb, 3);
    k_diag_reduce<<<g, kRedBlock, 0, L.stream>>>(scratch, c.n, lo, hi, part);
    k_diag_final<<<1, 32, 0, L.stream>>>(scratch, c.n, hi, part, nb, out4);
}

// ---- arithmetic throughput probe: 8 independent FMA chains per thread
template <typename T>
__global__ void k_fma_chains(T *out, int iters, T a, T b) {
    T x[8];
#pragma unroll
    for (int i = 0; i < 8; i++) x[i] = (T)(threadIdx.x * 1e-3 + i);
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int i = 0; i < 8; i++) x[i] = fma(x[i], a, b);
    }
    T s = 0;
#pragma unroll
    for (int i = 0; i < 8; i++) s += x[i];
    if (s == (T)12345.678) out[0] = s;  // keeps the chains live
}

// Dependent chains of correctly rounded divisions / square roots, eight per
// thread, to price them against the FMA chains above at full occupancy.
__global__ void k_div_chains(double *out, int iters, double a, double) {
    double x[8];
#pragma unroll
    for (int i = 0; i < 8; i++) x[i] = 1.0 + threadIdx.x * 1e-6 + i * 1e-3;
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int i = 0; i < 8; i++) x[i] = __ddiv_rn(a, x[i]);
    }
    double s = 0;
#pragma unroll
    for (int i = 0; i < 8; i++) s += x[i];
    if (s == 12345.678) out[0] = s;
}
__global__ void k_sqrt_chains(double *out, int iters, double a, double) {
    double x[8];
#pragma unroll
    for (int i = 0; i < 8; i++) x[i] = a + threadIdx.x * 1e-3 + i;
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int i = 0; i < 8; i++) x[i] = __dsqrt_rn(x[i]);
    }
    double s = 0;
#pragma unroll
    for (int i = 0; i < 8; i++) s += x[i];
    if (s == 12345.678) out[0] = s;
}

int probe_peaks(double *fp64_tflops, double *fp32_tflops, double *div_cost, double *sqrt_cost) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    void *buf = nullptr;
    if (cudaMalloc(&buf, 64) != cudaSuccess) return -1;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int blocks = sms * 8, threads = 256;
    // seconds per operation per thread-chain element (best of three)
    auto run = [&](auto kern, auto a, auto b, int iters) {
        kern<<<blocks, threads>>>((decltype(a) *)buf, 8, a, b);
        cudaDeviceSynchronize();
        float best = 1e30f;
        for (int r = 0; r < 3; r++) {
            cudaEventRecord(e0);
            kern<<<blocks, threads>>>((decltype(a) *)buf, iters, a, b);
            cudaEventRecord(e1);
            cudaEventSynchronize(e1);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            best = ms < best ? ms : best;
        }
        return (double)best * 1e-3 / ((double)blocks * threads * 8.0 * iters);
    };
    const double t_dfma = run(k_fma_chains<double>, 0.999999, 1e-7, 2000);
    const double t_ffma = run(k_fma_chains<float>, 0.999999f, 1e-7f, 20000);
    const double t_ddiv = run(k_div_chains, 1.0000001, 0.0, 100);
    const double t_dsqrt = run(k_sqrt_chains, 3.0, 0.0, 100);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(buf);
    if (fp64_tflops) *fp64_tflops = 2.0 / t_dfma / 1e12;
    if (fp32_tflops) *fp32_tflops = 2.0 / t_ffma / 1e12;
    if (div_cost) *div_cost = t_ddiv / t_dfma;
    if (sqrt_cost) *sqrt_cost = t_dsqrt / t_dfma;
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// ---- self-check of the division sequences against the hardware division
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__global__ void k_div_selftest(int64_t n, uint64_t seed, unsigned long long *bad) {
    unsigned long long nb = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t r1 = mix64(seed + 0x9E3779B97F4A7C15ull * (uint64_t)(2 * i + 1));
        const uint64_t r2 = mix64(seed + 0x9E3779B97F4A7C15ull * (uint64_t)(2 * i + 2));
        // random significands over 2^-40 .. 2^8, and quotients near rounding midpoints
        const double b = __longlong_as_double((long long)((r1 & 0x000FFFFFFFFFFFFFull) | ((uint64_t)(983 + (r1 >> 58) % 48) << 52)));
        double a = __longlong_as_double((long long)((r2 & 0x000FFFFFFFFFFFFFull) | ((uint64_t)(983 + (r2 >> 58) % 48) << 52)));
        if (i & 1) {  // a = RN(b (q + ulp(q)/2)) for q in [1, 2): a/b lies next to a midpoint
            const double q = __longlong_as_double((long long)((r2 & 0x000FFFFFFFFFFFFFull) | (1023ull << 52)));
            a = __fma_rn(b, q, __dmul_rn(b, 0x1p-53));
        }
        const double ref = __ddiv_rn(a, b);
        if (div_rn_recip(a, b, __drcp_rn(b)) != ref) nb++;
        if (div3_rn(a) != __ddiv_rn(a, 3.0)) nb++;
    }
    if (nb) atomicAdd(bad, nb);
}

// ---- self-check of the integer-pipe binary64 operations against the hardware
// One operand pair per index, from one of six classes: raw random bits (every
// exponent, zeros, subnormals, infinities, NaNs); normals of nearby
// exponents; short significands (exact ties in products and sums); exponents
// at the ends of the range (overflow, underflow, subnormal results); near
// cancellation (y = -x with its low bits changed); specials against normals.
__device__ __forceinline__ double emu_operand(uint64_t r, uint32_t cls, uint32_t e0) {
    uint64_t frac = r & kEmuFrac;
    uint32_t ex = e0;
    switch (cls) {
    case 0: return emu_double(r);
    case 2: frac &= 0x000FFFFFC0000000ull; break;  // 22 significant fraction bits
    default: break;
    }
    return emu_double((r & kEmuSign) | ((uint64_t)ex << 52) | frac);
}

__device__ __forceinline__ bool emu_same(double x, double y) {
    return emu_bits(x) == emu_bits(y) || (x != x && y != y);
}

__global__ void k_emu_selftest(int64_t n, uint64_t seed, unsigned long long *bad) {
    unsigned long long nb = 0;
    const double specials[8] = {0.0, -0.0, __longlong_as_double(1ll), __longlong_as_double(0x000FFFFFFFFFFFFFll),
                                __longlong_as_double(0x7FF0000000000000ll), __longlong_as_double((long long)0xFFF0000000000000ull),
                                __longlong_as_double(0x7FF8000000000000ll), 0x1p-1022};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t r1 = mix64(seed + 0x9E3779B97F4A7C15ull * (uint64_t)(3 * i + 1));
        const uint64_t r2 = mix64(seed + 0x9E3779B97F4A7C15ull * (uint64_t)(3 * i + 2));
        const uint64_t r3 = mix64(seed + 0x9E3779B97F4A7C15ull * (uint64_t)(3 * i + 3));
        const uint32_t cls = (uint32_t)(i % 6);
        double x, y;
        if (cls == 0) {
            x = emu_double(r1);
            y = emu_double(r2);
        } else if (cls == 1 || cls == 2) {
            // exponents 1000-1047 apart by 0 .. 63 (both classes): alignment
            // shifts of every length, carries, cancellation
            const uint32_t ex = 1000u + (uint32_t)(r3 % 48u);
            const uint32_t ey = 1000u + (uint32_t)((r3 >> 8) % 48u) + ((r3 >> 16) & 1u ? (uint32_t)((r3 >> 20) % 16u) : 0u);
            x = emu_operand(r1, cls, ex);
            y = emu_operand(r2, cls, ey);
        } else if (cls == 3) {
            // the ends of the range: products and sums near overflow and underflow
            const uint32_t lo = (uint32_t)(r3 & 1u);
            const uint32_t ex = lo ? 1u + (uint32_t)((r3 >> 1) % 64u) : 1983u + (uint32_t)((r3 >> 1) % 64u);
            const uint32_t ey = (r3 >> 8) & 1u ? 1023u + (uint32_t)((r3 >> 9) % 64u) - 32u
                                               : (lo ? 1u + (uint32_t)((r3 >> 9) % 64u) : 1983u + (uint32_t)((r3 >> 9) % 64u));
            x = emu_operand(r1, 1, ex);
            y = emu_operand(r2, 1, ey);
        } else if (cls == 4) {
            // near cancellation: y = -x with its low 0 .. 52 bits replaced, or
            // one exponent step away
            x = emu_operand(r1, 1, 900u + (uint32_t)(r3 % 256u));
            const uint32_t nbits = (uint32_t)((r3 >> 8) % 53u);
            const uint64_t mask = nbits ? ((1ull << nbits) - 1ull) : 0ull;
            uint64_t yb = (emu_bits(x) & ~mask) | (r2 & mask);
            if ((r3 >> 16) & 1u) yb += ((r3 >> 17) & 1u) ? (1ull << 52) : (uint64_t)-(int64_t)(1ull << 52);
            y = emu_double(yb ^ kEmuSign);
        } else {
            x = specials[r3 & 7u];
            y = emu_operand(r2, 1, 1u + (uint32_t)((r3 >> 3) % 2046u));
            if ((r3 >> 16) & 1u) { const double t = x; x = y; y = t; }
        }
        if (!emu_same(emu_mul(x, y), __dmul_rn(x, y))) nb++;
        if (!emu_same(emu_add(x, y), __dadd_rn(x, y))) nb++;
        if (!emu_same(emu_sub(x, y), __dsub_rn(x, y))) nb++;
        // square roots: the operands above, and squares of random 53-bit and
        // 26-bit significands moved by -2 .. +2 ulp (results next to rounding
        // midpoints and exact)
        double z = x;
        if (cls == 1 || cls == 4) {
            const double sq = emu_double(((uint64_t)(512u + (uint32_t)(r3 % 1024u)) << 52) | (r1 & kEmuFrac));
            z = emu_double(emu_bits(__dmul_rn(sq, sq)) + (uint64_t)((int64_t)((r2 >> 3) % 5u) - 2));
        } else if (cls == 2) {
            const double sq = emu_double(((uint64_t)(512u + (uint32_t)(r3 % 1024u)) << 52) | (r1 & 0x000FFFFFFC000000ull));
            z = __dmul_rn(sq, sq);  // exact: a perfect square
        }
        if (!emu_same(emu_sqrt(z), __dsqrt_rn(z))) nb++;
        // quotients: the operand pairs above (class 2: short significands,
        // exact quotients), and a = RN(b q) moved by -2 .. +2 ulp for random
        // significands q (quotients next to rounding boundaries)
        double num = x, den = y;
        if (cls == 1 && ((r3 >> 24) & 1u)) {
            const double q = emu_double((1023ull << 52) | (r1 & kEmuFrac));
            num = emu_double(emu_bits(__dmul_rn(y, q)) + (uint64_t)((int64_t)((r2 >> 5) % 5u) - 2));
        }
        const EmuDivisor dv = emu_divisor(den);
        if (!emu_same(emu_div(num, dv, den), __ddiv_rn(num, den))) nb++;
        // 1 - x, for x in [1/2, 1] from the operand's significand and for the operand itself
        const double xh = emu_double((1022ull << 52) | (r1 & kEmuFrac));
        if (!emu_same(emu_one_minus(xh), __dsub_rn(1.0, xh))) nb++;
        if (!emu_same(emu_one_minus(x), __dsub_rn(1.0, x))) nb++;
        if (!emu_same(emu_one_minus(1.0), __dsub_rn(1.0, 1.0))) nb++;
        // float pairs of the operands and of the products
        float h1, l1;
        emu_split_df(x, h1, l1);
        const float h0 = __double2float_rn(x), l0 = __double2float_rn(__dsub_rn(x, (double)h0));
        if (__float_as_uint(h1) != __float_as_uint(h0) && !(h1 != h1 && h0 != h0)) nb++;
        if (__float_as_uint(l1) != __float_as_uint(l0) && !(l1 != l1 && l0 != l0)) nb++;
        const double xy = __dmul_rn(x, y);
        emu_split_df(xy, h1, l1);
        const float h2 = __double2float_rn(xy), l2 = __double2float_rn(__dsub_rn(xy, (double)h2));
        if (__float_as_uint(h1) != __float_as_uint(h2) && !(h1 != h1 && h2 != h2)) nb++;
        if (__float_as_uint(l1) != __float_as_uint(l2) && !(l1 != l1 && l2 != l2)) nb++;
    }
    if (nb) atomicAdd(bad, nb);
}

int emu_selftest(int64_t n, uint64_t seed, long long *mismatches) {
    unsigned long long *d = nullptr;
    if (cudaMalloc(&d, sizeof *d) != cudaSuccess) return -1;
    cudaMemset(d, 0, sizeof *d);
    int sms = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    k_emu_selftest<<<sms * 8, 256>>>(n, seed, d);
    unsigned long long h = 0;
    cudaError_t e = cudaMemcpy(&h, d, sizeof h, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return -1;
    *mismatches = (long long)h;
    return 0;
}

int div_selftest(int64_t n, uint64_t seed, long long *mismatches) {
    unsigned long long *d = nullptr;
    if (cudaMalloc(&d, sizeof *d) != cudaSuccess) return -1;
    cudaMemset(d, 0, sizeof *d);
    int sms = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    k_div_selftest<<<sms * 8, 256>>>(n, seed, d);
    unsigned long long h = 0;
    cudaError_t e = cudaMemcpy(&h, d, sizeof h, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return -1;
    *mismatches = (long long)h;
    return 0;
}

}  // namespace sphgpu
