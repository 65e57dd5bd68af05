// k_knn.cu -- exact periodic k-nearest-neighbour search fused with the
// density, sound speed and pressure term.
//
// Replaces sim/nearest-neighbour.go:28-165 (nine tree traversals per particle
// with a sorted insertion queue) and the density / sound-speed loops of
// sim/sph.go:411-429. One thread per query particle:
//   1. radius guess R (previous smoothing length, or a density estimate from
//      the cell table at step 0);
//   2. pick the binning level whose cells are >= theta*R and visit the cells
//      that intersect the disc of radius R around every periodic image the
//      reference considers (offsets in {-dX,0,dX} x {-dY,0,dY});
//   3. FP32 squared distances from float-pair coordinates (error bounded by
//      eps below) filter candidates into a per-thread list in shared memory;
//      R is grown or shrunk until the list holds >= k and <= cap entries and
//      provably contains every candidate that can rank in the top k;
//   4. candidates whose FP32 order is not certain (within 2 eps of a
//      neighbour, or of the k-th) are re-ranked with the reference's FP64
//      squared distance, ties broken by (particle id, image code);
//   5. density (sim/sph.go:306-323), c = sqrt(gamma(gamma-1) u_pred)
//      (sim/sph.go:421-429) and c^2/(gamma rho) in the epilogue.
// The neighbour SET and its order are identical in every arithmetic mode.
#include "physics.cuh"

#include <algorithm>

namespace sphgpu {

struct KnnArgs {
    Ctx c;
    PArrays B;
    Derived D;
    const int32_t *start;
    int cap;
    float theta, hgrow;
};

// |d2_f32 - d2_ref| <= eps_rel * d2 + eps_abs(R): the float-pair difference
// carries ~2^-23 relative error, the two float products ~2^-24 each, and the
// reference's own rounding of (p + offset) adds ~2^-53 L absolute per axis.
constexpr float kEpsRel = 9.5367431640625e-7f;  // 2^-20 (about 8x the bound)

__device__ __forceinline__ float eps_of(float d2, float abs_term) { return kEpsRel * d2 + abs_term; }

template <int MODE>
__global__ void __launch_bounds__(128) k_knn(KnnArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int bs = blockDim.x, t = threadIdx.x;
    const int k = a.c.k, cap = a.cap;
    unsigned long long *keys = (unsigned long long *)smem_raw;
    uint32_t *codes = (uint32_t *)(smem_raw + (size_t)cap * bs * 8);
#define KEY(e) keys[(size_t)(e) * bs + t]
#define CODE(e) codes[(size_t)(e) * bs + t]
    const PArrays &B = a.B;
    unsigned fl = 0;

    for (int64_t q = blockIdx.x * (int64_t)bs + t; q < a.c.n; q += (int64_t)gridDim.x * bs) {
        const int s = find_sim(a.c.offs, a.c.nsims, q);
        const SimDev &S = a.c.sims[s];
        const double2 P = B.pos[q];
        const float4 pr = B.rec[q];
        const float pxr = pr.x + pr.z, pyr = pr.y + pr.w;
        const int level = S.level, G = 1 << level;
        const float sx0 = (float)S.s[0], sy0 = (float)S.s[1];
        const float tol = S.tol + S.overshoot;
        const int per0 = S.periodic[0], per1 = S.periodic[1];
        const float dXh = __double2float_rn(S.dimg[0]);
        const float dXl = __double2float_rn(S.dimg[0] - (double)dXh);
        const float dYh = __double2float_rn(S.dimg[1]);
        const float dYl = __double2float_rn(S.dimg[1] - (double)dYh);
        const int64_t coff = S.cell_off;
        const float Lmax = (float)fmax(S.L[0], S.L[1]);
        const float epsabs = 1.8e-15f * Lmax;  // ~2^-49 L: reference rounding of p+offset, float-pair residue

        // ---- radius guess
        float R = B.hprev[q] * a.hgrow;
        if (!(R > 0.f)) {
            int cx = cell_coord(S, 0, P.x), cy = cell_coord(S, 1, P.y);
            float smin = fminf(sx0, sy0);
            R = 2.f * Lmax;
            for (int sh = 0; sh <= level; sh++) {
                uint32_t mo = morton2((uint32_t)cx >> sh, (uint32_t)cy >> sh);
                int n0 = __ldg(a.start + coff + ((int64_t)mo << (2 * sh)));
                int n1 = __ldg(a.start + coff + ((int64_t)(mo + 1) << (2 * sh)));
                int cnt = n1 - n0;
                if (cnt >= (k + 3) / 4 || sh == level) {
                    float side = smin * (float)(1 << sh);
                    R = side * sqrtf((float)k / (3.14159265f * fmaxf((float)cnt, 1.f))) * 1.25f;
                    break;
                }
            }
        }
        const float Rmax = 2.5f * Lmax;
        float Rlo = 0.f, Rhi = 3.0e38f;
        int m = 0, ok = 0;
        float tau = 0.f, eps = 0.f;
        for (int att = 0; att < 48; att++) {
            R = fminf(R, Rmax);
            const float R2 = R * R;
            int sh = 0;
            {
                float smin = fminf(sx0, sy0), want = a.theta * R;
                while (sh < level && smin * (float)(1 << sh) < want) sh++;
            }
            const int Gl = G >> sh;
            const float Sx = sx0 * (float)(1 << sh), Sy = sy0 * (float)(1 << sh);
            const float Re = R + tol;
            int vx0 = (int)floorf((pxr - Re) / Sx), vx1 = (int)floorf((pxr + Re) / Sx);
            int vy0 = (int)floorf((pyr - Re) / Sy), vy1 = (int)floorf((pyr + Re) / Sy);
            if (per0) { vx0 = max(vx0, -Gl); vx1 = min(vx1, 2 * Gl - 1); }
            else { vx0 = max(vx0, 0); vx1 = min(vx1, Gl - 1); }
            if (per1) { vy0 = max(vy0, -Gl); vy1 = min(vy1, 2 * Gl - 1); }
            else { vy0 = max(vy0, 0); vy1 = min(vy1, Gl - 1); }
            m = 0;
            for (int vy = vy0; vy <= vy1; vy++) {
                const int wy = floordiv(vy, Gl);
                const int cyl = vy - wy * Gl;
                const float ylo = (float)vy * Sy;
                float dyc = fmaxf(fmaxf(ylo - pyr, pyr - (ylo + Sy)) - tol, 0.f);
                const float dyc2 = dyc * dyc;
                if (dyc2 > R2) continue;
                const int ib = -wy;
                const float By = ib > 0 ? dYh : 0.f;
                const float Ay = ib < 0 ? pr.y - dYh : pr.y;
                const float Cy = pr.w + (float)ib * dYl;
                for (int vx = vx0; vx <= vx1; vx++) {
                    const int wx = floordiv(vx, Gl);
                    const int cxl = vx - wx * Gl;
                    const float xlo = (float)vx * Sx;
                    float dxc = fmaxf(fmaxf(xlo - pxr, pxr - (xlo + Sx)) - tol, 0.f);
                    if (dxc * dxc + dyc2 > R2) continue;
                    const int ia = -wx;
                    const float Bx = ia > 0 ? dXh : 0.f;
                    const float Ax = ia < 0 ? pr.x - dXh : pr.x;
                    const float Cx = pr.z + (float)ia * dXl;
                    const uint32_t img = (uint32_t)((ia + 1) * 3 + (ib + 1));
                    const uint32_t mo = morton2((uint32_t)cxl, (uint32_t)cyl);
                    const int j0 = __ldg(a.start + coff + ((int64_t)mo << (2 * sh)));
                    const int j1 = __ldg(a.start + coff + ((int64_t)(mo + 1) << (2 * sh)));
                    for (int j = j0; j < j1; j++) {
                        const float4 r = __ldg(&B.rec[j]);
                        const float dx = ((r.x - Bx) - Ax) + (r.z - Cx);
                        const float dy = ((r.y - By) - Ay) + (r.w - Cy);
                        const float d2 = __fmaf_rn(dx, dx, dy * dy);
                        if (d2 <= R2 && j != (int)q) {
                            if (m < cap) {
                                KEY(m) = __float_as_uint(d2);
                                CODE(m) = ((uint32_t)j << kCodeShift) | img;
                            }
                            m++;
                        }
                    }
                }
            }
            if (m < k) {
                if (R >= Rmax) { fl |= FLAG_KNN_FEW; break; }
                Rlo = R;
                float g = m > 0 ? fmaxf(1.15f, sqrtf((float)k / (float)m) * 1.1f) : 2.f;
                R = Rhi < 3.0e38f ? 0.5f * (Rlo + Rhi) : R * g;
                continue;
            }
            if (m > cap) {
                Rhi = R;
                float g = sqrtf(0.5f * (float)(k + cap) / (float)m);
                R = Rlo > 0.f ? 0.5f * (Rlo + Rhi) : R * g;
                continue;
            }
            // sort [0, m) by (approximate d2, code)
            for (int e = 1; e < m; e++) {
                unsigned long long kk = KEY(e);
                uint32_t cc = CODE(e);
                int f = e - 1;
                while (f >= 0) {
                    unsigned long long kf = KEY(f);
                    if (kf < kk || (kf == kk && CODE(f) < cc)) break;
                    KEY(f + 1) = kf;
                    CODE(f + 1) = CODE(f);
                    f--;
                }
                KEY(f + 1) = kk;
                CODE(f + 1) = cc;
            }
            tau = __uint_as_float((uint32_t)KEY(k - 1));
            eps = eps_of(tau, epsabs * R);
            if (tau + 3.f * eps > R2 * (1.f - 4.8e-7f)) {
                Rlo = R;
                R = sqrtf((tau + 3.f * eps) * 1.00002f) * 1.0001f;
                continue;
            }
            ok = 1;
            break;
        }
        if (!ok) {
            if (!(fl & FLAG_KNN_FEW)) fl |= FLAG_KNN_ATTEMPTS;
            for (int e = 0; e < k; e++) a.D.nbr[q * k + e] = ((int32_t)q << kCodeShift) | 4;
            a.D.rho[q] = 0.0; a.D.c[q] = 0.0; a.D.h[q] = 0.0;
            if (MODE == MODE_MIXED) a.D.derf[q] = make_float4(0.f, 0.f, 0.f, 0.f);
            else {
                a.D.der[q] = make_double4(0.0, 0.0, 0.0, 0.0);
                for (int e = 0; e < k; e++) a.D.dist[q * k + e] = make_double2(0.0, 0.0);
            }
            continue;
        }

        // ---- exact re-ranking
        int send = k;
        {
            const float lim = tau + 2.f * eps;
            while (send < m && __uint_as_float((uint32_t)KEY(send)) <= lim) send++;
        }
        auto exact_d2 = [&](uint32_t code) -> double {
            uint32_t j = code >> kCodeShift;
            double ox, oy;
            img_shift(S, code & 15u, ox, oy);
            double2 Q = B.pos[j];
            return dist_sq_ref(P.x, P.y, ox, oy, Q.x, Q.y);
        };
        // strict order on (exact d2, particle id, image code)
        auto exact_greater = [&](unsigned long long ka, uint32_t ca, unsigned long long kb, uint32_t cb) {
            if (ka != kb) return ka > kb;
            int32_t ia = B.id[ca >> kCodeShift], ib = B.id[cb >> kCodeShift];
            if (ia != ib) return ia > ib;
            return (ca & 15u) > (cb & 15u);
        };
        auto exact_sort = [&](int lo, int hi) {  // [lo, hi)
            for (int e = lo + 1; e < hi; e++) {
                unsigned long long kk = KEY(e);
                uint32_t cc = CODE(e);
                int f = e - 1;
                while (f >= lo && exact_greater(KEY(f), CODE(f), kk, cc)) {
                    KEY(f + 1) = KEY(f);
                    CODE(f + 1) = CODE(f);
                    f--;
                }
                KEY(f + 1) = kk;
                CODE(f + 1) = cc;
            }
        };
        double dk2 = -1.0;
        if (MODE != MODE_MIXED) {
            for (int e = 0; e < send; e++) {
                uint32_t cc = CODE(e);
                KEY(e) = (unsigned long long)__double_as_longlong(exact_d2(cc));
                CODE(e) = cc | kCodeFlag;
            }
            exact_sort(0, send);
            dk2 = __longlong_as_double((long long)KEY(k - 1));
        } else {
            int rs = 0;
            for (int e = 0; e < send; e++) {
                bool brk = (e + 1 == send);
                if (!brk) {
                    float a0 = __uint_as_float((uint32_t)KEY(e)), a1 = __uint_as_float((uint32_t)KEY(e + 1));
                    brk = (a1 - a0) > 2.f * eps_of(a1, epsabs * R);
                }
                if (brk) {
                    if (e > rs) {
                        for (int f = rs; f <= e; f++) {
                            uint32_t cc = CODE(f);
                            KEY(f) = (unsigned long long)__double_as_longlong(exact_d2(cc));
                            CODE(f) = cc | kCodeFlag;
                        }
                        exact_sort(rs, e + 1);
                        if (rs <= k - 1 && k - 1 <= e) dk2 = __longlong_as_double((long long)KEY(k - 1));
                    }
                    rs = e + 1;
                }
            }
            if (dk2 < 0.0) dk2 = exact_d2(CODE(k - 1));
        }
        if (!(dk2 < 0.4)) fl |= FLAG_SENTINEL;

        // ---- density, sound speed, pressure term
        const double gamma = S.gamma;
        const double up = B.up[q];
        double h, rho, cs, cterm;
        if (MODE == MODE_EXACT64) {
            h = __dsqrt_rn(dk2);
            double acc = 0.0;
            for (int e = k - 1; e >= 0; e--) {  // farthest first, as sim/sph.go:313
                double d = __dsqrt_rn(__longlong_as_double((long long)KEY(e)));
                double x = __ddiv_rn(d, h);
                if (x > 1.0 || x < 0.0) fl |= FLAG_Q_RANGE;
                acc = __dadd_rn(acc, kf_exact(S.kernel, x));
                a.D.dist[q * k + e] = make_double2(d, 0.0);
            }
            rho = __ddiv_rn(__dmul_rn(__dmul_rn(S.fpref, S.mass), acc), __dmul_rn(h, h));
            cs = __dsqrt_rn(__dmul_rn(__dmul_rn(gamma, __dsub_rn(gamma, 1.0)), up));
            cterm = __ddiv_rn(__dmul_rn(cs, cs), __dmul_rn(gamma, rho));
        } else if (MODE == MODE_FAST64) {
            h = __dsqrt_rn(dk2);
            const double inv_h = 1.0 / h;
            double acc = 0.0;
            for (int e = k - 1; e >= 0; e--) {
                double d2 = __longlong_as_double((long long)KEY(e));
                double y = rsqrt(d2);
                double d = d2 * y;
                double x = fmin(d * inv_h, 1.0);
                if (!(x >= 0.0)) fl |= FLAG_Q_RANGE;
                acc += kf_fast(S.kernel, x);
                a.D.dist[q * k + e] = make_double2(d, y);
            }
            rho = S.fpref * S.mass * acc * (inv_h * inv_h);
            cs = sqrt(gamma * (gamma - 1.0) * up);
            cterm = cs * cs / (gamma * rho);
        } else {
            h = __dsqrt_rn(dk2);
            const float hf = __double2float_rn(h);
            const float inv_hf = 1.f / hf;
            KahanF acc;
            for (int e = k - 1; e >= 0; e--) {
                unsigned long long kk = KEY(e);
                float d2 = (CODE(e) & kCodeFlag) ? __double2float_rn(__longlong_as_double((long long)kk))
                                                 : __uint_as_float((uint32_t)kk);
                float x = fminf(sqrtf(d2) * inv_hf, 1.f);
                acc.add(kf_f32(S.kernel, x));
            }
            rho = (S.fpref * S.mass / (h * h)) * acc.value();
            cs = sqrt(gamma * (gamma - 1.0) * up);
            cterm = cs * cs / (gamma * rho);
        }
        for (int e = 0; e < k; e++) a.D.nbr[q * k + e] = (int32_t)(CODE(e) & ~kCodeFlag);
        a.D.rho[q] = rho;
        a.D.c[q] = cs;
        a.D.h[q] = h;
        if (MODE == MODE_MIXED)
            a.D.derf[q] = make_float4((float)cs, (float)rho, (float)h, (float)cterm);
        else
            a.D.der[q] = make_double4(cs, rho, h, cterm);
    }
    if (fl) atomicOr(a.c.flags, fl);
#undef KEY
#undef CODE
}

static size_t knn_smem(int block, int cap) { return (size_t)cap * block * 12; }

// Sets the dynamic shared-memory limit of every instantiation; must run
// before any stream capture.
void knn_init_attrs() {
    cudaFuncSetAttribute(k_knn<MODE_EXACT64>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(k_knn<MODE_FAST64>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(k_knn<MODE_MIXED>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
}

int knn_occupancy_blocks(int block, int cap, int mode) {
    int nb = 0;
    size_t smem = knn_smem(block, cap);
    if (mode == MODE_EXACT64)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_knn<MODE_EXACT64>, block, smem);
    else if (mode == MODE_FAST64)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_knn<MODE_FAST64>, block, smem);
    else
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_knn<MODE_MIXED>, block, smem);
    return nb;
}

template <int MODE>
static void run_knn(const KnnArgs &args, const Launch &L, const KnnTune &tune) {
    size_t smem = knn_smem(tune.block, args.cap);
    int64_t need = (args.c.n + tune.block - 1) / tune.block;
    int grid = (int)std::min<int64_t>(need, (int64_t)L.sms * std::max(tune.blocks_per_sm, 1));
    if (grid < 1) grid = 1;
    k_knn<MODE><<<grid, tune.block, smem, L.stream>>>(args);
}

void launch_knn(const Ctx &c, const Launch &L, const PArrays &B, const Derived &D,
                const Tables &T, int mode, const KnnTune &tune) {
    KnnArgs a;
    a.c = c;
    a.B = B;
    a.D = D;
    a.start = T.start;
    a.cap = tune.cap;
    a.theta = tune.theta;
    a.hgrow = tune.hgrow;
    if (mode == MODE_EXACT64) run_knn<MODE_EXACT64>(a, L, tune);
    else if (mode == MODE_FAST64) run_knn<MODE_FAST64>(a, L, tune);
    else run_knn<MODE_MIXED>(a, L, tune);
}

}  // namespace sphgpu
