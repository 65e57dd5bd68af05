// k_knn.cu -- exact periodic k-nearest-neighbour search (one warp per query
// particle) and the density / sound-speed pass that consumes its lists.
//
// Replaces sim/nearest-neighbour.go:28-165 (nine tree traversals per particle
// with a sorted insertion queue) and the density / sound-speed loops of
// sim/sph.go:411-429.
//
// k_knn, one warp per query:
//   1. radius guess R (previous smoothing length, or a density estimate from
//      the cell table at step 0);
//   2. the binning level whose cells are >= theta*R is chosen and the cells
//      of the block covering the disc of radius R around the query's images
//      (offsets in {-dX,0,dX} x {-dY,0,dY}, as the reference) are spread over
//      the lanes: one cell per lane, a warp prefix sum of their populations;
//   3. candidates are processed 32 at a time: FP32 squared distances from the
//      float-pair coordinates filter them against R^2 and a ballot compacts
//      the survivors into a per-warp list in shared memory; R grows or shrinks
//      (a warp-uniform decision) until the list holds >= k and <= CAP entries
//      and provably holds every candidate that can rank in the top k;
//   4. the list is sorted by a register bitonic network on 32-bit keys
//      (truncated FP32 squared distance | list slot);
//   5. every order the FP32 values cannot decide (entries within 2 eps of each
//      other) is settled with the reference's FP64 squared distance, ties
//      broken by (particle id, image code); the FP64 forms settle all of them.
// k_density, one thread per particle: smoothing length h = sqrt of the k-th
// FP64 squared distance, density (sim/sph.go:306-323),
// c = sqrt(gamma (gamma-1) u_pred) and c^2/(gamma rho).
// The neighbour set and its order are identical in every arithmetic form.
#include "knn_shared.cuh"

#include <algorithm>
#include <cstddef>

namespace sphgpu {

template <int NR>
struct ListShape {
    static constexpr int CAP = 32 * NR;
    static constexpr int SB = NR == 1 ? 5 : NR == 2 ? 6 : NR == 4 ? 7 : 8;  // slot bits
    static constexpr uint32_t SMASK = (1u << SB) - 1u;
};

// Ascending bitonic sort of 32*NR keys, element e = r*32 + lane in v[r].
template <int NR>
__device__ __forceinline__ void bitonic_sort(uint32_t (&v)[NR], int lane) {
    constexpr int N = 32 * NR;
#pragma unroll
    for (int size = 2; size <= N; size <<= 1) {
#pragma unroll
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            if (stride >= 32) {
                const int rs = stride >> 5;
#pragma unroll
                for (int r = 0; r < NR; r++) {
                    const int p = r ^ rs;
                    if (p > r) {
                        const bool asc = (((r << 5) | lane) & size) == 0;
                        const uint32_t a = v[r], b = v[p];
                        const uint32_t lo = min(a, b), hi = max(a, b);
                        v[r] = asc ? lo : hi;
                        v[p] = asc ? hi : lo;
                    }
                }
            } else {
#pragma unroll
                for (int r = 0; r < NR; r++) {
                    const bool asc = (((r << 5) | lane) & size) == 0;
                    const bool lower = (lane & stride) == 0;
                    const uint32_t o = __shfl_xor_sync(0xffffffffu, v[r], stride);
                    v[r] = (asc == lower) ? min(v[r], o) : max(v[r], o);
                }
            }
        }
    }
}

// strict order on (exact d2, particle id, image code)
__device__ __forceinline__ bool exact_greater(const PArrays &B, unsigned long long ka, uint32_t ca,
                                              unsigned long long kb, uint32_t cb) {
    if (ka != kb) return ka > kb;
    const int32_t ia = B.id[ca >> kCodeShift], ib = B.id[cb >> kCodeShift];
    if (ia != ib) return ia > ib;
    return (ca & 15u) > (cb & 15u);
}

// Exact selection of the k nearest among the m entries of a warp's list
// (skey: FP32 squared distances as bits, scode: (j << kCodeShift) | image)
// for query q, written to the neighbour list (slot 0 nearest in the FP64
// forms; the mixed form writes the set with the farthest in the last slot).
// Returns 0 when written, or 1 when the k-th FP32 value lies too close to the
// search radius R for the list to be complete (*Rnext: a radius that is).
template <int MODE, int NR>
__device__ int select_write(const KnnArgs &a, const SimDev &S, int64_t q, int m, float R, float epsabs,
                            uint32_t *skey, uint32_t *scode, uint32_t *sord, unsigned long long *sexact,
                            int lane, float *Rnext) {
    using LS = ListShape<NR>;
    const int k = a.c.k;
    const PArrays &B = a.B;
    const float R2 = R * R;
    uint32_t v[NR];
    float tau, eps;
    if (MODE == MODE_MIXED) {
        // The mixed form needs the set, not the order: drop the m-k largest
        // (unique keys: truncated FP32 value | slot) by warp max-reductions,
        // then verify with the full FP32 values that every kept entry lies
        // more than 2 eps below every dropped one and that the farthest kept
        // entry is unique by 2 eps.
#pragma unroll
        for (int r = 0; r < NR; r++) {
            const int e = (r << 5) | lane;
            // bit 31 tags a live entry (FP32 squared distances are >= 0)
            v[r] = e < m ? (0x80000000u | (skey[e] & ~LS::SMASK) | (uint32_t)e) : 0u;
        }
        uint32_t dropped_min = 0xffffffffu;  // smallest full FP32 bits among dropped entries
        for (int it = 0; it < m - k; it++) {
            uint32_t lm = 0;
#pragma unroll
            for (int r = 0; r < NR; r++) lm = max(lm, v[r]);
            const uint32_t gm = __reduce_max_sync(0xffffffffu, lm);
#pragma unroll
            for (int r = 0; r < NR; r++)
                if (v[r] == gm) v[r] = 0u;
            dropped_min = min(dropped_min, skey[gm & LS::SMASK]);
        }
        // largest and second largest full values among the kept entries
        uint32_t top = 0, second = 0;  // tagged with bit 31 when set
#pragma unroll
        for (int r = 0; r < NR; r++) {
            if (v[r]) {
                const uint32_t f = 0x80000000u | skey[v[r] & LS::SMASK];
                if (f > top) { second = top; top = f; } else if (f > second) second = f;
            }
        }
        const uint32_t gtop = __reduce_max_sync(0xffffffffu, top);
        // second: the largest of (each lane's top unless it is the global top) and seconds
        const uint32_t cand2 = top == gtop ? second : top;
        const uint32_t g2 = __reduce_max_sync(0xffffffffu, cand2);
        const uint32_t nties = __popc(__ballot_sync(0xffffffffu, top == gtop));
        tau = __uint_as_float(gtop & 0x7fffffffu);
        eps = eps_of(tau, epsabs * R);
        if (tau + 3.f * eps > R2 * (1.f - 4.8e-7f)) {
            *Rnext = sqrtf((tau + 3.f * eps) * 1.00002f) * 1.0001f;
            return 1;
        }
        const float fd = __uint_as_float(dropped_min), f2 = __uint_as_float(g2 & 0x7fffffffu);
        const bool set_ok = (m == k) || (fd - tau > 2.f * eps_of(fd, epsabs * R));
        const bool top_ok = nties == 1 && (k == 1 || tau - f2 > 2.f * eps);
        if (set_ok && top_ok) {
            // write the kept entries in slot order, the farthest last
            int pos = 0;
#pragma unroll
            for (int r = 0; r < NR; r++) {
                const bool live = v[r] != 0u;
                const bool is_top = live && (0x80000000u | skey[v[r] & LS::SMASK]) == gtop;
                const bool keep = live && !is_top;
                const uint32_t bal = __ballot_sync(0xffffffffu, keep);
                if (keep) {
                    const int o = pos + __popc(bal & lanemask_lt());
                    const uint32_t sl = v[r] & LS::SMASK;
                    a.D.nbr[q * k + o] = (int32_t)scode[sl];
                    a.D.d2f[q * k + o] = __uint_as_float(skey[sl]);
                }
                if (is_top) {
                    const uint32_t sl = v[r] & LS::SMASK;
                    a.D.nbr[q * k + k - 1] = (int32_t)scode[sl];
                    a.D.d2f[q * k + k - 1] = __uint_as_float(skey[sl]);
                }
                pos += __popc(bal);
            }
            __syncwarp();
            return 0;
        }
        // otherwise the sorted path below decides
    }
#pragma unroll
    for (int r = 0; r < NR; r++) {
        const int e = (r << 5) | lane;
        v[r] = e < m ? ((skey[e] & ~LS::SMASK) | (uint32_t)e) : 0xffffffffu;
    }
    bitonic_sort<NR>(v, lane);
#pragma unroll
    for (int r = 0; r < NR; r++) sord[(r << 5) | lane] = v[r] & LS::SMASK;
    __syncwarp();
    // tau: the largest FP32 value among the first k in truncated order (>= the k-th smallest)
    float tmax = 0.f;
    for (int e = lane; e < k; e += 32) tmax = fmaxf(tmax, __uint_as_float(skey[sord[e]]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) tmax = fmaxf(tmax, __shfl_xor_sync(0xffffffffu, tmax, o));
    tau = tmax;
    eps = eps_of(tau, epsabs * R);
    if (tau + 3.f * eps > R2 * (1.f - 4.8e-7f)) {
        *Rnext = sqrtf((tau + 3.f * eps) * 1.00002f) * 1.0001f;
        __syncwarp();
        return 1;
    }

    // ---- S = every entry whose FP32 value is within 2 eps of tau (a prefix)
    const float lim = tau + 2.f * eps;
    int last = -1;
    for (int e = lane; e < m; e += 32)
        if (__uint_as_float(skey[sord[e]]) <= lim) last = e;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) last = max(last, __shfl_xor_sync(0xffffffffu, last, o));
    const int send = last + 1;  // >= k

    // ---- orders the FP32 values cannot decide: FP64 keys, exact runs
    bool unc = false;
    for (int e = lane; e + 1 < send; e += 32) {
        const float fa = __uint_as_float(skey[sord[e]]), fb = __uint_as_float(skey[sord[e + 1]]);
        unc |= (fb - fa) <= 2.f * eps_of(fb, epsabs * R);
    }
    if (__any_sync(0xffffffffu, unc)) {
        const double2 P = B.pos[q];
        for (int e = lane; e < send; e += 32) {
            const float fe = __uint_as_float(skey[sord[e]]);
            bool need = false;
            if (e + 1 < send) {
                const float fn = __uint_as_float(skey[sord[e + 1]]);
                need |= (fn - fe) <= 2.f * eps_of(fn, epsabs * R);
            }
            if (e > 0) need |= (fe - __uint_as_float(skey[sord[e - 1]])) <= 2.f * eps_of(fe, epsabs * R);
            if (need) {
                const uint32_t code = scode[sord[e]];
                double ox, oy;
                img_shift(S, code & 15u, ox, oy);
                const double2 Q = B.pos[code >> kCodeShift];
                sexact[e] = (unsigned long long)__double_as_longlong(dist_sq_ref(P.x, P.y, ox, oy, Q.x, Q.y));
            }
        }
        __syncwarp();
        if (lane == 0) {
            int rs = 0;
            for (int e = 0; e < send; e++) {
                bool brk = (e + 1 == send);
                if (!brk) {
                    const float fa = __uint_as_float(skey[sord[e]]), fb = __uint_as_float(skey[sord[e + 1]]);
                    brk = (fb - fa) > 2.f * eps_of(fb, epsabs * R);
                }
                if (brk) {
                    // insertion sort of the run [rs, e] by (exact d2, id, image)
                    for (int x = rs + 1; x <= e; x++) {
                        const unsigned long long kk = sexact[x];
                        const uint32_t so = sord[x];
                        int f = x - 1;
                        while (f >= rs && exact_greater(B, sexact[f], scode[sord[f]], kk, scode[so])) {
                            sexact[f + 1] = sexact[f];
                            sord[f + 1] = sord[f];
                            f--;
                        }
                        sexact[f + 1] = kk;
                        sord[f + 1] = so;
                    }
                    rs = e + 1;
                }
            }
        }
        __syncwarp();
    }
    // ---- write the sorted list (slot 0 = nearest)
    for (int e = lane; e < k; e += 32) {
        a.D.nbr[q * k + e] = (int32_t)scode[sord[e]];
        if (MODE == MODE_MIXED) a.D.d2f[q * k + e] = __uint_as_float(skey[sord[e]]);
    }
    __syncwarp();
    return 0;
}

// Cells holding more than kHeavyCell particles are not scanned whole: they are
// split into their four children (the next finer level; contiguous ranges of
// the Morton-ordered table), which are pruned against the radius again. This
// bounds the work of a sparse query next to a dense region, whose cells at the
// level chosen from its radius can hold thousands of particles of which only
// a sliver lies within the radius. Up to kRefineQueue cells wait per warp;
// when the queue is full a heavy cell is scanned whole.
constexpr int kHeavyCell = 128;
constexpr int kRefineQueue = 64;
__host__ __device__ constexpr size_t knn_warp_bytes(int nr) {
    return (size_t)32 * nr * 20 + (size_t)kRefineQueue * sizeof(int4);
}

template <int MODE, int NR>
__global__ void __launch_bounds__(256, 3) k_knn(KnnArgs a) {
    using LS = ListShape<NR>;
    constexpr int CAP = LS::CAP;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, wpb = blockDim.x >> 5;
    // per-warp scratch: exact keys, full FP32 keys, codes, sorted order, and
    // the queue of heavy cells to refine
    unsigned char *base = smem_raw + (size_t)w * knn_warp_bytes(NR);
    unsigned long long *sexact = (unsigned long long *)base;
    uint32_t *skey = (uint32_t *)(base + CAP * 8);
    uint32_t *scode = skey + CAP;
    uint32_t *sord = scode + CAP;
    int4 *rq = (int4 *)(base + CAP * 20);
    const int k = a.c.k;
    const PArrays &B = a.B;
    unsigned fl = 0;

    const int64_t nq = a.use_defer ? (int64_t)*a.D.ndefer : a.c.n;
    for (int64_t qi = (int64_t)blockIdx.x * wpb + w; qi < nq; qi += (int64_t)gridDim.x * wpb) {
        const int64_t q = a.use_defer ? (int64_t)a.D.defer[qi] : qi;
        // Only FP32 / integer work below (FP64 would run 32-wide for one query).
        const int s = sim_of(a.c, q);
        const SimDev &S = a.c.sims[s];
        const float4 pr = B.rec[q];
        const float pxr = pr.x + pr.z, pyr = pr.y + pr.w;
        const int level = S.level;
        const float sx0 = S.fs[0], sy0 = S.fs[1], smin = fminf(sx0, sy0);
        const float tol = S.tol + S.overshoot;
        const int per0 = S.periodic[0], per1 = S.periodic[1];
        const float dXh = S.fimg_h[0], dXl = S.fimg_l[0], dYh = S.fimg_h[1], dYl = S.fimg_l[1];
        const int64_t coff = S.cell_off;
        const float Lmax = S.flmax;
        const float epsabs = 1.8e-15f * fmaxf(Lmax, S.fmag);  // the reference's rounding of p + offset
        // per-image constants of the float-pair difference (q - offset) - p
        const float axm = pr.x - dXh, aym = pr.y - dYh;
        const float cxp = pr.z + dXl, cxm = pr.z - dXl, cyp = pr.w + dYl, cym = pr.w - dYl;

        // ---- radius guess (identical in every lane)
        float R = B.hprev[q] * a.hgrow;
        if (!(R > 0.f)) {
            const int G = 1 << level;
            const int cx = min(max((int)floorf(pxr / sx0), 0), G - 1), cy = min(max((int)floorf(pyr / sy0), 0), G - 1);
            R = 2.f * Lmax;
            for (int sh = 0; sh <= level; sh++) {
                const uint32_t mo = morton2((uint32_t)cx >> sh, (uint32_t)cy >> sh);
                const int n0 = __ldg(a.start + coff + ((int64_t)mo << (2 * sh)));
                const int n1 = __ldg(a.start + coff + ((int64_t)(mo + 1) << (2 * sh)));
                const int cnt = n1 - n0;
                if (cnt >= (k + 3) / 4 || sh == level) {
                    const float side = smin * (float)(1 << sh);
                    R = side * sqrtf((float)k / (3.14159265f * fmaxf((float)cnt, 1.f))) * 1.25f;
                    break;
                }
            }
        }
        const float Rmax = 2.5f * Lmax;
        float Rlo = 0.f, Rhi = 3.0e38f;
        int m = 0, ok = 0;
        for (int att = 0; att < 48; att++) {
            __syncwarp();  // the previous attempt's reads of the list are done
            R = fminf(R, Rmax);
            const float R2 = R * R;
            // level: smallest sh with smin * 2^sh >= theta * R
            int sh = 0;
            {
                const float ratio = a.theta * R / smin;
                if (ratio > 1.f) {
                    const int rc = (int)fminf(ceilf(ratio), 1073741824.f);
                    sh = min(32 - __clz(rc - 1), level);
                }
            }
            const int shift = level - sh;           // Gl = 2^shift cells per axis at this level
            const int Gl = 1 << shift;
            const float pw = __int_as_float((127 + sh) << 23);  // 2^sh
            const float Sx = sx0 * pw, Sy = sy0 * pw;
            const float Re = R + tol;
            int vx0 = (int)floorf((pxr - Re) / Sx), vx1 = (int)floorf((pxr + Re) / Sx);
            int vy0 = (int)floorf((pyr - Re) / Sy), vy1 = (int)floorf((pyr + Re) / Sy);
            if (per0) { vx0 = max(vx0, -Gl); vx1 = min(vx1, 2 * Gl - 1); }
            else { vx0 = max(vx0, 0); vx1 = min(vx1, Gl - 1); }
            if (per1) { vy0 = max(vy0, -Gl); vy1 = min(vy1, 2 * Gl - 1); }
            else { vy0 = max(vy0, 0); vy1 = min(vy1, Gl - 1); }
            const int nx = max(vx1 - vx0 + 1, 0), ny = max(vy1 - vy0 + 1, 0);
            const int ncell = nx * ny;
            const float inv_nx = 1.f / (float)max(nx, 1);
            m = 0;
            int qn = 0;  // heavy cells waiting in rq (warp-uniform)
            // One cell per lane (`have`): cell (vx, vy) of the level 2^csh times
            // the finest, in virtual coordinates (images outside [0, Gl)). The
            // lane prunes it against the radius, queues it when heavy, else the
            // warp scans the cells' particles together.
            auto visit = [&](bool have, int vx, int vy, int csh) {
                const int cshift = level - csh;  // Gc = 2^cshift cells per axis at this level
                const int Gc = 1 << cshift;
                const float cpw = __int_as_float((127 + csh) << 23);  // 2^csh
                const float CSx = sx0 * cpw, CSy = sy0 * cpw;
                int cbase = 0, cnt = 0;
                uint32_t img = 4;
                float Ax = pr.x, Bx = 0.f, Cx = pr.z, Ay = pr.y, By = 0.f, Cy = pr.w;
                bool heavy = false;
                if (have) {
                    const int wx = vx >> cshift, wy = vy >> cshift;  // floor division by 2^cshift
                    const float xlo = (float)vx * CSx, ylo = (float)vy * CSy;
                    const float dxc = fmaxf(fmaxf(xlo - pxr, pxr - (xlo + CSx)) - tol, 0.f);
                    const float dyc = fmaxf(fmaxf(ylo - pyr, pyr - (ylo + CSy)) - tol, 0.f);
                    if (dxc * dxc + dyc * dyc <= R2) {
                        const uint32_t mo = morton2((uint32_t)(vx & (Gc - 1)), (uint32_t)(vy & (Gc - 1)));
                        const int j0 = __ldg(a.start + coff + ((int64_t)mo << (2 * csh)));
                        cnt = __ldg(a.start + coff + ((int64_t)(mo + 1) << (2 * csh))) - j0;
                        heavy = cnt > kHeavyCell && csh > 0;
                        img = (uint32_t)((1 - wx) * 3 + (1 - wy));
                        // image i = -w: hi part of q - i*d exact (Sterbenz) when i = +1,
                        // of p + i*d when i = -1
                        if (wx < 0) { Bx = dXh; Cx = cxp; } else if (wx > 0) { Ax = axm; Cx = cxm; }
                        if (wy < 0) { By = dYh; Cy = cyp; } else if (wy > 0) { Ay = aym; Cy = cym; }
                        cbase = j0;
                    }
                }
                // heavy cells go to the queue while it has room (else they are scanned)
                const uint32_t hb = __ballot_sync(0xffffffffu, heavy);
                if (heavy && qn + __popc(hb & lanemask_lt()) < kRefineQueue) {
                    rq[qn + __popc(hb & lanemask_lt())] = make_int4(vx, vy, csh, 0);
                    cnt = 0;
                }
                qn = min(qn + __popc(hb), kRefineQueue);
                int inc = cnt;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int y = __shfl_up_sync(0xffffffffu, inc, o);
                    if (lane >= o) inc += y;
                }
                const int tot = __shfl_sync(0xffffffffu, inc, 31);
                cbase -= inc - cnt;  // candidate t of this cell is particle cbase + t
                for (int t0 = 0; t0 < tot; t0 += 32) {
                    const int t = t0 + lane;
                    // source lane: the first lane whose inclusive count exceeds t
                    int src = 0;
#pragma unroll
                    for (int b = 16; b > 0; b >>= 1) {
                        const int iv = __shfl_sync(0xffffffffu, inc, src + b - 1);
                        if (iv <= t) src += b;
                    }
                    const int j = __shfl_sync(0xffffffffu, cbase, src) + t;
                    const uint32_t simg = __shfl_sync(0xffffffffu, img, src);
                    const float sAx = __shfl_sync(0xffffffffu, Ax, src), sBx = __shfl_sync(0xffffffffu, Bx, src);
                    const float sCx = __shfl_sync(0xffffffffu, Cx, src), sAy = __shfl_sync(0xffffffffu, Ay, src);
                    const float sBy = __shfl_sync(0xffffffffu, By, src), sCy = __shfl_sync(0xffffffffu, Cy, src);
                    bool pass = false;
                    float d2 = 0.f;
                    if (t < tot && j != (int)q) {
                        const float4 r = __ldg(&B.rec[j]);
                        const float dx = ((r.x - sBx) - sAx) + (r.z - sCx);
                        const float dy = ((r.y - sBy) - sAy) + (r.w - sCy);
                        d2 = __fmaf_rn(dx, dx, dy * dy);
                        pass = d2 <= R2;
                    }
                    const uint32_t bal = __ballot_sync(0xffffffffu, pass);
                    if (pass) {
                        const int pos = m + __popc(bal & lanemask_lt());
                        if (pos < CAP) {
                            skey[pos] = __float_as_uint(d2);
                            scode[pos] = ((uint32_t)j << kCodeShift) | simg;
                        }
                    }
                    m += __popc(bal);
                }
            };
            for (int cb = 0; cb < ncell; cb += 32) {
                const int ci = cb + lane;
                const int oy = (int)(((float)ci + 0.5f) * inv_nx);  // exact: ci, nx < 2^20
                visit(ci < ncell, vx0 + (ci - oy * nx), vy0 + oy, sh);
            }
            // refine the queued heavy cells: up to eight per round, a lane per child
            while (qn > 0) {
                const int take = min(qn, 8);
                __syncwarp();
                int4 e = make_int4(0, 0, 1, 0);
                const bool have = lane < 4 * take;
                if (have) e = rq[qn - take + (lane >> 2)];
                __syncwarp();  // the entries are read before visit() queues new ones
                qn -= take;
                visit(have, 2 * e.x + (lane & 1), 2 * e.y + ((lane >> 1) & 1), e.z - 1);
            }
            if (m < k) {
                if (R >= Rmax) { fl |= FLAG_KNN_FEW; break; }
                Rlo = R;
                const float g = m > 0 ? fmaxf(1.15f, sqrtf((float)k / (float)m) * 1.1f) : 2.f;
                R = Rhi < 3.0e38f ? 0.5f * (Rlo + Rhi) : R * g;
                continue;
            }
            if (m > CAP) {
                Rhi = R;
                const float g = sqrtf(0.5f * (float)(k + CAP) / (float)m);
                R = Rlo > 0.f ? 0.5f * (Rlo + Rhi) : R * g;
                continue;
            }
            __syncwarp();
            float Rn;
            if (select_write<MODE, NR>(a, S, q, m, R, epsabs, skey, scode, sord, sexact, lane, &Rn)) {
                Rlo = R;
                R = Rn;
                continue;
            }
            ok = 1;
            break;
        }
        if (!ok) {
            if (!(fl & FLAG_KNN_FEW)) fl |= FLAG_KNN_ATTEMPTS;
            for (int e = lane; e < k; e += 32) {
                a.D.nbr[q * k + e] = ((int32_t)q << kCodeShift) | 4;
                if (MODE == MODE_MIXED) a.D.d2f[q * k + e] = 0.f;
            }
        }
        __syncwarp();
    }
    if (fl && lane == 0) atomicOr(a.c.flags, fl);
}

// ---------------------------------------------------------------- group tiles
// k_knn_tile, one warp per group of 32 consecutive particles (consecutive in
// the Morton-sorted order, hence spatially compact), one lane per query:
//   1. every query takes the radius guess R = hgrow * previous h and the
//      rectangle of finest cells covering its square of half side R + tol;
//      the union of the rectangles is bounded by a box, taken at the finest
//      level with <= kTileBox cells and <= kTileRows rows;
//   2. each row of the box keeps the hull of the query rectangles crossing
//      it; the cells of those row hulls are contiguous particle ranges of the
//      sorted order, copied once into a shared-memory tile as FP32 positions
//      relative to the group's first particle (from the float-pair records;
//      for periodic images the shift is applied in FP64 before the rounding)
//      with their neighbour codes;
//   3. each lane scans the whole tile for its own query (broadcast reads) and
//      keeps every record within R as a 32-bit key: the squared distance in
//      units of R^2 / 2^23 (23 bits) above the tile slot (9 bits);
//   4. each lane keeps its k+1 smallest keys in ascending order (a
//      branch-free insertion chain in registers; an insertion sort in its
//      shared-memory column for k > 80) and accepts the first k when the FP32
//      values decide them:
//      the k-th lies 3 eps inside R (the tile held every candidate), the
//      (k+1)-th lies more than 2 eps beyond it (the set), and in the FP64
//      forms every neighbour is more than 2 eps from the next (the order;
//      the mixed form needs only the farthest to be unique, it fixes h).
// eps bounds |FP32 key - reference FP64 squared distance|: 2^-20 d2 for the
// products, 2^-19 D R for the relative coordinates (|coordinate| <= D, float
// pair differences), 2^-20 R^2 for the 23-bit key, and 2^-42 L R for the
// float-pair residues and the reference's own rounding of p + offset.
// Every other query goes to the deferred list that the per-query kernel
// finishes: short or overflowing lists, undecided sets or orders, tiles over
// capacity, no previous smoothing length (first evaluation), and queries of
// a group's second simulation (ensembles). Both paths return the same exact
// neighbour sets and, in the FP64 forms, the same order.
constexpr int kTileWarps = 4;
constexpr int kTileCap = 512;  // 9-bit tile slots
constexpr int kTileRows = 64;
constexpr int kTileBox = 1024;
constexpr int kTileCells = 511;  // cells whose record offsets a tile keeps (lane-rectangle scans)

template <int NR>
struct TileSmem {
    // per-query list capacity: k + 3 or more (k <= 37 for NR = 2); lists
    // longer than that go to the per-query kernel. 40 for NR = 2 measured
    // fastest at k = 32 (36 and 38 defer too many queries, 48 sorts more)
    static constexpr int LCAP = NR == 2 ? 40 : 24 * NR;
    // k <= 80: each lane sorts its whole list in registers with a network
    // (264, 610 or 2112 min/max for LCAP = 24, 40, 96); longer lists take a
    // shared-memory insertion sort
    static constexpr bool REG = NR <= 4;
    static constexpr bool NET = NR <= 4;
    static constexpr int A = NET ? LCAP : 81;
    float2 rec[kTileCap];             // candidate positions relative to the group origin
    uint32_t code[kTileCap];          // (slot << kCodeShift) | image
    int4 rect[32];                    // per query: cell rectangle at the tile level
    int32_t rx0[kTileRows], rx1[kTileRows], rpre[kTileRows + 1];
    int32_t self[32];                 // tile slot of each query's own record
    uint16_t cstart[kTileCells + 1];  // first record of each cell (one image block, <= kTileCells cells)
    alignas(16) uint32_t list[LCAP + 1][32];  // per-query keys, one column per query (+ a spare row)
};
static_assert(offsetof(TileSmem<1>, list) % 16 == 0 && offsetof(TileSmem<2>, list) % 16 == 0 &&
                  offsetof(TileSmem<4>, list) % 16 == 0 && offsetof(TileSmem<8>, list) % 16 == 0 &&
                  sizeof(TileSmem<2>) % 16 == 0 && offsetof(TileSmem<2>, rect) % 16 == 0,
              "tile shared-memory members must keep their alignment");

// Register budgets: the FP64 forms with lists of <= 40 entries get 128
// registers (four blocks per SM, which shared memory allows); the mixed form
// and longer lists compile without a block minimum (0), which measured
// spill-free where an explicit minimum of 1 or 4 did not.
template <int MODE, int NR>
__global__ void __launch_bounds__(kTileWarps * 32, (MODE == MODE_MIXED || NR > 2) ? 0 : 4) k_knn_tile(KnnArgs a) {
    using TS = TileSmem<NR>;
    constexpr int LCAP = TS::LCAP;
    constexpr uint32_t FULL = 0xffffffffu;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    TS &sm = reinterpret_cast<TS *>(smem_raw)[w];
    const int k = a.c.k;
    const int64_t n = a.c.n;
    const PArrays &B = a.B;
    const int64_t ngroups = (n + 31) >> 5;
    for (int64_t g = (int64_t)blockIdx.x * kTileWarps + w; g < ngroups; g += (int64_t)gridDim.x * kTileWarps) {
        const int64_t g0 = g << 5;
        const int64_t q = g0 + lane;
        const int s0 = sim_of(a.c, g0);
        const bool valid = q < n && sim_of(a.c, q) == s0;
        // a group that straddles two simulations of an ensemble searches for
        // the first one; the other simulation's queries are deferred
        defer_lanes(a, q < n && !valid, q, lane);
        const SimDev &S = a.c.sims[s0];
        const int level = S.level;
        const int G = 1 << level;
        const float sx0 = S.fs[0], sy0 = S.fs[1];
        const float tol = S.tol + S.overshoot;
        float4 pr = make_float4(0.f, 0.f, 0.f, 0.f);
        float R = 0.f;
        if (valid) {
            pr = B.rec[q];
            R = B.hprev[q] * a.hgrow;
        }
        const float pxr = pr.x + pr.z, pyr = pr.y + pr.w;
        // a radius guess well inside one period (no self image can come within R)
        const float Rcap = 0.25f * fminf(sx0, sy0) * (float)G;
        bool defer_all = __any_sync(FULL, valid && !(R > 0.f && R < Rcap));
        int x0 = INT_MAX, x1 = INT_MIN, y0 = INT_MAX, y1 = INT_MIN;
        if (valid && !defer_all) {
            const float Re = R + tol;
            x0 = (int)floorf((pxr - Re) / sx0);
            x1 = (int)floorf((pxr + Re) / sx0);
            y0 = (int)floorf((pyr - Re) / sy0);
            y1 = (int)floorf((pyr + Re) / sy0);
            if (S.periodic[0]) { x0 = max(x0, -G); x1 = min(x1, 2 * G - 1); }
            else { x0 = max(x0, 0); x1 = min(x1, G - 1); }
            if (S.periodic[1]) { y0 = max(y0, -G); y1 = min(y1, 2 * G - 1); }
            else { y0 = max(y0, 0); y1 = min(y1, G - 1); }
        }
        int sh = 0, BX0 = 0, BX1 = -1, BY0 = 0, BY1 = -1;
        if (!defer_all) {
            const int X0 = __reduce_min_sync(FULL, x0), X1 = __reduce_max_sync(FULL, x1);
            const int Y0 = __reduce_min_sync(FULL, y0), Y1 = __reduce_max_sync(FULL, y1);
            for (;; sh++) {
                const int nx = (X1 >> sh) - (X0 >> sh) + 1, ny = (Y1 >> sh) - (Y0 >> sh) + 1;
                if ((ny <= kTileRows && (int64_t)nx * ny <= kTileBox) || sh == level) {
                    defer_all = ny > kTileRows || (int64_t)nx * ny > kTileBox;
                    break;
                }
            }
            BX0 = X0 >> sh; BX1 = X1 >> sh; BY0 = Y0 >> sh; BY1 = Y1 >> sh;
        }
        // group origin: the first particle, as its FP64 position and as its
        // float-pair record (relative to the grid origin)
        const double2 P = valid ? B.pos[q] : make_double2(0.0, 0.0);
        const double gx = __shfl_sync(FULL, P.x, 0), gy = __shfl_sync(FULL, P.y, 0);
        const float ohx = __shfl_sync(FULL, pr.x, 0), olx = __shfl_sync(FULL, pr.z, 0);
        const float ohy = __shfl_sync(FULL, pr.y, 0), oly = __shfl_sync(FULL, pr.w, 0);
        int total = 0;
        bool rowscan = false;
        if (!defer_all) {
            const int shift = level - sh, Gl = 1 << shift;
            int ncell_one = INT_MAX;
            sm.rect[lane] = valid ? make_int4(x0 >> sh, x1 >> sh, y0 >> sh, y1 >> sh) : make_int4(1, 0, 1, 0);
            sm.self[lane] = -1;
            __syncwarp();
            // hull of the query rectangles crossing each row of the box
            const int ny = BY1 - BY0 + 1;
            for (int r = lane; r < ny; r += 32) {
                const int vy = BY0 + r;
                int hx0 = INT_MAX, hx1 = INT_MIN;
                for (int j = 0; j < 32; j++) {
                    const int4 rc = sm.rect[j];
                    if (rc.z <= vy && vy <= rc.w) { hx0 = min(hx0, rc.x); hx1 = max(hx1, rc.y); }
                }
                sm.rx0[r] = hx0;
                sm.rx1[r] = hx1;
            }
            __syncwarp();
            bool over = false;
            const double Lx = S.dimg[0], Ly = S.dimg[1];
            // image blocks: virtual rows / columns below 0 or from Gl on are images
            for (int wy = BY0 >> shift; wy <= (BY1 >> shift) && !over; wy++) {
                const int ry0 = max(BY0, wy * Gl) - BY0, ry1 = min(BY1, wy * Gl + Gl - 1) - BY0;
                const int nrow = ry1 - ry0 + 1;
                for (int wx = BX0 >> shift; wx <= (BX1 >> shift) && !over; wx++) {
                    const int xb0 = max(BX0, wx * Gl), xb1 = min(BX1, wx * Gl + Gl - 1);
                    const uint32_t img = (uint32_t)((1 - wx) * 3 + (1 - wy));
                    // exclusive prefix of the clipped row widths
                    int carry = 0;
                    for (int r0 = 0; r0 < nrow; r0 += 32) {
                        const int r = r0 + lane;
                        int wdt = 0;
                        if (r < nrow) {
                            const int c0 = max(sm.rx0[ry0 + r], xb0), c1 = min(sm.rx1[ry0 + r], xb1);
                            wdt = c1 >= c0 ? c1 - c0 + 1 : 0;  // rows no rectangle crosses hold INT_MAX / INT_MIN
                        }
                        int inc = wdt;
#pragma unroll
                        for (int o = 1; o < 32; o <<= 1) {
                            const int y = __shfl_up_sync(FULL, inc, o);
                            if (lane >= o) inc += y;
                        }
                        if (r < nrow) sm.rpre[r] = carry + inc - wdt;
                        carry += __shfl_sync(FULL, inc, 31);
                    }
                    const int ncell = carry;
                    __syncwarp();
                    for (int cb = 0; cb < ncell && !over; cb += 32) {
                        const int c = cb + lane;
                        int cnt = 0, j0 = 0;
                        if (c < ncell) {
                            // the row holding cell c: the last row whose prefix is <= c
                            int lo = 0, hi = nrow - 1;
                            while (lo < hi) {
                                const int mid = (lo + hi + 1) >> 1;
                                if (sm.rpre[mid] <= c) lo = mid; else hi = mid - 1;
                            }
                            const int vy = BY0 + ry0 + lo;
                            const int vx = max(sm.rx0[ry0 + lo], xb0) + (c - sm.rpre[lo]);
                            const uint32_t mo = morton2((uint32_t)(vx & (Gl - 1)), (uint32_t)(vy & (Gl - 1)));
                            j0 = __ldg(a.start + S.cell_off + ((int64_t)mo << (2 * sh)));
                            cnt = __ldg(a.start + S.cell_off + ((int64_t)(mo + 1) << (2 * sh))) - j0;
                        }
                        int inc = cnt;
#pragma unroll
                        for (int o = 1; o < 32; o <<= 1) {
                            const int y = __shfl_up_sync(FULL, inc, o);
                            if (lane >= o) inc += y;
                        }
                        const int tot = __shfl_sync(FULL, inc, 31);
                        if (total + tot > kTileCap) {
                            over = true;
                            break;
                        }
                        if (c <= kTileCells) sm.cstart[c] = (uint16_t)(total + inc - cnt);
                        // each lane copies its own cell's records (one contiguous
                        // range), four loads in flight
                        const int off = total + inc - cnt;  // tile slot of the cell's first record
                        if (img == 4) {
                            for (int r0 = 0; r0 < cnt; r0 += 4) {
                                // relative to the group origin from the float pairs (FP32 only)
                                float4 rv[4];
#pragma unroll
                                for (int u = 0; u < 4; u++)
                                    if (r0 + u < cnt) rv[u] = __ldg(&B.rec[j0 + r0 + u]);
#pragma unroll
                                for (int u = 0; u < 4; u++) {
                                    if (r0 + u < cnt) {
                                        const int j = j0 + r0 + u, t = off + r0 + u;
                                        sm.rec[t] = make_float2((rv[u].x - ohx) + (rv[u].z - olx),
                                                                (rv[u].y - ohy) + (rv[u].w - oly));
                                        sm.code[t] = ((uint32_t)j << kCodeShift) | img;
                                        if (j >= g0 && j < g0 + 32) sm.self[j - g0] = t;
                                    }
                                }
                            }
                        } else {
                            // an image: its virtual position (q shifted by wx periods) in
                            // FP64, relative to the group origin, rounded once to FP32
                            const double sx = (double)wx * Lx, sy = (double)wy * Ly;
                            for (int r = 0; r < cnt; r++) {
                                const double2 Q = B.pos[j0 + r];
                                const double qx = wx ? __dadd_rn(Q.x, sx) : Q.x;
                                const double qy = wy ? __dadd_rn(Q.y, sy) : Q.y;
                                sm.rec[off + r] = make_float2(__double2float_rn(__dsub_rn(qx, gx)),
                                                              __double2float_rn(__dsub_rn(qy, gy)));
                                sm.code[off + r] = ((uint32_t)(j0 + r) << kCodeShift) | img;
                            }
                        }
                        total += tot;
                    }
                    if (lane == 0 && ncell <= kTileCells) sm.cstart[ncell] = (uint16_t)total;
                    ncell_one = ncell;
                    __syncwarp();
                }
            }
            // one image block with few enough cells: each lane scans only the
            // cells of its own rectangle, row by row (contiguous record ranges)
            rowscan = (BX0 >> shift) == (BX1 >> shift) && (BY0 >> shift) == (BY1 >> shift) &&
                      ncell_one <= kTileCells;
            __syncwarp();
            defer_all = over || __any_sync(FULL, valid && sm.self[lane] < 0);
        }
        if (defer_all) {
            defer_lanes(a, valid, q, lane);
            __syncwarp();
            continue;
        }
        // ---- each lane scans the tile for its own query (its own record's
        // relative coordinates, computed as the tile's unshifted records are)
        const float rqx = (pr.x - ohx) + (pr.z - olx), rqy = (pr.y - ohy) + (pr.w - oly);
        const int myself = sm.self[lane];
        const float R2 = valid ? R * R : -1.f;
        const float qs = valid ? 8388608.f / R2 : 0.f;  // key units: R^2 / 2^23
        int cnt = 0;
        // branch-free: every record is written to the next free row (a spare
        // row once the list is full) and counted only when it passes
        auto visit = [&](int t, float2 c) {
            const float dx = c.x - rqx, dy = c.y - rqy;
            const float d2 = __fmaf_rn(dx, dx, dy * dy);
            const bool pass = d2 <= R2 && t != myself;
            const uint32_t kq = key23(d2, qs);
            sm.list[min(cnt, LCAP)][lane] = (kq << 9) | (uint32_t)t;
            cnt += pass ? 1 : 0;
        };
        if (rowscan) {
            // the cells of this query's rectangle: one record range per row
            // (invalid lanes hold an empty rectangle)
            const int lx0 = x0 >> sh, lx1 = x1 >> sh;
            for (int vy = y0 >> sh; vy <= (y1 >> sh); vy++) {
                const int rr = vy - BY0;
                const int base = sm.rpre[rr] - sm.rx0[rr];
                int t = sm.cstart[base + lx0];
                const int e = sm.cstart[base + lx1 + 1];
                for (; t + 2 <= e; t += 2) {
                    visit(t, sm.rec[t]);
                    visit(t + 1, sm.rec[t + 1]);
                }
                if (t < e) visit(t, sm.rec[t]);
            }
        } else {
            int t = 0;
            const float4 *rec2 = reinterpret_cast<const float4 *>(sm.rec);  // two records per load
            for (; t + 4 <= total; t += 4) {
                const float4 ab = rec2[t >> 1], cd = rec2[(t >> 1) + 1];
                visit(t, make_float2(ab.x, ab.y));
                visit(t + 1, make_float2(ab.z, ab.w));
                visit(t + 2, make_float2(cd.x, cd.y));
                visit(t + 3, make_float2(cd.z, cd.w));
            }
            for (; t < total; t++) visit(t, sm.rec[t]);
        }
        bool ok = valid && cnt >= k && cnt <= LCAP;
        // decisions in FP32 with the error bound eps
        const float unit = R2 * 1.1920928955078125e-7f;  // R^2 / 2^23
        const float ox = pxr - rqx, oy = pyr - rqy;      // group origin in grid coordinates
        const float Dx = fmaxf(fabsf((float)(BX0 << sh) * sx0 - ox), fabsf((float)((BX1 + 1) << sh) * sx0 - ox));
        const float Dy = fmaxf(fabsf((float)(BY0 << sh) * sy0 - oy), fabsf((float)((BY1 + 1) << sh) * sy0 - oy));
        // (the last term also covers the float-pair residues of the records, 2^-48 |p - origin|)
        const float ea = kEpsRel * (R2 + 2.f * R * (Dx + Dy)) + 2.3e-13f * fmaxf(S.flmax, S.fmag) * R;
        if (TS::REG) {
            // the A smallest keys, ascending, by a branch-free insertion chain
            // per list entry (registers only: no divergence, no smem latency chain)
            constexpr int A = TS::A;
            uint32_t arr[A];
            const int m = ok ? cnt : 0;
            if constexpr (TS::NET) {
#pragma unroll
                for (int i = 0; i < A; i++) arr[i] = i < m ? sm.list[i][lane] : 0xffffffffu;
                if (ok) OddEvenSort<A>{arr}.run();
            } else {
#pragma unroll
                for (int i = 0; i < A; i++) arr[i] = 0xffffffffu;
                for (int e = 0; e < m; e++) {
                    uint32_t v = sm.list[e][lane];
#pragma unroll
                    for (int i = 0; i < A; i++) {
                        const uint32_t lo = min(arr[i], v);
                        v = max(arr[i], v);
                        arr[i] = lo;
                    }
                }
            }
            // arr is ascending: the k-th key is the largest of the first k, the
            // (k+1)-th the smallest of the rest (reductions rather than
            // selects at i == k - 1, which the compiler turns into an indexed
            // load from local memory)
            uint32_t kth = 0, kprv = 0, knx = 0xffffffffu;
            bool order_ok = true;
#pragma unroll
            for (int i = 0; i < A; i++) {
                kth = max(kth, i < k ? arr[i] : 0u);
                kprv = max(kprv, i < k - 1 ? arr[i] : 0u);
                knx = min(knx, i >= k ? arr[i] : 0xffffffffu);
                if (MODE != MODE_MIXED && i > 0 && i < k) {
                    const float ki = (float)(arr[i] >> 9) * unit, kp = (float)(arr[i - 1] >> 9) * unit;
                    order_ok = order_ok && (ki - kp > 2.f * (kEpsRel * ki + ea));
                }
            }
            const float tau = (float)(kth >> 9) * unit, prv = (float)(kprv >> 9) * unit;
            const float nxt = cnt > k ? (float)(knx >> 9) * unit : 3.0e38f;
            const float et = kEpsRel * tau + ea;
            ok = ok && tau + 3.f * et <= R2 * (1.f - 4.8e-7f);
            ok = ok && (cnt == k || nxt - tau > 2.f * (kEpsRel * nxt + ea));
            if (MODE == MODE_MIXED) ok = ok && (k == 1 || tau - prv > 2.f * et);
            else ok = ok && order_ok;
            if (ok && MODE == MODE_MIXED) {
                // the mixed form needs the set, with the farthest last (it fixes h):
                // the entries up to the k-th key in tile (cell) order, which keeps
                // the force pass's gathers close in memory
                int32_t *out = a.D.nbr + q * k;
                float *o2 = a.D.d2f + q * k;
                int o = 0;
                for (int e = 0; e < cnt; e++) {
                    const uint32_t v = sm.list[e][lane];
                    if (v <= kth) {
                        const uint32_t slot = v & 511u;
                        const float2 c = sm.rec[slot];
                        const float dx = c.x - rqx, dy = c.y - rqy;
                        const int at = v == kth ? k - 1 : o++;
                        out[at] = (int32_t)sm.code[slot];
                        o2[at] = __fmaf_rn(dx, dx, dy * dy);
                    }
                }
            } else if (ok) {
                int32_t *out = a.D.nbr + q * k;
#pragma unroll
                for (int i = 0; i < A; i++) {
                    if (i < k) out[i] = (int32_t)sm.code[arr[i] & 511u];
                }
            }
        } else if (ok) {
            // insertion sort of this lane's keys in its shared-memory column
            for (int x = 1; x < cnt; x++) {
                const uint32_t v = sm.list[x][lane];
                int f = x - 1;
                uint32_t u = sm.list[f][lane];
                while (u > v) {
                    sm.list[f + 1][lane] = u;
                    if (--f < 0) break;
                    u = sm.list[f][lane];
                }
                sm.list[f + 1][lane] = v;
            }
            auto key = [&](int e) { return (float)(sm.list[e][lane] >> 9) * unit; };
            const float tau = key(k - 1);
            const float et = kEpsRel * tau + ea;
            ok = tau + 3.f * et <= R2 * (1.f - 4.8e-7f);
            if (ok && cnt > k) {
                const float nx = key(k);
                ok = nx - tau > 2.f * (kEpsRel * nx + ea);
            }
            if (ok) {
                if (MODE == MODE_MIXED) {
                    if (k > 1) ok = tau - key(k - 2) > 2.f * et;
                } else {
                    float prev = key(0);
                    for (int e = 1; e < k && ok; e++) {
                        const float cur = key(e);
                        ok = cur - prev > 2.f * (kEpsRel * cur + ea);
                        prev = cur;
                    }
                }
            }
            if (ok) {
                int32_t *out = a.D.nbr + q * k;
                for (int e = 0; e < k; e++) {
                    const uint32_t slot = sm.list[e][lane] & 511u;
                    out[e] = (int32_t)sm.code[slot];
                    if (MODE == MODE_MIXED) {
                        const float2 c = sm.rec[slot];
                        const float dx = c.x - rqx, dy = c.y - rqy;
                        a.D.d2f[q * k + e] = __fmaf_rn(dx, dx, dy * dy);
                    }
                }
            }
        }
        defer_lanes(a, valid && !ok, q, lane);
        __syncwarp();
    }
}

// ---------------------------------------------------------------- density
// five resident blocks (48 registers): the FP64 forms' first loop waits on the
// neighbour gathers, and more resident warps hide them (2.06 -> 2.02 ms at N = 1M)
template <int MODE>
__global__ void __launch_bounds__(256, 4) k_density(KnnArgs a) {
    const int k = a.c.k;
    const PArrays &B = a.B;
    unsigned fl = 0;
    // all particles, or (use_defer) only the queries the block tiles left to
    // the per-query search: the tiles computed the others' densities
    const int64_t nq = a.use_defer ? (int64_t)*a.D.ndefer : a.c.n;
    for (int64_t qi = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; qi < nq;
         qi += (int64_t)gridDim.x * blockDim.x) {
        const int64_t q = a.use_defer ? (int64_t)a.D.defer[qi] : qi;
        const int s = sim_of(a.c, q);
        const SimDev &S = a.c.sims[s];
        const double gamma = S.gamma;
        const double up = B.up[q];
        double h, rho, cs, cterm;
        if (MODE == MODE_EXACT64) {
            // sim/nearest-neighbour.go:64-66 square roots, sim/sph.go:306-323 sum farthest first
            double2 *dist = a.D.dist + q * k;
            const double2 P = B.pos[q];
            const int32_t *nb = a.D.nbr + q * k;
            const double dk2 = nbr_d2(S, B, P, (uint32_t)nb[k - 1]);
            if (!(dk2 < 0.4)) fl |= FLAG_SENTINEL;
            h = emu_sqrt(dk2);
            const EmuDivisor dh = emu_divisor(h);  // shared by the k quotients d/h
            // NNDists and q = NNDists/h; q grows with e (the list is sorted), so
            // the entries with q < 0.5 are a prefix of length s
            int s_lo = 0;
            for_each_nbr_desc(nb, k, [&](int e, uint32_t code) {
                const double d = e == k - 1 ? h : emu_sqrt(nbr_d2(S, B, P, code));
                // RN(d / h); in [0, 1] because d <= h
                const double x = emu_div(d, dh, h);
                s_lo += __double_as_longlong(x) < __double_as_longlong(0.5);  // x < 0.5 (x >= 0)
                dist[e] = make_double2(d, x);
            });
            // kernel sums farthest first (sim/sph.go:311-316), each branch of the
            // Monahan kernel in its own loop (no divergent branch per term); the
            // force's dF(q) replaces q in the list
            double acc = 0.0;
            if (S.kernel == SPH_KERNEL_WENDLAND) {
                for (int e = k - 1; e >= 0; e--) {
                    const double x = dist[e].y;
                    acc = __dadd_rn(acc, kf_exact(SPH_KERNEL_WENDLAND, x));
                    dist[e].y = kdf_exact(SPH_KERNEL_WENDLAND, x);
                }
            } else {
                for (int e = k - 1; e >= s_lo; e--) {  // q >= 0.5
                    const double x = dist[e].y;
                    const double a1 = emu_one_minus(x);  // x in [1/2, 1]: exact
                    const double a2 = emu_mul(a1, a1);
                    acc = __dadd_rn(acc, div3_rn(emu_mul(a2, a1)));
                    dist[e].y = -a2;
                }
                for (int e = s_lo - 1; e >= 0; e--) {  // q < 0.5
                    const double x = dist[e].y;
                    const double qq = emu_mul(x, x);
                    acc = __dadd_rn(acc, __dadd_rn(__dsub_rn(emu_mul(qq, x), qq), 1.0 / 6.0));
                    dist[e].y = __dsub_rn(emu_mul(emu_mul(3.0, x), x), emu_mul(2.0, x));
                }
            }
            const double hh = __dmul_rn(h, h);
            rho = emu_div(__dmul_rn(__dmul_rn(S.fpref, S.mass), acc), emu_divisor(hh), hh);
            if (!(rho >= 0.0 && rho < 1.0e308)) fl |= FLAG_Q_RANGE;  // a NaN or infinite distance
            cs = emu_sqrt(__dmul_rn(__dmul_rn(gamma, __dsub_rn(gamma, 1.0)), up));
            const double grho = __dmul_rn(gamma, rho);
            cterm = emu_div(__dmul_rn(cs, cs), emu_divisor(grho), grho);
        } else if (MODE == MODE_FAST64) {
            double2 *dist = a.D.dist + q * k;
            const double2 P = B.pos[q];
            const int32_t *nb = a.D.nbr + q * k;
            const double dk2 = nbr_d2(S, B, P, (uint32_t)nb[k - 1]);
            if (!(dk2 < 0.4)) fl |= FLAG_SENTINEL;
            h = emu_sqrt(dk2);
            const double inv_h = 1.0 / h;
            // q and 1/NNDists first; then the kernel sums and dF in branch-split
            // loops (q grows with e), leaving (dF, dF / NNDists) for the force
            int s_lo = 0;
            for_each_nbr_desc(nb, k, [&](int e, uint32_t code) {
                const double d2 = e == k - 1 ? dk2 : nbr_d2(S, B, P, code);
                const double y = rsqrt(d2);
                const double x = fmin(d2 * y * inv_h, 1.0);
                s_lo += x < 0.5;
                dist[e] = make_double2(x, y);
            });
            double acc = 0.0;
            if (S.kernel == SPH_KERNEL_WENDLAND) {
                for (int e = k - 1; e >= 0; e--) {
                    const double2 xy = dist[e];
                    acc += kf_fast(SPH_KERNEL_WENDLAND, xy.x);
                    const double drk = kdf_fast(SPH_KERNEL_WENDLAND, xy.x);
                    dist[e] = make_double2(drk, drk * xy.y);
                }
            } else {
                for (int e = k - 1; e >= s_lo; e--) {
                    const double2 xy = dist[e];
                    const double a1 = 1.0 - xy.x, a2 = a1 * a1;
                    acc += a2 * a1 * (1.0 / 3.0);
                    dist[e] = make_double2(-a2, -a2 * xy.y);
                }
                for (int e = s_lo - 1; e >= 0; e--) {
                    const double2 xy = dist[e];
                    acc += (xy.x - 1.0) * xy.x * xy.x + (1.0 / 6.0);
                    const double drk = (3.0 * xy.x - 2.0) * xy.x;
                    dist[e] = make_double2(drk, drk * xy.y);
                }
            }
            rho = S.fpref * S.mass * acc * (inv_h * inv_h);
            if (!(rho >= 0.0 && rho < 1.0e308)) fl |= FLAG_Q_RANGE;
            cs = sqrt(gamma * (gamma - 1.0) * up);
            cterm = cs * cs / (gamma * rho);
        } else {
            // FP64 only where it decides: the k-th neighbour's squared distance and h
            const double dk2 = nbr_d2(S, B, B.pos[q], (uint32_t)a.D.nbr[q * k + k - 1]);
            if (!(dk2 < 0.4)) fl |= FLAG_SENTINEL;
            h = emu_sqrt(dk2);
            // everything after h in FP32 (prefactors from FP32 copies)
            const float hf = __double2float_rn(h);
            const float inv_hf = 1.f / hf;
            const float *d2f = a.D.d2f + q * k;
            KahanF acc;
            auto term = [&](float v) { acc.add(kf_f32(S.kernel, fminf(sqrtf(v) * inv_hf, 1.f))); };
            if ((k & 3) == 0) {  // farthest first, four values per load
                const float4 *d4 = reinterpret_cast<const float4 *>(d2f);
                for (int b = (k >> 2) - 1; b >= 0; b--) {
                    const float4 v = d4[b];
                    term(v.w);
                    term(v.z);
                    term(v.y);
                    term(v.x);
                }
            } else {
                for (int e = k - 1; e >= 0; e--) term(d2f[e]);
            }
            const float rhof = S.ffm * (inv_hf * inv_hf) * acc.value_f();
            const float csf = sqrtf(S.fgg1 * __double2float_rn(up));
            const float ctf = csf * csf / (S.fgamma * rhof);
            a.D.rho[q] = rhof;
            a.D.c[q] = csf;
            a.D.h[q] = h;
            a.D.derf[q] = make_float4(csf, rhof, hf, ctf);
            continue;
        }
        a.D.rho[q] = rho;
        a.D.c[q] = cs;
        a.D.h[q] = h;
        a.D.der[q] = make_double4(cs, rho, h, cterm);
    }
    if (fl) atomicOr(a.c.flags, fl);
}

// ---------------------------------------------------------------- launch
constexpr int kKnnBlock = 256;

static int list_regs(int k) {
    const int need = (3 * k) / 2 + 8;
    return need <= 32 ? 1 : need <= 64 ? 2 : need <= 128 ? 4 : 8;
}
static size_t knn_smem(int nr) { return (size_t)(kKnnBlock / 32) * knn_warp_bytes(nr); }

template <int MODE, int NR>
static void knn_attr() {
    cudaFuncSetAttribute(k_knn<MODE, NR>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)knn_smem(NR));
    cudaFuncSetAttribute(k_knn_tile<MODE, NR>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)(kTileWarps * sizeof(TileSmem<NR>)));
}
template <int MODE>
static void knn_attrs_mode() {
    knn_attr<MODE, 1>();
    knn_attr<MODE, 2>();
    knn_attr<MODE, 4>();
    knn_attr<MODE, 8>();
}

// Sets the dynamic shared-memory limit of every instantiation; must run
// before any stream capture.
void knn_init_attrs() {
    knn_attrs_mode<MODE_EXACT64>();
    knn_attrs_mode<MODE_FAST64>();
    knn_attrs_mode<MODE_MIXED>();
    knn_block_init_attrs();
}

template <int MODE, int NR>
static int occ(int) {
    int nb = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_knn<MODE, NR>, kKnnBlock, knn_smem(NR));
    return nb;
}
template <int MODE, int NR>
static int occ_tile(int) {
    int nb = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_knn_tile<MODE, NR>, kTileWarps * 32,
                                                  kTileWarps * sizeof(TileSmem<NR>));
    return nb;
}

int knn_occupancy_blocks(int, int cap, int mode) {
    // cap carries k + slack; the list shape follows k
    const int nr = list_regs(std::max(1, cap - 16));
    auto pick = [&](auto f1, auto f2, auto f4, auto f8) { return nr == 1 ? f1(0) : nr == 2 ? f2(0) : nr == 4 ? f4(0) : f8(0); };
    if (mode == MODE_EXACT64) return pick(occ<MODE_EXACT64, 1>, occ<MODE_EXACT64, 2>, occ<MODE_EXACT64, 4>, occ<MODE_EXACT64, 8>);
    if (mode == MODE_FAST64) return pick(occ<MODE_FAST64, 1>, occ<MODE_FAST64, 2>, occ<MODE_FAST64, 4>, occ<MODE_FAST64, 8>);
    return pick(occ<MODE_MIXED, 1>, occ<MODE_MIXED, 2>, occ<MODE_MIXED, 4>, occ<MODE_MIXED, 8>);
}

int knn_tile_occupancy_blocks(int k, int mode) {
    const int nr = list_regs(k);
    auto pick = [&](auto f1, auto f2, auto f4, auto f8) { return nr == 1 ? f1(0) : nr == 2 ? f2(0) : nr == 4 ? f4(0) : f8(0); };
    if (mode == MODE_EXACT64)
        return pick(occ_tile<MODE_EXACT64, 1>, occ_tile<MODE_EXACT64, 2>, occ_tile<MODE_EXACT64, 4>, occ_tile<MODE_EXACT64, 8>);
    if (mode == MODE_FAST64)
        return pick(occ_tile<MODE_FAST64, 1>, occ_tile<MODE_FAST64, 2>, occ_tile<MODE_FAST64, 4>, occ_tile<MODE_FAST64, 8>);
    return pick(occ_tile<MODE_MIXED, 1>, occ_tile<MODE_MIXED, 2>, occ_tile<MODE_MIXED, 4>, occ_tile<MODE_MIXED, 8>);
}

// Queries whose neighbour set the block tiles decided but whose order the
// FP32 keys could not (two entries within the error bound): their list,
// written in FP32 order, is sorted by (the reference's FP64 squared distance,
// particle id, image code), the order the per-query search gives (it sorts
// the undecided runs by the same key; elsewhere the FP32 order agrees with
// it). One thread per query; lists of at most kRerankMaxK entries (the block
// tiles' longest).
constexpr int kRerankMaxK = 80;

template <int MODE>
__global__ void __launch_bounds__(128) k_rerank(KnnArgs a) {
    const int k = a.c.k;
    const int64_t nr = (int64_t)a.D.ndefer[1];
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nr; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t q = a.D.defer[a.c.n - 1 - i];
        const SimDev &S = a.c.sims[sim_of(a.c, q)];
        const double2 P = a.B.pos[q];
        int32_t *out = a.D.nbr + q * k;
        unsigned long long key[kRerankMaxK];
        uint32_t code[kRerankMaxK];
        for (int e = 0; e < k; e++) {  // insertion sort: the list is nearly sorted
            const uint32_t c = (uint32_t)out[e];
            const unsigned long long kk = (unsigned long long)__double_as_longlong(nbr_d2(S, a.B, P, c));
            int f = e - 1;
            while (f >= 0 && exact_greater(a.B, key[f], code[f], kk, c)) {
                key[f + 1] = key[f];
                code[f + 1] = code[f];
                f--;
            }
            key[f + 1] = kk;
            code[f + 1] = c;
        }
        for (int e = 0; e < k; e++) out[e] = (int32_t)code[e];
    }
}

bool knn_fuses_density(int k, int mode, const KnnTune &tune) {
    const int nr = list_regs(k);
    return mode == MODE_MIXED && tune.tile && tune.block_warps > 0 && nr <= 4 &&
           k == (nr == 1 ? 16 : nr == 2 ? 32 : 64);
}

template <int MODE, int NR>
static void launch_knn_nr(const KnnArgs &args, const Launch &L, const KnnTune &tune) {
    const int wpb = kKnnBlock / 32;
    const size_t smem = knn_smem(NR);
    const int resident = L.sms * std::max(tune.blocks_per_sm, 1);
    if (tune.tile && args.D.defer) {
        // group tiles, then the per-query kernel over the deferred queries
        cudaMemsetAsync(args.D.ndefer, 0, 2 * sizeof(int32_t), L.stream);
        KnnArgs b = args;
        b.rerank = MODE != MODE_MIXED && args.c.k <= kRerankMaxK ? 1 : 0;
        if (tune.block_warps > 0 && launch_knn_block(b, L, MODE, NR, tune.block_warps)) {
            if (b.rerank) k_rerank<MODE><<<L.sms * 4, 128, 0, L.stream>>>(b);
        } else {
            const int64_t groups = (args.c.n + 31) / 32;
            const int64_t tneed = (groups + kTileWarps - 1) / kTileWarps;
            const int tgrid = (int)std::max<int64_t>(
                1, std::min<int64_t>(tneed, (int64_t)L.sms * std::max(tune.tile_blocks_per_sm, 1)));
            k_knn_tile<MODE, NR><<<tgrid, kTileWarps * 32, kTileWarps * sizeof(TileSmem<NR>), L.stream>>>(args);
        }
        KnnArgs d = args;
        d.use_defer = 1;
        k_knn<MODE, NR><<<std::max(resident, 1), kKnnBlock, smem, L.stream>>>(d);
        return;
    }
    const int64_t need = (args.c.n + wpb - 1) / wpb;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(need, resident));
    k_knn<MODE, NR><<<grid, kKnnBlock, smem, L.stream>>>(args);
}

template <int MODE>
static void run_knn(const KnnArgs &args, const Launch &L, const KnnTune &tune) {
    const int nr = list_regs(args.c.k);
    if (nr == 1) launch_knn_nr<MODE, 1>(args, L, tune);
    else if (nr == 2) launch_knn_nr<MODE, 2>(args, L, tune);
    else if (nr == 4) launch_knn_nr<MODE, 4>(args, L, tune);
    else launch_knn_nr<MODE, 8>(args, L, tune);
}

template <int MODE>
static void run_density(const KnnArgs &args, const Launch &L) {
    const int64_t dneed = (args.c.n + 255) / 256;
    const int dgrid = (int)std::max<int64_t>(1, std::min<int64_t>(dneed, (int64_t)L.sms * 8));
    k_density<MODE><<<dgrid, 256, 0, L.stream>>>(args);
}

void launch_knn(const Ctx &c, const Launch &L, const PArrays &B, const Derived &D,
                const Tables &T, int mode, const KnnTune &tune) {
    KnnArgs a;
    a.c = c;
    a.B = B;
    a.D = D;
    a.start = T.start;
    a.theta = tune.theta;
    a.hgrow = tune.hgrow;
    a.use_defer = 0;
    a.fuse_density = knn_fuses_density(c.k, mode, tune) ? 1 : 0;
    if (mode == MODE_EXACT64) run_knn<MODE_EXACT64>(a, L, tune);
    else if (mode == MODE_FAST64) run_knn<MODE_FAST64>(a, L, tune);
    else run_knn<MODE_MIXED>(a, L, tune);
}

void launch_density(const Ctx &c, const Launch &L, const PArrays &B, const Derived &D, int mode,
                    const KnnTune *tune) {
    KnnArgs a{};
    a.c = c;
    a.B = B;
    a.D = D;
    a.use_defer = tune && D.defer && knn_fuses_density(c.k, mode, *tune) ? 1 : 0;
    if (mode == MODE_EXACT64) run_density<MODE_EXACT64>(a, L);
    else if (mode == MODE_FAST64) run_density<MODE_FAST64>(a, L);
    else run_density<MODE_MIXED>(a, L);
}

}  // namespace sphgpu
