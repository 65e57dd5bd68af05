// k_knn_block.cu -- exact periodic kNN with block tiles: the warps of a block
// share one candidate tile for 32 * WARPS consecutive (Morton-sorted, hence
// spatially compact) query particles, one thread per query.
//
// Replaces sim/nearest-neighbour.go:28-165 (nine tree traversals per particle
// with a sorted insertion queue) for every query whose neighbour set the FP32
// arithmetic below decides; the others go to the per-query kernel (k_knn).
//
// Per block tile:
//   1. each query takes the radius guess R = hgrow * previous h and the
//      rectangle of finest cells covering its square of half side R + tol, in
//      virtual cell coordinates (rows / columns below 0 or from G on are the
//      periodic images of the box); the block reduces them to a box and
//      picks the finest binning level at which the box has at most kRowCap
//      rows and kCellCap cells;
//   2. every row of the box keeps the hull of the query rectangles crossing
//      it (shared-memory atomics); the hull cells of all rows, laid out row
//      by row, are looked up in the cell table in one round (all loads in
//      flight), their populations prefix-summed by the block, and their
//      records copied with cp.async into a staging area (one round), then
//      converted to FP32 coordinates relative to the tile origin (image cells
//      in FP64 before the rounding); each row of the tile is then one
//      contiguous range of records ordered by cell column;
//   3. each thread scans, row by row, only the cells of its own rectangle that
//      the disc of radius R + tol reaches (the chord of the row), keeps every
//      record within R as a 32-bit key (squared distance in units of
//      R^2 / 2^KB above the tile slot) in its warp's list column, and decides
//      its set in FP32 with the same error bound as the warp tiles: the k-th
//      3 eps inside R, the (k+1)-th more than 2 eps beyond it, and in the FP64
//      forms every neighbour more than 2 eps from the next.
// The FP64 forms sort each list with Batcher's network (order needed); the
// mixed form at k = 16, 32 and 64 only selects the k smallest of its 24, 40
// or 96 list entries (TopGroups below) since it needs the set, the k-th and
// its neighbours in rank.
#include "knn_shared.cuh"

#include <algorithm>
#include <climits>
#include <cstddef>

namespace sphgpu {

namespace {

constexpr int kRowCap = 128;    // rows of a block tile
constexpr int kCellCap = 2048;  // cells of a block tile

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
    asm volatile("cp.async.commit_group;\ncp.async.wait_all;\n" ::: "memory");
}

// d2 in units of R^2 / 2^KB (qs = 2^KB / R^2) rounded to the nearest integer,
// clamped to KB bits: d2 qs + 2^23 lies in [2^23, 2^24), whose floats are the
// integers, so the mantissa is the key (no conversion instruction).
template <int KB>
__device__ __forceinline__ uint32_t key_of(float d2, float qs) {
    return min(__float_as_uint(__fmaf_rn(d2, qs, 8388608.f)) - 0x4B000000u, (1u << KB) - 1u);
}

// The G largest of A keys (A a multiple of G, G a power of two): A / G
// groups of G, each sorted by Batcher's odd-even merge network, then merged
// pairwise: the top G of two ascending groups a, b are the larger of each pair
// (a[i], b[G-1-i]), a bitonic sequence that a half-cleaner network sorts.
// Afterwards v[A-G..A-1] hold the G largest in ascending order and
// v[0..A-G-1] the others, unordered. A = 40, G = 8 takes 175 comparators
// (five 19-comparator sorts, four merges of 8 + 12) against the full sort's
// 610; A = 96, G = 32 takes 797 against 2112.
template <int A, int G>
struct TopGroups {
    uint32_t (&v)[A];
    __device__ __forceinline__ void ce(int i, int j) {
        const uint32_t lo = min(v[i], v[j]);
        v[j] = max(v[i], v[j]);
        v[i] = lo;
    }
    template <int GI>
    __device__ __forceinline__ void sort_groups() {
        if constexpr (GI < A / G) {
            OddEvenSort<A>{v}.template sort<GI * G, G>();
            sort_groups<GI + 1>();
        }
    }
    __device__ __forceinline__ void run() {
        static_assert(A % G == 0 && (G & (G - 1)) == 0, "groups of a power-of-two size");
        sort_groups<0>();
#pragma unroll
        for (int g = 0; g + 1 < A / G; g++) {
#pragma unroll
            for (int i = 0; i < G; i++) ce(g * G + i, (g + 2) * G - 1 - i);
            const int b = (g + 1) * G;
#pragma unroll
            for (int st = G / 2; st >= 1; st >>= 1) {
#pragma unroll
                for (int i = 0; i < G; i++)
                    if ((i & st) == 0) ce(b + i, b + i + st);
            }
        }
    }
};

template <int WARPS, int NR>
struct BlockSmem {
    static constexpr int Q = 32 * WARPS;           // queries per tile
    static constexpr int TCAP = 256 * WARPS;       // records per tile
    static constexpr int SB = WARPS == 8 ? 11 : WARPS == 4 ? 10 : 9;  // slot bits
    static constexpr int KB = 32 - SB;             // key bits
    static constexpr uint32_t SMASK = (1u << SB) - 1u;
    static constexpr int CCAP = kCellCap < TCAP ? kCellCap : TCAP;
    static constexpr int LCAP = NR == 2 ? 40 : 24 * NR;  // list entries per query (k + 3 or more)
    float2 rec[TCAP];        // FP32 position relative to the tile origin (during the build: cell words)
    uint32_t code[TCAP];     // (particle slot << kCodeShift) | image code
    uint16_t cstart[CCAP + 8];  // first record of each cell, cells row by row
    int32_t rx0[kRowCap], rx1[kRowCap], rpre[kRowCap + 1];
    int32_t self[Q];         // tile slot of each query's own record (-1: none)
    int32_t red[4 * WARPS + 8];
    // per-warp key lists (one column per query); during the build the
    // staging area of the raw records
    union alignas(16) {
        uint32_t list[WARPS][LCAP + 1][32];
        float4 staging[TCAP];
    } u;
};
using BS82 = BlockSmem<8, 2>;
using BS42 = BlockSmem<4, 2>;
using BS81 = BlockSmem<8, 1>;
using BS41 = BlockSmem<4, 1>;
using BS44 = BlockSmem<4, 4>;
static_assert(offsetof(BS82, u) % 16 == 0 && offsetof(BS42, u) % 16 == 0 && offsetof(BS81, u) % 16 == 0 &&
                  offsetof(BS41, u) % 16 == 0 && offsetof(BS44, u) % 16 == 0,
              "the staging area must be 16-byte aligned for cp.async");

}  // namespace

template <int MODE, int NR, int WARPS>
__global__ void __launch_bounds__(WARPS * 32, WARPS == 8 ? (NR <= 2 ? 3 : 1) : (NR <= 2 ? 6 : 2))
    k_knn_block(KnnArgs a) {
    using BS = BlockSmem<WARPS, NR>;
    constexpr int Q = BS::Q, TCAP = BS::TCAP, SB = BS::SB, KB = BS::KB, CCAP = BS::CCAP, LCAP = BS::LCAP;
    constexpr int NT = WARPS * 32;
    constexpr uint32_t FULL = 0xffffffffu;
    // the mixed form selects (rather than sorts) when k leaves a power-of-two
    // remainder of the list: k = 16 of 24, 32 of 40, 64 of 96
    constexpr bool SEL = MODE == MODE_MIXED && NR <= 4;
    constexpr int KSEL = NR == 1 ? 16 : NR == 2 ? 32 : 64;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    BS &sm = *reinterpret_cast<BS *>(smem_raw);
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int k = a.c.k;
    const int64_t n = a.c.n;
    const PArrays &B = a.B;
    const int64_t ntiles = (n + Q - 1) / Q;
    float4 *staging = sm.u.staging;
    uint32_t *cellw = reinterpret_cast<uint32_t *>(sm.rec);  // build phase: (first particle << 4) | image
    uint32_t (*mylist)[32] = sm.u.list[w];
    unsigned fl = 0;  // device error flags of this thread's queries

    for (int r = tid; r < kRowCap; r += NT) {
        sm.rx0[r] = INT_MAX;
        sm.rx1[r] = INT_MIN;
    }
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t q0 = tile * Q;
        const int64_t q = q0 + tid;
        const int64_t qlast = min(q0 + Q, n) - 1;
        // the simulations present in this tile (contiguous ranges): one pass each
        const int s_first = sim_of(a.c, q0), s_last = sim_of(a.c, qlast);
        for (int s = s_first; s <= s_last; s++) {
            const SimDev &S = a.c.sims[s];
            const int level = S.level;
            const int G = 1 << level;
            const float sx0 = S.fs[0], sy0 = S.fs[1];
            const float tol = S.tol + S.overshoot;
            const bool mine = q < n && sim_of(a.c, q) == s;
            float4 pr = make_float4(0.f, 0.f, 0.f, 0.f);
            float R = 0.f;
            if (mine) {
                pr = B.rec[q];
                R = B.hprev[q] * a.hgrow;
            }
            // a radius guess well inside one period (no self image within R)
            const float Rcap = 0.25f * fminf(sx0, sy0) * (float)G;
            const bool rok = R > 0.f && R < Rcap;
            defer_lanes(a, mine && !rok, q, lane);
            bool valid = mine && rok;
            const float pxr = pr.x + pr.z, pyr = pr.y + pr.w;
            int x0 = INT_MAX, x1 = INT_MIN, y0 = INT_MAX, y1 = INT_MIN;
            if (valid) {
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
            // ---- box of the rectangles, and each warp's first valid query
            {
                const int r0 = __reduce_min_sync(FULL, x0), r1 = __reduce_max_sync(FULL, x1);
                const int r2 = __reduce_min_sync(FULL, y0), r3 = __reduce_max_sync(FULL, y1);
                const unsigned vb = __ballot_sync(FULL, valid);
                if (lane == 0) {
                    sm.red[4 * w + 0] = r0;
                    sm.red[4 * w + 1] = r1;
                    sm.red[4 * w + 2] = r2;
                    sm.red[4 * w + 3] = r3;
                    sm.red[4 * WARPS + w] = vb ? w * 32 + __ffs(vb) - 1 : INT_MAX;
                }
            }
            sm.self[tid] = -1;
            __syncthreads();
            int X0 = INT_MAX, X1 = INT_MIN, Y0 = INT_MAX, Y1 = INT_MIN, org = INT_MAX;
#pragma unroll
            for (int i = 0; i < WARPS; i++) {
                X0 = min(X0, sm.red[4 * i]);
                X1 = max(X1, sm.red[4 * i + 1]);
                Y0 = min(Y0, sm.red[4 * i + 2]);
                Y1 = max(Y1, sm.red[4 * i + 3]);
            }
            // origin: the first valid query of the middle warp (or the next
            // warp with one), near the middle of the Morton-ordered tile
            for (int i = 0; i < WARPS && org == INT_MAX; i++) {
                const int wi = (WARPS / 2 + i) % WARPS;
                org = sm.red[4 * WARPS + wi];
            }
            if (org == INT_MAX) {  // no valid query in this pass
                __syncthreads();
                continue;
            }
            // level: the finest with at most kRowCap rows and CCAP cells
            int sh = 0;
            for (;; sh++) {
                const int nx = (X1 >> sh) - (X0 >> sh) + 1, ny = (Y1 >> sh) - (Y0 >> sh) + 1;
                if ((ny <= kRowCap && (int64_t)nx * ny <= CCAP) || sh == level) break;
            }
            const int BX0 = X0 >> sh, BX1 = X1 >> sh, BY0 = Y0 >> sh, BY1 = Y1 >> sh;
            const int ny = BY1 - BY0 + 1;
            bool tile_ok = ny <= kRowCap && (int64_t)(BX1 - BX0 + 1) * ny <= CCAP;
            const int shift = level - sh, Gl = 1 << shift;
            // a box wider than one period would hold a particle twice
            tile_ok = tile_ok && (BX1 - BX0 + 1) <= Gl && ny <= Gl;
            // ---- row hulls (the rows were reset at the end of the previous pass)
            if (tile_ok && valid) {
                const int lx0 = x0 >> sh, lx1 = x1 >> sh;
                for (int vy = y0 >> sh; vy <= (y1 >> sh); vy++) {
                    atomicMin(&sm.rx0[vy - BY0], lx0);
                    atomicMax(&sm.rx1[vy - BY0], lx1);
                }
            }
            __syncthreads();
            // ---- row prefix (one warp)
            if (tile_ok && w == 0) {
                int carry = 0;
                for (int r0 = 0; r0 < ny; r0 += 32) {
                    const int r = r0 + lane;
                    int wdt = 0;
                    if (r < ny) {
                        const int c0 = sm.rx0[r], c1 = sm.rx1[r];
                        wdt = c1 >= c0 ? c1 - c0 + 1 : 0;
                    }
                    int inc = wdt;
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const int y = __shfl_up_sync(FULL, inc, o);
                        if (lane >= o) inc += y;
                    }
                    if (r < ny) sm.rpre[r] = carry + inc - wdt;
                    carry += __shfl_sync(FULL, inc, 31);
                }
                if (lane == 0) sm.rpre[ny] = carry;
            }
            __syncthreads();
            const int ncell = tile_ok ? sm.rpre[ny] : 0;
            // ---- cell lookups, all in flight: cell c (row-major) -> first
            // particle, population; cells of image blocks carry their image
            constexpr int CPT = (CCAP + NT - 1) / NT;
            {
                int j0v[CPT], cntv[CPT];
                uint32_t imgv[CPT];
#pragma unroll
                for (int i = 0; i < CPT; i++) {
                    const int c = tid + i * NT;
                    j0v[i] = 0;
                    cntv[i] = 0;
                    imgv[i] = 4;
                    if (c < ncell) {
                        int lo = 0, hi = ny - 1;  // the row holding cell c: the last with rpre <= c
                        while (lo < hi) {
                            const int mid = (lo + hi + 1) >> 1;
                            if (sm.rpre[mid] <= c) lo = mid; else hi = mid - 1;
                        }
                        const int vy = BY0 + lo;
                        const int vx = sm.rx0[lo] + (c - sm.rpre[lo]);
                        const int wx = vx >> shift, wy = vy >> shift;  // image block (floor division)
                        imgv[i] = (uint32_t)((1 - wx) * 3 + (1 - wy));
                        const uint32_t mo = morton2((uint32_t)(vx & (Gl - 1)), (uint32_t)(vy & (Gl - 1)));
                        j0v[i] = __ldg(a.start + S.cell_off + ((int64_t)mo << (2 * sh)));
                        cntv[i] = __ldg(a.start + S.cell_off + ((int64_t)(mo + 1) << (2 * sh)));
                    }
                }
#pragma unroll
                for (int i = 0; i < CPT; i++) {
                    const int c = tid + i * NT;
                    if (c < ncell) {
                        const int cnt = cntv[i] - j0v[i];
                        cellw[c] = ((uint32_t)j0v[i] << 4) | imgv[i];
                        sm.cstart[c + 1] = (uint16_t)min(cnt, 0xffff);
                    }
                }
            }
            __syncthreads();
            // ---- exclusive prefix of the cell populations (block scan over
            // contiguous chunks of CPT cells per thread)
            int total = 0;
            {
                int loc[CPT], sum = 0;
#pragma unroll
                for (int i = 0; i < CPT; i++) {
                    const int c = tid * CPT + i;
                    loc[i] = c < ncell ? sm.cstart[c + 1] : 0;
                    sum += loc[i];
                }
                int inc = sum;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int y = __shfl_up_sync(FULL, inc, o);
                    if (lane >= o) inc += y;
                }
                if (lane == 31) sm.red[w] = inc;
                __syncthreads();
                int wbase = 0, all = 0;
#pragma unroll
                for (int i = 0; i < WARPS; i++) {
                    const int v = sm.red[i];
                    wbase += i < w ? v : 0;
                    all += v;
                }
                total = all;
                int run = wbase + inc - sum;
                // (the warp sums are next written in the next pass, after its barriers)
                if (tile_ok && total <= TCAP) {
#pragma unroll
                    for (int i = 0; i < CPT; i++) {
                        const int c = tid * CPT + i;
                        if (c < ncell) sm.cstart[c] = (uint16_t)run;
                        run += loc[i];
                    }
                    if (tid == 0) sm.cstart[ncell] = (uint16_t)total;
                }
            }
            __syncthreads();
            tile_ok = tile_ok && total <= TCAP;
            // ---- record copies into the staging area (cp.async, all in
            // flight): FP32 float-pair records, or FP64 positions for image cells
            if (tile_ok) {
                for (int c = tid; c < ncell; c += NT) {
                    const uint32_t cw = cellw[c];
                    const int j0 = (int)(cw >> 4);
                    const uint32_t img = cw & 15u;
                    const int t0 = sm.cstart[c], t1 = sm.cstart[c + 1];
                    for (int t = t0; t < t1; t++) {
                        const int j = j0 + (t - t0);
                        cp_async16(&staging[t], img == 4u ? (const void *)&B.rec[j] : (const void *)&B.pos[j]);
                        sm.code[t] = ((uint32_t)j << kCodeShift) | img;
                        if (img == 4u && j >= q0 && j < q0 + Q) sm.self[j - q0] = t;
                    }
                }
            }
            cp_async_wait_all();
            __syncthreads();
            // origin of the tile's relative coordinates
            const int64_t qo = q0 + org;
            const float4 po = B.rec[qo];
            const double2 Po = B.pos[qo];
            // ---- conversion to FP32 coordinates relative to the origin
            if (tile_ok) {
                const double Lx = S.dimg[0], Ly = S.dimg[1];
                for (int t = tid; t < total; t += NT) {
                    const float4 raw = staging[t];
                    const uint32_t img = sm.code[t] & 15u;
                    float2 c;
                    if (img == 4u) {
                        c = make_float2((raw.x - po.x) + (raw.z - po.z), (raw.y - po.y) + (raw.w - po.w));
                    } else {
                        // virtual position (q shifted by w periods) in FP64, relative to
                        // the origin, rounded once to FP32; image code i = -w
                        const double2 Qd = *reinterpret_cast<const double2 *>(&raw);
                        const int wx = 1 - (int)(img / 3u), wy = 1 - (int)(img % 3u);
                        const double qx = wx ? __dadd_rn(Qd.x, (double)wx * Lx) : Qd.x;
                        const double qy = wy ? __dadd_rn(Qd.y, (double)wy * Ly) : Qd.y;
                        c = make_float2(__double2float_rn(__dsub_rn(qx, Po.x)), __double2float_rn(__dsub_rn(qy, Po.y)));
                    }
                    sm.rec[t] = c;
                }
            }
            __syncthreads();  // the tile is complete; the list area is free again
            const int myself = sm.self[tid];
            valid = valid && tile_ok;
            // a query whose own record is not in the tile goes to the per-query search
            defer_lanes(a, mine && rok && (!tile_ok || myself < 0), q, lane);
            valid = valid && myself >= 0;
            // ---- each thread scans the cells of its rectangle that its disc reaches
            const float rqx = (pr.x - po.x) + (pr.z - po.z), rqy = (pr.y - po.y) + (pr.w - po.w);
            const float R2 = valid ? R * R : -1.f;
            const float qs = valid ? __int_as_float((127 + KB) << 23) / R2 : 0.f;  // key units: R^2 / 2^KB
            int cnt = 0;
            if (valid) {
                const float pw = __int_as_float((127 + sh) << 23);  // 2^sh
                const float Sx = sx0 * pw, Sy = sy0 * pw;
                const float Re = R + tol, Re2 = Re * Re;
                const int lx0 = x0 >> sh, lx1 = x1 >> sh;
                for (int vy = y0 >> sh; vy <= (y1 >> sh); vy++) {
                    // the chord of the disc in this row of cells
                    const float ylo = (float)vy * Sy;
                    const float dyc = fmaxf(fmaxf(ylo - pyr, pyr - (ylo + Sy)), 0.f);
                    if (dyc > Re) continue;
                    const float half = sqrtf(fmaxf(Re2 - dyc * dyc, 0.f)) * 1.0000005f;
                    const int cx0 = max(lx0, (int)floorf((pxr - half) / Sx));
                    const int cx1 = min(lx1, (int)floorf((pxr + half) / Sx));
                    const int rr = vy - BY0;
                    const int base = sm.rpre[rr] - sm.rx0[rr];
                    int t = cx0 <= cx1 ? sm.cstart[base + cx0] : 0;
                    const int e = cx0 <= cx1 ? sm.cstart[base + cx1 + 1] : 0;
                    // four records per round, their loads issued together (the
                    // round's tail repeats the row's last record and never passes)
                    for (; t < e; t += 4) {
                        float2 cc[4];
#pragma unroll
                        for (int u = 0; u < 4; u++) cc[u] = sm.rec[min(t + u, e - 1)];
#pragma unroll
                        for (int u = 0; u < 4; u++) {
                            const float dx = cc[u].x - rqx, dy = cc[u].y - rqy;
                            const float d2 = __fmaf_rn(dx, dx, dy * dy);
                            const bool pass = d2 <= R2 && t + u != myself && t + u < e;
                            mylist[min(cnt, LCAP)][lane] = (key_of<KB>(d2, qs) << SB) | (uint32_t)(t + u);
                            cnt += pass ? 1 : 0;
                        }
                    }
                }
            }
            bool ok = valid && cnt >= k && cnt <= LCAP;
            // decisions in FP32 with the error bound eps
            const float unit = __int_as_float((127 - KB) << 23) * R2;  // R^2 / 2^KB
            const float ox = pxr - rqx, oy = pyr - rqy;  // tile origin in grid coordinates
            const float Dx = fmaxf(fabsf((float)(BX0 << sh) * sx0 - ox), fabsf((float)((BX1 + 1) << sh) * sx0 - ox));
            const float Dy = fmaxf(fabsf((float)(BY0 << sh) * sy0 - oy), fabsf((float)((BY1 + 1) << sh) * sy0 - oy));
            const float ea = kEpsRel * (R2 + 2.f * R * (Dx + Dy)) + 2.3e-13f * fmaxf(S.flmax, S.fmag) * R;
            constexpr int A = LCAP;
            uint32_t arr[A];
            const int m = ok ? cnt : 0;
#pragma unroll
            for (int i = 0; i < A; i++) arr[i] = i < m ? mylist[i][lane] : 0xffffffffu;
            uint32_t kth = 0, kprv = 0, knx = 0xffffffffu;
            bool order_ok = true;
            auto sorted_path = [&]() {
                if (ok) OddEvenSort<A>{arr}.run();
#pragma unroll
                for (int i = 0; i < A; i++) {
                    kth = max(kth, i < k ? arr[i] : 0u);
                    kprv = max(kprv, i < k - 1 ? arr[i] : 0u);
                    knx = min(knx, i >= k ? arr[i] : 0xffffffffu);
                    if (MODE != MODE_MIXED && i > 0 && i < k) {
                        const float ki = (float)(arr[i] >> SB) * unit, kp = (float)(arr[i - 1] >> SB) * unit;
                        order_ok = order_ok && (ki - kp > 2.f * (kEpsRel * ki + ea));
                    }
                }
            };
            if constexpr (SEL) {
                if (k == KSEL) {
                    if (ok) TopGroups<A, A - KSEL>{arr}.run();
                    // the k-th smallest is the largest of v[0..k-1], the (k-1)-th
                    // the second largest, the (k+1)-th the smallest of the top group
#pragma unroll
                    for (int i = 0; i < KSEL; i++) {
                        kprv = max(kprv, min(kth, arr[i]));
                        kth = max(kth, arr[i]);
                    }
                    knx = arr[KSEL];
                } else {
                    sorted_path();
                }
            } else {
                sorted_path();
            }
            const float tau = (float)(kth >> SB) * unit, prv = (float)(kprv >> SB) * unit;
            const float nxt = cnt > k ? (float)(knx >> SB) * unit : 3.0e38f;
            const float et = kEpsRel * tau + ea;
            ok = ok && tau + 3.f * et <= R2 * (1.f - 4.8e-7f);
            ok = ok && (cnt == k || nxt - tau > 2.f * (kEpsRel * nxt + ea));
            // FP64 forms: a decided set whose order the FP32 keys cannot settle
            // (two entries within the error bound) is written in FP32 order and
            // re-sorted by the FP64 keys afterwards (k_rerank), when enabled
            bool rerank = false;
            if (MODE == MODE_MIXED) {
                ok = ok && (k == 1 || tau - prv > 2.f * et);
            } else {
                rerank = a.rerank && ok && !order_ok;
                ok = ok && (order_ok || rerank);
            }
            // Outputs go out four entries per store (each list row is 16-byte
            // aligned: q k 4 bytes with k a multiple of four).
            bool stored = false;
            if constexpr (SEL) {
                if (ok && k == KSEL) {
                    // the selected set straight from registers, the farthest last
                    // (it fixes h): kth and the entry in arr[k-1] trade places
                    int4 *out4 = reinterpret_cast<int4 *>(a.D.nbr + q * KSEL);
                    float4 *o24 = reinterpret_cast<float4 *>(a.D.d2f + q * KSEL);
                    // With the density fused (k_density's mixed form for this query):
                    // h from the farthest neighbour's FP64 squared distance in the
                    // reference's rounding, then the FP32 kernel sum over the
                    // squared distances written here, which then need not be stored
                    const bool fuse = a.fuse_density != 0;
                    double hq = 0.0;
                    float inv_hf = 0.f;
                    if (fuse) {
                        const double dk2 = nbr_d2(S, B, B.pos[q], sm.code[kth & BS::SMASK]);
                        if (!(dk2 < 0.4)) fl |= FLAG_SENTINEL;
                        hq = emu_sqrt(dk2);
                        inv_hf = 1.f / __double2float_rn(hq);
                    }
                    KahanF acc;  // farthest first, the order of k_density's sum
#pragma unroll
                    for (int c = KSEL / 4 - 1; c >= 0; c--) {
                        uint32_t cd[4];
                        float dd[4];
#pragma unroll
                        for (int u = 0; u < 4; u++) {
                            const int i = 4 * c + u;
                            const uint32_t v = i == KSEL - 1 ? kth : (arr[i] == kth ? arr[KSEL - 1] : arr[i]);
                            const uint32_t slot = v & BS::SMASK;
                            const float2 cc = sm.rec[slot];
                            const float dx = cc.x - rqx, dy = cc.y - rqy;
                            cd[u] = sm.code[slot];
                            dd[u] = __fmaf_rn(dx, dx, dy * dy);
                        }
                        out4[c] = make_int4((int)cd[0], (int)cd[1], (int)cd[2], (int)cd[3]);
                        if (fuse) {
#pragma unroll
                            for (int u = 3; u >= 0; u--) acc.add(kf_f32(S.kernel, fminf(sqrtf(dd[u]) * inv_hf, 1.f)));
                        } else {
                            o24[c] = make_float4(dd[0], dd[1], dd[2], dd[3]);
                        }
                    }
                    if (fuse) {
                        const float hf = __double2float_rn(hq);
                        const float rhof = S.ffm * (inv_hf * inv_hf) * acc.value_f();
                        const float csf = sqrtf(S.fgg1 * __double2float_rn(B.up[q]));
                        const float ctf = csf * csf / (S.fgamma * rhof);
                        a.D.rho[q] = rhof;
                        a.D.c[q] = csf;
                        a.D.h[q] = hq;
                        a.D.derf[q] = make_float4(csf, rhof, hf, ctf);
                    }
                    stored = true;
                }
            }
            if (ok && !stored && MODE == MODE_MIXED) {
                // the set with the farthest last (it fixes h), the rest in tile
                // (cell) order
                int32_t *out = a.D.nbr + q * k;
                float *o2 = a.D.d2f + q * k;
                int o = 0;
                for (int e0 = 0; e0 < cnt; e0 += 4) {
                    uint32_t v[4], cd[4];
                    float2 cc[4];
#pragma unroll
                    for (int u = 0; u < 4; u++) v[u] = e0 + u < cnt ? mylist[e0 + u][lane] : 0xffffffffu;
#pragma unroll
                    for (int u = 0; u < 4; u++) {
                        const uint32_t slot = min(v[u] & BS::SMASK, (uint32_t)(TCAP - 1));
                        cc[u] = sm.rec[slot];
                        cd[u] = sm.code[slot];
                    }
#pragma unroll
                    for (int u = 0; u < 4; u++) {
                        if (v[u] <= kth) {
                            const float dx = cc[u].x - rqx, dy = cc[u].y - rqy;
                            const int at = v[u] == kth ? k - 1 : o++;
                            out[at] = (int32_t)cd[u];
                            o2[at] = __fmaf_rn(dx, dx, dy * dy);
                        }
                    }
                }
            } else if (ok && MODE != MODE_MIXED) {
                // sorted, nearest first
                int32_t *out = a.D.nbr + q * k;
                if ((k & 3) == 0) {
                    int4 *out4 = reinterpret_cast<int4 *>(out);
#pragma unroll
                    for (int c = 0; c < A / 4; c++) {
                        if (4 * c < k)
                            out4[c] = make_int4((int)sm.code[arr[4 * c] & BS::SMASK], (int)sm.code[arr[4 * c + 1] & BS::SMASK],
                                                (int)sm.code[arr[4 * c + 2] & BS::SMASK],
                                                (int)sm.code[arr[4 * c + 3] & BS::SMASK]);
                    }
                } else {
#pragma unroll
                    for (int i = 0; i < A; i++) {
                        if (i < k) out[i] = (int32_t)sm.code[arr[i] & BS::SMASK];
                    }
                }
            }
            defer_lanes(a, valid && !ok, q, lane);
            if (MODE != MODE_MIXED) rerank_lanes(a, valid && rerank, q, lane);
            __syncthreads();  // every thread is done with the rows and the tile
            for (int r = tid; r < kRowCap; r += NT) {  // rows reset for the next pass
                sm.rx0[r] = INT_MAX;
                sm.rx1[r] = INT_MIN;
            }
        }
    }
    if (fl) atomicOr(a.c.flags, fl);
}

// ------------------------------------------------------------------ launch
template <int MODE, int NR, int WARPS>
static size_t block_smem() { return sizeof(BlockSmem<WARPS, NR>); }

// resident blocks per SM of each instantiation [mode][list shape 1, 2, 4][4 or 8 warps]
static int g_block_occ[3][3][2];

template <int MODE, int NR, int WARPS>
static void block_attr() {
    cudaFuncSetAttribute(k_knn_block<MODE, NR, WARPS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)block_smem<MODE, NR, WARPS>());
    int nb = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_knn_block<MODE, NR, WARPS>, WARPS * 32,
                                                  block_smem<MODE, NR, WARPS>());
    g_block_occ[MODE][NR == 1 ? 0 : NR == 2 ? 1 : 2][WARPS == 8] = std::max(nb, 1);
}

template <int MODE>
static void block_attrs_mode() {
    block_attr<MODE, 1, 4>();
    block_attr<MODE, 1, 8>();
    block_attr<MODE, 2, 4>();
    block_attr<MODE, 2, 8>();
    block_attr<MODE, 4, 4>();
}

// Sets the dynamic shared-memory limit of every block-tile instantiation and
// records its occupancy; must run before any stream capture.
void knn_block_init_attrs() {
    block_attrs_mode<MODE_EXACT64>();
    block_attrs_mode<MODE_FAST64>();
    block_attrs_mode<MODE_MIXED>();
}

template <int MODE, int NR, int WARPS>
static void block_launch(const KnnArgs &args, const Launch &L) {
    const int64_t ntiles = (args.c.n + 32 * WARPS - 1) / (32 * WARPS);
    const int occ = std::max(g_block_occ[MODE][NR == 1 ? 0 : NR == 2 ? 1 : 2][WARPS == 8], 1);
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(ntiles, (int64_t)L.sms * occ));
    k_knn_block<MODE, NR, WARPS><<<grid, WARPS * 32, block_smem<MODE, NR, WARPS>(), L.stream>>>(args);
}

template <int MODE>
static bool block_mode(const KnnArgs &args, const Launch &L, int nr, int warps) {
    if (nr == 1) {
        if (warps == 8) block_launch<MODE, 1, 8>(args, L);
        else block_launch<MODE, 1, 4>(args, L);
    } else if (nr == 2) {
        if (warps == 8) block_launch<MODE, 2, 8>(args, L);
        else block_launch<MODE, 2, 4>(args, L);
    } else if (nr == 4) {
        block_launch<MODE, 4, 4>(args, L);
    } else {
        return false;
    }
    return true;
}

// Block-tile search for list shape nr and `warps` warps per tile (4 or 8);
// false when no block kernel serves this list shape (the warp tiles do).
bool launch_knn_block(const KnnArgs &args, const Launch &L, int mode, int nr, int warps) {
    if (mode == MODE_EXACT64) return block_mode<MODE_EXACT64>(args, L, nr, warps);
    if (mode == MODE_FAST64) return block_mode<MODE_FAST64>(args, L, nr, warps);
    return block_mode<MODE_MIXED>(args, L, nr, warps);
}

}  // namespace sphgpu
