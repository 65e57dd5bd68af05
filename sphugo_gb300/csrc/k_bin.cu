// k_bin.cu -- cell binning: the GB300 replacement of the reference's spatial
// index (sim/core.go:126-224 Partition/Treebuild, rebuilt on every force
// evaluation at sim/sph.go:406). Instead of a pointer tree it builds, per
// simulation, a dense Morton-ordered cell table at a fine level: drift +
// cell key + histogram (one atomic per particle, whose return value is the
// particle's rank inside its cell), an exclusive scan of the histogram into
// cell starts, and a permute of the state into cell order. Every coarser
// level's cell is a contiguous range of the same table, which is what the
// neighbour search walks. All four passes are HBM streams.
#include "common.cuh"

namespace sphgpu {

// ------------------------------------------------------------------ prep
// Per-simulation reset of the per-binning reductions (one thread per sim).
__global__ void k_prep(Ctx c) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= c.nsims) return;
    SimDev &S = c.sims_rw[s];
    S.overshoot = 0.f;
    S.bbox[0] = ~0ull; S.bbox[1] = 0ull;
    S.bbox[2] = ~0ull; S.bbox[3] = 0ull;
}

void launch_prep(const Ctx &c, const Launch &L, bool) {
    k_prep<<<(c.nsims + 127) / 128, 128, 0, L.stream>>>(c);
}

// ------------------------------------------------------------------ bbox
// Bounding box of the predicted positions, for simulations with an open axis.
__global__ void k_bbox(Ctx c, PArrays A, int pred) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < c.n;
         i += (int64_t)gridDim.x * blockDim.x) {
        int s = sim_of(c, i);
        const SimDev &S = c.sims[s];
        if (S.periodic[0] && S.periodic[1]) continue;
        double2 p, vp;
        double up;
        predict(S, pred, A.pos[i], A.vel[i], A.acc[i], A.u[i], A.udot[i], A.vp[i], A.up[i], p, vp, up);
        SimDev &W = c.sims_rw[s];
        if (!S.periodic[0]) { atomicMin(&W.bbox[0], dkey(p.x)); atomicMax(&W.bbox[1], dkey(p.x)); }
        if (!S.periodic[1]) { atomicMin(&W.bbox[2], dkey(p.y)); atomicMax(&W.bbox[3], dkey(p.y)); }
    }
}

void launch_bbox(const Ctx &c, const Launch &L, const PArrays &A, int pred) {
    k_bbox<<<L.sms * 4, 256, 0, L.stream>>>(c, A, pred);
}

// Grid of open axes from the bounding box (one thread per sim).
__global__ void k_grid(Ctx c) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= c.nsims) return;
    SimDev &S = c.sims_rw[s];
    int G = 1 << S.level;
    for (int ax = 0; ax < 2; ax++) {
        if (S.periodic[ax]) continue;
        double mn = dkey_inv(S.bbox[2 * ax]), mx = dkey_inv(S.bbox[2 * ax + 1]);
        if (!(mn <= mx)) { mn = 0; mx = 1; }
        double w = mx - mn;
        if (!(w > 0)) w = 1e-300 + fabs(mn) * 1e-12 + 1e-12;
        double L = w * (1.0 + 1e-9) + 1e-300;
        S.lo[ax] = mn;
        S.L[ax] = L;
        S.s[ax] = L / G;
        S.inv_s[ax] = G / L;
    }
    double Lm = fmax(S.L[0], S.L[1]);
    S.tol = (float)(Lm * 4.0e-7);
    simdev_floats(S);
}

void launch_grid(const Ctx &c, const Launch &L) {
    k_grid<<<(c.nsims + 127) / 128, 128, 0, L.stream>>>(c);
}

// ------------------------------------------------------------------- bin
__global__ void k_bin(Ctx c, PArrays A, Tables T, int pred) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < c.n;
         i += (int64_t)gridDim.x * blockDim.x) {
        int s = sim_of(c, i);
        const SimDev &S = c.sims[s];
        // The cell of the drifted position, in cell units: the offset from the
        // grid origin in FP64, rounded once to FP32 (error <= 2^-24 G cells,
        // 6e-8 L), plus the drift vel * dth in FP32. The exact FP64 drift is
        // k_permute's; a particle within that error of a cell face may land in
        // the neighbouring cell, which the searches' slack S.tol (4e-7 L)
        // covers. The FP64 pipe is the binning's bound: this is 4 FP64
        // operations per axis instead of about 15.
        const double2 pos = A.pos[i];
        float tx = __double2float_rn(__dmul_rn(__dsub_rn(pos.x, S.lo[0]), S.inv_s[0]));
        float ty = __double2float_rn(__dmul_rn(__dsub_rn(pos.y, S.lo[1]), S.inv_s[1]));
        if (pred == PRED_DRIFT) {
            const double2 vel = A.vel[i];
            tx = __fmaf_rn(__double2float_rn(vel.x), S.fdtc[0], tx);
            ty = __fmaf_rn(__double2float_rn(vel.y), S.fdtc[1], ty);
        }
        if (!isfinite(tx) || !isfinite(ty)) atomicOr(c.flags, (unsigned)FLAG_NONFINITE);
        const int G = 1 << S.level;
        const float Gf = (float)G;
        const int cx = !(tx >= 0.f) ? 0 : tx >= Gf ? G - 1 : (int)tx;
        const int cy = !(ty >= 0.f) ? 0 : ty >= Gf ? G - 1 : (int)ty;
        // distance outside the periodic domain (the wrap moves at most one axis per step)
        float o = 0.f;
        if (S.periodic[0]) o = fmaxf(o, fmaxf(-tx, tx - Gf) * S.fs[0]);
        if (S.periodic[1]) o = fmaxf(o, fmaxf(-ty, ty - Gf) * S.fs[1]);
        if (o > 0.f) atomicMax((int *)&c.sims_rw[s].overshoot, __float_as_int(o * 1.0001f));
        int32_t key = (int32_t)(S.cell_off + morton2(cx, cy));
        T.key[i] = key;
        T.rank[i] = atomicAdd(&T.count[key], 1);
    }
}

void launch_bin(const Ctx &c, const Launch &L, const PArrays &A, const Tables &T, int pred) {
    k_bin<<<L.sms * 8, 256, 0, L.stream>>>(c, A, T, pred);
}

// ------------------------------------------------------------------ scan
// Exclusive scan of the cell counts into cell starts (three passes over
// tiles of kScanTile cells). The counts are zeroed per particle afterwards
// (k_group), so the passes over the whole cell table only read counts and
// write starts.
constexpr int kScanThreads = 512;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ int block_exclusive_scan(int v, int *warp_sums, int &total) {
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[w] = x;
    __syncthreads();
    if (w == 0) {
        int nw = blockDim.x >> 5;
        int t = lane < nw ? warp_sums[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        if (lane < nw) warp_sums[lane] = t;
    }
    __syncthreads();
    total = warp_sums[(blockDim.x >> 5) - 1];
    int before = w > 0 ? warp_sums[w - 1] : 0;
    int r = before + x - v;
    __syncthreads();
    return r;
}

// A thread's eight consecutive cells (32-byte aligned) as two 16-byte loads;
// cells past the end read as empty.
__device__ __forceinline__ void load_counts(const Tables &T, int64_t base, int (&v)[kScanItems]) {
    if (base + kScanItems <= T.ncells) {
        const int4 a = *reinterpret_cast<const int4 *>(T.count + base);
        const int4 b = *reinterpret_cast<const int4 *>(T.count + base + 4);
        v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
        v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
    } else {
#pragma unroll
        for (int j = 0; j < kScanItems; j++) v[j] = base + j < T.ncells ? T.count[base + j] : 0;
    }
}

__global__ void k_scan_tiles(Tables T) {
    __shared__ int ws[32];
    int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
    int v[kScanItems];
    load_counts(T, base, v);
    int sum = 0;
#pragma unroll
    for (int j = 0; j < kScanItems; j++) sum += v[j];
    int total;
    block_exclusive_scan(sum, ws, total);
    if (threadIdx.x == 0) T.partial[blockIdx.x] = total;
}

__global__ void k_scan_partials(Tables T, int ntiles) {
    __shared__ int ws[32];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int b = 0; b < ntiles; b += blockDim.x) {
        int idx = b + threadIdx.x;
        int v = idx < ntiles ? T.partial[idx] : 0;
        int total;
        int ex = block_exclusive_scan(v, ws, total);
        if (idx < ntiles) T.partial[idx] = ex + carry;
        __syncthreads();
        if (threadIdx.x == 0) carry += total;
        __syncthreads();
    }
    if (threadIdx.x == 0) T.start[T.ncells] = carry;
}

__global__ void k_scan_final(Tables T) {
    __shared__ int ws[32];
    int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
    int v[kScanItems];
    load_counts(T, base, v);
    int sum = 0;
#pragma unroll
    for (int j = 0; j < kScanItems; j++) sum += v[j];
    int total;
    int ex = block_exclusive_scan(sum, ws, total) + T.partial[blockIdx.x];
    int st[kScanItems];
#pragma unroll
    for (int j = 0; j < kScanItems; j++) {
        st[j] = ex;
        ex += v[j];
    }
    if (base + kScanItems <= T.ncells) {
        *reinterpret_cast<int4 *>(T.start + base) = make_int4(st[0], st[1], st[2], st[3]);
        *reinterpret_cast<int4 *>(T.start + base + 4) = make_int4(st[4], st[5], st[6], st[7]);
    } else {
#pragma unroll
        for (int j = 0; j < kScanItems; j++)
            if (base + j < T.ncells) T.start[base + j] = st[j];
    }
}

void launch_scan(const Ctx &, const Launch &L, const Tables &T) {
    int ntiles = (int)((T.ncells + kScanTile - 1) / kScanTile);
    k_scan_tiles<<<ntiles, kScanThreads, 0, L.stream>>>(T);
    k_scan_partials<<<1, 1024, 0, L.stream>>>(T, ntiles);
    k_scan_final<<<ntiles, kScanThreads, 0, L.stream>>>(T);
}

// ---------------------------------------------------------- stable order
// The histogram's atomic ranks order a cell's particles arbitrarily. To make
// every later order (and so every floating-point sum) reproducible, each
// particle's slot inside its cell is its rank by index in the previous order
// among the cell's members: the members are grouped by cell (k_group, which
// also zeroes the touched counts for the next binning), then every particle
// counts the members of its cell with a smaller index (k_rank). Both passes
// are per particle, so their cost does not grow with the cell table (the
// k = 64 stress workload bins into 4^14 mostly empty cells).
__global__ void k_group(Ctx c, Tables T) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < c.n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t key = T.key[i];
        T.tmp[T.start[key] + T.rank[i]] = (int32_t)i;
        T.count[key] = 0;
    }
}

__global__ void k_rank(Ctx c, Tables T) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < c.n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t key = T.key[i];
        const int a = T.start[key], b = T.start[key + 1];
        int r = a;
        for (int x = a; x < b; x++) r += T.tmp[x] < (int32_t)i ? 1 : 0;
        T.rank[i] = r;
    }
}

void launch_stable(const Ctx &c, const Launch &L, const Tables &T) {
    k_group<<<L.sms * 8, 256, 0, L.stream>>>(c, T);
    k_rank<<<L.sms * 8, 256, 0, L.stream>>>(c, T);
}

// --------------------------------------------------------------- permute
// Writes the predicted state into cell order (B), plus the float-pair
// position record relative to the grid origin used by the FP32 distance
// filter and the mixed-precision sums, and (vel_records) the predicted
// velocity as float pairs.
__global__ void k_permute(Ctx c, PArrays A, PArrays B, Tables T, int pred, int mixed) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < c.n;
         i += (int64_t)gridDim.x * blockDim.x) {
        int s = sim_of(c, i);
        const SimDev &S = c.sims[s];
        const int64_t d = T.rank[i];  // destination slot (stable within the cell)
        double2 pos = A.pos[i], vel = A.vel[i];
        double u = A.u[i];
        double2 p, vp;
        double up;
        predict(S, pred, pos, vel, A.acc[i], u, A.udot[i], A.vp[i], A.up[i], p, vp, up);
        B.pos[d] = p;
        B.vel[d] = vel;
        B.vp[d] = vp;
        B.u[d] = u;
        B.up[d] = up;
        B.id[d] = A.id[i];
        B.hprev[d] = A.hprev[i];
        float4 r;
        split_df(__dsub_rn(p.x, S.lo[0]), r.x, r.z);
        split_df(__dsub_rn(p.y, S.lo[1]), r.y, r.w);
        B.rec[d] = r;
        if (mixed) {
            float4 v;
            split_df(vp.x, v.x, v.z);
            split_df(vp.y, v.y, v.w);
            B.vrec[d] = v;
        }
    }
}

void launch_permute(const Ctx &c, const Launch &L, const PArrays &A, const PArrays &B,
                    const Tables &T, int pred, bool mixed) {
    k_permute<<<L.sms * 8, 256, 0, L.stream>>>(c, A, B, T, pred, mixed ? 1 : 0);
}

}  // namespace sphgpu
