// knn_shared.cuh -- pieces shared by the neighbour-search kernels: their
// arguments, the FP32 error bound's constants, the key packing and the
// in-register sorting network.
#pragma once

#include "physics.cuh"

namespace sphgpu {

struct KnnArgs {
    Ctx c;
    PArrays B;
    Derived D;
    const int32_t *start;
    float theta, hgrow;
    int use_defer;  // per-query kernel / density: walk the deferred list instead of every particle
    int fuse_density;  // mixed block tiles: each settled query's density computed with its list
    int rerank;  // FP64 forms, block tiles: a decided set whose order needs FP64 goes to the re-rank list
};

// |d2_f32 - d2_ref| <= kEpsRel * d2 + eps_abs(R): the float-pair difference
// carries ~2^-23 relative error, the two float products ~2^-24 each, and the
// reference's own rounding of (p + offset) adds ~2^-53 L absolute per axis.
constexpr float kEpsRel = 9.5367431640625e-7f;  // 2^-20 (about 8x the bound)

__device__ __forceinline__ float eps_of(float d2, float abs_term) { return kEpsRel * d2 + abs_term; }

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Batcher's odd-even merge sort (K. E. Batcher, "Sorting networks and their
// applications", 1968) of NS keys in registers, ascending: the network for the
// next power of two with every comparator that touches a position >= NS left
// out (those positions would hold +infinity and never move).
template <int NS>
struct OddEvenSort {
    uint32_t (&v)[NS];
    __device__ __forceinline__ void ce(int i, int j) {
        if (j < NS) {
            const uint32_t lo = min(v[i], v[j]);
            v[j] = max(v[i], v[j]);
            v[i] = lo;
        }
    }
    template <int LO, int N, int R>
    __device__ __forceinline__ void merge() {
        constexpr int M = 2 * R;
        if constexpr (M < N) {
            merge<LO, N, M>();
            merge<LO + R, N, M>();
#pragma unroll
            for (int i = LO + R; i + R < LO + N; i += M) ce(i, i + R);
        } else {
            ce(LO, LO + R);
        }
    }
    template <int LO, int N>
    __device__ __forceinline__ void sort() {
        if constexpr (N > 1 && LO < NS) {
            sort<LO, N / 2>();
            sort<LO + N / 2, N / 2>();
            merge<LO, N, 1>();
        }
    }
    __device__ __forceinline__ void run() {
        constexpr int P2 = NS <= 32 ? 32 : NS <= 64 ? 64 : 128;
        sort<0, P2>();
    }
};

// d2 in units of R^2 / 2^23 rounded to the nearest integer, clamped to 23
// bits, without a conversion instruction: for 0 <= d2 qs < 2^23 the FMA
// d2 qs + 2^23 lands in [2^23, 2^24), where the float's mantissa is the
// integer itself.
__device__ __forceinline__ uint32_t key23(float d2, float qs) {
    return min(__float_as_uint(__fmaf_rn(d2, qs, 8388608.f)) - 0x4B000000u, 8388607u);
}

__device__ __forceinline__ void defer_lanes(const KnnArgs &a, bool mine, int64_t q, int lane) {
    const uint32_t bal = __ballot_sync(0xffffffffu, mine);
    if (!bal) return;
    int base = 0;
    if (lane == 0) base = atomicAdd(a.D.ndefer, __popc(bal));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (mine) a.D.defer[base + __popc(bal & lanemask_lt())] = (int32_t)q;
}

// appends the lanes' queries to the re-rank list, stored from the end of the
// deferred-query array (a query is in at most one of the two lists), counted
// in ndefer[1]
__device__ __forceinline__ void rerank_lanes(const KnnArgs &a, bool mine, int64_t q, int lane) {
    const uint32_t bal = __ballot_sync(0xffffffffu, mine);
    if (!bal) return;
    int base = 0;
    if (lane == 0) base = atomicAdd(a.D.ndefer + 1, __popc(bal));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (mine) a.D.defer[a.c.n - 1 - (base + __popc(bal & lanemask_lt()))] = (int32_t)q;
}

// the reference's squared distance to the neighbour image a list code names
__device__ __forceinline__ double nbr_d2(const SimDev &S, const PArrays &B, double2 P, uint32_t code) {
    const double2 Q = B.pos[code >> kCodeShift];
    if ((code & 15u) == 4u) {
        // no offset: p + 0 = p (and -0 + 0 = +0 squares to the same value)
        const double dx = __dsub_rn(P.x, Q.x), dy = __dsub_rn(P.y, Q.y);
        return __dadd_rn(emu_mul(dx, dx), emu_mul(dy, dy));
    }
    double ox, oy;
    img_shift(S, code & 15u, ox, oy);
    return dist_sq_ref(P.x, P.y, ox, oy, Q.x, Q.y);
}

// block-tile search (k_knn_block.cu): false when no block kernel serves the
// list shape nr (the warp tiles do then)
bool launch_knn_block(const KnnArgs &args, const Launch &L, int mode, int nr, int warps);
// whether the block tiles compute the mixed form's densities of the queries
// they settle (the density pass then covers only the deferred queries)
bool knn_fuses_density(int k, int mode, const KnnTune &tune);
void knn_block_init_attrs();

}  // namespace sphgpu
