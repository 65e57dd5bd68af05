// physics.cuh -- SPH kernel functions in the three arithmetic forms.
//
// EXACT64 keeps the reference's operation order with every product and sum
// rounded separately (no contraction), so its results equal a -ffp-contract=off
// restatement of sim/sph.go bit for bit. FAST64 lets the compiler contract
// into FMA and replaces per-neighbour divisions by per-particle reciprocals
// (agreement within ~1e-14 relative). The float forms serve the mixed path.
#pragma once

#include "common.cuh"
#include "fp64emu.cuh"

namespace sphgpu {

// RN(a/3) in three FP64 instructions instead of a division. With
// y = RN(1/3) = (1/3)(1 - 2^-54): q0 = RN(a y) is within one ulp of a/3, the
// residual r = a - 3 q0 is a multiple of ulp(a/3) of at most three units and
// so exact in the FMA, and q0 + r y = a/3 - (r/3) 2^-54 differs from a/3 by far
// less than the distance from a/3 to any rounding midpoint (a/3 has a
// fractional part of 0, 1/3 or 2/3 in units of its ulp), so RN(q0 + r y) is
// RN(a/3). Valid for every finite a without underflow in r.
__device__ __forceinline__ double div3_rn(double a) {
    const double y = 0x1.5555555555555p-2;  // RN(1/3)
    const double q0 = emu_mul(a, y);
    const double r = __fma_rn(-3.0, q0, a);
    return __fma_rn(r, y, q0);
}

// RN(a/b) given y = RN(1/b) (shared by many quotients with the same b):
// q1 below is faithful (within one ulp of a/b), the residual a - b q1 is exact
// in the FMA, and Markstein's theorem (y within half an ulp of 1/b, q1
// faithful) makes RN(q1 + r1 y) the correctly rounded quotient. No
// overflow/underflow for the operands used here (distances and their ratios).
__device__ __forceinline__ double div_rn_recip(double a, double b, double y) {
    const double q0 = emu_mul(a, y);
    const double r0 = __fma_rn(-b, q0, a);
    const double q1 = __fma_rn(r0, y, q0);
    const double r1 = __fma_rn(-b, q1, a);
    return __fma_rn(r1, y, q1);
}

// sim/sph.go:258-276 Monahan2D and :284-304 Wendtland2D, reference rounding.
__device__ __forceinline__ double kf_exact(int kernel, double q) {
    if (kernel == SPH_KERNEL_WENDLAND) {
        double a = __dsub_rn(1.0, q);
        double t = __dmul_rn(__dmul_rn(__dmul_rn(a, a), a), a);
        return __dmul_rn(t, __dadd_rn(1.0, __dmul_rn(4.0, q)));
    }
    if (q < 0.5) {
        double qq = __dmul_rn(q, q);
        return __dadd_rn(__dsub_rn(__dmul_rn(qq, q), qq), 1.0 / 6.0);
    }
    double a = __dsub_rn(1.0, q);
    return div3_rn(__dmul_rn(__dmul_rn(a, a), a));
}
__device__ __forceinline__ double kdf_exact(int kernel, double q) {
    if (kernel == SPH_KERNEL_WENDLAND) {
        double a = __dsub_rn(1.0, q);
        return __dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(-10.0, q), a), a), a);
    }
    if (q < 0.5) return __dsub_rn(__dmul_rn(__dmul_rn(3.0, q), q), __dmul_rn(2.0, q));
    double a = __dsub_rn(1.0, q);
    return __dmul_rn(-a, a);
}

// contractible FP64 forms
__device__ __forceinline__ double kf_fast(int kernel, double q) {
    if (kernel == SPH_KERNEL_WENDLAND) {
        double a = 1.0 - q, a2 = a * a;
        return a2 * a2 * (1.0 + 4.0 * q);
    }
    if (q < 0.5) return (q - 1.0) * q * q + (1.0 / 6.0);
    double a = 1.0 - q;
    return a * a * a * (1.0 / 3.0);
}
__device__ __forceinline__ double kdf_fast(int kernel, double q) {
    if (kernel == SPH_KERNEL_WENDLAND) {
        double a = 1.0 - q;
        return -10.0 * q * a * a * a;
    }
    if (q < 0.5) return (3.0 * q - 2.0) * q;
    double a = 1.0 - q;
    return -(a * a);
}

// FP32 forms (mixed path)
__device__ __forceinline__ float kf_f32(int kernel, float q) {
    if (kernel == SPH_KERNEL_WENDLAND) {
        float a = 1.f - q, a2 = a * a;
        return a2 * a2 * (1.f + 4.f * q);
    }
    if (q < 0.5f) return (q - 1.f) * q * q + (1.f / 6.f);
    float a = 1.f - q;
    return a * a * a * (1.f / 3.f);
}
__device__ __forceinline__ float kdf_f32(int kernel, float q) {
    if (kernel == SPH_KERNEL_WENDLAND) {
        float a = 1.f - q;
        return -10.f * q * a * a * a;
    }
    if (q < 0.5f) return (3.f * q - 2.f) * q;
    float a = 1.f - q;
    return -(a * a);
}

// Calls f(e, code) for the neighbour list entries e = k-1 down to 0 (the
// reference's farthest-first order), reading four codes per load when k is a
// multiple of four (lists are 16-byte aligned then).
template <typename F>
__device__ __forceinline__ void for_each_nbr_desc(const int32_t *nb, int k, F f) {
    if ((k & 3) == 0) {
        const int4 *nb4 = reinterpret_cast<const int4 *>(nb);
        for (int b = (k >> 2) - 1; b >= 0; b--) {
            const int4 c = nb4[b];
            f(4 * b + 3, (uint32_t)c.w);
            f(4 * b + 2, (uint32_t)c.z);
            f(4 * b + 1, (uint32_t)c.y);
            f(4 * b, (uint32_t)c.x);
        }
    } else {
        for (int e = k - 1; e >= 0; e--) f(e, (uint32_t)nb[e]);
    }
}

// entries hi-1 down to lo of a list of k entries (16-byte loads when k, and
// with it every bound used here, is a multiple of four)
template <typename F>
__device__ __forceinline__ void for_each_nbr_desc_range(const int32_t *nb, int lo, int hi, int k, F f) {
    if ((k & 3) == 0) {
        const int4 *nb4 = reinterpret_cast<const int4 *>(nb);
        for (int b = (hi >> 2) - 1; b >= (lo >> 2); b--) {
            const int4 c = nb4[b];
            f(4 * b + 3, (uint32_t)c.w);
            f(4 * b + 2, (uint32_t)c.z);
            f(4 * b + 1, (uint32_t)c.y);
            f(4 * b, (uint32_t)c.x);
        }
    } else {
        for (int e = hi - 1; e >= lo; e--) f(e, (uint32_t)nb[e]);
    }
}

// r_AB = (q - offset) - p from the float-pair records of the neighbour (r)
// and the particle (pr), image code img (4 = no shift): the high parts'
// difference is exact by Sterbenz for neighbours within a period, so the
// result carries only the rounding of the low parts (about 2^-48 of the
// coordinates) and of the final sum.
__device__ __forceinline__ void float_pair_rel(const SimDev &S, float4 pr, float4 r, uint32_t img, float &rabx,
                                               float &raby) {
    if (img == 4u) {
        rabx = (r.x - pr.x) + (r.z - pr.z);
        raby = (r.y - pr.y) + (r.w - pr.w);
    } else {
        const float dXh = S.fimg_h[0], dXl = S.fimg_l[0], dYh = S.fimg_h[1], dYl = S.fimg_l[1];
        const int ia = (int)(img / 3u) - 1, ib = (int)(img % 3u) - 1;
        rabx = ((r.x - (ia > 0 ? dXh : 0.f)) - (ia < 0 ? pr.x - dXh : pr.x)) +
               (r.z - (pr.z + (ia > 0 ? dXl : ia < 0 ? -dXl : 0.f)));
        raby = ((r.y - (ib > 0 ? dYh : 0.f)) - (ib < 0 ? pr.y - dYh : pr.y)) +
               (r.w - (pr.w + (ib > 0 ? dYl : ib < 0 ? -dYl : 0.f)));
    }
}

// Kahan-compensated FP32 accumulator
struct KahanF {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float v) {
        float y = v - c;
        float t = s + y;
        c = (t - s) - y;
        s = t;
    }
    __device__ __forceinline__ float value_f() const { return s - c; }
};

// The reference's squared distance of the image-shifted query to a
// candidate: sim/nearest-neighbour.go:72 pos = p.Pos + offset, then
// sim/linear-algebra.go:64-67 DistSq. No contraction.
__device__ __forceinline__ double dist_sq_ref(double px, double py, double ox, double oy,
                                              double qx, double qy) {
    double dx = __dsub_rn(__dadd_rn(px, ox), qx);
    double dy = __dsub_rn(__dadd_rn(py, oy), qy);
    return __dadd_rn(emu_mul(dx, dx), emu_mul(dy, dy));
}

// image code (i+1)*3+(j+1) -> shift (i*dX, j*dY), as float64(i)*deltaX in
// sim/nearest-neighbour.go:59 (i = +-1: the product is exactly +-deltaX)
__device__ __forceinline__ void img_shift(const SimDev &S, uint32_t img, double &ox, double &oy) {
    int ia = (int)(img / 3u) - 1, ib = (int)(img % 3u) - 1;
    ox = ia ? (ia > 0 ? S.dimg[0] : -S.dimg[0]) : 0.0;
    oy = ib ? (ib > 0 ? S.dimg[1] : -S.dimg[1]) : 0.0;
}

}  // namespace sphgpu
