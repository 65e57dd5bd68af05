// physics.cuh -- SPH kernel functions in the three arithmetic forms.
//
// EXACT64 keeps the reference's operation order with every product and sum
// rounded separately (no contraction), so its results equal a -ffp-contract=off
// restatement of sim/sph.go bit for bit. FAST64 lets the compiler contract
// into FMA and replaces per-neighbour divisions by per-particle reciprocals
// (agreement within ~1e-14 relative). The float forms serve the mixed path.
#pragma once

#include "common.cuh"

namespace sphgpu {

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
    return __ddiv_rn(__dmul_rn(__dmul_rn(a, a), a), 3.0);
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

// Kahan-compensated FP32 accumulator
struct KahanF {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float v) {
        float y = v - c;
        float t = s + y;
        c = (t - s) - y;
        s = t;
    }
    __device__ __forceinline__ double value() const { return (double)s - (double)c; }
};

// The reference's squared distance of the image-shifted query to a
// candidate: sim/nearest-neighbour.go:72 pos = p.Pos + offset, then
// sim/linear-algebra.go:64-67 DistSq. No contraction.
__device__ __forceinline__ double dist_sq_ref(double px, double py, double ox, double oy,
                                              double qx, double qy) {
    double dx = __dsub_rn(__dadd_rn(px, ox), qx);
    double dy = __dsub_rn(__dadd_rn(py, oy), qy);
    return __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
}

// image code (i+1)*3+(j+1) -> shift (i*dX, j*dY), as float64(i)*deltaX in
// sim/nearest-neighbour.go:59
__device__ __forceinline__ void img_shift(const SimDev &S, uint32_t img, double &ox, double &oy) {
    int ia = (int)(img / 3u) - 1, ib = (int)(img % 3u) - 1;
    ox = ia ? __dmul_rn((double)ia, S.dimg[0]) : 0.0;
    oy = ib ? __dmul_rn((double)ib, S.dimg[1]) : 0.0;
}

}  // namespace sphgpu
