// fp64emu.cuh -- binary64 multiplication, addition and subtraction, rounded
// to nearest with ties to even (IEEE 754-2019, 4.3.1), computed with integer
// instructions.
//
// GB300 issues two FP64 lanes per SM per clock: one warp-wide FP64
// instruction holds a sub-partition's FP64 unit for about 64 cycles, while
// the same sub-partition can issue one instruction of another kind every
// cycle. The FP64-bound kernels leave about 90 % of the issue slots idle, so
// some of their operations are computed here, on the integer and FP32
// pipes, in parallel with the hardware FP64 instructions. Every result is
// the hardware instruction's, bit for bit (sph_selftest_fp64emu checks this
// against __dmul_rn / __dadd_rn / __dsub_rn).
//
// Method (the textbook guard digits and sticky bit, e.g. D. Goldberg, "What
// every computer scientist should know about floating-point arithmetic",
// ACM Computing Surveys 23(1), 1991):
//   * product: the exact 106-bit product of the two 53-bit significands, its
//     leading 53 bits rounded on the remaining bits (round bit, then "any
//     bit below it" as the sticky);
//   * sum: significands left-aligned with 10 guard bits, the smaller one
//     shifted right by the exponent difference with the shifted-out bits
//     jammed into its lowest bit, added or subtracted exactly, normalised,
//     rounded on the guard bits.
// Operands or results outside the normal range (zeros in a product,
// subnormals, infinities, NaNs, overflow in a sum, underflow) and sums of
// operands more than 63 binades apart take the hardware instruction, so
// those rare cases need no integer code at all.
// That instruction sits behind a branch that the warp takes only when one of
// its active lanes needs it, in a function that is never inlined: a fallback
// the compiler could compute speculatively (and select) would occupy the
// FP64 unit on every call.
#pragma once
#include <stdint.h>

namespace sphgpu {

#ifndef SPH_EMU_FALLBACK
#define SPH_EMU_FALLBACK 1
#endif
#if SPH_EMU_FALLBACK == 1
static __device__ __noinline__ double emu_native_mul(double x, double y) { return __dmul_rn(x, y); }
static __device__ __noinline__ double emu_native_add(double x, double y) { return __dadd_rn(x, y); }
static __device__ __noinline__ double emu_native_sub(double x, double y) { return __dsub_rn(x, y); }
#else
__device__ __forceinline__ double emu_native_mul(double x, double y) {
    double r;
    asm volatile("mul.rn.f64 %0, %1, %2;" : "=d"(r) : "d"(x), "d"(y));
    return r;
}
__device__ __forceinline__ double emu_native_add(double x, double y) {
    double r;
    asm volatile("add.rn.f64 %0, %1, %2;" : "=d"(r) : "d"(x), "d"(y));
    return r;
}
__device__ __forceinline__ double emu_native_sub(double x, double y) {
    double r;
    asm volatile("sub.rn.f64 %0, %1, %2;" : "=d"(r) : "d"(x), "d"(y));
    return r;
}
#endif

constexpr uint64_t kEmuSign = 0x8000000000000000ull;
constexpr uint64_t kEmuFrac = 0x000FFFFFFFFFFFFFull;
constexpr uint64_t kEmuHidden = 0x0010000000000000ull;

__device__ __forceinline__ uint64_t emu_bits(double x) { return (uint64_t)__double_as_longlong(x); }
__device__ __forceinline__ double emu_double(uint64_t b) { return __longlong_as_double((long long)b); }

// RN(x y), on 32-bit words: the 106-bit product of the significands from
// four 32 x 32 -> 64-bit products, its leading 53 bits taken by funnel shifts
__device__ __forceinline__ double emu_mul(double x, double y) {
    const uint64_t a = emu_bits(x), b = emu_bits(y);
    const uint32_t ah = (uint32_t)(a >> 32), al = (uint32_t)a, bh = (uint32_t)(b >> 32), bl = (uint32_t)b;
    const uint32_t ea = (ah >> 20) & 0x7ffu, eb = (bh >> 20) & 0x7ffu;
    const uint32_t mah = (ah & 0xfffffu) | 0x100000u, mbh = (bh & 0xfffffu) | 0x100000u;
    const uint64_t t0 = (uint64_t)al * bl, t1 = (uint64_t)mah * bl, t2 = (uint64_t)al * mbh;
    const uint64_t t3 = (uint64_t)mah * mbh;  // < 2^42
    const uint64_t mid = t1 + t2 + (t0 >> 32);  // < 2^55
    const uint64_t upper = t3 + (mid >> 32);  // P = upper 2^64 + (uint32)mid 2^32 + (uint32)t0
    const uint32_t w0 = (uint32_t)t0, w1 = (uint32_t)mid, w2 = (uint32_t)upper, w3 = (uint32_t)(upper >> 32);
    const uint32_t top = (w3 >> 9) & 1u;  // P >= 2^105: the significand is P >> 53, else P >> 52
    const uint32_t sh = 20u + top;
    const uint32_t mlo = __funnelshift_r(w1, w2, sh), mhi = __funnelshift_r(w2, w3, sh);
    const uint32_t rb = (w1 >> (sh - 1u)) & 1u;  // the round bit; below it the sticky bits
    const uint32_t sticky = (w1 & ((1u << (sh - 1u)) - 1u)) | w0;
    const uint32_t up = rb & ((sticky != 0u ? 1u : 0u) | (mlo & 1u));
    const int e = (int)(ea + eb) - 1023 + (int)top;  // biased exponent before rounding
    // (e - 1) << 20 plus the significand's hidden bit gives exponent field e;
    // a rounding carry moves it to e + 1 (2047: the correctly rounded infinity)
    const uint32_t rhi = ((ah ^ bh) & 0x80000000u) | (((uint32_t)(e - 1) << 20) + mhi);
    uint64_t r = (((uint64_t)rhi << 32) | mlo) + up;
    const bool ok = ea - 1u < 0x7feu && eb - 1u < 0x7feu && (uint32_t)(e - 1) < 2046u;
    if (__any_sync(__activemask(), !ok)) {
        if (!ok) r = emu_bits(emu_native_mul(x, y));
    }
    return emu_double(r);
}

// RN(x + y) (SUB = false) or RN(x - y) (SUB = true). The smaller operand's
// significand is shifted right by the exponent difference with the lost bits
// jammed into bit 0; after the exact sum or difference, one more jammed right
// shift (which absorbs a carry out) and a left shift by the leading zeros
// bring the leading bit to 62, leaving 10 guard bits. A jammed bit always
// sits at or below bit 2 there, so it never decides a rounding on its own.
template <bool SUB>
__device__ __forceinline__ double emu_addsub(double x, double y) {
    const uint64_t a = emu_bits(x), b = emu_bits(y) ^ (SUB ? kEmuSign : 0ull);
    const bool sw = (a & ~kEmuSign) < (b & ~kEmuSign);  // order by magnitude
    const uint64_t big = sw ? b : a, small = sw ? a : b;
    const uint32_t gh = (uint32_t)(big >> 32), gl = (uint32_t)big;
    const uint32_t sh = (uint32_t)(small >> 32), sl = (uint32_t)small;
    const uint32_t ea = (gh >> 20) & 0x7ffu, eb = (sh >> 20) & 0x7ffu;
    const uint32_t d = ea - eb;  // >= 0 when both are normal
    // significands with the hidden bit at bit 62
    const uint64_t ma = ((uint64_t)((gh & 0xfffffu) | 0x100000u) << 42) | ((uint64_t)gl << 10);
    const uint64_t mb = ((uint64_t)((sh & 0xfffffu) | 0x100000u) << 42) | ((uint64_t)sl << 10);
    const uint32_t dc = d < 63u ? d : 63u;
    const uint64_t mt = mb >> dc;
    const uint64_t mbs = mt | ((mt << dc) != mb ? 1ull : 0ull);
    const bool same = ((gh ^ sh) & 0x80000000u) == 0u;
    const uint64_t s = same ? ma + mbs : ma - mbs;  // exact; >= 0 (big >= small)
    const uint64_t t0 = (s >> 1) | (s & 1ull);
    const int lz = __clzll((long long)t0) - 1;  // 0 .. 63
    const uint64_t t = t0 << lz;
    const int e = (int)ea + 1 - lz;  // biased exponent before rounding
    const uint32_t th = (uint32_t)(t >> 32), tl = (uint32_t)t;
    const uint32_t mhi = th >> 10, mlo = __funnelshift_r(tl, th, 10);
    const uint32_t rest = tl & 0x3ffu;
    const uint32_t up = (rest > 0x200u || (rest == 0x200u && (mlo & 1u))) ? 1u : 0u;
    const uint32_t rhi = (gh & 0x80000000u) | (((uint32_t)(e - 1) << 20) + mhi);
    uint64_t r = (((uint64_t)rhi << 32) | mlo) + up;
    const bool zero = s == 0ull;  // exact cancellation: +0
    r = zero ? 0ull : r;
    const bool bign = ea - 1u < 0x7feu;
    bool ok = bign && eb - 1u < 0x7feu && d < 64u && (zero || (uint32_t)(e - 1) < 2046u);
    if (bign && (small & ~kEmuSign) == 0ull) {  // big + 0 = big for a normal big
        r = big;
        ok = true;
    }
    if (__any_sync(__activemask(), !ok)) {
        if (!ok) r = emu_bits(SUB ? emu_native_sub(x, y) : emu_native_add(x, y));
    }
    return emu_double(r);
}

__device__ __forceinline__ double emu_add(double x, double y) { return emu_addsub<false>(x, y); }
__device__ __forceinline__ double emu_sub(double x, double y) { return emu_addsub<true>(x, y); }

}  // namespace sphgpu
