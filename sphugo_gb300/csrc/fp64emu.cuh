// fp64emu.cuh -- binary64 multiplication, addition, subtraction, division
// and square root, rounded to nearest with ties to even (IEEE 754-2019,
// 4.3.1), and the split of a binary64 into a float pair, computed with
// integer instructions (and FP32 seeds and conversions).
//
// GB300 issues two FP64 lanes per SM per clock: one warp-wide FP64
// instruction holds a sub-partition's FP64 unit for about 64 cycles, while
// the same sub-partition can issue one instruction of another kind every
// cycle. The FP64-bound kernels leave about 90 % of the issue slots idle, so
// some of their operations are computed here, on the integer and FP32
// pipes, in parallel with the hardware FP64 instructions. Every result is
// the hardware instruction's, bit for bit (sph_selftest_fp64emu checks each
// against __dmul_rn, __dadd_rn, __dsub_rn, __ddiv_rn, __dsqrt_rn and the
// double -> float conversion).
//
// Method for products and sums (the textbook guard digits and sticky bit,
// e.g. D. Goldberg, "What every computer scientist should know about
// floating-point arithmetic", ACM Computing Surveys 23(1), 1991; quotients
// and square roots are described at their functions):
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
// That instruction sits in a function that is never inlined, behind a
// branch: a fallback the compiler could compute speculatively (and select)
// would occupy the FP64 unit on every call (measured: the emulated product
// then ran no faster than the hardware's).
#pragma once
#include <stdint.h>

namespace sphgpu {

static __device__ __noinline__ double emu_native_mul(double x, double y) { return __dmul_rn(x, y); }
static __device__ __noinline__ double emu_native_add(double x, double y) { return __dadd_rn(x, y); }
static __device__ __noinline__ double emu_native_sub(double x, double y) { return __dsub_rn(x, y); }
static __device__ __noinline__ double emu_native_sqrt(double x) { return __dsqrt_rn(x); }
static __device__ __noinline__ double emu_native_div(double x, double y) { return __ddiv_rn(x, y); }

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
    if (!ok) r = emu_bits(emu_native_mul(x, y));
    return emu_double(r);
}

// RN(1 - x) for x in [1/2, 1], where the difference is exact (Sterbenz):
// 1 - x = (2^53 - m) 2^-53 for the significand m of x in [1/2, 1), shifted to
// put its leading bit at bit 52. Other x take the hardware subtraction.
__device__ __forceinline__ double emu_one_minus(double x) {
    const uint64_t a = emu_bits(x);
    const uint64_t t = (1ull << 53) - ((a & kEmuFrac) | kEmuHidden);  // in (0, 2^52]
    const int lz = __clzll((long long)t) - 11;  // 0 .. 52
    uint64_t r = (((uint64_t)(1021 - lz)) << 52) + (t << lz);
    if (a == 0x3FF0000000000000ull) r = 0ull;  // 1 - 1 = +0
    else if ((a >> 52) != 1022ull) r = emu_bits(emu_native_sub(1.0, x));
    return emu_double(r);
}

// The float pair of v: hi = RN_float(v) and lo = RN_float(v - hi) (v - hi is
// exact in binary64). hi rounds the 53-bit significand to 24 bits; the
// remainder t = m - hi's significand 2^29 is an integer below 2^29 in
// magnitude, converted by the FP32 integer conversion (one rounding) and
// scaled by 2^(e - 1075) through its exponent field. Operands whose pair
// parts would leave the normal float range take the hardware conversions.
__device__ __forceinline__ void emu_split_df(double v, float &hi, float &lo) {
    const uint64_t a = emu_bits(v);
    const uint32_t ah = (uint32_t)(a >> 32);
    const uint32_t e = (ah >> 20) & 0x7ffu;
    const uint64_t m = (a & kEmuFrac) | kEmuHidden;
    const uint32_t q = (uint32_t)(m >> 29), rem = (uint32_t)m & 0x1fffffffu;
    const uint32_t qh = q + ((rem > 0x10000000u || (rem == 0x10000000u && (q & 1u))) ? 1u : 0u);  // <= 2^24
    // exponent field e - 896 with the hidden bit of qh adding one (a carry to
    // 2^24 adds one more)
    const uint32_t hb = (ah & 0x80000000u) | (((e - 897u) << 23) + qh);
    const int32_t t = (int32_t)((uint32_t)m & 0x1fffffffu) - (int32_t)((qh - q) << 29);  // m - qh 2^29
    const float tf = __int2float_rn((ah & 0x80000000u) ? -t : t);
    const uint32_t lb = __float_as_uint(tf) + ((e - 1075u) << 23);  // tf 2^(e - 1075)
    bool ok = e - 950u < 200u;  // hi and lo (if not zero) normal floats
    hi = __uint_as_float(hb);
    lo = t == 0 ? 0.f : __uint_as_float(lb);
    if (!ok) {
        hi = __double2float_rn(v);
        lo = __double2float_rn(emu_native_sub(v, (double)hi));
    }
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
    if (!ok) r = emu_bits(SUB ? emu_native_sub(x, y) : emu_native_add(x, y));
    return emu_double(r);
}

// S^2 for S < 2^54 as two 64-bit words
__device__ __forceinline__ void emu_sq_wide(uint64_t S, uint64_t &hi, uint64_t &lo) {
    const uint32_t sh = (uint32_t)(S >> 32), sl = (uint32_t)S;
    const uint64_t ll = (uint64_t)sl * sl, mid = ((uint64_t)sl * sh) << 1, hh = (uint64_t)sh * sh;
    lo = ll + (mid << 32);
    hi = hh + (mid >> 32) + (lo < ll ? 1ull : 0ull);
}

// RN(sqrt(x)). With x = M0 2^p (M0 the significand, shifted left once when
// p is odd) the result's significand is RN(sqrt(M)) for the integer
// M = M0 2^52 in [2^104, 2^106): S0 from the FP32 reciprocal square root
// y0 ~ 1/sqrt(M0 2^-52) (about 21 good bits), two Newton corrections
// S += (M - S^2) y0 / (2 sqrt(M)) evaluated on 32-bit windows of the exact
// 128-bit residual (the error falls from ~2^32 to ~2^12 to below 0.51), then
// the exact remainder r = M - S^2 makes S the floor (0 <= r <= 2S) and
// decides the rounding: up iff r > S (sqrt(M) > S + 1/2; never a tie for an
// integer M). The method is Newton's iteration for the square root with an
// exact integer remainder test, e.g. R. Brent and P. Zimmermann, "Modern
// Computer Arithmetic", 2010, section 1.5.1.
__device__ __forceinline__ double emu_sqrt(double x) {
    const uint64_t a = emu_bits(x);
    const uint32_t ah = (uint32_t)(a >> 32);
    const uint32_t e = ah >> 20;  // with the sign bit: > 2046 for negative x
    const uint32_t odd = ~e & 1u;  // the unbiased exponent e - 1075 is odd
    const uint64_t M0 = ((a & kEmuFrac) | kEmuHidden) << odd;  // [2^52, 2^54)
    const uint64_t Mhi = M0 >> 12, Mlo = M0 << 52;  // M = M0 2^52
    const float uf = __uint2float_rn((uint32_t)(M0 >> 30)) * 0x1p-22f;  // M0 2^-52 in [1, 4), 24 bits
    const float y0 = rsqrtf(uf);
    uint64_t S = (uint64_t)__float2uint_rn(uf * y0 * 0x1p23f) << 29;  // ~ sqrt(M)
    uint64_t hi, lo;
    // first correction: |M - S^2| < 2^86, read as bits 56 .. 87
    emu_sq_wide(S, hi, lo);
    {
        const uint64_t rlo = Mlo - lo, rhi = Mhi - hi - (Mlo < lo ? 1ull : 0ull);
        const int32_t w = (int32_t)__funnelshift_r((uint32_t)(rlo >> 32), (uint32_t)rhi, 24);
        // S += r y0 / 2^53 = w y0 2^3, rounded in units of 2^8
        S += (uint64_t)((int64_t)__float2int_rn((float)w * y0 * 0x1p-5f) * 256);
    }
    // second correction: |M - S^2| < 2^66, read as bits 36 .. 67
    emu_sq_wide(S, hi, lo);
    {
        const uint64_t rlo = Mlo - lo, rhi = Mhi - hi - (Mlo < lo ? 1ull : 0ull);
        const int32_t w = (int32_t)__funnelshift_r((uint32_t)(rlo >> 32), (uint32_t)rhi, 4);
        S += (uint64_t)(int64_t)__float2int_rn((float)w * y0 * 0x1p-17f);
    }
    // the exact remainder (|r| < 2^56: the low word suffices), floor, rounding
    int64_t r = (int64_t)(Mlo - S * S);
    if (r < 0) {
        S -= 1ull;
        r += (int64_t)(2ull * S + 1ull);
    }
    if (r > (int64_t)(2ull * S)) {
        r -= (int64_t)(2ull * S + 1ull);
        S += 1ull;
    }
    const uint64_t Sr = S + (r > (int64_t)S ? 1ull : 0ull);  // [2^52, 2^53]
    const int32_t er = ((int32_t)e - 1023 - (int32_t)odd) / 2 + 1023;  // exponent field of the result
    uint64_t res = ((uint64_t)(uint32_t)(er - 1) << 52) + Sr;
    const bool ok = e - 1u < 0x7feu;  // positive and normal
    if (!ok) res = emu_bits(emu_native_sqrt(x));
    return emu_double(res);
}

// A divisor b prepared for several quotients: its significand mb and
// inv ~ 2^115 / mb to within a few units (FP32 seed, two Newton corrections
// inv += inv (2^115 - mb inv) / 2^115 on 32-bit windows of the exact
// residual; the relative error falls from ~2^-21 to ~2^-42 to ~2^-61).
struct EmuDivisor {
    uint64_t mb, inv;
    uint32_t bh;  // high word of b: sign and exponent
};

__device__ __forceinline__ EmuDivisor emu_divisor(double b) {
    const uint64_t bb = emu_bits(b);
    EmuDivisor D;
    D.bh = (uint32_t)(bb >> 32);
    D.mb = (bb & kEmuFrac) | kEmuHidden;
    const float rf = __frcp_rn(__uint2float_rn((uint32_t)(D.mb >> 29)));  // ~ 2^29 / mb
    uint64_t inv = (uint64_t)__float2uint_rn(rf * 0x1p46f) << 40;  // ~ 2^115 / mb
    uint64_t hi = __umul64hi(D.mb, inv), lo = D.mb * inv;
    {
        // E = 2^115 - mb inv, |E| < 2^95: bits 64 .. 95; inv += inv E / 2^115
        // = w rf 2^35, rounded in units of 2^16
        const int32_t w = (int32_t)((1ull << 51) - hi - (lo != 0ull ? 1ull : 0ull));
        inv += (uint64_t)((int64_t)__float2int_rn((float)w * rf * 0x1p19f) * 65536);
    }
    hi = __umul64hi(D.mb, inv);
    lo = D.mb * inv;
    {
        // |E| < 2^75: bits 44 .. 75; inv += w rf 2^15
        const uint64_t elo = 0ull - lo, ehi = (1ull << 51) - hi - (lo != 0ull ? 1ull : 0ull);
        const int32_t w = (int32_t)__funnelshift_r((uint32_t)(elo >> 32), (uint32_t)ehi, 12);
        inv += (uint64_t)(int64_t)__float2int_rn((float)w * rf * 0x1p15f);
    }
    D.inv = inv;
    return D;
}

// RN(x / y) with D = emu_divisor(y). The significand quotient
// Q = floor(ma 2^(52+s) / mb) (s = 1 when ma < mb, so Q is in [2^52, 2^53))
// comes from ma inv to within one unit; the exact remainder
// R = ma 2^(52+s) - Q mb makes Q the floor (0 <= R < mb) and rounds: up iff
// 2R > mb (a quotient of two 53-bit significands is never a midpoint).
// Long division by a scaled reciprocal with remainder correction, e.g.
// R. Brent and P. Zimmermann, "Modern Computer Arithmetic", 2010, 1.4.1.
__device__ __forceinline__ double emu_div(double x, const EmuDivisor &D, double y) {
    const uint64_t a = emu_bits(x);
    const uint32_t ah = (uint32_t)(a >> 32);
    const uint32_t ea = (ah >> 20) & 0x7ffu, eb = (D.bh >> 20) & 0x7ffu;
    const uint64_t ma = (a & kEmuFrac) | kEmuHidden;
    const uint32_t s = ma < D.mb ? 1u : 0u;
    uint64_t Q = __umul64hi(ma << 11, D.inv) >> (10u - s);
    int64_t R = (int64_t)((ma << (52u + s)) - Q * D.mb);
    if (R < 0) {
        Q -= 1ull;
        R += (int64_t)D.mb;
    }
    if (R >= (int64_t)D.mb) {
        Q += 1ull;
        R -= (int64_t)D.mb;
    }
    const uint64_t up = (uint64_t)(2 * R) > D.mb ? 1ull : 0ull;
    const int e = (int)ea - (int)eb + 1023 - (int)s;  // biased exponent before rounding
    const uint64_t sign = (uint64_t)((ah ^ D.bh) & 0x80000000u) << 32;
    uint64_t r = sign | ((((uint64_t)(e - 1)) << 52) + Q + up);
    const bool bn = eb - 1u < 0x7feu;
    bool ok = bn && ea - 1u < 0x7feu && (uint32_t)(e - 1) < 2046u;
    if (bn && (a & ~kEmuSign) == 0ull) {  // +-0 / b
        r = sign;
        ok = true;
    }
    if (!ok) r = emu_bits(emu_native_div(x, y));
    return emu_double(r);
}

__device__ __forceinline__ double emu_add(double x, double y) { return emu_addsub<false>(x, y); }
__device__ __forceinline__ double emu_sub(double x, double y) { return emu_addsub<true>(x, y); }

// Out-of-line copies, one body per translation unit, for kernels whose loops
// would outgrow the instruction cache with every operation inlined (the FP64
// force kernel: inlined, ncu counted 4.5 cycles of "no instruction" stall per
// issued instruction; out of line, the kernel ran 1.3x faster). Kernels with
// short loops (the density) keep the inlined forms.
static __device__ __noinline__ double emu_mul_ol(double x, double y) { return emu_mul(x, y); }
static __device__ __noinline__ double emu_sqrt_ol(double x) { return emu_sqrt(x); }
static __device__ __noinline__ EmuDivisor emu_divisor_ol(double b) { return emu_divisor(b); }
// (the divisor by value: by reference it went through the stack, 5 % of the force's time)
static __device__ __noinline__ double emu_div_ol(double x, EmuDivisor D, double y) { return emu_div(x, D, y); }

}  // namespace sphgpu
