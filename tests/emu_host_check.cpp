// emu_host_check.cpp -- compiles the library's integer-pipe binary64
// operations (sphugo_gb300/csrc/fp64emu.cuh) for the host, with the CUDA
// intrinsics they call restated in portable C++, and compares every result
// with the host's IEEE arithmetic (round to nearest, no contraction) on seeded
// operands of the same classes as the device self-check. The FP32 seeds
// differ from the device's (here 1/sqrtf and 1/x, correctly rounded; on the
// device rsqrtf has up to 2 ulp of error), so this also checks that the
// Newton corrections do not depend on the seed's last bits.
//
//   g++ -O2 -std=c++17 -ffp-contract=off tests/emu_host_check.cpp -o check && ./check [n]
//
// Prints the number of differing results per operation; exit status 0 when
// every result matches.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>

// ---- the CUDA qualifiers and intrinsics used by fp64emu.cuh, for the host
#define __device__
#define __forceinline__ inline
#define __noinline__ __attribute__((noinline))

static inline long long __double_as_longlong(double d) {
    long long r;
    std::memcpy(&r, &d, 8);
    return r;
}
static inline double __longlong_as_double(long long x) {
    double d;
    std::memcpy(&d, &x, 8);
    return d;
}
static inline unsigned __float_as_uint(float f) {
    unsigned r;
    std::memcpy(&r, &f, 4);
    return r;
}
static inline float __uint_as_float(unsigned u) {
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}
static inline unsigned long long __umul64hi(unsigned long long a, unsigned long long b) {
    return (unsigned long long)(((unsigned __int128)a * b) >> 64);
}
// (hi:lo) >> (s mod 32), the low 32 bits
static inline unsigned __funnelshift_r(unsigned lo, unsigned hi, unsigned s) {
    const uint64_t v = ((uint64_t)hi << 32) | lo;
    return (unsigned)(v >> (s & 31u));
}
static inline int __clzll(long long x) { return x == 0 ? 64 : __builtin_clzll((unsigned long long)x); }
static inline float __int2float_rn(int x) { return (float)x; }
static inline float __uint2float_rn(unsigned x) { return (float)x; }
static inline int __float2int_rn(float x) { return (int)std::lrintf(x); }
static inline unsigned __float2uint_rn(float x) { return (unsigned)std::llrintf(x); }
static inline float __frcp_rn(float x) { return 1.0f / x; }
static inline float rsqrtf(float x) { return 1.0f / std::sqrt(x); }
static inline double __dmul_rn(double a, double b) { return a * b; }
static inline double __dadd_rn(double a, double b) { return a + b; }
static inline double __dsub_rn(double a, double b) { return a - b; }
static inline double __ddiv_rn(double a, double b) { return a / b; }
static inline double __dsqrt_rn(double a) { return std::sqrt(a); }
static inline float __double2float_rn(double a) { return (float)a; }

#include "../sphugo_gb300/csrc/fp64emu.cuh"

using namespace sphgpu;

static uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static bool same(double a, double b) { return emu_bits(a) == emu_bits(b) || (a != a && b != b); }
static bool samef(float a, float b) { return __float_as_uint(a) == __float_as_uint(b) || (a != a && b != b); }
static double normal(uint64_t r, uint32_t e, uint64_t fracmask = kEmuFrac) {
    return emu_double((r & kEmuSign) | ((uint64_t)e << 52) | (r & fracmask));
}

int main(int argc, char **argv) {
    const int64_t n = argc > 1 ? std::atoll(argv[1]) : 2000000;
    long long bad[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    const char *names[8] = {"mul", "add", "sub", "div", "sqrt", "1-x", "split hi", "split lo"};
    const double specials[8] = {0.0, -0.0, emu_double(1), emu_double(0x000FFFFFFFFFFFFFull), INFINITY, -INFINITY, NAN,
                                0x1p-1022};
    for (int64_t i = 0; i < n; i++) {
        const uint64_t r1 = mix64(0x51ull + 0x9E3779B97F4A7C15ull * (uint64_t)(3 * i + 1));
        const uint64_t r2 = mix64(0x51ull + 0x9E3779B97F4A7C15ull * (uint64_t)(3 * i + 2));
        const uint64_t r3 = mix64(0x51ull + 0x9E3779B97F4A7C15ull * (uint64_t)(3 * i + 3));
        const uint32_t cls = (uint32_t)(i % 6);
        double x, y;
        if (cls == 0) {  // raw bits: every exponent, zeros, subnormals, infinities, NaNs
            x = emu_double(r1);
            y = emu_double(r2);
        } else if (cls == 1 || cls == 2) {  // nearby exponents (class 2: short significands, ties)
            const uint64_t fm = cls == 2 ? 0x000FFFFFC0000000ull : kEmuFrac;
            x = normal(r1, 1000u + (uint32_t)(r3 % 48u), fm);
            y = normal(r2, 1000u + (uint32_t)((r3 >> 8) % 64u), fm);
        } else if (cls == 3) {  // the ends of the range
            const bool lo = r3 & 1u;
            x = normal(r1, lo ? 1u + (uint32_t)((r3 >> 1) % 64u) : 1983u + (uint32_t)((r3 >> 1) % 64u));
            y = normal(r2, (r3 >> 8) & 1u ? 991u + (uint32_t)((r3 >> 9) % 64u)
                                         : (lo ? 1u + (uint32_t)((r3 >> 9) % 64u) : 1983u + (uint32_t)((r3 >> 9) % 64u)));
        } else if (cls == 4) {  // near cancellation
            x = normal(r1, 900u + (uint32_t)(r3 % 256u));
            const uint32_t nb = (uint32_t)((r3 >> 8) % 53u);
            const uint64_t mask = nb ? ((1ull << nb) - 1ull) : 0ull;
            y = emu_double(((emu_bits(x) & ~mask) | (r2 & mask)) ^ kEmuSign);
        } else {  // specials against normals
            x = specials[r3 & 7u];
            y = normal(r2, 1u + (uint32_t)((r3 >> 3) % 2046u));
            if ((r3 >> 16) & 1u) std::swap(x, y);
        }
        if (!same(emu_mul(x, y), x * y)) bad[0]++;
        if (!same(emu_add(x, y), x + y)) bad[1]++;
        if (!same(emu_sub(x, y), x - y)) bad[2]++;
        // quotients, with a = RN(b q) +- 2 ulp next to boundaries for half of class 1
        double num = x, den = y;
        if (cls == 1 && ((r3 >> 24) & 1u)) {
            const double q = emu_double((1023ull << 52) | (r1 & kEmuFrac));
            num = emu_double(emu_bits(y * q) + (uint64_t)((int64_t)((r2 >> 5) % 5u) - 2));
        } else if (cls == 2) {  // exact quotients: short significands multiplied back
            const double q = emu_double((1023ull << 52) | (r1 & 0x000FFFFFFC000000ull));
            num = y * q;
        }
        if (!same(emu_div(num, emu_divisor(den), den), num / den)) bad[3]++;
        // square roots: the operand, and squares moved by -2 .. +2 ulp
        double z = x;
        if (cls == 1 || cls == 4) {
            const double sq = emu_double(((uint64_t)(512u + (uint32_t)(r3 % 1024u)) << 52) | (r1 & kEmuFrac));
            z = emu_double(emu_bits(sq * sq) + (uint64_t)((int64_t)((r2 >> 3) % 5u) - 2));
        } else if (cls == 2) {  // perfect squares
            const double sq = emu_double(((uint64_t)(512u + (uint32_t)(r3 % 1024u)) << 52) | (r1 & 0x000FFFFFFC000000ull));
            z = sq * sq;
        }
        if (!same(emu_sqrt(z), std::sqrt(z))) bad[4]++;
        const double xh = emu_double((1022ull << 52) | (r1 & kEmuFrac));
        if (!same(emu_one_minus(xh), 1.0 - xh) || !same(emu_one_minus(x), 1.0 - x)) bad[5]++;
        const double vs[2] = {x, x * y};
        for (double v : vs) {
            float h, l;
            emu_split_df(v, h, l);
            const float h0 = (float)v;
            const float l0 = (float)(v - (double)h0);
            if (!samef(h, h0)) bad[6]++;
            if (!samef(l, l0)) bad[7]++;
        }
    }
    long long total = 0;
    for (int j = 0; j < 8; j++) {
        std::printf("%-9s %lld\n", names[j], bad[j]);
        total += bad[j];
    }
    std::printf("cases %lld differing %lld\n", (long long)n, total);
    return total == 0 ? 0 : 1;
}
