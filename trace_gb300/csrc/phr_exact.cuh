// Exact float64 results of the PHR sweep from cheaper arithmetic.
//
// The reference evaluates its SAH sweep in float64 (phr.go:368-459,
// bounding.go:45-47).  GB300 runs float64 at a small fraction of its float32
// and integer rates, so these helpers give the same float64 results, or the
// same decisions, with float32 and integer operations, falling back to
// float64 only where that cannot be shown:
//   - bary_bits: the bits of fl64(fl64(a + b) * 0.5) for float32 a, b (the
//     barycenter sort key, phr.go:370-404) by an exact integer sum whenever
//     the operands' exponents are within 28 of each other;
//   - surface32 and the screening bounds: aabb.surface in float32 is within
//     5 units of float32 rounding of the exact value (every term is
//     non-negative, five roundings on any path), and float64's within 5 of
//     its own; a cost fl(SA_R * n_R) + fl(SA_L * n_L) adds at most three more
//     (products, sum, and the count's conversion).  The bounds need every
//     rounding to be relative, which holds when every box coordinate is 0 or
//     of magnitude in [2^-30, 2^30]: differences are then 0 or at least 2^-53,
//     products of two at least 2^-106 (no underflow) and costs below 2^96 (no
//     overflow).  phr_screen_ok tests one coordinate.
// This file is included by device code and by a host-side unit test.
#pragma once

#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define GBT_HD __host__ __device__ __forceinline__
// out of line: a rare path the compiler would otherwise predicate into every call
#define GBT_HD_RARE static __host__ __device__ __noinline__
#else
#define GBT_HD inline
#define GBT_HD_RARE static inline
#endif

namespace gbt_phr {

GBT_HD uint32_t f32_bits(float x) {
#ifdef __CUDA_ARCH__
    return __float_as_uint(x);
#else
    uint32_t u;
    memcpy(&u, &x, 4);
    return u;
#endif
}

GBT_HD uint64_t f64_bits(double x) {
#ifdef __CUDA_ARCH__
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t u;
    memcpy(&u, &x, 8);
    return u;
#endif
}

GBT_HD int clz64(uint64_t x) {
#ifdef __CUDA_ARCH__
    return __clzll((long long)x);
#else
    return __builtin_clzll(x);
#endif
}

// The rounded float64 form of bary_bits, for the operands it cannot sum exactly.
GBT_HD_RARE uint64_t bary_bits_rounded(float a, float b) {
    const double s = (double)a + (double)b;  // rounded (or inf/NaN): float64 as the reference
    return f64_bits(s * 0.5);
}

// fl64(fl64((double)a + (double)b) * 0.5) as bits.
GBT_HD uint64_t bary_bits(float a, float b) {
    const uint32_t ua = f32_bits(a), ub = f32_bits(b);
    const uint32_t ea = (ua >> 23) & 0xffu, eb = (ub >> 23) & 0xffu;
    if (ea != 0xffu && eb != 0xffu) {
        // value = m * 2^(x - 150); a zero exponent field is a subnormal with x = 1
        const int64_t ma = (int64_t)((ua & 0x7fffffu) | (ea ? 0x800000u : 0u));
        const int64_t mb = (int64_t)((ub & 0x7fffffu) | (eb ? 0x800000u : 0u));
        const int xa = ea ? (int)ea : 1, xb = eb ? (int)eb : 1;
        if (ma == 0 && mb == 0)  // +-0 + +-0: -0 only when both are -0; halving keeps it
            return (uint64_t)(ua & ub & 0x80000000u) << 32;
        int64_t hi_m = ma, lo_m = mb;
        int hi_x = xa, lo_x = xb;
        uint32_t hi_s = ua >> 31, lo_s = ub >> 31;
        if (xb > xa) {
            hi_m = mb; lo_m = ma; hi_x = xb; lo_x = xa; hi_s = ub >> 31; lo_s = ua >> 31;
        }
        const int d = hi_x - lo_x;
        if (lo_m == 0 || d <= 28) {
            // exact: |S| < 2^52 + 2^24 < 2^53, so the float64 sum is S * 2^(x - 150) unrounded
            int64_t A = lo_m == 0 ? hi_m : hi_m << d, B = lo_m;
            const int x = lo_m == 0 ? hi_x : lo_x;
            if (hi_s) A = -A;
            if (lo_s) B = -B;
            const int64_t S = A + B;
            if (S == 0) return 0;  // exact cancellation: +0
            const uint64_t sign = S < 0 ? 1u : 0u;
            const uint64_t U = (uint64_t)(S < 0 ? -S : S);
            const int msb = 63 - clz64(U);  // <= 52
            const int e2 = msb + x - 150;   // the sum is 1.f * 2^e2
            const uint64_t frac = (U << (52 - msb)) & ((1ull << 52) - 1);
            return (sign << 63) | ((uint64_t)(e2 - 1 + 1023) << 52) | frac;  // times 0.5
        }
    }
    return bary_bits_rounded(a, b);
}

// Orders like the float64 value (sort key of the bits).
GBT_HD unsigned long long key_of_bits(uint64_t b) {
    return (b >> 63) ? ~b : (b | 0x8000000000000000ULL);
}

// aabb.surface in float32, operations in the float64 version's order.
GBT_HD float surface32(const float *lo, const float *hi) {
    const float w = hi[0] - lo[0], h = hi[1] - lo[1], d = hi[2] - lo[2];
    const float a = (2.0f * w) * h, b = (2.0f * w) * d, c = (2.0f * h) * d;
    return (a + b) + c;
}

// float(c) for a count, within one float32 rounding (the screening bound allows
// one), from integer and float32 adds only: 2^23 + k has the bits 0x4b000000 | k
// for k < 2^23, and the two 12/20-bit halves convert exactly.
GBT_HD float count_f32(uint32_t c) {
    uint32_t hb = 0x4b000000u | (c >> 12), lb = 0x4b000000u | (c & 0xfffu);
    float h, l;
#ifdef __CUDA_ARCH__
    h = __uint_as_float(hb);
    l = __uint_as_float(lb);
#else
    memcpy(&h, &hb, 4);
    memcpy(&l, &lb, 4);
#endif
    return (h - 8388608.0f) * 4096.0f + (l - 8388608.0f);
}

// A box coordinate inside the range where the screening bounds hold.
GBT_HD bool phr_screen_ok(float c) {
    const float m = c < 0.f ? -c : c;
    return m == 0.f || (m >= 9.313225746154785e-10f && m <= 1073741824.0f);  // 2^-30, 2^30
}

// Split positions whose float32 cost is at most m * (1 + 2^-17), m the least
// float32 cost, include every position of least float64 cost: the two costs of
// one position differ by at most 16.1 units of float32 rounding relative.
constexpr float SCREEN_SLACK = 1.0f + 7.62939453125e-06f;  // 1 + 2^-17
// A surface compared with a threshold t: below t * (1 - 2^-19) in float32 is
// below t in float64, above t * (1 + 2^-19) is above it.
constexpr double THR_LO = 1.0 - 1.9073486328125e-06;  // 1 - 2^-19
constexpr double THR_HI = 1.0 + 1.9073486328125e-06;

}  // namespace gbt_phr
