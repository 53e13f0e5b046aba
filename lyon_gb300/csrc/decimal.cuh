// decimal.cuh — decimal text to f32, correctly rounded (round to nearest, ties to even), as
// Rust's `f32::from_str`, which lyon's SVG path parser calls on every number
// (crates/extra/src/parser.rs:413-467). Host and device share this code, so a string parses to
// the same bits on both.
//
// The number is its significant digits D (at most DEC_MAX_DIGITS kept; any further non-zero
// digit sets a sticky flag) and a decimal exponent e: value = D * 10^e. Three ways, fastest first:
//   1. D < 2^24 and |e| <= 10: D and 10^|e| are exact in f32, so one f32 multiply or divide
//      rounds once (the classic fast path of Clinger, "How to read floating point numbers
//      accurately", 1990).
//   2. D < 2^53 and |e| <= 22: one f64 multiply or divide rounds once to d; rounding d to f32
//      can only go wrong when d is exactly halfway between two floats, which is checked (and for
//      results below the normal range, which are sent to 3.).
//   3. Otherwise: a candidate from f64 arithmetic, then exact comparisons of D * 10^e with the
//      candidate's neighbouring midpoints in big-integer arithmetic, moving the candidate until
//      the value lies between them.
#pragma once

#include <cstdint>

#ifndef __CUDACC__
#define __host__
#define __device__
#endif

namespace lg {

constexpr int DEC_MAX_DIGITS = 120;  // digits kept exactly (more only set the sticky flag)
constexpr int BIG_LIMBS = 40;        // 1280-bit integers

struct Big {
    uint32_t w[BIG_LIMBS];
    int n;  // used limbs
};

__host__ __device__ inline void big_set(Big& b, uint64_t v) {
    b.w[0] = (uint32_t)v;
    b.w[1] = (uint32_t)(v >> 32);
    b.n = b.w[1] ? 2 : (b.w[0] ? 1 : 0);
}

__host__ __device__ inline void big_mul_small(Big& b, uint32_t m, uint32_t add = 0) {
    uint64_t carry = add;
    for (int i = 0; i < b.n; ++i) {
        const uint64_t p = (uint64_t)b.w[i] * m + carry;
        b.w[i] = (uint32_t)p;
        carry = p >> 32;
    }
    if (carry && b.n < BIG_LIMBS) b.w[b.n++] = (uint32_t)carry;
}

__host__ __device__ inline void big_mul_pow10(Big& b, int e) {
    while (e >= 9) {
        big_mul_small(b, 1000000000u);
        e -= 9;
    }
    uint32_t m = 1;
    while (e-- > 0) m *= 10u;
    if (m != 1) big_mul_small(b, m);
}

__host__ __device__ inline void big_shl(Big& b, int bits) {
    if (b.n == 0 || bits <= 0) return;
    const int words = bits / 32, r = bits % 32;
    int n = b.n + words + 1;
    if (n > BIG_LIMBS) n = BIG_LIMBS;
    for (int i = n - 1; i >= 0; --i) {
        const int s = i - words;
        uint32_t v = 0;
        if (s >= 0 && s < b.n) v = b.w[s] << r;
        if (r && s - 1 >= 0 && s - 1 < b.n) v |= b.w[s - 1] >> (32 - r);
        b.w[i] = v;
    }
    b.n = n;
    while (b.n > 0 && b.w[b.n - 1] == 0) --b.n;
}

__host__ __device__ inline int big_cmp(const Big& a, const Big& b) {
    if (a.n != b.n) return a.n < b.n ? -1 : 1;
    for (int i = a.n - 1; i >= 0; --i) {
        if (a.w[i] != b.w[i]) return a.w[i] < b.w[i] ? -1 : 1;
    }
    return 0;
}

// Exact powers of ten as f64 (10^0 .. 10^22) and as f32 (10^0 .. 10^10).
__host__ __device__ inline double pow10_exact_f64(int e) {
    double r = 1.0;
    for (int i = 0; i < e; ++i) r *= 10.0;  // exact for e <= 22
    return r;
}

__host__ __device__ inline uint32_t f32_bits(float f) {
#ifdef __CUDA_ARCH__
    return __float_as_uint(f);
#else
    uint32_t u;
    __builtin_memcpy(&u, &f, 4);
    return u;
#endif
}
__host__ __device__ inline float f32_from_bits(uint32_t u) {
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    float f;
    __builtin_memcpy(&f, &u, 4);
    return f;
#endif
}
__host__ __device__ inline uint64_t f64_bits(double d) {
#ifdef __CUDA_ARCH__
    return (uint64_t)__double_as_longlong(d);
#else
    uint64_t u;
    __builtin_memcpy(&u, &d, 8);
    return u;
#endif
}

struct Decimal {
    uint8_t digits[DEC_MAX_DIGITS];  // significant digits, no leading zeros
    int nd;                          // digits kept
    int exp10;                       // value = 0.d1 d2 ... * 10^(exp10 + nd) = D * 10^exp10
    bool sticky;                     // a non-zero digit beyond the kept ones
    bool negative;
};

// Sign of D * 10^e (+ sticky) - N * 2^k, with D the decimal's digits.
__host__ __device__ inline int compare_with(const Decimal& d, uint64_t N, int k) {
    Big left, right;
    left.n = 0;
    for (int i = 0; i < d.nd; ++i) big_mul_small(left, 10u, d.digits[i]);
    big_set(right, N);
    if (d.exp10 >= 0) {
        big_mul_pow10(left, d.exp10);
    } else {
        big_mul_pow10(right, -d.exp10);
    }
    if (k >= 0) {
        big_shl(right, k);
    } else {
        big_shl(left, -k);
    }
    const int c = big_cmp(left, right);
    if (c == 0 && d.sticky) return 1;
    return c;
}

// The midpoints around the positive finite float with bits `u` (u < 0x7F800000), as N * 2^k:
// `hi` between it and the next float up, `lo` between it and the next one down.
__host__ __device__ inline void midpoints(uint32_t u, uint64_t* nhi, int* khi, uint64_t* nlo,
                                          int* klo) {
    const uint32_t ex = u >> 23, frac = u & 0x7FFFFFu;
    uint64_t M;
    int E;
    if (ex == 0) {
        M = frac;
        E = -149;
    } else {
        M = (uint64_t)frac | 0x800000u;
        E = (int)ex - 150;
    }
    *nhi = 2 * M + 1;
    *khi = E - 1;
    if (ex > 1 && frac == 0) {
        // At the bottom of a binade the float below is half as far away.
        *nlo = 4 * M - 1;
        *klo = E - 2;
    } else {
        *nlo = 2 * M - 1;  // for u == 0 this is never used
        *klo = E - 1;
    }
}

// Correctly rounded f32 of a parsed decimal.
__host__ __device__ inline float decimal_to_f32(const Decimal& d) {
    const float sign = d.negative ? -1.0f : 1.0f;
    if (d.nd == 0) return sign * 0.0f;
    const int magnitude = d.exp10 + d.nd;  // value in [10^(magnitude-1), 10^magnitude)
    if (magnitude > 40) return sign * f32_from_bits(0x7F800000u);
    if (magnitude < -46) return sign * 0.0f;
    uint64_t D = 0;
    const bool small = d.nd <= 19 && !d.sticky;
    if (small) {
        for (int i = 0; i < d.nd; ++i) D = D * 10u + d.digits[i];
    }
    const int e = d.exp10;
    if (small && D < (1ull << 24) && e >= -10 && e <= 10) {
        float p = 1.0f;
        for (int i = 0; i < (e < 0 ? -e : e); ++i) p *= 10.0f;  // exact
        return sign * (e >= 0 ? (float)D * p : (float)D / p);
    }
    double approx;
    if (small && D < (1ull << 53) && e >= -22 && e <= 22) {
        const double p = pow10_exact_f64(e < 0 ? -e : e);
        const double v = e >= 0 ? (double)D * p : (double)D / p;
        const uint64_t b = f64_bits(v);
        const int ex = (int)((b >> 52) & 0x7FF);
        // An f32 result in the normal range whose f64 value is not exactly halfway between
        // two floats: rounding it to f32 is the correct rounding of the decimal.
        const bool normal = ex >= 1023 - 126 && ex <= 1023 + 127;
        const bool halfway = (b & 0x1FFFFFFFull) == 0x10000000ull;
        if (normal && !halfway) return sign * (float)v;
        approx = v;
    } else {
        // f64 estimate from the leading digits (within far less than an f32 ulp).
        double m = 0.0;
        const int lead = d.nd < 17 ? d.nd : 17;
        for (int i = 0; i < lead; ++i) m = m * 10.0 + (double)d.digits[i];
        int ex10 = e + (d.nd - lead);
        double p = 1.0;
        double base = ex10 < 0 ? 0.1 : 10.0;
        for (int i = 0; i < (ex10 < 0 ? -ex10 : ex10); ++i) p *= base;
        approx = m * p;
    }
    // Candidate, then exact comparisons with its neighbouring midpoints.
    float f = (float)approx;
    if (!(f == f)) f = 0.0f;
    uint32_t u = f32_bits(f < 0.0f ? -f : f);
    if (u >= 0x7F800000u) u = 0x7F7FFFFFu;  // start from the largest finite float
    for (int iter = 0; iter < 64; ++iter) {
        uint64_t nhi, nlo;
        int khi, klo;
        midpoints(u, &nhi, &khi, &nlo, &klo);
        const int chi = compare_with(d, nhi, khi);
        if (chi > 0 || (chi == 0 && (u & 1u))) {
            if (u == 0x7F7FFFFFu) return sign * f32_from_bits(0x7F800000u);
            ++u;
            continue;
        }
        if (u > 0) {
            const int clo = compare_with(d, nlo, klo);
            if (clo < 0 || (clo == 0 && (u & 1u))) {
                --u;
                continue;
            }
        }
        break;
    }
    return sign * f32_from_bits(u);
}

// Accumulates the digits of a number token: the integer part's digits, then `point()` and the
// fraction's digits, then `finish(e)` with the exponent part. value = (all digits as an integer)
// * 10^(e - fraction digits); only the first DEC_MAX_DIGITS significant digits are kept.
struct DecimalBuilder {
    Decimal d;
    bool after_point = false;
    int frac_digits = 0;  // every digit after the point, zeros included
    int dropped = 0;      // significant digits beyond the kept ones
    __host__ __device__ DecimalBuilder() {
        d.nd = 0;
        d.exp10 = 0;
        d.sticky = false;
        d.negative = false;
    }
    __host__ __device__ void digit(int v) {
        if (after_point && frac_digits < 1000000) ++frac_digits;
        if (d.nd == 0 && v == 0) return;  // a leading zero
        if (d.nd < DEC_MAX_DIGITS) {
            d.digits[d.nd++] = (uint8_t)v;
        } else {
            if (v != 0) d.sticky = true;
            if (dropped < 1000000) ++dropped;
        }
    }
    __host__ __device__ void point() { after_point = true; }
    __host__ __device__ float finish(long long e) {
        long long ex = e - frac_digits + dropped;
        if (ex > 100000) ex = 100000;
        if (ex < -100000) ex = -100000;
        d.exp10 = (int)ex;
        // Trailing zeros of the kept digits only scale them.
        while (d.nd > 0 && d.digits[d.nd - 1] == 0) {
            --d.nd;
            ++d.exp10;
        }
        return decimal_to_f32(d);
    }
};

}  // namespace lg
