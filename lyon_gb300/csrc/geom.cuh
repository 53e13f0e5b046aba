// geom.cuh — device geometry shared by the stroke, fill and flatten kernels.
//
// Every routine evaluates in f32 with the same operation order as lyon (the translation unit is
// compiled with --fmad=false, so no multiply-add is fused), so positions computed here are
// bit-identical to lyon's wherever only + - * / sqrt are involved. Angles from vectors use
// euclid's fast_atan2 polynomial, exactly as lyon does (pure f32 arithmetic); cosf, sinf,
// acosf and log2f use CUDA's accurate f32 functions, and the few places where their last bit
// could change a count are evaluated correctly rounded (see the call sites).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/lyon_gpu.h"

#if !defined(__CUDACC__) && !defined(__noinline__)
#define __noinline__ __attribute__((noinline))
#endif

namespace lg {

// ---- vectors (euclid::default::{Point2D, Vector2D} with f32) -------------------------------
struct V2 {
    float x, y;
};
__host__ __device__ __forceinline__ V2 v2(float x, float y) { return V2{x, y}; }
__host__ __device__ __forceinline__ V2 operator+(V2 a, V2 b) { return V2{a.x + b.x, a.y + b.y}; }
__host__ __device__ __forceinline__ V2 operator-(V2 a, V2 b) { return V2{a.x - b.x, a.y - b.y}; }
__host__ __device__ __forceinline__ V2 operator*(V2 a, float s) { return V2{a.x * s, a.y * s}; }
__host__ __device__ __forceinline__ V2 operator/(V2 a, float s) { return V2{a.x / s, a.y / s}; }
__host__ __device__ __forceinline__ V2 operator-(V2 a) { return V2{-a.x, -a.y}; }
__host__ __device__ __forceinline__ float dot(V2 a, V2 b) { return a.x * b.x + a.y * b.y; }
__host__ __device__ __forceinline__ float cross(V2 a, V2 b) { return a.x * b.y - a.y * b.x; }
__host__ __device__ __forceinline__ float sqlen(V2 a) { return a.x * a.x + a.y * a.y; }
__host__ __device__ __forceinline__ float vlength(V2 a) { return sqrtf(sqlen(a)); }
__host__ __device__ __forceinline__ V2 normalize(V2 a) { return a / vlength(a); }
__host__ __device__ __forceinline__ bool peq(V2 a, V2 b) { return a.x == b.x && a.y == b.y; }
__host__ __device__ __forceinline__ V2 perp(V2 v) { return V2{-v.y, v.x}; }  // utils.rs:15-17
__host__ __device__ __forceinline__ V2 lerp(V2 a, V2 b, float t) {
    float one_t = 1.0f - t;
    return V2{one_t * a.x + t * b.x, one_t * a.y + t * b.y};
}
#define LG_PI_F 3.14159265358979323846f
#define LG_FRAC_PI_2_F 1.57079632679489661923f
// euclid 0.22.9 `Vector2D::angle_from_x_axis` = `Trig::fast_atan2(y, x)` (euclid src/trig.rs),
// which lyon calls for join, cap and sharp-turn angles (stroke.rs:1812,1986-1987,2482-2483,3204).
// Published method: the polynomial approximation of atan on [0, 1] from math.stackexchange.com
// question 1098487 (answer 1105038), atan(a) ~ ((-0.0464964749 s + 0.15931422) s - 0.327622764)
// s a + a with s = a^2 and a = min(|x|,|y|) / max(|x|,|y|), reflected into the octant of (x, y).
// Only f32 + - * / and compares (no fused multiply-add in this build), so it rounds as lyon's.
// (0, 0) gives NaN (0 / 0), as euclid's does.
__host__ __device__ __forceinline__ float fast_atan2(float y, float x) {
    const float x_abs = fabsf(x);
    const float y_abs = fabsf(y);
    const float a = fminf(x_abs, y_abs) / fmaxf(x_abs, y_abs);
    const float s = a * a;
    float r = ((-0.0464964749f * s + 0.15931422f) * s - 0.327622764f) * s * a + a;
    if (y_abs > x_abs) r = LG_FRAC_PI_2_F - r;
    if (x < 0.0f) r = LG_PI_F - r;
    if (y < 0.0f) r = -r;
    return r;
}
__host__ __device__ __forceinline__ float angle_from_x_axis(V2 v) { return fast_atan2(v.y, v.x); }
// euclid 0.22.9 `Angle::angle_to` (euclid src/angle.rs): d = (to - from) % max, then
// (2 d) % max - d with max = PI * 2 and the exact float remainder (fmodf).
__host__ __device__ __forceinline__ float angle_to(float from, float to) {
    const float max = LG_PI_F * 2.0f;
    const float d = fmodf(to - from, max);
    return fmodf(2.0f * d, max) - d;
}
__host__ __device__ __forceinline__ bool isnan_f(float v) { return v != v; }

__device__ __forceinline__ V2 load_pt(const float* pts, uint32_t i) {
    float2 p = reinterpret_cast<const float2*>(pts)[i];
    return V2{p.x, p.y};
}

// Rust `as u32` on f32 (saturating, NaN -> 0).
__host__ __device__ __forceinline__ uint32_t sat_u32(float v) {
    if (!(v == v) || v <= 0.0f) return 0u;
    if (v >= 4294967295.0f) return 0xFFFFFFFFu;
    return (uint32_t)v;
}
// NumCast::to_u32 on f32: None (-> 1 in lyon's unwrap_or) outside (-1, 2^32).
__host__ __device__ __forceinline__ uint32_t to_u32_or1(float n) {
    if (n > -1.0f && n < 4294967296.0f) return (uint32_t)n;
    return 1u;
}

// ---- flattening segment counts (quadratic_bezier.rs:943-974, cubic_bezier.rs:1369-1403) -----
__host__ __device__ __forceinline__ float wang_from_err4(float err4) {
    // i^4 for i in 1..=24; the first i with err4 <= i^4 is ceil(err4^(1/4)).
    if (err4 <= 331776.0f) {
#pragma unroll 1
        for (int i = 1; i <= 24; ++i) {
            float f = (float)i;
            float lut = (f * f) * (f * f);
            if (err4 <= lut) return f;
        }
    }
    return fmaxf(sqrtf(sqrtf(err4)), 1.0f);
}

__host__ __device__ __forceinline__ float quad_wang(V2 from, V2 ctrl, V2 to, float tol) {
    V2 l = ((from - ctrl * 2.0f) + to) * 2.0f;
    float d = 1.0f / (8.0f * tol);
    float err4 = dot(l, l) * d * d;
    return wang_from_err4(err4);
}

__host__ __device__ __forceinline__ float cubic_wang(V2 from, V2 c1, V2 c2, V2 to, float tol) {
    V2 v1 = ((from - c1 * 2.0f) + c2) * 6.0f;
    V2 v2_ = ((c1 - c2 * 2.0f) + to) * 6.0f;
    float l = fmaxf(dot(v1, v1), dot(v2_, v2_));
    float d = 1.0f / (8.0f * tol);
    float err4 = l * d * d;
    return wang_from_err4(err4);
}

// Polynomial forms and Horner samples (quadratic_bezier.rs:891-900,928-938;
// cubic_bezier.rs:1318-1325,1350-1363). A quadratic is stored with a3 = 0 and `cubic` false.
struct Poly {
    V2 a0, a1, a2, a3;
    bool cubic;
};
__host__ __device__ __forceinline__ Poly quad_poly(V2 from, V2 ctrl, V2 to) {
    Poly p;
    p.a0 = from;
    p.a1 = (ctrl - from) * 2.0f;
    p.a2 = (from + to) - ctrl * 2.0f;
    p.a3 = V2{0.0f, 0.0f};
    p.cubic = false;
    return p;
}
__host__ __device__ __forceinline__ Poly cubic_poly(V2 from, V2 c1, V2 c2, V2 to) {
    Poly p;
    p.a0 = from;
    p.a1 = (c1 - from) * 3.0f;
    p.a2 = ((from * 3.0f) - (c1 * 6.0f)) + (c2 * 3.0f);
    p.a3 = (to - from) + ((c1 - c2) * 3.0f);
    p.cubic = true;
    return p;
}
__host__ __device__ __forceinline__ V2 poly_sample(const Poly& p, float t) {
    V2 v = p.a0;
    float t2 = t;
    v = v + p.a1 * t2;
    t2 *= t;
    v = v + p.a2 * t2;
    if (p.cubic) {
        t2 *= t;
        v = v + p.a3 * t2;
    }
    return v;
}

// quadratic_bezier.rs:35-41
__host__ __device__ __forceinline__ V2 quad_sample(V2 from, V2 ctrl, V2 to, float t) {
    float t2 = t * t;
    float one_t = 1.0f - t;
    float one_t2 = one_t * one_t;
    V2 r;
    r.x = from.x * one_t2 + ctrl.x * 2.0f * one_t * t + to.x * t2;
    r.y = from.y * one_t2 + ctrl.y * 2.0f * one_t * t + to.y * t2;
    return r;
}

// stroke.rs:3178-3212 (find_sharp_turn) with quadratic_bezier.rs:180-191.
static __device__ __noinline__ bool find_sharp_turn(V2 from, V2 ctrl, V2 to, float* t_out) {
    V2 baseline = to - from;
    V2 v = ctrl - from;
    V2 n = V2{-baseline.y, baseline.x};
    float v_dot_b = dot(v, baseline);
    float v_dot_n = dot(v, n);
    V2 long_axis;
    if ((v_dot_b >= 0.0f && v_dot_b <= dot(baseline, baseline)) ||
        fabsf(v_dot_n) * 2.0f >= fabsf(v_dot_b)) {
        if (sqlen(baseline) * 30.0f > sqlen(v)) return false;
        long_axis = v;
    } else {
        long_axis = baseline;
    }
    // Rotation2D::new(-long_axis.angle_from_x_axis()): euclid's fast_atan2, then the correctly
    // rounded f32 sine and cosine (evaluated in f64, rounded once), as the oracle does: the split
    // point feeds later integer decisions and must be bit-identical.
    float angle = -angle_from_x_axis(long_axis);
    float s = (float)sin((double)angle), c = (float)cos((double)angle);
    float cx = v.x * c - v.y * s;
    float tx = baseline.x * c - baseline.y * s;
    float div = 0.0f - 2.0f * cx + tx;
    if (div == 0.0f) return false;
    float t = (0.0f - cx) / div;
    if (t > 0.0f && t < 1.0f) {
        *t_out = t;
        return true;
    }
    return false;
}

// The k-th value (k >= 0) of lyon's accumulated flattening parameter: t_0 = 0 and
// t_{j+1} = fl(t_j + s) (quadratic_bezier.rs:368-391, cubic_bezier.rs:590-614), evaluated from
// a known earlier value (k0, t0) without the k - k0 sequential additions. Inside one binade
// [2^e, 2^(e+1)) every representable value is a multiple of the ulp u, so fl(t + s) - t only
// depends on s mod u — except at an exact tie, where round-to-even makes the first step land on
// an even multiple and every later step in the binade repeat the same increment. The walk
// therefore takes the first step of each binade explicitly and then jumps over the steps that
// stay inside it; the result equals the sequential loop bit for bit.
__host__ __device__ __forceinline__ uint32_t f2u(float f) {
#ifdef __CUDA_ARCH__
    return __float_as_uint(f);
#else
    uint32_t u;
    __builtin_memcpy(&u, &f, 4);
    return u;
#endif
}
__host__ __device__ __forceinline__ float u2f(uint32_t u) {
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    float f;
    __builtin_memcpy(&f, &u, 4);
    return f;
#endif
}

__host__ __device__ __forceinline__ float accumulate_t(float s, uint32_t k0, float t0, uint32_t k) {
    float t = t0;
    uint32_t j = k0;
    while (j < k) {
        if (t == 0.0f) {
            t = 0.0f + s;
            ++j;
            continue;
        }
        const uint32_t bits = f2u(t);
        const int e = (int)((bits >> 23) & 0xFFu);
        const float B = u2f((uint32_t)(e + 1) << 23);
        const float tn = t + s;
        ++j;
        t = tn;
        if (tn >= B || j >= k) continue;
        const float d = (t + s) - t;
        if (d == 0.0f) break;  // t + s rounds back to t: the sequence is stuck
        // Work in units of the binade's ulp u = 2^(e - 150): scaling by 1/u is exact.
        const float inv_u = u2f((uint32_t)(150 + 127 - e) << 23);
        const uint32_t W = (uint32_t)((B - t) * inv_u);
        const uint32_t D = (uint32_t)(d * inv_u);
        // m = (W - 1) / D, from a float estimate corrected to the exact quotient.
#ifdef __CUDA_ARCH__
        uint32_t m = (uint32_t)__fdividef((float)(W - 1u), (float)D);
#else
        uint32_t m = (uint32_t)((float)(W - 1u) / (float)D);
#endif
        while (m > 0 && m * D > W - 1u) --m;
        while ((m + 1) * D <= W - 1u) ++m;
        const uint32_t rem = k - j;
        const uint32_t take = m < rem ? m : rem;
        // take * d = (take * D) * u, exactly (u is a power of two, take * D < 2^24).
        const float u = e > 23 ? u2f((uint32_t)(e - 23) << 23) : d / (float)D;
        t = t + (float)(take * D) * u;
        j += take;
    }
    return t;
}

// accumulate_t when the value at k0 is known (t0 > 0) and the k - k0 steps stay in t0's binade
// [2^e, 2^(e+1)): after the first step every step adds the same d (see accumulate_t), so
// t_k = t_(k0+1) + (k - k0 - 1) * d, with every operation exact. Falls back to the binade walk
// otherwise.
__host__ __device__ __forceinline__ float accumulate_t_from(float s, uint32_t k0, float t0,
                                                            uint32_t k) {
    if (t0 > 0.0f && k > k0) {
        const uint32_t e = (f2u(t0) >> 23) & 0xFFu;
        const float B = u2f((e + 1u) << 23);
        const float t1 = t0 + s;
        if (t1 < B) {
            const float d = (t1 + s) - t1;
            const float r = t1 + (float)(k - k0 - 1u) * d;
            if (r < B) return r;
        }
    }
    return accumulate_t(s, k0, t0, k);
}

// ---- fill ordering predicates (fill.rs:2122-2151) --------------------------------------------
__host__ __device__ __forceinline__ int compare_positions(V2 a, V2 b) {
    if (a.y > b.y) return 1;
    if (a.y < b.y) return -1;
    if (a.x > b.x) return 1;
    if (a.x < b.x) return -1;
    return 0;
}
__host__ __device__ __forceinline__ bool is_after(V2 a, V2 b) {
    return a.y > b.y || (a.y == b.y && a.x > b.x);
}
__host__ __device__ __forceinline__ bool is_near(V2 a, V2 b) { return sqlen(a - b) < 0.000000001f; }

}  // namespace lg
