// lyon_oracle.cpp — TEST INFRASTRUCTURE ONLY (the oracle).
//
// A plain CPU restatement of lyon's tessellation hot path, used to check the GPU library:
// curve flattening, the fixed-width StrokeTessellator and the FillTessellator. It follows the
// reference algorithm step by step and in the same emission order, citing the lyon source file
// and line range of every routine (paths are relative to the lyon repository). Only tests,
// `__graft_entry__.smoke()` and the CPU-baseline leg of `bench.py` may load it; the product path
// never calls it.
//
// Arithmetic conventions (compile with -ffp-contract=off so no multiply-add is fused, as in Rust):
//   * f32 wherever lyon uses f32, f64 exactly where lyon converts to f64
//     (stroke.rs:2169-2173,2243-2247,2285-2312; fill.rs:1634-1676);
//   * f32 math functions (acosf, cosf, sinf, atan2f, log2f) from the platform libm, as Rust's std;
//   * helpers that live in the third-party crate euclid 0.22.9 (Cargo.lock:603-605; not part of
//     the lyon sources) are restated from euclid's published source: `normalize` = v / |v|,
//     `lerp(a, b, t)` = a * (1 - t) + b * t, `angle_from_x_axis` = euclid's `Trig::fast_atan2`
//     (a degree-7 polynomial for atan on [0, 1], folded into the quadrants; see fast_atan2
//     below), `Angle::angle_to` = `(2d) % 2pi - d` with `d = (to - from) % 2pi`,
//     `Rotation2D::transform_vector` = (x cos - y sin, y cos + x sin). These use only + - * /
//     and fmod, so they round exactly as lyon's calls do;
//   * cos/sin/acos/asin with a count or a split point depending on their last bit are
//     evaluated in f64 and rounded once (the correctly rounded f32 value, which the GPU
//     reproduces), documented at each site.
//
// Where lyon would panic (an `assert!`, an `unwrap` of a NaN comparison) the oracle reports
// LYON_ERR_INTERNAL for that path instead.

#include <cmath>
#include <cfloat>
#include <cstdint>
#include <cstring>
#include <cstdlib>
#include <vector>
#include <algorithm>
#include <thread>
#include <atomic>
#include <memory>

#include "../include/lyon_gpu.h"

namespace lo {

// --------------------------------------------------------------------------------------------
// Vector helpers (euclid::default::{Point2D, Vector2D} with f32).
// --------------------------------------------------------------------------------------------
struct P {
    float x, y;
};
static inline P pt(float x, float y) { return P{x, y}; }
static inline P add(P a, P b) { return P{a.x + b.x, a.y + b.y}; }
static inline P sub(P a, P b) { return P{a.x - b.x, a.y - b.y}; }
static inline P mul(P a, float s) { return P{a.x * s, a.y * s}; }
static inline P dvs(P a, float s) { return P{a.x / s, a.y / s}; }
static inline P neg(P a) { return P{-a.x, -a.y}; }
static inline float dot(P a, P b) { return a.x * b.x + a.y * b.y; }
static inline float cross(P a, P b) { return a.x * b.y - a.y * b.x; }
static inline float sqlen(P a) { return a.x * a.x + a.y * a.y; }
static inline float length(P a) { return sqrtf(sqlen(a)); }
static inline P normalize(P a) { return dvs(a, length(a)); }
static inline bool peq(P a, P b) { return a.x == b.x && a.y == b.y; }
static inline P lerp(P a, P b, float t) {
    float one_t = 1.0f - t;
    return P{one_t * a.x + t * b.x, one_t * a.y + t * b.y};
}
static inline P tangent(P v) { return P{-v.y, v.x}; }  // geom/src/utils.rs:15-17
static const float PI_F = 3.14159265358979323846f;
static const float FRAC_PI_2_F = 1.57079632679489661923f;
// euclid 0.22.9 `impl Trig for f32 { fn fast_atan2 }` (euclid src/trig.rs), which lyon reaches
// through `Vector2D::angle_from_x_axis` (stroke.rs:1812,1986-1987,2482-2483,3204; arc.rs:129-131).
// Published method: the polynomial approximation of atan(a) on [0, 1] given at
// math.stackexchange.com/questions/1098487 (answer 1105038),
//   atan(a) ~ ((-0.0464964749 s + 0.15931422) s - 0.327622764) s a + a,  s = a^2,
// with a = min(|x|, |y|) / max(|x|, |y|), then reflected into the octant of (x, y). Evaluated
// left to right in f32 without fused multiply-adds, as Rust evaluates it. (0, 0) gives NaN
// (0 / 0), as euclid's does.
static inline float fast_atan2(float y, float x) {
    const float x_abs = fabsf(x);
    const float y_abs = fabsf(y);
    const float a = fminf(x_abs, y_abs) / fmaxf(x_abs, y_abs);
    const float s = a * a;
    float r = ((-0.0464964749f * s + 0.15931422f) * s - 0.327622764f) * s * a + a;
    if (y_abs > x_abs) r = FRAC_PI_2_F - r;
    if (x < 0.0f) r = PI_F - r;
    if (y < 0.0f) r = -r;
    return r;
}
static inline float angle_from_x_axis(P v) { return fast_atan2(v.y, v.x); }
// euclid 0.22.9 `Angle::angle_to` (euclid src/angle.rs): the shortest signed angle, computed as
// `d = (to - from) % max; (2 * d) % max - d` with `max = PI * 2` and Rust's float remainder
// (C's fmodf: exact).
static inline float angle_to(float from, float to) {
    const float max = PI_F * 2.0f;
    const float d = fmodf(to - from, max);
    return fmodf(2.0f * d, max) - d;
}
static inline bool is_nan_f(float v) { return v != v; }

struct D {
    double x, y;
};
static inline D dd(P p) { return D{(double)p.x, (double)p.y}; }

// Near-tie bookkeeping: every integer decision taken from a fractional value (flattening
// segment counts, round-join subdivision counts) bumps this counter when the value lies within
// 1e-6 (relative) of the integer boundary, so that parity tests can count such cases.
static thread_local uint32_t g_near_ties = 0;
static inline void note_tie(double v) {
    if (!(v == v) || v > 1e12) return;
    double r = std::nearbyint(v);
    if (std::fabs(v - r) <= 1e-6 * std::max(1.0, std::fabs(v)) && r >= 1.0) ++g_near_ties;
}

// Rust `as u32` on f32 saturates; NaN -> 0.
static inline uint32_t sat_u32(float v) {
    if (!(v == v)) return 0;
    if (v <= 0.0f) return 0;
    if (v >= 4294967295.0f) return 0xFFFFFFFFu;
    return (uint32_t)v;
}

// NumCast::to_u32 for f32: None outside (-1, 2^32), truncation inside.
static inline uint32_t to_u32_or1(float n) {
    if (n > -1.0f && n < 4294967296.0f) return (uint32_t)n;
    return 1;
}

// --------------------------------------------------------------------------------------------
// Flattening (crates/geom/src/quadratic_bezier.rs, crates/geom/src/cubic_bezier.rs).
// --------------------------------------------------------------------------------------------
static const float WANG_LUT[24] = {1.0f,      16.0f,     81.0f,     256.0f,    625.0f,
                                   1296.0f,   2401.0f,   4096.0f,   6561.0f,   10000.0f,
                                   14641.0f,  20736.0f,  28561.0f,  38416.0f,  50625.0f,
                                   65536.0f,  83521.0f,  104976.0f, 130321.0f, 160000.0f,
                                   194481.0f, 234256.0f, 279841.0f, 331776.0f};

// quadratic_bezier.rs:943-974 / cubic_bezier.rs:1369-1403 (shared tail).
static float wang_from_err4(float err4) {
    note_tie(std::sqrt(std::sqrt((double)err4)));
    if (err4 <= 331776.0f) {
        for (int i = 0; i < 24; ++i) {
            if (err4 <= WANG_LUT[i]) return (float)(i + 1);
        }
    }
    return fmaxf(sqrtf(sqrtf(err4)), 1.0f);
}

struct Quad {
    P from, ctrl, to;
};
struct Cubic {
    P from, ctrl1, ctrl2, to;
};

static float quad_wang(const Quad& c, float tol) {
    // quadratic_bezier.rs:943-951
    P l = mul(add(sub(c.from, mul(c.ctrl, 2.0f)), c.to), 2.0f);
    float d = 1.0f / (8.0f * tol);
    float err4 = dot(l, l) * d * d;
    return wang_from_err4(err4);
}

static float cubic_wang(const Cubic& c, float tol) {
    // cubic_bezier.rs:1369-1379
    P v1 = mul(add(sub(c.from, mul(c.ctrl1, 2.0f)), c.ctrl2), 6.0f);
    P v2 = mul(add(sub(c.ctrl1, mul(c.ctrl2, 2.0f)), c.to), 6.0f);
    float l = fmaxf(dot(v1, v1), dot(v2, v2));
    float d = 1.0f / (8.0f * tol);
    float err4 = l * d * d;
    return wang_from_err4(err4);
}

// quadratic_bezier.rs:891-900 (polynomial form) and 928-938 (Horner sample).
struct QuadPoly {
    P a0, a1, a2;
    explicit QuadPoly(const Quad& c) {
        a0 = c.from;
        a1 = mul(sub(c.ctrl, c.from), 2.0f);
        a2 = sub(add(c.from, c.to), mul(c.ctrl, 2.0f));
    }
    P sample(float t) const {
        P v = a0;
        float t2 = t;
        v = add(v, mul(a1, t2));
        t2 *= t;
        v = add(v, mul(a2, t2));
        return v;
    }
};

// cubic_bezier.rs:1318-1325 (polynomial form) and 1350-1363 (Horner sample).
struct CubicPoly {
    P a0, a1, a2, a3;
    explicit CubicPoly(const Cubic& c) {
        a0 = c.from;
        a1 = mul(sub(c.ctrl1, c.from), 3.0f);
        a2 = add(sub(mul(c.from, 3.0f), mul(c.ctrl1, 6.0f)), mul(c.ctrl2, 3.0f));
        a3 = add(sub(c.to, c.from), mul(sub(c.ctrl1, c.ctrl2), 3.0f));
    }
    P sample(float t) const {
        P v = a0;
        float t2 = t;
        v = add(v, mul(a1, t2));
        t2 *= t;
        v = add(v, mul(a2, t2));
        t2 *= t;
        v = add(v, mul(a3, t2));
        return v;
    }
};

// for_each_flattened_with_t: quadratic_bezier.rs:368-391, cubic_bezier.rs:590-614.
// cb(from, to, t0, t1)
template <class Poly, class F>
static void flatten_with_t(const Poly& poly, P from0, P to_end, float n, F&& cb) {
    float step = 1.0f / n;
    float t0 = 0.0f;
    uint32_t count = to_u32_or1(n) - 1;
    P from = from0;
    for (uint32_t i = 0; i < count; ++i) {
        float t1 = t0 + step;
        P to = poly.sample(t1);
        cb(from, to, t0, t1);
        from = to;
        t0 = t1;
    }
    cb(from, to_end, t0, 1.0f);
}

template <class F>
static void quad_flatten_with_t(const Quad& c, float tol, F&& cb) {
    float n = quad_wang(c, tol);
    QuadPoly poly(c);
    flatten_with_t(poly, c.from, c.to, n, cb);
}

template <class F>
static void cubic_flatten_with_t(const Cubic& c, float tol, F&& cb) {
    float n = cubic_wang(c, tol);
    CubicPoly poly(c);
    flatten_with_t(poly, c.from, c.to, n, cb);
}

// quadratic_bezier.rs:35-41
static P quad_sample(const Quad& c, float t) {
    float t2 = t * t;
    float one_t = 1.0f - t;
    float one_t2 = one_t * one_t;
    P r;
    r.x = c.from.x * one_t2 + c.ctrl.x * 2.0f * one_t * t + c.to.x * t2;
    r.y = c.from.y * one_t2 + c.ctrl.y * 2.0f * one_t * t + c.to.y * t2;
    return r;
}

// quadratic_bezier.rs:208-224
static void quad_split(const Quad& c, float t, Quad* before, Quad* after) {
    P split_point = quad_sample(c, t);
    before->from = c.from;
    before->ctrl = lerp(c.from, c.ctrl, t);
    before->to = split_point;
    after->from = split_point;
    after->ctrl = lerp(c.ctrl, c.to, t);
    after->to = c.to;
}

// quadratic_bezier.rs:180-191
static bool quad_local_x_extremum_t(const Quad& c, float* out) {
    float div = c.from.x - 2.0f * c.ctrl.x + c.to.x;
    if (div == 0.0f) return false;
    float t = (c.from.x - c.ctrl.x) / div;
    if (t > 0.0f && t < 1.0f) {
        *out = t;
        return true;
    }
    return false;
}

// --------------------------------------------------------------------------------------------
// Path iteration (crates/path/src/path.rs:843-909).
// --------------------------------------------------------------------------------------------
enum EvtKind { EV_BEGIN, EV_LINE, EV_QUAD, EV_CUBIC, EV_END };
struct Evt {
    EvtKind kind;
    P from, ctrl1, ctrl2, to;  // Begin: to = at. End: from = last, to = first.
    bool close;
    float w_from = NAN, w_to = NAN;  // endpoint width factors (variable line width only)
    // Endpoint ids (IdEvent, crates/path/src/events.rs): the index of the endpoint's point in the
    // path's point array, as lyon's Path::id_iter gives them for a path without attributes.
    uint32_t id_from = 0, id_to = 0;
};

struct PathIter {
    const uint8_t* verbs;
    uint32_t nverbs;
    const float* pts;
    uint32_t npts;
    // Optional per-point width factors (the endpoint attribute that
    // StrokeOptions::variable_line_width names, stroke.rs:646-767); indexed like the points.
    const float* widths = nullptr;
    uint32_t vi = 0, pi = 0;
    P current{0, 0}, first{0, 0};
    float cur_w = NAN, first_w = NAN;
    uint32_t cur_id = 0, first_id = 0;
    uint32_t last_idx = 0;
    bool bad = false;
    P take() {
        if (pi >= npts) {
            bad = true;
            last_idx = npts;
            return P{NAN, NAN};
        }
        P p{pts[2 * pi], pts[2 * pi + 1]};
        last_idx = pi;
        ++pi;
        return p;
    }
    float width_at(uint32_t idx) const { return widths && idx < npts ? widths[idx] : NAN; }
    bool next(Evt* e) {
        if (vi >= nverbs) return false;
        uint8_t v = verbs[vi++];
        switch (v) {
            case LYON_VERB_BEGIN:
                current = take();
                cur_w = width_at(last_idx);
                cur_id = first_id = last_idx;
                first = current;
                first_w = cur_w;
                e->w_to = cur_w;
                e->id_to = cur_id;
                e->kind = EV_BEGIN;
                e->to = current;
                return true;
            case LYON_VERB_LINE_TO:
                e->kind = EV_LINE;
                e->from = current;
                e->w_from = cur_w;
                e->id_from = cur_id;
                current = take();
                cur_w = width_at(last_idx);
                cur_id = e->id_to = last_idx;
                e->w_to = cur_w;
                e->to = current;
                return true;
            case LYON_VERB_QUADRATIC_TO:
                e->kind = EV_QUAD;
                e->from = current;
                e->w_from = cur_w;
                e->id_from = cur_id;
                e->ctrl1 = take();
                current = take();
                cur_w = width_at(last_idx);
                cur_id = e->id_to = last_idx;
                e->w_to = cur_w;
                e->to = current;
                return true;
            case LYON_VERB_CUBIC_TO:
                e->kind = EV_CUBIC;
                e->from = current;
                e->w_from = cur_w;
                e->id_from = cur_id;
                e->ctrl1 = take();
                e->ctrl2 = take();
                current = take();
                cur_w = width_at(last_idx);
                cur_id = e->id_to = last_idx;
                e->w_to = cur_w;
                e->to = current;
                return true;
            case LYON_VERB_CLOSE:
                e->kind = EV_END;
                e->from = current;
                e->id_from = cur_id;
                e->id_to = first_id;
                (void)take();
                e->to = first;
                e->w_from = cur_w;
                e->w_to = first_w;
                e->close = true;
                return true;
            case LYON_VERB_END:
                e->kind = EV_END;
                e->from = current;
                e->id_from = cur_id;
                e->id_to = first_id;
                current = first;
                e->to = first;
                e->w_from = cur_w;
                e->w_to = first_w;
                cur_w = first_w;
                cur_id = first_id;
                e->close = false;
                return true;
            default:
                bad = true;
                return false;
        }
    }
};

// --------------------------------------------------------------------------------------------
// Output: BuffersBuilder over VertexBuffers<Point, u16|u32> (geometry_builder.rs:300-351,451-508).
// --------------------------------------------------------------------------------------------
static const uint32_t INVALID_ID = 0xFFFFFFFFu;
static const uint32_t NO_ENDPOINT = 0xFFFFFFFFu;

struct Src {  // VertexSource (lib.rs:282-291)
    uint32_t from = NO_ENDPOINT, to = NO_ENDPOINT;
    float t = 0.0f;
};
static inline Src endpoint_src(uint32_t id) { return Src{id, NO_ENDPOINT, 0.0f}; }
// The source of a point at parameter t of a curve between two endpoints: the end point itself
// at t == 1 (stroke.rs:1007-1016, 1045-1053).
static inline Src curve_src(uint32_t from, uint32_t to, float t) {
    return t == 1.0f ? endpoint_src(to) : Src{from, to, t};
}

struct Output {
    std::vector<float> vertices;     // x, y
    std::vector<uint32_t> indices;   // VertexId values; exported as u16 (truncating) or u32
    // With want_attributes, the stroke vertex attributes (StrokeVertex, stroke.rs:2667-2720):
    // normal x, normal y, advancement (f32 bits) and side, four words per vertex.
    bool want_attributes = false;
    std::vector<uint32_t> attributes;
    // With want_sources, each stroke vertex's VertexSource (lib.rs:282-291; StrokeVertex::source,
    // stroke.rs:2719-2722): from, to, t (f32 bits); `to` is NO_ENDPOINT for Endpoint { id: from }.
    bool want_sources = false;
    std::vector<uint32_t> sources;
    // A fill with want_sources records each vertex's sources (FillVertex::sources,
    // fill.rs:2172-2178, 2294-2337) instead: any number per vertex, three words each, with the
    // number per vertex in fill_source_counts.
    std::vector<uint32_t> fill_sources, fill_source_counts;
    size_t first_fill_source = 0;
    uint64_t max_index = 0xFFFFFFFEull;
    uint64_t vertex_offset = 0;
    size_t first_vertex = 0, first_index = 0;

    void begin_geometry() {
        first_vertex = vertices.size() / 2;
        first_index = indices.size();
        first_fill_source = fill_sources.size() / 3;
    }
    bool add_vertex(P p, uint32_t* id) {
        uint64_t i = vertices.size() / 2 + vertex_offset;
        if (i > max_index) return false;
        vertices.push_back(p.x);
        vertices.push_back(p.y);
        *id = (uint32_t)i;
        return true;
    }
    void add_triangle(uint32_t a, uint32_t b, uint32_t c) {
        indices.push_back(a);
        indices.push_back(b);
        indices.push_back(c);
    }
    void abort_geometry() {
        vertices.resize(first_vertex * 2);
        indices.resize(first_index);
        if (want_attributes) attributes.resize(first_vertex * 4);
        if (want_sources) sources.resize(first_vertex * 3);
        if (!fill_source_counts.empty() || !fill_sources.empty()) {
            fill_sources.resize(first_fill_source * 3);
            fill_source_counts.resize(first_vertex);
        }
    }
};

struct TessError {
    int code;
    int internal;
};

// --------------------------------------------------------------------------------------------
// Stroke tessellator, fixed line width (crates/tessellation/src/stroke.rs).
// --------------------------------------------------------------------------------------------
enum { SIDE_POSITIVE = 0, SIDE_NEGATIVE = 1 };

struct SidePoints {  // stroke.rs:300-307
    P prev, next;
    bool has_single;
    P single;
    uint32_t prev_vertex, next_vertex;
};

struct EndpointData {  // stroke.rs:309-342
    P position{0, 0};
    float half_width = NAN;
    float advancement = NAN;
    int line_join = LYON_JOIN_MITER;
    SidePoints side[2];
    bool fold[2] = {false, false};
    bool is_flattening_step = false;
    Src src;
    EndpointData() {
        for (int s = 0; s < 2; ++s) {
            side[s].prev = P{NAN, NAN};
            side[s].next = P{NAN, NAN};
            side[s].has_single = false;
            side[s].single = P{0, 0};
            side[s].prev_vertex = INVALID_ID;
            side[s].next_vertex = INVALID_ID;
        }
    }
};

struct PointBuffer {  // stroke.rs:2371-2457
    EndpointData points[3];
    size_t start = 0, count = 0;
    void push(const EndpointData& p) {
        if (count < 3) {
            points[count] = p;
            ++count;
            return;
        }
        points[start] = p;
        start += 1;
        if (start == 3) start = 0;
    }
    void replace_last(const EndpointData& p) {  // stroke.rs:2400-2406
        size_t idx = start;
        if (idx == 0) idx = count;
        points[idx - 1] = p;
    }
    void clear() { count = 0, start = 0; }
    EndpointData& get(size_t idx) { return points[(idx + start) % 3]; }
    EndpointData& last() { return get(count - 1); }
    EndpointData& second_last() { return points[(start + count - 2) % 3]; }
};

struct StrokeVertexData {  // stroke.rs:2656-2665
    P position_on_path{0, 0};
    float half_width = 0;
    P normal{0, 0};
    float advancement = 0;
    int side = SIDE_NEGATIVE;
    Src src;
};

// math_utils.rs:16-40
static P compute_normal(P v1, P v2) {
    const float epsilon = 1e-4f;
    P n1 = P{-v1.y, v1.x};
    P v12 = add(v1, v2);
    if (sqlen(v12) < epsilon) return P{0.0f, 0.0f};
    P tan = normalize(v12);
    P n = P{-tan.y, tan.x};
    float inv_len = dot(n, n1);
    if (fabsf(inv_len) < epsilon) return n1;
    return dvs(n, inv_len);
}

// geom line.rs:562-578 (Line::intersection with S = f64)
static bool line_intersection_f64(D p0, D v0, D p1, D v1, D* out) {
    double det = v0.x * v1.y - v0.y * v1.x;
    if (std::fabs(det) <= 1e-8) return false;
    double inv_det = 1.0 / det;
    D self_p2{p0.x + v0.x, p0.y + v0.y};
    D other_p2{p1.x + v1.x, p1.y + v1.y};
    double a = p0.x * self_p2.y - p0.y * self_p2.x;
    double b = p1.x * other_p2.y - p1.y * other_p2.x;
    out->x = (b * v0.x - a * v1.x) * inv_det;
    out->y = (b * v0.y - a * v1.y) * inv_det;
    return true;
}

// stroke.rs:2320-2322
static bool miter_limit_is_exceeded(P normal, float miter_limit) {
    return sqlen(normal) > miter_limit * miter_limit * 4.0f;
}

// stroke.rs:2279-2315
static void get_clip_intersections(P previous_normal, P next_normal, P normal, float clip_distance,
                                   P* i1, P* i2) {
    P clip_pt = mul(normalize(normal), clip_distance);
    P clip_vec = tangent(normal);
    P prev_pt = previous_normal, prev_vec = tangent(previous_normal);
    P next_pt = next_normal, next_vec = tangent(next_normal);
    D r;
    if (line_intersection_f64(dd(clip_pt), dd(clip_vec), dd(prev_pt), dd(prev_vec), &r)) {
        *i1 = P{(float)r.x, (float)r.y};
    } else {
        *i1 = normal;
    }
    if (line_intersection_f64(dd(clip_pt), dd(clip_vec), dd(next_pt), dd(next_vec), &r)) {
        *i2 = P{(float)r.x, (float)r.y};
    } else {
        *i2 = normal;
    }
}

// Arc subdivision depth (stroke.rs:2001-2004, 2487-2490). lyon recurses 2^depth - 1 times; a
// depth above this bound would mean more than a million vertices per arc (or, for a zero step,
// no end at all), so both the oracle and the GPU report LYON_ERR_UNSUPPORTED instead.
static const uint32_t MAX_ARC_DEPTH = 20;

// Arc step (stroke.rs:2749-2753, circle_flattening_step) is evaluated inline below:
// 2 * acos((radius - min(tol, radius)) / radius).
static uint32_t depth_of(float x) {
    float num_segments = ceilf(x);
    uint32_t d = sat_u32(roundf(log2f(num_segments)));
    if (d > MAX_ARC_DEPTH) throw TessError{LYON_ERR_UNSUPPORTED, 0};
    return d;
}

static inline float cr_acos(float x) { return (float)acos((double)x); }

// The arc's subdivision count is ceil(|diff| / step) (stroke.rs:2001-2004, 2487-2490). diff comes
// from fast_atan2 and angle_to, which round identically everywhere; step = 2 acos(..) comes from
// the platform's f32 libm, whose last bit varies between platforms, so the quotient can move by
// an ulp or two. Where it lies within 2e-6 (relative) of an integer, step is re-evaluated
// correctly rounded (f64 acos, one rounding; the GPU does the same), so both sides take the same
// ceil. A quotient within 1e-6 (relative) of an integer is a near tie: lyon itself may round it
// either way depending on its libm, so it is counted in `g_near_ties` (reported per path).
static inline float arc_step(float radius, float tol) {  // stroke.rs:2749-2753
    float t = fminf(tol, radius);
    return 2.0f * acosf((radius - t) / radius);
}
static inline float arc_quotient(float adiff, float radius, float tol, float step) {
    float x = adiff / step;
    if (!(fabsf(x - rintf(x)) <= 2e-6f * fmaxf(1.0f, x))) return x;
    float t = fminf(tol, radius);
    float xc = adiff / (2.0f * cr_acos((radius - t) / radius));
    if (rintf(xc) >= 1.0f && fabsf(xc - rintf(xc)) <= 1e-6f * fmaxf(1.0f, xc)) ++g_near_ties;
    return xc;
}
static inline float cr_cos(float x) { return (float)cos((double)x); }
static inline float cr_sin(float x) { return (float)sin((double)x); }
static inline float cr_asin(float x) { return (float)asin((double)x); }

struct Stroker {
    lyon_stroke_options options;
    int error = 0;
    Output* out;
    StrokeVertexData vertex;
    PointBuffer point_buffer;
    std::vector<EndpointData> firsts;
    float sub_path_start_advancement = 0.0f;
    float square_merge_threshold;
    bool may_need_empty_cap = false;
    bool vw = false;  // StrokeOptions::variable_line_width set

    // stroke.rs:591-631
    Stroker(const lyon_stroke_options& o, Output* output) : options(o), out(output) {
        out->begin_geometry();
        square_merge_threshold =
            fmaxf(fminf(o.tolerance * o.tolerance * 0.5f, o.line_width * o.line_width * 0.05f),
                  1e-8f);
        vertex.half_width = o.line_width * 0.5f;
        firsts.reserve(2);
    }

    void set_error(int code) {
        if (error == 0) error = code;
    }

    uint32_t add_stroke_vertex() {
        // StrokeVertex::position (stroke.rs:2673-2676)
        P pos = add(vertex.position_on_path, mul(vertex.normal, vertex.half_width));
        uint32_t id;
        if (!out->add_vertex(pos, &id)) throw TessError{LYON_ERR_TOO_MANY_VERTICES, 0};
        if (out->want_attributes) {
            uint32_t w[3];
            std::memcpy(&w[0], &vertex.normal.x, 4);
            std::memcpy(&w[1], &vertex.normal.y, 4);
            std::memcpy(&w[2], &vertex.advancement, 4);
            out->attributes.insert(out->attributes.end(), w, w + 3);
            out->attributes.push_back((uint32_t)vertex.side);
        }
        if (out->want_sources) {
            uint32_t tb;
            std::memcpy(&tb, &vertex.src.t, 4);
            out->sources.push_back(vertex.src.from);
            out->sources.push_back(vertex.src.to);
            out->sources.push_back(tb);
        }
        return id;
    }

    bool points_are_too_close(P p0, P p1) const {  // stroke.rs:1318-1320
        return sqlen(sub(p0, p1)) < square_merge_threshold;
    }

    // stroke.rs:1869-1904
    void add_edge_triangles(const EndpointData& p0, const EndpointData& p1) {
        uint32_t p0_neg = p0.side[SIDE_NEGATIVE].next_vertex;
        uint32_t p0_pos = p0.side[SIDE_POSITIVE].next_vertex;
        uint32_t p1_neg = p1.side[SIDE_NEGATIVE].prev_vertex;
        uint32_t p1_pos = p1.side[SIDE_POSITIVE].prev_vertex;
        if (p0.fold[SIDE_POSITIVE]) p0_neg = p0.side[SIDE_POSITIVE].prev_vertex;
        if (p0.fold[SIDE_NEGATIVE]) p0_pos = p0.side[SIDE_NEGATIVE].prev_vertex;
        if (p1.fold[SIDE_POSITIVE]) p1_neg = p1.side[SIDE_POSITIVE].next_vertex;
        if (p1.fold[SIDE_NEGATIVE]) p1_pos = p1.side[SIDE_NEGATIVE].next_vertex;
        if (p0_neg == p1_pos) return;
        if (p0_neg != p0_pos && p0_pos != p1_pos) out->add_triangle(p0_neg, p0_pos, p1_pos);
        if (p0_neg != p1_neg && p1_pos != p1_neg) out->add_triangle(p0_neg, p1_pos, p1_neg);
    }

    // stroke.rs:2612-2653
    void tessellate_arc(float a0, float a1, uint32_t va, uint32_t vb, uint32_t n) {
        if (n == 0) return;
        float mid_angle = (a0 + a1) * 0.5f;
        vertex.normal = P{cosf(mid_angle), sinf(mid_angle)};
        uint32_t vid = add_stroke_vertex();
        out->add_triangle(va, vid, vb);
        tessellate_arc(a0, mid_angle, va, vid, n - 1);
        tessellate_arc(mid_angle, a1, vid, vb, n - 1);
    }

    // stroke.rs:1968-2021
    void tessellate_round_join(EndpointData& join, int side) {
        P center = join.position;
        float radius = join.half_width;
        P start_normal = sub(join.side[side].prev, center);
        P end_normal = sub(join.side[side].next, center);
        uint32_t start_vertex = join.side[side].prev_vertex;
        uint32_t end_vertex = join.side[side].next_vertex;
        float angle_sign = side == SIDE_NEGATIVE ? 1.0f : -1.0f;
        float start_angle = angle_from_x_axis(start_normal);
        float diff = angle_to(start_angle, angle_from_x_axis(end_normal));
        if (diff * angle_sign < 0.0f) diff = angle_sign * (2.0f * PI_F - fabsf(diff));
        float end_angle = start_angle + diff;
        if (side == SIDE_NEGATIVE) {
            std::swap(start_angle, end_angle);
            std::swap(start_vertex, end_vertex);
        }
        float step = arc_step(radius, options.tolerance);
        uint32_t num_subdivisions =
            depth_of(arc_quotient(fabsf(diff), radius, options.tolerance, step));
        vertex.side = side;
        tessellate_arc(start_angle, end_angle, start_vertex, end_vertex, num_subdivisions);
    }

    // stroke.rs:1907-1965
    void tessellate_join(EndpointData& join) {
        bool side_needs_join[2] = {
            !join.side[SIDE_POSITIVE].has_single && !join.fold[SIDE_NEGATIVE],
            !join.side[SIDE_NEGATIVE].has_single && !join.fold[SIDE_POSITIVE],
        };
        if (!join.fold[SIDE_POSITIVE] && !join.fold[SIDE_NEGATIVE]) {
            const SidePoints& sp = join.side[SIDE_POSITIVE];
            const SidePoints& sn = join.side[SIDE_NEGATIVE];
            if (side_needs_join[0] && side_needs_join[1]) {
                out->add_triangle(sp.prev_vertex, sp.next_vertex, sn.next_vertex);
                out->add_triangle(sp.prev_vertex, sn.next_vertex, sn.prev_vertex);
            } else if (!side_needs_join[0] && side_needs_join[1]) {
                out->add_triangle(sn.prev_vertex, sp.prev_vertex, sn.next_vertex);
            } else if (side_needs_join[0] && !side_needs_join[1]) {
                out->add_triangle(sn.prev_vertex, sp.prev_vertex, sp.next_vertex);
            }
        }
        for (int side = 0; side < 2; ++side) {
            if (!side_needs_join[side]) continue;
            if (join.line_join == LYON_JOIN_ROUND) tessellate_round_join(join, side);
        }
    }

    // stroke.rs:2024-2055
    void add_join_base_vertices(EndpointData& join, int side) {
        vertex.side = side;
        if (join.side[side].has_single) {
            vertex.normal = dvs(sub(join.side[side].single, join.position), join.half_width);
            uint32_t v = add_stroke_vertex();
            join.side[side].prev_vertex = v;
            join.side[side].next_vertex = v;
        } else {
            vertex.normal = dvs(sub(join.side[side].prev, join.position), join.half_width);
            uint32_t pv = add_stroke_vertex();
            vertex.normal = dvs(sub(join.side[side].next, join.position), join.half_width);
            uint32_t nv = add_stroke_vertex();
            join.side[side].prev_vertex = pv;
            join.side[side].next_vertex = nv;
        }
    }

    // stroke.rs:1643-1733
    void compute_join_side_positions_fixed_width(const EndpointData& prev, EndpointData& join,
                                                 const EndpointData& next, float miter_limit) {
        P prev_tangent = sub(join.position, prev.position);
        P next_tangent = sub(next.position, join.position);
        float prev_length = length(prev_tangent);
        float next_length = length(next_tangent);
        prev_tangent = dvs(prev_tangent, prev_length);
        next_tangent = dvs(next_tangent, next_length);
        if (is_nan_f(join.advancement)) join.advancement = prev.advancement + prev_length;
        vertex.advancement = join.advancement;

        P normal = compute_normal(prev_tangent, next_tangent);
        int front_side;
        P front_normal;
        if (cross(prev_tangent, next_tangent) >= 0.0f) {
            front_side = SIDE_NEGATIVE;
            front_normal = neg(normal);
        } else {
            front_side = SIDE_POSITIVE;
            front_normal = normal;
        }
        int back_side = 1 - front_side;

        P extruded_normal = mul(front_normal, vertex.half_width);
        bool unclipped_miter =
            (join.line_join == LYON_JOIN_MITER || join.line_join == LYON_JOIN_MITER_CLIP) &&
            !miter_limit_is_exceeded(front_normal, miter_limit);

        bool fold = false;
        bool angle_is_sharp = dot(next_tangent, prev_tangent) < 0.0f;
        if (!unclipped_miter && angle_is_sharp) {
            float d_next = dot(extruded_normal, neg(next_tangent)) - next_length;
            float d_prev = dot(extruded_normal, prev_tangent) - prev_length;
            if (fminf(d_next, d_prev) > 0.0f || sqlen(normal) < 1e-5f) {
                join.fold[front_side] = true;
                fold = true;
            }
        }

        P n0 = mul(P{-prev_tangent.y, prev_tangent.x}, vertex.half_width);
        P n1 = mul(P{-next_tangent.y, next_tangent.x}, vertex.half_width);
        join.side[SIDE_POSITIVE].prev = add(join.position, n0);
        join.side[SIDE_POSITIVE].next = add(join.position, n1);
        join.side[SIDE_NEGATIVE].prev = sub(join.position, n0);
        join.side[SIDE_NEGATIVE].next = sub(join.position, n1);

        if (!fold) {
            P miter_pos[2] = {add(join.position, mul(normal, vertex.half_width)),
                              sub(join.position, mul(normal, vertex.half_width))};
            join.side[back_side].has_single = true;
            join.side[back_side].single = miter_pos[back_side];
            if (unclipped_miter) {
                join.side[front_side].has_single = true;
                join.side[front_side].single = miter_pos[front_side];
            } else if (join.line_join == LYON_JOIN_MITER_CLIP) {
                P a = sub(join.side[front_side].prev, join.position);
                P b = sub(join.side[front_side].next, join.position);
                P pn, nn;
                get_clip_intersections(a, b, front_normal, miter_limit * vertex.half_width, &pn,
                                       &nn);
                join.side[front_side].prev = add(join.position, pn);
                join.side[front_side].next = add(join.position, nn);
            }
        }
    }

    // stroke.rs:1743-1806. Returns true when the join is skipped.
    bool flattened_step(EndpointData& prev, EndpointData& join, EndpointData& next) {
        P prev_edge = sub(join.position, prev.position);
        float prev_length = length(prev_edge);
        P prev_tangent = dvs(prev_edge, prev_length);
        P next_edge = sub(next.position, join.position);
        float next_length = length(next_edge);
        P next_tangent = dvs(next_edge, next_length);
        P normal = compute_normal(prev_tangent, next_tangent);
        if (is_nan_f(join.advancement)) join.advancement = prev.advancement + prev_length;
        if (is_nan_f(next.advancement)) next.advancement = join.advancement + next_length;
        vertex.advancement = join.advancement;

        P p0 = add(join.position, mul(normal, vertex.half_width));
        join.side[SIDE_POSITIVE].prev = p0;
        join.side[SIDE_POSITIVE].next = p0;
        join.side[SIDE_POSITIVE].has_single = true;
        join.side[SIDE_POSITIVE].single = p0;
        P p1 = sub(join.position, mul(normal, vertex.half_width));
        join.side[SIDE_NEGATIVE].prev = p1;
        join.side[SIDE_NEGATIVE].next = p1;
        join.side[SIDE_NEGATIVE].has_single = true;
        join.side[SIDE_NEGATIVE].single = p1;

        P v0 = sub(p0, prev.side[SIDE_POSITIVE].next);
        P v1 = sub(p1, prev.side[SIDE_NEGATIVE].next);
        if (dot(prev_edge, v0) < 0.0f && dot(prev_edge, v1) < 0.0f) return true;

        vertex.normal = normal;
        vertex.side = SIDE_POSITIVE;
        uint32_t pos_vertex = add_stroke_vertex();
        vertex.normal = neg(normal);
        vertex.side = SIDE_NEGATIVE;
        uint32_t neg_vertex = add_stroke_vertex();
        join.side[SIDE_POSITIVE].prev_vertex = pos_vertex;
        join.side[SIDE_POSITIVE].next_vertex = pos_vertex;
        join.side[SIDE_NEGATIVE].prev_vertex = neg_vertex;
        join.side[SIDE_NEGATIVE].next_vertex = neg_vertex;
        return false;
    }

    // stroke.rs:1521-1632
    bool fixed_width_step_impl(EndpointData next) {
        size_t count = point_buffer.count;
        if (count > 0) {
            if (points_are_too_close(point_buffer.last().position, next.position)) {
                if (count == 1) may_need_empty_cap = true;
                return false;
            }
            if (count == 1) {
                EndpointData& first = point_buffer.last();
                P edge = sub(next.position, first.position);
                float len = length(edge);
                if (is_nan_f(next.advancement)) next.advancement = first.advancement + len;
                P tan = dvs(edge, len);
                P n = mul(P{-tan.y, tan.x}, next.half_width);
                first.side[SIDE_POSITIVE].next = add(first.position, n);
                first.side[SIDE_NEGATIVE].next = sub(first.position, n);
            }
        }
        if (count > 1) {
            EndpointData& prev = point_buffer.second_last();
            EndpointData& join = point_buffer.last();
            vertex.position_on_path = join.position;
            vertex.half_width = join.half_width;
            vertex.src = join.src;
            bool fast_path = false;
            if (join.is_flattening_step) {
                P v0 = sub(join.position, prev.position);
                P v1 = sub(next.position, join.position);
                fast_path = dot(v0, v1) > 0.0f;
            }
            if (fast_path) {
                join.line_join = LYON_JOIN_MITER;
                (void)flattened_step(prev, join, next);
            } else {
                compute_join_side_positions_fixed_width(prev, join, next, options.miter_limit);
                add_join_base_vertices(join, SIDE_NEGATIVE);
                add_join_base_vertices(join, SIDE_POSITIVE);
            }
            if (count > 2) add_edge_triangles(prev, join);
            tessellate_join(join);
            if (count == 2) {
                firsts.push_back(prev);
                firsts.push_back(join);
            }
        }
        point_buffer.push(next);
        return true;
    }

    void fixed_width_step(const EndpointData& next) {  // stroke.rs:1626-1631
        try {
            fixed_width_step_impl(next);
        } catch (const TessError& e) {
            set_error(e.code);
        }
    }

    // ---- Variable line width (StrokeOptions::variable_line_width) --------------------------
    // The edge's angle is euclid's fast_atan2 (exact f32 arithmetic); the attachment angles'
    // asin/cos/sin come from the platform's f32 libm in lyon, whose last bit varies between
    // platforms. Here (and on the GPU) those are evaluated in f64 and rounded once, so both sides
    // agree bit for bit.

    // stroke.rs:1842-1866
    static void compute_side_attachment_positions(EndpointData& p0, EndpointData& p1,
                                                  float edge_angle, float vwidth_angle,
                                                  int side) {
        float nl = side == SIDE_NEGATIVE ? -1.0f : 1.0f;
        float normal_angle = edge_angle + nl * (PI_F * 0.5f + vwidth_angle);
        P normal = P{cr_cos(normal_angle), cr_sin(normal_angle)};
        p0.side[side].next = add(p0.position, mul(normal, p0.half_width));
        p1.side[side].prev = add(p1.position, mul(normal, p1.half_width));
    }

    // stroke.rs:1808-1840
    static void compute_edge_attachment_positions(EndpointData& p0, EndpointData& p1) {
        P edge = sub(p1.position, p0.position);
        float d = length(edge);
        float edge_angle = angle_from_x_axis(edge);  // stroke.rs:1812
        float sin_vwidth_angle = (p1.half_width - p0.half_width) / d;
        float vwidth_angle = cr_asin(sin_vwidth_angle);
        if (is_nan_f(vwidth_angle)) vwidth_angle = 0.0f;
        compute_side_attachment_positions(p0, p1, edge_angle, vwidth_angle, SIDE_POSITIVE);
        compute_side_attachment_positions(p0, p1, edge_angle, vwidth_angle, SIDE_NEGATIVE);
        if (is_nan_f(p1.advancement)) p1.advancement = p0.advancement + d;
    }

    // stroke.rs:2060-2128
    static void compute_join_side_positions_vw(const EndpointData& prev, EndpointData& join,
                                               const EndpointData& next, float miter_limit,
                                               int side) {
        float sign = side == SIDE_NEGATIVE ? -1.0f : 1.0f;
        P v0 = normalize(sub(join.side[side].prev, prev.side[side].next));
        P v1 = normalize(sub(next.side[side].prev, join.side[side].next));
        bool inward = cross(v0, v1) * sign > 0.0f;
        bool forward = dot(v0, v1) > 0.0f;
        P normal = mul(compute_normal(v0, v1), sign);
        P path_v0 = normalize(sub(join.position, prev.position));
        P path_v1 = normalize(sub(next.position, join.position));
        bool normal_same_side = dot(add(v0, v1), add(path_v0, path_v1)) >= 0.0f;
        bool angle_is_sharp = inward && !forward && normal_same_side;
        if (angle_is_sharp) {
            P extruded_normal = mul(normal, join.half_width);
            float prev_length = join.advancement - prev.advancement;
            float next_length = next.advancement - join.advancement;
            float d_next = dot(extruded_normal, v1) - next_length;
            float d_prev = dot(extruded_normal, neg(v0)) - prev_length;
            if (fminf(d_next, d_prev) > 0.0f || sqlen(normal) < 1e-5f) join.fold[side] = true;
        }
        bool concave = inward && normal_same_side && !join.fold[side];
        if (concave || ((join.line_join == LYON_JOIN_MITER || join.line_join == LYON_JOIN_MITER_CLIP) &&
                        !miter_limit_is_exceeded(normal, miter_limit))) {
            join.side[side].has_single = true;
            join.side[side].single = add(join.position, mul(normal, join.half_width));
        } else if (join.line_join == LYON_JOIN_MITER_CLIP) {
            P n0 = sub(join.side[side].prev, join.position);
            P n1 = sub(join.side[side].next, join.position);
            P pn, nn;
            get_clip_intersections(n0, n1, normal, miter_limit * join.half_width, &pn, &nn);
            join.side[side].prev = add(join.position, pn);
            join.side[side].next = add(join.position, nn);
        }
    }

    // stroke.rs:1380-1512 (step_impl)
    bool step_vw_impl(EndpointData next) {
        size_t count = point_buffer.count;
        if (count > 0 && points_are_too_close(point_buffer.last().position, next.position)) {
            if (count == 1) may_need_empty_cap = true;
            return false;
        }
        if (count > 0) {
            EndpointData& join = point_buffer.last();
            if (!join.is_flattening_step || !next.is_flattening_step)
                compute_edge_attachment_positions(join, next);
        }
        bool skip = false;
        if (count > 1) {
            EndpointData& prev = point_buffer.second_last();
            EndpointData& join = point_buffer.last();
            vertex.position_on_path = join.position;
            vertex.half_width = join.half_width;
            vertex.advancement = join.advancement;
            vertex.src = join.src;
            bool fast_path = false;
            if (join.is_flattening_step) {
                P v0 = sub(join.position, prev.position);
                P v1 = sub(next.position, join.position);
                fast_path = dot(v0, v1) > 0.0f;
            }
            if (fast_path) {
                join.line_join = LYON_JOIN_MITER;
                skip = flattened_step(prev, join, next);
            } else {
                compute_join_side_positions_vw(prev, join, next, options.miter_limit,
                                               SIDE_POSITIVE);
                compute_join_side_positions_vw(prev, join, next, options.miter_limit,
                                               SIDE_NEGATIVE);
                // Prevent folding when the other side is concave.
                if (join.side[SIDE_POSITIVE].has_single) join.fold[SIDE_NEGATIVE] = false;
                if (join.side[SIDE_NEGATIVE].has_single) join.fold[SIDE_POSITIVE] = false;
                add_join_base_vertices(join, SIDE_NEGATIVE);
                add_join_base_vertices(join, SIDE_POSITIVE);
            }
            if (!skip) {
                if (count > 2) add_edge_triangles(prev, join);
                tessellate_join(join);
                if (count == 2) {
                    firsts.push_back(prev);
                    firsts.push_back(join);
                }
            }
        }
        if (skip) {
            point_buffer.replace_last(next);
        } else {
            point_buffer.push(next);
        }
        return true;
    }

    // The step of the active mode: fixed width (stroke.rs:1521-1632) or variable.
    bool step_impl(const EndpointData& next) {
        return vw ? step_vw_impl(next) : fixed_width_step_impl(next);
    }

    void step(const EndpointData& next) {  // stroke.rs:1515-1519
        try {
            step_impl(next);
        } catch (const TessError& e) {
            set_error(e.code);
        }
    }

    // Events of tessellate_with_ids_vw (stroke.rs:654-767): the half width of an endpoint is
    // line_width x its factor x 0.5; along a curve the width is interpolated linearly in t
    // (stroke.rs:996-1067, with flatten_quad's t mapping, stroke.rs:2755-2779).
    void begin_vw(P position, float w, Src src) {
        may_need_empty_cap = false;
        EndpointData d = make_point(position);
        d.half_width = options.line_width * w * 0.5f;
        d.advancement = sub_path_start_advancement;
        d.src = src;
        step(d);
    }
    void line_to_vw(P to, float w, Src src) {
        EndpointData d = make_point(to);
        d.half_width = options.line_width * w * 0.5f;
        d.src = src;
        step(d);
    }
    void curve_point_vw(P position, float t, bool is_flattening_step, float start_width,
                        float end_width, Src src) {
        EndpointData d = make_point(position);
        d.half_width = (start_width * (1.0f - t) + end_width * t) * 0.5f;
        d.is_flattening_step = is_flattening_step;
        d.src = src;
        step(d);
    }
    // flatten_quad (stroke.rs:2755-2779): `cb(position, t, is_flattening_step)` with t on the
    // whole curve when it is split at a sharp turn.
    template <class F>
    static void flatten_quad(const Quad& curve, float tolerance, F&& cb) {
        float t_split;
        if (find_sharp_turn(curve, &t_split)) {
            Quad before, after;
            quad_split(curve, t_split, &before, &after);
            quad_flatten_with_t(before, tolerance, [&](P, P to, float, float t1) {
                cb(to, t1 * t_split, t1 != 1.0f);
            });
            quad_flatten_with_t(after, tolerance, [&](P, P to, float, float t1) {
                cb(to, t_split + t1 * (1.0f - t_split), t1 != 1.0f);
            });
        } else {
            quad_flatten_with_t(curve, tolerance,
                                [&](P, P to, float, float t1) { cb(to, t1, t1 != 1.0f); });
        }
    }
    void quadratic_bezier_to_vw(const Quad& curve, float w0, float w1, uint32_t from_id,
                                uint32_t to_id) {
        float sw = options.line_width * w0, ew = options.line_width * w1;
        flatten_quad(curve, options.tolerance, [&](P to, float t, bool flat) {
            curve_point_vw(to, t, flat, sw, ew, curve_src(from_id, to_id, t));
        });
    }
    void cubic_bezier_to_vw(const Cubic& curve, float w0, float w1, uint32_t from_id,
                            uint32_t to_id) {
        float sw = options.line_width * w0, ew = options.line_width * w1;
        cubic_flatten_with_t(curve, options.tolerance, [&](P, P to, float, float t1) {
            curve_point_vw(to, t1, t1 != 1.0f, sw, ew, curve_src(from_id, to_id, t1));
        });
    }

    EndpointData make_point(P position) const {
        EndpointData d;
        d.position = position;
        d.half_width = options.line_width * 0.5f;
        d.line_join = options.line_join;
        return d;
    }

    void begin_fw(P position, Src src) {  // stroke.rs:1069-1087
        may_need_empty_cap = false;
        EndpointData d = make_point(position);
        d.advancement = sub_path_start_advancement;
        d.src = src;
        fixed_width_step(d);
    }

    void line_to_fw(P to, Src src) {  // stroke.rs:1089-1106
        EndpointData d = make_point(to);
        d.src = src;
        fixed_width_step(d);
    }

    // stroke.rs:3178-3212
    static bool find_sharp_turn(const Quad& curve, float* t_out) {
        P baseline = sub(curve.to, curve.from);
        P v = sub(curve.ctrl, curve.from);
        P n = P{-baseline.y, baseline.x};
        float v_dot_b = dot(v, baseline);
        float v_dot_n = dot(v, n);
        P long_axis;
        if ((v_dot_b >= 0.0f && v_dot_b <= dot(baseline, baseline)) ||
            fabsf(v_dot_n) * 2.0f >= fabsf(v_dot_b)) {
            if (sqlen(baseline) * 30.0f > sqlen(v)) return false;
            long_axis = v;
        } else {
            long_axis = baseline;
        }
        // Rotation2D::new(-long_axis.angle_from_x_axis()): the angle is euclid's fast_atan2
        // (exact f32 arithmetic); its sin/cos are evaluated in f64 and rounded once, the
        // correctly rounded f32 values, which the GPU reproduces (lyon takes them from the
        // platform's f32 libm, within an ulp of these). The split point feeds segment counts,
        // whose near ties are counted.
        float angle = -angle_from_x_axis(long_axis);
        float s = cr_sin(angle), c = cr_cos(angle);
        Quad rotated;
        rotated.from = P{0.0f, 0.0f};
        rotated.ctrl = P{v.x * c - v.y * s, v.x * s + v.y * c};
        rotated.to = P{baseline.x * c - baseline.y * s, baseline.x * s + baseline.y * c};
        return quad_local_x_extremum_t(rotated, t_out);
    }

    void flattened_point(P position, bool is_flattening_step, Src src) {
        EndpointData d = make_point(position);
        d.is_flattening_step = is_flattening_step;
        d.src = src;
        fixed_width_step(d);
    }

    // stroke.rs:1108-1143 and 2755-2779 (flatten_quad)
    void quadratic_bezier_to_fw(const Quad& curve, uint32_t from_id, uint32_t to_id) {
        flatten_quad(curve, options.tolerance, [&](P to, float t, bool flat) {
            flattened_point(to, flat, curve_src(from_id, to_id, t));
        });
    }

    // stroke.rs:1145-1177
    void cubic_bezier_to_fw(const Cubic& curve, uint32_t from_id, uint32_t to_id) {
        cubic_flatten_with_t(curve, options.tolerance, [&](P, P to, float, float t1) {
            flattened_point(to, t1 != 1.0f, curve_src(from_id, to_id, t1));
        });
    }

    // stroke.rs:2459-2524
    void tessellate_round_cap(P center, float radius, P start_normal, uint32_t start_vertex,
                              uint32_t end_vertex, P edge_normal, bool is_start) {
        if (radius < options.tolerance) return;
        int first_side = (is_start ^ (cross(edge_normal, start_normal) >= 0.0f)) ? SIDE_POSITIVE
                                                                                : SIDE_NEGATIVE;
        float start_angle = angle_from_x_axis(start_normal);
        float diff = angle_to(start_angle, angle_from_x_axis(edge_normal));
        float mid_angle = start_angle + diff;
        float end_angle = mid_angle + diff;
        float step = arc_step(radius, options.tolerance);
        uint32_t num_subdivisions =
            depth_of(arc_quotient(fabsf(diff), radius, options.tolerance, step));
        vertex.position_on_path = center;
        vertex.half_width = radius;
        vertex.side = first_side;
        vertex.normal = normalize(edge_normal);
        uint32_t mid_vertex = add_stroke_vertex();
        out->add_triangle(start_vertex, mid_vertex, end_vertex);
        tessellate_arc(start_angle, mid_angle, start_vertex, mid_vertex, num_subdivisions);
        vertex.side = 1 - first_side;
        tessellate_arc(mid_angle, end_angle, mid_vertex, end_vertex, num_subdivisions);
    }

    // stroke.rs:2526-2560
    void tessellate_empty_square_cap(P position) {
        vertex.position_on_path = position;
        vertex.normal = P{1.0f, 1.0f};
        vertex.side = SIDE_NEGATIVE;
        uint32_t a = add_stroke_vertex();
        vertex.normal = P{1.0f, -1.0f};
        vertex.side = SIDE_POSITIVE;
        uint32_t b = add_stroke_vertex();
        vertex.normal = P{-1.0f, -1.0f};
        vertex.side = SIDE_POSITIVE;
        uint32_t c = add_stroke_vertex();
        vertex.normal = P{-1.0f, 1.0f};
        vertex.side = SIDE_NEGATIVE;
        uint32_t d = add_stroke_vertex();
        out->add_triangle(a, b, c);
        out->add_triangle(a, c, d);
    }

    // stroke.rs:2562-2609
    void tessellate_empty_round_cap(P center) {
        float radius = vertex.half_width;
        vertex.position_on_path = center;
        vertex.normal = P{-1.0f, 0.0f};
        vertex.side = SIDE_POSITIVE;
        uint32_t left_id = add_stroke_vertex();
        vertex.normal = P{1.0f, 0.0f};
        vertex.side = SIDE_NEGATIVE;
        uint32_t right_id = add_stroke_vertex();
        tessellate_round_cap(center, radius, P{-1.0f, 0.0f}, left_id, right_id, P{0.0f, 1.0f},
                             true);
        tessellate_round_cap(center, radius, P{1.0f, 0.0f}, right_id, left_id, P{0.0f, -1.0f},
                             false);
    }

    // stroke.rs:1282-1316
    void tessellate_empty_cap() {
        EndpointData& point = point_buffer.get(0);
        vertex.advancement = point.advancement;
        vertex.half_width = point.half_width;
        vertex.src = point.src;
        if (options.start_cap == LYON_CAP_SQUARE) {
            tessellate_empty_square_cap(point.position);
        } else if (options.start_cap == LYON_CAP_ROUND) {
            tessellate_empty_round_cap(point.position);
        }
    }

    // stroke.rs:2130-2206
    void tessellate_last_edge(const EndpointData& p0, EndpointData& p1, bool is_first_edge) {
        P v = sub(p1.position, p0.position);
        p1.advancement = p0.advancement + length(v);
        vertex.position_on_path = p1.position;
        vertex.advancement = p1.advancement;
        vertex.half_width = p1.half_width;
        vertex.src = p1.src;
        for (int side = 0; side < 2; ++side) {
            P side_position = p1.side[side].prev;
            bool has_clip = options.end_cap == LYON_CAP_SQUARE || options.end_cap == LYON_CAP_BUTT;
            if (has_clip) {
                float clip = options.end_cap == LYON_CAP_SQUARE ? p1.half_width : 0.0f;
                P normal = normalize(sub(p1.position, p0.position));
                P clip_pt = add(p1.position, mul(normal, clip));
                P clip_vec = tangent(normal);
                P side_vec = sub(side_position, p0.side[side].next);
                D r;
                P intersection = p1.side[side].prev;
                if (line_intersection_f64(dd(clip_pt), dd(clip_vec), dd(side_position),
                                          dd(side_vec), &r)) {
                    intersection = P{(float)r.x, (float)r.y};
                }
                p1.side[side].prev = intersection;
            }
            vertex.side = side;
            vertex.normal = dvs(sub(p1.side[side].prev, p1.position), p1.half_width);
            p1.side[side].prev_vertex = add_stroke_vertex();
        }
        if (!is_first_edge) add_edge_triangles(p0, p1);
        if (options.end_cap == LYON_CAP_ROUND) {
            tessellate_round_cap(p1.position, p1.half_width,
                                 sub(p1.side[SIDE_POSITIVE].prev, p1.position),
                                 p1.side[SIDE_POSITIVE].prev_vertex,
                                 p1.side[SIDE_NEGATIVE].prev_vertex, v, false);
        }
    }

    // stroke.rs:2208-2276
    void tessellate_first_edge(EndpointData& first, const EndpointData& second) {
        vertex.position_on_path = first.position;
        vertex.advancement = first.advancement;
        vertex.half_width = first.half_width;
        vertex.src = first.src;
        for (int side = 0; side < 2; ++side) {
            P side_position = first.side[side].next;
            bool has_clip =
                options.start_cap == LYON_CAP_SQUARE || options.start_cap == LYON_CAP_BUTT;
            if (has_clip) {
                float clip = options.start_cap == LYON_CAP_SQUARE ? first.half_width : 0.0f;
                P normal = normalize(sub(first.position, second.position));
                P clip_pt = add(first.position, mul(normal, clip));
                P clip_vec = tangent(normal);
                P side_vec = sub(side_position, second.side[side].prev);
                D r;
                P intersection = first.side[side].next;
                if (line_intersection_f64(dd(clip_pt), dd(clip_vec), dd(side_position),
                                          dd(side_vec), &r)) {
                    intersection = P{(float)r.x, (float)r.y};
                }
                side_position = intersection;
            }
            vertex.side = side;
            vertex.normal = dvs(sub(side_position, first.position), first.half_width);
            first.side[side].next_vertex = add_stroke_vertex();
        }
        add_edge_triangles(first, second);
        if (options.start_cap == LYON_CAP_ROUND) {
            tessellate_round_cap(first.position, first.half_width,
                                 sub(first.side[SIDE_NEGATIVE].next, first.position),
                                 first.side[SIDE_NEGATIVE].next_vertex,
                                 first.side[SIDE_POSITIVE].next_vertex,
                                 sub(first.position, second.position), true);
        }
    }

    // stroke.rs:1322-1378
    void end_with_caps() {
        size_t count = point_buffer.count;
        if (may_need_empty_cap && count == 1) {
            tessellate_empty_cap();
            return;
        }
        if (count >= 2) {
            EndpointData p0 = point_buffer.second_last();
            EndpointData p1 = point_buffer.last();
            if (!vw) {
                // With a fixed width only the joins have side points so far (stroke.rs:1338-1346).
                P tan = normalize(sub(p1.position, p0.position));
                P n = mul(P{-tan.y, tan.x}, p1.half_width);
                p1.side[SIDE_POSITIVE].prev = add(p1.position, n);
                p1.side[SIDE_NEGATIVE].prev = sub(p1.position, n);
            }
            bool is_first = count == 2;
            tessellate_last_edge(p0, p1, is_first);
            sub_path_start_advancement = p1.advancement;
            if (count > 2) {
                p0 = firsts[0];
                p1 = firsts[1];
            }
            tessellate_first_edge(p0, p1);
        }
    }

    // stroke.rs:1206-1279
    void close() {
        if (point_buffer.count == 1) tessellate_empty_cap();
        if (point_buffer.count <= 2) return;
        EndpointData p = firsts[0];
        float advancement = p.advancement;
        p.advancement = NAN;
        bool segment_added = step_impl(p);
        if (!segment_added) point_buffer.last().position = p.position;
        if (firsts.size() >= 2) {
            EndpointData p2 = firsts[1];
            step_impl(p2);
            EndpointData& p0 = point_buffer.second_last();
            EndpointData& p1 = point_buffer.last();
            vertex.position_on_path = p0.position;
            vertex.half_width = p0.half_width;
            vertex.advancement = advancement;
            vertex.src = p0.src;
            for (int side = 0; side < 2; ++side) {
                vertex.side = side;
                if (p0.side[side].has_single) {
                    vertex.normal = dvs(sub(p0.side[side].single, p0.position), p0.half_width);
                } else {
                    vertex.normal = dvs(sub(p0.side[side].next, p0.position), p0.half_width);
                }
                p0.side[side].next_vertex = add_stroke_vertex();
            }
            add_edge_triangles(p0, p1);
        }
    }

    // stroke.rs:1179-1193
    void end(bool close_path) {
        may_need_empty_cap |= close_path && point_buffer.count == 1;
        try {
            if (close_path && point_buffer.count > 2) {
                close();
            } else {
                end_with_caps();
            }
        } catch (const TessError& e) {
            set_error(e.code);
        }
        point_buffer.clear();
        firsts.clear();
    }

    // stroke.rs:872-952 (tessellate_fw) + 1195-1204 (build)
    int tessellate(PathIter it) {
        Evt e;
        while (it.next(&e)) {
            switch (e.kind) {
                case EV_BEGIN:
                    if (vw) begin_vw(e.to, e.w_to, endpoint_src(e.id_to));
                    else begin_fw(e.to, endpoint_src(e.id_to));
                    break;
                case EV_LINE:
                    if (vw) line_to_vw(e.to, e.w_to, endpoint_src(e.id_to));
                    else line_to_fw(e.to, endpoint_src(e.id_to));
                    break;
                case EV_QUAD:
                    if (vw)
                        quadratic_bezier_to_vw(Quad{e.from, e.ctrl1, e.to}, e.w_from, e.w_to,
                                               e.id_from, e.id_to);
                    else
                        quadratic_bezier_to_fw(Quad{e.from, e.ctrl1, e.to}, e.id_from, e.id_to);
                    break;
                case EV_CUBIC:
                    if (vw)
                        cubic_bezier_to_vw(Cubic{e.from, e.ctrl1, e.ctrl2, e.to}, e.w_from,
                                           e.w_to, e.id_from, e.id_to);
                    else
                        cubic_bezier_to_fw(Cubic{e.from, e.ctrl1, e.ctrl2, e.to}, e.id_from,
                                           e.id_to);
                    break;
                case EV_END:
                    end(e.close);
                    break;
            }
            if (error) {
                out->abort_geometry();
                return error;
            }
        }
        if (it.bad) {
            out->abort_geometry();
            return LYON_ERR_INVALID_ARGUMENT;
        }
        return LYON_OK;
    }
};

// --------------------------------------------------------------------------------------------
// Fill: event queue (crates/tessellation/src/event_queue.rs).
// --------------------------------------------------------------------------------------------
static const uint32_t INVALID_EVENT = 0xFFFFFFFFu;

// fill.rs:2122-2151
static inline int compare_positions(P a, P b) {
    if (a.y > b.y) return 1;
    if (a.y < b.y) return -1;
    if (a.x > b.x) return 1;
    if (a.x < b.x) return -1;
    return 0;
}
static inline bool is_after(P a, P b) { return a.y > b.y || (a.y == b.y && a.x > b.x); }
static inline bool is_near(P a, P b) { return sqlen(sub(a, b)) < 0.000000001f; }

struct Event {
    uint32_t next_sibling, next_event;
    P position;
};
struct EdgeData {  // event_queue.rs:28-36
    P to;
    float range_start, range_end;
    int16_t winding;
    bool is_edge;
    uint32_t from_id = NO_ENDPOINT, to_id = NO_ENDPOINT;  // the source edge's endpoints
};

struct EventQueue {
    std::vector<Event> events;
    std::vector<EdgeData> edge_data;
    uint32_t first = INVALID_EVENT;

    void reset() {
        events.clear();
        edge_data.clear();
        first = INVALID_EVENT;
    }
    void push_unsorted(P position) {
        events.push_back(Event{INVALID_EVENT, INVALID_EVENT, position});
    }
    uint32_t next_id(uint32_t id) const { return events[id].next_event; }
    uint32_t next_sibling_id(uint32_t id) const { return events[id].next_sibling; }
    P position(uint32_t id) const { return events[id].position; }

    // event_queue.rs:252-274
    void insert_into_sorted_list(uint32_t idx, P position, uint32_t after) {
        uint32_t prev = after, current = after;
        while (current != INVALID_EVENT) {
            P pos = events[current].position;
            if (peq(pos, position)) {
                events[idx].next_sibling = events[current].next_sibling;
                events[current].next_sibling = idx;
                return;
            } else if (is_after(pos, position)) {
                events[prev].next_event = idx;
                events[idx].next_event = current;
                return;
            }
            prev = current;
            current = next_id(current);
        }
        events[prev].next_event = idx;
    }

    // event_queue.rs:188-213
    uint32_t insert_sorted(P position, const EdgeData& data, uint32_t after) {
        uint32_t idx = (uint32_t)events.size();
        events.push_back(Event{INVALID_EVENT, INVALID_EVENT, position});
        edge_data.push_back(data);
        insert_into_sorted_list(idx, position, after);
        return idx;
    }

    // event_queue.rs:215-230
    void insert_sibling(uint32_t sibling, P position, const EdgeData& data) {
        uint32_t idx = (uint32_t)events.size();
        uint32_t next_sibling = events[sibling].next_sibling;
        events.push_back(Event{next_sibling, INVALID_EVENT, position});
        edge_data.push_back(data);
        events[sibling].next_sibling = idx;
    }

    // event_queue.rs:232-250
    void vertex_event_sorted(P position, uint32_t endpoint_id, uint32_t after) {
        uint32_t idx = (uint32_t)events.size();
        push_unsorted(position);
        edge_data.push_back(EdgeData{P{NAN, NAN}, 0.0f, 0.0f, 0, false, endpoint_id, endpoint_id});
        insert_into_sorted_list(idx, position, after);
    }

    uint32_t find_last_sibling(uint32_t id) const {  // event_queue.rs:386-395
        uint32_t current_sibling = id;
        uint32_t next_sibling = next_sibling_id(id);
        while (next_sibling != INVALID_EVENT) {
            current_sibling = next_sibling;
            next_sibling = next_sibling_id(current_sibling);
        }
        return current_sibling;
    }

    // event_queue.rs:328-384
    uint32_t merge(uint32_t a, uint32_t b) {
        if (a == INVALID_EVENT) return b;
        if (b == INVALID_EVENT) return a;
        bool first_node = true;
        uint32_t sorted_head = INVALID_EVENT;
        uint32_t prev = INVALID_EVENT;
        for (;;) {
            if (a == INVALID_EVENT) {
                if (!first_node) events[prev].next_event = b;
                break;
            }
            if (b == INVALID_EVENT) {
                if (!first_node) events[prev].next_event = a;
                break;
            }
            uint32_t node;
            int c = compare_positions(events[a].position, events[b].position);
            if (c < 0) {
                node = a;
                a = events[a].next_event;
            } else if (c > 0) {
                node = b;
                b = events[b].next_event;
            } else {
                uint32_t a_sib = find_last_sibling(a);
                events[a_sib].next_sibling = b;
                b = events[b].next_event;
                continue;
            }
            if (first_node) {
                first_node = false;
                sorted_head = node;
            } else {
                events[prev].next_event = node;
            }
            prev = node;
        }
        if (sorted_head == INVALID_EVENT) sorted_head = a;
        return sorted_head;
    }

    // event_queue.rs:316-326
    uint32_t merge_sort(size_t start, size_t end) {
        size_t split = (start + end) / 2;
        if (split == start) return (uint32_t)start;
        uint32_t a_head = merge_sort(start, split);
        uint32_t b_head = merge_sort(split, end);
        return merge(a_head, b_head);
    }

    void sort() {  // event_queue.rs:301-310
        if (events.empty()) return;
        first = merge_sort(0, events.size());
    }
};

// event_queue.rs:441-905
struct EventQueueBuilder {
    P current{NAN, NAN}, prev{NAN, NAN}, second{NAN, NAN};
    uint32_t nth = 0;
    uint32_t prev_endpoint_id = NO_ENDPOINT;
    EventQueue* queue;
    float tolerance;

    void vertex_event(P at, uint32_t endpoint_id) {  // event_queue.rs:637-647
        queue->push_unsorted(at);
        queue->edge_data.push_back(
            EdgeData{P{NAN, NAN}, 0.0f, 0.0f, 0, false, endpoint_id, endpoint_id});
    }
    void vertex_event_on_curve(P at, float t, uint32_t from_id, uint32_t to_id) {  // :649-659
        queue->push_unsorted(at);
        queue->edge_data.push_back(EdgeData{P{NAN, NAN}, t, t, 0, false, from_id, to_id});
    }

    void end(P first, uint32_t first_id) {  // event_queue.rs:661-682
        if (nth == 0) return;
        line_segment(first, first_id, 0.0f, 1.0f);
        if (is_after(first, prev) && is_after(first, second)) vertex_event(first, first_id);
        prev_endpoint_id = first_id;
        nth = 0;
    }

    void begin(P to, uint32_t to_id) {  // event_queue.rs:684-691
        nth = 0;
        current = to;
        prev_endpoint_id = to_id;
    }

    void add_edge(P from, P to, int16_t winding, uint32_t from_id, uint32_t to_id, float t0,
                  float t1) {  // :693-726
        if (peq(from, to)) return;
        P evt_pos = from, evt_to = to;
        if (is_after(evt_pos, to)) {
            evt_to = evt_pos;
            evt_pos = to;
            std::swap(t0, t1);
            winding = (int16_t)(-winding);
        }
        queue->push_unsorted(evt_pos);
        queue->edge_data.push_back(EdgeData{evt_to, t0, t1, winding, true, from_id, to_id});
        nth += 1;
    }

    void line_segment(P to, uint32_t to_id, float t0, float t1) {  // :728-756
        P from = current;
        if (peq(from, to)) return;
        if (is_after(from, to) && nth > 0 && is_after(from, prev))
            vertex_event(from, prev_endpoint_id);
        if (nth == 0) second = to;
        add_edge(from, to, 1, prev_endpoint_id, to_id, t0, t1);
        prev = current;
        prev_endpoint_id = to_id;
        current = to;
    }

    // The t values of a swapped curve are those of the swapped (downward) segment while the ids
    // stay the original from and to, as in lyon.
    template <class FlattenFn>
    void curve_segment(P original_from, P original_to, uint32_t to_id, bool needs_swap,
                       FlattenFn&& flatten) {
        // Shared body of quadratic_bezier_segment / cubic_bezier_segment (:758-900).
        int16_t winding = needs_swap ? -1 : 1;
        P seg_from = needs_swap ? original_to : original_from;
        P prev_pt = seg_from;
        bool have_first = false;
        P first{0, 0};
        bool is_first_edge = nth == 0;
        flatten([&](P lf, P lt, float t0, float t1) {
            if (peq(lf, lt)) return;
            if (!have_first) {
                have_first = true;
                first = lt;
            } else if (is_after(lf, lt) && is_after(lf, prev_pt)) {
                vertex_event_on_curve(lf, t0, prev_endpoint_id, to_id);
            }
            add_edge(lf, lt, winding, prev_endpoint_id, to_id, t0, t1);
            prev_pt = lf;
        });
        if (have_first) {
            P second_pt, previous;
            if (needs_swap) {
                second_pt = prev_pt;
                previous = first;
            } else {
                second_pt = first;
                previous = prev_pt;
            }
            if (is_first_edge) {
                second = second_pt;
            } else if (is_after(original_from, prev) && is_after(original_from, second_pt)) {
                vertex_event(original_from, prev_endpoint_id);
            }
            prev = previous;
            current = original_to;
            prev_endpoint_id = to_id;
        }
    }

    void quadratic_bezier_segment(P ctrl, P to, uint32_t to_id) {  // :758-826
        Quad original{current, ctrl, to};
        bool needs_swap = is_after(original.from, original.to);
        Quad segment = original;
        if (needs_swap) std::swap(segment.from, segment.to);
        curve_segment(original.from, original.to, to_id, needs_swap, [&](auto&& cb) {
            quad_flatten_with_t(segment, tolerance, cb);
        });
    }

    void cubic_bezier_segment(P ctrl1, P ctrl2, P to, uint32_t to_id) {  // :828-900
        Cubic original{current, ctrl1, ctrl2, to};
        bool needs_swap = is_after(original.from, original.to);
        Cubic segment = original;
        if (needs_swap) {
            std::swap(segment.from, segment.to);
            std::swap(segment.ctrl1, segment.ctrl2);
        }
        curve_segment(original.from, original.to, to_id, needs_swap, [&](auto&& cb) {
            cubic_flatten_with_t(segment, tolerance, cb);
        });
    }
};

// --------------------------------------------------------------------------------------------
// Monotone tessellators (crates/tessellation/src/monotone.rs).
// --------------------------------------------------------------------------------------------
enum FSide { LEFT = 0, RIGHT = 1 };

struct MonotoneVertex {
    P pos;
    uint32_t id;
    int side;
};

struct BasicMonotone {  // monotone.rs:9-139
    std::vector<MonotoneVertex> stack;
    MonotoneVertex previous{P{0, 0}, 0, LEFT};
    std::vector<uint32_t> triangles;  // triples

    void begin(P pos, uint32_t id) {
        MonotoneVertex first{pos, id, LEFT};
        previous = first;
        triangles.clear();
        stack.clear();
        stack.push_back(first);
    }
    void push_triangle_ids(uint32_t a, uint32_t b, uint32_t c) {
        triangles.push_back(a);
        triangles.push_back(b);
        triangles.push_back(c);
    }
    void monotone_vertex(MonotoneVertex current) {
        bool changed_side = current.side != previous.side;
        if (changed_side) {
            for (size_t i = 0; i + 1 < stack.size(); ++i) {
                MonotoneVertex a = stack[i], b = stack[i + 1];
                bool winding = cross(sub(a.pos, b.pos), sub(current.pos, b.pos)) >= 0.0f;
                if (!winding) std::swap(a, b);
                push_triangle_ids(a.id, b.id, current.id);
            }
            stack.clear();
            stack.push_back(previous);
        } else {
            bool have_last = !stack.empty();
            MonotoneVertex last_popped{};
            if (have_last) {
                last_popped = stack.back();
                stack.pop_back();
            }
            while (!stack.empty()) {
                MonotoneVertex a = last_popped;
                MonotoneVertex b = stack.back();
                if (current.side == RIGHT) std::swap(a, b);
                float c = cross(sub(current.pos, b.pos), sub(a.pos, b.pos));
                if (c >= 0.0f) {
                    push_triangle_ids(b.id, a.id, current.id);
                    have_last = !stack.empty();
                    if (have_last) {
                        last_popped = stack.back();
                        stack.pop_back();
                    }
                } else {
                    break;
                }
            }
            if (have_last) stack.push_back(last_popped);
        }
        stack.push_back(current);
        previous = current;
    }
    void vertex(P pos, uint32_t id, int side) { monotone_vertex(MonotoneVertex{pos, id, side}); }
    void end(P pos, uint32_t id) {
        int side = previous.side == LEFT ? RIGHT : LEFT;
        vertex(pos, id, side);
        stack.clear();
    }
    void flush(Output* out) {
        for (size_t i = 0; i < triangles.size(); i += 3) {
            out->add_triangle(triangles[i], triangles[i + 1], triangles[i + 2]);
        }
        triangles.clear();
    }
};

struct SideEvents {  // monotone.rs:189-210
    P reference_point{0, 0};
    float conservative_reference_x = 0.0f;
    std::vector<uint32_t> events;
    P prev{0, 0};
    MonotoneVertex last{P{0, 0}, 0, LEFT};
    void push(MonotoneVertex v) {
        events.push_back(v.id);
        prev = last.pos;
        last = v;
    }
};

// monotone.rs:362-404
static bool flush_side(SideEvents& side, int s, BasicMonotone& tess, MonotoneVertex* out) {
    size_t len = side.events.size();
    if (len < 2) return false;
    size_t step = 1;
    while (step * 2 < len) {
        size_t last_index = 0;
        size_t imax = (len - 1) / (2 * step);
        for (size_t i = 0; i < imax; ++i) {
            size_t a = i * 2 * step;
            size_t b = a + step;
            last_index = b + step;
            if (s == RIGHT) std::swap(a, b);
            tess.push_triangle_ids(side.events[a], side.events[b], side.events[last_index]);
        }
        if (last_index + step < len) {
            size_t b = last_index;
            size_t c = last_index + step;
            if (s == RIGHT) std::swap(b, c);
            tess.push_triangle_ids(side.events[0], side.events[b], side.events[c]);
        }
        step *= 2;
    }
    side.events.clear();
    side.push(side.last);
    side.reference_point = side.last.pos;
    *out = side.last;
    return true;
}

struct AdvancedMonotone {  // monotone.rs:212-359
    BasicMonotone tess;
    SideEvents left, right;
    bool flushing = false;

    void begin(P pos, uint32_t id) {
        tess.begin(pos, id);
        left.reference_point = pos;
        left.conservative_reference_x = pos.x;
        right.reference_point = pos;
        right.conservative_reference_x = pos.x;
        left.prev = pos;
        right.prev = pos;
        flushing = false;
        left.events.clear();
        right.events.clear();
        left.push(MonotoneVertex{pos, id, LEFT});
        right.push(MonotoneVertex{pos, id, RIGHT});
    }

    void vertex(P pos, uint32_t id, int side) {
        if (side == LEFT) {
            left.reference_point.x = fmaxf(left.reference_point.x, pos.x);
            left.conservative_reference_x =
                fmaxf(left.conservative_reference_x, left.reference_point.x);
        } else {
            right.reference_point.x = fminf(right.reference_point.x, pos.x);
            right.conservative_reference_x =
                fminf(right.conservative_reference_x, right.reference_point.x);
        }
        float dx = right.conservative_reference_x - left.conservative_reference_x;
        SideEvents& side_ev = side == LEFT ? left : right;
        SideEvents& opposite_side_ev = side == LEFT ? right : left;
        float dy = pos.y - side_ev.reference_point.y;
        bool sides_are_close = dx < dy * 0.1f;
        size_t len = side_ev.events.size();
        bool outward_turn = false;
        if (!sides_are_close && len >= 2) {
            float sign = side == LEFT ? 1.0f : -1.0f;
            P prev = side_ev.prev;
            P last = side_ev.last.pos;
            outward_turn = cross(sub(prev, last), sub(pos, last)) * sign < 0.0f;
        }
        if (outward_turn || sides_are_close) {
            bool must_flush_opposite_side = is_after(side_ev.last.pos, opposite_side_ev.last.pos);
            MonotoneVertex v;
            if (must_flush_opposite_side) {
                if (flush_side(opposite_side_ev, side == LEFT ? RIGHT : LEFT, tess, &v)) {
                    tess.monotone_vertex(v);
                    side_ev.conservative_reference_x = side_ev.reference_point.x;
                }
            }
            if (flush_side(side_ev, side, tess, &v)) {
                tess.monotone_vertex(v);
                opposite_side_ev.conservative_reference_x = opposite_side_ev.reference_point.x;
            }
        }
        side_ev.push(MonotoneVertex{pos, id, side});
    }

    void end(P pos, uint32_t id) {
        MonotoneVertex a, b;
        bool ha = flush_side(left, LEFT, tess, &a);
        bool hb = flush_side(right, RIGHT, tess, &b);
        if (ha && !hb) {
            tess.monotone_vertex(a);
        } else if (!ha && hb) {
            tess.monotone_vertex(b);
        } else if (ha && hb) {
            MonotoneVertex v1 = a, v2 = b;
            if (is_after(v1.pos, v2.pos)) std::swap(v1, v2);
            tess.monotone_vertex(v1);
            tess.monotone_vertex(v2);
        }
        tess.end(pos, id);
    }

    void flush(Output* out) { tess.flush(out); }
};

// --------------------------------------------------------------------------------------------
// Fill sweep line (crates/tessellation/src/fill.rs).
// --------------------------------------------------------------------------------------------
static inline float fmax_lyon(float a, float b) { return a > b ? a : b; }  // fill.rs:55-62

static inline float slope(P v) { return v.x / fmaxf(v.y, FLT_MIN); }  // fill.rs:64-66

static inline bool fill_rule_is_in(int rule, int16_t w) {  // path/src/lib.rs:267-281
    if (rule == LYON_FILL_EVEN_ODD) return (w % 2) != 0;
    return w != 0;
}

struct WindingState {  // fill.rs:88-113
    int32_t span_index = -1;
    int16_t number = 0;
    bool is_in = false;
    void update(int rule, int16_t w) {
        number = (int16_t)(number + w);
        is_in = fill_rule_is_in(rule, number);
        if (is_in) span_index += 1;
    }
};

struct ActiveEdge {  // fill.rs:153-170
    P from, to;
    int16_t winding;
    bool is_merge;
    uint32_t from_id;
    uint32_t src_edge;
    float range_end;
    float min_x() const { return fminf(from.x, to.x); }
    float max_x() const { return fmax_lyon(from.x, to.x); }
    // fill.rs:185-200 with geom line.rs:56-71
    float solve_x_for_y(float y) const {
        float dy = to.y - from.y;
        float t = dy == 0.0f ? 0.0f : (y - from.y) / dy;
        float x = from.x * (1.0f - t) + to.x * t;
        return fminf(fmaxf(x, min_x()), max_x());
    }
};

struct PendingEdge {  // fill.rs:304-312
    P to;
    float sort_key;
    uint32_t src_edge;
    int16_t winding;
    float range_end;
};

struct Span {
    std::unique_ptr<AdvancedMonotone> tess;
};

struct ActiveEdgeScan {  // fill.rs:115-151
    std::vector<std::pair<int32_t, int>> vertex_events;
    std::vector<size_t> edges_to_split;
    std::vector<int32_t> spans_to_end;
    bool merge_event = false, split_event = false, merge_split_event = false;
    size_t above_start = 0, above_end = 0;
    WindingState winding_before_point;
    void reset() {
        vertex_events.clear();
        edges_to_split.clear();
        spans_to_end.clear();
        merge_event = split_event = merge_split_event = false;
        above_start = above_end = 0;
        winding_before_point = WindingState();
    }
};

// fill.rs:2339-2347
static float remap_t_in_range(float val, float start, float end) {
    if (end > start) {
        float d = end - start;
        return start + val * d;
    }
    float d = start - end;
    return end + (1.0f - val) * d;
}

// geom line.rs:217-253 with S = f64
static bool segment_intersection_t(D sf, D st, D of, D ot, double* ta, double* tb) {
    if ((st.x == ot.x && st.y == ot.y) || (sf.x == of.x && sf.y == of.y) ||
        (sf.x == ot.x && sf.y == ot.y) || (st.x == of.x && st.y == of.y)) {
        return false;
    }
    D v1{st.x - sf.x, st.y - sf.y};
    D v2{ot.x - of.x, ot.y - of.y};
    double v1_cross_v2 = v1.x * v2.y - v1.y * v2.x;
    if (v1_cross_v2 == 0.0) return false;
    double sign = v1_cross_v2 > 0.0 ? 1.0 : -1.0;
    double abs_c = std::fabs(v1_cross_v2);
    D v3{of.x - sf.x, of.y - sf.y};
    double t = (v3.x * v2.y - v3.y * v2.x) * sign;
    double u = (v3.x * v1.y - v3.y * v1.x) * sign;
    if (t < 0.0 || t > abs_c || u < 0.0 || u > abs_c) return false;
    *ta = t / abs_c;
    *tb = u / abs_c;
    return true;
}

struct Filler {
    P current_position{-FLT_MAX, -FLT_MAX};
    uint32_t current_vertex = INVALID_ID;
    uint32_t current_event_id = INVALID_EVENT;
    std::vector<ActiveEdge> active;
    std::vector<PendingEdge> edges_below;
    int fill_rule = LYON_FILL_EVEN_ODD;
    int orientation = LYON_ORIENTATION_VERTICAL;
    float tolerance = 0.1f;
    std::vector<Span> spans;
    bool assume_no_intersection = false;
    ActiveEdgeScan scan;
    EventQueue events;
    Output* out = nullptr;

    void begin_span(int32_t span_idx, P position, uint32_t vertex) {  // fill.rs:223-233
        if (span_idx < 0 || (size_t)span_idx > spans.size()) throw TessError{LYON_ERR_INTERNAL, 110};
        std::unique_ptr<AdvancedMonotone> t(new AdvancedMonotone());
        t->begin(position, vertex);
        spans.insert(spans.begin() + span_idx, Span{std::move(t)});
    }
    void end_span(int32_t span_idx, P position, uint32_t id) {  // fill.rs:235-254
        Span& span = spans[(size_t)span_idx];
        if (!span.tess) throw TessError{LYON_ERR_INTERNAL, 100};
        span.tess->end(position, id);
        span.tess->flush(out);
        span.tess.reset();
    }
    void cleanup_spans() {  // fill.rs:291-294
        spans.erase(std::remove_if(spans.begin(), spans.end(),
                                   [](const Span& s) { return !s.tess; }),
                    spans.end());
    }
    AdvancedMonotone& span_tess(int32_t idx) {
        if (idx < 0 || (size_t)idx >= spans.size() || !spans[(size_t)idx].tess)
            throw TessError{LYON_ERR_INTERNAL, 101};
        return *spans[(size_t)idx].tess;
    }

    // fill.rs:1295-1324. Returns 0 or an IncorrectActiveEdgeOrder code.
    int check_remaining_edges(size_t active_edge_idx, float current_x) const {
        for (size_t i = active_edge_idx; i < active.size(); ++i) {
            const ActiveEdge& e = active[i];
            if (e.is_merge) continue;
            if (e.max_x() < current_x) return 1;
            if (peq(current_position, e.to)) return 2;
            if (e.min_x() < current_x && e.solve_x_for_y(current_position.y) < current_x) return 3;
        }
        return 0;
    }

    // fill.rs:1328-1378. Returns -1 (error, *err set), 0 (not connecting), 1 (connecting).
    int is_edge_connecting(const ActiveEdge& e, size_t active_edge_idx, int* err) {
        if (peq(current_position, e.to)) return 1;
        float current_x = current_position.x;
        float threshold = tolerance;
        float min_x = e.min_x(), max_x = e.max_x();
        if (max_x + threshold < current_x || e.to.y < current_position.y) {
            *err = 4;
            return -1;
        }
        if (min_x > current_x) return 0;
        float ex;
        if (e.from.y != e.to.y) {
            ex = e.solve_x_for_y(current_position.y);
        } else if (max_x >= current_x && min_x <= current_x) {
            ex = current_x;
        } else {
            ex = e.to.x;
        }
        if (fabsf(ex - current_x) <= threshold) {
            scan.edges_to_split.push_back(active_edge_idx);
            return 1;
        }
        if (ex < current_x) {
            *err = 5;
            return -1;
        }
        return 0;
    }

    // fill.rs:1045-1291. Returns 0 or an internal error code (>0).
    int scan_active_edges() {
        scan.reset();
        float current_x = current_position.x;
        bool connecting_edges = false;
        size_t active_edge_idx = 0;
        WindingState winding;
        bool previous_was_merge = false;

        for (const ActiveEdge& e : active) {
            if (e.is_merge) {
                winding.span_index += 1;
                active_edge_idx += 1;
                previous_was_merge = true;
                continue;
            }
            bool edge_is_before_current_point;
            if (peq(current_position, e.to)) {
                connecting_edges = true;
                edge_is_before_current_point = false;
            } else if (e.max_x() < current_x) {
                edge_is_before_current_point = true;
            } else if (e.min_x() > current_x) {
                edge_is_before_current_point = false;
            } else if (e.from.y == e.to.y) {
                connecting_edges = true;
                edge_is_before_current_point = false;
            } else {
                float ex = e.solve_x_for_y(current_position.y);
                if (fabsf(ex - current_x) <= tolerance) {
                    connecting_edges = true;
                    edge_is_before_current_point = false;
                } else if (ex > current_x) {
                    edge_is_before_current_point = false;
                } else {
                    edge_is_before_current_point = true;
                }
            }
            if (!edge_is_before_current_point) break;
            winding.update(fill_rule, e.winding);
            previous_was_merge = false;
            active_edge_idx += 1;
        }

        scan.above_start = active_edge_idx;
        scan.winding_before_point = winding;

        if (previous_was_merge) {
            scan.winding_before_point.span_index -= 1;
            scan.above_start -= 1;
            if (!connecting_edges) {
                scan.vertex_events.push_back({winding.span_index - 1, RIGHT});
                scan.vertex_events.push_back({winding.span_index, LEFT});
                scan.merge_split_event = true;
            }
        }

        scan.split_event = !connecting_edges && winding.is_in && !scan.merge_split_event;

        if (connecting_edges) {
            bool in_before_vertex = winding.is_in;
            bool first_connecting_edge = !previous_was_merge;
            for (size_t i = active_edge_idx; i < active.size(); ++i) {
                const ActiveEdge& e = active[i];
                if (e.is_merge) {
                    if (!winding.is_in) return 200;  // MergeVertexOutside
                    scan.spans_to_end.push_back(winding.span_index);
                    winding.span_index += 1;
                    active_edge_idx += 1;
                    first_connecting_edge = false;
                    continue;
                }
                int err = 0;
                int c = is_edge_connecting(e, active_edge_idx, &err);
                if (c < 0) return err;
                if (c == 0) break;
                if (!first_connecting_edge && winding.is_in) {
                    scan.spans_to_end.push_back(winding.span_index);
                }
                winding.update(fill_rule, e.winding);
                if (winding.is_in && winding.span_index >= (int32_t)spans.size()) {
                    return 201;  // InsufficientNumberOfSpans
                }
                active_edge_idx += 1;
                first_connecting_edge = false;
            }
            bool in_after_vertex = winding.is_in;
            bool vertex_is_merge_event = in_before_vertex && in_after_vertex &&
                                         edges_below.empty() && scan.edges_to_split.empty();
            if (vertex_is_merge_event) scan.merge_event = true;
            if (in_before_vertex) {
                scan.vertex_events.push_back({scan.winding_before_point.span_index, RIGHT});
            }
            if (in_after_vertex) scan.vertex_events.push_back({winding.span_index, LEFT});
        }

        scan.above_end = active_edge_idx;
        return check_remaining_edges(active_edge_idx, current_x);
    }

    // fill.rs:1381-1452
    void process_edges_above() {
        for (auto& ve : scan.vertex_events) {
            span_tess(ve.first).vertex(current_position, current_vertex, ve.second);
        }
        for (int32_t span_index : scan.spans_to_end) {
            if (span_index < 0 || (size_t)span_index >= spans.size())
                throw TessError{LYON_ERR_INTERNAL, 102};
            end_span(span_index, current_position, current_vertex);
        }
        cleanup_spans();
        for (size_t edge_idx : scan.edges_to_split) {
            ActiveEdge& e = active[edge_idx];
            P to = e.to;
            edges_below.push_back(
                PendingEdge{to, slope(sub(to, current_position)), e.src_edge, e.winding,
                            e.range_end});
            e.to = current_position;
        }
        if (scan.merge_event) {
            ActiveEdge& e = active[scan.above_start];
            e.is_merge = true;
            e.from = e.to;
            e.winding = 0;
            e.from_id = current_vertex;
            scan.above_start += 1;
        }
    }

    // fill.rs:2010-2013: sort_unstable_by on sort_key (partial_cmp, NaN -> Equal). Lyon's slices
    // are short; insertion sort gives the order Rust's small-slice sort gives.
    void sort_edges_below() {
        for (size_t i = 1; i < edges_below.size(); ++i) {
            size_t j = i;
            while (j > 0 && edges_below[j].sort_key < edges_below[j - 1].sort_key) {
                std::swap(edges_below[j], edges_below[j - 1]);
                --j;
            }
        }
    }

    // fill.rs:2050-2106
    void merge_coincident_edges(size_t a_idx, size_t b_idx) {
        P a_to = edges_below[a_idx].to;
        P b_to = edges_below[b_idx].to;
        size_t lower_idx, upper_idx;
        bool split;
        int c = compare_positions(a_to, b_to);
        if (c > 0) {
            lower_idx = a_idx;
            upper_idx = b_idx;
            split = true;
        } else if (c < 0) {
            lower_idx = b_idx;
            upper_idx = a_idx;
            split = true;
        } else {
            lower_idx = a_idx;
            upper_idx = b_idx;
            split = false;
        }
        edges_below[upper_idx].winding =
            (int16_t)(edges_below[upper_idx].winding + edges_below[lower_idx].winding);
        P split_point = edges_below[upper_idx].to;
        PendingEdge edge = edges_below[lower_idx];
        edges_below.erase(edges_below.begin() + lower_idx);
        if (!split) return;
        EdgeData src = events.edge_data[edge.src_edge];
        float dy = edge.to.y - current_position.y;
        float t = dy == 0.0f ? 0.0f : (split_point.y - current_position.y) / dy;
        float t_remapped = remap_t_in_range(t, src.range_start, edge.range_end);
        EdgeData data{edge.to, t_remapped, edge.range_end, edge.winding, true, src.from_id,
                      src.to_id};
        events.insert_sorted(split_point, data, current_event_id);
    }

    // fill.rs:2016-2048
    void handle_coincident_edges_below() {
        if (edges_below.size() < 2) return;
        for (long idx = (long)edges_below.size() - 2; idx >= 0; --idx) {
            size_t a_idx = (size_t)idx, b_idx = (size_t)idx + 1;
            float a_slope = edges_below[a_idx].sort_key;
            float b_slope = edges_below[b_idx].sort_key;
            const float THRESHOLD = 0.00005f;
            bool angle_is_close;
            if (fabsf(a_slope) <= 1.0f) {
                angle_is_close = fabsf(a_slope - b_slope) < THRESHOLD;
            } else {
                angle_is_close = fabsf(1.0f / a_slope - 1.0f / b_slope) < THRESHOLD;
            }
            if (angle_is_close) merge_coincident_edges(a_idx, b_idx);
        }
    }

    // fill.rs:1563-1608
    void split_event(size_t left_enclosing_edge_idx, int32_t left_span_idx) {
        size_t right_enclosing_edge_idx = left_enclosing_edge_idx + 1;
        if (right_enclosing_edge_idx >= active.size()) throw TessError{LYON_ERR_INTERNAL, 103};
        P upper_left = active[left_enclosing_edge_idx].from;
        P upper_right = active[right_enclosing_edge_idx].from;
        int32_t right_span_idx = left_span_idx + 1;
        P upper_position;
        uint32_t upper_id;
        int32_t new_span_idx;
        if (is_after(upper_left, upper_right)) {
            upper_position = upper_left;
            upper_id = active[left_enclosing_edge_idx].from_id;
            new_span_idx = left_span_idx;
        } else {
            upper_position = upper_right;
            upper_id = active[right_enclosing_edge_idx].from_id;
            new_span_idx = right_span_idx;
        }
        if (new_span_idx < 0 || (size_t)new_span_idx > spans.size())
            throw TessError{LYON_ERR_INTERNAL, 104};
        begin_span(new_span_idx, upper_position, upper_id);
        span_tess(left_span_idx).vertex(current_position, current_vertex, RIGHT);
        span_tess(right_span_idx).vertex(current_position, current_vertex, LEFT);
    }

    // fill.rs:1455-1524
    void process_edges_below() {
        WindingState winding = scan.winding_before_point;
        sort_edges_below();
        handle_coincident_edges_below();
        if (scan.split_event) {
            if (scan.above_start == 0) throw TessError{LYON_ERR_INTERNAL, 105};
            split_event(scan.above_start - 1, winding.span_index);
        }
        bool first_pending_edge = true;
        for (const PendingEdge& pe : edges_below) {
            if (!first_pending_edge && winding.is_in) {
                if (winding.span_index < 0 || (size_t)winding.span_index > spans.size())
                    throw TessError{LYON_ERR_INTERNAL, 106};
                begin_span(winding.span_index, current_position, current_vertex);
            }
            winding.update(fill_rule, pe.winding);
            first_pending_edge = false;
        }
    }

    // fill.rs:1689-1846
    void process_intersection(double ta, double tb, size_t active_edge_idx,
                              PendingEdge& edge_below, D below_from, D below_to) {
        // LineSegment<f64>::sample (line.rs:21-23) = from.lerp(to, t)
        double one_t = 1.0 - tb;
        P intersection_position{(float)(one_t * below_from.x + tb * below_to.x),
                                (float)(one_t * below_from.y + tb * below_to.y)};
        ActiveEdge& ae = active[active_edge_idx];
        if (peq(current_position, intersection_position)) {
            ae.from = intersection_position;
            EdgeData& src = events.edge_data[ae.src_edge];
            src.range_start = remap_t_in_range((float)ta, src.range_start, ae.range_end);
            return;
        }
        if (!is_after(intersection_position, current_position)) {
            intersection_position.y = nextafterf(current_position.y, INFINITY);
        }
        if (!is_after(intersection_position, current_position)) {
            throw TessError{LYON_ERR_INTERNAL, 107};  // lyon: assert! (panic)
        }
        if (is_near(intersection_position, edge_below.to)) {
            intersection_position = edge_below.to;
        } else if (is_near(intersection_position, ae.to)) {
            intersection_position = ae.to;
        }
        EdgeData a_src = events.edge_data[ae.src_edge];
        EdgeData b_src = events.edge_data[edge_below.src_edge];
        bool has_inserted = false;
        uint32_t inserted_evt = 0;
        bool flipped_active = false;
        if (!peq(ae.to, intersection_position) && !peq(ae.from, intersection_position)) {
            float remapped_ta = remap_t_in_range((float)ta, a_src.range_start, ae.range_end);
            if (is_after(ae.to, intersection_position)) {
                EdgeData d{ae.to, remapped_ta, ae.range_end, ae.winding, true, a_src.from_id,
                           a_src.to_id};
                inserted_evt = events.insert_sorted(intersection_position, d, current_event_id);
                has_inserted = true;
            } else {
                flipped_active = true;
                EdgeData d{intersection_position, ae.range_end, remapped_ta,
                           (int16_t)(-ae.winding), true, a_src.from_id, a_src.to_id};
                events.insert_sorted(ae.to, d, current_event_id);
            }
            ae.to = intersection_position;
            ae.range_end = remapped_ta;
        }
        if (!peq(edge_below.to, intersection_position) &&
            !peq(current_position, intersection_position)) {
            float remapped_tb =
                remap_t_in_range((float)tb, b_src.range_start, edge_below.range_end);
            if (is_after(edge_below.to, intersection_position)) {
                EdgeData d{edge_below.to, remapped_tb, edge_below.range_end, edge_below.winding,
                           true, b_src.from_id, b_src.to_id};
                if (has_inserted) {
                    events.insert_sibling(inserted_evt, intersection_position, d);
                } else {
                    events.insert_sorted(intersection_position, d, current_event_id);
                }
            } else {
                EdgeData d{intersection_position, edge_below.range_end, remapped_tb,
                           (int16_t)(-edge_below.winding), true, b_src.from_id, b_src.to_id};
                events.insert_sorted(edge_below.to, d, current_event_id);
                if (flipped_active) {
                    events.vertex_event_sorted(intersection_position, b_src.to_id,
                                               current_event_id);
                }
            }
            edge_below.to = intersection_position;
            edge_below.range_end = remapped_tb;
        }
    }

    // fill.rs:1611-1686
    void handle_intersections(size_t skip_start, size_t skip_end) {
        std::vector<PendingEdge> below;
        below.swap(edges_below);
        for (PendingEdge& eb : below) {
            float below_min_x = fminf(current_position.x, eb.to.x);
            float below_max_x = fmax_lyon(current_position.x, eb.to.x);
            D bf = dd(current_position), bt = dd(eb.to);
            double tb_min = 1.0;
            bool found = false;
            double fta = 0, ftb = 0;
            size_t fidx = 0;
            for (size_t i = 0; i < active.size(); ++i) {
                if (i >= skip_start && i < skip_end) continue;
                const ActiveEdge& ae = active[i];
                if (ae.is_merge || below_min_x > ae.max_x()) continue;
                if (below_max_x < ae.min_x()) continue;
                double ta, tb;
                if (segment_intersection_t(dd(ae.from), dd(ae.to), bf, bt, &ta, &tb)) {
                    if (tb < tb_min && tb > 0.0 && ta > 0.0 && ta <= 1.0) {
                        tb_min = tb;
                        found = true;
                        fta = ta;
                        ftb = tb;
                        fidx = i;
                    }
                }
            }
            if (found) process_intersection(fta, ftb, fidx, eb, bf, bt);
        }
        edges_below.swap(below);
    }

    // fill.rs:1527-1561
    void update_active_edges() {
        size_t s = scan.above_start, e = scan.above_end;
        if (!assume_no_intersection) handle_intersections(s, e);
        std::vector<ActiveEdge> repl;
        repl.reserve(edges_below.size());
        for (const PendingEdge& pe : edges_below) {
            repl.push_back(ActiveEdge{current_position, pe.to, pe.winding, false, current_vertex,
                                      pe.src_edge, pe.range_end});
        }
        edges_below.clear();
        active.erase(active.begin() + s, active.begin() + e);
        active.insert(active.begin() + s, repl.begin(), repl.end());
    }

    // fill.rs:929-965. Returns 0 or an internal error code.
    int process_events() {
        int err = scan_active_edges();
        if (err) return err;
        process_edges_above();
        process_edges_below();
        update_active_edges();
        return 0;
    }

    // fill.rs:1848-1953 (stable sort, as Vec::sort_by)
    void sort_active_edges() {
        float y = current_position.y;
        std::vector<std::pair<float, size_t>> keys;
        keys.reserve(active.size());
        bool has_merge_vertex = false;
        float prev_x = NAN;
        for (size_t i = 0; i < active.size(); ++i) {
            const ActiveEdge& e = active[i];
            if (e.is_merge) {
                has_merge_vertex = true;
                keys.push_back({prev_x, i});
            } else {
                bool eq_to = e.to.y == y;
                bool eq_from = e.from.y == y;
                float x;
                if (eq_to && eq_from) {
                    float current_x = current_position.x;
                    if (e.max_x() >= current_x && e.min_x() <= current_x) {
                        x = current_position.x;
                    } else {
                        x = e.min_x();
                    }
                } else if (eq_from) {
                    x = e.from.x;
                } else if (eq_to) {
                    x = e.to.x;
                } else {
                    x = e.solve_x_for_y(y);
                }
                keys.push_back({fmax_lyon(x, e.min_x()), i});
                prev_x = x;
            }
        }
        if (keys.size() > 1) {
            for (auto& k : keys) {
                if (k.first != k.first) throw TessError{LYON_ERR_INTERNAL, 108};  // unwrap on NaN
            }
        }
        std::stable_sort(keys.begin(), keys.end(), [&](const auto& a, const auto& b) {
            if (a.first < b.first) return true;
            if (a.first > b.first) return false;
            const ActiveEdge& ea = active[a.second];
            const ActiveEdge& eb = active[b.second];
            if (!ea.is_merge && !eb.is_merge) {
                float slope_a = slope(sub(ea.to, ea.from));
                float slope_b = slope(sub(eb.to, eb.from));
                return slope_b < slope_a;  // slope_b.partial_cmp(&slope_a) == Less
            }
            if (ea.is_merge && !eb.is_merge) return false;  // Greater
            if (!ea.is_merge && eb.is_merge) return true;   // Less
            return false;
        });
        std::vector<ActiveEdge> sorted;
        sorted.reserve(active.size());
        for (auto& k : keys) sorted.push_back(active[k.second]);
        active.swap(sorted);
        if (!has_merge_vertex) return;
        int16_t winding_number = 0;
        for (size_t i = 0; i < active.size(); ++i) {
            bool needs_swap;
            if (active[i].is_merge) {
                needs_swap = !fill_rule_is_in(fill_rule, winding_number);
            } else {
                winding_number = (int16_t)(winding_number + active[i].winding);
                needs_swap = false;
            }
            if (needs_swap) {
                int16_t w = winding_number;
                size_t idx = i;
                while (idx > 0) {
                    w = (int16_t)(w - active[idx - 1].winding);
                    std::swap(active[idx], active[idx - 1]);
                    if (fill_rule_is_in(fill_rule, w)) break;
                    idx -= 1;
                }
            }
        }
    }

    // fill.rs:1956-2007
    void recover_from_error() {
        sort_active_edges();
        size_t len = active.size();
        if (len > 1 && active[len - 1].is_merge) std::swap(active[len - 1], active[len - 2]);
        WindingState winding;
        for (const ActiveEdge& e : active) {
            if (e.is_merge) {
                winding.span_index += 1;
            } else {
                winding.update(fill_rule, e.winding);
            }
            if (winding.span_index >= (int32_t)spans.size()) {
                begin_span(winding.span_index, e.from, e.from_id);
            }
        }
        while ((int64_t)spans.size() > (int64_t)winding.span_index + 1) {
            if (!spans.back().tess) throw TessError{LYON_ERR_INTERNAL, 109};
            spans.back().tess->flush(out);
            spans.pop_back();
        }
    }

    // VertexSourceIterator (fill.rs:2294-2337): every sibling event at the vertex gives its
    // edge's endpoint (t = 0 or 1) or the point at t on it; a source equal to the previous one is
    // skipped.
    void record_sources(uint32_t evt) {
        bool have_prev = false;
        Src prev;
        uint32_t count = 0;
        for (uint32_t id = evt; id != INVALID_EVENT; id = events.events[id].next_sibling) {
            const EdgeData& e = events.edge_data[id];
            const float t = e.range_start;
            const Src src = t == 0.0f   ? endpoint_src(e.from_id)
                            : t == 1.0f ? endpoint_src(e.to_id)
                                        : Src{e.from_id, e.to_id, t};
            const bool same = have_prev && src.from == prev.from && src.to == prev.to &&
                              (src.to == NO_ENDPOINT || src.t == prev.t);
            if (same) continue;
            uint32_t tb;
            std::memcpy(&tb, &src.t, 4);
            out->fill_sources.push_back(src.from);
            out->fill_sources.push_back(src.to);
            out->fill_sources.push_back(tb);
            prev = src;
            have_prev = true;
            ++count;
        }
        out->fill_source_counts.push_back(count);
    }

    // fill.rs:869-925
    void initialize_events() {
        uint32_t current_event = current_event_id;
        current_position = events.position(current_event);
        if (is_nan_f(current_position.x) || is_nan_f(current_position.y)) {
            throw TessError{LYON_ERR_POSITION_IS_NAN, 0};
        }
        P position = orientation == LYON_ORIENTATION_VERTICAL
                         ? current_position
                         : P{current_position.y, -current_position.x};
        uint32_t id;
        if (!out->add_vertex(position, &id)) throw TessError{LYON_ERR_TOO_MANY_VERTICES, 0};
        current_vertex = id;
        if (out->want_sources) record_sources(current_event);
        uint32_t sib = current_event;
        while (sib != INVALID_EVENT) {
            const EdgeData& edge = events.edge_data[sib];
            if (edge.is_edge) {
                P to = edge.to;
                edges_below.push_back(
                    PendingEdge{to, slope(sub(to, current_position)), sib, edge.winding,
                                edge.range_end});
            }
            sib = events.next_sibling_id(sib);
        }
    }

    // fill.rs:836-867
    void tessellator_loop() {
        current_event_id = events.first;
        while (current_event_id != INVALID_EVENT) {
            initialize_events();
            int err = process_events();
            if (err) {
                recover_from_error();
                err = process_events();
                if (err) throw TessError{LYON_ERR_INTERNAL, err};
            }
            current_event_id = events.next_id(current_event_id);
        }
    }

    // fill.rs:749-821
    int tessellate_impl(const lyon_fill_options& options) {
        if (is_nan_f(options.tolerance) || options.tolerance <= 0.0f)
            return LYON_ERR_TOLERANCE_IS_NAN;
        fill_rule = options.fill_rule;
        orientation = options.sweep_orientation;
        assume_no_intersection = !options.handle_intersections;
        tolerance = options.tolerance * 0.5f;
        out->begin_geometry();
        try {
            tessellator_loop();
        } catch (const TessError& e) {
            out->abort_geometry();
            return e.code;
        }
        if (assume_no_intersection && (!active.empty() || !spans.empty())) {
            out->abort_geometry();
            return LYON_ERR_INTERNAL;
        }
        for (Span& s : spans) {
            if (s.tess) s.tess->flush(out);
        }
        spans.clear();
        return LYON_OK;
    }

    // fill.rs:578-596 + event_queue.rs:483-551 (set_path) + build.
    int tessellate(PathIter it, const lyon_fill_options& options) {
        events.reset();
        EventQueueBuilder b;
        b.queue = &events;
        b.tolerance = options.tolerance;
        bool horizontal = options.sweep_orientation == LYON_ORIENTATION_HORIZONTAL;
        auto ro = [&](P p) { return horizontal ? P{-p.y, p.x} : p; };  // event_queue.rs:13-16
        Evt e;
        while (it.next(&e)) {
            switch (e.kind) {
                case EV_BEGIN:
                    b.begin(ro(e.to), e.id_to);
                    break;
                case EV_LINE:
                    b.line_segment(ro(e.to), e.id_to, 0.0f, 1.0f);
                    break;
                case EV_QUAD:
                    b.quadratic_bezier_segment(ro(e.ctrl1), ro(e.to), e.id_to);
                    break;
                case EV_CUBIC:
                    b.cubic_bezier_segment(ro(e.ctrl1), ro(e.ctrl2), ro(e.to), e.id_to);
                    break;
                case EV_END:
                    b.end(ro(e.to), e.id_to);
                    break;
            }
        }
        if (it.bad) return LYON_ERR_INVALID_ARGUMENT;
        events.sort();
        return tessellate_impl(options);
    }
};

// --------------------------------------------------------------------------------------------
// Path-level flattening: path.iter().flattened(tol) (crates/path/src/iterator.rs:125-215).
// Appends the `to` point of every Line event; counts[v] = number of points for verb v.
// --------------------------------------------------------------------------------------------
static void flatten_path(const uint8_t* verbs, uint32_t nverbs, const float* pts, uint32_t npts,
                         float tol, std::vector<float>* out_pts, std::vector<uint32_t>* counts) {
    PathIter it{verbs, nverbs, pts, npts};
    Evt e;
    while (it.next(&e)) {
        uint32_t n = 0;
        switch (e.kind) {
            case EV_LINE:
                out_pts->push_back(e.to.x);
                out_pts->push_back(e.to.y);
                n = 1;
                break;
            case EV_QUAD: {
                Quad q{e.from, e.ctrl1, e.to};
                quad_flatten_with_t(q, tol, [&](P, P to, float, float) {
                    out_pts->push_back(to.x);
                    out_pts->push_back(to.y);
                    ++n;
                });
                break;
            }
            case EV_CUBIC: {
                Cubic c{e.from, e.ctrl1, e.ctrl2, e.to};
                cubic_flatten_with_t(c, tol, [&](P, P to, float, float) {
                    out_pts->push_back(to.x);
                    out_pts->push_back(to.y);
                    ++n;
                });
                break;
            }
            default:
                break;
        }
        counts->push_back(n);
    }
}

// --------------------------------------------------------------------------------------------
// Basic shapes (crates/tessellation/src/basic_shapes.rs): FillTessellator::tessellate_rectangle
// and tessellate_circle, which bypass the sweep.
// --------------------------------------------------------------------------------------------
// basic_shapes.rs:12-38
static int fill_rectangle(Output* out, P min, P max) {
    out->begin_geometry();
    P corners[4] = {min, P{min.x, max.y}, max, P{max.x, min.y}};
    uint32_t id[4];
    for (int k = 0; k < 4; ++k) {
        if (!out->add_vertex(corners[k], &id[k])) {
            out->abort_geometry();
            return LYON_ERR_TOO_MANY_VERTICES;
        }
    }
    out->add_triangle(id[0], id[1], id[2]);
    out->add_triangle(id[0], id[2], id[3]);
    return LYON_OK;
}

// basic_shapes.rs:151-155
static float circle_flattening_step_fill(float radius, float tolerance) {
    tolerance = fminf(tolerance, radius);
    return 2.0f * sqrtf(2.0f * tolerance * radius - tolerance * tolerance);
}

// basic_shapes.rs:158-207
static bool fill_border_radius(Output* out, P center, float a0, float a1, float radius,
                               uint32_t va, uint32_t vb, uint32_t num_recursions) {
    if (num_recursions == 0) return true;
    float mid_angle = (a0 + a1) * 0.5f;
    P normal = P{cosf(mid_angle), sinf(mid_angle)};
    P position = add(center, mul(normal, radius));
    uint32_t v;
    if (!out->add_vertex(position, &v)) return false;
    out->add_triangle(vb, v, va);
    return fill_border_radius(out, center, a0, mid_angle, radius, va, v, num_recursions - 1) &&
           fill_border_radius(out, center, mid_angle, a1, radius, v, vb, num_recursions - 1);
}

// basic_shapes.rs:40-124
static int fill_circle(Output* out, P center, float radius, float tolerance) {
    radius = fabsf(radius);
    if (radius == 0.0f) return LYON_OK;
    float arc_len = 0.5f * PI_F * radius;
    float step = circle_flattening_step_fill(radius, tolerance);
    float num_segments = ceilf(arc_len / step);
    uint32_t num_recursions = sat_u32(log2f(num_segments));  // `as u32`
    // More than four million vertices for one circle: reported as unsupported (the GPU's bound).
    if (num_recursions > 20) return LYON_ERR_UNSUPPORTED;
    out->begin_geometry();
    const P dirs[4] = {P{-1.0f, 0.0f}, P{0.0f, -1.0f}, P{1.0f, 0.0f}, P{0.0f, 1.0f}};
    uint32_t v[4];
    for (int k = 0; k < 4; ++k) {
        if (!out->add_vertex(add(center, mul(dirs[k], radius)), &v[k])) {
            out->abort_geometry();
            return LYON_ERR_TOO_MANY_VERTICES;
        }
    }
    out->add_triangle(v[0], v[3], v[1]);
    out->add_triangle(v[1], v[3], v[2]);
    const float angles[4][2] = {{PI_F, 1.5f * PI_F},
                                {1.5f * PI_F, 2.0f * PI_F},
                                {0.0f, PI_F * 0.5f},
                                {PI_F * 0.5f, PI_F}};
    for (int k = 0; k < 4; ++k) {
        if (!fill_border_radius(out, center, angles[k][0], angles[k][1], radius, v[k],
                                v[(k + 1) % 4], num_recursions)) {
            out->abort_geometry();
            return LYON_ERR_TOO_MANY_VERTICES;
        }
    }
    return LYON_OK;
}

// --------------------------------------------------------------------------------------------
// Elliptic arcs (crates/geom/src/arc.rs). cos/sin/acos are evaluated in f64 and rounded once, as
// on the GPU; lyon takes them from the platform's f32 libm, which may differ in the last bit.
// --------------------------------------------------------------------------------------------
struct ArcF {  // arc.rs:21-28
    P center, radii;
    float start_angle, sweep_angle, x_rotation;
};

// sample (arc.rs:194-197) = center + sample_ellipse(radii, x_rotation, get_angle(t))
// (arc.rs:217-219, 741-746; euclid's Rotation2D::transform_point).
static P arc_sample(const ArcF& a, float t) {
    const float angle = a.start_angle + a.sweep_angle * t;
    const float ex = a.radii.x * cr_cos(angle), ey = a.radii.y * cr_sin(angle);
    const float c = cr_cos(a.x_rotation), s = cr_sin(a.x_rotation);
    return P{a.center.x + (ex * c - ey * s), a.center.y + (ex * s + ey * c)};
}

// flattening_step (arc.rs:369-389).
static float arc_flattening_step(const ArcF& a, float tolerance) {
    const P from = arc_sample(a, 0.0f);
    const float r = length(sub(from, a.center));
    const float ang = 2.0f * cr_acos((r - tolerance) / r);
    const float result = fminf(ang / fabsf(a.sweep_angle), 1.0f);
    if (result < 1.1920929e-7f) return 1.0f;  // f32::EPSILON
    return result;
}

// Arcs with more segments than this fail with LYON_ERR_UNSUPPORTED (the GPU's bound).
static const uint64_t MAX_ARC_SEGMENTS = 1ull << 22;

// for_each_flattened_with_t (arc.rs:339-367): the start point (t = 0), then every segment's end
// point and t1. `pts`/`ts` may be NULL (counting). Returns the number of points or
// UINT64_MAX when the arc needs more than MAX_ARC_SEGMENTS segments.
static uint64_t arc_flatten(const ArcF& arc, float tolerance, float* pts, float* ts) {
    ArcF iter = arc;
    float t0 = 0.0f;
    P from = arc_sample(arc, 0.0f);
    uint64_t k = 0;
    auto put = [&](P p, float t) {
        if (pts) {
            pts[2 * k] = p.x;
            pts[2 * k + 1] = p.y;
        }
        if (ts) ts[k] = t;
        ++k;
    };
    put(from, 0.0f);
    for (;;) {
        const float step = arc_flattening_step(iter, tolerance);
        if (step >= 1.0f) break;
        if (k > MAX_ARC_SEGMENTS) return UINT64_MAX;
        // after_split (arc.rs:286-296)
        const float split_angle = iter.sweep_angle * step;
        iter.start_angle = iter.start_angle + split_angle;
        iter.sweep_angle = iter.sweep_angle - split_angle;
        const float t1 = t0 + step * (1.0f - t0);
        put(arc_sample(iter, 0.0f), t1);
        t0 = t1;
    }
    put(arc_sample(arc, 1.0f), 1.0f);
    return k;
}

// --------------------------------------------------------------------------------------------
// Hatching and dots (crates/algorithms/src/hatching.rs). The rotation of the pattern is given as
// cos/sin pairs computed once by the caller (lyon's Rotation2D takes them from f32 libm).
// --------------------------------------------------------------------------------------------
struct HatchParams {
    float tolerance;
    float c, s;    // Rotation::new(angle)
    float ci, si;  // Rotation::new(-angle)
    float uv_x, uv_y;  // options.uv_origin
    float interval;    // RegularHatchingPattern::interval, or the dots' row interval
    bool compute_tangents;
    bool dots;
    float column_interval;  // RegularDotPattern::column_interval
};
struct HatchSeg {  // HatchSegment (hatching.rs:181-205)
    P a, a_tan;
    float a_u;
    P b, b_tan;
    float b_u;
    uint32_t row;
    float v;
};
struct DotOut {  // Dot (hatching.rs:216-227)
    P position;
    float u, v;
    uint32_t column, row;
};
struct Edge2 {
    P from, to;
};

// Rows and dots beyond these bounds fail the path (lyon loops on, e.g. when the interval is too
// small to move y): LYON_ERR_UNSUPPORTED.
static const uint64_t MAX_HATCH_ROWS = 1u << 24;
static const uint64_t MAX_DOTS = 1u << 26;

static int cmp_pos(P a, P b) {  // hatching.rs:617-632
    if (a.y > b.y) return 1;
    if (a.y < b.y) return -1;
    if (a.x > b.x) return 1;
    if (a.x < b.x) return -1;
    return 0;
}

struct Hatcher {
    HatchParams hp;
    std::vector<Edge2> edges, active;
    P first{0, 0}, current{0, 0};
    std::vector<HatchSeg>* segs = nullptr;
    std::vector<DotOut>* dots = nullptr;
    uint64_t rows = 0, ndots = 0;
    uint32_t column = 0;
    bool too_many = false;
    P uv{0, 0};  // the rotated uv origin (hatching.rs:307)

    P rot(P p, float c, float s) const { return P{p.x * c - p.y * s, p.x * s + p.y * c}; }

    void add_edge(P from, P to) {  // hatching.rs:471-482
        if (peq(from, to)) return;
        P f = rot(from, hp.c, hp.s), t = rot(to, hp.c, hp.s);
        if (cmp_pos(f, t) > 0) std::swap(f, t);
        edges.push_back(Edge2{f, t});
    }
    // EventsBuilder (hatching.rs:500-577) over the path's events.
    bool build(PathIter it) {
        Evt e;
        while (it.next(&e)) {
            switch (e.kind) {
                case EV_BEGIN:
                    first = current = e.to;
                    break;
                case EV_LINE:
                    add_edge(current, e.to);
                    current = e.to;
                    break;
                case EV_QUAD:
                    quad_flatten_with_t(Quad{current, e.ctrl1, e.to}, hp.tolerance,
                                        [&](P, P to, float, float) {
                                            add_edge(current, to);
                                            current = to;
                                        });
                    break;
                case EV_CUBIC:
                    cubic_flatten_with_t(Cubic{current, e.ctrl1, e.ctrl2, e.to}, hp.tolerance,
                                         [&](P, P to, float, float) {
                                             add_edge(current, to);
                                             current = to;
                                         });
                    break;
                case EV_END:
                    add_edge(current, first);
                    break;
            }
        }
        if (it.bad) return false;
        std::stable_sort(edges.begin(), edges.end(),
                         [](const Edge2& a, const Edge2& b) { return cmp_pos(a.from, b.from) < 0; });
        return true;
    }
    static float x_for_y(const Edge2& e, float y) {  // geom line.rs:56-71
        const float dy = e.to.y - e.from.y;
        const float t = dy == 0.0f ? 0.0f : (y - e.from.y) / dy;
        return e.from.x * (1.0f - t) + e.to.x * t;
    }
    // HatchesToDots::add_segment (hatching.rs:677-714) with RegularDotPattern.
    void seg_to_dots(const HatchSeg& g) {
        float u = 0.0f;
        const float u_start = g.a_u;
        const float d = hp.column_interval;
        const float m = u_start >= 0.0f ? fmodf(u_start, d) : d + fmodf(u_start, d);
        if (m != 0.0f) u += d - m;
        const P a = g.a;
        const P ab = normalize(sub(g.b, a));
        while (u_start + u < g.b_u) {
            if (++ndots > MAX_DOTS) {
                too_many = true;
                return;
            }
            if (dots) dots->push_back(DotOut{add(a, mul(ab, u)), g.a_u + u, g.v, column, g.row});
            column += 1;
            const float du = hp.column_interval;
            if (du <= 0.0f) return;
            u += du;
        }
    }
    // hatch_line (hatching.rs:381-428).
    void hatch_line(float y, uint32_t row) {
        std::stable_sort(active.begin(), active.end(), [&](const Edge2& a, const Edge2& b) {
            return x_for_y(a, y) < x_for_y(b, y);
        });
        bool inside = false;
        float prev_x = NAN;
        P prev_tan{NAN, NAN}, tan{NAN, NAN};
        const float v = y - uv.y;
        for (const Edge2& e : active) {
            if (e.to.y <= y) continue;
            const float x = x_for_y(e, y);
            if (hp.compute_tangents) tan = normalize(rot(sub(e.to, e.from), hp.ci, hp.si));
            if (inside) {
                HatchSeg g;
                g.a = rot(P{prev_x, y}, hp.ci, hp.si);
                g.b = rot(P{x, y}, hp.ci, hp.si);
                g.a_u = prev_x - uv.x;
                g.b_u = x - uv.x;
                g.a_tan = hp.compute_tangents ? prev_tan : P{NAN, NAN};
                g.b_tan = hp.compute_tangents ? tan : P{NAN, NAN};
                g.row = row;
                g.v = v;
                if (hp.dots) {
                    seg_to_dots(g);
                    if (too_many) return;
                } else if (segs) {
                    segs->push_back(g);
                }
            }
            inside = !inside;
            prev_x = x;
            prev_tan = tan;
        }
    }
    // hatch (hatching.rs:300-347). Returns LYON_OK, or LYON_ERR_UNSUPPORTED past the bounds.
    int hatch() {
        if (edges.empty()) return LYON_OK;
        uv = rot(P{hp.uv_x, hp.uv_y}, hp.c, hp.s);
        uint32_t row = 0;
        float y = edges[0].from.y + hp.interval;
        float y_max = y;
        auto line = [&]() -> bool {  // hatch_line, then next_offset (column reset for dots)
            if (++rows > MAX_HATCH_ROWS) {
                too_many = true;
                return false;
            }
            hatch_line(y, row);
            if (too_many) return false;
            row += 1;
            column = 0;
            y += hp.interval;
            return hp.interval > 0.0f;
        };
        for (const Edge2& e : edges) {
            while (y < e.from.y)
                if (!line()) return too_many ? LYON_ERR_UNSUPPORTED : LYON_OK;
            y_max = fmaxf(y_max, e.to.y);
            // update_sweep_line (hatching.rs:374-379)
            active.erase(std::remove_if(active.begin(), active.end(),
                                        [&](const Edge2& a) { return cmp_pos(a.to, e.from) < 0; }),
                         active.end());
            active.push_back(e);
        }
        while (y < y_max)
            if (!line()) return too_many ? LYON_ERR_UNSUPPORTED : LYON_OK;
        return LYON_OK;
    }
};

}  // namespace lo

// ============================================================================================
// C interface of the oracle (used by tests through ctypes).
// ============================================================================================
using namespace lo;

struct lyon_oracle_out {
    Output out;
    int index_bits = 32;
    std::vector<uint16_t> idx16;
    uint32_t near_ties = 0;
};

extern "C" {

lyon_oracle_out* lyon_oracle_out_new(int index_bits, uint64_t vertex_offset) {
    lyon_oracle_out* o = new lyon_oracle_out();
    o->index_bits = index_bits == 16 ? 16 : 32;
    o->out.max_index = index_bits == 16 ? 65535ull : 0xFFFFFFFEull;
    o->out.vertex_offset = vertex_offset;
    return o;
}
void lyon_oracle_out_free(lyon_oracle_out* o) { delete o; }
void lyon_oracle_out_clear(lyon_oracle_out* o) {
    o->out.vertices.clear();
    o->out.indices.clear();
    o->out.attributes.clear();
    o->out.sources.clear();
    o->out.fill_sources.clear();
    o->out.fill_source_counts.clear();
    o->near_ties = 0;
}
// Stroke vertex attributes (four words per vertex: normal x, normal y, advancement, side),
// recorded from the next call on.
void lyon_oracle_out_set_attributes(lyon_oracle_out* o, int enabled) {
    o->out.want_attributes = enabled != 0;
}
const uint32_t* lyon_oracle_out_attributes(const lyon_oracle_out* o) {
    return o->out.attributes.data();
}
// Stroke vertex sources (three words per vertex: from, to, t bits; `to` = 0xFFFFFFFF for an
// endpoint), recorded from the next call on. Ids index the path's point array.
void lyon_oracle_out_set_sources(lyon_oracle_out* o, int enabled) {
    o->out.want_sources = enabled != 0;
}
const uint32_t* lyon_oracle_out_sources(const lyon_oracle_out* o) {
    return o->out.sources.data();
}
// After a fill with sources on: every vertex's sources (three words each, path-local ids) and
// the number of sources of each vertex.
uint64_t lyon_oracle_out_num_fill_sources(const lyon_oracle_out* o) {
    return o->out.fill_sources.size() / 3;
}
const uint32_t* lyon_oracle_out_fill_sources(const lyon_oracle_out* o) {
    return o->out.fill_sources.data();
}
const uint32_t* lyon_oracle_out_fill_source_counts(const lyon_oracle_out* o) {
    return o->out.fill_source_counts.data();
}
uint64_t lyon_oracle_out_num_vertices(const lyon_oracle_out* o) { return o->out.vertices.size() / 2; }
uint64_t lyon_oracle_out_num_indices(const lyon_oracle_out* o) { return o->out.indices.size(); }
const float* lyon_oracle_out_vertices(const lyon_oracle_out* o) { return o->out.vertices.data(); }
const uint32_t* lyon_oracle_out_indices32(const lyon_oracle_out* o) { return o->out.indices.data(); }
uint32_t lyon_oracle_out_near_ties(const lyon_oracle_out* o) { return o->near_ties; }

// euclid's angle helpers as the oracle restates them (for the known-answer tests).
float lyon_oracle_fast_atan2(float y, float x) { return lo::fast_atan2(y, x); }
float lyon_oracle_angle_to(float from, float to) { return lo::angle_to(from, to); }

// StrokeTessellator::tessellate_path appending to the output (BuffersBuilder semantics).
int lyon_oracle_stroke_path(lyon_oracle_out* o, const uint8_t* verbs, uint32_t num_verbs,
                            const float* points, uint32_t num_points,
                            const lyon_stroke_options* options) {
    g_near_ties = 0;
    Stroker s(*options, &o->out);
    int r = s.tessellate(PathIter{verbs, num_verbs, points, num_points});
    o->near_ties += g_near_ties;
    return r;
}

// The same with StrokeOptions::variable_line_width: `widths` holds one factor per point (only
// the endpoints' are read); an endpoint's line width is options->line_width times its factor
// (stroke.rs:646-767).
int lyon_oracle_stroke_path_vw(lyon_oracle_out* o, const uint8_t* verbs, uint32_t num_verbs,
                               const float* points, uint32_t num_points, const float* widths,
                               const lyon_stroke_options* options) {
    g_near_ties = 0;
    Stroker s(*options, &o->out);
    s.vw = true;
    PathIter it{verbs, num_verbs, points, num_points};
    it.widths = widths;
    int r = s.tessellate(it);
    o->near_ties += g_near_ties;
    return r;
}

// Arc::for_each_flattened_with_t for `n` arcs of 7 floats (center x, y, radii x, y, start angle,
// sweep angle, x rotation). Counting call (pts NULL): counts[i] = points of arc i (start point
// included) and status. Output call: points and t at `offsets`.
void lyon_oracle_flatten_arcs(const float* arcs, uint32_t n, float tolerance, uint32_t* counts,
                              int32_t* status, const uint64_t* offsets, float* pts, float* ts) {
    for (uint32_t i = 0; i < n; ++i) {
        const float* a = arcs + 7 * (size_t)i;
        ArcF arc{P{a[0], a[1]}, P{a[2], a[3]}, a[4], a[5], a[6]};
        uint64_t k;
        if (pts && offsets) {
            k = arc_flatten(arc, tolerance, pts + 2 * offsets[i], ts ? ts + offsets[i] : nullptr);
        } else {
            k = arc_flatten(arc, tolerance, nullptr, nullptr);
        }
        if (counts) counts[i] = k == UINT64_MAX ? 0u : (uint32_t)k;
        if (status) status[i] = k == UINT64_MAX ? LYON_ERR_UNSUPPORTED : LYON_OK;
    }
}

// Hatcher::hatch_path / dot_path (hatching.rs:276-298) with a regular pattern for every path of a
// batch. params: tolerance, cos(angle), sin(angle), cos(-angle), sin(-angle), uv origin x, y,
// interval (hatches) or row interval (dots), compute_tangents (0/1), dots (0/1), column
// interval. Counting call (outputs NULL): counts and statuses. Output call: 12 words per hatch
// segment (a: x, y, tangent x, y, u; b: the same; row; v) or 6 per dot (x, y, u, v, column,
// row) at `offsets`.
void lyon_oracle_hatch(const lyon_path_batch* batch, const float* params, uint32_t* counts,
                       int32_t* status, const uint64_t* offsets, uint32_t* out) {
    HatchParams hp{params[0], params[1], params[2], params[3], params[4], params[5], params[6],
                   params[7], params[8] != 0.0f, params[9] != 0.0f, params[10]};
    for (uint32_t i = 0; i < batch->num_paths; ++i) {
        uint32_t v0 = batch->verb_offsets[i], v1 = batch->verb_offsets[i + 1];
        uint32_t p0 = batch->point_offsets[i], p1 = batch->point_offsets[i + 1];
        Hatcher h;
        h.hp = hp;
        std::vector<HatchSeg> segs;
        std::vector<DotOut> dots;
        const bool write = out && offsets;
        if (write) {
            if (hp.dots) h.dots = &dots;
            else h.segs = &segs;
        } else if (!hp.dots) {
            h.segs = &segs;
        }
        int st = LYON_OK;
        if (!h.build(PathIter{batch->verbs + v0, v1 - v0, batch->points + 2 * (size_t)p0,
                              p1 - p0}))
            st = LYON_ERR_INVALID_ARGUMENT;
        else
            st = h.hatch();
        const uint64_t n = st != LYON_OK ? 0 : (hp.dots ? h.ndots : segs.size());
        if (counts) counts[i] = (uint32_t)n;
        if (status) status[i] = st;
        if (!write || st != LYON_OK) continue;
        if (hp.dots) {
            uint32_t* d = out + 6 * offsets[i];
            for (size_t k = 0; k < dots.size(); ++k) {
                const DotOut& o = dots[k];
                std::memcpy(d + 6 * k, &o.position.x, 4);
                std::memcpy(d + 6 * k + 1, &o.position.y, 4);
                std::memcpy(d + 6 * k + 2, &o.u, 4);
                std::memcpy(d + 6 * k + 3, &o.v, 4);
                d[6 * k + 4] = o.column;
                d[6 * k + 5] = o.row;
            }
        } else {
            uint32_t* d = out + 12 * offsets[i];
            for (size_t k = 0; k < segs.size(); ++k) {
                const HatchSeg& g = segs[k];
                const float f[12] = {g.a.x, g.a.y, g.a_tan.x, g.a_tan.y, g.a_u,
                                     g.b.x, g.b.y, g.b_tan.x, g.b_tan.y, g.b_u, 0.0f, g.v};
                std::memcpy(d + 12 * k, f, sizeof f);
                d[12 * k + 10] = g.row;
            }
        }
    }
}

// FillTessellator::tessellate_rectangle / tessellate_circle appending to the output.
int lyon_oracle_fill_rectangle(lyon_oracle_out* o, float min_x, float min_y, float max_x,
                               float max_y) {
    return fill_rectangle(&o->out, P{min_x, min_y}, P{max_x, max_y});
}
int lyon_oracle_fill_circle(lyon_oracle_out* o, float cx, float cy, float radius,
                            float tolerance) {
    return fill_circle(&o->out, P{cx, cy}, radius, tolerance);
}

// FillTessellator::tessellate_path appending to the output.
int lyon_oracle_fill_path(lyon_oracle_out* o, const uint8_t* verbs, uint32_t num_verbs,
                          const float* points, uint32_t num_points,
                          const lyon_fill_options* options) {
    g_near_ties = 0;
    Filler f;
    f.out = &o->out;
    int r = f.tessellate(PathIter{verbs, num_verbs, points, num_points}, *options);
    o->near_ties += g_near_ties;
    return r;
}

// Per-verb flattened point counts and points of path.iter().flattened(tol).
// Returns the number of points written; `counts` has num_verbs entries. Pass NULL buffers to
// query the size first.
uint64_t lyon_oracle_flatten_path(const uint8_t* verbs, uint32_t num_verbs, const float* points,
                                  uint32_t num_points, float tolerance, uint32_t* counts,
                                  float* out_points, uint64_t capacity) {
    std::vector<float> pts;
    std::vector<uint32_t> cnt;
    lo::flatten_path(verbs, num_verbs, points, num_points, tolerance, &pts, &cnt);
    if (counts) std::memcpy(counts, cnt.data(), cnt.size() * sizeof(uint32_t));
    if (out_points && capacity >= pts.size() / 2)
        std::memcpy(out_points, pts.data(), pts.size() * sizeof(float));
    return pts.size() / 2;
}

// Wang segment count of one quadratic (n_ctrl = 3 points) or cubic (4 points), as the float
// `flattened_segments_wang` returns (before the u32 truncation).
float lyon_oracle_wang(const float* pts, int n_ctrl, float tolerance) {
    if (n_ctrl == 3) {
        Quad q{P{pts[0], pts[1]}, P{pts[2], pts[3]}, P{pts[4], pts[5]}};
        return quad_wang(q, tolerance);
    }
    Cubic c{P{pts[0], pts[1]}, P{pts[2], pts[3]}, P{pts[4], pts[5]}, P{pts[6], pts[7]}};
    return cubic_wang(c, tolerance);
}

// Batched CPU baseline: every path tessellated into its own buffers, paths statically chunked
// over `num_threads` std::threads (one tessellator per thread). Writes per-path vertex and
// index counts, statuses and near-tie counts; when `vertices`/`indices` are non-NULL the
// outputs are concatenated in path order (indices per path, i.e. LYON_INDEX_PER_PATH) and the
// caller must size them from a previous counting call. kind: 0 = stroke, 1 = fill.
static int batch_impl(int kind, const lyon_path_batch* batch, const float* widths,
                      const void* options, uint32_t num_options, int index_bits, int num_threads,
                      uint32_t* vtx_counts, uint32_t* idx_counts, int32_t* status,
                      uint32_t* near_ties, float* vertices, uint32_t* indices,
                      const uint64_t* vtx_offsets, const uint64_t* idx_offsets,
                      uint32_t* attributes, uint32_t* sources = nullptr) {
    uint32_t n = batch->num_paths;
    if (num_threads < 1) num_threads = 1;
    std::atomic<uint32_t> next{0};
    auto worker = [&]() {
        lyon_oracle_out o;
        o.out.max_index = index_bits == 16 ? 65535ull : 0xFFFFFFFEull;
        o.out.want_attributes = attributes != nullptr;
        o.out.want_sources = sources != nullptr;
        for (;;) {
            uint32_t begin = next.fetch_add(64);
            if (begin >= n) break;
            uint32_t end = std::min(n, begin + 64);
            for (uint32_t i = begin; i < end; ++i) {
                o.out.vertices.clear();
                o.out.indices.clear();
                o.out.attributes.clear();
                o.out.sources.clear();
                o.near_ties = 0;
                uint32_t v0 = batch->verb_offsets[i], v1 = batch->verb_offsets[i + 1];
                uint32_t p0 = batch->point_offsets[i], p1 = batch->point_offsets[i + 1];
                int r;
                if (kind == 0) {
                    const lyon_stroke_options* so =
                        (const lyon_stroke_options*)options + (num_options > 1 ? i : 0);
                    if (widths) {
                        r = lyon_oracle_stroke_path_vw(&o, batch->verbs + v0, v1 - v0,
                                                       batch->points + 2 * (size_t)p0, p1 - p0,
                                                       widths + p0, so);
                    } else {
                        r = lyon_oracle_stroke_path(&o, batch->verbs + v0, v1 - v0,
                                                    batch->points + 2 * (size_t)p0, p1 - p0, so);
                    }
                } else {
                    const lyon_fill_options* fo =
                        (const lyon_fill_options*)options + (num_options > 1 ? i : 0);
                    r = lyon_oracle_fill_path(&o, batch->verbs + v0, v1 - v0,
                                              batch->points + 2 * (size_t)p0, p1 - p0, fo);
                }
                uint32_t nv = (uint32_t)(o.out.vertices.size() / 2);
                uint32_t ni = (uint32_t)o.out.indices.size();
                if (vtx_counts) vtx_counts[i] = nv;
                if (idx_counts) idx_counts[i] = ni;
                if (status) status[i] = r;
                if (near_ties) near_ties[i] = o.near_ties;
                if (vertices && vtx_offsets) {
                    std::memcpy(vertices + 2 * vtx_offsets[i], o.out.vertices.data(),
                                o.out.vertices.size() * sizeof(float));
                }
                if (indices && idx_offsets) {
                    std::memcpy(indices + idx_offsets[i], o.out.indices.data(),
                                o.out.indices.size() * sizeof(uint32_t));
                }
                if (attributes && vtx_offsets) {
                    std::memcpy(attributes + 4 * vtx_offsets[i], o.out.attributes.data(),
                                o.out.attributes.size() * sizeof(uint32_t));
                }
                if (sources && vtx_offsets) {
                    // Path-local endpoint ids made batch-global (indices into the batch's points).
                    uint32_t* d = sources + 3 * vtx_offsets[i];
                    for (size_t k = 0; k + 2 < o.out.sources.size(); k += 3) {
                        d[k] = o.out.sources[k] + p0;
                        d[k + 1] = o.out.sources[k + 1] == NO_ENDPOINT ? NO_ENDPOINT
                                                                        : o.out.sources[k + 1] + p0;
                        d[k + 2] = o.out.sources[k + 2];
                    }
                }
            }
        }
    };
    if (num_threads == 1) {
        worker();
    } else {
        std::vector<std::thread> th;
        for (int t = 0; t < num_threads; ++t) th.emplace_back(worker);
        for (auto& t : th) t.join();
    }
    return LYON_OK;
}

int lyon_oracle_batch(int kind, const lyon_path_batch* batch, const void* options,
                      uint32_t num_options, int index_bits, int num_threads,
                      uint32_t* vtx_counts, uint32_t* idx_counts, int32_t* status,
                      uint32_t* near_ties, float* vertices, uint32_t* indices,
                      const uint64_t* vtx_offsets, const uint64_t* idx_offsets) {
    return batch_impl(kind, batch, nullptr, options, num_options, index_bits, num_threads,
                      vtx_counts, idx_counts, status, near_ties, vertices, indices, vtx_offsets,
                      idx_offsets, nullptr);
}

// Batched stroke with a variable line width (`widths`: one factor per point of the batch) and,
// when `attributes` is set, the stroke vertex attributes (four words per vertex).
int lyon_oracle_batch_stroke_vw(const lyon_path_batch* batch, const float* widths,
                                const void* options, uint32_t num_options, int index_bits,
                                int num_threads, uint32_t* vtx_counts, uint32_t* idx_counts,
                                int32_t* status, uint32_t* near_ties, float* vertices,
                                uint32_t* indices, const uint64_t* vtx_offsets,
                                const uint64_t* idx_offsets, uint32_t* attributes) {
    return batch_impl(0, batch, widths, options, num_options, index_bits, num_threads,
                      vtx_counts, idx_counts, status, near_ties, vertices, indices, vtx_offsets,
                      idx_offsets, attributes);
}

// Batched stroke (fixed width when `widths` is NULL) recording every vertex's VertexSource
// (three words per vertex, endpoint ids indexing the batch's points) and, when `attributes` is
// set, the stroke vertex attributes.
int lyon_oracle_batch_stroke_sources(const lyon_path_batch* batch, const float* widths,
                                     const void* options, uint32_t num_options, int index_bits,
                                     int num_threads, uint32_t* vtx_counts, uint32_t* idx_counts,
                                     int32_t* status, float* vertices, uint32_t* indices,
                                     const uint64_t* vtx_offsets, const uint64_t* idx_offsets,
                                     uint32_t* attributes, uint32_t* sources) {
    return batch_impl(0, batch, widths, options, num_options, index_bits, num_threads,
                      vtx_counts, idx_counts, status, nullptr, vertices, indices, vtx_offsets,
                      idx_offsets, attributes, sources);
}

// Batched fill recording every vertex's sources. Counting call (outputs NULL): per-path vertex,
// index and source counts and statuses. Output call: vertices, indices (per-path ids), sources
// (three words each, ids indexing the batch's points) at the offsets of a counting call, and the
// number of sources of every vertex (at the vertex offsets).
int lyon_oracle_batch_fill_sources(const lyon_path_batch* batch, const void* options,
                                   uint32_t num_options, int index_bits, int num_threads,
                                   uint32_t* vtx_counts, uint32_t* idx_counts,
                                   uint32_t* src_counts, int32_t* status, float* vertices,
                                   uint32_t* indices, uint32_t* sources, uint32_t* source_counts,
                                   const uint64_t* vtx_offsets, const uint64_t* idx_offsets,
                                   const uint64_t* src_offsets) {
    uint32_t n = batch->num_paths;
    if (num_threads < 1) num_threads = 1;
    std::atomic<uint32_t> next{0};
    auto worker = [&]() {
        lyon_oracle_out o;
        o.out.max_index = index_bits == 16 ? 65535ull : 0xFFFFFFFEull;
        o.out.want_sources = true;
        for (;;) {
            uint32_t begin = next.fetch_add(64);
            if (begin >= n) break;
            uint32_t end = std::min(n, begin + 64);
            for (uint32_t i = begin; i < end; ++i) {
                lyon_oracle_out_clear(&o);
                uint32_t v0 = batch->verb_offsets[i], v1 = batch->verb_offsets[i + 1];
                uint32_t p0 = batch->point_offsets[i], p1 = batch->point_offsets[i + 1];
                const lyon_fill_options* fo =
                    (const lyon_fill_options*)options + (num_options > 1 ? i : 0);
                int r = lyon_oracle_fill_path(&o, batch->verbs + v0, v1 - v0,
                                              batch->points + 2 * (size_t)p0, p1 - p0, fo);
                const uint32_t nv = (uint32_t)(o.out.vertices.size() / 2);
                const size_t ns = o.out.fill_sources.size() / 3;
                if (vtx_counts) vtx_counts[i] = nv;
                if (idx_counts) idx_counts[i] = (uint32_t)o.out.indices.size();
                if (src_counts) src_counts[i] = (uint32_t)ns;
                if (status) status[i] = r;
                if (vertices && vtx_offsets)
                    std::memcpy(vertices + 2 * vtx_offsets[i], o.out.vertices.data(),
                                o.out.vertices.size() * sizeof(float));
                if (indices && idx_offsets)
                    std::memcpy(indices + idx_offsets[i], o.out.indices.data(),
                                o.out.indices.size() * sizeof(uint32_t));
                if (source_counts && vtx_offsets)
                    std::memcpy(source_counts + vtx_offsets[i], o.out.fill_source_counts.data(),
                                nv * sizeof(uint32_t));
                if (sources && src_offsets) {
                    uint32_t* d = sources + 3 * src_offsets[i];
                    for (size_t k = 0; k < ns; ++k) {
                        const uint32_t* w = o.out.fill_sources.data() + 3 * k;
                        d[3 * k] = w[0] + p0;
                        d[3 * k + 1] = w[1] == NO_ENDPOINT ? NO_ENDPOINT : w[1] + p0;
                        d[3 * k + 2] = w[2];
                    }
                }
            }
        }
    };
    std::vector<std::thread> th;
    for (int t = 1; t < num_threads; ++t) th.emplace_back(worker);
    worker();
    for (auto& t : th) t.join();
    return LYON_OK;
}

// FillVertex::interpolated_attributes (fill.rs:2208-2286) for `n` vertices whose sources are
// sources[offsets[v] .. offsets[v + 1]) (three words each): the first source's attributes
// (the endpoint's, or a * (1 - t) + b * t), the next ones added in order, then a division by
// the number of sources when there are several.
void lyon_oracle_interpolate_fill(const uint32_t* sources, const uint64_t* offsets, uint64_t n,
                                  const float* attrs, uint32_t na, float* out) {
    for (uint64_t v = 0; v < n; ++v) {
        float* o = out + v * na;
        float div = 1.0f;
        for (uint64_t k = offsets[v]; k < offsets[v + 1]; ++k) {
            const uint32_t* s = sources + 3 * k;
            float t;
            std::memcpy(&t, &s[2], 4);
            const float* a = attrs + (uint64_t)s[0] * na;
            const float* b = s[1] == NO_ENDPOINT ? nullptr : attrs + (uint64_t)s[1] * na;
            for (uint32_t i = 0; i < na; ++i) {
                const float x = b ? a[i] * (1.0f - t) + b[i] * t : a[i];
                o[i] = k == offsets[v] ? x : o[i] + x;
            }
            if (k != offsets[v]) div += 1.0f;
        }
        if (div > 1.0f)
            for (uint32_t i = 0; i < na; ++i) o[i] /= div;
    }
}

// StrokeVertex::interpolated_attributes (stroke.rs:2728-2747) for `n` vertex sources (three
// words each) over an attribute store of `na` floats per endpoint, on `num_threads` threads.
void lyon_oracle_interpolate(const uint32_t* sources, uint64_t n, const float* attrs, uint32_t na,
                             float* out, int num_threads) {
    if (num_threads < 1) num_threads = 1;
    auto work = [&](uint64_t v0, uint64_t v1) {
        for (uint64_t v = v0; v < v1; ++v) {
            const uint32_t* s = sources + 3 * v;
            float t;
            std::memcpy(&t, &s[2], 4);
            const float* a = attrs + (uint64_t)s[0] * na;
            float* o = out + v * na;
            if (s[1] == NO_ENDPOINT) {
                for (uint32_t i = 0; i < na; ++i) o[i] = a[i];
            } else {
                const float* b = attrs + (uint64_t)s[1] * na;
                for (uint32_t i = 0; i < na; ++i) o[i] = a[i] * (1.0f - t) + b[i] * t;
            }
        }
    };
    std::vector<std::thread> th;
    const uint64_t per = (n + num_threads - 1) / num_threads;
    for (int k = 1; k < num_threads; ++k) {
        const uint64_t v0 = std::min(n, per * k), v1 = std::min(n, per * (k + 1));
        th.emplace_back(work, v0, v1);
    }
    work(0, std::min(n, per));
    for (auto& t : th) t.join();
}

// The stroke vertex attributes of every path of a batch (four words per vertex, see
// lyon_oracle_out_set_attributes), written at `vtx_offsets` (from a counting call).
int lyon_oracle_batch_stroke_attributes(const lyon_path_batch* batch, const void* options,
                                        uint32_t num_options, int num_threads,
                                        const uint64_t* vtx_offsets, uint32_t* attributes) {
    uint32_t n = batch->num_paths;
    if (num_threads < 1) num_threads = 1;
    std::atomic<uint32_t> next{0};
    auto worker = [&]() {
        lyon_oracle_out o;
        o.out.want_attributes = true;
        for (;;) {
            uint32_t begin = next.fetch_add(64);
            if (begin >= n) break;
            uint32_t end = std::min(n, begin + 64);
            for (uint32_t i = begin; i < end; ++i) {
                o.out.vertices.clear();
                o.out.indices.clear();
                o.out.attributes.clear();
                uint32_t v0 = batch->verb_offsets[i], v1 = batch->verb_offsets[i + 1];
                uint32_t p0 = batch->point_offsets[i], p1 = batch->point_offsets[i + 1];
                const lyon_stroke_options* so =
                    (const lyon_stroke_options*)options + (num_options > 1 ? i : 0);
                lyon_oracle_stroke_path(&o, batch->verbs + v0, v1 - v0,
                                        batch->points + 2 * (size_t)p0, p1 - p0, so);
                std::memcpy(attributes + 4 * vtx_offsets[i], o.out.attributes.data(),
                            o.out.attributes.size() * sizeof(uint32_t));
            }
        }
    };
    std::vector<std::thread> th;
    for (int t = 1; t < num_threads; ++t) th.emplace_back(worker);
    worker();
    for (auto& t : th) t.join();
    return LYON_OK;
}

}  // extern "C"
