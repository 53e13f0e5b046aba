// stroke_core.cuh — lyon's fixed-width stroke logic for the GPU (crates/tessellation/src/stroke.rs).
//
// The per-join work of `fixed_width_step_impl` (stroke.rs:1521-1632) is split in three parts so
// that a warp can process 32 joins at once: geometry (side points, folds, single vertices),
// counts (vertices and indices, from which the warp scans output offsets), and emission through a
// Sink that writes vertices/indices at the scanned offsets. The sub-path tail (caps, closing,
// empty caps) runs sequentially on one lane with the same primitives.
#pragma once

#include "geom.cuh"

namespace lg {

constexpr uint32_t INVALID_ID = 0xFFFFFFFFu;
constexpr int SP = 0;  // SIDE_POSITIVE
constexpr int SN = 1;  // SIDE_NEGATIVE
// lyon recurses 2^depth - 1 times per arc (stroke.rs:2001-2004,2487-2490). A depth above this
// bound means more than a million vertices per arc (or, for a zero step, no end at all): the
// path then fails with LYON_ERR_UNSUPPORTED, identically in the oracle.
constexpr uint32_t MAX_ARC_DEPTH = 20;

struct SidePts {  // stroke.rs:300-307
    V2 prev, next, single;
    uint32_t prev_vertex, next_vertex;
    bool has_single;
};

struct DEP {  // EndpointData, stroke.rs:309-342
    V2 pos;
    float hw;
    float adv;  // advancement: NaN until computed (only the vertex attribute output reads it)
    int join;
    bool is_flat;
    bool fold[2];
    SidePts s[2];
};

__device__ __forceinline__ void dep_init(DEP& d, V2 pos, float hw, int join, bool flat) {
    d.pos = pos;
    d.hw = hw;
    d.adv = __int_as_float(0x7fc00000);
    d.join = join;
    d.is_flat = flat;
    d.fold[0] = d.fold[1] = false;
#pragma unroll
    for (int i = 0; i < 2; ++i) {
        d.s[i].prev = V2{__int_as_float(0x7fc00000), __int_as_float(0x7fc00000)};
        d.s[i].next = d.s[i].prev;
        d.s[i].single = V2{0.0f, 0.0f};
        d.s[i].prev_vertex = INVALID_ID;
        d.s[i].next_vertex = INVALID_ID;
        d.s[i].has_single = false;
    }
}

// Output sink: vertices get consecutive ids starting at `id_base`; when `vout`/`rout`/`iout`
// are null only the counters move (count pass). `vcap`/`icap` bound the writes to what the count
// pass measured for this sink's range, so a disagreement between the passes can never write
// outside the caller's buffers (it is reported through `overflow`). With `rout`, every vertex
// is a lyon_stroke_vertex record: the position, the normal and side the emission site gives and
// the advancement of the join or end being emitted (`adv`, set by the caller), as lyon's
// StrokeVertexData holds them when the vertex is added (stroke.rs:2656-2720).
template <bool REC>
struct SinkT {
    static constexpr bool kRec = REC;
    static constexpr bool kSrc = false;  // writes vertex sources (the sequential stepper's sink)
    uint32_t id_base;
    uint32_t nv, ni;
    float2* vout;
    void* iout;
    int index_bits;
    uint32_t vcap = 0xFFFFFFFFu, icap = 0xFFFFFFFFu;
    bool overflow = false;
    lyon_stroke_vertex* rout = nullptr;
    float adv = 0.0f;

    __device__ __forceinline__ uint32_t vertex(V2 p, V2 n, int side) {
        uint32_t id = id_base + nv;
        if constexpr (REC) {
            if (nv < vcap) {
                float2* d = reinterpret_cast<float2*>(rout + nv);
                d[0] = make_float2(p.x, p.y);
                d[1] = make_float2(n.x, n.y);
                d[2] = make_float2(adv, __uint_as_float((uint32_t)side));
            } else {
                overflow = true;
            }
        } else if (vout) {
            if (nv < vcap) vout[nv] = make_float2(p.x, p.y);
            else overflow = true;
        }
        ++nv;
        return id;
    }
    __device__ __forceinline__ void tri(uint32_t a, uint32_t b, uint32_t c) {
        if (iout && ni + 3 > icap) {
            overflow = true;
        } else if (iout) {
            if (index_bits == 16) {
                uint16_t* o = reinterpret_cast<uint16_t*>(iout) + ni;
                o[0] = (uint16_t)a;
                o[1] = (uint16_t)b;
                o[2] = (uint16_t)c;
            } else {
                uint32_t* o = reinterpret_cast<uint32_t*>(iout) + ni;
                o[0] = a;
                o[1] = b;
                o[2] = c;
            }
        }
        ni += 3;
    }
};
using Sink = SinkT<false>;     // positions
using RecSink = SinkT<true>;  // lyon_stroke_vertex records

struct StrokeParams {
    float hw;          // line_width * 0.5
    float miter_limit;
    float tolerance;
    float merge_threshold;  // square_merge_threshold, stroke.rs:603-605
    int line_join;
    int start_cap, end_cap;
};

__device__ __forceinline__ StrokeParams make_params(const lyon_stroke_options& o) {
    StrokeParams p;
    p.hw = o.line_width * 0.5f;
    p.miter_limit = o.miter_limit;
    p.tolerance = o.tolerance;
    p.merge_threshold = fmaxf(
        fminf(o.tolerance * o.tolerance * 0.5f, o.line_width * o.line_width * 0.05f), 1e-8f);
    p.line_join = o.line_join;
    p.start_cap = o.start_cap;
    p.end_cap = o.end_cap;
    return p;
}

__device__ __forceinline__ bool too_close(V2 a, V2 b, float thr) {  // stroke.rs:1318-1320
    return sqlen(a - b) < thr;
}

// math_utils.rs:16-40
__device__ __forceinline__ V2 compute_normal(V2 v1, V2 v2_) {
    const float epsilon = 1e-4f;
    V2 n1 = V2{-v1.y, v1.x};
    V2 v12 = v1 + v2_;
    if (sqlen(v12) < epsilon) return V2{0.0f, 0.0f};
    V2 tan = normalize(v12);
    V2 n = V2{-tan.y, tan.x};
    float inv_len = dot(n, n1);
    if (fabsf(inv_len) < epsilon) return n1;
    return n / inv_len;
}

// geom line.rs:562-578 with S = f64.
__device__ __forceinline__ bool line_intersection_f64(V2 p0, V2 v0, V2 p1, V2 v1, V2* out) {
    double p0x = p0.x, p0y = p0.y, v0x = v0.x, v0y = v0.y;
    double p1x = p1.x, p1y = p1.y, v1x = v1.x, v1y = v1.y;
    double det = v0x * v1y - v0y * v1x;
    if (fabs(det) <= 1e-8) return false;
    double inv_det = 1.0 / det;
    double s2x = p0x + v0x, s2y = p0y + v0y;
    double o2x = p1x + v1x, o2y = p1y + v1y;
    double a = p0x * s2y - p0y * s2x;
    double b = p1x * o2y - p1y * o2x;
    out->x = (float)((b * v0x - a * v1x) * inv_det);
    out->y = (float)((b * v0y - a * v1y) * inv_det);
    return true;
}

__device__ __forceinline__ bool miter_limit_exceeded(V2 n, float ml) {  // stroke.rs:2320-2322
    return sqlen(n) > ml * ml * 4.0f;
}

// stroke.rs:2279-2315
__device__ __forceinline__ void get_clip_intersections(V2 prev_n, V2 next_n, V2 normal,
                                                       float clip_distance, V2* i1, V2* i2) {
    V2 clip_pt = normalize(normal) * clip_distance;
    V2 clip_vec = perp(normal);
    if (!line_intersection_f64(clip_pt, clip_vec, prev_n, perp(prev_n), i1)) *i1 = normal;
    if (!line_intersection_f64(clip_pt, clip_vec, next_n, perp(next_n), i2)) *i2 = normal;
}

// Correctly rounded f32 transcendentals (f64 evaluation, one rounding).
__device__ __forceinline__ float cr_acos(float x) { return (float)acos((double)x); }
__device__ __forceinline__ float cr_cos(float x) { return (float)cos((double)x); }
__device__ __forceinline__ float cr_sin(float x) { return (float)sin((double)x); }
__device__ __forceinline__ float cr_asin(float x) { return (float)asin((double)x); }

// An arc's subdivision count is ceil(|diff| / step) (stroke.rs:1986-2004, 2482-2490, 2749-2753).
// diff comes from fast_atan2 and angle_to, identical on every platform; step = 2 acos(..) from
// an f32 libm whose last bit differs between platforms, which moves the quotient by an ulp or
// two. Within 2e-6 (relative) of an integer, step is re-evaluated correctly rounded, as the
// oracle does, so both take the same ceil (the oracle counts the quotients within 1e-6 of an
// integer as near ties: lyon on another libm may round those the other way).
__device__ __forceinline__ float arc_quotient(float adiff, float radius, float tol) {
    const float t = fminf(tol, radius);
    const float arg = (radius - t) / radius;
    const float x = adiff / (2.0f * acosf(arg));
    if (!(fabsf(x - rintf(x)) <= 2e-6f * fmaxf(1.0f, x))) return x;
    return adiff / (2.0f * cr_acos(arg));
}

// round(log2(ceil(x))) as u32 (stroke.rs:2003-2004).
__device__ __forceinline__ uint32_t depth_of(float x, int* status) {
    float num_segments = ceilf(x);
    uint32_t d = sat_u32(roundf(log2f(num_segments)));
    if (d > MAX_ARC_DEPTH) {
        *status = LYON_ERR_UNSUPPORTED;
        return 0;
    }
    return d;
}

// ---- join geometry ----------------------------------------------------------------------------

struct JoinGeo {
    bool fast;
    bool skip;
    V2 normal;  // fast path normal
};

// stroke.rs:1643-1733
__device__ __forceinline__ void compute_join_side_positions_fw(V2 prev_pos, DEP& join, V2 next_pos,
                                                               float miter_limit) {
    V2 prev_tangent = join.pos - prev_pos;
    V2 next_tangent = next_pos - join.pos;
    float prev_length = vlength(prev_tangent);
    float next_length = vlength(next_tangent);
    prev_tangent = prev_tangent / prev_length;
    next_tangent = next_tangent / next_length;
    float hw = join.hw;
    V2 normal = compute_normal(prev_tangent, next_tangent);
    int front_side;
    V2 front_normal;
    if (cross(prev_tangent, next_tangent) >= 0.0f) {
        front_side = SN;
        front_normal = -normal;
    } else {
        front_side = SP;
        front_normal = normal;
    }
    int back_side = 1 - front_side;
    V2 extruded_normal = front_normal * hw;
    bool unclipped_miter = (join.join == LYON_JOIN_MITER || join.join == LYON_JOIN_MITER_CLIP) &&
                           !miter_limit_exceeded(front_normal, miter_limit);
    bool fold = false;
    bool angle_is_sharp = dot(next_tangent, prev_tangent) < 0.0f;
    if (!unclipped_miter && angle_is_sharp) {
        float d_next = dot(extruded_normal, -next_tangent) - next_length;
        float d_prev = dot(extruded_normal, prev_tangent) - prev_length;
        if (fminf(d_next, d_prev) > 0.0f || sqlen(normal) < 1e-5f) {
            join.fold[front_side] = true;
            fold = true;
        }
    }
    V2 n0 = V2{-prev_tangent.y, prev_tangent.x} * hw;
    V2 n1 = V2{-next_tangent.y, next_tangent.x} * hw;
    join.s[SP].prev = join.pos + n0;
    join.s[SP].next = join.pos + n1;
    join.s[SN].prev = join.pos - n0;
    join.s[SN].next = join.pos - n1;
    if (!fold) {
        V2 mp = join.pos + normal * hw;
        V2 mn = join.pos - normal * hw;
        join.s[back_side].has_single = true;
        join.s[back_side].single = back_side == SP ? mp : mn;
        if (unclipped_miter) {
            join.s[front_side].has_single = true;
            join.s[front_side].single = front_side == SP ? mp : mn;
        } else if (join.join == LYON_JOIN_MITER_CLIP) {
            V2 a = join.s[front_side].prev - join.pos;
            V2 b = join.s[front_side].next - join.pos;
            V2 pn, nn;
            get_clip_intersections(a, b, front_normal, miter_limit * hw, &pn, &nn);
            join.s[front_side].prev = join.pos + pn;
            join.s[front_side].next = join.pos + nn;
        }
    }
}

// Geometry of the join at `join` (stroke.rs:1559-1608 up to the vertex emission). The fast path
// (stroke.rs:1743-1806) needs the previous join's side points for its skip test; callers that
// process joins in parallel pass them after exchanging them (see flattened_skip).
__device__ __forceinline__ JoinGeo join_geometry(V2 prev_pos, DEP& join, V2 next_pos,
                                                 float miter_limit) {
    JoinGeo g;
    g.fast = false;
    g.skip = false;
    g.normal = V2{0.0f, 0.0f};
    if (join.is_flat) {
        V2 v0 = join.pos - prev_pos;
        V2 v1 = next_pos - join.pos;
        g.fast = dot(v0, v1) > 0.0f;
    }
    if (g.fast) {
        join.join = LYON_JOIN_MITER;
        V2 prev_edge = join.pos - prev_pos;
        float prev_length = vlength(prev_edge);
        V2 prev_tangent = prev_edge / prev_length;
        V2 next_edge = next_pos - join.pos;
        float next_length = vlength(next_edge);
        V2 next_tangent = next_edge / next_length;
        V2 normal = compute_normal(prev_tangent, next_tangent);
        V2 p0 = join.pos + normal * join.hw;
        V2 p1 = join.pos - normal * join.hw;
        join.s[SP].prev = p0;
        join.s[SP].next = p0;
        join.s[SP].single = p0;
        join.s[SP].has_single = true;
        join.s[SN].prev = p1;
        join.s[SN].next = p1;
        join.s[SN].single = p1;
        join.s[SN].has_single = true;
        g.normal = normal;
    } else {
        compute_join_side_positions_fw(prev_pos, join, next_pos, miter_limit);
    }
    return g;
}

// The skip test of flattened_step (stroke.rs:1785-1789), given the previous join's side points.
__device__ __forceinline__ bool flattened_skip(V2 prev_pos, V2 prev_pos_next, V2 prev_neg_next,
                                               const DEP& join) {
    V2 prev_edge = join.pos - prev_pos;
    V2 v0 = join.s[SP].single - prev_pos_next;
    V2 v1 = join.s[SN].single - prev_neg_next;
    return dot(prev_edge, v0) < 0.0f && dot(prev_edge, v1) < 0.0f;
}

__device__ __forceinline__ void side_needs_join(const DEP& j, bool out[2]) {  // stroke.rs:1914-1917
    out[SP] = !j.s[SP].has_single && !j.fold[SN];
    out[SN] = !j.s[SN].has_single && !j.fold[SP];
}

// Number of interior join triangles (stroke.rs:1919-1950).
__device__ __forceinline__ uint32_t join_interior_tris(const DEP& j) {
    if (j.fold[SP] || j.fold[SN]) return 0;
    bool nj[2];
    side_needs_join(j, nj);
    if (nj[SP] && nj[SN]) return 2;
    if (nj[SP] != nj[SN]) return 1;
    return 0;
}

// Round join arc of one side (stroke.rs:1968-2021): angles and subdivision depth.
struct ArcPlan {
    float a0, a1;
    uint32_t depth;
    int st;  // LYON_OK, or LYON_ERR_UNSUPPORTED for a depth past MAX_ARC_DEPTH
};

// Out of line with its inputs and result by value, so that no caller's join is kept in local
// memory for it.
static __device__ __noinline__ ArcPlan round_join_plan(V2 center, float radius, V2 side_prev,
                                                       V2 side_next, int side, float tol) {
    V2 sn = side_prev - center;
    V2 en = side_next - center;
    float angle_sign = side == SN ? 1.0f : -1.0f;
    const float start_angle = angle_from_x_axis(sn);
    float diff = angle_to(start_angle, angle_from_x_axis(en));
    if (diff * angle_sign < 0.0f) diff = angle_sign * (2.0f * LG_PI_F - fabsf(diff));
    const float end_angle = start_angle + diff;
    ArcPlan p;
    p.st = LYON_OK;
    if (side == SN) {
        p.a0 = end_angle;
        p.a1 = start_angle;
    } else {
        p.a0 = start_angle;
        p.a1 = end_angle;
    }
    p.depth = depth_of(arc_quotient(fabsf(diff), radius, tol), &p.st);
    return p;
}

__device__ __forceinline__ ArcPlan join_arc_plan(const DEP& j, int side, float tol, int* status) {
    const ArcPlan a = round_join_plan(j.pos, j.hw, j.s[side].prev, j.s[side].next, side, tol);
    if (a.st != LYON_OK) *status = a.st;
    return a;
}

__device__ __forceinline__ uint32_t arc_vertex_count(uint32_t depth) {
    return depth == 0 ? 0u : ((1u << depth) - 1u);
}

// stroke.rs:2612-2653. lyon's recursion visits a perfect binary tree of `depth` levels in
// pre-order: each node emits the vertex at the middle of its angle range (the halving of its
// parent's range) and the triangle (range start vertex, it, range end vertex), then recurses into
// the lower half and the upper half. Node k of the pre-order is found by descending from the
// root, halving the range exactly as the recursion does, so the angles are the recursion's bit
// for bit. Vertices get consecutive ids in pre-order, so an ancestor's id is the first arc
// vertex's id plus its pre-order index. No per-lane stack: everything stays in registers (the
// sink is taken and returned by value for the same reason).
template <class SK>
__device__ __noinline__ SK tessellate_arc(V2 center, float radius, float a0, float a1, uint32_t va,
                                          uint32_t vb, uint32_t depth, int side, SK sink) {
    if (depth == 0) return sink;
    const uint32_t total = (1u << depth) - 1u;
    uint32_t first_id = 0;
    for (uint32_t k = 0; k < total; ++k) {
        float lo = a0, hi = a1;
        uint32_t ilo = va, ihi = vb;
        uint32_t p = 0;      // pre-order index of the node reached
        uint32_t n = depth;  // levels of its subtree
        float mid = (lo + hi) * 0.5f;
        while (p != k) {
            // The lower half's subtree holds 2^(n-1) - 1 nodes, so the upper half starts at
            // p + 2^(n-1).
            const uint32_t upper = p + (1u << (n - 1));
            if (k < upper) {
                hi = mid;
                ihi = first_id + p;
                p += 1;
            } else {
                lo = mid;
                ilo = first_id + p;
                p = upper;
            }
            --n;
            mid = (lo + hi) * 0.5f;
        }
        V2 normal = V2{cosf(mid), sinf(mid)};
        uint32_t vid = sink.vertex(center + normal * radius, normal, side);
        if (k == 0) first_id = vid;
        sink.tri(ilo, vid, ihi);
    }
    return sink;
}

// ---- emission ---------------------------------------------------------------------------------

// stroke.rs:2024-2055
template <class SK>
__device__ __forceinline__ void add_join_base_vertices(DEP& j, int side, SK& sink) {
    if (j.s[side].has_single) {
        V2 normal = (j.s[side].single - j.pos) / j.hw;
        uint32_t v = sink.vertex(j.pos + normal * j.hw, normal, side);
        j.s[side].prev_vertex = v;
        j.s[side].next_vertex = v;
    } else {
        V2 n0 = (j.s[side].prev - j.pos) / j.hw;
        uint32_t pv = sink.vertex(j.pos + n0 * j.hw, n0, side);
        V2 n1 = (j.s[side].next - j.pos) / j.hw;
        uint32_t nv = sink.vertex(j.pos + n1 * j.hw, n1, side);
        j.s[side].prev_vertex = pv;
        j.s[side].next_vertex = nv;
    }
}

// Base vertices of a join: fast path +,- (stroke.rs:1791-1797) or regular -,+ (:1595-1608).
template <class SK>
__device__ __forceinline__ void emit_join_base(DEP& j, const JoinGeo& g, SK& sink) {
    if (g.fast) {
        if (g.skip) return;
        uint32_t pv = sink.vertex(j.pos + g.normal * j.hw, g.normal, SP);
        uint32_t nv = sink.vertex(j.pos + (-g.normal) * j.hw, -g.normal, SN);
        j.s[SP].prev_vertex = pv;
        j.s[SP].next_vertex = pv;
        j.s[SN].prev_vertex = nv;
        j.s[SN].next_vertex = nv;
    } else {
        add_join_base_vertices(j, SN, sink);
        add_join_base_vertices(j, SP, sink);
    }
}

__device__ __forceinline__ uint32_t join_base_vertex_count(const DEP& j, const JoinGeo& g) {
    if (g.fast) return g.skip ? 0u : 2u;
    return (j.s[SN].has_single ? 1u : 2u) + (j.s[SP].has_single ? 1u : 2u);
}

// Ids an edge (p0 -> p1) uses, after the fold substitutions of stroke.rs:1874-1889.
struct EdgeIds {
    uint32_t p0_neg, p0_pos;
};
__device__ __forceinline__ void edge_ids_from(const DEP& p0, uint32_t* neg, uint32_t* pos) {
    *neg = p0.fold[SP] ? p0.s[SP].prev_vertex : p0.s[SN].next_vertex;
    *pos = p0.fold[SN] ? p0.s[SN].prev_vertex : p0.s[SP].next_vertex;
}
__device__ __forceinline__ void edge_ids_to(const DEP& p1, uint32_t* neg, uint32_t* pos) {
    *neg = p1.fold[SP] ? p1.s[SP].next_vertex : p1.s[SN].prev_vertex;
    *pos = p1.fold[SN] ? p1.s[SN].next_vertex : p1.s[SP].prev_vertex;
}

// stroke.rs:1869-1904 on already-resolved ids. Returns the number of triangles.
template <class SK>
__device__ __forceinline__ uint32_t edge_triangles(uint32_t p0_neg, uint32_t p0_pos,
                                                   uint32_t p1_neg, uint32_t p1_pos, SK* sink) {
    if (p0_neg == p1_pos) return 0;
    uint32_t n = 0;
    if (p0_neg != p0_pos && p0_pos != p1_pos) {
        if (sink) sink->tri(p0_neg, p0_pos, p1_pos);
        ++n;
    }
    if (p0_neg != p1_neg && p1_pos != p1_neg) {
        if (sink) sink->tri(p0_neg, p1_pos, p1_neg);
        ++n;
    }
    return n;
}

template <class SK>
__device__ __forceinline__ void add_edge_triangles(const DEP& p0, const DEP& p1, SK& sink) {
    uint32_t a, b, c, d;
    edge_ids_from(p0, &a, &b);
    edge_ids_to(p1, &c, &d);
    edge_triangles(a, b, c, d, &sink);
}

// stroke.rs:1907-1965 (interior triangles then round arcs).
template <class SK>
__device__ __forceinline__ void tessellate_join(const DEP& j, const StrokeParams& P, SK& sink,
                                                int* status) {
    bool nj[2];
    side_needs_join(j, nj);
    if (!j.fold[SP] && !j.fold[SN]) {
        const SidePts& sp = j.s[SP];
        const SidePts& sn = j.s[SN];
        if (nj[SP] && nj[SN]) {
            sink.tri(sp.prev_vertex, sp.next_vertex, sn.next_vertex);
            sink.tri(sp.prev_vertex, sn.next_vertex, sn.prev_vertex);
        } else if (!nj[SP] && nj[SN]) {
            sink.tri(sn.prev_vertex, sp.prev_vertex, sn.next_vertex);
        } else if (nj[SP] && !nj[SN]) {
            sink.tri(sn.prev_vertex, sp.prev_vertex, sp.next_vertex);
        }
    }
    if (j.join == LYON_JOIN_ROUND) {
        for (int side = 0; side < 2; ++side) {
            if (!nj[side]) continue;
            ArcPlan a = join_arc_plan(j, side, P.tolerance, status);
            uint32_t va = side == SN ? j.s[side].next_vertex : j.s[side].prev_vertex;
            uint32_t vb = side == SN ? j.s[side].prev_vertex : j.s[side].next_vertex;
            sink = tessellate_arc(j.pos, j.hw, a.a0, a.a1, va, vb, a.depth, side, sink);
        }
    }
}

// Vertex and triangle counts of tessellate_join's arcs (0 unless the join is round).
__device__ __forceinline__ uint32_t join_arc_vertices(const DEP& j, const StrokeParams& P,
                                                      int* status) {
    if (j.join != LYON_JOIN_ROUND) return 0;
    bool nj[2];
    side_needs_join(j, nj);
    uint32_t n = 0;
    for (int side = 0; side < 2; ++side) {
        if (!nj[side]) continue;
        ArcPlan a = join_arc_plan(j, side, P.tolerance, status);
        n += arc_vertex_count(a.depth);
    }
    return n;
}

// stroke.rs:2459-2524. Sink and status are taken and returned by value (see tessellate_arc).
template <class SK>
struct CapOut {
    SK sink;
    int st;
};
template <class SK>
__device__ __noinline__ CapOut<SK> tessellate_round_cap_v(V2 center, float radius, V2 start_normal,
                                                          uint32_t start_vertex,
                                                          uint32_t end_vertex, V2 edge_normal,
                                                          bool is_start, float tolerance, SK sink) {
    int st = LYON_OK;
    if (radius < tolerance) return CapOut<SK>{sink, st};
    const int first_side = (is_start ^ (cross(edge_normal, start_normal) >= 0.0f)) ? SP : SN;
    const float start_angle = angle_from_x_axis(start_normal);
    const float diff = angle_to(start_angle, angle_from_x_axis(edge_normal));
    const float mid_angle = start_angle + diff;
    const float end_angle = mid_angle + diff;
    const uint32_t depth = depth_of(arc_quotient(fabsf(diff), radius, tolerance), &st);
    const V2 mid_normal = normalize(edge_normal);
    uint32_t mid_vertex = sink.vertex(center + mid_normal * radius, mid_normal, first_side);
    sink.tri(start_vertex, mid_vertex, end_vertex);
    sink = tessellate_arc(center, radius, start_angle, mid_angle, start_vertex, mid_vertex, depth,
                          first_side, sink);
    sink = tessellate_arc(center, radius, mid_angle, end_angle, mid_vertex, end_vertex, depth,
                          1 - first_side, sink);
    return CapOut<SK>{sink, st};
}

template <class SK>
__device__ __forceinline__ void tessellate_round_cap(V2 center, float radius, V2 start_normal,
                                                     uint32_t start_vertex, uint32_t end_vertex,
                                                     V2 edge_normal, bool is_start,
                                                     const StrokeParams& P, SK& sink,
                                                     int* status) {
    const CapOut<SK> r = tessellate_round_cap_v(center, radius, start_normal, start_vertex,
                                                end_vertex, edge_normal, is_start, P.tolerance,
                                                sink);
    sink = r.sink;
    if (r.st != LYON_OK) *status = r.st;
}

// stroke.rs:2526-2560
template <class SK>
__device__ __forceinline__ void tessellate_empty_square_cap(V2 pos, float hw, SK& sink) {
    uint32_t a = sink.vertex(pos + V2{1.0f, 1.0f} * hw, V2{1.0f, 1.0f}, SN);
    uint32_t b = sink.vertex(pos + V2{1.0f, -1.0f} * hw, V2{1.0f, -1.0f}, SP);
    uint32_t c = sink.vertex(pos + V2{-1.0f, -1.0f} * hw, V2{-1.0f, -1.0f}, SP);
    uint32_t d = sink.vertex(pos + V2{-1.0f, 1.0f} * hw, V2{-1.0f, 1.0f}, SN);
    sink.tri(a, b, c);
    sink.tri(a, c, d);
}

// stroke.rs:2562-2609
template <class SK>
__device__ __forceinline__ void tessellate_empty_round_cap(V2 center, float hw,
                                                           const StrokeParams& P, SK& sink,
                                                           int* status) {
    uint32_t left_id = sink.vertex(center + V2{-1.0f, 0.0f} * hw, V2{-1.0f, 0.0f}, SP);
    uint32_t right_id = sink.vertex(center + V2{1.0f, 0.0f} * hw, V2{1.0f, 0.0f}, SN);
    tessellate_round_cap(center, hw, V2{-1.0f, 0.0f}, left_id, right_id, V2{0.0f, 1.0f}, true, P,
                         sink, status);
    tessellate_round_cap(center, hw, V2{1.0f, 0.0f}, right_id, left_id, V2{0.0f, -1.0f}, false,
                         P, sink, status);
}

// stroke.rs:2130-2206
template <class SK>
__device__ __forceinline__ void tessellate_last_edge(const DEP& p0, DEP& p1, bool is_first_edge,
                                                     const StrokeParams& P, SK& sink,
                                                     int* status) {
    V2 v = p1.pos - p0.pos;
    if constexpr (SK::kRec) {
        p1.adv = p0.adv + vlength(v);
        sink.adv = p1.adv;
    }
    for (int side = 0; side < 2; ++side) {
        V2 side_position = p1.s[side].prev;
        if (P.end_cap == LYON_CAP_SQUARE || P.end_cap == LYON_CAP_BUTT) {
            float clip = P.end_cap == LYON_CAP_SQUARE ? p1.hw : 0.0f;
            V2 normal = normalize(p1.pos - p0.pos);
            V2 clip_pt = p1.pos + normal * clip;
            V2 r;
            if (line_intersection_f64(clip_pt, perp(normal), side_position,
                                      side_position - p0.s[side].next, &r)) {
                p1.s[side].prev = r;
            }
        }
        V2 normal = (p1.s[side].prev - p1.pos) / p1.hw;
        p1.s[side].prev_vertex = sink.vertex(p1.pos + normal * p1.hw, normal, side);
    }
    if (!is_first_edge) add_edge_triangles(p0, p1, sink);
    if (P.end_cap == LYON_CAP_ROUND) {
        tessellate_round_cap(p1.pos, p1.hw, p1.s[SP].prev - p1.pos, p1.s[SP].prev_vertex,
                             p1.s[SN].prev_vertex, v, false, P, sink, status);
    }
}

// stroke.rs:2208-2276
template <class SK>
__device__ __forceinline__ void tessellate_first_edge(DEP& first, const DEP& second,
                                                      const StrokeParams& P, SK& sink,
                                                      int* status) {
    sink.adv = first.adv;
    for (int side = 0; side < 2; ++side) {
        V2 side_position = first.s[side].next;
        if (P.start_cap == LYON_CAP_SQUARE || P.start_cap == LYON_CAP_BUTT) {
            float clip = P.start_cap == LYON_CAP_SQUARE ? first.hw : 0.0f;
            V2 normal = normalize(first.pos - second.pos);
            V2 clip_pt = first.pos + normal * clip;
            V2 r;
            if (line_intersection_f64(clip_pt, perp(normal), side_position,
                                      side_position - second.s[side].prev, &r)) {
                side_position = r;
            } else {
                side_position = first.s[side].next;
            }
        }
        V2 normal = (side_position - first.pos) / first.hw;
        first.s[side].next_vertex = sink.vertex(first.pos + normal * first.hw, normal, side);
    }
    add_edge_triangles(first, second, sink);
    if (P.start_cap == LYON_CAP_ROUND) {
        tessellate_round_cap(first.pos, first.hw, first.s[SN].next - first.pos,
                             first.s[SN].next_vertex, first.s[SP].next_vertex,
                             first.pos - second.pos, true, P, sink, status);
    }
}

// Sets the side "next" points of the first point of a sub-path from its first edge
// (stroke.rs:1538-1556).
__device__ __forceinline__ void first_point_sides(DEP& first, V2 next_pos, float next_hw) {
    V2 edge = next_pos - first.pos;
    float len = vlength(edge);
    V2 tan = edge / len;
    V2 n = V2{-tan.y, tan.x} * next_hw;
    first.s[SP].next = first.pos + n;
    first.s[SN].next = first.pos - n;
}

// ---- parallel join processing: summaries exchanged between neighbouring joins -------------

// Which ids an edge uses at one of its ends (after fold substitutions): flags for the
// structural edge-triangle count (ids of different joins never coincide unless both invalid).
enum : uint32_t { EF_NEG_INV = 1u, EF_POS_INV = 2u, EF_SELF_EQ = 4u };

__device__ __forceinline__ uint32_t id_flags(uint32_t neg, uint32_t pos) {
    return (neg == INVALID_ID ? EF_NEG_INV : 0u) | (pos == INVALID_ID ? EF_POS_INV : 0u) |
           (neg == pos ? EF_SELF_EQ : 0u);
}

// Number of triangles add_edge_triangles (stroke.rs:1869-1904) emits for an edge whose ends have
// the given id structures.
__device__ __forceinline__ uint32_t edge_count_flags(uint32_t from_f, uint32_t to_f) {
    bool p0_neg_inv = from_f & EF_NEG_INV, p0_pos_inv = from_f & EF_POS_INV;
    bool p0_self_eq = from_f & EF_SELF_EQ;
    bool p1_neg_inv = to_f & EF_NEG_INV, p1_pos_inv = to_f & EF_POS_INV;
    bool p1_self_eq = to_f & EF_SELF_EQ;
    if (p0_neg_inv && p1_pos_inv) return 0;
    uint32_t n = 0;
    if (!p0_self_eq && !(p0_pos_inv && p1_pos_inv)) ++n;
    if (!(p0_neg_inv && p1_neg_inv) && !p1_self_eq) ++n;
    return n;
}

// Result of the general (non flattening-step) join geometry.
struct SlowJoin {
    V2 pn, nn;           // side "next" points (for the following join's skip test)
    uint32_t from_f, to_f;
    uint32_t from_neg_rel, from_pos_rel;  // ids relative to the join's first vertex (or INVALID)
    uint32_t vcount;     // base + arc vertices
    uint32_t jtris;      // interior + arc triangles
    bool sym;            // side next points symmetric about the join point
    int st;              // LYON_OK or the arcs' LYON_ERR_UNSUPPORTED
};

// stroke.rs:1586-1608 for a join that is not a flattening step: side positions and folds.
__device__ __forceinline__ DEP general_join_geometry(V2 prev, V2 cur, bool flat, V2 nxt,
                                                     const StrokeParams& P) {
    DEP J;
    dep_init(J, cur, P.hw, P.line_join, flat);
    compute_join_side_positions_fw(prev, J, nxt, P.miter_limit);
    return J;
}

// The counts and id layout of a general join. Out of line with its inputs and result by value:
// the join itself stays in the callee's registers (a join written through a pointer would live
// in local memory, in the caller's frame).
static __device__ __noinline__ SlowJoin slow_join_summary(V2 prev, V2 cur, bool flat, V2 nxt,
                                                          StrokeParams P) {
    DEP J = general_join_geometry(prev, cur, flat, nxt, P);
    SlowJoin r;
    r.st = LYON_OK;
    Sink probe{0u, 0, 0, nullptr, nullptr, 32};
    DEP K = J;
    add_join_base_vertices(K, SN, probe);
    add_join_base_vertices(K, SP, probe);
    uint32_t a, b;
    edge_ids_from(K, &a, &b);
    r.from_neg_rel = a;
    r.from_pos_rel = b;
    r.from_f = id_flags(a, b);
    edge_ids_to(K, &a, &b);
    r.to_f = id_flags(a, b);
    uint32_t varc = join_arc_vertices(J, P, &r.st);
    r.vcount = probe.nv + varc;
    r.jtris = join_interior_tris(J) + varc;
    r.pn = J.s[SP].next;
    r.nn = J.s[SN].next;
    // Only a clipped miter moves one side's points off the symmetric offsets.
    r.sym = J.join != LYON_JOIN_MITER_CLIP;
    return r;
}

// Emission of a general join: its geometry (the same operations on the same points as
// slow_join_summary), base vertices (- then +), the edge triangles from the previous join, then
// tessellate_join. The sink is taken by value and its counters returned.
struct JoinEmitOut {
    uint32_t nv, ni;
    bool overflow;
    int st;
};
template <class SK>
__device__ __noinline__ JoinEmitOut slow_join_emit_at(V2 prev, V2 cur, bool flat, V2 nxt,
                                                      StrokeParams P, SK s, bool has_edge,
                                                      uint32_t pfn, uint32_t pfp) {
    DEP J = general_join_geometry(prev, cur, flat, nxt, P);
    int st = LYON_OK;
    add_join_base_vertices(J, SN, s);
    add_join_base_vertices(J, SP, s);
    if (has_edge) {
        uint32_t c, d;
        edge_ids_to(J, &c, &d);
        edge_triangles(pfn, pfp, c, d, &s);
    }
    tessellate_join(J, P, s, &st);
    return JoinEmitOut{s.nv, s.ni, s.overflow, st};
}

// The join of a flattening step (stroke.rs:1743-1806) as a DEP, for the tail.
__device__ __forceinline__ void fast_join_dep(DEP& d, V2 cur, float hw, V2 pn, V2 nn,
                                              uint32_t pos_id, uint32_t neg_id) {
    dep_init(d, cur, hw, LYON_JOIN_MITER, true);
    d.s[SP].prev = d.s[SP].next = d.s[SP].single = pn;
    d.s[SP].has_single = true;
    d.s[SN].prev = d.s[SN].next = d.s[SN].single = nn;
    d.s[SN].has_single = true;
    d.s[SP].prev_vertex = d.s[SP].next_vertex = pos_id;
    d.s[SN].prev_vertex = d.s[SN].next_vertex = neg_id;
}

// A three-point buffer and the sequential fixed_width_step_impl (stroke.rs:1521-1632), used by
// the sub-path tail on one lane.
struct SeqBuffer {
    DEP pts[3];
    uint32_t start, count;  // count saturates at 3 entries stored; `n` is the logical count
    uint32_t n;
    __device__ __forceinline__ DEP& last() { return pts[(start + (count - 1)) % 3]; }
    __device__ __forceinline__ DEP& second_last() { return pts[(start + count - 2) % 3]; }
    __device__ __forceinline__ void push(const DEP& p) {
        if (count < 3) {
            pts[count] = p;
            ++count;
        } else {
            pts[start] = p;
            start = (start + 1) % 3;
        }
        ++n;
    }
    __device__ __forceinline__ DEP& first() { return pts[start % 3]; }
    // PointBuffer::replace_last (stroke.rs:2400-2406).
    __device__ __forceinline__ void replace_last(const DEP& p) {
        const uint32_t idx = start == 0 ? count : start;
        pts[idx - 1] = p;
    }
};

template <class SK>
__device__ __noinline__ bool seq_step(SeqBuffer& pb, DEP next, const StrokeParams& P, SK& sink,
                                      bool* may_need_empty_cap, int* status) {
    uint32_t count = pb.n;
    if (count > 0) {
        if (too_close(pb.last().pos, next.pos, P.merge_threshold)) {
            if (count == 1) *may_need_empty_cap = true;
            return false;
        }
        if (count == 1) {
            DEP& first = pb.last();
            first_point_sides(first, next.pos, next.hw);
            if (SK::kRec && isnan(next.adv)) next.adv = first.adv + vlength(next.pos - first.pos);
        }
    }
    if (count > 1) {
        DEP& prev = pb.second_last();
        DEP& join = pb.last();
        // Advancements (stroke.rs:1657-1662, 1759-1771): the join's from its predecessor, and
        // on a flattening step the next point's from the join.
        if (SK::kRec && isnan(join.adv)) join.adv = prev.adv + vlength(join.pos - prev.pos);
        JoinGeo g = join_geometry(prev.pos, join, next.pos, P.miter_limit);
        if (SK::kRec && g.fast && isnan(next.adv))
            next.adv = join.adv + vlength(next.pos - join.pos);
        sink.adv = join.adv;
        if (g.fast) g.skip = flattened_skip(prev.pos, prev.s[SP].next, prev.s[SN].next, join);
        emit_join_base(join, g, sink);
        if (count > 2) add_edge_triangles(prev, join, sink);
        tessellate_join(join, P, sink, status);
    }
    pb.push(next);
    return true;
}


// ---- variable line width (StrokeOptions::variable_line_width) -------------------------------
// One thread strokes a whole path with lyon's sequential variable-width stepper. The edge angle
// is euclid's fast_atan2, as lyon's; the attachment angles' asin/cos/sin are evaluated in f64
// with one rounding (cr_*), as in the oracle (lyon takes them from the platform's f32 libm).

struct VwState {
    SeqBuffer pb;
    DEP firsts[2];
    uint32_t nfirsts;
    bool mnec;          // may_need_empty_cap
    float start_adv;    // sub_path_start_advancement
};

// stroke.rs:1842-1866
__device__ __forceinline__ void vw_side_attachment(DEP& p0, DEP& p1, float edge_angle,
                                                   float vwidth_angle, int side) {
    const float nl = side == SN ? -1.0f : 1.0f;
    const float normal_angle = edge_angle + nl * (LG_PI_F * 0.5f + vwidth_angle);
    const V2 normal = V2{cr_cos(normal_angle), cr_sin(normal_angle)};
    p0.s[side].next = p0.pos + normal * p0.hw;
    p1.s[side].prev = p1.pos + normal * p1.hw;
}

// stroke.rs:1808-1840
static __device__ __noinline__ void vw_edge_attachments(DEP& p0, DEP& p1) {
    const V2 edge = p1.pos - p0.pos;
    const float d = vlength(edge);
    const float edge_angle = angle_from_x_axis(edge);  // stroke.rs:1812
    const float sin_vwidth_angle = (p1.hw - p0.hw) / d;
    float vwidth_angle = cr_asin(sin_vwidth_angle);
    if (isnan(vwidth_angle)) vwidth_angle = 0.0f;
    vw_side_attachment(p0, p1, edge_angle, vwidth_angle, SP);
    vw_side_attachment(p0, p1, edge_angle, vwidth_angle, SN);
    if (isnan(p1.adv)) p1.adv = p0.adv + d;
}

// stroke.rs:2060-2128
static __device__ __noinline__ void vw_join_sides(const DEP& prev, DEP& join, const DEP& next,
                                           float miter_limit, int side) {
    const float sign = side == SN ? -1.0f : 1.0f;
    const V2 v0 = normalize(join.s[side].prev - prev.s[side].next);
    const V2 v1 = normalize(next.s[side].prev - join.s[side].next);
    const bool inward = cross(v0, v1) * sign > 0.0f;
    const bool forward = dot(v0, v1) > 0.0f;
    const V2 normal = compute_normal(v0, v1) * sign;
    const V2 path_v0 = normalize(join.pos - prev.pos);
    const V2 path_v1 = normalize(next.pos - join.pos);
    const bool normal_same_side = dot(v0 + v1, path_v0 + path_v1) >= 0.0f;
    const bool angle_is_sharp = inward && !forward && normal_same_side;
    if (angle_is_sharp) {
        const V2 extruded_normal = normal * join.hw;
        const float prev_length = join.adv - prev.adv;
        const float next_length = next.adv - join.adv;
        const float d_next = dot(extruded_normal, v1) - next_length;
        const float d_prev = dot(extruded_normal, -v0) - prev_length;
        if (fminf(d_next, d_prev) > 0.0f || sqlen(normal) < 1e-5f) join.fold[side] = true;
    }
    const bool concave = inward && normal_same_side && !join.fold[side];
    if (concave || ((join.join == LYON_JOIN_MITER || join.join == LYON_JOIN_MITER_CLIP) &&
                    !miter_limit_exceeded(normal, miter_limit))) {
        join.s[side].has_single = true;
        join.s[side].single = join.pos + normal * join.hw;
    } else if (join.join == LYON_JOIN_MITER_CLIP) {
        const V2 n0 = join.s[side].prev - join.pos;
        const V2 n1 = join.s[side].next - join.pos;
        V2 pn, nn;
        get_clip_intersections(n0, n1, normal, miter_limit * join.hw, &pn, &nn);
        join.s[side].prev = join.pos + pn;
        join.s[side].next = join.pos + nn;
    }
}

// step_impl (stroke.rs:1380-1512). Returns false when `next` merged into the last point.
template <class SK>
__device__ __noinline__ bool vw_step(VwState& W, DEP next, const StrokeParams& P, SK& sink,
                                     int* status) {
    SeqBuffer& pb = W.pb;
    const uint32_t count = pb.count;
    if (count > 0 && too_close(pb.last().pos, next.pos, P.merge_threshold)) {
        if (count == 1) W.mnec = true;
        return false;
    }
    if (count > 0) {
        DEP& join = pb.last();
        if (!join.is_flat || !next.is_flat) vw_edge_attachments(join, next);
    }
    bool skip = false;
    if (count > 1) {
        DEP& prev = pb.second_last();
        DEP& join = pb.last();
        sink.adv = join.adv;
        bool fast = false;
        if (join.is_flat) fast = dot(join.pos - prev.pos, next.pos - join.pos) > 0.0f;
        if (fast) {
            // flattened_step (stroke.rs:1743-1806)
            join.join = LYON_JOIN_MITER;
            const V2 prev_edge = join.pos - prev.pos;
            const float prev_length = vlength(prev_edge);
            const V2 prev_tangent = prev_edge / prev_length;
            const V2 next_edge = next.pos - join.pos;
            const float next_length = vlength(next_edge);
            const V2 next_tangent = next_edge / next_length;
            const V2 normal = compute_normal(prev_tangent, next_tangent);
            if (isnan(join.adv)) join.adv = prev.adv + prev_length;
            if (isnan(next.adv)) next.adv = join.adv + next_length;
            sink.adv = join.adv;
            const V2 p0 = join.pos + normal * join.hw;
            const V2 p1 = join.pos - normal * join.hw;
            join.s[SP].prev = join.s[SP].next = join.s[SP].single = p0;
            join.s[SP].has_single = true;
            join.s[SN].prev = join.s[SN].next = join.s[SN].single = p1;
            join.s[SN].has_single = true;
            const V2 v0 = p0 - prev.s[SP].next;
            const V2 v1 = p1 - prev.s[SN].next;
            if (dot(prev_edge, v0) < 0.0f && dot(prev_edge, v1) < 0.0f) {
                skip = true;
            } else {
                const uint32_t pv = sink.vertex(join.pos + normal * join.hw, normal, SP);
                const uint32_t nv = sink.vertex(join.pos + (-normal) * join.hw, -normal, SN);
                join.s[SP].prev_vertex = join.s[SP].next_vertex = pv;
                join.s[SN].prev_vertex = join.s[SN].next_vertex = nv;
            }
        } else {
            vw_join_sides(prev, join, next, P.miter_limit, SP);
            vw_join_sides(prev, join, next, P.miter_limit, SN);
            // Prevent folding when the other side is concave.
            if (join.s[SP].has_single) join.fold[SN] = false;
            if (join.s[SN].has_single) join.fold[SP] = false;
            add_join_base_vertices(join, SN, sink);
            add_join_base_vertices(join, SP, sink);
        }
        if (!skip) {
            if (count > 2) add_edge_triangles(prev, join, sink);
            tessellate_join(join, P, sink, status);
            if (count == 2) {
                W.firsts[0] = prev;
                W.firsts[1] = join;
                W.nfirsts = 2;
            }
        }
    }
    if (skip) {
        pb.replace_last(next);
    } else {
        pb.push(next);
    }
    return true;
}

}  // namespace lg
