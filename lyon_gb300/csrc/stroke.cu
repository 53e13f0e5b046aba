// stroke.cu — batched fixed-width stroke tessellation (count and emit kernels).
//
// One warp strokes one path at a time; warps of a persistent grid take paths from an atomic
// work counter. lyon's stroker (stroke.rs:1521-1632) is a sequential state machine over the
// flattened points of a sub-path, but every step only looks at its two predecessors, so the
// warp runs 32 consecutive steps at once, one per lane:
//   1. a window of up to 32 verbs (ending at the sub-path's End/Close) is decoded, one verb per
//      lane: lyon's segment counts (`flattened_segments_wang`, quadratic_bezier.rs:943-974,
//      cubic_bezier.rs:1369-1403) and the sharp-turn split of quadratics (stroke.rs:2755-2779);
//      a warp scan of the per-verb step counts gives every step its verb;
//   2. the general joins the window will need, at the end points of its lines and curves, are
//      computed ahead, one per lane, from the neighbours they will have unless the merge filter
//      removes one (`speculate_joins`); a join uses that result only after checking that its
//      actual neighbours are the assumed ones, bit for bit, and computes its own otherwise;
//   3. the window's steps are processed 32 at a time, lane = step: the flattened point (lyon's
//      accumulated parameter t is reproduced bit for bit in closed form by accumulate_t, from
//      the previous chunk's last value), then the merge filter (stroke.rs:1530-1536): a ballot
//      finds points within the threshold of their predecessor and only then is the chain
//      replayed and the kept points compacted across lanes;
//   4. lane L then performs the join at the previous kept point, whose neighbours come from
//      lanes L-1 and L-2 (or the carry from the previous chunk): flattening-step joins
//      (stroke.rs:1743-1806) are straight-line register arithmetic; a warp scan of the per-join
//      vertex/index counts places every join's output and each lane writes its own; the output
//      of the general joins computed ahead is written at the end of the window, one per lane;
//   5. the tail of the path's last sub-path (caps, closing, empty caps) is queued; the warp
//      processes its queue 32 paths at a time, one per lane. Tails of earlier sub-paths of a
//      multi-sub-path path run at once on lane 0 (the next sub-path's output follows them).
// The count kernel performs the same walk without writing (it proves, by a bound, that the skip
// test of flattened_step cannot fire instead of evaluating it, see below); a look-back scan turns
// its per-path counts into offsets; the emit kernel repeats the walk and writes at those offsets.
#include "stroke_core.cuh"
#include "stroke_out.cuh"
#include "kernels.h"

namespace lg {

#ifndef LG_STROKE_WARPS
#define LG_STROKE_WARPS 8
#endif
#ifndef LG_STROKE_MIN_BLOCKS
#define LG_STROKE_MIN_BLOCKS 2
#endif
#ifndef LG_WINDOW_VERBS
#define LG_WINDOW_VERBS 32
#endif
#ifndef LG_TAIL_QUEUE
#define LG_TAIL_QUEUE 32
#endif
constexpr int STROKE_WARPS = LG_STROKE_WARPS;
constexpr uint32_t WINDOW = LG_WINDOW_VERBS;  // verbs decoded per window (<= 32)
constexpr uint32_t TAILQ = LG_TAIL_QUEUE;     // sub-path tails queued per warp (<= 32)
constexpr uint32_t FULL = 0xFFFFFFFFu;
constexpr uint32_t MAX_VERB_STEPS = 1u << 26;
constexpr uint32_t NO_VERB = 0xFFFFFFFFu;
constexpr uint32_t NO_SLOT = 0xFFu;
constexpr uint32_t EF_ALLINV = EF_NEG_INV | EF_POS_INV | EF_SELF_EQ;

struct VerbSlot {
    Poly pA, pB;
    V2 toA, toB;
    float sA, sB;
    uint32_t mA, mB;
    uint32_t excl, steps;  // first step of the verb within the window, step count
    int kind;
};

// A general join at the end point of a unit (a line, a curve, or one part of a split quadratic),
// computed before the window's chunks from the neighbours it assumed.
struct SpecSlot {
    V2 prev, cur, next;
    V2 pn, nn;
    uint32_t from_f, to_f, fneg_rel, fpos_rel, vcount, jtris;
    int st;
    uint32_t flags;  // SPEC_VALID, SPEC_SYM
};
constexpr uint32_t SPEC_VALID = 1u, SPEC_SYM = 2u;

// Output of a join computed ahead, written at the end of the window.
struct EmitJob {
    uint32_t slot, vo, io, base, pfn, pfp, has_edge;
    float adv;  // the join's advancement (attribute output)
};

// Everything the tail of a sub-path needs (stroke.rs:1179-1378): the first three and the last
// three kept points and how their joins were done.
struct TailJob {
    uint32_t path, n, flags, base1, jbase, vcur, icur;
    V2 p0, p1, p2, c3, c2, c1;
    float adv0, adv2, adv1;  // advancements of p0, c2 and c1 (read by the attribute output only)
};
enum : uint32_t {
    TJ_CLOSED = 1u, TJ_MNEC = 2u, TJ_FLAT1 = 4u, TJ_FAST1 = 8u, TJ_SKIP1 = 16u, TJ_F1 = 32u,
    TJ_F2 = 64u, TJ_JFAST = 128u, TJ_JSKIP = 256u
};

struct WarpSmem {
    VerbSlot verbs[WINDOW];
    SpecSlot spec[2 * WINDOW];
    EmitJob ej[2 * WINDOW];
    TailJob tq[TAILQ];
};

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v, int lane) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t n = __shfl_up_sync(FULL, v, o);
        if (lane >= o) v += n;
    }
    return v;
}

__device__ __forceinline__ V2 shfl_v2(V2 v, int src) {
    return V2{__shfl_sync(FULL, v.x, src), __shfl_sync(FULL, v.y, src)};
}
__device__ __forceinline__ V2 shfl_up_v2(V2 v, int d) {
    return V2{__shfl_up_sync(FULL, v.x, d), __shfl_up_sync(FULL, v.y, d)};
}
__device__ __forceinline__ bool same_bits(V2 a, V2 b) {
    return __float_as_uint(a.x) == __float_as_uint(b.x) &&
           __float_as_uint(a.y) == __float_as_uint(b.y);
}

// t state carried across step chunks: the chunk's last step.
struct TCarry {
    uint32_t verb;  // absolute verb index, or NO_VERB when the last step was not inside a curve
    uint32_t unit;
    uint32_t k;
    float t;
};

// Warp-uniform state of the sub-path being stroked (every lane holds the same values).
struct SubState {
    uint32_t n;      // kept points so far
    V2 c1, c2, c3;   // the last three kept points: P[n-1], P[n-2], P[n-3]
    bool f1, f2;     // flattening-step flags of c1 and c2
    uint32_t s1;     // spec slot of c1 (NO_SLOT unless it is a unit end point)
    V2 jtan;         // tangent of the edge c2 -> c1
    // The last processed join (at P[n-2]); when n == 2, the first point (its sides only).
    V2 jpn, jnn;        // its side "next" points
    bool jside_valid;   // jpn/jnn are known (the count pass computes them only when needed)
    uint32_t jfneg, jfpos;  // ids the next edge starts from
    uint32_t jfrom_f;       // their id structure (EF_* flags)
    bool jsym;              // side next points symmetric about the join point
    bool jfast, jskip;
    uint32_t jbase;         // id of the join's first vertex
    bool mnec;              // lyon's may_need_empty_cap
    // The first three kept points and the first join (lyon's firsts, stroke.rs:1624-1627).
    V2 p0, p1, p2;
    bool flat1, fast1, skip1;
    uint32_t base1;
    TCarry tc;
    // Advancements (attribute output only): of the first point, of c1 and of c2.
    float adv0, adv1, adv2;
};

// Flattening parameters of one verb of a window (lane = verb): lines and Begin give one step;
// quadratics are split at a sharp turn (stroke.rs:2755-2779, 3178-3212) and each part gets lyon's
// segment count (quadratic_bezier.rs:943-974); cubics likewise (cubic_bezier.rs:1369-1403).
// Returns the number of flattened points the verb contributes and the verb's status (by value,
// so that the caller keeps no status word in local memory).
struct VerbSetup {
    uint32_t steps;
    int st;
};
__device__ __noinline__ VerbSetup setup_verb(VerbSlot& out, int kind, uint32_t pofs,
                                             uint32_t pcount, uint32_t p_end, const float* points,
                                             float tolerance) {
    int vst = LYON_OK;
    VerbSlot sl;
    sl.kind = kind;
    sl.mA = 0;
    sl.mB = 0;
    sl.sA = sl.sB = 0.0f;
    uint32_t steps = 0;
    if (pofs + pcount > p_end || kind < 0) {
        vst = LYON_ERR_INVALID_ARGUMENT;
    } else if (kind == LYON_VERB_BEGIN || kind == LYON_VERB_LINE_TO) {
        sl.toA = load_pt(points, pofs);
        steps = 1;
    } else if (kind == LYON_VERB_QUADRATIC_TO) {
        V2 from = load_pt(points, pofs - 1);
        V2 ctrl = load_pt(points, pofs);
        V2 to = load_pt(points, pofs + 1);
        float ts;
        if (find_sharp_turn(from, ctrl, to, &ts)) {
            V2 sp = quad_sample(from, ctrl, to, ts);
            V2 bc = lerp(from, ctrl, ts);
            V2 ac = lerp(ctrl, to, ts);
            float nA = quad_wang(from, bc, sp, tolerance);
            float nB = quad_wang(sp, ac, to, tolerance);
            sl.pA = quad_poly(from, bc, sp);
            sl.pB = quad_poly(sp, ac, to);
            sl.mA = to_u32_or1(nA);
            sl.mB = to_u32_or1(nB);
            sl.sA = 1.0f / nA;
            sl.sB = 1.0f / nB;
            sl.toA = sp;
            sl.toB = to;
        } else {
            float nA = quad_wang(from, ctrl, to, tolerance);
            sl.pA = quad_poly(from, ctrl, to);
            sl.mA = to_u32_or1(nA);
            sl.sA = 1.0f / nA;
            sl.toA = to;
        }
        steps = sl.mA + sl.mB;
    } else if (kind == LYON_VERB_CUBIC_TO) {
        V2 from = load_pt(points, pofs - 1);
        V2 c1 = load_pt(points, pofs);
        V2 c2 = load_pt(points, pofs + 1);
        V2 to = load_pt(points, pofs + 2);
        float nA = cubic_wang(from, c1, c2, to, tolerance);
        sl.pA = cubic_poly(from, c1, c2, to);
        sl.mA = to_u32_or1(nA);
        sl.sA = 1.0f / nA;
        sl.toA = to;
        steps = sl.mA;
    }
    if (sl.mA > MAX_VERB_STEPS || sl.mB > MAX_VERB_STEPS) {
        vst = LYON_ERR_UNSUPPORTED;
        steps = 0;
    }
    sl.steps = steps;
    sl.excl = 0;
    out = sl;
    return VerbSetup{steps, vst};
}

// The general joins at the end points of the window's units, one verb per lane (slots 2j and
// 2j + 1 for the two units of verb j). Each assumes that the end point's neighbours are the
// steps just before and after it (what they are unless the merge filter drops one); the step
// before a unit's end point is its flattened point m - 1, the step after it the first point of
// the next unit. `c1` is the sub-path's last kept point before the window, if any. Inlined (its
// join routine stays out of line): measured 1.3 % faster on the batched stroke workload, where
// inlining any of the out-of-line join, arc or verb routines made it 2-22 % slower.
__device__ __forceinline__ void speculate_joins(WarpSmem& sm, int lane, uint32_t nv, uint32_t S_w,
                                             StrokeParams P, V2 c1, bool have_c1) {
    if ((uint32_t)lane >= nv) return;
    const int j = lane;
    const VerbSlot& sl = sm.verbs[j];
    sm.spec[2 * j].flags = 0;
    sm.spec[2 * j + 1].flags = 0;
    const int kind = sl.kind;
    if (kind != LYON_VERB_LINE_TO && kind != LYON_VERB_QUADRATIC_TO &&
        kind != LYON_VERB_CUBIC_TO)
        return;
    const uint32_t nunits = kind == LYON_VERB_LINE_TO ? 1u : (sl.mB > 0 ? 2u : 1u);
    for (uint32_t u = 0; u < nunits; ++u) {
        const bool line = kind == LYON_VERB_LINE_TO;
        const uint32_t m = line ? 1u : (u == 0 ? sl.mA : sl.mB);
        const uint32_t ge = sl.excl + (line ? 0u : (u == 0 ? sl.mA - 1 : sl.mA + sl.mB - 1));
        if (ge + 1 >= S_w) continue;
        const V2 E = u == 0 ? sl.toA : sl.toB;
        V2 next;
        if (u == 0 && nunits == 2) {
            next = sl.mB >= 2 ? poly_sample(sl.pB, sl.sB) : sl.toB;
        } else {
            const VerbSlot& nx = sm.verbs[j + 1];
            if (nx.kind == LYON_VERB_LINE_TO) {
                next = nx.toA;
            } else if (nx.kind == LYON_VERB_QUADRATIC_TO || nx.kind == LYON_VERB_CUBIC_TO) {
                next = nx.mA >= 2 ? poly_sample(nx.pA, nx.sA) : nx.toA;
            } else {
                continue;
            }
        }
        V2 prev;
        if (m >= 2) {
            const float s = u == 0 ? sl.sA : sl.sB;
            const float t = accumulate_t(s, 0, 0.0f, m - 1);
            prev = poly_sample(u == 0 ? sl.pA : sl.pB, t);
        } else if (u == 1) {
            prev = sl.toA;
        } else if (j > 0) {
            const VerbSlot& pv = sm.verbs[j - 1];
            prev = (pv.kind == LYON_VERB_QUADRATIC_TO && pv.mB > 0) ? pv.toB : pv.toA;
        } else if (have_c1) {
            prev = c1;
        } else {
            continue;
        }
        const SlowJoin sj = slow_join_summary(prev, E, false, next, P);
        const int st = sj.st;
        SpecSlot& o = sm.spec[2 * j + u];
        o.prev = prev;
        o.cur = E;
        o.next = next;
        o.pn = sj.pn;
        o.nn = sj.nn;
        o.from_f = sj.from_f;
        o.to_f = sj.to_f;
        o.fneg_rel = sj.from_neg_rel;
        o.fpos_rel = sj.from_pos_rel;
        o.vcount = sj.vcount;
        o.jtris = sj.jtris;
        o.st = st;
        o.flags = SPEC_VALID | (sj.sym ? SPEC_SYM : 0u);
    }
}

// Writes the output of the joins computed ahead (one per lane). Returns the worst status.
template <bool ATTR>
__device__ __noinline__ int emit_spec_joins(WarpSmem& sm, int lane, uint32_t count,
                                            StrokeParams P, const PathOut& po) {
    int worst = LYON_OK;
    for (uint32_t i = (uint32_t)lane; i < count; i += 32) {
        const EmitJob job = sm.ej[i];
        const SpecSlot& sp = sm.spec[job.slot];
        SinkT<ATTR> s;
        s.id_base = job.base;
        s.nv = 0;
        s.ni = 0;
        s.vout = po.vout ? po.vout + job.vo : nullptr;
        s.rout = po.rout ? po.rout + job.vo : nullptr;
        s.adv = job.adv;
        s.index_bits = po.bits;
        s.iout = po.bits == 16 ? (void*)((uint16_t*)po.iout + job.io)
                               : (void*)((uint32_t*)po.iout + job.io);
        s.vcap = cap_left(po.vmax, job.vo);
        s.icap = cap_left(po.imax, job.io);
        s.overflow = false;
        const JoinEmitOut r = slow_join_emit_at(sp.prev, sp.cur, false, sp.next, P, s,
                                                job.has_edge != 0, job.pfn, job.pfp);
        int st = r.st;
        if (r.overflow && st == LYON_OK) st = LYON_ERR_INTERNAL;
        if (st > worst) worst = st;
    }
    return worst;
}

// A join as lyon's EndpointData after its processing, with vertex ids starting at base_id (the
// fast layout of flattened_step, or the general layout), for firsts[1] and the tail.
__device__ __noinline__ void join_dep_with_ids(DEP* out, V2 prev, V2 cur, V2 nxt, bool flat,
                                               bool fast, bool skip, uint32_t base_id,
                                               const StrokeParams& P, int* status) {
    if (fast) {
        V2 pe = cur - prev;
        V2 pt = pe / vlength(pe);
        V2 ne = nxt - cur;
        V2 nt = ne / vlength(ne);
        V2 nrm = compute_normal(pt, nt);
        fast_join_dep(*out, cur, P.hw, cur + nrm * P.hw, cur - nrm * P.hw,
                      skip ? INVALID_ID : base_id, skip ? INVALID_ID : base_id + 1);
    } else {
        DEP d = general_join_geometry(prev, cur, flat, nxt, P);
        join_arc_vertices(d, P, status);
        Sink probe{base_id, 0, 0, nullptr, nullptr, 32};
        add_join_base_vertices(d, SN, probe);
        add_join_base_vertices(d, SP, probe);
        *out = d;
    }
}

// Side "next" points of the join at `cur` (neighbours `prev`, `nxt`) when it was a flattening
// step: what the emit pass computed for it (stroke.rs:1760-1776).
struct SidePair {
    V2 pn, nn;
};
__device__ __noinline__ SidePair fast_join_sides(V2 prev, V2 cur, V2 nxt, float hw) {
    V2 pe = cur - prev;
    V2 pt = pe / vlength(pe);
    V2 ne = nxt - cur;
    V2 nt = ne / vlength(ne);
    V2 nrm = compute_normal(pt, nt);
    return SidePair{cur + nrm * hw, cur - nrm * hw};
}

// The tail of a sub-path: stroke.rs:1179-1279 (end, close) and 1322-1378 (end_with_caps), from
// lyon's firsts (the first kept point with its sides, the first join) and the last join, which
// are rebuilt here from the recorded points. Writes through `s` (positioned at the tail).
template <class SK>
__device__ __noinline__ void run_tail(const TailJob& j, const StrokeParams& P, SK& s,
                                      int* status) {
    const uint32_t n = j.n;
    const bool close = (j.flags & TJ_CLOSED) != 0;
    bool may_need_empty_cap = (j.flags & TJ_MNEC) != 0;
    DEP first0, first1, last;
    dep_init(first0, j.p0, P.hw, P.line_join, false);
    first0.adv = j.adv0;
    if (n >= 2) first_point_sides(first0, j.p1, P.hw);
    if (n >= 3) {
        join_dep_with_ids(&first1, j.p0, j.p1, j.p2, (j.flags & TJ_FLAT1) != 0,
                          (j.flags & TJ_FAST1) != 0, (j.flags & TJ_SKIP1) != 0, j.base1, P,
                          status);
        join_dep_with_ids(&last, j.c3, j.c2, j.c1, (j.flags & TJ_F2) != 0,
                          (j.flags & TJ_JFAST) != 0, (j.flags & TJ_JSKIP) != 0, j.jbase, P,
                          status);
        last.adv = j.adv2;
    }
    const V2 lastp = j.c1;
    const bool lastflat = (j.flags & TJ_F1) != 0;
    may_need_empty_cap |= close && n == 1;
    if (close && n > 2) {
        SeqBuffer pb;
        pb.pts[0] = last;
        dep_init(pb.pts[1], lastp, P.hw, P.line_join, lastflat);
        // The last point's advancement is known to lyon here only when the join before it was
        // a flattening step (stroke.rs:1765-1769); otherwise it is computed again from the
        // point's position, which the merge below may have moved (stroke.rs:1225-1236).
        if (j.flags & TJ_JFAST) pb.pts[1].adv = j.adv1;
        pb.start = 0;
        pb.count = 2;
        pb.n = n;
        bool mnec = false;
        // close (stroke.rs:1206-1279): the first point is stepped again with its advancement
        // recomputed; the two vertices re-made for the first edge keep the starting one.
        DEP p = first0;
        p.adv = __int_as_float(0x7fc00000);
        bool added = seq_step(pb, p, P, s, &mnec, status);
        if (!added) pb.last().pos = p.pos;
        DEP p2 = first1;
        seq_step(pb, p2, P, s, &mnec, status);
        DEP& p0 = pb.second_last();
        DEP& p1 = pb.last();
        s.adv = j.adv0;
        for (int side = 0; side < 2; ++side) {
            V2 sp = p0.s[side].has_single ? p0.s[side].single : p0.s[side].next;
            V2 normal = (sp - p0.pos) / p0.hw;
            p0.s[side].next_vertex = s.vertex(p0.pos + normal * p0.hw, normal, side);
        }
        add_edge_triangles(p0, p1, s);
        return;
    }
    if (may_need_empty_cap && n == 1) {
        V2 pos = first0.pos;
        s.adv = first0.adv;
        if (P.start_cap == LYON_CAP_SQUARE) {
            tessellate_empty_square_cap(pos, P.hw, s);
        } else if (P.start_cap == LYON_CAP_ROUND) {
            tessellate_empty_round_cap(pos, P.hw, P, s, status);
        }
        return;
    }
    if (n >= 2) {
        DEP p0 = (n == 2) ? first0 : last;
        DEP p1;
        dep_init(p1, lastp, P.hw, P.line_join, lastflat);
        p1.adv = j.adv1;
        V2 tan = normalize(p1.pos - p0.pos);
        V2 nn = V2{-tan.y, tan.x} * p1.hw;
        p1.s[SP].prev = p1.pos + nn;
        p1.s[SN].prev = p1.pos - nn;
        tessellate_last_edge(p0, p1, n == 2, P, s, status);
        if (n > 2) {
            p0 = first0;
            p1 = first1;
        }
        tessellate_first_edge(p0, p1, P, s, status);
    }
}

// Runs a tail at the output position (vcur, icur) of its path. Returns the counts it added.
template <bool ATTR>
__device__ __forceinline__ void tail_at(const TailJob& j, const StrokeParams& P,
                                        const PathOut& po, uint32_t* tv, uint32_t* ti,
                                        int* st) {
    SinkT<ATTR> s;
    s.id_base = po.id_base + j.vcur;
    s.nv = 0;
    s.ni = 0;
    s.vout = po.vout ? po.vout + j.vcur : nullptr;
    s.rout = po.rout ? po.rout + j.vcur : nullptr;
    s.iout = nullptr;
    if (po.vout || po.rout) {
        s.iout = po.bits == 16 ? (void*)((uint16_t*)po.iout + j.icur)
                               : (void*)((uint32_t*)po.iout + j.icur);
    }
    s.index_bits = po.bits;
    s.vcap = cap_left(po.vmax, j.vcur);
    s.icap = cap_left(po.imax, j.icur);
    s.overflow = false;
    int tst = LYON_OK;
    run_tail(j, P, s, &tst);
    if (s.overflow && tst == LYON_OK) tst = LYON_ERR_INTERNAL;
    *tv = s.nv;
    *ti = s.ni;
    *st = tst;
}

// Processes the warp's queued tails, one per lane, and finishes their paths.
template <bool EMIT, bool ATTR>
__device__ __noinline__ void flush_tails(WarpSmem& sm, int lane, uint32_t count,
                                         const StrokeArgs& A) {
    if ((uint32_t)lane < count) {
        const TailJob j = sm.tq[lane];
        const lyon_stroke_options opt = A.options[A.num_options > 1 ? j.path : 0];
        const StrokeParams P = make_params(opt);
        const PathOut po = path_out<EMIT, ATTR>(A, j.path);
        uint32_t tv, ti;
        int st;
        tail_at<ATTR>(j, P, po, &tv, &ti, &st);
        finish_path<EMIT>(A, j.path, j.vcur + tv, j.icur + ti, st, po);
    }
    __syncwarp();
}

// Steps [cb, cb + 32) of the current verb window (lane = step): flattened points, merge filter,
// joins, output. See the file comment. `ejn` counts the joins queued for emission.
template <bool EMIT, bool ATTR>
__device__ __forceinline__ void process_chunk(WarpSmem& sm, const int lane, const uint32_t vi,
                                              const uint32_t nv, const uint32_t sincl,
                                              const uint32_t S_w, const uint32_t cb,
                                              const StrokeParams& P, const PathOut& po,
                                              SubState& S, uint32_t& vcur, uint32_t& icur,
                                              uint32_t& ejn, int& status) {
    const uint32_t nsteps = min(32u, S_w - cb);
    const bool active = (uint32_t)lane < nsteps;

    // ---- 1. the flattened point of step cb + lane ----
    V2 q;
    bool flat = false;
    uint32_t sid = NO_SLOT;
    uint32_t my_verb = NO_VERB, my_unit = 0, my_k = 0;
    float my_t = 0.0f;
    {
        const uint32_t gq = min(cb + (uint32_t)lane, S_w - 1);
        // Owner verb: the number of verbs that end at or before the step (lanes past the
        // window hold sincl == S_w, which no step reaches). The chunk's steps span the verbs
        // [vfirst, vlast]; usually one or two.
        const uint32_t vfirst = __popc(__ballot_sync(FULL, sincl <= cb));
        const uint32_t vlast = __popc(__ballot_sync(FULL, sincl <= cb + nsteps - 1));
        uint32_t lo = vfirst;
        for (uint32_t jv = vfirst; jv < vlast; ++jv) {
            if (gq >= __shfl_sync(FULL, sincl, (int)jv)) lo = jv + 1;
        }
        const VerbSlot& sl = sm.verbs[lo];
        const uint32_t r = gq - sl.excl;
        const int kind = sl.kind;
        if (kind == LYON_VERB_BEGIN || kind == LYON_VERB_LINE_TO) {
            q = sl.toA;
            if (kind == LYON_VERB_LINE_TO) sid = 2 * lo;
        } else {
            const uint32_t mA = sl.mA;
            const bool unitA = r < mA;
            const uint32_t kk = unitA ? r + 1 : r - mA + 1;
            const uint32_t m = unitA ? mA : sl.mB;
            if (kk < m) {
                const float s = unitA ? sl.sA : sl.sB;
                const uint32_t u = unitA ? 0u : 1u;
                uint32_t bk = 0;
                float bt = 0.0f;
                if (S.tc.verb == vi + lo && S.tc.unit == u && S.tc.k <= kk) {
                    bk = S.tc.k;
                    bt = S.tc.t;
                }
                const float t = accumulate_t_from(s, bk, bt, kk);
                const Poly* pp = unitA ? &sl.pA : &sl.pB;
                q = poly_sample(*pp, t);
                flat = t != 1.0f;
                my_verb = vi + lo;
                my_unit = u;
                my_k = kk;
                my_t = t;
            } else {
                q = unitA ? sl.toA : sl.toB;
                sid = 2 * lo + (unitA ? 0u : 1u);
            }
        }
    }
    {
        const int ow = (int)nsteps - 1;
        S.tc.verb = __shfl_sync(FULL, my_verb, ow);
        S.tc.unit = __shfl_sync(FULL, my_unit, ow);
        S.tc.k = __shfl_sync(FULL, my_k, ow);
        S.tc.t = __shfl_sync(FULL, my_t, ow);
    }

    // ---- 2. merge filter (stroke.rs:1530-1536) ----
    const uint32_t n0 = S.n;
    uint32_t keep = __ballot_sync(FULL, active);
    {
        V2 qp = shfl_up_v2(q, 1);
        if (lane == 0) qp = S.c1;
        const bool close =
            active && (lane > 0 || n0 > 0) && too_close(qp, q, P.merge_threshold);
        if (__any_sync(FULL, close)) {
            // Replay the chain in order (every lane computes the same mask), then compact.
            uint32_t km = 0, cnt = n0;
            V2 L = S.c1;
            bool mn = S.mnec;
            for (uint32_t i = 0; i < nsteps; ++i) {
                const V2 qi = shfl_v2(q, (int)i);
                if (cnt > 0 && too_close(L, qi, P.merge_threshold)) {
                    if (cnt == 1) mn = true;
                } else {
                    km |= 1u << i;
                    L = qi;
                    ++cnt;
                }
            }
            keep = km;
            S.mnec = mn;
            const uint32_t nkk = __popc(km);
            const int src = (uint32_t)lane < nkk ? (int)__fns(km, 0, lane + 1) : 0;
            q = shfl_v2(q, src);
            flat = __shfl_sync(FULL, (int)flat, src) != 0;
            sid = __shfl_sync(FULL, sid, src);
        }
    }
    const uint32_t nk = __popc(keep);
    if (nk == 0) return;
    const bool live = (uint32_t)lane < nk;

    // ---- 3. joins: lane L performs the join at kept point n0 + L - 1 ----
    const int k = (int)n0 + lane - 1;
    V2 cur = shfl_up_v2(q, 1);
    V2 prv = shfl_up_v2(q, 2);
    bool fcur = __shfl_up_sync(FULL, (int)flat, 1) != 0;
    uint32_t scur = __shfl_up_sync(FULL, sid, 1);
    if (lane == 0) {
        cur = S.c1;
        prv = S.c2;
        fcur = S.f1;
        scur = S.s1;
    } else if (lane == 1) {
        prv = S.c1;
    }
    const V2 ne = q - cur;
    // Tangent of the edge cur -> q. The count pass needs tangents only at a sub-path's first
    // point and when it evaluates the skip test exactly (below), so it computes them there.
    V2 nt = V2{0.0f, 0.0f};
    float len_ne = 0.0f;
    if (EMIT || (live && k == 0)) {
        len_ne = vlength(ne);
        nt = ne / len_ne;
    }
    // Advancement of each kept point (attribute output): lyon adds the edge lengths one after
    // the other in f32 (stroke.rs:1546-1550, 1657-1662, 1759-1771), so the sum runs through the
    // lanes in order; a sub-path's first point starts from the carried advancement.
    float adv_q = 0.0f, adv_join = 0.0f;
    if (EMIT && ATTR) {
        float carry = S.adv1;
        for (int i = 0; i < (int)nk; ++i) {
            if (lane == i) adv_q = k < 0 ? S.adv0 : carry + len_ne;
            carry = __shfl_sync(FULL, adv_q, i);
        }
        adv_join = __shfl_up_sync(FULL, adv_q, 1);
        if (lane == 0) adv_join = S.adv1;
    }
    const V2 pe = cur - prv;
    const bool isjoin = live && k >= 1;
    const bool fast = isjoin && fcur && dot(pe, ne) > 0.0f;
    const bool slow = isjoin && !fast;

    uint32_t vcnt = 0, jt = 0, to_f = 0, from_f = EF_ALLINV;
    uint32_t fneg_rel = INVALID_ID, fpos_rel = INVALID_ID;
    bool sym = true, skip = false, have_sides = false;
    V2 pn = V2{0.0f, 0.0f}, nn = V2{0.0f, 0.0f};
    int st = LYON_OK;
    if (fast) {
        vcnt = 2;
        from_f = 0;
        fneg_rel = 1;
        fpos_rel = 0;
    }
    if (live && k == 0) {
        // The first point: side points from its first edge (stroke.rs:1538-1556).
        const V2 n = V2{-nt.y, nt.x} * P.hw;
        pn = cur + n;
        nn = cur - n;
        have_sides = true;
    }
    bool spec = false;
    if (slow && scur != NO_SLOT) {
        const SpecSlot& sp = sm.spec[scur];
        spec = (sp.flags & SPEC_VALID) && same_bits(sp.prev, prv) && same_bits(sp.cur, cur) &&
               same_bits(sp.next, q);
        if (spec) {
            vcnt = sp.vcount;
            jt = sp.jtris;
            to_f = sp.to_f;
            from_f = sp.from_f;
            fneg_rel = sp.fneg_rel;
            fpos_rel = sp.fpos_rel;
            sym = (sp.flags & SPEC_SYM) != 0;
            pn = sp.pn;
            nn = sp.nn;
            have_sides = true;
            st = sp.st;
        }
    }
    if (slow && !spec) {
        const SlowJoin sj = slow_join_summary(prv, cur, fcur, q, P);
        if (sj.st != LYON_OK) st = sj.st;
        vcnt = sj.vcount;
        jt = sj.jtris;
        to_f = sj.to_f;
        from_f = sj.from_f;
        fneg_rel = sj.from_neg_rel;
        fpos_rel = sj.from_pos_rel;
        sym = sj.sym;
        pn = sj.pn;
        nn = sj.nn;
        have_sides = true;
    }
    // flattened_step's skip test (stroke.rs:1778-1782). The emit pass evaluates it. The count pass
    // first tries a bound: with the previous join's side points symmetric about the previous
    // point, the test needs the previous edge to be shorter than a few ulps of the coordinates
    // involved (2^-17 times their magnitude plus 3 half widths covers the roundings of both
    // joins' side points), so when every fast lane's edge is longer the test cannot fire;
    // otherwise the count pass evaluates it exactly as well.
    bool exact = EMIT;
    V2 fast_nrm = V2{0.0f, 0.0f};
    if (!EMIT) {
        bool psym = __shfl_up_sync(FULL, (int)sym, 1) != 0;
        if (lane == 0) psym = S.jsym;
        bool ok = true;
        if (fast) {
            const float m = fmaxf(fmaxf(fabsf(cur.x), fabsf(cur.y)),
                                  fmaxf(fabsf(prv.x), fabsf(prv.y))) + 3.0f * P.hw;
            const float bnd = m * 7.62939453125e-06f;  // 2^-17
            ok = psym && sqlen(pe) > bnd * bnd;
        }
        exact = __any_sync(FULL, !ok);
    }
    if (exact) {
        if (!EMIT) nt = ne / vlength(ne);
        V2 pt = shfl_up_v2(nt, 1);
        if (lane == 0) {
            // The previous edge's tangent: carried by the emit pass, recomputed by the count
            // pass with the same operations (c2 -> c1 is the edge into lane 0's join point).
            if (EMIT) {
                pt = S.jtan;
            } else {
                const V2 e = S.c1 - S.c2;
                pt = e / vlength(e);
            }
        }
        if (fast) {
            const V2 nrm = compute_normal(pt, nt);
            pn = cur + nrm * P.hw;
            nn = cur - nrm * P.hw;
            fast_nrm = nrm;
            have_sides = true;
        }
        V2 ppn = shfl_up_v2(pn, 1), pnn = shfl_up_v2(nn, 1);
        if (lane == 0) {
            if (!S.jside_valid) {
                const SidePair sp2 = fast_join_sides(S.c3, S.c2, S.c1, P.hw);
                S.jpn = sp2.pn;
                S.jnn = sp2.nn;
            }
            ppn = S.jpn;
            pnn = S.jnn;
        }
        skip = fast && dot(pe, pn - ppn) < 0.0f && dot(pe, nn - pnn) < 0.0f;
        if (skip) {
            vcnt = 0;
            from_f = to_f = EF_ALLINV;
            fneg_rel = fpos_rel = INVALID_ID;
        }
    }

    // ---- 4. counts, offsets, output ----
    uint32_t pf = __shfl_up_sync(FULL, from_f, 1);
    if (lane == 0) pf = S.jfrom_f;
    const uint32_t e = (isjoin && k >= 2) ? edge_count_flags(pf, to_f) : 0u;
    const uint32_t icnt = 3u * (jt + e);
    const uint32_t vincl = warp_incl_scan(vcnt, lane);
    const uint32_t iincl = warp_incl_scan(icnt, lane);
    const uint32_t vtot = __shfl_sync(FULL, vincl, 31);
    const uint32_t itot = __shfl_sync(FULL, iincl, 31);
    const uint32_t vrel = vincl - vcnt;
    const uint32_t irel = iincl - icnt;
    const uint32_t base = po.id_base + vcur + vrel;
    const uint32_t fneg = fneg_rel == INVALID_ID ? INVALID_ID : base + fneg_rel;
    const uint32_t fpos = fpos_rel == INVALID_ID ? INVALID_ID : base + fpos_rel;

    if (EMIT) {
        uint32_t pfn = __shfl_up_sync(FULL, fneg, 1);
        uint32_t pfp = __shfl_up_sync(FULL, fpos, 1);
        if (lane == 0) {
            pfn = S.jfneg;
            pfp = S.jfpos;
        }
        const uint32_t vo = vcur + vrel;
        const uint32_t io = icur + irel;
        if (fast) {
            if (ATTR && !skip) {
                // flattened_step's two vertices, + then - (stroke.rs:1791-1797).
                if (vo + 2 <= po.vmax) {
                    float2* dst = reinterpret_cast<float2*>(po.rout + vo);
                    dst[0] = make_float2(pn.x, pn.y);
                    dst[1] = make_float2(fast_nrm.x, fast_nrm.y);
                    dst[2] = make_float2(adv_join, __uint_as_float((uint32_t)SP));
                    dst[3] = make_float2(nn.x, nn.y);
                    dst[4] = make_float2(-fast_nrm.x, -fast_nrm.y);
                    dst[5] = make_float2(adv_join, __uint_as_float((uint32_t)SN));
                } else {
                    st = LYON_ERR_INTERNAL;
                }
            } else if (!skip) {
                if (vo + 2 <= po.vmax) {
                    float2* dst = po.vout + vo;
                    if ((reinterpret_cast<uintptr_t>(dst) & 15u) == 0) {
                        *reinterpret_cast<float4*>(dst) = make_float4(pn.x, pn.y, nn.x, nn.y);
                    } else {
                        dst[0] = make_float2(pn.x, pn.y);
                        dst[1] = make_float2(nn.x, nn.y);
                    }
                } else {
                    st = LYON_ERR_INTERNAL;
                }
            }
            if (k >= 2) {
                // add_edge_triangles (stroke.rs:1869-1904) on the resolved ids.
                const uint32_t pos_id = skip ? INVALID_ID : base;
                const uint32_t neg_id = skip ? INVALID_ID : base + 1;
                const bool triA = pfn != pos_id && pfn != pfp && pfp != pos_id;
                const bool triB = pfn != pos_id && pfn != neg_id && pos_id != neg_id;
                // Triangle A = (pfn, pfp, pos_id), then B = (pfn, pos_id, neg_id).
                const uint32_t a1 = triA ? pfp : pos_id, a2 = triA ? pos_id : neg_id;
                const uint32_t ni = (triA ? 3u : 0u) + (triB ? 3u : 0u);
                if (io + ni > po.imax) {
                    st = LYON_ERR_INTERNAL;
                } else if (po.bits == 32) {
                    uint32_t* dst = (uint32_t*)po.iout + io;
                    if (ni == 6 && (reinterpret_cast<uintptr_t>(dst) & 7u) == 0) {
                        uint2* d2 = reinterpret_cast<uint2*>(dst);
                        d2[0] = make_uint2(pfn, pfp);
                        d2[1] = make_uint2(pos_id, pfn);
                        d2[2] = make_uint2(pos_id, neg_id);
                    } else if (ni != 0) {
                        dst[0] = pfn;
                        dst[1] = a1;
                        dst[2] = a2;
                        if (ni == 6) {
                            dst[3] = pfn;
                            dst[4] = pos_id;
                            dst[5] = neg_id;
                        }
                    }
                } else if (ni != 0) {
                    uint16_t* dst = (uint16_t*)po.iout + io;
                    dst[0] = (uint16_t)pfn;
                    dst[1] = (uint16_t)a1;
                    dst[2] = (uint16_t)a2;
                    if (ni == 6) {
                        dst[3] = (uint16_t)pfn;
                        dst[4] = (uint16_t)pos_id;
                        dst[5] = (uint16_t)neg_id;
                    }
                }
            }
        }
        // Joins computed ahead are written at the end of the window.
        const uint32_t qmask = __ballot_sync(FULL, spec);
        if (spec) {
            const uint32_t slot_i = ejn + __popc(qmask & ((1u << lane) - 1u));
            EmitJob& job = sm.ej[slot_i];
            job.slot = scur;
            job.vo = vo;
            job.io = io;
            job.base = base;
            job.pfn = pfn;
            job.pfp = pfp;
            job.has_edge = k >= 2 ? 1u : 0u;
            job.adv = ATTR ? adv_join : 0.0f;
        }
        ejn += __popc(qmask);
        if (slow && !spec) {
            SinkT<ATTR> s;
            s.id_base = base;
            s.nv = 0;
            s.ni = 0;
            s.vout = po.vout ? po.vout + vo : nullptr;
            s.rout = po.rout ? po.rout + vo : nullptr;
            s.adv = adv_join;
            s.index_bits = po.bits;
            s.iout = po.bits == 16 ? (void*)((uint16_t*)po.iout + io)
                                   : (void*)((uint32_t*)po.iout + io);
            s.vcap = cap_left(po.vmax, vo);
            s.icap = cap_left(po.imax, io);
            s.overflow = false;
            const JoinEmitOut r = slow_join_emit_at(prv, cur, fcur, q, P, s, k >= 2, pfn, pfp);
            if (r.st != LYON_OK) st = r.st;
            if (r.overflow) st = LYON_ERR_INTERNAL;
        }
    }

    // ---- the first three kept points and the first join (lyon's firsts) ----
    if (n0 < 3) {
        if (n0 == 0) S.p0 = shfl_v2(q, 0);
        if (n0 <= 1 && 1 - (int)n0 < (int)nk) S.p1 = shfl_v2(q, 1 - (int)n0);
        const int l1 = 2 - (int)n0;  // the lane of the first join (k == 1)
        if (l1 < (int)nk) {
            S.p2 = shfl_v2(q, l1);
            S.flat1 = __shfl_sync(FULL, (int)fcur, l1) != 0;
            S.fast1 = __shfl_sync(FULL, (int)fast, l1) != 0;
            S.skip1 = __shfl_sync(FULL, (int)skip, l1) != 0;
            S.base1 = __shfl_sync(FULL, base, l1);
        }
    }

    // ---- carry to the next chunk ----
    {
        const int last = (int)nk - 1;
        const V2 q3 = shfl_v2(q, last >= 2 ? last - 2 : 0);
        const V2 q2 = shfl_v2(q, last >= 1 ? last - 1 : 0);
        const bool fl2 = __shfl_sync(FULL, (int)flat, last >= 1 ? last - 1 : 0) != 0;
        const V2 q1 = shfl_v2(q, last);
        const bool fl1 = __shfl_sync(FULL, (int)flat, last) != 0;
        const V2 oc1 = S.c1, oc2 = S.c2;
        const bool of1 = S.f1;
        if (EMIT && ATTR) {
            const float a2 = __shfl_sync(FULL, adv_q, last >= 1 ? last - 1 : 0);
            const float a1 = __shfl_sync(FULL, adv_q, last);
            S.adv2 = nk >= 2 ? a2 : S.adv1;
            S.adv1 = a1;
        }
        S.c3 = nk >= 3 ? q3 : (nk == 2 ? oc1 : oc2);
        S.c2 = nk >= 2 ? q2 : oc1;
        S.f2 = nk >= 2 ? fl2 : of1;
        S.c1 = q1;
        S.f1 = fl1;
        S.s1 = __shfl_sync(FULL, sid, last);
        if (EMIT) S.jtan = shfl_v2(nt, last);
        S.jpn = shfl_v2(pn, last);
        S.jnn = shfl_v2(nn, last);
        S.jside_valid = __shfl_sync(FULL, (int)have_sides, last) != 0;
        S.jfneg = __shfl_sync(FULL, fneg, last);
        S.jfpos = __shfl_sync(FULL, fpos, last);
        S.jfrom_f = __shfl_sync(FULL, from_f, last);
        S.jsym = __shfl_sync(FULL, (int)sym, last) != 0;
        S.jfast = __shfl_sync(FULL, (int)fast, last) != 0;
        S.jskip = __shfl_sync(FULL, (int)skip, last) != 0;
        S.jbase = __shfl_sync(FULL, base, last);
        S.n = n0 + nk;
    }
    if (__any_sync(FULL, st != LYON_OK)) {
        const int em = __reduce_max_sync(FULL, st);
        if (status == LYON_OK) status = em;
    }
    vcur += vtot;
    icur += itot;
    __syncwarp();
}

// Strokes one path with the whole warp. On return vcur/icur/status hold the path's counts so
// far; when the tail of its last sub-path was queued (`deferred`), the queue finishes the path.
template <bool EMIT, bool ATTR>
__device__ void stroke_path(WarpSmem& sm, int lane, const StrokeArgs& A, uint32_t path,
                            const PathOut& po, uint32_t& vcur, uint32_t& icur, int& status,
                            uint32_t& tqn, bool& deferred) {
    const uint32_t v_begin = A.verb_offsets[path], v_end = A.verb_offsets[path + 1];
    const uint32_t p_begin = A.point_offsets[path], p_end = A.point_offsets[path + 1];
    const lyon_stroke_options opt = A.options[A.num_options > 1 ? path : 0];
    const StrokeParams P = make_params(opt);
    vcur = 0;
    icur = 0;
    status = LYON_OK;
    deferred = false;
    uint32_t vi = v_begin;
    uint32_t pc = p_begin;
    float start_adv = 0.0f;  // sub_path_start_advancement (stroke.rs:585, 1359)
    while (vi < v_end && status == LYON_OK) {
        // A sub-path starts with Begin (crates/path/src/path.rs:843-909).
        if (A.verbs[vi] != LYON_VERB_BEGIN) {
            status = LYON_ERR_INVALID_ARGUMENT;
            break;
        }
        SubState S;
        S.n = 0;
        S.c1 = S.c2 = S.c3 = V2{0.0f, 0.0f};
        S.f1 = S.f2 = false;
        S.s1 = NO_SLOT;
        S.jtan = V2{0.0f, 0.0f};
        S.jpn = S.jnn = V2{0.0f, 0.0f};
        S.jside_valid = false;
        S.jfneg = S.jfpos = INVALID_ID;
        S.jfrom_f = EF_ALLINV;
        S.jsym = true;
        S.jfast = S.jskip = false;
        S.jbase = 0;
        S.mnec = false;
        S.p0 = S.p1 = S.p2 = V2{0.0f, 0.0f};
        S.flat1 = S.fast1 = S.skip1 = false;
        S.base1 = 0;
        S.tc.verb = NO_VERB;
        S.tc.unit = 0;
        S.tc.k = 0;
        S.tc.t = 0.0f;
        S.adv0 = start_adv;
        S.adv1 = S.adv2 = 0.0f;
        bool ended = false, closed = false;
        while (vi < v_end && status == LYON_OK) {
            // ---- verb window ----
            const uint32_t v = vi + (uint32_t)lane;
            const bool valid = v < v_end;
            int kind = valid ? (int)A.verbs[v] : LYON_VERB_END;
            const bool is_end = valid && (kind == LYON_VERB_END || kind == LYON_VERB_CLOSE);
            const bool bad_begin = valid && lane > 0 && kind == LYON_VERB_BEGIN;
            const uint32_t endmask = __ballot_sync(FULL, is_end || bad_begin);
            uint32_t nv = min(WINDOW, v_end - vi);
            if (endmask) nv = min(nv, (uint32_t)(__ffs(endmask)));
            const bool inwin = (uint32_t)lane < nv;
            if (inwin && bad_begin) kind = -1;
            const uint32_t pcount = inwin ? points_of_verb(kind) : 0u;
            const uint32_t pincl = warp_incl_scan(pcount, lane);
            const uint32_t pofs = pc + pincl - pcount;
            uint32_t steps = 0;
            int vst = LYON_OK;
            if (inwin) {
                const VerbSetup su = setup_verb(sm.verbs[lane], kind, pofs, pcount, p_end,
                                                A.points, P.tolerance);
                steps = su.steps;
                vst = su.st;
            }
            if (__any_sync(FULL, vst != LYON_OK)) {
                status = __reduce_max_sync(FULL, vst);
                break;
            }
            const uint32_t sincl = warp_incl_scan(steps, lane);
            if (inwin) sm.verbs[lane].excl = sincl - steps;
            const uint32_t S_w = __shfl_sync(FULL, sincl, 31);
            const int last_kind = __shfl_sync(FULL, kind, nv - 1);
            __syncwarp();
            speculate_joins(sm, lane, nv, S_w, P, S.c1, S.n > 0);
            __syncwarp();
            uint32_t ejn = 0;
            for (uint32_t cb = 0; cb < S_w; cb += 32) {
                process_chunk<EMIT, ATTR>(sm, lane, vi, nv, sincl, S_w, cb, P, po, S, vcur, icur, ejn,
                                    status);
            }
            if (EMIT && ejn > 0) {
                __syncwarp();
                int est = emit_spec_joins<ATTR>(sm, lane, ejn, P, po);
                est = __reduce_max_sync(FULL, est);
                if (est != LYON_OK && status == LYON_OK) status = est;
            }
            __syncwarp();
            vi += nv;
            pc += __shfl_sync(FULL, pincl, 31);
            if (last_kind == LYON_VERB_END || last_kind == LYON_VERB_CLOSE) {
                ended = true;
                closed = last_kind == LYON_VERB_CLOSE;
                break;
            }
        }
        if (!ended || status != LYON_OK) break;
        // ---- tail ----
        TailJob job;
        job.path = path;
        job.n = S.n;
        job.flags = (closed ? TJ_CLOSED : 0u) | (S.mnec ? TJ_MNEC : 0u) |
                    (S.flat1 ? TJ_FLAT1 : 0u) | (S.fast1 ? TJ_FAST1 : 0u) |
                    (S.skip1 ? TJ_SKIP1 : 0u) | (S.f1 ? TJ_F1 : 0u) | (S.f2 ? TJ_F2 : 0u) |
                    (S.jfast ? TJ_JFAST : 0u) | (S.jskip ? TJ_JSKIP : 0u);
        job.base1 = S.base1;
        job.jbase = S.jbase;
        job.vcur = vcur;
        job.icur = icur;
        job.p0 = S.p0;
        job.p1 = S.p1;
        job.p2 = S.p2;
        job.c3 = S.c3;
        job.c2 = S.c2;
        job.c1 = S.c1;
        job.adv0 = job.adv1 = job.adv2 = 0.0f;
        if (ATTR) {
            job.adv0 = S.adv0;
            job.adv1 = S.adv1;
            job.adv2 = S.adv2;
            // end_with_caps carries the last advancement to the next sub-path (stroke.rs:1359).
            if (S.n >= 2 && !(closed && S.n > 2)) start_adv = S.adv1;
        }
        if (vi >= v_end) {
            // The path's last sub-path: queue its tail.
            if (tqn == TAILQ) {
                flush_tails<EMIT, ATTR>(sm, lane, tqn, A);
                tqn = 0;
            }
            if (lane == 0) sm.tq[tqn] = job;
            ++tqn;
            deferred = true;
            __syncwarp();
            break;
        }
        uint32_t tv = 0, ti = 0;
        int tst = LYON_OK;
        if (lane == 0) tail_at<ATTR>(job, P, po, &tv, &ti, &tst);
        tv = __shfl_sync(FULL, tv, 0);
        ti = __shfl_sync(FULL, ti, 0);
        tst = __shfl_sync(FULL, tst, 0);
        if (tst != LYON_OK && status == LYON_OK) status = tst;
        vcur += tv;
        icur += ti;
        __syncwarp();
    }
}

// One thread strokes one short line-only path: lyon's sequential step (seq_step, the
// fixed_width_step_impl of stroke.rs:1521-1632) over its points, then the sub-path tail through
// run_tail, as the warp walk does. Verbs are checked per window of up to WINDOW verbs ending at
// an End/Close (a Begin inside it, or points missing for it, fail the path before any of its
// steps), so that a path fails with the status the warp walk gives it.
template <bool EMIT, bool ATTR>
__device__ __noinline__ void stroke_path_seq(const StrokeArgs& A, uint32_t path) {
    const PathOut po = path_out<EMIT, ATTR>(A, path);
    const uint32_t v_begin = A.verb_offsets[path], v_end = A.verb_offsets[path + 1];
    const uint32_t p_end = A.point_offsets[path + 1];
    const StrokeParams P = make_params(A.options[A.num_options > 1 ? path : 0]);
    SinkT<ATTR> s;
    s.id_base = po.id_base;
    s.nv = 0;
    s.ni = 0;
    s.vout = po.vout;
    s.rout = po.rout;
    s.iout = po.iout;
    s.index_bits = po.bits;
    s.vcap = po.vmax;
    s.icap = po.imax;
    s.overflow = false;
    int status = LYON_OK;
    uint32_t vi = v_begin, pc = A.point_offsets[path];
    float start_adv = 0.0f;  // sub_path_start_advancement (stroke.rs:585, 1359)
    while (vi < v_end && status == LYON_OK) {
        if (A.verbs[vi] != LYON_VERB_BEGIN) {
            status = LYON_ERR_INVALID_ARGUMENT;
            break;
        }
        SeqBuffer pb;
        pb.start = 0;
        pb.count = 0;
        pb.n = 0;
        TailJob job;
        job.path = path;
        job.base1 = job.jbase = 0;
        job.p0 = job.p1 = job.p2 = job.c3 = job.c2 = job.c1 = V2{0.0f, 0.0f};
        bool mnec = false, ended = false, closed = false;
        while (vi < v_end && status == LYON_OK) {
            uint32_t nv = 0, need = 0;
            int last_kind = LYON_VERB_END;
            while (nv < WINDOW && vi + nv < v_end) {
                const int k = A.verbs[vi + nv];
                ++nv;
                last_kind = k;
                if (nv > 1 && k == LYON_VERB_BEGIN) {
                    status = LYON_ERR_INVALID_ARGUMENT;
                    break;
                }
                need += points_of_verb(k);
                if (k == LYON_VERB_END || k == LYON_VERB_CLOSE) break;
            }
            if (status != LYON_OK || pc + need > p_end) {
                status = LYON_ERR_INVALID_ARGUMENT;
                break;
            }
            for (uint32_t j = 0; j < nv; ++j) {
                const int k = A.verbs[vi + j];
                if (k == LYON_VERB_CLOSE) ++pc;
                if (k != LYON_VERB_BEGIN && k != LYON_VERB_LINE_TO) continue;
                const V2 p = load_pt(A.points, pc++);
                DEP d;
                dep_init(d, p, P.hw, P.line_join, false);
                if (k == LYON_VERB_BEGIN) d.adv = start_adv;
                const uint32_t base = s.id_base + s.nv;
                if (!seq_step(pb, d, P, s, &mnec, &status)) continue;
                job.c3 = job.c2;
                job.c2 = job.c1;
                job.c1 = p;
                if (pb.n == 1) {
                    job.p0 = p;
                } else if (pb.n == 2) {
                    job.p1 = p;
                } else {
                    if (pb.n == 3) {
                        job.p2 = p;
                        job.base1 = base;
                    }
                    job.jbase = base;
                }
            }
            vi += nv;
            if (last_kind == LYON_VERB_END || last_kind == LYON_VERB_CLOSE) {
                ended = true;
                closed = last_kind == LYON_VERB_CLOSE;
                break;
            }
        }
        if (!ended || status != LYON_OK) break;
        job.n = pb.n;
        job.flags = (closed ? TJ_CLOSED : 0u) | (mnec ? TJ_MNEC : 0u);
        job.adv0 = start_adv;
        job.adv1 = job.adv2 = start_adv;
        if (ATTR && pb.n >= 2) {
            const DEP& l = pb.last();
            const DEP& sl = pb.second_last();
            job.adv2 = sl.adv;
            job.adv1 = isnan(l.adv) ? sl.adv + vlength(l.pos - sl.pos) : l.adv;
            if (!(closed && pb.n > 2)) start_adv = job.adv1;
        }
        int tst = LYON_OK;
        run_tail(job, P, s, &tst);
        if (tst != LYON_OK) status = tst;
    }
    if (s.overflow && status == LYON_OK) status = LYON_ERR_INTERNAL;
    finish_path<EMIT>(A, path, s.nv, s.ni, status, po);
}

// The short line-only paths (items [split, num_paths) of the order): 32 per warp, one per lane.
template <bool EMIT, bool ATTR>
__device__ __noinline__ void stroke_short_paths(const StrokeArgs& A, uint32_t split, int lane) {
    for (;;) {
        uint32_t first = 0;
        if (lane == 0) first = atomicAdd(A.seq_counter, 32u);
        first = __shfl_sync(FULL, first, 0);
        if (first >= A.num_paths - split) break;
        const uint32_t item = split + first + (uint32_t)lane;
        if (item < A.num_paths) {
            const uint32_t path = A.order[item];
            if (!EMIT || A.status[path] == LYON_OK) stroke_path_seq<EMIT, ATTR>(A, path);
        }
        __syncwarp();
    }
}

template <bool EMIT, bool ATTR>
__global__ void __launch_bounds__(STROKE_WARPS * 32, LG_STROKE_MIN_BLOCKS)
    stroke_kernel(StrokeArgs A) {
    extern __shared__ unsigned char smem_raw[];
    WarpSmem* smem = reinterpret_cast<WarpSmem*>(smem_raw);
    const int lane = threadIdx.x & 31;
    const int w = threadIdx.x >> 5;
    WarpSmem& sm = smem[w];
    uint32_t tqn = 0;  // queued tails
    const uint32_t split = A.item_split ? min(*A.item_split, A.num_paths) : A.num_paths;
    for (;;) {
        uint32_t item = 0;
        if (lane == 0) item = atomicAdd(A.work_counter, 1u);
        item = __shfl_sync(FULL, item, 0);
        if (item >= split) break;
        const uint32_t path = A.order ? A.order[item] : item;
        if (EMIT && A.status[path] != LYON_OK) continue;
        const PathOut po = path_out<EMIT, ATTR>(A, path);
        uint32_t vc, ic;
        int st;
        bool deferred;
        stroke_path<EMIT, ATTR>(sm, lane, A, path, po, vc, ic, st, tqn, deferred);
        if (!deferred && lane == 0) finish_path<EMIT>(A, path, vc, ic, st, po);
        __syncwarp();
    }
    if (tqn > 0) flush_tails<EMIT, ATTR>(sm, lane, tqn, A);
    if (split < A.num_paths) stroke_short_paths<EMIT, ATTR>(A, split, lane);
}

constexpr size_t STROKE_SMEM = sizeof(WarpSmem) * STROKE_WARPS;
constexpr int MAX_CONFIGURED_DEVICES = 64;
static bool smem_configured[MAX_CONFIGURED_DEVICES] = {};

// The dynamic shared memory limit is a per-device attribute of each kernel: set it once per
// device the kernels run on.
static void configure_smem() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_CONFIGURED_DEVICES) return;
    if (smem_configured[dev]) return;
    if (STROKE_SMEM > 48 * 1024) {
        cudaFuncSetAttribute(stroke_kernel<true, false>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)STROKE_SMEM);
        cudaFuncSetAttribute(stroke_kernel<true, true>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)STROKE_SMEM);
        cudaFuncSetAttribute(stroke_kernel<false, false>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)STROKE_SMEM);
    }
    smem_configured[dev] = true;
}

int stroke_blocks_per_sm() {
    configure_smem();
    int n = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, stroke_kernel<true, false>,
                                                  STROKE_WARPS * 32, STROKE_SMEM);
    return n > 0 ? n : 1;
}

cudaError_t launch_stroke(const StrokeArgs& args, bool emit, int grid, cudaStream_t stream) {
    // Variable line width and the custom-attribute output use lyon's sequential stepper, one
    // path per thread (stroke_seq.cu). A fixed-width custom-attribute call counts with this
    // file's warp kernel: both restate the same stroker, so the counts agree (and an emit pass
    // that disagreed would flag its path LYON_ERR_INTERNAL, its writes bounded by the counts).
    if (args.widths || (args.sequential && emit))
        return launch_stroke_seq(args, emit, grid, stream);
    configure_smem();
    // The attribute output is its own instantiation, so the positions kernel carries none of
    // its work (the advancement chain, the record stores).
    if (emit && args.vertex_attrs) {
        stroke_kernel<true, true><<<grid, STROKE_WARPS * 32, STROKE_SMEM, stream>>>(args);
    } else if (emit) {
        stroke_kernel<true, false><<<grid, STROKE_WARPS * 32, STROKE_SMEM, stream>>>(args);
    } else {
        stroke_kernel<false, false><<<grid, STROKE_WARPS * 32, STROKE_SMEM, stream>>>(args);
    }
    note_launches(1);
    return cudaGetLastError();
}

}  // namespace lg
