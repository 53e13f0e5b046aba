// stroke.cu — batched fixed-width stroke tessellation (count and emit kernels).
//
// One warp strokes one path at a time; warps of a persistent grid take paths from an atomic
// work counter. For each sub-path the warp
//   1. loads up to 32 verbs (a window ending at the sub-path's End/Close), derives each curve's
//      flattening parameters (lyon's `flattened_segments_wang`, and the sharp-turn split of
//      quadratics from stroke.rs:2755-2779), and scans the per-verb step counts;
//   2. generates the flattened points in chunks of CH = 32 * RUN: lane i owns RUN consecutive
//      points, evaluates lyon's accumulated parameter t in closed form for its first point
//      (accumulate_t) and then sequentially (t += step, exactly as lyon), and writes the points
//      into a per-warp ring in shared memory;
//   3. applies the merge filter of stroke.rs:1530-1536: every lane checks its points against
//      their predecessors; only when one is within the threshold does lane 0 replay the chain
//      and compact the chunk;
//   4. processes the joins in chunks of CH (lane i owns RUN consecutive joins): a counting pass
//      (flattening-step joins need no arithmetic beyond a bound that proves lyon's skip test
//      cannot fire), a warp scan for the output offsets, then the emission pass, which stages
//      the chunk's vertices and indices in shared memory and copies them out coalesced;
//   5. runs the sub-path tail (caps, closing, empty caps) on lane 0.
// The count kernel runs steps 1-5 without writing; a look-back scan turns its per-path counts
// into offsets; the emit kernel repeats the walk and writes at those offsets.
#include "stroke_core.cuh"
#include "kernels.h"

namespace lg {

#ifndef LG_STROKE_WARPS
#define LG_STROKE_WARPS 4
#endif
#ifndef LG_STROKE_MIN_BLOCKS
#define LG_STROKE_MIN_BLOCKS 1
#endif
#ifndef LG_RUN
#define LG_RUN 4
#endif
constexpr int STROKE_WARPS = LG_STROKE_WARPS;
constexpr uint32_t RUN = LG_RUN;          // points (and joins) per lane
constexpr uint32_t CH = 32 * RUN;         // points per chunk
constexpr uint32_t RING = 4 * CH;         // kept-point ring (power of two)
constexpr uint32_t RMASK = RING - 1;
constexpr uint32_t STAGE_V = 2 * CH + 64;  // staged vertices per join chunk
constexpr uint32_t STAGE_I = 6 * CH + 192; // staged indices per join chunk
constexpr uint32_t FULL = 0xFFFFFFFFu;
constexpr uint32_t MAX_VERB_STEPS = 1u << 26;

struct VerbSlot {
    Poly pA, pB;
    V2 toA, toB;
    float sA, sB;
    uint32_t mA, mB;
    uint32_t excl, steps;  // first step of the verb within the window, step count
    int kind;
};

struct WarpSmem {
    VerbSlot verbs[32];
    float2 kp[RING];
    uint8_t kflat[RING];
    float2 sv[STAGE_V];
    uint32_t si[STAGE_I];
    DEP carry;   // last join processed (J_{next_join - 1}), with ids
    DEP first0;  // first kept point of the sub-path, with its side points
    DEP first1;  // J_1 after its processing (lyon's firsts[1])
};

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v, int lane) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t n = __shfl_up_sync(FULL, v, o);
        if (lane >= o) v += n;
    }
    return v;
}

struct PathOut {
    uint32_t id_base;  // id of the path's first vertex
    float2* vout;      // null when counting
    void* iout;
    int bits;
    uint32_t vmax, imax;  // the path's counts from the count pass (write bounds when emitting)
};

__device__ __forceinline__ uint32_t cap_left(uint32_t total, uint32_t used) {
    return used < total ? total - used : 0u;
}

// Warp-uniform summary of the last processed join (lyon's point buffer entry before the next
// join), used by lane 0 of the next chunk.
struct JCarry {
    V2 pn, nn;            // side next points
    uint32_t from_f;      // id structure of the edge leaving the join
    uint32_t fneg, fpos;  // ids the next edge starts from
    bool sym;             // side next points symmetric about the join point
};

__device__ __forceinline__ JCarry carry_from_dep(const DEP& d, bool sym) {
    JCarry c;
    c.pn = d.s[SP].next;
    c.nn = d.s[SN].next;
    edge_ids_from(d, &c.fneg, &c.fpos);
    c.from_f = id_flags(c.fneg, c.fpos);
    c.sym = sym;
    return c;
}

// t state carried across step chunks: the chunk's last step.
struct TCarry {
    uint32_t verb;  // absolute verb index, or ~0 when the last step was not inside a curve
    uint32_t unit;
    uint32_t k;
    float t;
};

__device__ __forceinline__ uint32_t points_of_verb(int kind) {
    switch (kind) {
        case LYON_VERB_LINE_TO: return 1;
        case LYON_VERB_QUADRATIC_TO: return 2;
        case LYON_VERB_CUBIC_TO: return 3;
        case LYON_VERB_BEGIN: return 1;
        case LYON_VERB_CLOSE: return 1;
        default: return 0;
    }
}

// Flattening parameters of one verb of a window (lane = verb): lines and Begin give one step;
// quadratics are split at a sharp turn (stroke.rs:2755-2779, 3178-3212) and each part gets lyon's
// segment count (quadratic_bezier.rs:943-974); cubics likewise (cubic_bezier.rs:1369-1403).
// Returns the number of flattened points the verb contributes.
__device__ __noinline__ uint32_t setup_verb(VerbSlot& out, int kind, uint32_t pofs,
                                            uint32_t pcount, uint32_t p_end, const float* points,
                                            float tolerance, int* vst) {
    VerbSlot sl;
    sl.kind = kind;
    sl.mA = 0;
    sl.mB = 0;
    sl.sA = sl.sB = 0.0f;
    uint32_t steps = 0;
    if (pofs + pcount > p_end || kind < 0) {
        *vst = LYON_ERR_INVALID_ARGUMENT;
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
        *vst = LYON_ERR_UNSUPPORTED;
        steps = 0;
    }
    sl.steps = steps;
    sl.excl = 0;
    out = sl;
    return steps;
}

// The merge filter replayed on lane 0 over a chunk whose points start at kept index n0
// (stroke.rs:1530-1536): points within the threshold of the last kept point are dropped and the
// kept ones compacted in place. Returns the new kept count.
__device__ __noinline__ uint32_t merge_compact(WarpSmem& sm, uint32_t n0, uint32_t nsteps,
                                               V2 lastk, float thr, bool* mnec) {
    V2 L = lastk;
    uint32_t cnt = n0;
    for (uint32_t i = 0; i < nsteps; ++i) {
        float2 q = sm.kp[(n0 + i) & RMASK];
        V2 pi = V2{q.x, q.y};
        uint8_t fl = sm.kflat[(n0 + i) & RMASK];
        if (cnt > 0 && too_close(L, pi, thr)) {
            if (cnt == 1) *mnec = true;
            continue;
        }
        sm.kp[cnt & RMASK] = q;
        sm.kflat[cnt & RMASK] = fl;
        L = pi;
        ++cnt;
    }
    return cnt;
}

// A join's DEP with ids (fast joins: the flattened_step layout; general joins: recomputed), for
// the carry and lyon's firsts[1].
__device__ __noinline__ void join_dep_with_ids(DEP* out, V2 prev, V2 cur, V2 nxt, bool flat,
                                               bool fast, bool skip, uint32_t base_id,
                                               const StrokeParams& P, int* status) {
    if (fast) {
        V2 pe = cur - prev;
        float pl = vlength(pe);
        V2 pt = pe / pl;
        V2 ne = nxt - cur;
        float nl = vlength(ne);
        V2 nt = ne / nl;
        V2 nrm = compute_normal(pt, nt);
        fast_join_dep(*out, cur, P.hw, cur + nrm * P.hw, cur - nrm * P.hw,
                      skip ? INVALID_ID : base_id, skip ? INVALID_ID : base_id + 1);
    } else {
        SlowJoin sj;
        DEP d;
        slow_join_geometry(&d, prev, cur, flat, nxt, P, &sj, status);
        Sink probe{base_id, 0, 0, nullptr, nullptr, 32};
        add_join_base_vertices(d, SN, probe);
        add_join_base_vertices(d, SP, probe);
        *out = d;
    }
}

// Side "next" points of the join at kept index k (exact path of the skip test).
__device__ __noinline__ void join_side_next(const WarpSmem& sm, uint32_t k, const StrokeParams& P,
                                            V2* pn, V2* nn) {
    float2 a = sm.kp[(k - 1) & RMASK], b = sm.kp[k & RMASK], c = sm.kp[(k + 1) & RMASK];
    V2 prev = V2{a.x, a.y}, cur = V2{b.x, b.y}, nxt = V2{c.x, c.y};
    bool flat = sm.kflat[k & RMASK] != 0;
    if (flat && dot(cur - prev, nxt - cur) > 0.0f) {
        V2 pe = cur - prev;
        V2 pt = pe / vlength(pe);
        V2 ne = nxt - cur;
        V2 nt = ne / vlength(ne);
        V2 nrm = compute_normal(pt, nt);
        *pn = cur + nrm * P.hw;
        *nn = cur - nrm * P.hw;
    } else {
        DEP d;
        SlowJoin sj;
        int st = LYON_OK;
        slow_join_geometry(&d, prev, cur, flat, nxt, P, &sj, &st);
        *pn = sj.pn;
        *nn = sj.nn;
    }
}

// Whether the join at kept index k has symmetric side points (all but clipped miters).
__device__ __forceinline__ bool join_is_sym(const WarpSmem& sm, uint32_t k, const StrokeParams& P) {
    if (P.line_join != LYON_JOIN_MITER_CLIP) return true;
    float2 a = sm.kp[(k - 1) & RMASK], b = sm.kp[k & RMASK], c = sm.kp[(k + 1) & RMASK];
    bool flat = sm.kflat[k & RMASK] != 0;
    return flat && ((b.x - a.x) * (c.x - b.x) + (b.y - a.y) * (c.y - b.y)) > 0.0f;
}

// Processes `count` (1..CH) joins starting at kept index `nj` (lane i owns RUN consecutive
// joins). Updates the carry, first1 and the output cursors.
template <bool EMIT>
__device__ __noinline__ void process_joins(WarpSmem& sm, int lane, uint32_t nj, uint32_t count,
                                           const StrokeParams& P, const PathOut& po,
                                           uint32_t& vcur, uint32_t& icur, int& status,
                                           JCarry& jc) {
    const uint32_t k0 = nj + (uint32_t)lane * RUN;
    const uint32_t kend = min(k0 + RUN, nj + count);
    int st = LYON_OK;

    // ---- pass 1: counts ----
    // Flattening-step joins (stroke.rs:1743-1806) take 2 vertices and their edge 2 triangles,
    // unless flattened_step's skip test fires; with side points symmetric about the previous
    // point that needs the previous edge to be shorter than a few ulps of the coordinates (the
    // bound below follows from the roundings of p0, p1 and the side points), so the test is only
    // evaluated exactly when the bound fails somewhere in the chunk.
    uint32_t V = 0, I = 0;
    uint32_t first_to_f = 0, pf = 0;
    uint32_t last_voff = 0, last_fneg_rel = INVALID_ID, last_fpos_rel = INVALID_ID;
    bool last_fast = true, last_skip = false;
    bool k1_fast = true, k1_skip = false;
    bool exact = false;
    for (int attempt = 0; attempt < 2; ++attempt) {
        V = 0;
        I = 0;
        bool need = false;
        V2 ppn = V2{0.0f, 0.0f}, pnn = V2{0.0f, 0.0f};
        bool psym = true;
        if (k0 < kend) {
            if (k0 == nj) {
                ppn = jc.pn;
                pnn = jc.nn;
                psym = jc.sym;
            } else {
                psym = join_is_sym(sm, k0 - 1, P);
                if (exact) join_side_next(sm, k0 - 1, P, &ppn, &pnn);
            }
        }
        for (uint32_t k = k0; k < kend; ++k) {
            float2 a = sm.kp[(k - 1) & RMASK], b = sm.kp[k & RMASK], c = sm.kp[(k + 1) & RMASK];
            V2 prev = V2{a.x, a.y}, cur = V2{b.x, b.y}, nxt = V2{c.x, c.y};
            bool flat = sm.kflat[k & RMASK] != 0;
            V2 pe = cur - prev;
            bool fast = flat && dot(pe, nxt - cur) > 0.0f;
            uint32_t vc, jt, to_f, from_f, fneg_rel, fpos_rel;
            bool skip = false, sym = true;
            if (fast) {
                if (exact) {
                    V2 pt = pe / vlength(pe);
                    V2 ne = nxt - cur;
                    V2 nt = ne / vlength(ne);
                    V2 nrm = compute_normal(pt, nt);
                    V2 pn = cur + nrm * P.hw, nn = cur - nrm * P.hw;
                    skip = dot(pe, pn - ppn) < 0.0f && dot(pe, nn - pnn) < 0.0f;
                    ppn = pn;
                    pnn = nn;
                } else {
                    float m = fmaxf(fmaxf(fabsf(cur.x), fabsf(cur.y)),
                                    fmaxf(fabsf(prev.x), fabsf(prev.y))) + 3.0f * P.hw;
                    float bnd = m * 7.62939453125e-06f;  // 2^-17
                    if (!(psym && sqlen(pe) > bnd * bnd)) need = true;
                }
                vc = skip ? 0u : 2u;
                jt = 0;
                to_f = from_f = skip ? (EF_NEG_INV | EF_POS_INV | EF_SELF_EQ) : 0u;
                fneg_rel = skip ? INVALID_ID : 1u;
                fpos_rel = skip ? INVALID_ID : 0u;
            } else {
                DEP d;
                SlowJoin sj;
                slow_join_geometry(&d, prev, cur, flat, nxt, P, &sj, &st);
                vc = sj.vcount;
                jt = sj.jtris;
                to_f = sj.to_f;
                from_f = sj.from_f;
                fneg_rel = sj.from_neg_rel;
                fpos_rel = sj.from_pos_rel;
                sym = sj.sym;
                ppn = sj.pn;
                pnn = sj.nn;
            }
            uint32_t e = 0;
            if (k == k0) {
                first_to_f = to_f;
            } else if (k >= 2) {
                e = edge_count_flags(pf, to_f);
            }
            last_voff = V;
            last_fneg_rel = fneg_rel;
            last_fpos_rel = fpos_rel;
            last_fast = fast;
            last_skip = skip;
            if (k == 1) {
                k1_fast = fast;
                k1_skip = skip;
            }
            V += vc;
            I += 3u * (jt + e);
            pf = from_f;
            psym = fast ? true : sym;
        }
        if (exact || !__any_sync(FULL, need)) break;
        exact = true;
    }
    // Edge triangles of each run's first join need the previous run's last join.
    uint32_t pff = __shfl_up_sync(FULL, pf, 1);
    if (lane == 0) pff = jc.from_f;
    if (k0 < kend && k0 >= 2) I += 3u * edge_count_flags(pff, first_to_f);
    const uint32_t vincl = warp_incl_scan(V, lane);
    const uint32_t iincl = warp_incl_scan(I, lane);
    const uint32_t vtot = __shfl_sync(FULL, vincl, 31);
    const uint32_t itot = __shfl_sync(FULL, iincl, 31);
    const uint32_t vrel = vincl - V;
    const uint32_t irel = iincl - I;
    const uint32_t base_id = po.id_base + vcur + vrel;
    // Ids the next run's first edge starts from.
    uint32_t fneg = INVALID_ID, fpos = INVALID_ID;
    if (k0 < kend) {
        fneg = last_fneg_rel == INVALID_ID ? INVALID_ID : base_id + last_voff + last_fneg_rel;
        fpos = last_fpos_rel == INVALID_ID ? INVALID_ID : base_id + last_voff + last_fpos_rel;
    }
    uint32_t pfn = __shfl_up_sync(FULL, fneg, 1);
    uint32_t pfp = __shfl_up_sync(FULL, fpos, 1);
    if (lane == 0) {
        pfn = jc.fneg;
        pfp = jc.fpos;
    }

    // ---- pass 2: emission ----
    if (EMIT) {
        const bool staged = vtot <= STAGE_V && itot <= STAGE_I;
        float2* vdst = staged ? sm.sv : po.vout + vcur;
        uint32_t* i32dst = staged ? sm.si : (po.bits == 32 ? (uint32_t*)po.iout + icur : nullptr);
        uint16_t* i16dst = (!staged && po.bits == 16) ? (uint16_t*)po.iout + icur : nullptr;
        const uint32_t vlim = staged ? STAGE_V : cap_left(po.vmax, vcur);
        const uint32_t ilim = staged ? STAGE_I : cap_left(po.imax, icur);
        uint32_t vo = vrel, io = irel;
        uint32_t pneg = pfn, ppos = pfp;
        V2 ppn = jc.pn, pnn = jc.nn;
        if (k0 < kend && k0 != nj && exact) join_side_next(sm, k0 - 1, P, &ppn, &pnn);
        for (uint32_t k = k0; k < kend; ++k) {
            float2 a = sm.kp[(k - 1) & RMASK], b = sm.kp[k & RMASK], c = sm.kp[(k + 1) & RMASK];
            V2 prev = V2{a.x, a.y}, cur = V2{b.x, b.y}, nxt = V2{c.x, c.y};
            bool flat = sm.kflat[k & RMASK] != 0;
            V2 pe = cur - prev;
            bool fast = flat && dot(pe, nxt - cur) > 0.0f;
            const uint32_t my_id = po.id_base + vcur + vo;
            if (fast) {
                V2 pt = pe / vlength(pe);
                V2 ne = nxt - cur;
                V2 nt = ne / vlength(ne);
                V2 nrm = compute_normal(pt, nt);
                V2 pn = cur + nrm * P.hw, nn = cur - nrm * P.hw;
                bool skip = exact && dot(pe, pn - ppn) < 0.0f && dot(pe, nn - pnn) < 0.0f;
                ppn = pn;
                pnn = nn;
                uint32_t pos_id = INVALID_ID, neg_id = INVALID_ID;
                if (!skip) {
                    if (vo + 2 <= vlim) {
                        vdst[vo] = make_float2(pn.x, pn.y);
                        vdst[vo + 1] = make_float2(nn.x, nn.y);
                    } else {
                        st = LYON_ERR_INTERNAL;
                    }
                    pos_id = my_id;
                    neg_id = my_id + 1;
                    vo += 2;
                }
                if (k >= 2) {
                    Sink s{my_id, 0, 0, nullptr, nullptr, 32};
                    if (i32dst) s.iout = i32dst + io;
                    if (i16dst) {
                        s.iout = i16dst + io;
                        s.index_bits = 16;
                    }
                    s.icap = cap_left(ilim, io);
                    edge_triangles(pneg, ppos, neg_id, pos_id, &s);
                    if (s.overflow) st = LYON_ERR_INTERNAL;
                    io += s.ni;
                }
                pneg = neg_id;
                ppos = pos_id;
            } else {
                DEP d;
                SlowJoin sj;
                slow_join_geometry(&d, prev, cur, flat, nxt, P, &sj, &st);
                ppn = sj.pn;
                pnn = sj.nn;
                Sink s;
                s.id_base = my_id;
                s.nv = 0;
                s.ni = 0;
                s.vout = vdst + vo;
                s.index_bits = i16dst ? 16 : 32;
                s.iout = i16dst ? (void*)(i16dst + io) : (void*)(i32dst + io);
                s.vcap = cap_left(vlim, vo);
                s.icap = cap_left(ilim, io);
                s.overflow = false;
                slow_join_emit(&d, &d, s, k >= 2, pneg, ppos, true, P, &st);
                if (s.overflow) st = LYON_ERR_INTERNAL;
                edge_ids_from(d, &pneg, &ppos);
                vo += s.nv;
                io += s.ni;
            }
        }
        __syncwarp();
        if (staged) {
            // Coalesced copy-out of the chunk's vertices and indices.
            const float* sf = reinterpret_cast<const float*>(sm.sv);
            float* df = reinterpret_cast<float*>(po.vout + vcur);
            for (uint32_t w = lane; w < 2 * vtot; w += 32) df[w] = sf[w];
            if (po.bits == 16) {
                uint16_t* di = (uint16_t*)po.iout + icur;
                for (uint32_t w = lane; w < itot; w += 32) di[w] = (uint16_t)sm.si[w];
            } else {
                uint32_t* di = (uint32_t*)po.iout + icur;
                for (uint32_t w = lane; w < itot; w += 32) di[w] = sm.si[w];
            }
        }
    }

    // ---- carry, firsts[1] ----
    const uint32_t last_k = nj + count - 1;
    if (k0 <= last_k && last_k < kend) {
        float2 a = sm.kp[(last_k - 1) & RMASK], b = sm.kp[last_k & RMASK],
               c = sm.kp[(last_k + 1) & RMASK];
        join_dep_with_ids(&sm.carry, V2{a.x, a.y}, V2{b.x, b.y}, V2{c.x, c.y},
                          sm.kflat[last_k & RMASK] != 0, last_fast, last_skip,
                          base_id + last_voff, P, &st);
    }
    if (k0 <= 1 && 1 < kend) {
        // J_1 is the first join of lane 0's run in the first chunk of the sub-path.
        float2 a = sm.kp[0], b = sm.kp[1], c = sm.kp[2];
        join_dep_with_ids(&sm.first1, V2{a.x, a.y}, V2{b.x, b.y}, V2{c.x, c.y},
                          sm.kflat[1] != 0, k1_fast, k1_skip, base_id, P, &st);
    }
    __syncwarp();
    const uint32_t owner = (last_k - nj) / RUN;
    bool lsym = __shfl_sync(FULL, last_fast ? true : (P.line_join != LYON_JOIN_MITER_CLIP),
                            (int)owner);
    jc = carry_from_dep(sm.carry, lsym);
    if (__any_sync(FULL, st != LYON_OK)) {
        int e = __reduce_max_sync(FULL, st);
        if (status == LYON_OK) status = e;
    }
    vcur += vtot;
    icur += itot;
    __syncwarp();
}

// The tail of a sub-path on lane 0: stroke.rs:1179-1279 (end, close) and 1322-1378
// (end_with_caps).
__device__ __noinline__ void subpath_tail(WarpSmem& sm, uint32_t n, bool close,
                                          bool may_need_empty_cap, const StrokeParams& P,
                                          Sink& s, int* status) {
    may_need_empty_cap |= close && n == 1;
    if (close && n > 2) {
        SeqBuffer pb;
        pb.pts[0] = sm.carry;
        float2 ql = sm.kp[(n - 1) & RMASK];
        dep_init(pb.pts[1], V2{ql.x, ql.y}, P.hw, P.line_join, sm.kflat[(n - 1) & RMASK] != 0);
        pb.start = 0;
        pb.count = 2;
        pb.n = n;
        bool mnec = false;
        DEP p = sm.first0;
        bool added = seq_step(pb, p, P, s, &mnec, status);
        if (!added) pb.last().pos = p.pos;
        DEP p2 = sm.first1;
        seq_step(pb, p2, P, s, &mnec, status);
        DEP& p0 = pb.second_last();
        DEP& p1 = pb.last();
        for (int side = 0; side < 2; ++side) {
            V2 sp = p0.s[side].has_single ? p0.s[side].single : p0.s[side].next;
            V2 normal = (sp - p0.pos) / p0.hw;
            p0.s[side].next_vertex = s.vertex(p0.pos + normal * p0.hw);
        }
        add_edge_triangles(p0, p1, s);
        return;
    }
    if (may_need_empty_cap && n == 1) {
        V2 pos = sm.first0.pos;
        if (P.start_cap == LYON_CAP_SQUARE) {
            tessellate_empty_square_cap(pos, P.hw, s);
        } else if (P.start_cap == LYON_CAP_ROUND) {
            tessellate_empty_round_cap(pos, P.hw, P, s, status);
        }
        return;
    }
    if (n >= 2) {
        DEP p0 = (n == 2) ? sm.first0 : sm.carry;
        DEP p1;
        float2 ql = sm.kp[(n - 1) & RMASK];
        dep_init(p1, V2{ql.x, ql.y}, P.hw, P.line_join, sm.kflat[(n - 1) & RMASK] != 0);
        V2 tan = normalize(p1.pos - p0.pos);
        V2 nn = V2{-tan.y, tan.x} * p1.hw;
        p1.s[SP].prev = p1.pos + nn;
        p1.s[SN].prev = p1.pos - nn;
        tessellate_last_edge(p0, p1, n == 2, P, s, status);
        if (n > 2) {
            p0 = sm.first0;
            p1 = sm.first1;
        }
        tessellate_first_edge(p0, p1, P, s, status);
    }
}

// Generates the window steps [cb, min(cb + CH, S_w)) into the ring at kept indices n0...
// (lane i owns RUN consecutive steps) and updates the t carry.
__device__ __forceinline__ void gen_steps(WarpSmem& sm, int lane, uint32_t vi, uint32_t nv,
                                          uint32_t sincl, uint32_t S_w, uint32_t cb, uint32_t n0,
                                          TCarry& tc) {
    const uint32_t g0 = cb + (uint32_t)lane * RUN;
    const uint32_t gend = min(g0 + RUN, S_w);
    // Owner verb of g0: first lane whose inclusive step count exceeds it.
    const uint32_t gq = min(g0, S_w - 1);
    uint32_t lo = 0, hi = nv - 1;
#pragma unroll
    for (int it = 0; it < 5; ++it) {
        uint32_t mid = (lo + hi) >> 1;
        uint32_t vmid = __shfl_sync(FULL, sincl, mid);
        if (vmid > gq) hi = mid; else lo = mid + 1;
        if (lo > hi) lo = hi;
    }
    uint32_t j = lo;
    const TCarry c0 = tc;
    uint32_t my_verb = 0xFFFFFFFFu, my_unit = 0, my_k = 0;
    float my_t = 0.0f;
    if (g0 < gend) {
        uint32_t r = g0 - sm.verbs[j].excl;
        int kind = sm.verbs[j].kind;
        uint32_t vsteps = sm.verbs[j].steps;
        int tunit = -1;
        uint32_t tk = 0;
        float t = 0.0f;
        for (uint32_t g = g0; g < gend; ++g) {
            while (r >= vsteps) {
                ++j;
                r = 0;
                kind = sm.verbs[j].kind;
                vsteps = sm.verbs[j].steps;
                tunit = -1;
            }
            const VerbSlot& sl = sm.verbs[j];
            V2 pos;
            bool flat = false;
            my_verb = 0xFFFFFFFFu;
            if (kind == LYON_VERB_BEGIN || kind == LYON_VERB_LINE_TO) {
                pos = sl.toA;
            } else {
                const uint32_t mA = sl.mA;
                const bool unitA = r < mA;
                const uint32_t kk = unitA ? r + 1 : r - mA + 1;
                const uint32_t m = unitA ? mA : sl.mB;
                const int u = unitA ? 0 : 1;
                if (kk < m) {
                    const float s = unitA ? sl.sA : sl.sB;
                    if (tunit == u && tk + 1 == kk) {
                        t = t + s;
                    } else {
                        uint32_t bk = 0;
                        float bt = 0.0f;
                        if (c0.verb == vi + j && c0.unit == (uint32_t)u && c0.k <= kk) {
                            bk = c0.k;
                            bt = c0.t;
                        }
                        t = accumulate_t(s, bk, bt, kk);
                    }
                    tunit = u;
                    tk = kk;
                    pos = poly_sample(unitA ? sl.pA : sl.pB, t);
                    flat = t != 1.0f;
                    my_verb = vi + j;
                    my_unit = (uint32_t)u;
                    my_k = kk;
                    my_t = t;
                } else {
                    pos = unitA ? sl.toA : sl.toB;
                    tunit = -1;
                }
            }
            const uint32_t idx = (n0 + (g - cb)) & RMASK;
            sm.kp[idx] = make_float2(pos.x, pos.y);
            sm.kflat[idx] = flat ? 1 : 0;
            ++r;
        }
    }
    // t carry: the state after the chunk's last step.
    const uint32_t last_g = min(cb + CH, S_w) - 1;
    const int owner = (int)((last_g - cb) / RUN);
    tc.verb = __shfl_sync(FULL, my_verb, owner);
    tc.unit = __shfl_sync(FULL, my_unit, owner);
    tc.k = __shfl_sync(FULL, my_k, owner);
    tc.t = __shfl_sync(FULL, my_t, owner);
    __syncwarp();
}

// Strokes one path with the whole warp. Returns the path's vertex/index counts via vcur/icur.
template <bool EMIT>
__device__ void stroke_path(WarpSmem& sm, int lane, const StrokeArgs& A, uint32_t path,
                            const PathOut& po, uint32_t& vcur, uint32_t& icur, int& status) {
    const uint32_t v_begin = A.verb_offsets[path], v_end = A.verb_offsets[path + 1];
    const uint32_t p_begin = A.point_offsets[path], p_end = A.point_offsets[path + 1];
    const lyon_stroke_options opt = A.options[A.num_options > 1 ? path : 0];
    const StrokeParams P = make_params(opt);
    vcur = 0;
    icur = 0;
    status = LYON_OK;
    uint32_t vi = v_begin;
    uint32_t pc = p_begin;
    while (vi < v_end && status == LYON_OK) {
        // A sub-path starts with Begin (crates/path/src/path.rs:843-909).
        if (A.verbs[vi] != LYON_VERB_BEGIN) {
            status = LYON_ERR_INVALID_ARGUMENT;
            break;
        }
        uint32_t n_kept = 0;
        uint32_t next_join = 1;
        bool mnec = false;
        V2 lastk = V2{0.0f, 0.0f};
        TCarry tc;
        tc.verb = 0xFFFFFFFFu;
        tc.unit = 0;
        tc.k = 0;
        tc.t = 0.0f;
        bool ended = false, closed = false;
        bool first_sides_done = false;
        JCarry jc;
        jc.pn = jc.nn = V2{0.0f, 0.0f};
        jc.from_f = EF_NEG_INV | EF_POS_INV | EF_SELF_EQ;
        jc.fneg = jc.fpos = INVALID_ID;
        jc.sym = true;
        while (vi < v_end && status == LYON_OK) {
            // ---- 1. verb window ----
            const uint32_t v = vi + (uint32_t)lane;
            const bool valid = v < v_end;
            int kind = valid ? (int)A.verbs[v] : LYON_VERB_END;
            const bool is_end = valid && (kind == LYON_VERB_END || kind == LYON_VERB_CLOSE);
            const bool bad_begin = valid && lane > 0 && kind == LYON_VERB_BEGIN;
            const uint32_t endmask = __ballot_sync(FULL, is_end || bad_begin);
            uint32_t nv = min(32u, v_end - vi);
            if (endmask) nv = min(nv, (uint32_t)(__ffs(endmask)));
            const bool inwin = (uint32_t)lane < nv;
            if (inwin && bad_begin) kind = -1;
            const uint32_t pcount = inwin ? points_of_verb(kind) : 0u;
            const uint32_t pincl = warp_incl_scan(pcount, lane);
            const uint32_t pofs = pc + pincl - pcount;
            uint32_t steps = 0;
            int vst = LYON_OK;
            if (inwin) steps = setup_verb(sm.verbs[lane], kind, pofs, pcount, p_end, A.points,
                                          P.tolerance, &vst);
            if (__any_sync(FULL, vst != LYON_OK)) {
                status = __reduce_max_sync(FULL, vst);
                break;
            }
            const uint32_t sincl = warp_incl_scan(steps, lane);
            if (inwin) sm.verbs[lane].excl = sincl - steps;
            const uint32_t S_w = __shfl_sync(FULL, sincl, 31);
            const int last_kind = __shfl_sync(FULL, kind, nv - 1);
            __syncwarp();

            // ---- 2./3. points, CH at a time ----
            for (uint32_t cb = 0; cb < S_w; cb += CH) {
                const uint32_t nsteps = min(CH, S_w - cb);
                const uint32_t n0 = n_kept;
                gen_steps(sm, lane, vi, nv, sincl, S_w, cb, n0, tc);
                // Merge filter (stroke.rs:1530-1536).
                bool close_any = false;
                {
                    const uint32_t g0 = (uint32_t)lane * RUN;
                    const uint32_t ge = min(g0 + RUN, nsteps);
                    for (uint32_t g = g0; g < ge; ++g) {
                        const uint32_t idx = n0 + g;
                        if (idx == 0) continue;
                        float2 q = sm.kp[idx & RMASK];
                        V2 prevp;
                        if (g == 0) {
                            prevp = lastk;
                        } else {
                            float2 pq = sm.kp[(idx - 1) & RMASK];
                            prevp = V2{pq.x, pq.y};
                        }
                        if (too_close(prevp, V2{q.x, q.y}, P.merge_threshold)) close_any = true;
                    }
                }
                if (__any_sync(FULL, close_any)) {
                    uint32_t nk = 0;
                    bool m = mnec;
                    if (lane == 0) nk = merge_compact(sm, n0, nsteps, lastk, P.merge_threshold, &m);
                    n_kept = __shfl_sync(FULL, nk, 0);
                    mnec = __shfl_sync(FULL, m, 0);
                } else {
                    n_kept = n0 + nsteps;
                }
                __syncwarp();
                {
                    float2 lq = sm.kp[(n_kept - 1) & RMASK];
                    lastk = V2{lq.x, lq.y};
                }
                if (!first_sides_done && n_kept >= 2) {
                    if (lane == 0) {
                        float2 q0 = sm.kp[0];
                        float2 q1 = sm.kp[1];
                        dep_init(sm.first0, V2{q0.x, q0.y}, P.hw, P.line_join, false);
                        first_point_sides(sm.first0, V2{q1.x, q1.y}, P.hw);
                    }
                    first_sides_done = true;
                    __syncwarp();
                    jc = carry_from_dep(sm.first0, true);
                } else if (n_kept == 1 && lane == 0 && !first_sides_done) {
                    float2 q0 = sm.kp[0];
                    dep_init(sm.first0, V2{q0.x, q0.y}, P.hw, P.line_join, false);
                }
                __syncwarp();
                // ---- 4. joins, CH at a time ----
                while (n_kept >= next_join + 2 && n_kept - 1 - next_join >= CH) {
                    process_joins<EMIT>(sm, lane, next_join, CH, P, po, vcur, icur, status, jc);
                    next_join += CH;
                }
            }
            vi += nv;
            pc += __shfl_sync(FULL, pincl, 31);
            if (last_kind == LYON_VERB_END || last_kind == LYON_VERB_CLOSE) {
                ended = true;
                closed = last_kind == LYON_VERB_CLOSE;
                break;
            }
        }
        if (!ended || status != LYON_OK) break;
        // Remaining joins.
        while (n_kept >= 3 && next_join <= n_kept - 2) {
            const uint32_t cnt = min(CH, n_kept - 1 - next_join);
            process_joins<EMIT>(sm, lane, next_join, cnt, P, po, vcur, icur, status, jc);
            next_join += cnt;
        }
        // ---- 5. tail ----
        uint32_t tv = 0, ti = 0;
        int tst = LYON_OK;
        if (lane == 0) {
            Sink s;
            s.id_base = po.id_base + vcur;
            s.nv = 0;
            s.ni = 0;
            s.vout = EMIT ? po.vout + vcur : nullptr;
            s.iout = nullptr;
            if (EMIT) {
                s.iout = po.bits == 16 ? (void*)((uint16_t*)po.iout + icur)
                                       : (void*)((uint32_t*)po.iout + icur);
            }
            s.index_bits = po.bits;
            s.vcap = cap_left(po.vmax, vcur);
            s.icap = cap_left(po.imax, icur);
            s.overflow = false;
            subpath_tail(sm, n_kept, closed, mnec, P, s, &tst);
            if (s.overflow && tst == LYON_OK) tst = LYON_ERR_INTERNAL;
            tv = s.nv;
            ti = s.ni;
        }
        tv = __shfl_sync(FULL, tv, 0);
        ti = __shfl_sync(FULL, ti, 0);
        tst = __shfl_sync(FULL, tst, 0);
        if (tst != LYON_OK && status == LYON_OK) status = tst;
        vcur += tv;
        icur += ti;
        __syncwarp();
    }
}

template <bool EMIT>
__global__ void __launch_bounds__(STROKE_WARPS * 32, LG_STROKE_MIN_BLOCKS)
    stroke_kernel(StrokeArgs A) {
    extern __shared__ unsigned char smem_raw[];
    WarpSmem* smem = reinterpret_cast<WarpSmem*>(smem_raw);
    const int lane = threadIdx.x & 31;
    const int w = threadIdx.x >> 5;
    WarpSmem& sm = smem[w];
    for (;;) {
        uint32_t item = 0;
        if (lane == 0) item = atomicAdd(A.work_counter, 1u);
        item = __shfl_sync(FULL, item, 0);
        if (item >= A.num_paths) break;
        const uint32_t path = A.order ? A.order[item] : item;
        PathOut po;
        po.bits = A.index_bits;
        if (EMIT) {
            if (A.status[path] != LYON_OK) continue;
            const uint64_t vo = A.vtx_offsets[path];
            const uint64_t io = A.idx_offsets[path];
            po.vout = reinterpret_cast<float2*>(A.vertices) + vo;
            po.iout = A.index_bits == 16 ? (void*)((uint16_t*)A.indices + io)
                                         : (void*)((uint32_t*)A.indices + io);
            po.id_base = A.vertex_offset +
                         (A.index_mode == LYON_INDEX_GLOBAL ? (uint32_t)vo : 0u);
            po.vmax = A.vtx_counts[path];
            po.imax = A.idx_counts[path];
        } else {
            po.vout = nullptr;
            po.iout = nullptr;
            po.id_base = 0;
            po.vmax = 0xFFFFFFFFu;
            po.imax = 0xFFFFFFFFu;
        }
        uint32_t vc, ic;
        int st;
        stroke_path<EMIT>(sm, lane, A, path, po, vc, ic, st);
        if (!EMIT && lane == 0) {
            A.vtx_counts[path] = st == LYON_OK ? vc : 0u;
            A.idx_counts[path] = st == LYON_OK ? ic : 0u;
            A.status[path] = st;
        }
        if (EMIT && lane == 0 && (st != LYON_OK || vc != po.vmax || ic != po.imax)) {
            // The emit walk disagreed with the count walk: flag the path (its bytes were
            // bounded by the path's range).
            A.status[path] = st != LYON_OK ? st : LYON_ERR_INTERNAL;
        }
        __syncwarp();
    }
}

constexpr size_t STROKE_SMEM = sizeof(WarpSmem) * STROKE_WARPS;

static bool smem_configured = false;

static void configure_smem() {
    if (smem_configured) return;
    cudaFuncSetAttribute(stroke_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)STROKE_SMEM);
    cudaFuncSetAttribute(stroke_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)STROKE_SMEM);
    smem_configured = true;
}

int stroke_blocks_per_sm() {
    configure_smem();
    int n = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, stroke_kernel<true>, STROKE_WARPS * 32,
                                                  STROKE_SMEM);
    return n > 0 ? n : 1;
}

cudaError_t launch_stroke(const StrokeArgs& args, bool emit, int grid, cudaStream_t stream) {
    configure_smem();
    if (emit) {
        stroke_kernel<true><<<grid, STROKE_WARPS * 32, STROKE_SMEM, stream>>>(args);
    } else {
        stroke_kernel<false><<<grid, STROKE_WARPS * 32, STROKE_SMEM, stream>>>(args);
    }
    return cudaGetLastError();
}

}  // namespace lg
