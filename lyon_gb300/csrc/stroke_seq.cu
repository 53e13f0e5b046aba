// stroke_seq.cu — lyon's sequential stroke stepper, one path per thread.
//
// The warp-per-path kernel (stroke.cu) reproduces the fixed-width stroker's output without
// running its state machine step by step. Two outputs need the state machine itself:
//   * variable line width (StrokeOptions::variable_line_width, stroke.rs:654-767): every edge's
//     side attachments depend on both endpoints' widths (step_impl, stroke.rs:1380-1512);
//   * vertex sources (StrokeVertex::source, stroke.rs:2719-2722): every vertex carries the
//     VertexSource of the join, cap or edge it was made for, and custom attributes are
//     interpolated from those (StrokeVertex::interpolated_attributes, stroke.rs:2728-2747).
// Here one thread walks a path's events as tessellate_with_ids_fw/_vw do (stroke.rs:654-870):
// each endpoint or flattened curve point is stepped with fixed_width_step_impl
// (stroke.rs:1521-1632) or step_impl, and the sub-path ends with end/close/end_with_caps
// (stroke.rs:1179-1378). The sources of the points in the stepper's three-point buffer and of
// its `firsts` are kept beside them, so every emitted vertex gets its source the way lyon's
// `self.vertex.src` does. Both passes (count and emit) run this walk, so their counts agree by
// construction.
#include "stroke_core.cuh"
#include "stroke_out.cuh"
#include "kernels.h"

namespace lg {

namespace {

constexpr uint32_t FULL = 0xFFFFFFFFu;

__device__ __forceinline__ lyon_vertex_source endpoint_src(uint32_t id) {
    return lyon_vertex_source{id, LYON_NO_ENDPOINT, 0.0f};
}

// A point at parameter t of the curve between two endpoints; at t == 1 the end point itself
// (stroke.rs:1007-1016, 1045-1053, 1119-1128, 1154-1163).
__device__ __forceinline__ lyon_vertex_source curve_src(uint32_t from, uint32_t to, float t) {
    return t == 1.0f ? endpoint_src(to) : lyon_vertex_source{from, to, t};
}

// A sink that also writes every vertex's source: `src` is set by the stepper before each group
// of vertices, as `adv` is.
template <bool REC>
struct SrcSinkT : SinkT<REC> {
    static constexpr bool kSrc = true;
    lyon_vertex_source* sout;
    lyon_vertex_source src;
    __device__ __forceinline__ uint32_t vertex(V2 p, V2 n, int side) {
        if (this->nv < this->vcap) sout[this->nv] = src;
        return SinkT<REC>::vertex(p, n, side);
    }
};

template <class SK>
__device__ __forceinline__ void set_src(SK&, const lyon_vertex_source&) {}
template <bool REC>
__device__ __forceinline__ void set_src(SrcSinkT<REC>& s, const lyon_vertex_source& v) {
    s.src = v;
}
template <class SK>
__device__ __forceinline__ void set_sout(SK&, lyon_vertex_source*) {}
template <bool REC>
__device__ __forceinline__ void set_sout(SrcSinkT<REC>& s, lyon_vertex_source* p) {
    s.sout = p;
}

// The stepper's state (point buffer, firsts, may_need_empty_cap, sub_path_start_advancement)
// and the sources of the buffered points, slot for slot.
struct SeqStroker {
    VwState W;
    lyon_vertex_source src[3];
    lyon_vertex_source first_src[2];
};

__device__ __forceinline__ uint32_t slot_last(const SeqBuffer& pb) {
    return (pb.start + pb.count - 1) % 3;
}
__device__ __forceinline__ uint32_t slot_second_last(const SeqBuffer& pb) {
    return (pb.start + pb.count - 2) % 3;
}

// One step (fixed_width_step_impl or step_impl) of a point whose source is `src`. The vertices
// the step emits belong to the join at the buffer's last point, so they take its source. Without
// a source-writing sink the bookkeeping compiles away.
template <bool VW, class SK>
__device__ __forceinline__ bool seq_step_any(SeqStroker& S, const DEP& next,
                                             lyon_vertex_source src, const StrokeParams& P,
                                             SK& sink, int* status) {
    VwState& W = S.W;
    SeqBuffer& pb = W.pb;
    const uint32_t count0 = pb.count, start0 = pb.start, n0 = pb.n, nfirsts0 = W.nfirsts;
    if constexpr (SK::kSrc) {
        if (count0 > 0) set_src(sink, S.src[slot_last(pb)]);
    }
    bool ok;
    if constexpr (VW) {
        ok = vw_step(W, next, P, sink, status);
    } else {
        ok = seq_step(pb, next, P, sink, &W.mnec, status);
        // The first join records the sub-path's first two points (stroke.rs:1624-1627).
        if (ok && count0 == 2) {
            W.firsts[0] = pb.pts[0];
            W.firsts[1] = pb.pts[1];
            W.nfirsts = 2;
        }
    }
    if (!ok) return false;
    if constexpr (SK::kSrc) {
        if (nfirsts0 < 2 && W.nfirsts == 2) {
            S.first_src[0] = S.src[0];
            S.first_src[1] = S.src[1];
        }
        if (pb.n > n0) {
            S.src[count0 < 3 ? count0 : start0] = src;  // SeqBuffer::push
        } else {
            S.src[slot_last(pb)] = src;  // SeqBuffer::replace_last (a skipped flattening step)
        }
    }
    return true;
}

// end (stroke.rs:1179-1193) with close (1206-1279), end_with_caps (1322-1378) and the empty cap
// (1282-1316), on the stepper's own points.
template <bool VW, class SK>
__device__ __noinline__ void seq_end(SeqStroker& S, bool close, const StrokeParams& P, SK& sink,
                                     int* status) {
    VwState& W = S.W;
    SeqBuffer& pb = W.pb;
    const uint32_t count = pb.count;
    W.mnec |= close && count == 1;
    if (close && count > 2) {
        DEP p = W.firsts[0];
        const float start_adv = p.adv;
        p.adv = __int_as_float(0x7fc00000);
        const lyon_vertex_source s0 = S.first_src[0], s1 = S.first_src[1];
        if (!seq_step_any<VW>(S, p, s0, P, sink, status)) pb.last().pos = p.pos;
        if (W.nfirsts >= 2) {
            seq_step_any<VW>(S, W.firsts[1], s1, P, sink, status);
            DEP& p0 = pb.second_last();
            DEP& p1 = pb.last();
            sink.adv = start_adv;
            set_src(sink, S.src[slot_second_last(pb)]);
            for (int side = 0; side < 2; ++side) {
                const V2 sp = p0.s[side].has_single ? p0.s[side].single : p0.s[side].next;
                const V2 normal = (sp - p0.pos) / p0.hw;
                p0.s[side].next_vertex = sink.vertex(p0.pos + normal * p0.hw, normal, side);
            }
            add_edge_triangles(p0, p1, sink);
        }
    } else if (W.mnec && count == 1) {
        const DEP& point = pb.first();
        sink.adv = point.adv;
        set_src(sink, S.src[pb.start % 3]);
        if (P.start_cap == LYON_CAP_SQUARE) {
            tessellate_empty_square_cap(point.pos, point.hw, sink);
        } else if (P.start_cap == LYON_CAP_ROUND) {
            tessellate_empty_round_cap(point.pos, point.hw, P, sink, status);
        }
    } else if (count >= 2) {
        DEP p0 = pb.second_last();
        DEP p1 = pb.last();
        if (!VW) {
            // With a fixed width only the joins have side points so far (stroke.rs:1338-1346).
            const V2 tan = normalize(p1.pos - p0.pos);
            const V2 n = V2{-tan.y, tan.x} * p1.hw;
            p1.s[SP].prev = p1.pos + n;
            p1.s[SN].prev = p1.pos - n;
        }
        // tessellate_last_edge sets the last point's advancement (stroke.rs:2140), which the
        // next sub-path starts from.
        p1.adv = p0.adv + vlength(p1.pos - p0.pos);
        set_src(sink, S.src[slot_last(pb)]);
        tessellate_last_edge(p0, p1, count == 2, P, sink, status);
        W.start_adv = p1.adv;
        lyon_vertex_source fs = S.src[slot_second_last(pb)];
        if (count > 2) {
            p0 = W.firsts[0];
            p1 = W.firsts[1];
            fs = S.first_src[0];
        }
        set_src(sink, fs);
        tessellate_first_edge(p0, p1, P, sink, status);
    }
    pb.start = pb.count = pb.n = 0;
    W.nfirsts = 0;
}

// A flattened run of a curve: lyon's for_each_flattened_with_t loop (quadratic_bezier.rs:891-938,
// cubic_bezier.rs:1318-1363: t advances by 1/n, the last point is the end point at t = 1), with
// the curve parameter mapped to the whole curve as flatten_quad does for a split quadratic
// (stroke.rs:2755-2779: t = tadd + t_run * tmul). That t gives the point's source and, with a
// variable width, its half width (linear in t between the endpoints' widths, stroke.rs:1022,
// 1060).
template <bool VW, class SK>
__device__ __noinline__ void seq_flatten(SeqStroker& S, const Poly& poly, V2 to, float n,
                                         float tmul, float tadd, float sw, float ew,
                                         uint32_t from_id, uint32_t to_id, const StrokeParams& P,
                                         SK& sink, int* status) {
    const float step = 1.0f / n;
    const uint32_t count = to_u32_or1(n) - 1;
    float t0 = 0.0f;
    for (uint32_t i = 0; i <= count; ++i) {
        const bool last = i == count;
        const float t1 = last ? 1.0f : t0 + step;
        const V2 q = last ? to : poly_sample(poly, t1);
        const float t = tadd + t1 * tmul;
        DEP d;
        dep_init(d, q, VW ? (sw * (1.0f - t) + ew * t) * 0.5f : P.hw, P.line_join, t1 != 1.0f);
        seq_step_any<VW>(S, d, curve_src(from_id, to_id, t), P, sink, status);
        t0 = t1;
    }
}

// One thread strokes one path (tessellate_with_ids_fw / _vw, stroke.rs:654-870). With a variable
// width an endpoint's half width is line_width x its factor x 0.5. Endpoint ids are the points'
// indices in the batch. Verbs are checked as they come (a Begin inside a sub-path, a sub-path
// without Begin, missing points or an unknown verb fail the path with
// LYON_ERR_INVALID_ARGUMENT).
template <bool EMIT, bool VW, class SK>
__device__ __noinline__ void stroke_path_sequential(const StrokeArgs& A, uint32_t path) {
    const PathOut po = path_out<EMIT, SK::kRec>(A, path);
    const uint32_t v_begin = A.verb_offsets[path], v_end = A.verb_offsets[path + 1];
    const uint32_t p_end = A.point_offsets[path + 1];
    const lyon_stroke_options opt = A.options[A.num_options > 1 ? path : 0];
    const StrokeParams P = make_params(opt);
    const float lw = opt.line_width;
    const size_t ws = A.width_stride ? A.width_stride : 1u;
    SK s;
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
    s.adv = 0.0f;
    if (EMIT) set_sout(s, A.sources + A.vtx_offsets[path]);
    set_src(s, endpoint_src(LYON_NO_ENDPOINT));
    SeqStroker S;
    S.W.pb.start = S.W.pb.count = S.W.pb.n = 0;
    S.W.nfirsts = 0;
    S.W.mnec = false;
    S.W.start_adv = 0.0f;
    int status = LYON_OK;
    bool open = false;
    V2 cur = V2{0.0f, 0.0f};
    float cur_w = 1.0f;
    uint32_t cur_id = 0;
    uint32_t pc = A.point_offsets[path];
    for (uint32_t vi = v_begin; vi < v_end && status == LYON_OK; ++vi) {
        const int k = A.verbs[vi];
        if (k > LYON_VERB_END || pc + points_of_verb(k) > p_end ||
            (k == LYON_VERB_BEGIN) == open) {
            status = LYON_ERR_INVALID_ARGUMENT;
            break;
        }
        if (k == LYON_VERB_BEGIN || k == LYON_VERB_LINE_TO) {
            cur = load_pt(A.points, pc);
            if (VW) cur_w = A.widths[pc * ws];
            cur_id = pc;
            ++pc;
            DEP d;
            dep_init(d, cur, VW ? lw * cur_w * 0.5f : P.hw, P.line_join, false);
            if (k == LYON_VERB_BEGIN) {
                open = true;
                S.W.mnec = false;
                d.adv = S.W.start_adv;
            }
            seq_step_any<VW>(S, d, endpoint_src(cur_id), P, s, &status);
        } else if (k == LYON_VERB_QUADRATIC_TO) {
            const V2 ctrl = load_pt(A.points, pc);
            const V2 to = load_pt(A.points, pc + 1);
            const uint32_t to_id = pc + 1;
            const float w1 = VW ? A.widths[(pc + 1) * ws] : 1.0f;
            pc += 2;
            const float sw = lw * cur_w, ew = lw * w1;
            float ts;
            if (find_sharp_turn(cur, ctrl, to, &ts)) {
                const V2 sp = quad_sample(cur, ctrl, to, ts);
                const V2 bc = lerp(cur, ctrl, ts);
                const V2 ac = lerp(ctrl, to, ts);
                seq_flatten<VW>(S, quad_poly(cur, bc, sp), sp, quad_wang(cur, bc, sp, P.tolerance),
                                ts, 0.0f, sw, ew, cur_id, to_id, P, s, &status);
                seq_flatten<VW>(S, quad_poly(sp, ac, to), to, quad_wang(sp, ac, to, P.tolerance),
                                1.0f - ts, ts, sw, ew, cur_id, to_id, P, s, &status);
            } else {
                seq_flatten<VW>(S, quad_poly(cur, ctrl, to), to,
                                quad_wang(cur, ctrl, to, P.tolerance), 1.0f, 0.0f, sw, ew, cur_id,
                                to_id, P, s, &status);
            }
            cur = to;
            cur_w = w1;
            cur_id = to_id;
        } else if (k == LYON_VERB_CUBIC_TO) {
            const V2 c1 = load_pt(A.points, pc);
            const V2 c2 = load_pt(A.points, pc + 1);
            const V2 to = load_pt(A.points, pc + 2);
            const uint32_t to_id = pc + 2;
            const float w1 = VW ? A.widths[(pc + 2) * ws] : 1.0f;
            pc += 3;
            seq_flatten<VW>(S, cubic_poly(cur, c1, c2, to), to,
                            cubic_wang(cur, c1, c2, to, P.tolerance), 1.0f, 0.0f, lw * cur_w,
                            lw * w1, cur_id, to_id, P, s, &status);
            cur = to;
            cur_w = w1;
            cur_id = to_id;
        } else {  // Close or End
            if (k == LYON_VERB_CLOSE) ++pc;
            seq_end<VW>(S, k == LYON_VERB_CLOSE, P, s, &status);
            open = false;
        }
    }
    if (s.overflow && status == LYON_OK) status = LYON_ERR_INTERNAL;
    finish_path<EMIT>(A, path, s.nv, s.ni, status, po);
}

// 32 paths per warp, one per lane, from the launch's work counter.
template <bool EMIT, bool VW, class SK>
__global__ void __launch_bounds__(256) stroke_seq_kernel(StrokeArgs A) {
    const int lane = threadIdx.x & 31;
    for (;;) {
        uint32_t first = 0;
        if (lane == 0) first = atomicAdd(A.work_counter, 32u);
        first = __shfl_sync(FULL, first, 0);
        if (first >= A.num_paths) break;
        const uint32_t path = first + (uint32_t)lane;
        if (path < A.num_paths && (!EMIT || A.status[path] == LYON_OK))
            stroke_path_sequential<EMIT, VW, SK>(A, path);
        __syncwarp();
    }
}

template <bool VW>
void launch_seq(const StrokeArgs& a, bool emit, int grid, cudaStream_t s) {
    if (!emit) {
        stroke_seq_kernel<false, VW, Sink><<<grid, 256, 0, s>>>(a);
    } else if (a.sources && a.vertex_attrs) {
        stroke_seq_kernel<true, VW, SrcSinkT<true>><<<grid, 256, 0, s>>>(a);
    } else if (a.sources) {
        stroke_seq_kernel<true, VW, SrcSinkT<false>><<<grid, 256, 0, s>>>(a);
    } else if (a.vertex_attrs) {
        stroke_seq_kernel<true, VW, RecSink><<<grid, 256, 0, s>>>(a);
    } else {
        stroke_seq_kernel<true, VW, Sink><<<grid, 256, 0, s>>>(a);
    }
}

}  // namespace

cudaError_t launch_stroke_seq(const StrokeArgs& args, bool emit, int grid, cudaStream_t stream) {
    if (args.widths) {
        launch_seq<true>(args, emit, grid, stream);
    } else {
        launch_seq<false>(args, emit, grid, stream);
    }
    note_launches(1);
    return cudaGetLastError();
}

}  // namespace lg
