// fill_sweep.cuh — the per-path sweep of the fill tessellator (see fill.cu for the batching).
// The Filler runs one path from event-queue construction to the last span flush; it compiles for
// the device (one thread per path) and, for tests and profiling, for the host.
#pragma once

#include "fill_core.cuh"

namespace lg {
namespace fillk {

// The monotone tessellator's two large routines are called from several places; out of line on
// the device they exist once in the instruction cache (measured: 11 % faster than inlined).
#ifdef __CUDA_ARCH__
#define LG_FILL_SHARED_FN __noinline__
#else
#define LG_FILL_SHARED_FN
#endif

// SRC: the fill also records every vertex's sources (an instantiation of its own, so that plain
// fills carry none of that work).
template <bool SRC>
struct FillerT {
    static constexpr bool want_sources = SRC;
    Heap h;
    int err;  // 0, a LYON_ERR_* code, or FILL_ERR_HEAP
    // output in the heap (path-relative ids)
    Vec<V2> out_v;
    Vec<uint32_t> out_i;
    // With want_sources: every vertex's sources (FillVertex::sources), three words each with
    // path-local endpoint ids, and each vertex's first source.
    Vec<uint32_t> out_src;
    Vec<uint32_t> out_sfirst;
    // event queue
    Vec<Event> events;
    Vec<EdgeData> edge_data;
    // With want_sources: the endpoint ids (path-local) of each event's source edge, two words per
    // event, beside edge_data so that plain fills carry none of it.
    Vec<uint32_t> edge_ids;
    uint32_t first;
    // sweep
    V2 current_position;
    uint32_t current_vertex;
    uint32_t current_event_id;
    Vec<ActiveEdge> active;
    Vec<PendingEdge> edges_below;
    Vec<Span> spans;
    int fill_rule, orientation;
    float tolerance;
    bool assume_no_intersection;
    // active edge scan (fill.rs:115-151)
    Vec<VertexEvent> sc_vertex_events;
    Vec<uint32_t> sc_edges_to_split;
    Vec<int32_t> sc_spans_to_end;
    bool sc_merge_event, sc_split_event, sc_merge_split_event;
    uint32_t sc_above_start, sc_above_end;
    WindingState sc_winding_before_point;

    __host__ __device__ __forceinline__ void fail(int code) {
        if (err == 0) err = code;
    }
    __host__ __device__ __forceinline__ bool ok() {
        if (h.oom && err == 0) err = FILL_ERR_HEAP;
        return err == 0;
    }

    // ---- output ----
    __host__ __device__ __forceinline__ uint32_t add_vertex(V2 p) {
        uint32_t id = out_v.n;
        out_v.push(h, p);
        return id;
    }
    __host__ __device__ __forceinline__ void add_triangle(uint32_t a, uint32_t b, uint32_t c) {
        if (out_i.reserve(h, out_i.n + 3)) {
            uint32_t* d = out_i.p(h) + out_i.n;
            d[0] = a;
            d[1] = b;
            d[2] = c;
            out_i.n += 3;
        }
    }

    // ---- event queue (event_queue.rs) ----
    __host__ __device__ void push_event(V2 pos, const EdgeData& d, uint32_t from_id,
                                        uint32_t to_id) {
        events.push(h, Event{NONE, NONE, pos});
        edge_data.push(h, d);
        if (SRC && edge_ids.reserve(h, edge_ids.n + 2)) {
            uint32_t* w = edge_ids.p(h) + edge_ids.n;
            w[0] = from_id;
            w[1] = to_id;
            edge_ids.n += 2;
        }
    }
    __host__ __device__ __forceinline__ EdgeData no_edge(float t) {
        return EdgeData{V2{u2f(0x7fc00000u), u2f(0x7fc00000u)}, t, t, 0, 0u};
    }
    // The endpoint ids of event `e`'s source edge (want_sources only).
    __host__ __device__ __forceinline__ uint32_t from_id_of(uint32_t e) {
        return SRC ? edge_ids.at(h, 2 * e) : LYON_NO_ENDPOINT;
    }
    __host__ __device__ __forceinline__ uint32_t to_id_of(uint32_t e) {
        return SRC ? edge_ids.at(h, 2 * e + 1) : LYON_NO_ENDPOINT;
    }
    // event_queue.rs:252-274
    __host__ __device__ void insert_into_sorted_list(uint32_t idx, V2 position, uint32_t after) {
        Event* ev = events.p(h);
        uint32_t prev = after, current = after;
        while (current != NONE) {
            V2 pos = ev[current].pos;
            if (peq(pos, position)) {
                ev[idx].next_sibling = ev[current].next_sibling;
                ev[current].next_sibling = idx;
                return;
            } else if (is_after(pos, position)) {
                ev[prev].next_event = idx;
                ev[idx].next_event = current;
                return;
            }
            prev = current;
            current = ev[current].next_event;
        }
        ev[prev].next_event = idx;
    }
    // event_queue.rs:188-213
    __host__ __device__ uint32_t insert_sorted(V2 position, const EdgeData& data, uint32_t after,
                                               uint32_t from_id, uint32_t to_id) {
        uint32_t idx = events.n;
        push_event(position, data, from_id, to_id);
        if (!ok()) return idx;
        insert_into_sorted_list(idx, position, after);
        return idx;
    }
    // event_queue.rs:215-230
    __host__ __device__ void insert_sibling(uint32_t sibling, V2 position, const EdgeData& data,
                                            uint32_t from_id, uint32_t to_id) {
        uint32_t idx = events.n;
        push_event(position, data, from_id, to_id);
        if (!ok()) return;
        Event* ev = events.p(h);
        ev[idx].next_sibling = ev[sibling].next_sibling;
        ev[sibling].next_sibling = idx;
    }
    // event_queue.rs:232-250
    __host__ __device__ void vertex_event_sorted(V2 position, uint32_t endpoint_id,
                                                 uint32_t after) {
        uint32_t idx = events.n;
        push_event(position, no_edge(0.0f), endpoint_id, endpoint_id);
        if (!ok()) return;
        insert_into_sorted_list(idx, position, after);
    }
    // event_queue.rs:328-384
    __host__ __device__ uint32_t merge(uint32_t a, uint32_t b) {
        if (a == NONE) return b;
        if (b == NONE) return a;
        Event* ev = events.p(h);
        bool first_node = true;
        uint32_t sorted_head = NONE, prev = NONE;
        for (;;) {
            if (a == NONE) {
                if (!first_node) ev[prev].next_event = b;
                break;
            }
            if (b == NONE) {
                if (!first_node) ev[prev].next_event = a;
                break;
            }
            uint32_t node;
            int c = compare_positions(ev[a].pos, ev[b].pos);
            if (c < 0) {
                node = a;
                a = ev[a].next_event;
            } else if (c > 0) {
                node = b;
                b = ev[b].next_event;
            } else {
                uint32_t s = a;  // find_last_sibling (event_queue.rs:386-395)
                while (ev[s].next_sibling != NONE) s = ev[s].next_sibling;
                ev[s].next_sibling = b;
                b = ev[b].next_event;
                continue;
            }
            if (first_node) {
                first_node = false;
                sorted_head = node;
            } else {
                ev[prev].next_event = node;
            }
            prev = node;
        }
        if (sorted_head == NONE) sorted_head = a;
        return sorted_head;
    }
    // event_queue.rs:301-326: the recursive top-down merge sort, with an explicit stack.
    __host__ __device__ void sort_events() {
        first = NONE;
        if (events.n == 0) return;
        struct Frame {
            uint32_t s, e, stage, a;
        };
        Frame stk[40];
        int sp = 0;
        uint32_t ret = 0;
        stk[sp++] = Frame{0, events.n, 0, 0};
        while (sp > 0) {
            Frame& f = stk[sp - 1];
            const uint32_t split = (f.s + f.e) / 2;
            if (f.stage == 0) {
                if (split == f.s) {
                    ret = f.s;
                    --sp;
                    continue;
                }
                f.stage = 1;
                stk[sp++] = Frame{f.s, split, 0, 0};
            } else if (f.stage == 1) {
                f.a = ret;
                f.stage = 2;
                stk[sp++] = Frame{split, f.e, 0, 0};
            } else {
                ret = merge(f.a, ret);
                --sp;
            }
        }
        first = ret;
    }

    // ---- monotone tessellators (monotone.rs) ----
    __host__ __device__ void span_init(Span& s) {
        s.stack.init();
        s.triangles.init();
        s.left.events.init();
        s.right.events.init();
        s.alive = 1;
    }
    __host__ __device__ void side_push(SideEvents& side, MV v) {  // monotone.rs:202-209
        side.events.push(h, v.id);
        side.prev = side.last.pos;
        side.last = v;
    }
    __host__ __device__ void tri_ids(Span& s, uint32_t a, uint32_t b, uint32_t c) {
        if (s.triangles.reserve(h, s.triangles.n + 3)) {
            uint32_t* d = s.triangles.p(h) + s.triangles.n;
            d[0] = a;
            d[1] = b;
            d[2] = c;
            s.triangles.n += 3;
        }
    }
    // monotone.rs:9-139 (BasicMonotoneTessellator)
    __host__ __device__ void basic_begin(Span& s, V2 pos, uint32_t id) {
        MV first_v{pos, id, LEFT};
        s.previous = first_v;
        s.triangles.clear();
        s.stack.clear();
        s.stack.push(h, first_v);
    }
    __host__ __device__ LG_FILL_SHARED_FN void monotone_vertex(Span& s, MV current) {
        const bool changed_side = current.side != s.previous.side;
        if (changed_side) {
            for (uint32_t i = 0; i + 1 < s.stack.n; ++i) {
                MV a = s.stack.at(h, i), b = s.stack.at(h, i + 1);
                bool winding = cross(a.pos - b.pos, current.pos - b.pos) >= 0.0f;
                if (!winding) {
                    MV t = a;
                    a = b;
                    b = t;
                }
                tri_ids(s, a.id, b.id, current.id);
            }
            s.stack.clear();
            s.stack.push(h, s.previous);
        } else {
            bool have_last = s.stack.n > 0;
            MV last_popped{V2{0.0f, 0.0f}, 0, LEFT};
            if (have_last) last_popped = s.stack.at(h, --s.stack.n);
            while (s.stack.n > 0) {
                MV a = last_popped;
                MV b = s.stack.at(h, s.stack.n - 1);
                if (current.side == RIGHT) {
                    MV t = a;
                    a = b;
                    b = t;
                }
                float c = cross(current.pos - b.pos, a.pos - b.pos);
                if (c >= 0.0f) {
                    tri_ids(s, b.id, a.id, current.id);
                    have_last = s.stack.n > 0;
                    if (have_last) last_popped = s.stack.at(h, --s.stack.n);
                } else {
                    break;
                }
            }
            if (have_last) s.stack.push(h, last_popped);
        }
        s.stack.push(h, current);
        s.previous = current;
    }
    __host__ __device__ void basic_end(Span& s, V2 pos, uint32_t id) {
        int side = s.previous.side == LEFT ? RIGHT : LEFT;
        monotone_vertex(s, MV{pos, id, side});
        s.stack.clear();
    }
    __host__ __device__ void flush_triangles(Span& s) {
        const uint32_t* t = s.triangles.p(h);
        for (uint32_t i = 0; i + 2 < s.triangles.n; i += 3)
            add_triangle(t[i], t[i + 1], t[i + 2]);
        s.triangles.clear();
    }
    // monotone.rs:362-404
    __host__ __device__ LG_FILL_SHARED_FN bool flush_side(Span& s, SideEvents& side, int sd,
                                                          MV* out) {
        const uint32_t len = side.events.n;
        if (len < 2) return false;
        uint32_t step = 1;
        while (step * 2 < len) {
            uint32_t last_index = 0;
            const uint32_t imax = (len - 1) / (2 * step);
            for (uint32_t i = 0; i < imax; ++i) {
                uint32_t a = i * 2 * step;
                uint32_t b = a + step;
                last_index = b + step;
                if (sd == RIGHT) {
                    uint32_t t = a;
                    a = b;
                    b = t;
                }
                const uint32_t* ev = side.events.p(h);
                tri_ids(s, ev[a], ev[b], ev[last_index]);
            }
            if (last_index + step < len) {
                uint32_t b = last_index;
                uint32_t c = last_index + step;
                if (sd == RIGHT) {
                    uint32_t t = b;
                    b = c;
                    c = t;
                }
                const uint32_t* ev = side.events.p(h);
                tri_ids(s, ev[0], ev[b], ev[c]);
            }
            step *= 2;
        }
        side.events.clear();
        side_push(side, side.last);
        side.reference_point = side.last.pos;
        *out = side.last;
        return true;
    }
    // monotone.rs:212-359 (AdvancedMonotoneTessellator)
    __host__ __device__ void adv_begin(Span& s, V2 pos, uint32_t id) {
        basic_begin(s, pos, id);
        s.left.reference_point = pos;
        s.left.conservative_reference_x = pos.x;
        s.right.reference_point = pos;
        s.right.conservative_reference_x = pos.x;
        s.left.prev = pos;
        s.right.prev = pos;
        s.left.last = MV{V2{0.0f, 0.0f}, 0, LEFT};
        s.right.last = MV{V2{0.0f, 0.0f}, 0, LEFT};
        s.left.events.clear();
        s.right.events.clear();
        side_push(s.left, MV{pos, id, LEFT});
        side_push(s.right, MV{pos, id, RIGHT});
    }
    __host__ __device__ void adv_vertex(Span& s, V2 pos, uint32_t id, int side) {
        if (side == LEFT) {
            s.left.reference_point.x = fmaxf(s.left.reference_point.x, pos.x);
            s.left.conservative_reference_x =
                fmaxf(s.left.conservative_reference_x, s.left.reference_point.x);
        } else {
            s.right.reference_point.x = fminf(s.right.reference_point.x, pos.x);
            s.right.conservative_reference_x =
                fminf(s.right.conservative_reference_x, s.right.reference_point.x);
        }
        const float dx = s.right.conservative_reference_x - s.left.conservative_reference_x;
        SideEvents& side_ev = side == LEFT ? s.left : s.right;
        SideEvents& opp = side == LEFT ? s.right : s.left;
        const float dy = pos.y - side_ev.reference_point.y;
        const bool sides_are_close = dx < dy * 0.1f;
        const uint32_t len = side_ev.events.n;
        bool outward_turn = false;
        if (!sides_are_close && len >= 2) {
            const float sign = side == LEFT ? 1.0f : -1.0f;
            outward_turn = cross(side_ev.prev - side_ev.last.pos, pos - side_ev.last.pos) * sign <
                           0.0f;
        }
        if (outward_turn || sides_are_close) {
            const bool must_flush_opposite_side = is_after(side_ev.last.pos, opp.last.pos);
            MV v;
            if (must_flush_opposite_side) {
                if (flush_side(s, opp, side == LEFT ? RIGHT : LEFT, &v)) {
                    monotone_vertex(s, v);
                    side_ev.conservative_reference_x = side_ev.reference_point.x;
                }
            }
            if (flush_side(s, side_ev, side, &v)) {
                monotone_vertex(s, v);
                opp.conservative_reference_x = opp.reference_point.x;
            }
        }
        side_push(side_ev, MV{pos, id, side});
    }
    __host__ __device__ void adv_end(Span& s, V2 pos, uint32_t id) {
        MV a, b;
        const bool ha = flush_side(s, s.left, LEFT, &a);
        const bool hb = flush_side(s, s.right, RIGHT, &b);
        if (ha && !hb) {
            monotone_vertex(s, a);
        } else if (!ha && hb) {
            monotone_vertex(s, b);
        } else if (ha && hb) {
            MV v1 = a, v2 = b;
            if (is_after(v1.pos, v2.pos)) {
                MV t = v1;
                v1 = v2;
                v2 = t;
            }
            monotone_vertex(s, v1);
            monotone_vertex(s, v2);
        }
        basic_end(s, pos, id);
    }

    // ---- spans (fill.rs:203-294) ----
    __host__ __device__ void begin_span(int32_t idx, V2 position, uint32_t vertex) {
        if (idx < 0 || (uint32_t)idx > spans.n) {
            fail(LYON_ERR_INTERNAL);
            return;
        }
        Span s;
        span_init(s);
        adv_begin(s, position, vertex);
        if (!ok()) return;
        spans.insert(h, (uint32_t)idx, s);
    }
    __host__ __device__ Span* span_tess(int32_t idx) {
        if (idx < 0 || (uint32_t)idx >= spans.n || !spans.at(h, (uint32_t)idx).alive) {
            fail(LYON_ERR_INTERNAL);
            return nullptr;
        }
        return &spans.at(h, (uint32_t)idx);
    }
    __host__ __device__ void end_span(int32_t idx, V2 position, uint32_t id) {  // fill.rs:235-254
        Span* s = span_tess(idx);
        if (!s) return;
        adv_end(*s, position, id);
        flush_triangles(*s);
        s->alive = 0;
        free_span(*s);
    }
    __host__ __device__ void free_span(Span& s) {
        s.stack.release(h);
        s.triangles.release(h);
        s.left.events.release(h);
        s.right.events.release(h);
    }
    __host__ __device__ void cleanup_spans() {  // fill.rs:291-294
        Span* d = spans.p(h);
        uint32_t w = 0;
        for (uint32_t r = 0; r < spans.n; ++r) {
            if (d[r].alive) {
                if (w != r) d[w] = d[r];
                ++w;
            }
        }
        spans.n = w;
    }

    // ---- active edge scan (fill.rs:1045-1378) ----
    __host__ __device__ int check_remaining_edges(uint32_t idx, float current_x) {  // fill.rs:1295-1324
        const ActiveEdge* a = active.p(h);
        for (uint32_t i = idx; i < active.n; ++i) {
            const ActiveEdge& e = a[i];
            if (e.is_merge) continue;
            if (e.max_x() < current_x) return 1;
            if (peq(current_position, e.to)) return 2;
            if (e.min_x() < current_x && e.solve_x_for_y(current_position.y) < current_x) return 3;
        }
        return 0;
    }
    // fill.rs:1328-1378: -1 error (*code set), 0 not connecting, 1 connecting
    __host__ __device__ int is_edge_connecting(const ActiveEdge& e, uint32_t idx, int* code) {
        if (peq(current_position, e.to)) return 1;
        const float current_x = current_position.x;
        const float threshold = tolerance;
        const float min_x = e.min_x(), max_x = e.max_x();
        if (max_x + threshold < current_x || e.to.y < current_position.y) {
            *code = 4;
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
            sc_edges_to_split.push(h, idx);
            return 1;
        }
        if (ex < current_x) {
            *code = 5;
            return -1;
        }
        return 0;
    }
    __host__ __device__ int scan_active_edges() {  // fill.rs:1045-1291
        sc_vertex_events.clear();
        sc_edges_to_split.clear();
        sc_spans_to_end.clear();
        sc_merge_event = sc_split_event = sc_merge_split_event = false;
        sc_above_start = sc_above_end = 0;
        sc_winding_before_point.reset();
        const float current_x = current_position.x;
        bool connecting_edges = false;
        uint32_t idx = 0;
        WindingState winding;
        winding.reset();
        bool previous_was_merge = false;
        for (uint32_t i = 0; i < active.n; ++i) {
            const ActiveEdge e = active.at(h, i);
            if (e.is_merge) {
                winding.span_index += 1;
                idx += 1;
                previous_was_merge = true;
                continue;
            }
            bool before;
            if (peq(current_position, e.to)) {
                connecting_edges = true;
                before = false;
            } else if (e.max_x() < current_x) {
                before = true;
            } else if (e.min_x() > current_x) {
                before = false;
            } else if (e.from.y == e.to.y) {
                connecting_edges = true;
                before = false;
            } else {
                float ex = e.solve_x_for_y(current_position.y);
                if (fabsf(ex - current_x) <= tolerance) {
                    connecting_edges = true;
                    before = false;
                } else {
                    before = !(ex > current_x);
                }
            }
            if (!before) break;
            winding.update(fill_rule, w16(e.winding));
            previous_was_merge = false;
            idx += 1;
        }
        sc_above_start = idx;
        sc_winding_before_point = winding;
        if (previous_was_merge) {
            sc_winding_before_point.span_index -= 1;
            sc_above_start -= 1;
            if (!connecting_edges) {
                sc_vertex_events.push(h, VertexEvent{winding.span_index - 1, RIGHT});
                sc_vertex_events.push(h, VertexEvent{winding.span_index, LEFT});
                sc_merge_split_event = true;
            }
        }
        sc_split_event = !connecting_edges && winding.is_in && !sc_merge_split_event;
        if (connecting_edges) {
            const bool in_before_vertex = winding.is_in;
            bool first_connecting_edge = !previous_was_merge;
            for (uint32_t i = idx; i < active.n; ++i) {
                const ActiveEdge e = active.at(h, i);
                if (e.is_merge) {
                    if (!winding.is_in) return 200;  // MergeVertexOutside
                    sc_spans_to_end.push(h, winding.span_index);
                    winding.span_index += 1;
                    idx += 1;
                    first_connecting_edge = false;
                    continue;
                }
                int code = 0;
                int c = is_edge_connecting(e, idx, &code);
                if (c < 0) return code;
                if (c == 0) break;
                if (!first_connecting_edge && winding.is_in) {
                    sc_spans_to_end.push(h, winding.span_index);
                }
                winding.update(fill_rule, w16(e.winding));
                if (winding.is_in && winding.span_index >= (int32_t)spans.n) return 201;
                idx += 1;
                first_connecting_edge = false;
            }
            const bool in_after_vertex = winding.is_in;
            const bool vertex_is_merge_event = in_before_vertex && in_after_vertex &&
                                               edges_below.n == 0 && sc_edges_to_split.n == 0;
            if (vertex_is_merge_event) sc_merge_event = true;
            if (in_before_vertex) {
                sc_vertex_events.push(h, VertexEvent{sc_winding_before_point.span_index, RIGHT});
            }
            if (in_after_vertex) sc_vertex_events.push(h, VertexEvent{winding.span_index, LEFT});
        }
        sc_above_end = idx;
        return check_remaining_edges(idx, current_x);
    }

    // ---- events above / below the current point (fill.rs:1381-1524) ----
    __host__ __device__ void process_edges_above() {
        for (uint32_t i = 0; i < sc_vertex_events.n; ++i) {
            const VertexEvent ve = sc_vertex_events.at(h, i);
            Span* s = span_tess(ve.span);
            if (!s) return;
            adv_vertex(*s, current_position, current_vertex, ve.side);
            if (!ok()) return;
        }
        for (uint32_t i = 0; i < sc_spans_to_end.n; ++i) {
            const int32_t span_index = sc_spans_to_end.at(h, i);
            if (span_index < 0 || (uint32_t)span_index >= spans.n) {
                fail(LYON_ERR_INTERNAL);
                return;
            }
            end_span(span_index, current_position, current_vertex);
            if (!ok()) return;
        }
        cleanup_spans();
        for (uint32_t i = 0; i < sc_edges_to_split.n; ++i) {
            ActiveEdge& e = active.at(h, sc_edges_to_split.at(h, i));
            const V2 to = e.to;
            edges_below.push(h, PendingEdge{to, slope(to - current_position), e.src_edge,
                                            e.winding, e.range_end});
            if (!ok()) return;
            active.at(h, sc_edges_to_split.at(h, i)).to = current_position;
        }
        if (sc_merge_event) {
            ActiveEdge& e = active.at(h, sc_above_start);
            e.is_merge = 1;
            e.from = e.to;
            e.winding = 0;
            e.from_id = current_vertex;
            sc_above_start += 1;
        }
    }
    // fill.rs:2010-2013 (sort_unstable_by on the sort key; insertion order for short slices)
    __host__ __device__ void sort_edges_below() {
        PendingEdge* d = edges_below.p(h);
        for (uint32_t i = 1; i < edges_below.n; ++i) {
            uint32_t j = i;
            while (j > 0 && d[j].sort_key < d[j - 1].sort_key) {
                PendingEdge t = d[j];
                d[j] = d[j - 1];
                d[j - 1] = t;
                --j;
            }
        }
    }
    __host__ __device__ void merge_coincident_edges(uint32_t a_idx, uint32_t b_idx) {  // fill.rs:2050-2106
        PendingEdge* d = edges_below.p(h);
        const V2 a_to = d[a_idx].to, b_to = d[b_idx].to;
        uint32_t lower_idx, upper_idx;
        bool split;
        const int c = compare_positions(a_to, b_to);
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
        d[upper_idx].winding = w16(d[upper_idx].winding + d[lower_idx].winding);
        const V2 split_point = d[upper_idx].to;
        const PendingEdge edge = d[lower_idx];
        edges_below.erase(h, lower_idx);
        if (!split) return;
        const EdgeData src = edge_data.at(h, edge.src_edge);
        const float dy = edge.to.y - current_position.y;
        const float t = dy == 0.0f ? 0.0f : (split_point.y - current_position.y) / dy;
        const float t_remapped = remap_t_in_range(t, src.range_start, edge.range_end);
        insert_sorted(split_point, EdgeData{edge.to, t_remapped, edge.range_end, edge.winding, 1u},
                      current_event_id, from_id_of(edge.src_edge), to_id_of(edge.src_edge));
    }
    __host__ __device__ void handle_coincident_edges_below() {  // fill.rs:2016-2048
        if (edges_below.n < 2) return;
        for (int idx = (int)edges_below.n - 2; idx >= 0; --idx) {
            const uint32_t a_idx = (uint32_t)idx, b_idx = a_idx + 1;
            const float a_slope = edges_below.at(h, a_idx).sort_key;
            const float b_slope = edges_below.at(h, b_idx).sort_key;
            const float THRESHOLD = 0.00005f;
            bool angle_is_close;
            if (fabsf(a_slope) <= 1.0f) {
                angle_is_close = fabsf(a_slope - b_slope) < THRESHOLD;
            } else {
                angle_is_close = fabsf(1.0f / a_slope - 1.0f / b_slope) < THRESHOLD;
            }
            if (angle_is_close) {
                merge_coincident_edges(a_idx, b_idx);
                if (!ok()) return;
            }
        }
    }
    __host__ __device__ void split_event(uint32_t left_idx, int32_t left_span_idx) {  // fill.rs:1563-1608
        const uint32_t right_idx = left_idx + 1;
        if (right_idx >= active.n) {
            fail(LYON_ERR_INTERNAL);
            return;
        }
        const ActiveEdge le = active.at(h, left_idx), re = active.at(h, right_idx);
        const int32_t right_span_idx = left_span_idx + 1;
        V2 upper_position;
        uint32_t upper_id;
        int32_t new_span_idx;
        if (is_after(le.from, re.from)) {
            upper_position = le.from;
            upper_id = le.from_id;
            new_span_idx = left_span_idx;
        } else {
            upper_position = re.from;
            upper_id = re.from_id;
            new_span_idx = right_span_idx;
        }
        begin_span(new_span_idx, upper_position, upper_id);
        if (!ok()) return;
        Span* s = span_tess(left_span_idx);
        if (!s) return;
        adv_vertex(*s, current_position, current_vertex, RIGHT);
        if (!ok()) return;
        s = span_tess(right_span_idx);
        if (!s) return;
        adv_vertex(*s, current_position, current_vertex, LEFT);
    }
    __host__ __device__ void process_edges_below() {  // fill.rs:1455-1524
        WindingState winding = sc_winding_before_point;
        sort_edges_below();
        handle_coincident_edges_below();
        if (!ok()) return;
        if (sc_split_event) {
            if (sc_above_start == 0) {
                fail(LYON_ERR_INTERNAL);
                return;
            }
            split_event(sc_above_start - 1, winding.span_index);
            if (!ok()) return;
        }
        bool first_pending_edge = true;
        for (uint32_t i = 0; i < edges_below.n; ++i) {
            if (!first_pending_edge && winding.is_in) {
                begin_span(winding.span_index, current_position, current_vertex);
                if (!ok()) return;
            }
            winding.update(fill_rule, w16(edges_below.at(h, i).winding));
            first_pending_edge = false;
        }
    }

    // ---- intersections (fill.rs:1611-1846) ----
    __host__ __device__ void process_intersection(double ta, double tb, uint32_t ai, uint32_t bi,
                                         double bfx, double bfy, double btx, double bty) {
        const double one_t = 1.0 - tb;
        V2 ip = V2{(float)(one_t * bfx + tb * btx), (float)(one_t * bfy + tb * bty)};
        if (peq(current_position, ip)) {
            ActiveEdge& ae = active.at(h, ai);
            ae.from = ip;
            EdgeData& src = edge_data.at(h, ae.src_edge);
            src.range_start = remap_t_in_range((float)ta, src.range_start, ae.range_end);
            return;
        }
        if (!is_after(ip, current_position)) ip.y = nextafterf(current_position.y, INFINITY);
        if (!is_after(ip, current_position)) {
            fail(LYON_ERR_INTERNAL);  // lyon asserts here
            return;
        }
        {
            const PendingEdge eb = edges_below.at(h, bi);
            const ActiveEdge ae = active.at(h, ai);
            if (is_near(ip, eb.to)) {
                ip = eb.to;
            } else if (is_near(ip, ae.to)) {
                ip = ae.to;
            }
        }
        const ActiveEdge ae0 = active.at(h, ai);
        const EdgeData a_src = edge_data.at(h, ae0.src_edge);
        const uint32_t b_src_edge = edges_below.at(h, bi).src_edge;
        const EdgeData b_src = edge_data.at(h, b_src_edge);
        const uint32_t a_from = from_id_of(ae0.src_edge), a_to = to_id_of(ae0.src_edge);
        const uint32_t b_from = from_id_of(b_src_edge), b_to = to_id_of(b_src_edge);
        bool has_inserted = false;
        uint32_t inserted_evt = 0;
        bool flipped_active = false;
        if (!peq(ae0.to, ip) && !peq(ae0.from, ip)) {
            const float remapped_ta = remap_t_in_range((float)ta, a_src.range_start, ae0.range_end);
            if (is_after(ae0.to, ip)) {
                inserted_evt = insert_sorted(
                    ip, EdgeData{ae0.to, remapped_ta, ae0.range_end, ae0.winding, 1u},
                    current_event_id, a_from, a_to);
                has_inserted = true;
            } else {
                flipped_active = true;
                insert_sorted(ae0.to,
                              EdgeData{ip, ae0.range_end, remapped_ta, (int32_t)w16(-ae0.winding),
                                       1u},
                              current_event_id, a_from, a_to);
            }
            if (!ok()) return;
            ActiveEdge& ae = active.at(h, ai);
            ae.to = ip;
            ae.range_end = remapped_ta;
        }
        const PendingEdge eb = edges_below.at(h, bi);
        if (!peq(eb.to, ip) && !peq(current_position, ip)) {
            const float remapped_tb = remap_t_in_range((float)tb, b_src.range_start, eb.range_end);
            if (is_after(eb.to, ip)) {
                const EdgeData d{eb.to, remapped_tb, eb.range_end, eb.winding, 1u};
                if (has_inserted) {
                    insert_sibling(inserted_evt, ip, d, b_from, b_to);
                } else {
                    insert_sorted(ip, d, current_event_id, b_from, b_to);
                }
            } else {
                insert_sorted(eb.to,
                              EdgeData{ip, eb.range_end, remapped_tb, (int32_t)w16(-eb.winding), 1u},
                              current_event_id, b_from, b_to);
                if (ok() && flipped_active) vertex_event_sorted(ip, b_to, current_event_id);
            }
            if (!ok()) return;
            PendingEdge& e = edges_below.at(h, bi);
            e.to = ip;
            e.range_end = remapped_tb;
        }
    }
    __host__ __device__ void handle_intersections(uint32_t skip_start, uint32_t skip_end) {
        for (uint32_t bi = 0; bi < edges_below.n; ++bi) {
            const PendingEdge eb = edges_below.at(h, bi);
            const float below_min_x = fminf(current_position.x, eb.to.x);
            const float below_max_x = fmax_lyon(current_position.x, eb.to.x);
            const double bfx = current_position.x, bfy = current_position.y;
            const double btx = eb.to.x, bty = eb.to.y;
            double tb_min = 1.0, fta = 0.0, ftb = 0.0;
            bool found = false;
            uint32_t fidx = 0;
            for (uint32_t i = 0; i < active.n; ++i) {
                if (i >= skip_start && i < skip_end) continue;
                const ActiveEdge ae = active.at(h, i);
                if (ae.is_merge || below_min_x > ae.max_x()) continue;
                if (below_max_x < ae.min_x()) continue;
                if (!may_intersect(ae.from, ae.to, current_position, eb.to)) continue;
                double ta, tb;
                if (segment_intersection_t(ae.from.x, ae.from.y, ae.to.x, ae.to.y, bfx, bfy, btx,
                                           bty, &ta, &tb)) {
                    if (tb < tb_min && tb > 0.0 && ta > 0.0 && ta <= 1.0) {
                        tb_min = tb;
                        found = true;
                        fta = ta;
                        ftb = tb;
                        fidx = i;
                    }
                }
            }
            if (found) {
                process_intersection(fta, ftb, fidx, bi, bfx, bfy, btx, bty);
                if (!ok()) return;
            }
        }
    }
    __host__ __device__ void update_active_edges() {  // fill.rs:1527-1561
        const uint32_t s = sc_above_start, e = sc_above_end;
        if (!assume_no_intersection) {
            handle_intersections(s, e);
            if (!ok()) return;
        }
        const uint32_t nb = edges_below.n;
        const uint32_t old_n = active.n;
        const uint32_t new_n = old_n - (e - s) + nb;
        if (!active.reserve(h, new_n)) {
            ok();
            return;
        }
        ActiveEdge* a = active.p(h);
        if (nb > e - s) {
            for (uint32_t k = old_n; k > e; --k) a[k - 1 + nb - (e - s)] = a[k - 1];
        } else if (nb < e - s) {
            for (uint32_t k = e; k < old_n; ++k) a[k - (e - s) + nb] = a[k];
        }
        const PendingEdge* pb = edges_below.p(h);
        for (uint32_t k = 0; k < nb; ++k) {
            ActiveEdge ne;
            ne.from = current_position;
            ne.to = pb[k].to;
            ne.winding = pb[k].winding;
            ne.is_merge = 0;
            ne.from_id = current_vertex;
            ne.src_edge = pb[k].src_edge;
            ne.range_end = pb[k].range_end;
            ne.pad = 0;
            a[s + k] = ne;
        }
        active.n = new_n;
        edges_below.clear();
    }
    __host__ __device__ int process_events() {  // fill.rs:929-965
        int code = scan_active_edges();
        if (!ok()) return 0;
        if (code) return code;
        process_edges_above();
        if (!ok()) return 0;
        process_edges_below();
        if (!ok()) return 0;
        update_active_edges();
        return 0;
    }

    // ---- error recovery (fill.rs:1848-2007) ----
    __host__ __device__ bool key_less(float ka, uint32_t ia, float kb, uint32_t ib) {
        if (ka < kb) return true;
        if (ka > kb) return false;
        const ActiveEdge& ea = active.at(h, ia);
        const ActiveEdge& eb = active.at(h, ib);
        if (!ea.is_merge && !eb.is_merge) {
            return slope(eb.to - eb.from) < slope(ea.to - ea.from);
        }
        if (ea.is_merge && !eb.is_merge) return false;
        if (!ea.is_merge && eb.is_merge) return true;
        return false;
    }
    __host__ __device__ void sort_active_edges() {
        const float y = current_position.y;
        const uint32_t n = active.n;
        Vec<float> keys;
        Vec<uint32_t> order;
        Vec<ActiveEdge> sorted;
        keys.init();
        order.init();
        sorted.init();
        if (!keys.reserve(h, n) || !order.reserve(h, n) || !sorted.reserve(h, n)) {
            ok();
            return;
        }
        bool has_merge_vertex = false;
        float prev_x = u2f(0x7fc00000u);
        for (uint32_t i = 0; i < n; ++i) {
            const ActiveEdge& e = active.at(h, i);
            float key;
            if (e.is_merge) {
                has_merge_vertex = true;
                key = prev_x;
            } else {
                const bool eq_to = e.to.y == y, eq_from = e.from.y == y;
                float x;
                if (eq_to && eq_from) {
                    const float current_x = current_position.x;
                    x = (e.max_x() >= current_x && e.min_x() <= current_x) ? current_position.x
                                                                            : e.min_x();
                } else if (eq_from) {
                    x = e.from.x;
                } else if (eq_to) {
                    x = e.to.x;
                } else {
                    x = e.solve_x_for_y(y);
                }
                key = fmax_lyon(x, e.min_x());
                prev_x = x;
            }
            keys.p(h)[i] = key;
            order.p(h)[i] = i;
        }
        keys.n = order.n = n;
        if (n > 1) {
            for (uint32_t i = 0; i < n; ++i) {
                const float k = keys.at(h, i);
                if (k != k) {
                    fail(LYON_ERR_INTERNAL);  // lyon unwraps a NaN comparison here
                    return;
                }
            }
        }
        float* K = keys.p(h);
        uint32_t* O = order.p(h);
        for (uint32_t i = 1; i < n; ++i) {  // stable insertion sort (Vec::sort_by is stable)
            uint32_t j = i;
            while (j > 0 && key_less(K[j], O[j], K[j - 1], O[j - 1])) {
                float tk = K[j];
                K[j] = K[j - 1];
                K[j - 1] = tk;
                uint32_t to = O[j];
                O[j] = O[j - 1];
                O[j - 1] = to;
                --j;
            }
        }
        ActiveEdge* S = sorted.p(h);
        for (uint32_t i = 0; i < n; ++i) S[i] = active.at(h, O[i]);
        ActiveEdge* A = active.p(h);
        for (uint32_t i = 0; i < n; ++i) A[i] = S[i];
        sorted.release(h);
        order.release(h);
        keys.release(h);
        if (!has_merge_vertex) return;
        int16_t winding_number = 0;
        for (uint32_t i = 0; i < n; ++i) {
            bool needs_swap;
            if (A[i].is_merge) {
                needs_swap = !fill_rule_is_in(fill_rule, winding_number);
            } else {
                winding_number = w16(winding_number + A[i].winding);
                needs_swap = false;
            }
            if (needs_swap) {
                int16_t w = winding_number;
                uint32_t idx = i;
                while (idx > 0) {
                    w = w16(w - A[idx - 1].winding);
                    ActiveEdge t = A[idx];
                    A[idx] = A[idx - 1];
                    A[idx - 1] = t;
                    if (fill_rule_is_in(fill_rule, w)) break;
                    idx -= 1;
                }
            }
        }
    }
    __host__ __device__ void recover_from_error() {  // fill.rs:1956-2007
        sort_active_edges();
        if (!ok()) return;
        const uint32_t len = active.n;
        if (len > 1 && active.at(h, len - 1).is_merge) {
            ActiveEdge t = active.at(h, len - 1);
            active.at(h, len - 1) = active.at(h, len - 2);
            active.at(h, len - 2) = t;
        }
        WindingState winding;
        winding.reset();
        for (uint32_t i = 0; i < active.n; ++i) {
            const ActiveEdge e = active.at(h, i);
            if (e.is_merge) {
                winding.span_index += 1;
            } else {
                winding.update(fill_rule, w16(e.winding));
            }
            if (winding.span_index >= (int32_t)spans.n) {
                begin_span(winding.span_index, e.from, e.from_id);
                if (!ok()) return;
            }
        }
        while ((int64_t)spans.n > (int64_t)winding.span_index + 1) {
            Span& s = spans.at(h, spans.n - 1);
            if (!s.alive) {
                fail(LYON_ERR_INTERNAL);
                return;
            }
            flush_triangles(s);
            free_span(s);
            spans.n -= 1;
        }
    }

    // VertexSourceIterator (fill.rs:2294-2337): every sibling event at the vertex gives its
    // edge's endpoint (t = 0 or 1) or the point at t on it; a source equal to the previous one is
    // skipped.
    __host__ __device__ void record_sources(uint32_t ev) {
        out_sfirst.push(h, out_src.n / 3);
        uint32_t pf = 0, pt = 0;
        float ptt = 0.0f;
        bool have_prev = false;
        for (uint32_t id = ev; id != NONE; id = events.at(h, id).next_sibling) {
            const float t = edge_data.at(h, id).range_start;
            const uint32_t e_from = edge_ids.at(h, 2 * id), e_to = edge_ids.at(h, 2 * id + 1);
            uint32_t f = e_from, to = LYON_NO_ENDPOINT;
            float tt = 0.0f;
            if (t == 1.0f) {
                f = e_to;
            } else if (t != 0.0f) {
                to = e_to;
                tt = t;
            }
            if (have_prev && f == pf && to == pt && (to == LYON_NO_ENDPOINT || tt == ptt)) continue;
            if (!out_src.reserve(h, out_src.n + 3)) return;
            uint32_t* d = out_src.p(h) + out_src.n;
            d[0] = f;
            d[1] = to;
            d[2] = f2u(tt);
            out_src.n += 3;
            pf = f;
            pt = to;
            ptt = tt;
            have_prev = true;
        }
    }

    // ---- main loop (fill.rs:749-925) ----
    __host__ __device__ void initialize_events() {
        const uint32_t ce = current_event_id;
        current_position = events.at(h, ce).pos;
        if (current_position.x != current_position.x || current_position.y != current_position.y) {
            fail(LYON_ERR_POSITION_IS_NAN);
            return;
        }
        const V2 position = orientation == LYON_ORIENTATION_VERTICAL
                                ? current_position
                                : V2{current_position.y, -current_position.x};
        current_vertex = add_vertex(position);
        if constexpr (SRC) record_sources(ce);
        uint32_t sib = ce;
        while (sib != NONE) {
            const EdgeData edge = edge_data.at(h, sib);
            if (edge.is_edge) {
                edges_below.push(h, PendingEdge{edge.to, slope(edge.to - current_position), sib,
                                                edge.winding, edge.range_end});
            }
            sib = events.at(h, sib).next_sibling;
        }
        ok();
    }
    __host__ __device__ void tessellator_loop() {  // fill.rs:836-867
        current_event_id = first;
        while (current_event_id != NONE) {
            initialize_events();
            if (!ok()) return;
            int code = process_events();
            if (!ok()) return;
            if (code) {
                recover_from_error();
                if (!ok()) return;
                code = process_events();
                if (!ok()) return;
                if (code) {
                    fail(LYON_ERR_INTERNAL);
                    return;
                }
            }
            current_event_id = events.at(h, current_event_id).next_event;
        }
    }

    // ---- event queue construction (event_queue.rs:441-905) ----
    struct Builder {
        V2 current, prev, second;
        uint32_t nth;
        uint32_t prev_id;  // prev_endpoint_id
        float tolerance;
    };
    __host__ __device__ void eq_vertex_event(V2 at, uint32_t id) {
        push_event(at, no_edge(0.0f), id, id);
    }
    __host__ __device__ void eq_vertex_event_on_curve(V2 at, float t, uint32_t from_id,
                                                      uint32_t to_id) {
        push_event(at, no_edge(t), from_id, to_id);
    }
    __host__ __device__ void eq_add_edge(Builder& b, V2 from, V2 to, int16_t winding, float t0,
                                         float t1, uint32_t from_id, uint32_t to_id) {
        if (peq(from, to)) return;
        V2 evt_pos = from, evt_to = to;
        if (is_after(evt_pos, to)) {
            evt_to = evt_pos;
            evt_pos = to;
            const float tt = t0;
            t0 = t1;
            t1 = tt;
            winding = w16(-winding);
        }
        push_event(evt_pos, EdgeData{evt_to, t0, t1, winding, 1u}, from_id, to_id);
        b.nth += 1;
    }
    __host__ __device__ void eq_line_segment(Builder& b, V2 to, uint32_t to_id, float t0,
                                             float t1) {
        const V2 from = b.current;
        if (peq(from, to)) return;
        if (is_after(from, to) && b.nth > 0 && is_after(from, b.prev))
            eq_vertex_event(from, b.prev_id);
        if (b.nth == 0) b.second = to;
        eq_add_edge(b, from, to, 1, t0, t1, b.prev_id, to_id);
        b.prev = b.current;
        b.prev_id = to_id;
        b.current = to;
    }
    __host__ __device__ void eq_end(Builder& b, V2 first_pt, uint32_t first_id) {
        if (b.nth == 0) return;
        eq_line_segment(b, first_pt, first_id, 0.0f, 1.0f);
        if (is_after(first_pt, b.prev) && is_after(first_pt, b.second))
            eq_vertex_event(first_pt, first_id);
        b.prev_id = first_id;
        b.nth = 0;
    }
    // Shared body of quadratic_bezier_segment / cubic_bezier_segment (event_queue.rs:758-900):
    // the (possibly swapped) segment flattened with lyon's for_each_flattened_with_t. A swapped
    // curve's t values are those of the swapped segment while its ids stay the original ones.
    __host__ __device__ void eq_curve(Builder& b, V2 original_from, V2 original_to, uint32_t to_id,
                                      bool needs_swap, const Poly& poly, V2 seg_from, V2 seg_to,
                                      float n) {
        const int16_t winding = needs_swap ? -1 : 1;
        V2 prev_pt = seg_from;
        bool have_first = false;
        V2 first_pt = V2{0.0f, 0.0f};
        const bool is_first_edge = b.nth == 0;
        // flatten_with_t: count = to_u32(n) - 1 interior steps, t += 1/n, then the end point.
        const float step = 1.0f / n;
        float t0 = 0.0f;
        const uint32_t count = to_u32_or1(n) - 1;
        V2 from = seg_from;
        for (uint32_t i = 0; i <= count; ++i) {
            float t1;
            V2 to;
            if (i < count) {
                t1 = t0 + step;
                to = poly_sample(poly, t1);
            } else {
                t1 = 1.0f;
                to = seg_to;
            }
            if (!peq(from, to)) {
                if (!have_first) {
                    have_first = true;
                    first_pt = to;
                } else if (is_after(from, to) && is_after(from, prev_pt)) {
                    eq_vertex_event_on_curve(from, t0, b.prev_id, to_id);
                }
                eq_add_edge(b, from, to, winding, t0, t1, b.prev_id, to_id);
                prev_pt = from;
            }
            from = to;
            t0 = t1;
            if (h.oom) return;
        }
        if (have_first) {
            V2 second_pt, previous;
            if (needs_swap) {
                second_pt = prev_pt;
                previous = first_pt;
            } else {
                second_pt = first_pt;
                previous = prev_pt;
            }
            if (is_first_edge) {
                b.second = second_pt;
            } else if (is_after(original_from, b.prev) && is_after(original_from, second_pt)) {
                eq_vertex_event(original_from, b.prev_id);
            }
            b.prev = previous;
            b.current = original_to;
            b.prev_id = to_id;
        }
    }
    __host__ __device__ void eq_quad(Builder& b, V2 ctrl, V2 to, uint32_t to_id) {
        const V2 from = b.current;
        const bool needs_swap = is_after(from, to);
        V2 sf = from, st = to;
        if (needs_swap) {
            sf = to;
            st = from;
        }
        const float n = quad_wang(sf, ctrl, st, b.tolerance);
        const Poly poly = quad_poly(sf, ctrl, st);
        eq_curve(b, from, to, to_id, needs_swap, poly, sf, st, n);
    }
    __host__ __device__ void eq_cubic(Builder& b, V2 c1, V2 c2, V2 to, uint32_t to_id) {
        const V2 from = b.current;
        const bool needs_swap = is_after(from, to);
        V2 sf = from, sc1 = c1, sc2 = c2, st = to;
        if (needs_swap) {
            sf = to;
            st = from;
            sc1 = c2;
            sc2 = c1;
        }
        const float n = cubic_wang(sf, sc1, sc2, st, b.tolerance);
        const Poly poly = cubic_poly(sf, sc1, sc2, st);
        eq_curve(b, from, to, to_id, needs_swap, poly, sf, st, n);
    }

    // Number of edges the event queue builder will produce at most (lines, flattened curve
    // segments, closing edges); an estimate for reservations only.
    __host__ __device__ uint32_t count_segments(const uint8_t* verbs, uint32_t nverbs,
                                                const float* pts, uint32_t npts,
                                                const lyon_fill_options& o) {
        uint32_t segs = 0, pi = 0;
        V2 cur = V2{0.0f, 0.0f};
        for (uint32_t vi = 0; vi < nverbs; ++vi) {
            const uint8_t v = verbs[vi];
            const uint32_t np = v == LYON_VERB_QUADRATIC_TO ? 2u : v == LYON_VERB_CUBIC_TO ? 3u
                                : (v == LYON_VERB_END ? 0u : 1u);
            if (pi + np > npts) break;
            if (v == LYON_VERB_QUADRATIC_TO) {
                V2 c = V2{pts[2 * pi], pts[2 * pi + 1]}, t = V2{pts[2 * pi + 2], pts[2 * pi + 3]};
                segs += to_u32_or1(quad_wang(cur, c, t, o.tolerance));
                cur = t;
            } else if (v == LYON_VERB_CUBIC_TO) {
                V2 c1 = V2{pts[2 * pi], pts[2 * pi + 1]}, c2 = V2{pts[2 * pi + 2], pts[2 * pi + 3]};
                V2 t = V2{pts[2 * pi + 4], pts[2 * pi + 5]};
                segs += to_u32_or1(cubic_wang(cur, c1, c2, t, o.tolerance));
                cur = t;
            } else {
                if (np) cur = V2{pts[2 * pi], pts[2 * pi + 1]};
                segs += 1;
            }
            pi += np;
        }
        return segs > (1u << 20) ? (1u << 20) : segs;
    }

    // Builds the event queue of a path (event_queue.rs:483-551 set_path). Returns false on a
    // malformed path.
    __host__ __device__ bool build_events(const uint8_t* verbs, uint32_t nverbs, const float* pts,
                                 uint32_t npts, const lyon_fill_options& o) {
        Builder b;
        b.current = b.prev = b.second = V2{u2f(0x7fc00000u), u2f(0x7fc00000u)};
        b.nth = 0;
        b.prev_id = LYON_NO_ENDPOINT;
        b.tolerance = o.tolerance;
        const bool horizontal = o.sweep_orientation == LYON_ORIENTATION_HORIZONTAL;
        uint32_t pi = 0;
        V2 first_pt = V2{0.0f, 0.0f};
        uint32_t first_id = LYON_NO_ENDPOINT;
        auto take = [&](bool* bad) -> V2 {
            if (pi >= npts) {
                *bad = true;
                return V2{0.0f, 0.0f};
            }
            V2 p = V2{pts[2 * pi], pts[2 * pi + 1]};
            ++pi;
            return horizontal ? V2{-p.y, p.x} : p;  // event_queue.rs:13-16
        };
        bool bad = false;
        for (uint32_t vi = 0; vi < nverbs && !bad; ++vi) {
            switch (verbs[vi]) {
                case LYON_VERB_BEGIN: {
                    V2 p = take(&bad);
                    first_pt = p;
                    first_id = pi - 1;
                    b.nth = 0;
                    b.current = p;
                    b.prev_id = first_id;
                    break;
                }
                case LYON_VERB_LINE_TO: {
                    V2 p = take(&bad);
                    if (!bad) eq_line_segment(b, p, pi - 1, 0.0f, 1.0f);
                    break;
                }
                case LYON_VERB_QUADRATIC_TO: {
                    V2 c = take(&bad);
                    V2 p = take(&bad);
                    if (!bad) eq_quad(b, c, p, pi - 1);
                    break;
                }
                case LYON_VERB_CUBIC_TO: {
                    V2 c1 = take(&bad);
                    V2 c2 = take(&bad);
                    V2 p = take(&bad);
                    if (!bad) eq_cubic(b, c1, c2, p, pi - 1);
                    break;
                }
                case LYON_VERB_CLOSE:
                    (void)take(&bad);
                    if (!bad) eq_end(b, first_pt, first_id);
                    break;
                case LYON_VERB_END:
                    eq_end(b, first_pt, first_id);
                    break;
                default:
                    bad = true;
                    break;
            }
            if (h.oom) return true;
        }
        return !bad;
    }

    // fill.rs:578-596 + 749-821
    __host__ __device__ void tessellate(const uint8_t* verbs, uint32_t nverbs, const float* pts,
                               uint32_t npts, const lyon_fill_options& o) {
        err = 0;
        out_v.init();
        out_i.init();
        out_src.init();
        out_sfirst.init();
        events.init();
        edge_data.init();
        edge_ids.init();
        active.init();
        edges_below.init();
        spans.init();
        sc_vertex_events.init();
        sc_edges_to_split.init();
        sc_spans_to_end.init();
        first = NONE;
        current_position = V2{-3.40282347e38f, -3.40282347e38f};
        current_vertex = NONE;
        current_event_id = NONE;
        {
            // Room for every flattened edge and a vertex event per edge, so the event arrays
            // rarely grow (a growth copies them).
            const uint32_t segs = count_segments(verbs, nverbs, pts, npts, o);
            events.reserve(h, segs + segs / 4 + 8);
            edge_data.reserve(h, segs + segs / 4 + 8);
            if constexpr (SRC) edge_ids.reserve(h, 2 * (segs + segs / 4 + 8));
        }
        if (!build_events(verbs, nverbs, pts, npts, o)) {
            fail(LYON_ERR_INVALID_ARGUMENT);
            return;
        }
        if (!ok()) return;
        sort_events();
        out_v.reserve(h, events.n + 8);
        out_i.reserve(h, 6 * events.n + 24);
        if constexpr (SRC) {
            out_sfirst.reserve(h, events.n + 8);
            out_src.reserve(h, 3 * events.n + 24);
        }
        if (o.tolerance != o.tolerance || o.tolerance <= 0.0f) {
            fail(LYON_ERR_TOLERANCE_IS_NAN);
            return;
        }
        fill_rule = o.fill_rule;
        orientation = o.sweep_orientation;
        assume_no_intersection = !o.handle_intersections;
        tolerance = o.tolerance * 0.5f;
        tessellator_loop();
        if (!ok()) return;
        if (assume_no_intersection && (active.n != 0 || spans.n != 0)) {
            fail(LYON_ERR_INTERNAL);
            return;
        }
        for (uint32_t i = 0; i < spans.n; ++i) {
            Span& s = spans.at(h, i);
            if (s.alive) flush_triangles(s);
        }
        spans.clear();
        ok();
    }
};
using Filler = FillerT<false>;

}  // namespace fillk
}  // namespace lg
