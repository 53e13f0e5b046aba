// hatch.cu — batched hatching and dot patterns: lyon_algorithms' Hatcher::hatch_path / dot_path
// (crates/algorithms/src/hatching.rs) with the regular patterns (RegularHatchingPattern,
// RegularDotPattern), one thread per path.
//
//   1. bound kernel: each path's edge count at most (lines, flattened curve segments, one
//      closing edge per sub-path); the library's scan places each path's scratch;
//   2. count kernel: the EventsBuilder (hatching.rs:464-577): flattened edges rotated by the
//      pattern angle and oriented downwards, then sorted by their upper end (a stable bottom-up
//      merge sort in scratch); the sweep (hatching.rs:300-428) counts the segments (or dots);
//   3. emit kernel: the sweep again over the sorted edges, writing at the scanned offsets.
// The sweep keeps lyon's active list: edges that may still cross the scan line, sorted in place
// (stably) by their x on every row.
#include "geom.cuh"
#include "kernels.h"

namespace lg {
namespace {

struct HEdge {
    V2 from, to;
};

__device__ __forceinline__ int cmp_pos(V2 a, V2 b) {  // hatching.rs:617-632
    if (a.y > b.y) return 1;
    if (a.y < b.y) return -1;
    if (a.x > b.x) return 1;
    if (a.x < b.x) return -1;
    return 0;
}

__device__ __forceinline__ V2 rot(V2 p, float c, float s) {
    return V2{p.x * c - p.y * s, p.x * s + p.y * c};
}

__device__ __forceinline__ float x_for_y(const HEdge& e, float y) {  // geom line.rs:56-71
    const float dy = e.to.y - e.from.y;
    const float t = dy == 0.0f ? 0.0f : (y - e.from.y) / dy;
    return e.from.x * (1.0f - t) + e.to.x * t;
}

__device__ __forceinline__ uint32_t verb_points(int k) {
    return k == LYON_VERB_QUADRATIC_TO ? 2u : k == LYON_VERB_CUBIC_TO ? 3u
           : (k == LYON_VERB_END ? 0u : (k <= LYON_VERB_CLOSE ? 1u : 0u));
}

// Step 1: edges a path can produce at most.
__global__ void hatch_bound_kernel(HatchArgs A) {
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < A.num_paths;
         p += gridDim.x * blockDim.x) {
        const uint32_t v0 = A.verb_offsets[p], v1 = A.verb_offsets[p + 1];
        uint32_t pc = A.point_offsets[p];
        const uint32_t pe = A.point_offsets[p + 1];
        uint32_t n = 0;
        V2 cur = V2{0.0f, 0.0f};
        for (uint32_t vi = v0; vi < v1; ++vi) {
            const int k = A.verbs[vi];
            const uint32_t np = verb_points(k);
            if (pc + np > pe) break;
            if (k == LYON_VERB_QUADRATIC_TO) {
                const V2 c = load_pt(A.points, pc), t = load_pt(A.points, pc + 1);
                n += to_u32_or1(quad_wang(cur, c, t, A.tolerance));
                cur = t;
            } else if (k == LYON_VERB_CUBIC_TO) {
                const V2 c1 = load_pt(A.points, pc), c2 = load_pt(A.points, pc + 1);
                const V2 t = load_pt(A.points, pc + 2);
                n += to_u32_or1(cubic_wang(cur, c1, c2, t, A.tolerance));
                cur = t;
            } else {
                if (np) cur = load_pt(A.points, pc);
                n += 1;
            }
            pc += np;
        }
        A.edge_bound[p] = n;
    }
}

struct Builder {
    HEdge* edges;
    uint32_t n, cap;
    V2 first, current;
    float c, s;
    __device__ void add_edge(V2 from, V2 to) {  // hatching.rs:471-482
        if (from.x == to.x && from.y == to.y) return;
        V2 f = rot(from, c, s), t = rot(to, c, s);
        if (cmp_pos(f, t) > 0) {
            const V2 x = f;
            f = t;
            t = x;
        }
        if (n < cap) edges[n] = HEdge{f, t};
        ++n;
    }
    __device__ void flatten(const Poly& poly, V2 to, float nseg) {
        const float step = 1.0f / nseg;
        const uint32_t count = to_u32_or1(nseg) - 1;
        float t0 = 0.0f;
        for (uint32_t i = 0; i <= count; ++i) {
            const bool last = i == count;
            const float t1 = last ? 1.0f : t0 + step;
            const V2 q = last ? to : poly_sample(poly, t1);
            add_edge(current, q);
            current = q;
            t0 = t1;
        }
    }
};

// Stable bottom-up merge sort of edges by their upper end (`sort_by(compare_positions)`).
__device__ void sort_edges(HEdge* a, HEdge* tmp, uint32_t n) {
    HEdge* src = a;
    HEdge* dst = tmp;
    for (uint32_t w = 1; w < n; w *= 2) {
        for (uint32_t lo = 0; lo < n; lo += 2 * w) {
            const uint32_t mid = min(lo + w, n), hi = min(lo + 2 * w, n);
            uint32_t i = lo, j = mid, k = lo;
            while (i < mid && j < hi) dst[k++] = cmp_pos(src[j].from, src[i].from) < 0 ? src[j++]
                                                                                       : src[i++];
            while (i < mid) dst[k++] = src[i++];
            while (j < hi) dst[k++] = src[j++];
        }
        HEdge* x = src;
        src = dst;
        dst = x;
    }
    if (src != a)
        for (uint32_t i = 0; i < n; ++i) a[i] = src[i];
}

// The sweep (hatching.rs:300-428) with the regular patterns, counting or writing.
struct Sweep {
    const HatchArgs* A;
    const HEdge* edges;
    uint32_t ne;
    HEdge* active;
    uint32_t na;
    V2 uv;
    uint32_t column;
    uint64_t rows, count;
    bool too_many;
    lyon_hatch_segment* segs;  // write targets (emit pass), else null
    lyon_dot* dots;

    __device__ void emit_segment(const lyon_hatch_segment& g) {
        if (!A->dots) {
            if (segs) segs[count] = g;
            ++count;
            return;
        }
        // HatchesToDots::add_segment (hatching.rs:677-714) with RegularDotPattern.
        float u = 0.0f;
        const float u_start = g.a_u;
        const float d = A->column_interval;
        const float m = u_start >= 0.0f ? fmodf(u_start, d) : d + fmodf(u_start, d);
        if (m != 0.0f) u += d - m;
        const V2 a = V2{g.a_x, g.a_y};
        const V2 ab = normalize(V2{g.b_x, g.b_y} - a);
        while (u_start + u < g.b_u) {
            if (count >= LYON_MAX_HATCH_DOTS) {
                too_many = true;
                return;
            }
            if (dots) {
                const V2 q = a + ab * u;
                dots[count] = lyon_dot{q.x, q.y, g.a_u + u, g.v, column, g.row};
            }
            ++count;
            column += 1;
            const float du = A->column_interval;
            if (du <= 0.0f) return;
            u += du;
        }
    }

    __device__ void hatch_line(float y, uint32_t row) {
        // Stable insertion sort of the active edges by x at y (sort_by_key, in place).
        for (uint32_t i = 1; i < na; ++i) {
            const HEdge e = active[i];
            const float x = x_for_y(e, y);
            uint32_t j = i;
            while (j > 0 && x_for_y(active[j - 1], y) > x) {
                active[j] = active[j - 1];
                --j;
            }
            active[j] = e;
        }
        bool inside = false;
        float prev_x = __int_as_float(0x7fc00000);
        const V2 nan2 = V2{__int_as_float(0x7fc00000), __int_as_float(0x7fc00000)};
        V2 prev_tan = nan2, tan = nan2;
        const float v = y - uv.y;
        for (uint32_t i = 0; i < na; ++i) {
            const HEdge e = active[i];
            if (e.to.y <= y) continue;
            const float x = x_for_y(e, y);
            if (A->compute_tangents) tan = normalize(rot(e.to - e.from, A->ci, A->si));
            if (inside) {
                const V2 pa = rot(V2{prev_x, y}, A->ci, A->si);
                const V2 pb = rot(V2{x, y}, A->ci, A->si);
                const V2 ta = A->compute_tangents ? prev_tan : nan2;
                const V2 tb = A->compute_tangents ? tan : nan2;
                emit_segment(lyon_hatch_segment{pa.x, pa.y, ta.x, ta.y, prev_x - uv.x, pb.x,
                                                pb.y, tb.x, tb.y, x - uv.x, row, v});
                if (too_many) return;
            }
            inside = !inside;
            prev_x = x;
            prev_tan = tan;
        }
    }

    // hatch_line then next_offset; false ends the sweep.
    __device__ bool line(float& y, uint32_t& row) {
        if (++rows > LYON_MAX_HATCH_ROWS) {
            too_many = true;
            return false;
        }
        hatch_line(y, row);
        if (too_many) return false;
        row += 1;
        column = 0;
        y += A->interval;
        return A->interval > 0.0f;
    }

    __device__ void run() {
        if (ne == 0) return;
        uv = rot(V2{A->uv_x, A->uv_y}, A->c, A->s);
        uint32_t row = 0;
        float y = edges[0].from.y + A->interval;
        float y_max = y;
        for (uint32_t i = 0; i < ne; ++i) {
            const HEdge e = edges[i];
            while (y < e.from.y)
                if (!line(y, row)) return;
            y_max = fmaxf(y_max, e.to.y);
            // update_sweep_line (hatching.rs:374-379): a stable removal, then the new edge.
            uint32_t k = 0;
            for (uint32_t j = 0; j < na; ++j)
                if (cmp_pos(active[j].to, e.from) >= 0) active[k++] = active[j];
            active[k++] = e;
            na = k;
        }
        while (y < y_max)
            if (!line(y, row)) return;
    }
};

// Step 2: edges built and sorted in the path's scratch; outputs counted.
__global__ void hatch_count_kernel(HatchArgs A) {
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < A.num_paths;
         j += gridDim.x * blockDim.x) {
        const uint32_t p = A.order ? A.order[j] : j;
        const uint64_t so = A.scratch_offsets[p];
        const uint32_t cap = (uint32_t)(A.scratch_offsets[p + 1] - so);
        HEdge* edges = reinterpret_cast<HEdge*>(A.scratch) + so;
        HEdge* tmp = edges + A.scratch_total;
        HEdge* active = tmp + A.scratch_total;
        Builder b;
        b.edges = edges;
        b.n = 0;
        b.cap = cap;
        b.first = b.current = V2{0.0f, 0.0f};
        b.c = A.c;
        b.s = A.s;
        const uint32_t v0 = A.verb_offsets[p], v1 = A.verb_offsets[p + 1];
        uint32_t pc = A.point_offsets[p];
        const uint32_t pe = A.point_offsets[p + 1];
        int st = LYON_OK;
        for (uint32_t vi = v0; vi < v1 && st == LYON_OK; ++vi) {
            const int k = A.verbs[vi];
            const uint32_t np = verb_points(k);
            if (k > LYON_VERB_END || pc + np > pe) {
                st = LYON_ERR_INVALID_ARGUMENT;
                break;
            }
            if (k == LYON_VERB_BEGIN) {
                b.first = b.current = load_pt(A.points, pc);
            } else if (k == LYON_VERB_LINE_TO) {
                const V2 t = load_pt(A.points, pc);
                b.add_edge(b.current, t);
                b.current = t;
            } else if (k == LYON_VERB_QUADRATIC_TO) {
                const V2 c = load_pt(A.points, pc), t = load_pt(A.points, pc + 1);
                b.flatten(quad_poly(b.current, c, t), t, quad_wang(b.current, c, t, A.tolerance));
            } else if (k == LYON_VERB_CUBIC_TO) {
                const V2 c1 = load_pt(A.points, pc), c2 = load_pt(A.points, pc + 1);
                const V2 t = load_pt(A.points, pc + 2);
                b.flatten(cubic_poly(b.current, c1, c2, t), t,
                          cubic_wang(b.current, c1, c2, t, A.tolerance));
            } else {  // Close or End: the closing edge, whether or not the sub-path is closed
                b.add_edge(b.current, b.first);
            }
            pc += np;
        }
        if (st == LYON_OK && b.n > cap) st = LYON_ERR_INTERNAL;
        uint64_t count = 0;
        if (st == LYON_OK) {
            sort_edges(edges, tmp, b.n);
            Sweep sw{&A, edges, b.n, active, 0, V2{0.0f, 0.0f}, 0, 0, 0, false, nullptr,
                     nullptr};
            sw.run();
            if (sw.too_many) st = LYON_ERR_UNSUPPORTED;
            count = sw.count;
        }
        if (st == LYON_OK && count > 0xFFFFFFFFull) st = LYON_ERR_UNSUPPORTED;
        A.edge_count[p] = st == LYON_OK ? b.n : 0u;
        A.counts[p] = st == LYON_OK ? (uint32_t)count : 0u;
        A.status[p] = st;
    }
}

// Step 3: the sweep over the sorted edges again, writing.
__global__ void hatch_emit_kernel(HatchArgs A) {
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < A.num_paths;
         j += gridDim.x * blockDim.x) {
        const uint32_t p = A.order ? A.order[j] : j;
        if (A.status[p] != LYON_OK || A.counts[p] == 0) continue;
        const uint64_t so = A.scratch_offsets[p];
        HEdge* edges = reinterpret_cast<HEdge*>(A.scratch) + so;
        HEdge* active = edges + 2 * A.scratch_total;
        const uint64_t o = A.out_offsets[p];
        Sweep sw{&A, edges, A.edge_count[p], active, 0, V2{0.0f, 0.0f}, 0, 0, 0, false,
                 A.dots ? nullptr : A.segments + o, A.dots ? A.dot_out + o : nullptr};
        sw.run();
    }
}

unsigned grid_for(uint32_t n, int num_sms) {
    const uint32_t need = (n + 127) / 128;
    const uint32_t cap = (uint32_t)(num_sms > 0 ? num_sms : 1) * 16;
    return need < cap ? need : cap;
}

}  // namespace

cudaError_t launch_hatch(const HatchArgs& args, int phase, int num_sms, cudaStream_t stream) {
    if (args.num_paths == 0) return cudaSuccess;
    const unsigned g = grid_for(args.num_paths, num_sms);
    if (phase == 0) {
        hatch_bound_kernel<<<g, 128, 0, stream>>>(args);
    } else if (phase == 1) {
        hatch_count_kernel<<<g, 128, 0, stream>>>(args);
    } else {
        hatch_emit_kernel<<<g, 128, 0, stream>>>(args);
    }
    note_launches(1);
    return cudaGetLastError();
}

}  // namespace lg
