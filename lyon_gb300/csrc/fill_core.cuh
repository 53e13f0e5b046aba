// fill_core.cuh — lyon's FillTessellator (crates/tessellation/src/fill.rs, event_queue.rs,
// monotone.rs) as device code run by one thread per path.
//
// The sweep line is sequential within a path, so a thread owns a path from event-queue
// construction to the last span flush. Its growable arrays (events, active edges, spans and
// each span's monotone tessellator state) live in a private bump-allocated heap in device
// memory; a heap that runs out marks the path (FILL_ERR_HEAP) and the host re-runs such paths
// with larger heaps. Every arithmetic step follows lyon's order of operations in f32 (f64 where
// lyon uses f64: segment intersections), so outputs match the CPU implementation bit for bit.
#pragma once

#include "geom.cuh"

namespace lg {
namespace fillk {

constexpr uint32_t NONE = 0xFFFFFFFFu;
constexpr int LEFT = 0, RIGHT = 1;
constexpr int FILL_ERR_HEAP = 1000;  // internal: the path's heap was too small (retried)

// ---- per-path heap and growable arrays --------------------------------------------------------

__host__ __device__ __forceinline__ uint32_t ceil_log2(uint32_t x) {
    uint32_t c = 0;
    while ((1u << c) < x) ++c;
    return c;
}

// Bump allocation of power-of-two blocks (8 words and up) with one free list per size, so the
// arrays a path outgrows and the state of ended spans are reused.
constexpr uint32_t HEAP_CLASSES = 28;

struct Heap {
    uint32_t* w;
    uint32_t cap, top;
    bool oom;
    uint32_t free_head[HEAP_CLASSES];
    __host__ __device__ void reset() {
        top = 0;
        oom = false;
        for (uint32_t c = 0; c < HEAP_CLASSES; ++c) free_head[c] = NONE;
    }
    __host__ __device__ __forceinline__ uint32_t alloc(uint32_t words) {
        const uint32_t start = (top + 1u) & ~1u;  // 8-byte alignment for float2 members
        if (oom || start > cap || words > cap - start) {
            oom = true;
            return 0;
        }
        top = start + words;
        return start;
    }
    // A block of at least `words` words; *cls receives its size class (2^cls words).
    __host__ __device__ uint32_t alloc_block(uint32_t words, uint32_t* cls) {
        uint32_t c = ceil_log2(words < 8 ? 8 : words);
        *cls = c;
        if (c < HEAP_CLASSES && free_head[c] != NONE) {
            const uint32_t o = free_head[c];
            free_head[c] = w[o];
            return o;
        }
        return alloc(1u << c);
    }
    __host__ __device__ void free_block(uint32_t off, uint32_t c) {
        if (c >= HEAP_CLASSES || oom) return;
        w[off] = free_head[c];
        free_head[c] = off;
    }
};

template <class T>
struct Vec {
    uint32_t off, n, cap;
    __host__ __device__ __forceinline__ void init() { off = 0; n = 0; cap = 0; }
    __host__ __device__ __forceinline__ T* p(const Heap& h) const {
        return reinterpret_cast<T*>(h.w + off);
    }
    __host__ __device__ __forceinline__ T& at(const Heap& h, uint32_t i) const { return p(h)[i]; }
    static constexpr uint32_t WPE = (uint32_t)((sizeof(T) + 3) / 4);  // words per element
    // Out of line on the device: growth is rare, and inlining it at every push bloats the sweep
    // past the instruction cache (measured: 18 % slower inlined).
    __host__ __device__
#ifdef __CUDA_ARCH__
    __noinline__
#endif
    bool reserve(Heap& h, uint32_t want) {
        if (want <= cap) return true;
        uint32_t nc = cap < 4 ? 4 : cap * 2;
        while (nc < want) nc *= 2;
        uint32_t cls;
        const uint32_t o = h.alloc_block(nc * WPE, &cls);
        if (h.oom) return false;
        T* dst = reinterpret_cast<T*>(h.w + o);
        const T* src = p(h);
        for (uint32_t i = 0; i < n; ++i) dst[i] = src[i];
        if (cap > 0) h.free_block(off, ceil_log2(cap * WPE));
        off = o;
        cap = (1u << cls) / WPE;
        return true;
    }
    // Returns the array's block to the heap (the array becomes empty).
    __host__ __device__ void release(Heap& h) {
        if (cap > 0) h.free_block(off, ceil_log2(cap * WPE));
        off = 0;
        cap = 0;
        n = 0;
    }
    __host__ __device__ __forceinline__ bool push(Heap& h, const T& v) {
        if (!reserve(h, n + 1)) return false;
        p(h)[n++] = v;
        return true;
    }
    __host__ __device__ bool insert(Heap& h, uint32_t i, const T& v) {
        if (!reserve(h, n + 1)) return false;
        T* d = p(h);
        for (uint32_t k = n; k > i; --k) d[k] = d[k - 1];
        d[i] = v;
        ++n;
        return true;
    }
    __host__ __device__ void erase(Heap& h, uint32_t i) {
        T* d = p(h);
        for (uint32_t k = i; k + 1 < n; ++k) d[k] = d[k + 1];
        --n;
    }
    __host__ __device__ __forceinline__ void clear() { n = 0; }
};

// ---- event queue (event_queue.rs) ---------------------------------------------------------------

struct Event {
    uint32_t next_sibling, next_event;
    V2 pos;
};
struct EdgeData {  // event_queue.rs:28-36
    V2 to;
    float range_start, range_end;
    int32_t winding;  // lyon's i16, wrapped on every update
    uint32_t is_edge;
};

__host__ __device__ __forceinline__ int16_t w16(int v) { return (int16_t)v; }

// ---- monotone tessellators (monotone.rs) ------------------------------------------------------

struct MV {
    V2 pos;
    uint32_t id;
    int32_t side;
};

struct SideEvents {  // monotone.rs:189-210
    V2 reference_point;
    float conservative_reference_x;
    uint32_t pad;
    Vec<uint32_t> events;
    uint32_t pad2;
    V2 prev;
    MV last;
};

struct Span {  // an AdvancedMonotone (monotone.rs:212-359) with its BasicMonotone
    Vec<MV> stack;
    uint32_t alive;
    MV previous;
    Vec<uint32_t> triangles;
    uint32_t pad;
    SideEvents left, right;
};

// ---- sweep structures (fill.rs) --------------------------------------------------------------

struct ActiveEdge {  // fill.rs:153-170
    V2 from, to;
    int32_t winding;
    uint32_t is_merge;
    uint32_t from_id, src_edge;
    float range_end;
    uint32_t pad;
    __host__ __device__ __forceinline__ float min_x() const { return fminf(from.x, to.x); }
    __host__ __device__ __forceinline__ float max_x() const { return from.x > to.x ? from.x : to.x; }
    // fill.rs:185-200 with geom line.rs:56-71
    __host__ __device__ __forceinline__ float solve_x_for_y(float y) const {
        float dy = to.y - from.y;
        float t = dy == 0.0f ? 0.0f : (y - from.y) / dy;
        float x = from.x * (1.0f - t) + to.x * t;
        return fminf(fmaxf(x, min_x()), max_x());
    }
};

struct PendingEdge {  // fill.rs:304-312
    V2 to;
    float sort_key;
    uint32_t src_edge;
    int32_t winding;
    float range_end;
};

struct VertexEvent {
    int32_t span;
    int32_t side;
};

__host__ __device__ __forceinline__ float fmax_lyon(float a, float b) { return a > b ? a : b; }
__host__ __device__ __forceinline__ float slope(V2 v) { return v.x / fmaxf(v.y, 1.17549435e-38f); }
__host__ __device__ __forceinline__ bool fill_rule_is_in(int rule, int16_t w) {  // path/src/lib.rs:267-281
    if (rule == LYON_FILL_EVEN_ODD) return (w % 2) != 0;
    return w != 0;
}

struct WindingState {  // fill.rs:88-113
    int32_t span_index;
    int16_t number;
    bool is_in;
    __host__ __device__ __forceinline__ void reset() {
        span_index = -1;
        number = 0;
        is_in = false;
    }
    __host__ __device__ __forceinline__ void update(int rule, int16_t w) {
        number = w16(number + w);
        is_in = fill_rule_is_in(rule, number);
        if (is_in) span_index += 1;
    }
};

// fill.rs:2339-2347
__host__ __device__ __forceinline__ float remap_t_in_range(float val, float start, float end) {
    if (end > start) {
        float d = end - start;
        return start + val * d;
    }
    float d = start - end;
    return end + (1.0f - val) * d;
}

// Side of p relative to the line a -> b, (a - p) x (b - a), in f32 with a bound on its rounding
// error: (a.x - p.x) and (a.y - p.y) round once, the products and the difference once more, so
// the error stays below 4 * 2^-24 * (|t1| + |t2|); 1e-5 leaves a wide margin, and 1e-30 covers
// underflow. NaN or infinite terms compare false and leave the sign unknown.
__host__ __device__ __forceinline__ float orient_f32(V2 p, V2 a, V2 b, float* bound) {
    const float t1 = (a.x - p.x) * (b.y - a.y);
    const float t2 = (a.y - p.y) * (b.x - a.x);
    *bound = 1e-5f * (fabsf(t1) + fabsf(t2)) + 1e-30f;
    return t1 - t2;
}

// False only when segments s and o certainly do not intersect: both end points of one lie
// strictly on the same side of the other's line, beyond the rounding bound. lyon's f64 test
// (below) computes the same two orientations per segment, so it returns false in exactly
// those cases; pairs that pass this filter go through the f64 test unchanged.
__host__ __device__ __forceinline__ bool may_intersect(V2 sf, V2 st, V2 of, V2 ot) {
    float b1, b2, b3, b4;
    const float o1 = orient_f32(sf, of, ot, &b1), o2 = orient_f32(st, of, ot, &b2);
    if ((o1 > b1 && o2 > b2) || (o1 < -b1 && o2 < -b2)) return false;
    const float o3 = orient_f32(of, sf, st, &b3), o4 = orient_f32(ot, sf, st, &b4);
    if ((o3 > b3 && o4 > b4) || (o3 < -b3 && o4 < -b4)) return false;
    return true;
}

// geom line.rs:217-253 with S = f64
static __host__ __device__ bool segment_intersection_t(double sfx, double sfy, double stx, double sty,
                                       double ofx, double ofy, double otx, double oty,
                                       double* ta, double* tb) {
    if ((stx == otx && sty == oty) || (sfx == ofx && sfy == ofy) ||
        (sfx == otx && sfy == oty) || (stx == ofx && sty == ofy)) {
        return false;
    }
    double v1x = stx - sfx, v1y = sty - sfy;
    double v2x = otx - ofx, v2y = oty - ofy;
    double v1_cross_v2 = v1x * v2y - v1y * v2x;
    if (v1_cross_v2 == 0.0) return false;
    double sign = v1_cross_v2 > 0.0 ? 1.0 : -1.0;
    double abs_c = fabs(v1_cross_v2);
    double v3x = ofx - sfx, v3y = ofy - sfy;
    double t = (v3x * v2y - v3y * v2x) * sign;
    double u = (v3x * v1y - v3y * v1x) * sign;
    if (t < 0.0 || t > abs_c || u < 0.0 || u > abs_c) return false;
    *ta = t / abs_c;
    *tb = u / abs_c;
    return true;
}

}  // namespace fillk
}  // namespace lg
