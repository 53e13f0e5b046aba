// shapes.cu — batched basic shapes (crates/tessellation/src/basic_shapes.rs): the fills that
// FillTessellator::tessellate_rectangle and tessellate_circle produce without the sweep.
//
// One thread per shape. The count kernel computes each shape's vertex and index counts in
// closed form (a rectangle: 4 and 6; a circle: 4 + 4 (2^n - 1) vertices and 2 + 4 (2^n - 1)
// triangles, n from the circle's flattening step); the library's scan turns them into offsets
// and the emit kernel writes every shape at its offsets in lyon's order (the four axis vertices,
// two triangles, then the four quarter arcs, each bisected depth first).
#include "geom.cuh"
#include "kernels.h"

namespace lg {

namespace {

// basic_shapes.rs:151-155
__device__ __forceinline__ float fill_circle_step(float radius, float tolerance) {
    tolerance = fminf(tolerance, radius);
    return 2.0f * sqrtf(2.0f * tolerance * radius - tolerance * tolerance);
}

// The bisection depth of a circle's quarter arcs (basic_shapes.rs:98-101). Deeper than
// MAX_SHAPE_DEPTH (more than four million vertices for one circle) fails the shape with
// LYON_ERR_UNSUPPORTED, as the oracle does.
constexpr uint32_t MAX_SHAPE_DEPTH = 20;
__device__ __forceinline__ uint32_t circle_depth(float radius, float tolerance) {
    const float arc_len = 0.5f * LG_PI_F * radius;
    const float step = fill_circle_step(radius, tolerance);
    const float num_segments = ceilf(arc_len / step);
    return sat_u32(log2f(num_segments));  // `as u32`
}

__global__ void shapes_count_kernel(ShapeArgs A) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.n) return;
    uint32_t nv = 0, ni = 0;
    int st = LYON_OK;
    if (A.kind == LYON_SHAPE_RECTANGLE) {
        nv = 4;
        ni = 6;
    } else {
        const float r = fabsf(A.params[3 * i + 2]);
        if (r != 0.0f) {
            const lyon_fill_options o = A.options[A.num_options > 1 ? i : 0];
            const uint32_t d = circle_depth(r, o.tolerance);
            if (d > MAX_SHAPE_DEPTH) {
                st = LYON_ERR_UNSUPPORTED;
            } else {
                const uint32_t arc = (1u << d) - 1u;
                nv = 4 + 4 * arc;
                ni = 3 * (2 + 4 * arc);
            }
        }
    }
    A.vtx_counts[i] = st == LYON_OK ? nv : 0u;
    A.idx_counts[i] = st == LYON_OK ? ni : 0u;
    A.status[i] = st;
}

struct ShapeOut {
    float2* v;
    uint32_t* i32;
    uint16_t* i16;
    uint32_t nv, ni, base;
    __device__ __forceinline__ uint32_t vertex(V2 p) {
        v[nv] = make_float2(p.x, p.y);
        return base + nv++;
    }
    __device__ __forceinline__ void tri(uint32_t a, uint32_t b, uint32_t c) {
        if (i32) {
            i32[ni] = a;
            i32[ni + 1] = b;
            i32[ni + 2] = c;
        } else {
            i16[ni] = (uint16_t)a;
            i16[ni + 1] = (uint16_t)b;
            i16[ni + 2] = (uint16_t)c;
        }
        ni += 3;
    }
};

// fill_border_radius (basic_shapes.rs:158-207): the recursion made iterative with an explicit
// stack, visiting the bisections in the same order.
__device__ __noinline__ void fill_quarter(ShapeOut& o, V2 center, float radius, float a0,
                                          float a1, uint32_t va, uint32_t vb, uint32_t depth) {
    struct Frame {
        float a0, a1;
        uint32_t va, vb, n;
    };
    Frame st[MAX_SHAPE_DEPTH + 2];
    int sp = 0;
    st[sp++] = Frame{a0, a1, va, vb, depth};
    while (sp > 0) {
        const Frame f = st[--sp];
        if (f.n == 0) continue;
        const float mid = (f.a0 + f.a1) * 0.5f;
        const V2 normal = V2{cosf(mid), sinf(mid)};
        const uint32_t v = o.vertex(center + normal * radius);
        o.tri(f.vb, v, f.va);
        st[sp++] = Frame{mid, f.a1, v, f.vb, f.n - 1};
        st[sp++] = Frame{f.a0, mid, f.va, v, f.n - 1};
    }
}

__global__ void shapes_emit_kernel(ShapeArgs A) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.n || A.status[i] != LYON_OK || A.vtx_counts[i] == 0) return;
    const uint64_t vo = A.vtx_offsets[i], io = A.idx_offsets[i];
    ShapeOut o;
    o.v = reinterpret_cast<float2*>(A.vertices) + vo;
    o.i32 = A.index_bits == 32 ? reinterpret_cast<uint32_t*>(A.indices) + io : nullptr;
    o.i16 = A.index_bits == 16 ? reinterpret_cast<uint16_t*>(A.indices) + io : nullptr;
    o.nv = 0;
    o.ni = 0;
    o.base = A.vertex_offset + (A.index_mode == LYON_INDEX_GLOBAL ? (uint32_t)vo : 0u);
    if (A.kind == LYON_SHAPE_RECTANGLE) {
        // basic_shapes.rs:12-38
        const float* r = A.params + 4 * (size_t)i;
        const V2 mn = V2{r[0], r[1]}, mx = V2{r[2], r[3]};
        const uint32_t a = o.vertex(mn);
        const uint32_t b = o.vertex(V2{mn.x, mx.y});
        const uint32_t c = o.vertex(mx);
        const uint32_t d = o.vertex(V2{mx.x, mn.y});
        o.tri(a, b, c);
        o.tri(a, c, d);
    } else {
        // basic_shapes.rs:40-124
        const float* p = A.params + 3 * (size_t)i;
        const V2 center = V2{p[0], p[1]};
        const float radius = fabsf(p[2]);
        const lyon_fill_options opt = A.options[A.num_options > 1 ? i : 0];
        uint32_t v[4];
        v[0] = o.vertex(center + V2{-1.0f, 0.0f} * radius);
        v[1] = o.vertex(center + V2{0.0f, -1.0f} * radius);
        v[2] = o.vertex(center + V2{1.0f, 0.0f} * radius);
        v[3] = o.vertex(center + V2{0.0f, 1.0f} * radius);
        o.tri(v[0], v[3], v[1]);
        o.tri(v[1], v[3], v[2]);
        const float angles[4][2] = {{LG_PI_F, 1.5f * LG_PI_F},
                                    {1.5f * LG_PI_F, 2.0f * LG_PI_F},
                                    {0.0f, LG_PI_F * 0.5f},
                                    {LG_PI_F * 0.5f, LG_PI_F}};
        const uint32_t depth = circle_depth(radius, opt.tolerance);
        for (int k = 0; k < 4; ++k)
            fill_quarter(o, center, radius, angles[k][0], angles[k][1], v[k], v[(k + 1) % 4],
                         depth);
    }
}

}  // namespace

cudaError_t launch_shapes(const ShapeArgs& args, bool emit, cudaStream_t stream) {
    if (args.n == 0) return cudaSuccess;
    const uint32_t blocks = (args.n + 255) / 256;
    if (emit) {
        shapes_emit_kernel<<<blocks, 256, 0, stream>>>(args);
    } else {
        shapes_count_kernel<<<blocks, 256, 0, stream>>>(args);
    }
    note_launches(1);
    return cudaGetLastError();
}

}  // namespace lg
