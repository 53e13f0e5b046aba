// arcs.cu — batched flattening of elliptic arcs: lyon_geom's Arc::for_each_flattened_with_t
// (crates/geom/src/arc.rs:339-367) with its adaptive flattening_step (:369-389).
//
// One thread per arc: each step depends on the remaining arc (the step is taken from the
// radius at the arc's current start), so an arc is a sequential walk. The count kernel walks
// without writing; the library's scan turns the counts into offsets; the emit kernel walks again
// and writes every point (the start point first) and its t. cos, sin and acos are evaluated in
// f64 and rounded once, as the oracle does.
#include "kernels.h"

namespace lg {
namespace {

__device__ __forceinline__ float dcos(float x) { return (float)cos((double)x); }
__device__ __forceinline__ float dsin(float x) { return (float)sin((double)x); }
__device__ __forceinline__ float dacos(float x) { return (float)acos((double)x); }

struct ArcState {
    float cx, cy, rx, ry, start, sweep;
    float rc, rs;  // cos and sin of x_rotation (the same for every sample of the arc)
};

// sample (arc.rs:194-197): center + Rotation2D(x_rotation) applied to (rx cos a, ry sin a).
__device__ __forceinline__ float2 arc_sample(const ArcState& a, float t) {
    const float angle = a.start + a.sweep * t;
    // cos and sin of the angle in f64 from one shared argument reduction, each rounded once.
    double sd, cd;
    sincos((double)angle, &sd, &cd);
    const float ex = a.rx * (float)cd, ey = a.ry * (float)sd;
    return make_float2(a.cx + (ex * a.rc - ey * a.rs), a.cy + (ex * a.rs + ey * a.rc));
}

// flattening_step (arc.rs:369-389) of an arc whose start point, sample(0), is `from` (the
// point the walk emitted last: the same value lyon recomputes).
__device__ __forceinline__ float arc_step(const ArcState& a, float2 from, float tolerance) {
    const float dx = from.x - a.cx, dy = from.y - a.cy;
    const float r = sqrtf(dx * dx + dy * dy);
    const float ang = 2.0f * dacos((r - tolerance) / r);
    const float result = fminf(ang / fabsf(a.sweep), 1.0f);
    return result < 1.1920929e-7f ? 1.0f : result;  // f32::EPSILON
}

// Walks one arc; with `pts` it writes the points and t values. Returns the point count, or
// ARC_TOO_LONG past the segment bound (the arc then fails with LYON_ERR_UNSUPPORTED).
constexpr uint32_t ARC_TOO_LONG = 0xFFFFFFFFu;
__device__ uint32_t walk_arc(const lyon_arc& in, float tolerance, float2* pts, float* ts) {
    const ArcState arc{in.center_x, in.center_y, in.radius_x, in.radius_y, in.start_angle,
                       in.sweep_angle, dcos(in.x_rotation), dsin(in.x_rotation)};
    ArcState it = arc;
    float t0 = 0.0f;
    float2 from = arc_sample(arc, 0.0f);
    if (pts) {
        pts[0] = from;
        ts[0] = 0.0f;
    }
    uint32_t k = 1;
    for (;;) {
        const float step = arc_step(it, from, tolerance);
        if (step >= 1.0f) break;
        if (k > LYON_MAX_ARC_SEGMENTS) return ARC_TOO_LONG;
        const float split = it.sweep * step;  // after_split (arc.rs:286-296)
        it.start = it.start + split;
        it.sweep = it.sweep - split;
        const float t1 = t0 + step * (1.0f - t0);
        from = arc_sample(it, 0.0f);
        if (pts) {
            pts[k] = from;
            ts[k] = t1;
        }
        ++k;
        t0 = t1;
    }
    if (pts) {
        pts[k] = arc_sample(arc, 1.0f);
        ts[k] = 1.0f;
    }
    return k + 1;
}

// A rough step count (f32, mean radius) that only orders the count pass.
__global__ void __launch_bounds__(256) arcs_estimate_kernel(const lyon_arc* arcs, uint32_t n,
                                                            float tolerance, uint32_t* est) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const lyon_arc a = arcs[i];
        const float r = 0.5f * (fabsf(a.radius_x) + fabsf(a.radius_y));
        const float c = fminf(fmaxf((r - tolerance) / r, -1.0f), 1.0f);
        const float step = 2.0f * acosf(c);
        const float k = fabsf(a.sweep_angle) / fmaxf(step, 1e-7f);
        est[i] = k == k ? (uint32_t)fminf(k + 1.0f, 4.0e6f) : 1u;
    }
}

__global__ void __launch_bounds__(256) arcs_count_kernel(const lyon_arc* arcs, uint32_t n,
                                                         float tolerance, uint32_t* counts,
                                                         int32_t* status, const uint32_t* order) {
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        const uint32_t i = order ? order[j] : j;
        const uint32_t k = walk_arc(arcs[i], tolerance, nullptr, nullptr);
        counts[i] = k == ARC_TOO_LONG ? 0u : k;
        status[i] = k == ARC_TOO_LONG ? LYON_ERR_UNSUPPORTED : LYON_OK;
    }
}

// Arcs in decreasing size class (`order`), so that the 32 arcs of a warp take similar numbers of
// steps.
__global__ void __launch_bounds__(256) arcs_emit_kernel(const lyon_arc* arcs, uint32_t n,
                                                        float tolerance, const int32_t* status,
                                                        const uint64_t* offsets, float2* pts,
                                                        float* ts, const uint32_t* order) {
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const uint32_t i = order ? order[k] : k;
        if (status[i] != LYON_OK) continue;
        const uint64_t o = offsets[i];
        walk_arc(arcs[i], tolerance, pts + o, ts + o);
    }
}

}  // namespace

cudaError_t launch_arcs(const lyon_arc* arcs, uint32_t n, float tolerance, uint32_t* counts,
                        int32_t* status, const uint64_t* offsets, float* pts, float* ts,
                        int num_sms, cudaStream_t stream, const uint32_t* order) {
    if (n == 0) return cudaSuccess;
    const uint32_t need = (n + 255) / 256;
    const uint32_t cap = (uint32_t)(num_sms > 0 ? num_sms : 1) * 8;
    const uint32_t grid = need < cap ? need : cap;
    if (pts) {
        arcs_emit_kernel<<<grid, 256, 0, stream>>>(arcs, n, tolerance, status, offsets,
                                                   reinterpret_cast<float2*>(pts), ts, order);
    } else {
        arcs_count_kernel<<<grid, 256, 0, stream>>>(arcs, n, tolerance, counts, status, order);
    }
    note_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_arcs_estimate(const lyon_arc* arcs, uint32_t n, float tolerance,
                                 uint32_t* est, int num_sms, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    const uint32_t need = (n + 255) / 256;
    const uint32_t cap = (uint32_t)(num_sms > 0 ? num_sms : 1) * 8;
    arcs_estimate_kernel<<<need < cap ? need : cap, 256, 0, stream>>>(arcs, n, tolerance, est);
    note_launches(1);
    return cudaGetLastError();
}

}  // namespace lg
