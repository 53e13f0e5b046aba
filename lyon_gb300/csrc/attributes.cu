// attributes.cu — interpolation of custom endpoint attributes at output vertices, from the
// vertices' sources (lyon_vertex_source: an endpoint, or a point at t on the edge between two).
//   stroke: StrokeVertex::interpolated_attributes (crates/tessellation/src/stroke.rs:2728-2747),
//           one source per vertex;
//   fill:   FillVertex::interpolated_attributes (crates/tessellation/src/fill.rs:2208-2286), any
//           number of sources per vertex, averaged.
// One thread per vertex over a grid-stride loop; the attribute rows are gathered (consecutive
// vertices mostly share endpoints, so they are L2 hits). f32 operations in lyon's order (the
// library builds without contraction).
#include "kernels.h"

namespace lg {
namespace {

__device__ __forceinline__ bool source_ok(const lyon_vertex_source& s, uint64_t ne) {
    return s.from < ne && (s.to == LYON_NO_ENDPOINT || s.to < ne);
}

// The source's own attribute value i: the endpoint's, or a * (1 - t) + b * t.
__device__ __forceinline__ float source_value(const lyon_vertex_source& s, const float* attrs,
                                              uint32_t na, uint32_t i) {
    const float a = attrs[(uint64_t)s.from * na + i];
    if (s.to == LYON_NO_ENDPOINT) return a;
    const float b = attrs[(uint64_t)s.to * na + i];
    return a * (1.0f - s.t) + b * s.t;
}

__global__ void __launch_bounds__(256)
    interpolate_kernel(const lyon_vertex_source* __restrict__ src, uint64_t n,
                       const float* __restrict__ attrs, uint32_t na, uint64_t ne,
                       float* __restrict__ out) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += stride) {
        const lyon_vertex_source s = src[v];
        float* o = out + v * na;
        const bool ok = source_ok(s, ne);
        for (uint32_t i = 0; i < na; ++i)
            o[i] = ok ? source_value(s, attrs, na, i) : __int_as_float(0x7fc00000);
    }
}

__global__ void __launch_bounds__(256)
    interpolate_fill_kernel(const lyon_vertex_source* __restrict__ src,
                            const uint64_t* __restrict__ offsets, uint64_t n,
                            const float* __restrict__ attrs, uint32_t na, uint64_t ne,
                            float* __restrict__ out) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += stride) {
        const uint64_t k0 = offsets[v], k1 = offsets[v + 1];
        float* o = out + v * na;
        bool ok = k1 > k0;
        for (uint64_t k = k0; k < k1 && ok; ++k) ok = source_ok(src[k], ne);
        if (!ok) {
            for (uint32_t i = 0; i < na; ++i) o[i] = __int_as_float(0x7fc00000);
            continue;
        }
        // The sum runs over the sources in order, then one division by their number.
        const float div = (float)(k1 - k0);
        for (uint32_t i = 0; i < na; ++i) {
            float acc = source_value(src[k0], attrs, na, i);
            for (uint64_t k = k0 + 1; k < k1; ++k) acc = acc + source_value(src[k], attrs, na, i);
            o[i] = k1 - k0 > 1 ? acc / div : acc;
        }
    }
}

unsigned grid_for(uint64_t n, int num_sms) {
    const uint64_t need = (n + 255) / 256;
    const uint64_t cap = (uint64_t)(num_sms > 0 ? num_sms : 1) * 8;
    return (unsigned)(need < cap ? need : cap);
}

}  // namespace

cudaError_t launch_interpolate(const lyon_vertex_source* sources, uint64_t n,
                               const float* attributes, uint32_t num_attributes,
                               uint64_t num_endpoints, float* out, int num_sms,
                               cudaStream_t stream) {
    if (n == 0 || num_attributes == 0) return cudaSuccess;
    interpolate_kernel<<<grid_for(n, num_sms), 256, 0, stream>>>(sources, n, attributes,
                                                                 num_attributes, num_endpoints,
                                                                 out);
    note_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_interpolate_fill(const lyon_vertex_source* sources,
                                    const uint64_t* source_offsets, uint64_t n,
                                    const float* attributes, uint32_t num_attributes,
                                    uint64_t num_endpoints, float* out, int num_sms,
                                    cudaStream_t stream) {
    if (n == 0 || num_attributes == 0) return cudaSuccess;
    interpolate_fill_kernel<<<grid_for(n, num_sms), 256, 0, stream>>>(
        sources, source_offsets, n, attributes, num_attributes, num_endpoints, out);
    note_launches(1);
    return cudaGetLastError();
}

}  // namespace lg
