// kernels.h — launch interfaces between the C ABI layer (api.cu) and the kernels.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/lyon_gpu.h"

namespace lg {

// Kernel launches issued by this library in this process (every context and thread): each
// launch site notes its launches here.
void note_launches(uint32_t k);
uint64_t launches_total();

struct StrokeArgs {
    const uint8_t* verbs;
    const float* points;
    const uint32_t* verb_offsets;
    const uint32_t* point_offsets;
    uint32_t num_paths;
    const lyon_stroke_options* options;
    uint32_t num_options;
    const uint32_t* order;     // optional processing order (null: path index order)
    uint32_t* work_counter;    // zeroed before each launch
    // count pass outputs / emit pass inputs
    uint32_t* vtx_counts;
    uint32_t* idx_counts;
    int32_t* status;
    const uint64_t* vtx_offsets;
    const uint64_t* idx_offsets;
    float* vertices;
    void* indices;
    int index_bits;
    int index_mode;
    uint32_t vertex_offset;
    // Non-zero: `vertices` receives lyon_stroke_vertex records (position, normal, advancement,
    // side) instead of positions.
    int vertex_attrs;
    // Non-null: variable line width, one width factor per point of the batch (indexed like
    // `points`); the paths are stroked by the variable-width kernel (one thread per path).
    const float* widths;
    // Optional, per path: the first path of the request it belongs to. In LYON_INDEX_GLOBAL mode
    // ids then count from that path's first vertex (one VertexBuffers per request of a batch).
    const uint32_t* request_first;
    // Optional, with `order`: items [0, *item_split) of the order are stroked one path per warp,
    // the rest (short line-only paths) one path per thread, 32 per warp, once a warp finds no
    // warp items left; `seq_counter` (zeroed before each launch) hands out those.
    const uint32_t* item_split;
    uint32_t* seq_counter;
    // Non-zero: every path is stroked by lyon's sequential stepper, one path per thread, in both
    // passes (set by the custom-attribute calls; `widths` implies it). With `sources` the emit
    // pass writes each vertex's lyon_vertex_source next to it.
    int sequential;
    lyon_vertex_source* sources;
    uint32_t width_stride;  // floats from one point's width factor to the next's (0 means 1)
};

// Basic shapes (shapes.cu): `params` holds 4 floats per rectangle (min x, min y, max x, max y)
// or 3 per circle (center x, center y, radius).
struct ShapeArgs {
    int kind;  // LYON_SHAPE_RECTANGLE or LYON_SHAPE_CIRCLE
    const float* params;
    uint32_t n;
    const lyon_fill_options* options;
    uint32_t num_options;
    uint32_t* vtx_counts;
    uint32_t* idx_counts;
    int32_t* status;
    const uint64_t* vtx_offsets;
    const uint64_t* idx_offsets;
    float* vertices;
    void* indices;
    int index_bits;
    int index_mode;
    uint32_t vertex_offset;
};
cudaError_t launch_shapes(const ShapeArgs& args, bool emit, cudaStream_t stream);

int stroke_blocks_per_sm();
cudaError_t launch_stroke(const StrokeArgs& args, bool emit, int grid, cudaStream_t stream);
// The sequential stepper (stroke_seq.cu): variable line width and the vertex-source output.
cudaError_t launch_stroke_seq(const StrokeArgs& args, bool emit, int grid, cudaStream_t stream);
// StrokeVertex::interpolated_attributes over `n` vertex sources (attributes.cu).
cudaError_t launch_interpolate(const lyon_vertex_source* sources, uint64_t n,
                               const float* attributes, uint32_t num_attributes,
                               uint64_t num_endpoints, float* out, int num_sms,
                               cudaStream_t stream);
// FillVertex::interpolated_attributes over `n` vertices whose sources are
// sources[source_offsets[v] .. source_offsets[v + 1]) (attributes.cu).
cudaError_t launch_interpolate_fill(const lyon_vertex_source* sources,
                                    const uint64_t* source_offsets, uint64_t n,
                                    const float* attributes, uint32_t num_attributes,
                                    uint64_t num_endpoints, float* out, int num_sms,
                                    cudaStream_t stream);

// Hatching and dots (hatch.cu).
struct HatchArgs {
    const uint8_t* verbs;
    const float* points;
    const uint32_t* verb_offsets;
    const uint32_t* point_offsets;
    uint32_t num_paths;
    float tolerance;
    float c, s;    // cos / sin of the pattern angle
    float ci, si;  // cos / sin of its negation
    float uv_x, uv_y;
    float interval, column_interval;
    int compute_tangents;
    int dots;
    uint32_t* edge_bound;            // phase 0 output
    const uint64_t* scratch_offsets; // per path, in edges (num_paths + 1)
    uint64_t scratch_total;          // edges per scratch region (three regions)
    void* scratch;
    uint32_t* edge_count;            // phase 1 output
    uint32_t* counts;                // phase 1 output
    int32_t* status;                 // phase 1 output
    const uint64_t* out_offsets;     // phase 2 input
    const uint32_t* order;           // phases 1 and 2: paths largest first (null: index order)
    lyon_hatch_segment* segments;    // phase 2 output (hatches)
    lyon_dot* dot_out;               // phase 2 output (dots)
};
// phase 0: edge bounds, 1: build, sort and count, 2: emit.
cudaError_t launch_hatch(const HatchArgs& args, int phase, int num_sms, cudaStream_t stream);

// Arc flattening (arcs.cu): count pass (pts null: counts and status) or emit pass.
// Both passes take the arcs in `order` (null: index order).
cudaError_t launch_arcs(const lyon_arc* arcs, uint32_t n, float tolerance, uint32_t* counts,
                        int32_t* status, const uint64_t* offsets, float* pts, float* ts,
                        int num_sms, cudaStream_t stream, const uint32_t* order = nullptr);
// A rough per-arc step count, to order the count pass.
cudaError_t launch_arcs_estimate(const lyon_arc* arcs, uint32_t n, float tolerance,
                                 uint32_t* est, int num_sms, cudaStream_t stream);

// Exclusive scan of two u32 arrays into two u64 arrays (decoupled look-back), plus totals at
// out_a[n] / out_b[n]. `tile_state` holds 2 * num_tiles(n) u64 and `counter` one u32; both are
// reset by the call. `error` receives 1 if a look-back wait exceeded its bound.
__host__ __device__ size_t scan_tile_count(uint32_t n);
cudaError_t launch_scan_pairs(const uint32_t* a, const uint32_t* b, uint64_t* out_a,
                              uint64_t* out_b, uint32_t n, unsigned long long* tile_state,
                              uint32_t* counter, int* error, cudaStream_t stream);

// Per-path index-range check for LYON_INDEX_PER_PATH (geometry_builder.rs:338-350): a path whose
// last vertex id exceeds max_index fails with TOO_MANY_VERTICES and produces nothing.
cudaError_t launch_per_path_limit(uint32_t* vtx_counts, uint32_t* idx_counts, int32_t* status,
                                  uint32_t n, uint64_t vertex_offset, uint64_t max_index,
                                  uint32_t* failed, cudaStream_t stream);

cudaError_t launch_narrow_u64(const uint64_t* in, uint32_t* out, uint32_t n, cudaStream_t s);

// lyon's SVG path parser (svg.cu) on the device, one thread per string: the counting pass
// (verb/point counts, status, error position) or, with `write`, the writing pass at the scanned
// offsets.
cudaError_t launch_svg_parse(const char* text, const uint64_t* string_offsets, uint32_t n,
                             uint32_t num_attributes, long long stop_at, bool write,
                             uint32_t* verb_counts, uint32_t* point_counts, int32_t* status,
                             int32_t* error_line, int32_t* error_column,
                             const uint64_t* verb_offsets, const uint64_t* point_offsets,
                             uint8_t* verbs, float* points, float* widths, int num_sms,
                             cudaStream_t stream);

// Writes out_a[n], out_b[n] (the scan totals) and the two u32 words at `words` into `host_dst`
// (mapped pinned host memory) with a kernel, so that the read-back does not queue behind large
// device->host copies on the copy engines.
cudaError_t launch_read_totals(const uint64_t* a_total, const uint64_t* b_total,
                               const uint32_t* words, uint64_t* host_dst, cudaStream_t s);

// Processing order by class: paths with more than `big_points` points (0: none) first, then the
// other paths, then line-only paths of at most `short_points` points (0: none; at most
// CLASSIFY_MAX_SHORT_POINTS) by decreasing point count: the one-thread-per-path phase of the
// stroke kernel takes those. `path_class` holds one byte per path; `counters` 2 * (3 +
// short_points) + 1 words (bin sizes, placement cursors, then the first short item), reset here.
constexpr uint32_t CLASSIFY_MAX_SHORT_POINTS = 64;
constexpr uint32_t CLASSIFY_MAX_BINS = 3 + CLASSIFY_MAX_SHORT_POINTS;
constexpr uint32_t CLASSIFY_COUNTER_WORDS = 2 * CLASSIFY_MAX_BINS + 1;
cudaError_t launch_classify_paths(const uint8_t* verbs, const uint32_t* verb_offsets,
                                  const uint32_t* point_offsets, uint32_t n, uint32_t big_points,
                                  uint32_t short_points, uint8_t* path_class, uint32_t* order,
                                  uint32_t* counters, cudaStream_t s);

// Processing order by decreasing size (powers of two of the point count, largest first), for
// work queues whose last items should be the cheap ones. `cls` holds one byte per path,
// `counters` 2 * SIZE_ORDER_BINS words; both are scratch.
constexpr uint32_t SIZE_ORDER_BINS = 33;
// With `sizes`, the items' sizes are read from it instead of point_offsets differences.
cudaError_t launch_size_order(const uint32_t* point_offsets, uint32_t n, uint8_t* cls,
                              uint32_t* order, uint32_t* counters, cudaStream_t s,
                              const uint32_t* sizes = nullptr);

// Processing order for a batch: paths with more than `big_points` points first (their work can
// exceed the rest of a launch), then the others. `counters` holds two u32 and is reset here.
// Outputs do not depend on the order (offsets come from the scan by path index).
cudaError_t launch_big_first_order(const uint32_t* point_offsets, uint32_t n, uint32_t big_points,
                                   uint32_t* order, uint32_t* counters, cudaStream_t s);

}  // namespace lg
