/*
 * lyon_gpu.h — C ABI of the GB300 tessellation library (liblyon_gb300.so).
 *
 * The library implements lyon's tessellation hot path on the GPU:
 *   - curve flattening   (lyon_geom quadratic/cubic `for_each_flattened`),
 *   - StrokeTessellator  (fixed line width: miter, miter-clip, bevel and round joins,
 *                         butt, square and round caps),
 *   - FillTessellator    (even-odd and non-zero fill rules, holes, self-intersections).
 *
 * Every entry point below replaces one call a lyon user makes; each declaration cites the
 * reference interface (file:line inside the lyon repository) whose behaviour it reproduces.
 * Signatures use plain pointers and sizes only.
 *
 * Path layout ("lyon_path_batch") is lyon's own `Path` storage (crates/path/src/path.rs:75-79):
 * one verb byte per event and the endpoint/control points in order; `Close` stores the first
 * point of the sub-path again (crates/path/src/path.rs:534-542). A batch concatenates paths and
 * adds offset arrays.
 *
 * Vertex output is the `Positions` layout (crates/tessellation/src/geometry_builder.rs:403-415):
 * two f32 per vertex. Index output is u16 or u32, with lyon's `BuffersBuilder` semantics
 * (crates/tessellation/src/geometry_builder.rs:338-350): an index is the vertex's position in the
 * destination vertex buffer plus the builder's vertex offset.
 */
#ifndef LYON_GPU_H
#define LYON_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- Path verbs: same order as lyon's `Verb` (crates/path/src/path.rs:29-36). ------------- */
enum {
    LYON_VERB_LINE_TO = 0,
    LYON_VERB_QUADRATIC_TO = 1,
    LYON_VERB_CUBIC_TO = 2,
    LYON_VERB_BEGIN = 3,
    LYON_VERB_CLOSE = 4,
    LYON_VERB_END = 5
};

/* ---- Options (crates/path/src/lib.rs:170-281, crates/tessellation/src/lib.rs:315-537). ---- */
enum { LYON_CAP_BUTT = 0, LYON_CAP_SQUARE = 1, LYON_CAP_ROUND = 2 };
enum { LYON_JOIN_MITER = 0, LYON_JOIN_MITER_CLIP = 1, LYON_JOIN_ROUND = 2, LYON_JOIN_BEVEL = 3 };
enum { LYON_FILL_EVEN_ODD = 0, LYON_FILL_NON_ZERO = 1 };
enum { LYON_ORIENTATION_VERTICAL = 0, LYON_ORIENTATION_HORIZONTAL = 1 };

/* Mirrors `StrokeOptions` (crates/tessellation/src/lib.rs:315-433) for the fixed-width path.
 * Defaults (StrokeOptions::DEFAULT): butt caps, miter join, width 1, miter limit 4, tol 0.1. */
typedef struct lyon_stroke_options {
    int32_t start_cap;
    int32_t end_cap;
    int32_t line_join;
    float line_width;
    float miter_limit;
    float tolerance;
} lyon_stroke_options;

/* Mirrors `FillOptions` (crates/tessellation/src/lib.rs:445-537).
 * Defaults: tolerance 0.1, even-odd, vertical sweep, intersections handled. */
typedef struct lyon_fill_options {
    float tolerance;
    int32_t fill_rule;
    int32_t sweep_orientation;
    int32_t handle_intersections;
} lyon_fill_options;

/* ---- Status codes: mirror `TessellationError` (crates/tessellation/src/error.rs:1-142). --- */
enum {
    LYON_OK = 0,
    /* TessellationError::UnsupportedParamater(PositionIsNaN) */
    LYON_ERR_POSITION_IS_NAN = 1,
    /* TessellationError::UnsupportedParamater(ToleranceIsNaN) */
    LYON_ERR_TOLERANCE_IS_NAN = 2,
    /* TessellationError::GeometryBuilder(TooManyVertices) */
    LYON_ERR_TOO_MANY_VERTICES = 3,
    /* TessellationError::GeometryBuilder(InvalidVertex) */
    LYON_ERR_INVALID_VERTEX = 4,
    /* TessellationError::Internal(..): the fill sweep gave up (its retry also failed). */
    LYON_ERR_INTERNAL = 5,
    /* Library-level errors (no lyon counterpart). */
    LYON_ERR_INVALID_ARGUMENT = 100,
    LYON_ERR_CUDA = 101,
    LYON_ERR_OUT_OF_MEMORY = 102,
    LYON_ERR_CAPACITY = 103,      /* a caller-provided buffer or a fixed device arena is too small */
    LYON_ERR_UNSUPPORTED = 104    /* an option this build does not implement */
};

/* Index output modes for batched calls. */
enum {
    /* Each path is appended to one shared VertexBuffers, as if `tessellate_path` were called
     * on every path in order with the same BuffersBuilder: indices are absolute positions in the
     * concatenated vertex buffer (plus `vertex_offset`). A path whose last index would exceed the
     * index type's maximum fails with TOO_MANY_VERTICES and is rolled back (abort_geometry), and
     * later paths continue from the rolled-back length. */
    LYON_INDEX_GLOBAL = 0,
    /* Each path has its own VertexBuffers: indices start at 0 (plus `vertex_offset`) per path. */
    LYON_INDEX_PER_PATH = 1
};

/* A batch of paths in lyon's `Path` layout. All pointers are either all host or all device,
 * as each entry point states. */
typedef struct lyon_path_batch {
    const uint8_t* verbs;          /* LYON_VERB_* per event, all paths concatenated */
    const float* points;           /* x, y pairs, all paths concatenated */
    const uint32_t* verb_offsets;  /* num_paths + 1 entries, into verbs */
    const uint32_t* point_offsets; /* num_paths + 1 entries, into points (in points, not floats) */
    uint32_t num_paths;
} lyon_path_batch;

typedef struct lyon_gpu_context lyon_gpu_context;

/* Creates a context on the given CUDA device: a stream, device scratch arenas that grow on
 * demand, and pinned host staging buffers for the single-path entry points. Returns NULL on
 * failure. The equivalent of constructing a `StrokeTessellator`/`FillTessellator`
 * (crates/tessellation/src/stroke.rs:108-118, crates/tessellation/src/fill.rs:523-575),
 * which own their scratch allocations and are reused across calls. */
lyon_gpu_context* lyon_gpu_create(int device);
void lyon_gpu_destroy(lyon_gpu_context* ctx);
/* The CUDA stream (cudaStream_t) the context launches on. */
void* lyon_gpu_stream(lyon_gpu_context* ctx);
/* Last error message recorded on the context (never NULL). */
const char* lyon_gpu_last_error(lyon_gpu_context* ctx);

/* ----------------------------------------------------------------------------------------- */
/* Single-path drop-ins (host memory in, host memory out, synchronous).                       */
/* ----------------------------------------------------------------------------------------- */

/* Result of a single-path call: views into the context's pinned staging buffers, valid until
 * the next call on the same context. Indices are u16 or u32 as requested, already offset by
 * `index_base`. On failure num_vertices == num_indices == 0 (abort_geometry). */
typedef struct lyon_gpu_result {
    const float* vertices;
    uint32_t num_vertices;
    const void* indices;
    uint32_t num_indices;
    int32_t status;
} lyon_gpu_result;

/* StrokeTessellator::tessellate_path(path, options, &mut BuffersBuilder)
 * (crates/tessellation/src/stroke.rs:164-177), fixed line width, `Positions` vertices.
 * `index_base` is the id of the first vertex the builder would hand out
 * (vertices.len() + vertex_offset, crates/tessellation/src/geometry_builder.rs:338-350);
 * `index_bits` is 16 or 32 and selects u16/u32 indices and MaxIndex
 * (crates/tessellation/src/geometry_builder.rs:562-603). Returns the status code. */
int lyon_gpu_stroke_path(lyon_gpu_context* ctx, const uint8_t* verbs, uint32_t num_verbs,
                         const float* points, uint32_t num_points,
                         const lyon_stroke_options* options, int index_bits, uint32_t index_base,
                         lyon_gpu_result* result);

/* One stroke output vertex with the attributes lyon's StrokeVertex hands a vertex constructor
 * (crates/tessellation/src/stroke.rs:2667-2720): position(), normal() (the length that inflates
 * the stroke by 1 on each side, not a unit vector at miters), advancement() (distance along the
 * path, carried from one sub-path to the next as lyon does) and side() (0 = Side::Positive,
 * 1 = Side::Negative, crates/path/src/lib.rs:224-227). 24 bytes. */
typedef struct lyon_stroke_vertex {
    float x, y;
    float normal_x, normal_y;
    float advancement;
    uint32_t side;
} lyon_stroke_vertex;

/* lyon_gpu_stroke_path with a BuffersBuilder whose vertex constructor reads the StrokeVertex
 * attributes: `result->vertices` points at `num_vertices` lyon_stroke_vertex records (cast the
 * pointer). Indices, statuses and positions are those of lyon_gpu_stroke_path. */
int lyon_gpu_stroke_path_attributes(lyon_gpu_context* ctx, const uint8_t* verbs,
                                    uint32_t num_verbs, const float* points, uint32_t num_points,
                                    const lyon_stroke_options* options, int index_bits,
                                    uint32_t index_base, lyon_gpu_result* result);

/* lyon_gpu_stroke_path with StrokeOptions::variable_line_width: `widths` (host memory) holds one
 * width factor per point, as for lyon_gpu_stroke_paths_variable_width. `vertex_attributes`
 * non-zero makes `result->vertices` point at lyon_stroke_vertex records. */
int lyon_gpu_stroke_path_variable_width(lyon_gpu_context* ctx, const uint8_t* verbs,
                                        uint32_t num_verbs, const float* points,
                                        uint32_t num_points, const float* widths,
                                        const lyon_stroke_options* options, int index_bits,
                                        uint32_t index_base, int vertex_attributes,
                                        lyon_gpu_result* result);

/* FillTessellator::tessellate_path(path, options, &mut BuffersBuilder)
 * (crates/tessellation/src/fill.rs:628-641), `Positions` vertices. Same conventions as above. */
int lyon_gpu_fill_path(lyon_gpu_context* ctx, const uint8_t* verbs, uint32_t num_verbs,
                       const float* points, uint32_t num_points, const lyon_fill_options* options,
                       int index_bits, uint32_t index_base, lyon_gpu_result* result);

/* ----------------------------------------------------------------------------------------- */
/* Batched, device-resident entry points (the `tessellate_paths` hot path).                   */
/* All pointers are device pointers; work is queued on the context's stream and the call      */
/* returns after the last kernel is queued, unless stated otherwise.                          */
/* ----------------------------------------------------------------------------------------- */

/* Output of a batched call: device buffers owned by the context (grown on demand, reused by
 * the next batched call of the same kind), plus host-visible totals. */
typedef struct lyon_gpu_batch_output {
    float* vertices;            /* device, 2 * total_vertices floats */
    void* indices;              /* device, total_indices u16/u32 */
    uint64_t* vertex_offsets;   /* device, num_paths + 1: first vertex of each path (exclusive
                                   scan of the per-path vertex counts; the last entry is the total) */
    uint64_t* index_offsets;    /* device, num_paths + 1: same for indices */
    int32_t* status;            /* device, one status per path */
    uint64_t total_vertices;
    uint64_t total_indices;
    uint32_t num_failed_paths;  /* paths whose status is not LYON_OK */
} lyon_gpu_batch_output;

/* Batched `StrokeTessellator::tessellate_path` over every path of `batch`
 * (crates/tessellation/src/stroke.rs:164-177 applied path by path; no lyon counterpart for the
 * batching itself). `options` points to `num_options` records in device memory: 1 record shared
 * by all paths, or one per path. `index_mode` is LYON_INDEX_GLOBAL or LYON_INDEX_PER_PATH.
 * Runs the count kernel, the look-back scan and the emit kernel; synchronises once to read the
 * totals (needed to size the output). */
int lyon_gpu_stroke_paths(lyon_gpu_context* ctx, const lyon_path_batch* batch,
                          const lyon_stroke_options* options, uint32_t num_options,
                          int index_bits, int index_mode, uint32_t vertex_offset,
                          lyon_gpu_batch_output* out);

/* The plain per-path GPU method, the baseline the batched call is measured against: paths
 * [first, first + count) of `batch` (device memory) each run through their own batched call of
 * one path (count kernel, look-back scan, one host wait for the totals, emit kernel), one after
 * the other, into the context's output buffers (per-path indices). `*total_vertices` receives
 * the sum of their vertex counts. No lyon counterpart: lyon strokes one path per
 * `tessellate_path` call (crates/tessellation/src/stroke.rs:164-177), and this is that call
 * pattern on the GPU. */
int lyon_gpu_stroke_paths_each(lyon_gpu_context* ctx, const lyon_path_batch* batch,
                               const lyon_stroke_options* options, uint32_t num_options,
                               int index_bits, uint32_t first, uint32_t count,
                               uint64_t* total_vertices);

/* lyon_gpu_stroke_paths with lyon_stroke_vertex records (position, normal, advancement, side):
 * `out->vertices` points at `total_vertices` records in device memory (cast the pointer); the
 * rest of `out` is as for lyon_gpu_stroke_paths. */
int lyon_gpu_stroke_paths_attributes(lyon_gpu_context* ctx, const lyon_path_batch* batch,
                                     const lyon_stroke_options* options, uint32_t num_options,
                                     int index_bits, int index_mode, uint32_t vertex_offset,
                                     lyon_gpu_batch_output* out);

/* StrokeTessellator::tessellate_path with StrokeOptions::variable_line_width
 * (crates/tessellation/src/stroke.rs:646-767, 954-1067, 1380-1512): the path's endpoints carry a
 * width factor and an endpoint's line width is options.line_width times its factor (linearly
 * interpolated along curves). `widths` (device memory) holds one factor per point of the batch,
 * indexed like `points`; entries of control points and of Close's repeated point are not read.
 * `vertex_attributes` non-zero writes lyon_stroke_vertex records instead of positions. The rest
 * is as for lyon_gpu_stroke_paths. Each path is stroked by one thread. */
int lyon_gpu_stroke_paths_variable_width(lyon_gpu_context* ctx, const lyon_path_batch* batch,
                                         const float* widths,
                                         const lyon_stroke_options* options,
                                         uint32_t num_options, int index_bits, int index_mode,
                                         uint32_t vertex_offset, int vertex_attributes,
                                         lyon_gpu_batch_output* out);

/* ---- Custom endpoint attributes: vertex sources and interpolated attributes ---------------- */

/* VertexSource (crates/tessellation/src/lib.rs:282-291), what StrokeVertex::source returns
 * (crates/tessellation/src/stroke.rs:2719-2722): the path endpoint a vertex was made for
 * (`to` == LYON_NO_ENDPOINT: Endpoint { id: from }) or a point at parameter `t` of the curve
 * between two endpoints (Edge { from, to, t }). Endpoint ids index the batch's point array (for a
 * one-path call: the path's, which are lyon's EndpointId values for a Path built without
 * attributes). 12 bytes. */
#define LYON_NO_ENDPOINT 0xFFFFFFFFu
typedef struct lyon_vertex_source {
    uint32_t from;
    uint32_t to;
    float t;
} lyon_vertex_source;

/* The per-vertex outputs of lyon_gpu_stroke_paths_custom, in device memory owned by the context
 * (valid until its next call). */
typedef struct lyon_gpu_custom_output {
    const lyon_vertex_source* sources; /* total_vertices records */
    const float* attributes;           /* num_attributes floats per vertex, NULL when none */
} lyon_gpu_custom_output;

/* StrokeTessellator::tessellate_path for paths that carry custom endpoint attributes
 * (crates/tessellation/src/stroke.rs:164-177 taking its `path.num_attributes() > 0` branch:
 * tessellate_with_ids, :641-652), with a vertex constructor that reads StrokeVertex::source and
 * StrokeVertex::interpolated_attributes (:2719-2747). `attributes` (device memory) holds
 * `num_attributes` floats per point of the batch, indexed like `points` (entries of control points
 * and of Close's repeated point are not read); `width_attribute` is
 * StrokeOptions::variable_line_width: -1 for a fixed line width, else the index of the attribute
 * that scales options.line_width. Writes positions, or lyon_stroke_vertex records when
 * `vertex_attributes` is non-zero, to `out` as lyon_gpu_stroke_paths does, and each vertex's
 * source and interpolated attributes to `custom`. The output pass strokes each path on one
 * thread with lyon's sequential stepper (with a variable width, the count pass too). */
int lyon_gpu_stroke_paths_custom(lyon_gpu_context* ctx, const lyon_path_batch* batch,
                                 const float* attributes, uint32_t num_attributes,
                                 int32_t width_attribute, const lyon_stroke_options* options,
                                 uint32_t num_options, int index_bits, int index_mode,
                                 uint32_t vertex_offset, int vertex_attributes,
                                 lyon_gpu_batch_output* out, lyon_gpu_custom_output* custom);

/* StrokeVertex::interpolated_attributes (crates/tessellation/src/stroke.rs:2728-2747) over many
 * vertices (device memory, context's stream): out[v * num_attributes + i] is
 * attributes[from * num_attributes + i] for an endpoint source and a * (1 - t) + b * t (f32, in
 * that order) for an edge. A source whose ids are not below `num_endpoints` gives NaN. */
int lyon_gpu_interpolate_attributes(lyon_gpu_context* ctx, const lyon_vertex_source* sources,
                                    uint64_t num_vertices, const float* attributes,
                                    uint32_t num_attributes, uint64_t num_endpoints, float* out);

/* One path with custom attributes (host memory in and out): lyon_gpu_stroke_paths_custom on a
 * one-path batch. `result` is as for lyon_gpu_stroke_path (records when `vertex_attributes`);
 * `*sources` and `*vertex_attribute_values` (num_attributes floats per vertex) point at host
 * memory valid until the next call on the context. */
int lyon_gpu_stroke_path_custom(lyon_gpu_context* ctx, const uint8_t* verbs, uint32_t num_verbs,
                                const float* points, uint32_t num_points,
                                const float* attributes, uint32_t num_attributes,
                                int32_t width_attribute, const lyon_stroke_options* options,
                                int index_bits, uint32_t index_base, int vertex_attributes,
                                lyon_gpu_result* result, const lyon_vertex_source** sources,
                                const float** vertex_attribute_values);

/* The per-vertex outputs of lyon_gpu_fill_paths_custom, in device memory owned by the context
 * (valid until its next call). A fill vertex has one source per edge event at its position
 * (FillVertex::sources, crates/tessellation/src/fill.rs:2172-2178, 2294-2337): vertex v's sources
 * are sources[source_offsets[v] .. source_offsets[v + 1]). */
typedef struct lyon_gpu_fill_custom_output {
    const lyon_vertex_source* sources;  /* total_sources records, in vertex order */
    const uint64_t* source_offsets;     /* total_vertices + 1 entries */
    uint64_t total_sources;
    const float* attributes;            /* num_attributes floats per vertex, NULL when none */
} lyon_gpu_fill_custom_output;

/* FillTessellator::tessellate_path for paths that carry custom endpoint attributes
 * (crates/tessellation/src/fill.rs:628-641 taking its `path.num_attributes() > 0` branch:
 * tessellate_with_ids, event_queue.rs:553-630), with a vertex constructor that reads
 * FillVertex::sources and FillVertex::interpolated_attributes (fill.rs:2172-2286).
 * `attributes` (device memory) holds `num_attributes` floats per point of the batch, indexed
 * like `points` (may be NULL when num_attributes is 0). Writes positions and indices to `out` as
 * lyon_gpu_fill_paths does, and every vertex's sources and interpolated attributes to `custom`.
 * Note lyon's convention for a curve flattened downwards from its end: its sources' t runs from
 * the curve's `to` end while from/to stay the curve's own endpoints. */
int lyon_gpu_fill_paths_custom(lyon_gpu_context* ctx, const lyon_path_batch* batch,
                               const float* attributes, uint32_t num_attributes,
                               const lyon_fill_options* options, uint32_t num_options,
                               int index_bits, int index_mode, uint32_t vertex_offset,
                               lyon_gpu_batch_output* out, lyon_gpu_fill_custom_output* custom);

/* FillVertex::interpolated_attributes (crates/tessellation/src/fill.rs:2208-2286) over many
 * vertices (device memory, context's stream): the first source's attributes (the endpoint's, or
 * a * (1 - t) + b * t), each further source's added in order, then a division by the number of
 * sources when there are several. A vertex with an id not below `num_endpoints`, or without
 * sources, gives NaN. */
int lyon_gpu_interpolate_fill_attributes(lyon_gpu_context* ctx,
                                         const lyon_vertex_source* sources,
                                         const uint64_t* source_offsets, uint64_t num_vertices,
                                         const float* attributes, uint32_t num_attributes,
                                         uint64_t num_endpoints, float* out);

/* One path with custom attributes (host memory in and out): lyon_gpu_fill_paths_custom on a
 * one-path batch. `*sources`, `*source_offsets` (num_vertices + 1 entries) and
 * `*vertex_attribute_values` point at host memory valid until the next call on the context. */
int lyon_gpu_fill_path_custom(lyon_gpu_context* ctx, const uint8_t* verbs, uint32_t num_verbs,
                              const float* points, uint32_t num_points, const float* attributes,
                              uint32_t num_attributes, const lyon_fill_options* options,
                              int index_bits, uint32_t index_base, lyon_gpu_result* result,
                              const lyon_vertex_source** sources,
                              const uint64_t** source_offsets,
                              const float** vertex_attribute_values);

/* Basic shapes: FillTessellator::tessellate_rectangle and tessellate_circle
 * (crates/tessellation/src/fill.rs:654-673 with crates/tessellation/src/basic_shapes.rs:12-124),
 * which fill without the sweep, over a batch of shapes. `params` (device memory) holds 4 floats
 * per rectangle (min x, min y, max x, max y) or 3 per circle (center x, center y, radius);
 * `options` 1 shared record or one per shape (circles read the tolerance). Each shape is one
 * "path" of `out` (per-shape offsets, statuses, index modes as for lyon_gpu_fill_paths). A circle
 * that would need more than 2^20 bisections per quarter fails with LYON_ERR_UNSUPPORTED. */
enum { LYON_SHAPE_RECTANGLE = 0, LYON_SHAPE_CIRCLE = 1 };
int lyon_gpu_fill_shapes(lyon_gpu_context* ctx, int shape_kind, const float* params,
                         uint32_t num_shapes, const lyon_fill_options* options,
                         uint32_t num_options, int index_bits, int index_mode,
                         uint32_t vertex_offset, lyon_gpu_batch_output* out);

/* ---- Sizing and emitting separately (caller-allocated outputs) ---------------------------- */

/* The sizing half of lyon_gpu_stroke_paths / lyon_gpu_fill_paths (`kind`: LYON_KIND_STROKE or
 * LYON_KIND_FILL, declared with the serving loop below): the count pass and
 * the scan, then one synchronisation. `*total_vertices`, `*total_indices` and
 * `*num_failed_paths` receive the batch's totals so that the caller can allocate the outputs;
 * per-path counts, offsets and statuses stay in the context for lyon_gpu_emit_into. */
int lyon_gpu_query_sizes(lyon_gpu_context* ctx, int kind, const lyon_path_batch* batch,
                         const void* options, uint32_t num_options, int index_bits,
                         int index_mode, uint32_t vertex_offset, uint64_t* total_vertices,
                         uint64_t* total_indices, uint32_t* num_failed_paths);

/* The emitting half, after lyon_gpu_query_sizes with the same batch and arguments and no other
 * batched call on the context in between: writes the vertices (2 floats each) and indices into
 * the caller's device buffers, which hold at least the queried totals. `out` receives the
 * caller's buffers with the context's per-path offsets and statuses and the totals. Returns
 * LYON_ERR_INVALID_ARGUMENT when no matching query precedes it. */
int lyon_gpu_emit_into(lyon_gpu_context* ctx, int kind, const lyon_path_batch* batch,
                       const void* options, uint32_t num_options, int index_bits, int index_mode,
                       uint32_t vertex_offset, float* vertices, void* indices,
                       lyon_gpu_batch_output* out);

/* Largest batch lyon_gpu_stroke_paths_noalloc accepts (its fixed scratch holds this many paths). */
#define LYON_NOALLOC_MAX_PATHS 262144u

/* lyon_gpu_stroke_paths for callers that cannot allocate device memory: a plugin handed device
 * buffers by a host application that owns every GPU allocation, or code running under a memory
 * pool or budget that forbids cudaMalloc. This entry point has no counterpart in the reference
 * (lyon allocates its own buffers); it is an addition of this library.
 *
 * It allocates nothing: no cudaMalloc, cudaFree or allocating library call, and no context.
 * The batch and options are device memory; the caller also passes every output in device
 * memory: `vertices` (2 floats per vertex, `vertex_capacity` vertices), `indices`
 * (`index_capacity` u16/u32), `vertex_offsets` and `index_offsets` (num_paths + 1 u64 each) and
 * `status` (num_paths i32). The pipeline's scratch is a fixed array of about 2 MiB inside the
 * library, held by every GPU that loads it until the process exits; batches of more than
 * LYON_NOALLOC_MAX_PATHS paths are rejected with LYON_ERR_CAPACITY and a message. When the
 * outputs are too small the call returns LYON_ERR_CAPACITY with *total_vertices /
 * *total_indices set to the sizes needed and writes no vertices or indices.
 *
 * Runs on the calling thread's current device, on `stream` (a cudaStream_t; NULL is the default
 * stream). The first call on a device resolves the scratch array's address for that device;
 * make that first call before capturing any stream into a CUDA graph. Every call on a device
 * shares the one scratch array and it keeps the previous call's contents: calls whose GPU work
 * overlaps (other streams, other threads) race and give wrong results. The call synchronises
 * `stream` once to read the totals; the emit kernel is still running when it returns.
 * `error_text` (optional, `error_text_len` bytes) receives a message on failure. */
int lyon_gpu_stroke_paths_noalloc(const lyon_path_batch* batch,
                                  const lyon_stroke_options* options, uint32_t num_options,
                                  int index_bits, int index_mode, uint32_t vertex_offset,
                                  float* vertices, uint64_t vertex_capacity, void* indices,
                                  uint64_t index_capacity, uint64_t* vertex_offsets,
                                  uint64_t* index_offsets, int32_t* status,
                                  uint64_t* total_vertices, uint64_t* total_indices,
                                  uint32_t* num_failed_paths, void* stream, char* error_text,
                                  size_t error_text_len);

/* Batched `FillTessellator::tessellate_path` (crates/tessellation/src/fill.rs:628-641 applied
 * path by path). Same conventions as lyon_gpu_stroke_paths. */
int lyon_gpu_fill_paths(lyon_gpu_context* ctx, const lyon_path_batch* batch,
                        const lyon_fill_options* options, uint32_t num_options, int index_bits,
                        int index_mode, uint32_t vertex_offset, lyon_gpu_batch_output* out);

/* Per-segment flattened point counts, as computed by `flattened_segments_wang` and the
 * `to_u32` truncation of `for_each_flattened` (crates/geom/src/quadratic_bezier.rs:337-359,
 * 943-974; crates/geom/src/cubic_bezier.rs:563-583, 1369-1403). One u32 per verb: lines give 1,
 * quadratics and cubics their flattened segment count, Begin/Close/End give 0. Device pointers. */
int lyon_gpu_flatten_counts(lyon_gpu_context* ctx, const lyon_path_batch* batch, float tolerance,
                            uint32_t* counts);

/* `path.iter().flattened(tolerance)` (crates/path/src/iterator.rs:125-215) for every path:
 * writes the flattened polyline points (the `to` point of every Line event, in event order) and
 * per-verb offsets into `out_points`. `out_offsets` has total_verbs + 1 entries (exclusive scan
 * of the per-verb counts). The output buffers are owned by the context (device pointers). */
int lyon_gpu_flatten_paths(lyon_gpu_context* ctx, const lyon_path_batch* batch, float tolerance,
                           float** out_points, uint32_t** out_offsets, uint64_t* total_points);

/* lyon_geom::Arc (crates/geom/src/arc.rs:21-28): an elliptic arc, angles in radians. 28 bytes. */
typedef struct lyon_arc {
    float center_x, center_y;
    float radius_x, radius_y;
    float start_angle, sweep_angle, x_rotation;
} lyon_arc;

/* Arcs that need more segments than this fail with LYON_ERR_UNSUPPORTED. */
#define LYON_MAX_ARC_SEGMENTS 4194304u

/* Output of lyon_gpu_flatten_arcs: device memory owned by the context (valid until its next
 * call). Arc i's points are points[offsets[i] .. offsets[i + 1]): its start point (t = 0), then
 * the end point of every segment with that segment's t1. */
typedef struct lyon_gpu_arc_output {
    const float* points;      /* 2 floats per point */
    const float* t;           /* one per point */
    const uint64_t* offsets;  /* num_arcs + 1 entries */
    const int32_t* status;    /* per arc: LYON_OK or LYON_ERR_UNSUPPORTED */
    uint64_t total_points;
} lyon_gpu_arc_output;

/* Arc::for_each_flattened_with_t (crates/geom/src/arc.rs:339-367, flattening_step :369-389) for
 * `num_arcs` arcs in device memory, one tolerance for all. cos, sin and acos are evaluated in f64
 * and rounded once (lyon's f32 libm results may differ in the last bit). Synchronises once to
 * size the output. */
int lyon_gpu_flatten_arcs(lyon_gpu_context* ctx, const lyon_arc* arcs, uint32_t num_arcs,
                          float tolerance, lyon_gpu_arc_output* out);

/* ---- Hatching and dots (lyon_algorithms::hatching, crates/algorithms/src/hatching.rs) ------- */

/* HatchingOptions / DotOptions (hatching.rs:44-179) with the regular patterns' intervals
 * (RegularHatchingPattern::interval, RegularDotPattern::row_interval / column_interval,
 * hatching.rs:640-675). */
typedef struct lyon_hatching_options {
    float tolerance;
    float angle;             /* radians */
    float uv_origin_x, uv_origin_y;
    float interval;          /* distance between rows (hatches), row_interval (dots) */
    float column_interval;   /* dots: distance between dots in a row */
    int32_t compute_tangents;  /* hatches only */
} lyon_hatching_options;

/* HatchSegment (hatching.rs:181-205): endpoints a (left) and b (right) with the outline's
 * tangent there (NaN when tangents are not computed) and their u; row index and v. 48 bytes. */
typedef struct lyon_hatch_segment {
    float a_x, a_y, a_tangent_x, a_tangent_y, a_u;
    float b_x, b_y, b_tangent_x, b_tangent_y, b_u;
    uint32_t row;
    float v;
} lyon_hatch_segment;

/* Dot (hatching.rs:216-227). 24 bytes. */
typedef struct lyon_dot {
    float x, y, u, v;
    uint32_t column, row;
} lyon_dot;

/* A path needing more rows than this, or more dots, fails with LYON_ERR_UNSUPPORTED (lyon keeps
 * looping, e.g. when the interval is too small to move the scan line). */
#define LYON_MAX_HATCH_ROWS 16777216u
#define LYON_MAX_HATCH_DOTS 67108864u

/* Output of lyon_gpu_hatch_paths / lyon_gpu_dot_paths, device memory owned by the context
 * (valid until its next call). Path i's records are [offsets[i], offsets[i + 1]). */
typedef struct lyon_gpu_hatch_output {
    const lyon_hatch_segment* segments;  /* hatches */
    const lyon_dot* dots;                /* dots */
    const uint64_t* offsets;             /* num_paths + 1 */
    const int32_t* status;               /* per path */
    uint64_t total;
} lyon_gpu_hatch_output;

/* Hatcher::hatch_path with a RegularHatchingPattern (hatching.rs:276-347, 374-428, 464-577)
 * for every path of `batch` (device memory), `options` in host memory. A path without edges
 * produces nothing (lyon panics on it). */
int lyon_gpu_hatch_paths(lyon_gpu_context* ctx, const lyon_path_batch* batch,
                         const lyon_hatching_options* options, lyon_gpu_hatch_output* out);

/* Hatcher::dot_path with a RegularDotPattern (hatching.rs:286-298, 349-372, 671-722). */
int lyon_gpu_dot_paths(lyon_gpu_context* ctx, const lyon_path_batch* batch,
                       const lyon_hatching_options* options, lyon_gpu_hatch_output* out);

/* Batched stroke with HOST buffers (the end-to-end form of lyon_gpu_stroke_paths): the batch
 * and options live in host memory, outputs are written to host memory. The call processes the
 * paths in chunks, overlapping each chunk's host->device copy, kernels and device->host copy with
 * its neighbours', and returns when every output byte is on the host (pinned host buffers let
 * the copies run at the link's full rate). `vertices`/`indices` must
 * hold `vertex_capacity` vertices and `index_capacity` indices; if they are too small the call
 * returns LYON_ERR_CAPACITY after setting *total_vertices / *total_indices to the sizes needed.
 * `status` (host, num_paths entries) receives the per-path status and may be NULL.
 * Index semantics are those of lyon_gpu_stroke_paths. No lyon counterpart (batching). */
int lyon_gpu_stroke_paths_host(lyon_gpu_context* ctx, const lyon_path_batch* batch,
                               const lyon_stroke_options* options, uint32_t num_options,
                               int index_bits, int index_mode, uint32_t vertex_offset,
                               float* vertices, uint64_t vertex_capacity, void* indices,
                               uint64_t index_capacity, int32_t* status,
                               uint64_t* total_vertices, uint64_t* total_indices);

/* Host memory for the host-buffer calls: page-locked (registered with CUDA, so copies run
 * asynchronously) and backed by transparent huge pages where the system allows them, so that
 * the device's address translation covers a large buffer with few entries. Returns NULL on
 * failure; free with lyon_gpu_host_free. On the virtual machines measured (GB300, 64 KB base
 * pages), a 40-52 GB buffer from here took the device's copies at 190-192 GB/s in some
 * allocations and 22-93 GB/s in others, and ordinary pinned memory at 57-93 GB/s: the rate
 * follows where the allocation lands in the machine's memory, which the process does not
 * control. */
void* lyon_gpu_host_alloc(size_t bytes);
int lyon_gpu_host_free(void* ptr);

/* Batched fill with host buffers; same conventions as lyon_gpu_stroke_paths_host. */
int lyon_gpu_fill_paths_host(lyon_gpu_context* ctx, const lyon_path_batch* batch,
                             const lyon_fill_options* options, uint32_t num_options,
                             int index_bits, int index_mode, uint32_t vertex_offset,
                             float* vertices, uint64_t vertex_capacity, void* indices,
                             uint64_t index_capacity, int32_t* status, uint64_t* total_vertices,
                             uint64_t* total_indices);

/* Kernel timing: when enabled, batched calls record CUDA events around their count, scan and
 * emit phases on the context's stream; lyon_gpu_last_timings returns the durations (ms) of the
 * last batched call: [0] count kernel, [1] scan (+ index-range check), [2] emit kernel,
 * [3] whole call. */
void lyon_gpu_set_timing(lyon_gpu_context* ctx, int enabled);
int lyon_gpu_last_timings(lyon_gpu_context* ctx, float* ms4);

/* ----------------------------------------------------------------------------------------- */
/* Serving loop. No lyon counterpart: lyon is a library called once per path; this is the    */
/* runtime that turns a stream of tessellation requests into batched launches.               */
/* ----------------------------------------------------------------------------------------- */

enum { LYON_KIND_STROKE = 0, LYON_KIND_FILL = 1 };

typedef struct lyon_srv lyon_srv;

typedef struct lyon_srv_config {
    int device;
    uint32_t num_workers;          /* batches in flight at once, each on its own stream; 0 -> 2.
                                      With stroke workers, these take fill requests only. */
    uint32_t max_batch_paths;      /* most paths coalesced into one launch; 0 -> 65536 */
    uint64_t device_budget_bytes;  /* device memory for batches and resident outputs; 0 -> 40 GB.
                                      A request that does not fit waits until released outputs
                                      free enough of it: release results as they complete (a
                                      caller that waits for requests in submission order while
                                      holding later results can wait forever) */
    uint32_t num_stroke_workers;   /* workers reserved for stroke requests, on streams of the
                                      device's highest priority and with one stroke block per SM,
                                      so that their launches start beside running fill sweeps
                                      instead of queueing behind them; 0 -> none (every worker
                                      takes both kinds, oldest request first) */
    uint32_t fill_blocks_per_sm;   /* fill sweep blocks per SM for each fill worker; 0 -> 8
                                      with stroke workers (half the library's default), else the
                                      library's default */
    uint32_t max_stroke_batch_paths; /* most paths per stroke launch; 0 -> max_batch_paths */
} lyon_srv_config;

/* A finished request. Its output stays on the device until lyon_srv_release. */
typedef struct lyon_srv_result {
    int status;                 /* LYON_OK, or the error that failed the request's batch */
    uint32_t num_paths;
    uint32_t num_failed_paths;  /* paths whose own status (path_status) is not LYON_OK */
    const float* vertices;      /* device: 2 floats per vertex */
    uint64_t num_vertices;
    const uint32_t* indices;    /* device: u32 ids counted from the request's first vertex, as
                                   lyon's BuffersBuilder over one VertexBuffers per request */
    uint64_t num_indices;
    const uint64_t* path_vertex_offsets;  /* device, num_paths + 1; subtract vertex_base */
    const uint64_t* path_index_offsets;   /* device, num_paths + 1; subtract index_base */
    const int32_t* path_status;           /* device, num_paths */
    uint64_t vertex_base, index_base;
    double queue_ms;    /* arrival to the start of its batch */
    double latency_ms;  /* arrival to its output being resident on the device */
} lyon_srv_result;

/* Starts the workers. Returns NULL on failure. */
lyon_srv* lyon_srv_create(const lyon_srv_config* config);
/* Stops the workers (after their current batch) and frees everything. */
void lyon_srv_destroy(lyon_srv* srv);
/* The configuration the loop runs with, defaults resolved (worker counts, fill_blocks_per_sm). */
int lyon_srv_get_config(const lyon_srv* srv, lyon_srv_config* out);
/* Queues a request: `batch` (host memory) stroked (LYON_KIND_STROKE, lyon_stroke_options) or
 * filled (LYON_KIND_FILL, lyon_fill_options) with 1 shared or num_paths option records. The
 * batch and options are read while the request runs: keep them valid until it completes.
 * Returns a ticket, or 0 for an invalid request. */
uint64_t lyon_srv_submit(lyon_srv* srv, int kind, const lyon_path_batch* batch,
                         const void* options, uint32_t num_options);
/* LYON_OK and *out filled when the request finished; 1 while it is pending. */
int lyon_srv_poll(lyon_srv* srv, uint64_t ticket, lyon_srv_result* out);
/* Blocks until the request finishes, then fills *out. */
int lyon_srv_wait(lyon_srv* srv, uint64_t ticket, lyon_srv_result* out);
/* Frees a finished request and its share of the device output. */
int lyon_srv_release(lyon_srv* srv, uint64_t ticket);

/* Open-loop load: requests drawn in turn from `items`, arriving as a Poisson process at
 * `rate_per_s` for `duration_s` seconds (arrival times from `seed`); each is released as soon as
 * it completes. Latency is measured from the scheduled arrival. `latencies_ms` (optional)
 * receives the per-request latencies in arrival order. */
typedef struct lyon_srv_load_item {
    int kind;
    lyon_path_batch batch;
    const void* options;
    uint32_t num_options;
} lyon_srv_load_item;

typedef struct lyon_srv_load_stats {
    uint32_t submitted, completed, failed;
    double offered_rate, elapsed_s, achieved_rate;
    uint64_t paths, vertices, indices;
    double p50_ms, p99_ms, p999_ms, max_ms;
    uint64_t batches;
    double mean_batch_paths;
} lyon_srv_load_stats;

int lyon_srv_run_load(lyon_srv* srv, const lyon_srv_load_item* items, uint32_t num_items,
                      double rate_per_s, double duration_s, uint64_t seed,
                      lyon_srv_load_stats* stats, double* latencies_ms, uint32_t latencies_cap);

/* ---- Coverage check (no lyon counterpart) -------------------------------------------------- */

/* Per-sample coverage of two tessellations of the same paths, for checking fill output: for each
 * of `num_paths` paths a `grid` x `grid` (at most 4096) grid of sample points spans the path's box
 * (`boxes`: x0, y0, x1, y1 per path; samples at x0 + (i + 0.5)(x1 - x0) / grid, likewise y). A
 * triangle covers a sample strictly inside it or on an edge that the tie rule gives it (edges
 * are evaluated from their lexicographically smaller end point; a counter-clockwise edge keeps
 * ties when it points down, or right when horizontal), so triangles sharing an edge cover each
 * sample on it once. Each tessellation is given as device arrays in the per-path layout:
 * vertices (2 floats each), u32 indices relative to the path's first vertex, and num_paths + 1
 * vertex and index offsets. `counts` (device, 3 u64 per path) receives the samples covered by A,
 * the samples covered by B and the samples whose coverage counts differ. Asynchronous on
 * `stream`. */
int lyon_gpu_coverage_compare(const float* boxes, uint32_t num_paths, uint32_t grid,
                              const float* vertices_a, const uint32_t* indices_a,
                              const uint64_t* vertex_offsets_a, const uint64_t* index_offsets_a,
                              const float* vertices_b, const uint32_t* indices_b,
                              const uint64_t* vertex_offsets_b, const uint64_t* index_offsets_b,
                              uint64_t* counts, void* stream);

/* ---- Stroke launch settings and autotuner (no lyon counterpart) ---------------------------- */

/* Runtime settings of the stroke kernels on a context. */
typedef struct lyon_gpu_stroke_tuning {
    uint32_t long_path_points;  /* paths with more points are scheduled first (so that no long
                                   path is left running alone at the end of a launch);
                                   0: path order. Default 1024. */
    uint32_t blocks_per_sm;     /* resident blocks per SM of the persistent grid; 0: as many as
                                   fit (default) */
    uint32_t short_path_points; /* line-only paths of at most this many points are stroked one
                                   path per thread instead of one per warp; 0: none, at most 64.
                                   Default 32. */
} lyon_gpu_stroke_tuning;

int lyon_gpu_set_stroke_tuning(lyon_gpu_context* ctx, const lyon_gpu_stroke_tuning* tuning);
int lyon_gpu_get_stroke_tuning(lyon_gpu_context* ctx, lyon_gpu_stroke_tuning* tuning);

/* Times the batched stroke (device buffers, u32 per-path indices) on the first `sample_paths`
 * paths of `batch` (0: all) for each candidate setting — long_path_points in {0, 256, 1024,
 * 8192} x blocks_per_sm in {as many as fit, 1} x short_path_points in {0, 32} — and keeps the
 * fastest on the context, so that later calls on paths of the same length distribution use it.
 * `best` receives the choice; `times_ms` (optional, 16 entries) the candidates' times in that
 * order (long_path_points varies fastest, short_path_points slowest); `num_candidates` the
 * count. Outputs of later calls do not depend on the settings. */
int lyon_gpu_autotune_stroke(lyon_gpu_context* ctx, const lyon_path_batch* batch,
                             const lyon_stroke_options* options, uint32_t num_options,
                             uint32_t sample_paths, lyon_gpu_stroke_tuning* best,
                             float* times_ms, uint32_t* num_candidates);

/* Runtime settings of the fill sweep on a context: lyon's sweep of one path runs on one thread
 * (a sweeper); a one-warp block holds up to 32 of them. */
typedef struct lyon_gpu_fill_tuning {
    uint32_t blocks_per_sm; /* sweep blocks per SM; 0: the default (16) */
    uint32_t lanes;         /* sweepers per block: 1 (a path owns its warp) to 32 (a warp shared by
                               32 paths, which share its instruction fetch and issue slots);
                               0: chosen per launch (1 below two paths per block, else up to 12) */
} lyon_gpu_fill_tuning;

int lyon_gpu_set_fill_tuning(lyon_gpu_context* ctx, const lyon_gpu_fill_tuning* tuning);
int lyon_gpu_get_fill_tuning(lyon_gpu_context* ctx, lyon_gpu_fill_tuning* tuning);

/* Times the batched fill (device buffers, u32 per-path indices) on the first `sample_paths`
 * paths of `batch` (0: all) for each candidate setting — blocks_per_sm in {16, 8} x lanes in
 * {1, 4, 8, 12, 16} — and keeps the fastest on the context, so that later calls on paths of the
 * same size distribution use it: the split between a path owning its warp and paths sharing one.
 * `best` receives the choice, `times_ms` (optional, 10 entries, lanes varying fastest) the
 * candidates' times, `num_candidates` the count. Outputs do not depend on the settings. The
 * sample must give each sweeper about as many paths as the whole batch will: with too few
 * paths per sweeper, a path owning its warp wins on the sample and loses on the batch. */
int lyon_gpu_autotune_fill(lyon_gpu_context* ctx, const lyon_path_batch* batch,
                           const lyon_fill_options* options, uint32_t num_options,
                           uint32_t sample_paths, lyon_gpu_fill_tuning* best, float* times_ms,
                           uint32_t* num_candidates);

/* Synchronise the context's stream. Returns LYON_OK or LYON_ERR_CUDA. */
int lyon_gpu_synchronize(lyon_gpu_context* ctx);

/* ---- SVG path data (no lyon_gpu counterpart; lyon_extra's PathParser) ----------------------- */

/* Parse errors of lyon's PathParser (crates/extra/src/parser.rs:14-33), per string. */
#define LYON_SVG_ERR_NUMBER 110          /* expected a number */
#define LYON_SVG_ERR_FLAG 111            /* expected an arc flag (0/1) */
#define LYON_SVG_ERR_COMMAND 112         /* invalid command */
#define LYON_SVG_ERR_MISSING_MOVE_TO 113 /* a command after Z other than M */

typedef struct lyon_svg_parse_options {
    uint32_t num_attributes; /* per endpoint (ParserOptions::num_attributes): 0, or 1 to read a
                                width factor per endpoint into `widths` */
    int32_t stop_at;         /* ParserOptions::stop_at: a character that ends parsing, or -1 */
    uint32_t num_threads;    /* host threads; 0: all */
} lyon_svg_parse_options;

/* PathParser::parse (crates/extra/src/parser.rs:154-490) of `num_strings` SVG path data strings
 * (UTF-8; string i is text[string_offsets[i] .. string_offsets[i + 1]]) into one host path batch:
 * path i gets verbs[verb_offsets[i] ..], points[point_offsets[i] ..] as lyon's Path builder
 * would hold them (arcs as quadratic beziers, crates/geom/src/arc.rs:58-138,668-703). `status[i]`
 * is LYON_OK or a LYON_SVG_ERR_* code with its line and column (as lyon reports them); a failed
 * string keeps what was built before the error, ended, as lyon's builder does. Call with null
 * output arrays (or too small capacities) to get *total_verbs / *total_points: the call then
 * returns LYON_ERR_CAPACITY. `widths` (optional, one float per point) receives the endpoint
 * attribute when options->num_attributes is 1 (control points get 0). All buffers are host
 * memory; the strings are parsed on the host's threads. */
int lyon_svg_parse_paths(const char* text, const uint64_t* string_offsets, uint32_t num_strings,
                         const lyon_svg_parse_options* options, uint8_t* verbs,
                         uint64_t verb_capacity, float* points, uint64_t point_capacity,
                         float* widths, uint32_t* verb_offsets, uint32_t* point_offsets,
                         int32_t* status, int32_t* error_line, int32_t* error_column,
                         uint64_t* total_verbs, uint64_t* total_points);

/* A batch parsed on the device by lyon_gpu_svg_parse_paths (device memory owned by the context
 * until its next lyon_gpu_svg_parse_paths call). */
typedef struct lyon_gpu_svg_output {
    lyon_path_batch batch;  /* verbs, points, verb_offsets / point_offsets (num_strings + 1) */
    float* widths;          /* one per point when num_attributes is 1, else NULL */
    int32_t* status;        /* per string: LYON_OK or a LYON_SVG_ERR_* code */
    int32_t* error_line;    /* per string */
    int32_t* error_column;  /* per string */
    uint64_t total_verbs;
    uint64_t total_points;
    uint32_t num_failed;    /* strings whose status is not LYON_OK */
} lyon_gpu_svg_output;

/* lyon_svg_parse_paths on the device: the same parser (PathParser::parse, crates/extra/src/
 * parser.rs:154-490) and the same output layout, statuses and error positions, with the strings
 * (`text`, `string_offsets`: device memory) parsed one per thread in a counting pass, a scan of
 * the counts and a writing pass, so a scene's path data becomes a device batch that the batched
 * tessellation calls read as it is. Numbers are rounded to f32 exactly as Rust's
 * `f32::from_str` (and the host parser) rounds them; arc points go through the device's
 * cosf/sinf/tanf, which can differ from the host libm's in the last bit. `options->num_threads`
 * is ignored. Synchronises once to size the outputs. */
int lyon_gpu_svg_parse_paths(lyon_gpu_context* ctx, const char* text,
                             const uint64_t* string_offsets, uint32_t num_strings,
                             const lyon_svg_parse_options* options, lyon_gpu_svg_output* out);

/* Library version and build information (static string). */
const char* lyon_gpu_version(void);

/* Number of kernel launches this library has issued in this process so far (all contexts and
 * threads; no lyon counterpart). The difference across a call is that call's launch count. */
uint64_t lyon_gpu_kernel_launches(void);

#ifdef __cplusplus
}
#endif

#endif /* LYON_GPU_H */
