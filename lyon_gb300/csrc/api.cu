// api.cu — the C ABI of liblyon_gb300.so (declarations and reference citations in
// include/lyon_gpu.h): contexts, device arenas, the batched pipelines (device and host buffers)
// and the single-path drop-ins.
//
// Every batched call is count -> index-range policy -> look-back scan -> (one host read of the
// totals) -> emit. The host-buffer form runs that pipeline per chunk of paths and overlaps each
// chunk's device->host copy (second stream) with the next chunk's kernels.
#include <sys/mman.h>
#include <unistd.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "kernels.h"
#include "kernels_flatten.h"
#include "fill.h"

namespace {

struct DevBuf {
    void* ptr = nullptr;
    size_t cap = 0;
    bool pooled = false;  // from the context's memory pool (freed stream-ordered)
};

struct HostBuf {
    void* ptr = nullptr;
    size_t cap = 0;
};

enum Kind { KIND_STROKE = 0, KIND_FILL = 1 };

}  // namespace

struct lyon_gpu_context {
    int device = 0;
    int num_sms = 1;
    int stroke_bps = 1;
    cudaStream_t stream = nullptr;       // kernels
    cudaStream_t copy_stream = nullptr;  // device->host copies of the host-buffer calls
    // Serving contexts: buffers come from the server's memory pool, allocated and freed in
    // `stream` order. A plain cudaFree can wait for every kernel on the device (another
    // worker's fill sweep included), which a stroke request must not wait behind.
    cudaMemPool_t pool = nullptr;
    std::string last_error;
    // per-path work arrays
    DevBuf vtx_counts, idx_counts, status, vtx_offsets, idx_offsets, scan_state;
    DevBuf small;  // [0] work counter, [1] scan counter, [2] error flag, [3] failed paths,
                   // [4..5] processing-order counters
    DevBuf order;  // processing order of the current stroke batch (long paths first)
    // lyon_gpu_svg_parse_paths: counts, diagnostics, offsets and the parsed batch.
    DevBuf svg_counts, svg_diag, svg_off64, svg_off32, svg_verbs, svg_points, svg_widths;
    bool order_valid = false;
    DevBuf path_class, class_counters;  // classification for the one-thread-per-path phase
    bool split_valid = false;           // class_counters holds the first short item
    // stroke launch settings (the autotuner's knobs)
    uint32_t long_path_points = 1024;  // paths with more points go first; 0: path order
    uint32_t blocks_per_sm = 0;        // 0: as many as fit
    uint32_t short_path_points = 32;   // line-only paths up to this size: one per thread
    bool vertex_attrs = false;  // during a *_attributes call: lyon_stroke_vertex records
    const float* vw_widths = nullptr;  // during a variable-width call: width factors (device)
    uint32_t width_stride = 1;         // floats between consecutive points' width factors
    bool want_sources = false;  // during a custom-attribute call: sequential stepper + sources
    DevBuf out_sources, out_attrs;      // per-vertex sources and interpolated attributes
    // fill sources: per-path counts and offsets (+ scan scratch), per-vertex first source
    DevBuf src_counts, src_offsets, src_scratch, out_source_offsets;
    uint64_t total_sources = 0;
    // arc flattening
    DevBuf arc_counts, arc_status, arc_offsets, arc_points, arc_t, arc_order;
    // the last lyon_gpu_query_sizes (for lyon_gpu_emit_into)
    struct {
        bool valid = false;
        int kind = 0, index_bits = 0, index_mode = 0;
        const void* verbs = nullptr;
        uint32_t num_paths = 0, vertex_offset = 0;
        uint64_t tv = 0, ti = 0;
        uint32_t failed = 0;
    } query;
    // hatching
    DevBuf hatch_bound, hatch_edge_count, hatch_counts, hatch_status, hatch_offsets,
        hatch_scratch, hatch_out, hatch_order;
    DevBuf in_attrs;                    // single-path custom attributes (staged)
    HostBuf h_out_src, h_out_attrs, h_out_soff;
    // outputs of device-buffer batched calls
    DevBuf out_vertices, out_indices;
    // host-buffer calls: inputs and double-buffered outputs
    DevBuf h_in_verbs, h_in_points, h_in_voff, h_in_poff, h_in_opts;
    DevBuf slot_v[2], slot_i[2], slot_status[2];
    cudaEvent_t slot_done[2] = {nullptr, nullptr};
    cudaEvent_t emitted = nullptr;
    // fill scratch / staging
    lg::FillBuffers fill;
    // flatten outputs
    DevBuf flat_counts, flat_offsets, flat_points;
    // single-path staging
    DevBuf in_verbs, in_points, in_offsets, in_options, in_widths;
    HostBuf h_verbs, h_points, h_out_v, h_out_i, h_small, h_offs, h_status;
    // optional per-path first path of its request (serving batches: one id space per request)
    const uint32_t* request_first = nullptr;
    // timing
    bool timing = false;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    float last_ms[4] = {0, 0, 0, 0};
};

namespace {

const char* kVersion = "lyon_gb300 0.1 (sm_103a)";

bool set_err(lyon_gpu_context* ctx, const char* what, cudaError_t e) {
    if (e == cudaSuccess) return true;
    char buf[512];
    snprintf(buf, sizeof buf, "%s: %s", what, cudaGetErrorString(e));
    ctx->last_error = buf;
    return false;
}

bool ensure(lyon_gpu_context* ctx, DevBuf& b, size_t bytes) {
    if (bytes <= b.cap && b.ptr) return true;
    if (b.ptr) {
        if (b.pooled) {
            cudaFreeAsync(b.ptr, ctx->stream);
        } else {
            cudaStreamSynchronize(ctx->stream);
            cudaStreamSynchronize(ctx->copy_stream);
            cudaFree(b.ptr);
        }
        b.ptr = nullptr;
        b.cap = 0;
    }
    size_t cap = bytes < 256 ? 256 : bytes + bytes / 8;
    b.pooled = ctx->pool != nullptr;
    cudaError_t e = b.pooled ? cudaMallocFromPoolAsync(&b.ptr, cap, ctx->pool, ctx->stream)
                             : cudaMalloc(&b.ptr, cap);
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_err(ctx, "cudaMalloc", e);
        return false;
    }
    b.cap = cap;
    return true;
}

bool ensure_host(lyon_gpu_context* ctx, HostBuf& b, size_t bytes) {
    if (bytes <= b.cap && b.ptr) return true;
    if (b.ptr) {
        cudaStreamSynchronize(ctx->stream);
        cudaFreeHost(b.ptr);
        b.ptr = nullptr;
        b.cap = 0;
    }
    size_t cap = bytes < 4096 ? 4096 : bytes + bytes / 4;
    cudaError_t e = cudaMallocHost(&b.ptr, cap);
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_err(ctx, "cudaMallocHost", e);
        return false;
    }
    b.cap = cap;
    return true;
}

template <class T>
T* as(DevBuf& b) {
    return reinterpret_cast<T*>(b.ptr);
}

uint64_t max_index_for(int bits) { return bits == 16 ? 65535ull : 0xFFFFFFFEull; }

// The device address of a pinned, mapped host buffer, or null for any other memory.
template <class T>
T* direct_host_pointer(void* p) {
    if (!p) return nullptr;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type != cudaMemoryTypeHost || !a.devicePointer) return nullptr;
    return reinterpret_cast<T*>(a.devicePointer);
}

uint32_t* small_words(lyon_gpu_context* ctx) { return as<uint32_t>(ctx->small); }

// Pooled buffers too: cudaFree of a stream-ordered allocation does not synchronize, and the
// context's streams are idle when this runs.
void free_buf(DevBuf& b) {
    if (b.ptr) cudaFree(b.ptr);
    b.ptr = nullptr;
    b.cap = 0;
    b.pooled = false;
}
void free_host(HostBuf& b) {
    if (b.ptr) cudaFreeHost(b.ptr);
    b.ptr = nullptr;
    b.cap = 0;
}

void mark(lyon_gpu_context* ctx, int i) {
    if (ctx->timing) cudaEventRecord(ctx->ev[i], ctx->stream);
}

// Sequential index assignment for LYON_INDEX_GLOBAL when the batch overflows the index type:
// BuffersBuilder semantics (geometry_builder.rs:338-350, 478-481) applied path by path, on the
// host. Only taken when the parallel totals exceed the index range.
bool global_overflow_fixup(lyon_gpu_context* ctx, uint32_t n, uint64_t vertex_offset,
                           uint64_t max_index) {
    std::vector<uint32_t> vc(n), ic(n);
    std::vector<int32_t> st(n);
    cudaStream_t s = ctx->stream;
    if (!set_err(ctx, "D2H counts",
                 cudaMemcpyAsync(vc.data(), ctx->vtx_counts.ptr, n * 4ull,
                                 cudaMemcpyDeviceToHost, s)))
        return false;
    cudaMemcpyAsync(ic.data(), ctx->idx_counts.ptr, n * 4ull, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(st.data(), ctx->status.ptr, n * 4ull, cudaMemcpyDeviceToHost, s);
    if (!set_err(ctx, "sync", cudaStreamSynchronize(s))) return false;
    uint64_t len = 0;
    for (uint32_t i = 0; i < n; ++i) {
        if (st[i] != LYON_OK) continue;
        if (vc[i] > 0 && vertex_offset + len + vc[i] - 1 > max_index) {
            st[i] = LYON_ERR_TOO_MANY_VERTICES;
            vc[i] = 0;
            ic[i] = 0;
            continue;
        }
        len += vc[i];
    }
    cudaMemcpyAsync(ctx->vtx_counts.ptr, vc.data(), n * 4ull, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(ctx->idx_counts.ptr, ic.data(), n * 4ull, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(ctx->status.ptr, st.data(), n * 4ull, cudaMemcpyHostToDevice, s);
    return set_err(ctx, "sync", cudaStreamSynchronize(s));
}

bool alloc_path_arrays(lyon_gpu_context* ctx, uint32_t n) {
    return ensure(ctx, ctx->vtx_counts, (size_t)n * 4 + 4) &&
           ensure(ctx, ctx->idx_counts, (size_t)n * 4 + 4) &&
           ensure(ctx, ctx->status, (size_t)n * 4 + 4) &&
           ensure(ctx, ctx->vtx_offsets, ((size_t)n + 1) * 8) &&
           ensure(ctx, ctx->idx_offsets, ((size_t)n + 1) * 8) &&
           ensure(ctx, ctx->scan_state, 2 * lg::scan_tile_count(n) * 8 + 16);
}

// Index-range policy + scan + totals. On return the offsets are valid and *tv / *ti hold the
// totals (one host synchronisation).
bool finish_counts(lyon_gpu_context* ctx, uint32_t n, int index_bits, int index_mode,
                   uint64_t vertex_offset, uint64_t* tv, uint64_t* ti, uint32_t* failed) {
    cudaStream_t s = ctx->stream;
    uint32_t* sw = small_words(ctx);
    uint64_t maxi = max_index_for(index_bits);
    cudaMemsetAsync(sw + 2, 0, 8, s);
    // Per-path mode applies the index range per path; the global mode only counts failures.
    if (!set_err(ctx, "per-path limit",
                 lg::launch_per_path_limit(
                     as<uint32_t>(ctx->vtx_counts), as<uint32_t>(ctx->idx_counts),
                     as<int32_t>(ctx->status), n, vertex_offset,
                     index_mode == LYON_INDEX_PER_PATH ? maxi : ~0ull, sw + 3, s)))
        return false;
    for (int pass = 0; pass < 2; ++pass) {
        if (!set_err(ctx, "scan",
                     lg::launch_scan_pairs(as<uint32_t>(ctx->vtx_counts),
                                           as<uint32_t>(ctx->idx_counts),
                                           as<uint64_t>(ctx->vtx_offsets),
                                           as<uint64_t>(ctx->idx_offsets), n,
                                           as<unsigned long long>(ctx->scan_state), sw + 1,
                                           reinterpret_cast<int*>(sw + 2), s)))
            return false;
        if (!ensure_host(ctx, ctx->h_small, 64)) return false;
        uint64_t* hs = reinterpret_cast<uint64_t*>(ctx->h_small.ptr);
        uint64_t* hs_dev = direct_host_pointer<uint64_t>(hs);
        if (hs_dev) {
            lg::launch_read_totals(as<uint64_t>(ctx->vtx_offsets) + n,
                                   as<uint64_t>(ctx->idx_offsets) + n, sw + 2, hs_dev, s);
        } else {
            cudaMemcpyAsync(hs, as<uint64_t>(ctx->vtx_offsets) + n, 8, cudaMemcpyDeviceToHost, s);
            cudaMemcpyAsync(hs + 1, as<uint64_t>(ctx->idx_offsets) + n, 8, cudaMemcpyDeviceToHost,
                            s);
            cudaMemcpyAsync(hs + 2, sw + 2, 8, cudaMemcpyDeviceToHost, s);
        }
        if (!set_err(ctx, "sync", cudaStreamSynchronize(s))) return false;
        *tv = hs[0];
        *ti = hs[1];
        uint32_t* hw = reinterpret_cast<uint32_t*>(hs + 2);
        if (hw[0] != 0) {
            ctx->last_error = "scan look-back wait exceeded its bound";
            return false;
        }
        *failed = hw[1];
        if (index_mode == LYON_INDEX_GLOBAL && *tv > 0 && vertex_offset + *tv - 1 > maxi &&
            pass == 0) {
            if (!global_overflow_fixup(ctx, n, vertex_offset, maxi)) return false;
            cudaMemsetAsync(sw + 2, 0, 8, s);
            if (!set_err(ctx, "count failures",
                         lg::launch_per_path_limit(as<uint32_t>(ctx->vtx_counts),
                                                   as<uint32_t>(ctx->idx_counts),
                                                   as<int32_t>(ctx->status), n, vertex_offset,
                                                   ~0ull, sw + 3, s)))
                return false;
            continue;
        }
        break;
    }
    return true;
}

bool valid_args(lyon_gpu_context* ctx, const lyon_path_batch* batch, const void* options,
                uint32_t num_options, int index_bits, int index_mode) {
    if (!ctx || !batch || !options || num_options == 0 || (index_bits != 16 && index_bits != 32) ||
        (index_mode != LYON_INDEX_GLOBAL && index_mode != LYON_INDEX_PER_PATH) ||
        (num_options != 1 && num_options != batch->num_paths)) {
        if (ctx) ctx->last_error = "invalid argument";
        return false;
    }
    return true;
}

lg::StrokeArgs stroke_args(lyon_gpu_context* ctx, const lyon_path_batch* batch,
                           const lyon_stroke_options* options, uint32_t num_options,
                           int index_bits, int index_mode, uint64_t vertex_offset) {
    lg::StrokeArgs a;
    memset(&a, 0, sizeof a);
    a.verbs = batch->verbs;
    a.points = batch->points;
    a.verb_offsets = batch->verb_offsets;
    a.point_offsets = batch->point_offsets;
    a.num_paths = batch->num_paths;
    a.options = options;
    a.num_options = num_options;
    a.order = ctx->order_valid ? as<uint32_t>(ctx->order) : nullptr;
    a.work_counter = small_words(ctx);
    a.vtx_counts = as<uint32_t>(ctx->vtx_counts);
    a.idx_counts = as<uint32_t>(ctx->idx_counts);
    a.status = as<int32_t>(ctx->status);
    a.index_bits = index_bits;
    a.index_mode = index_mode;
    a.vertex_offset = (uint32_t)vertex_offset;
    a.vertex_attrs = ctx->vertex_attrs ? 1 : 0;
    a.widths = ctx->vw_widths;
    a.width_stride = ctx->width_stride;
    a.sequential = ctx->want_sources ? 1 : 0;
    a.sources = ctx->want_sources ? as<lyon_vertex_source>(ctx->out_sources) : nullptr;
    a.request_first = ctx->request_first;
    if (ctx->split_valid) {
        a.item_split = as<uint32_t>(ctx->class_counters) + 2 * (3 + ctx->short_path_points);
        a.seq_counter = small_words(ctx) + 6;
    }
    a.vtx_offsets = as<uint64_t>(ctx->vtx_offsets);
    a.idx_offsets = as<uint64_t>(ctx->idx_offsets);
    return a;
}

int stroke_grid(lyon_gpu_context* ctx, uint32_t n) {
    const int bps = ctx->blocks_per_sm > 0 && (int)ctx->blocks_per_sm < ctx->stroke_bps
                        ? (int)ctx->blocks_per_sm
                        : ctx->stroke_bps;
    const int max_grid = ctx->num_sms * bps;
    const int needed = (int)((n + 3) / 4);
    return needed < max_grid ? (needed > 0 ? needed : 1) : max_grid;
}

// Count pass + scan for one device-resident batch.
int pipeline_count(lyon_gpu_context* ctx, int kind, const lyon_path_batch* batch,
                   const void* options, uint32_t num_options, int index_bits, int index_mode,
                   uint64_t vertex_offset, uint64_t* tv, uint64_t* ti, uint32_t* failed) {
    const uint32_t n = batch->num_paths;
    if (!alloc_path_arrays(ctx, n)) return LYON_ERR_OUT_OF_MEMORY;
    cudaStream_t s = ctx->stream;
    mark(ctx, 0);
    ctx->order_valid = false;
    ctx->split_valid = false;
    if (kind == KIND_STROKE) {
        // Long paths first, so that no single long path is left running at the end of a launch;
        // short line-only paths last, for the one-thread-per-path phase.
        if (ctx->vw_widths) {
            // The variable-width stepper takes paths in index order (both passes).
        } else if (n > 0 && ctx->short_path_points > 0) {
            if (ensure(ctx, ctx->order, (size_t)n * 4) && ensure(ctx, ctx->path_class, n) &&
                ensure(ctx, ctx->class_counters, lg::CLASSIFY_COUNTER_WORDS * 4) &&
                lg::launch_classify_paths(batch->verbs, batch->verb_offsets,
                                          batch->point_offsets, n, ctx->long_path_points,
                                          ctx->short_path_points,
                                          as<uint8_t>(ctx->path_class), as<uint32_t>(ctx->order),
                                          as<uint32_t>(ctx->class_counters), s) == cudaSuccess)
                ctx->order_valid = ctx->split_valid = true;
        } else if (n > 0 && ctx->long_path_points > 0 && ensure(ctx, ctx->order, (size_t)n * 4) &&
                   lg::launch_big_first_order(batch->point_offsets, n, ctx->long_path_points,
                                              as<uint32_t>(ctx->order), small_words(ctx) + 4,
                                              s) == cudaSuccess) {
            ctx->order_valid = true;
        }
        lg::StrokeArgs a = stroke_args(ctx, batch, (const lyon_stroke_options*)options,
                                       num_options, index_bits, index_mode, vertex_offset);
        if (n > 0) {
            cudaMemsetAsync(small_words(ctx), 0, 4, s);
            if (a.seq_counter) cudaMemsetAsync(a.seq_counter, 0, 4, s);
            if (!set_err(ctx, "stroke count", lg::launch_stroke(a, false, stroke_grid(ctx, n), s)))
                return LYON_ERR_CUDA;
        }
    } else {
        lg::FillSourceArgs fsa{};
        if (ctx->want_sources) {
            if (!ensure(ctx, ctx->src_counts, (size_t)n * 4 + 16)) return LYON_ERR_OUT_OF_MEMORY;
            fsa.src_counts = as<uint32_t>(ctx->src_counts);
        }
        int r = lg::fill_count(ctx->fill, batch, (const lyon_fill_options*)options, num_options,
                               ctx->num_sms, as<uint32_t>(ctx->vtx_counts),
                               as<uint32_t>(ctx->idx_counts), as<int32_t>(ctx->status),
                               small_words(ctx), s, &ctx->last_error,
                               ctx->want_sources ? &fsa : nullptr);
        if (r != LYON_OK) return r;
    }
    mark(ctx, 1);
    if (!finish_counts(ctx, n, index_bits, index_mode, vertex_offset, tv, ti, failed))
        return LYON_ERR_CUDA;
    mark(ctx, 2);
    return LYON_OK;
}

// Emit pass into caller-chosen device buffers (after pipeline_count on the same batch).
int pipeline_emit(lyon_gpu_context* ctx, int kind, const lyon_path_batch* batch,
                  const void* options, uint32_t num_options, int index_bits, int index_mode,
                  uint64_t vertex_offset, float* vout, void* iout, uint64_t tv) {
    const uint32_t n = batch->num_paths;
    cudaStream_t s = ctx->stream;
    if (kind == KIND_STROKE) {
        lg::StrokeArgs a = stroke_args(ctx, batch, (const lyon_stroke_options*)options,
                                       num_options, index_bits, index_mode, vertex_offset);
        a.vertices = vout;
        a.indices = iout;
        if (n > 0 && tv > 0) {
            cudaMemsetAsync(small_words(ctx), 0, 4, s);
            if (a.seq_counter) cudaMemsetAsync(a.seq_counter, 0, 4, s);
            if (!set_err(ctx, "stroke emit", lg::launch_stroke(a, true, stroke_grid(ctx, n), s)))
                return LYON_ERR_CUDA;
        }
    } else {
        lg::FillSourceArgs fsa{};
        if (ctx->want_sources) {
            fsa.src_offsets = as<uint64_t>(ctx->src_offsets);
            fsa.point_offsets = batch->point_offsets;
            fsa.sources = as<lyon_vertex_source>(ctx->out_sources);
            fsa.source_offsets = as<uint64_t>(ctx->out_source_offsets);
        }
        if (!set_err(ctx, "fill emit",
                     lg::fill_emit(ctx->fill, n, as<uint32_t>(ctx->vtx_counts),
                                   as<uint32_t>(ctx->idx_counts), as<int32_t>(ctx->status),
                                   as<uint64_t>(ctx->vtx_offsets),
                                   as<uint64_t>(ctx->idx_offsets), vout, iout, index_bits,
                                   index_mode, (uint32_t)vertex_offset, ctx->request_first, s,
                                   ctx->want_sources ? &fsa : nullptr)))
            return LYON_ERR_CUDA;
    }
    mark(ctx, 3);
    if (ctx->timing) {
        cudaEventSynchronize(ctx->ev[3]);
        cudaEventElapsedTime(&ctx->last_ms[0], ctx->ev[0], ctx->ev[1]);
        cudaEventElapsedTime(&ctx->last_ms[1], ctx->ev[1], ctx->ev[2]);
        cudaEventElapsedTime(&ctx->last_ms[2], ctx->ev[2], ctx->ev[3]);
        cudaEventElapsedTime(&ctx->last_ms[3], ctx->ev[0], ctx->ev[3]);
    }
    return LYON_OK;
}

// Fill sources after the count phase: per-path source offsets (paths that failed count none),
// the total, and room for every vertex's first source plus the closing total.
int fill_source_offsets(lyon_gpu_context* ctx, uint32_t n, uint64_t tv) {
    cudaStream_t s = ctx->stream;
    ctx->total_sources = 0;
    if (!ensure(ctx, ctx->src_offsets, ((size_t)n + 1) * 8 + 16) ||
        !ensure(ctx, ctx->src_scratch, ((size_t)n + 1) * 8 + 16) ||
        !ensure(ctx, ctx->out_source_offsets, (tv + 1) * 8 + 16) ||
        !ensure(ctx, ctx->src_counts, (size_t)n * 4 + 16) ||
        !ensure_host(ctx, ctx->h_small, 64))
        return LYON_ERR_OUT_OF_MEMORY;
    uint32_t* sw = small_words(ctx);
    uint64_t* hs = reinterpret_cast<uint64_t*>(ctx->h_small.ptr);
    if (n > 0) {
        cudaMemsetAsync(sw + 2, 0, 4, s);
        if (!set_err(ctx, "fill sources",
                     lg::fill_zero_failed_source_counts(as<uint32_t>(ctx->src_counts),
                                                        as<int32_t>(ctx->status), n, s)) ||
            !set_err(ctx, "scan",
                     lg::launch_scan_pairs(as<uint32_t>(ctx->src_counts),
                                           as<uint32_t>(ctx->src_counts),
                                           as<uint64_t>(ctx->src_offsets),
                                           as<uint64_t>(ctx->src_scratch), n,
                                           as<unsigned long long>(ctx->scan_state), sw + 1,
                                           reinterpret_cast<int*>(sw + 2), s)))
            return LYON_ERR_CUDA;
        cudaMemcpyAsync(hs, as<uint64_t>(ctx->src_offsets) + n, 8, cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(hs + 1, sw + 2, 4, cudaMemcpyDeviceToHost, s);
        if (!set_err(ctx, "sync", cudaStreamSynchronize(s))) return LYON_ERR_CUDA;
        if (reinterpret_cast<uint32_t*>(hs + 1)[0] != 0) {
            ctx->last_error = "scan look-back wait exceeded its bound";
            return LYON_ERR_CUDA;
        }
        ctx->total_sources = hs[0];
    }
    // The closing entry: vertex v's sources are [offsets[v], offsets[v + 1]).
    hs[2] = ctx->total_sources;
    cudaMemcpyAsync(as<uint64_t>(ctx->out_source_offsets) + tv, hs + 2, 8,
                    cudaMemcpyHostToDevice, s);
    if (!set_err(ctx, "sync", cudaStreamSynchronize(s))) return LYON_ERR_CUDA;
    return LYON_OK;
}

int batched_device(lyon_gpu_context* ctx, int kind, const lyon_path_batch* batch,
                   const void* options, uint32_t num_options, int index_bits, int index_mode,
                   uint32_t vertex_offset, lyon_gpu_batch_output* out) {
    if (!out || !valid_args(ctx, batch, options, num_options, index_bits, index_mode))
        return LYON_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    memset(out, 0, sizeof(*out));
    uint64_t tv = 0, ti = 0;
    uint32_t failed = 0;
    int r = pipeline_count(ctx, kind, batch, options, num_options, index_bits, index_mode,
                           vertex_offset, &tv, &ti, &failed);
    if (r != LYON_OK) return r;
    const size_t vbytes = ctx->vertex_attrs ? sizeof(lyon_stroke_vertex) : 8;
    if (kind == KIND_FILL && ctx->want_sources) {
        r = fill_source_offsets(ctx, batch->num_paths, tv);
        if (r != LYON_OK) return r;
    }
    const uint64_t nsrc = kind == KIND_FILL ? ctx->total_sources : tv;
    if (!ensure(ctx, ctx->out_vertices, tv * vbytes + 16) ||
        !ensure(ctx, ctx->out_indices, ti * (index_bits / 8) + 16) ||
        (ctx->want_sources &&
         !ensure(ctx, ctx->out_sources, nsrc * sizeof(lyon_vertex_source) + 16)))
        return LYON_ERR_OUT_OF_MEMORY;
    r = pipeline_emit(ctx, kind, batch, options, num_options, index_bits, index_mode,
                      vertex_offset, as<float>(ctx->out_vertices), ctx->out_indices.ptr, tv);
    if (r != LYON_OK) return r;
    out->vertices = as<float>(ctx->out_vertices);
    out->indices = ctx->out_indices.ptr;
    out->vertex_offsets = as<uint64_t>(ctx->vtx_offsets);
    out->index_offsets = as<uint64_t>(ctx->idx_offsets);
    out->status = as<int32_t>(ctx->status);
    out->total_vertices = tv;
    out->total_indices = ti;
    out->num_failed_paths = failed;
    return LYON_OK;
}

// Host-buffer batched call: chunks of paths; inputs copied in, outputs copied out with the
// copy of chunk c overlapping the kernels of chunk c + 1.
int batched_host(lyon_gpu_context* ctx, int kind, const lyon_path_batch* hb, const void* hopts,
                 size_t opt_size, uint32_t num_options, int index_bits, int index_mode,
                 uint32_t vertex_offset, float* hv, uint64_t vcap, void* hi, uint64_t icap,
                 int32_t* hstatus, uint64_t* total_v, uint64_t* total_i) {
    if (!valid_args(ctx, hb, hopts, num_options, index_bits, index_mode))
        return LYON_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    const uint32_t n = hb->num_paths;
    const size_t isz = index_bits / 8;
    // Chunks of at most CH paths (LYON_GB300_HOST_CHUNK_PATHS overrides) and ~64 MB of points.
    uint32_t CH = 1u << 17;
    if (const char* env = getenv("LYON_GB300_HOST_CHUNK_PATHS")) {
        long v = atol(env);
        if (v > 0 && v < (1l << 30)) CH = (uint32_t)v;
    }
    if (hstatus && n > 0 && !ensure_host(ctx, ctx->h_status, (size_t)n * 4))
        return LYON_ERR_OUT_OF_MEMORY;
    uint64_t run_v = 0, run_i = 0;
    bool capacity_ok = true;
    int slot = 0;
    uint32_t c0 = 0;
    // The first chunk's kernels run before any copy can start, so chunks start small and double
    // up to CH: the copy stream, which bounds the call, starts sooner.
    uint32_t ch = CH < 16384u ? CH : 16384u;
    while (c0 < n || (n == 0 && c0 == 0)) {
        uint32_t c1 = c0 + ch < n ? c0 + ch : n;
        ch = ch < CH / 2 ? ch * 2 : CH;
        while (c1 > c0 + 1 &&
               (uint64_t)(hb->point_offsets[c1] - hb->point_offsets[c0]) * 8 > (64ull << 20))
            c1 = c0 + (c1 - c0) / 2;
        const uint32_t cn = c1 - c0;
        const uint32_t vb = hb->verb_offsets[c0], ve = hb->verb_offsets[c1];
        const uint32_t pb = hb->point_offsets[c0], pe = hb->point_offsets[c1];
        cudaStream_t s = ctx->stream;
        // Inputs (offsets rebased on the host).
        if (!ensure(ctx, ctx->h_in_verbs, (size_t)(ve - vb) + 16) ||
            !ensure(ctx, ctx->h_in_points, (size_t)(pe - pb) * 8 + 16) ||
            !ensure(ctx, ctx->h_in_voff, ((size_t)cn + 1) * 4) ||
            !ensure(ctx, ctx->h_in_poff, ((size_t)cn + 1) * 4) ||
            !ensure(ctx, ctx->h_in_opts, (num_options > 1 ? (size_t)cn : 1) * opt_size) ||
            !ensure_host(ctx, ctx->h_offs, ((size_t)cn + 1) * 8))
            return LYON_ERR_OUT_OF_MEMORY;
        // The host staging of offsets is reused per chunk: wait for its previous copy.
        cudaStreamSynchronize(s);
        uint32_t* ho = reinterpret_cast<uint32_t*>(ctx->h_offs.ptr);
        for (uint32_t i = 0; i <= cn; ++i) {
            ho[i] = hb->verb_offsets[c0 + i] - vb;
            ho[cn + 1 + i] = hb->point_offsets[c0 + i] - pb;
        }
        cudaMemcpyAsync(ctx->h_in_voff.ptr, ho, ((size_t)cn + 1) * 4, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(ctx->h_in_poff.ptr, ho + cn + 1, ((size_t)cn + 1) * 4,
                        cudaMemcpyHostToDevice, s);
        if (ve > vb)
            cudaMemcpyAsync(ctx->h_in_verbs.ptr, hb->verbs + vb, ve - vb, cudaMemcpyHostToDevice, s);
        if (pe > pb)
            cudaMemcpyAsync(ctx->h_in_points.ptr, hb->points + 2 * (size_t)pb, (size_t)(pe - pb) * 8,
                            cudaMemcpyHostToDevice, s);
        const unsigned char* op = reinterpret_cast<const unsigned char*>(hopts);
        size_t ob = (num_options > 1 ? (size_t)cn : 1) * opt_size;
        cudaMemcpyAsync(ctx->h_in_opts.ptr, op + (num_options > 1 ? (size_t)c0 * opt_size : 0), ob,
                        cudaMemcpyHostToDevice, s);
        lyon_path_batch db;
        db.verbs = as<uint8_t>(ctx->h_in_verbs);
        db.points = as<float>(ctx->h_in_points);
        db.verb_offsets = as<uint32_t>(ctx->h_in_voff);
        db.point_offsets = as<uint32_t>(ctx->h_in_poff);
        db.num_paths = cn;
        uint64_t tv = 0, ti = 0;
        uint32_t failed = 0;
        uint64_t voff = index_mode == LYON_INDEX_GLOBAL ? vertex_offset + run_v : vertex_offset;
        int r = pipeline_count(ctx, kind, &db, ctx->h_in_opts.ptr, num_options > 1 ? cn : 1,
                               index_bits, index_mode, voff, &tv, &ti, &failed);
        if (r != LYON_OK) return r;
        if (run_v + tv > vcap || run_i + ti > icap || !hv || (ti && !hi)) capacity_ok = false;
        if (capacity_ok && cn > 0) {
            // Wait until this slot's previous device->host copy is done, then emit into it.
            cudaEventSynchronize(ctx->slot_done[slot]);
            if (!ensure(ctx, ctx->slot_v[slot], tv * 8 + 16) ||
                !ensure(ctx, ctx->slot_i[slot], ti * isz + 16))
                return LYON_ERR_OUT_OF_MEMORY;
            r = pipeline_emit(ctx, kind, &db, ctx->h_in_opts.ptr, num_options > 1 ? cn : 1,
                              index_bits, index_mode, voff, as<float>(ctx->slot_v[slot]),
                              ctx->slot_i[slot].ptr, tv);
            if (r != LYON_OK) return r;
            if (hstatus) {
                if (!ensure(ctx, ctx->slot_status[slot], (size_t)cn * 4)) return LYON_ERR_OUT_OF_MEMORY;
                cudaMemcpyAsync(ctx->slot_status[slot].ptr, ctx->status.ptr, (size_t)cn * 4,
                                cudaMemcpyDeviceToDevice, s);
            }
            cudaEventRecord(ctx->emitted, s);
            cudaStreamWaitEvent(ctx->copy_stream, ctx->emitted, 0);
            if (tv)
                cudaMemcpyAsync(hv + 2 * run_v, ctx->slot_v[slot].ptr, tv * 8,
                                cudaMemcpyDeviceToHost, ctx->copy_stream);
            if (ti)
                cudaMemcpyAsync(reinterpret_cast<unsigned char*>(hi) + run_i * isz,
                                ctx->slot_i[slot].ptr, ti * isz, cudaMemcpyDeviceToHost,
                                ctx->copy_stream);
            if (hstatus)  // into pinned staging: a copy into pageable memory would block
                cudaMemcpyAsync(reinterpret_cast<int32_t*>(ctx->h_status.ptr) + c0,
                                ctx->slot_status[slot].ptr, (size_t)cn * 4,
                                cudaMemcpyDeviceToHost, ctx->copy_stream);
            cudaEventRecord(ctx->slot_done[slot], ctx->copy_stream);
            slot ^= 1;
        }
        run_v += tv;
        run_i += ti;
        if (n == 0) break;
        c0 = c1;
    }
    if (!set_err(ctx, "sync", cudaStreamSynchronize(ctx->copy_stream)) ||
        !set_err(ctx, "sync", cudaStreamSynchronize(ctx->stream)))
        return LYON_ERR_CUDA;
    if (hstatus && capacity_ok && n > 0) std::memcpy(hstatus, ctx->h_status.ptr, (size_t)n * 4);
    if (total_v) *total_v = run_v;
    if (total_i) *total_i = run_i;
    if (!capacity_ok) {
        ctx->last_error = "output buffers too small";
        return LYON_ERR_CAPACITY;
    }
    return LYON_OK;
}

// Copies a host path into the context's device input arena (one-path batch).
bool stage_single_path(lyon_gpu_context* ctx, const uint8_t* verbs, uint32_t num_verbs,
                       const float* points, uint32_t num_points, const void* options,
                       size_t options_size, lyon_path_batch* batch,
                       const float* widths = nullptr, uint32_t floats_per_point = 1) {
    cudaStream_t s = ctx->stream;
    size_t vb = num_verbs, pb = (size_t)num_points * 8;
    size_t wb = widths ? (size_t)num_points * floats_per_point * 4 : 0;
    if (!ensure(ctx, ctx->in_verbs, vb + 16) || !ensure(ctx, ctx->in_points, pb + 16) ||
        !ensure(ctx, ctx->in_offsets, 64) || !ensure(ctx, ctx->in_options, 64) ||
        (widths && !ensure(ctx, ctx->in_widths, wb + 16)) ||
        !ensure_host(ctx, ctx->h_verbs, vb + 128 + options_size) ||
        !ensure_host(ctx, ctx->h_points, pb + wb + 16))
        return false;
    cudaStreamSynchronize(s);
    unsigned char* hv = reinterpret_cast<unsigned char*>(ctx->h_verbs.ptr);
    uint32_t* hoff = reinterpret_cast<uint32_t*>(hv);
    hoff[0] = 0;
    hoff[1] = num_verbs;
    hoff[2] = 0;
    hoff[3] = num_points;
    memcpy(hv + 16, options, options_size);
    if (num_verbs) memcpy(hv + 64, verbs, vb);
    if (num_points) memcpy(ctx->h_points.ptr, points, pb);
    cudaMemcpyAsync(ctx->in_offsets.ptr, hv, 16, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(ctx->in_options.ptr, hv + 16, options_size, cudaMemcpyHostToDevice, s);
    if (num_verbs) cudaMemcpyAsync(ctx->in_verbs.ptr, hv + 64, vb, cudaMemcpyHostToDevice, s);
    if (num_points)
        cudaMemcpyAsync(ctx->in_points.ptr, ctx->h_points.ptr, pb, cudaMemcpyHostToDevice, s);
    if (widths && num_points) {
        unsigned char* hw = reinterpret_cast<unsigned char*>(ctx->h_points.ptr) + pb;
        memcpy(hw, widths, wb);
        cudaMemcpyAsync(ctx->in_widths.ptr, hw, wb, cudaMemcpyHostToDevice, s);
    }
    batch->verbs = as<uint8_t>(ctx->in_verbs);
    batch->points = as<float>(ctx->in_points);
    batch->verb_offsets = as<uint32_t>(ctx->in_offsets);
    batch->point_offsets = as<uint32_t>(ctx->in_offsets) + 2;
    batch->num_paths = 1;
    return true;
}

int single_path(lyon_gpu_context* ctx, int kind, const uint8_t* verbs, uint32_t num_verbs,
                const float* points, uint32_t num_points, const void* options, size_t opt_size,
                int index_bits, uint32_t index_base, lyon_gpu_result* result,
                const float* point_floats = nullptr, uint32_t floats_per_point = 1,
                int32_t width_index = 0) {
    if (!ctx || !options || !result || (index_bits != 16 && index_bits != 32) ||
        (num_verbs && !verbs) || (num_points && !points)) {
        if (ctx) ctx->last_error = "invalid argument";
        return LYON_ERR_INVALID_ARGUMENT;
    }
    cudaSetDevice(ctx->device);
    memset(result, 0, sizeof(*result));
    lyon_path_batch b;
    if (!stage_single_path(ctx, verbs, num_verbs, points, num_points, options, opt_size, &b,
                           point_floats, floats_per_point))
        return LYON_ERR_OUT_OF_MEMORY;
    if (point_floats && width_index >= 0) {
        ctx->vw_widths = as<float>(ctx->in_widths) + width_index;
        ctx->width_stride = floats_per_point;
    }
    lyon_gpu_batch_output bo;
    int r = batched_device(ctx, kind, &b, ctx->in_options.ptr, 1, index_bits,
                           LYON_INDEX_PER_PATH, index_base, &bo);
    if (r != LYON_OK) return r;
    cudaStream_t s = ctx->stream;
    if (!ensure_host(ctx, ctx->h_small, 64)) return LYON_ERR_OUT_OF_MEMORY;
    size_t vb = bo.total_vertices * (ctx->vertex_attrs ? sizeof(lyon_stroke_vertex) : 8);
    size_t ib = bo.total_indices * (index_bits / 8);
    if (!ensure_host(ctx, ctx->h_out_v, vb + 16) || !ensure_host(ctx, ctx->h_out_i, ib + 16))
        return LYON_ERR_OUT_OF_MEMORY;
    if (ctx->want_sources) {
        // Custom attributes: the vertices' sources and their interpolated attributes (a fill
        // vertex has any number of sources, located by per-vertex offsets).
        const bool fill = kind == KIND_FILL;
        const uint64_t ns = fill ? ctx->total_sources : bo.total_vertices;
        const size_t sb = ns * sizeof(lyon_vertex_source);
        const size_t ob = fill ? (bo.total_vertices + 1) * 8 : 0;
        const size_t ab = point_floats ? bo.total_vertices * floats_per_point * 4 : 0;
        if (!ensure_host(ctx, ctx->h_out_src, sb + 16) ||
            !ensure_host(ctx, ctx->h_out_soff, ob + 16) ||
            !ensure_host(ctx, ctx->h_out_attrs, ab + 16) ||
            (ab && !ensure(ctx, ctx->out_attrs, ab + 16)))
            return LYON_ERR_OUT_OF_MEMORY;
        cudaError_t e = cudaSuccess;
        if (ab && fill) {
            e = lg::launch_interpolate_fill(as<lyon_vertex_source>(ctx->out_sources),
                                            as<uint64_t>(ctx->out_source_offsets),
                                            bo.total_vertices, as<float>(ctx->in_widths),
                                            floats_per_point, num_points,
                                            as<float>(ctx->out_attrs), ctx->num_sms, s);
        } else if (ab) {
            e = lg::launch_interpolate(as<lyon_vertex_source>(ctx->out_sources),
                                       bo.total_vertices, as<float>(ctx->in_widths),
                                       floats_per_point, num_points, as<float>(ctx->out_attrs),
                                       ctx->num_sms, s);
        }
        if (!set_err(ctx, "interpolate", e)) return LYON_ERR_CUDA;
        if (sb) cudaMemcpyAsync(ctx->h_out_src.ptr, ctx->out_sources.ptr, sb,
                                cudaMemcpyDeviceToHost, s);
        if (ob) cudaMemcpyAsync(ctx->h_out_soff.ptr, ctx->out_source_offsets.ptr, ob,
                                cudaMemcpyDeviceToHost, s);
        if (ab) cudaMemcpyAsync(ctx->h_out_attrs.ptr, ctx->out_attrs.ptr, ab,
                                cudaMemcpyDeviceToHost, s);
    }
    cudaMemcpyAsync(ctx->h_small.ptr, bo.status, 4, cudaMemcpyDeviceToHost, s);
    if (vb) cudaMemcpyAsync(ctx->h_out_v.ptr, bo.vertices, vb, cudaMemcpyDeviceToHost, s);
    if (ib) cudaMemcpyAsync(ctx->h_out_i.ptr, bo.indices, ib, cudaMemcpyDeviceToHost, s);
    if (!set_err(ctx, "sync", cudaStreamSynchronize(s))) return LYON_ERR_CUDA;
    int32_t st = *reinterpret_cast<int32_t*>(ctx->h_small.ptr);
    result->status = st;
    result->vertices = reinterpret_cast<const float*>(ctx->h_out_v.ptr);
    result->indices = ctx->h_out_i.ptr;
    if (st != LYON_OK) return st;
    result->num_vertices = (uint32_t)bo.total_vertices;
    result->num_indices = (uint32_t)bo.total_indices;
    return LYON_OK;
}

}  // namespace

// Entry points for the serving loop (serve.cu): one batched call split in its count and emit
// halves, u32 indices, one id space per request (`request_first`).
namespace lg {

int srv_count(lyon_gpu_context* ctx, int kind, const lyon_path_batch* batch, const void* options,
              uint32_t num_options, const uint32_t* request_first, uint64_t* tv, uint64_t* ti,
              uint32_t* failed) {
    cudaSetDevice(ctx->device);
    ctx->request_first = request_first;
    int r = pipeline_count(ctx, kind, batch, options, num_options, 32, LYON_INDEX_GLOBAL, 0, tv,
                           ti, failed);
    ctx->request_first = nullptr;
    return r;
}

int srv_emit(lyon_gpu_context* ctx, int kind, const lyon_path_batch* batch, const void* options,
             uint32_t num_options, const uint32_t* request_first, float* vout, void* iout,
             uint64_t tv) {
    ctx->request_first = request_first;
    int r = pipeline_emit(ctx, kind, batch, options, num_options, 32, LYON_INDEX_GLOBAL, 0, vout,
                          iout, tv);
    ctx->request_first = nullptr;
    return r;
}

const uint64_t* srv_vtx_offsets(lyon_gpu_context* ctx) { return as<uint64_t>(ctx->vtx_offsets); }
const uint64_t* srv_idx_offsets(lyon_gpu_context* ctx) { return as<uint64_t>(ctx->idx_offsets); }
const int32_t* srv_status(lyon_gpu_context* ctx) { return as<int32_t>(ctx->status); }
cudaStream_t srv_stream(lyon_gpu_context* ctx) { return ctx->stream; }

// Settings of a serving worker's context. A stroke lane gets a stream of the device's highest
// priority (its blocks are dispatched before queued blocks of other streams) and one stroke block
// per SM; `fill_blocks_per_sm` (0: default) bounds the fill sweep's residency.
int srv_configure(lyon_gpu_context* ctx, bool stroke_lane, uint32_t fill_blocks_per_sm,
                  cudaMemPool_t pool) {
    ctx->fill.blocks_per_sm_cap = fill_blocks_per_sm;
    ctx->pool = pool;
    // The fill buffers are all allocated by the first fill call, so they are all pooled or none.
    if (!ctx->fill.scratch && !ctx->fill.stage_v && !ctx->fill.work) ctx->fill.pool = pool;
    if (!stroke_lane) return LYON_OK;
    ctx->blocks_per_sm = 1;
    int least = 0, greatest = 0;
    if (cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess) {
        cudaGetLastError();
        return LYON_OK;  // priorities unsupported: keep the default stream
    }
    cudaStream_t s = nullptr;
    if (cudaStreamCreateWithPriority(&s, cudaStreamNonBlocking, greatest) != cudaSuccess) {
        cudaGetLastError();
        return LYON_OK;
    }
    cudaStreamSynchronize(ctx->stream);
    cudaStreamDestroy(ctx->stream);
    ctx->stream = s;
    return LYON_OK;
}

}  // namespace lg

extern "C" {

const char* lyon_gpu_version(void) { return kVersion; }

// ---- host buffers for the host-buffer calls ---------------------------------------------------

namespace {
struct HostMapping {
    void* base;
    size_t len;
};
std::mutex g_host_mu;
std::unordered_map<void*, HostMapping> g_host_maps;

// The transparent huge page size (2 MB with 4 KB base pages, 512 MB with 64 KB ones).
size_t thp_size() {
    size_t v = 0;
    if (FILE* f = fopen("/sys/kernel/mm/transparent_hugepage/hpage_pmd_size", "r")) {
        unsigned long long x = 0;
        if (fscanf(f, "%llu", &x) == 1) v = (size_t)x;
        fclose(f);
    }
    return v >= 4096 && v <= (1ull << 31) ? v : (2u << 20);
}
}  // namespace

void* lyon_gpu_host_alloc(size_t bytes) {
    if (bytes == 0) return nullptr;
    const size_t page = (size_t)sysconf(_SC_PAGESIZE);
    const size_t huge = thp_size();
    // Whole huge pages, on a huge-page boundary: map one huge page more and start at the first
    // boundary inside the mapping.
    const size_t len = (bytes + huge - 1) / huge * huge;
    const size_t map_len = len + huge;
    void* base = mmap(nullptr, map_len, PROT_READ | PROT_WRITE, MAP_PRIVATE | MAP_ANONYMOUS, -1, 0);
    if (base == MAP_FAILED) return nullptr;
    char* p = reinterpret_cast<char*>(((uintptr_t)base + huge - 1) / huge * huge);
    madvise(p, len, MADV_HUGEPAGE);  // a hint: without transparent huge pages, base pages
    // Fault the pages in now (one write per huge page), then pin them for DMA.
    for (size_t off = 0; off < len; off += page < huge ? huge : page) p[off] = 0;
    if (cudaHostRegister(p, len, cudaHostRegisterDefault) != cudaSuccess) {
        cudaGetLastError();
        munmap(base, map_len);
        return nullptr;
    }
    std::lock_guard<std::mutex> g(g_host_mu);
    g_host_maps[p] = HostMapping{base, map_len};
    return p;
}

int lyon_gpu_host_free(void* ptr) {
    if (!ptr) return LYON_OK;
    HostMapping m;
    {
        std::lock_guard<std::mutex> g(g_host_mu);
        auto it = g_host_maps.find(ptr);
        if (it == g_host_maps.end()) return LYON_ERR_INVALID_ARGUMENT;
        m = it->second;
        g_host_maps.erase(it);
    }
    cudaHostUnregister(ptr);
    cudaGetLastError();
    munmap(m.base, m.len);
    return LYON_OK;
}

uint64_t lyon_gpu_kernel_launches(void) { return lg::launches_total(); }

lyon_gpu_context* lyon_gpu_create(int device) {
    lyon_gpu_context* ctx = new lyon_gpu_context();
    ctx->device = device;
    cudaDeviceProp prop;
    if (cudaSetDevice(device) != cudaSuccess ||
        cudaGetDeviceProperties(&prop, device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        delete ctx;
        return nullptr;
    }
    ctx->num_sms = prop.multiProcessorCount;
    ctx->stroke_bps = lg::stroke_blocks_per_sm();
    for (int i = 0; i < 4; ++i) cudaEventCreate(&ctx->ev[i]);
    cudaEventCreateWithFlags(&ctx->slot_done[0], cudaEventDisableTiming);
    cudaEventCreateWithFlags(&ctx->slot_done[1], cudaEventDisableTiming);
    cudaEventCreateWithFlags(&ctx->emitted, cudaEventDisableTiming);
    if (!ensure(ctx, ctx->small, 64)) {
        lyon_gpu_destroy(ctx);
        return nullptr;
    }
    cudaMemsetAsync(ctx->small.ptr, 0, 64, ctx->stream);
    cudaStreamSynchronize(ctx->stream);
    return ctx;
}

void lyon_gpu_destroy(lyon_gpu_context* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->copy_stream) cudaStreamSynchronize(ctx->copy_stream);
    DevBuf* bufs[] = {&ctx->vtx_counts, &ctx->idx_counts,  &ctx->status,      &ctx->vtx_offsets,
                      &ctx->idx_offsets, &ctx->scan_state, &ctx->small,       &ctx->out_vertices,
                      &ctx->out_indices, &ctx->h_in_verbs, &ctx->h_in_points, &ctx->h_in_voff,
                      &ctx->h_in_poff,  &ctx->h_in_opts,   &ctx->slot_v[0],   &ctx->slot_v[1],
                      &ctx->slot_i[0],  &ctx->slot_i[1],   &ctx->flat_counts, &ctx->flat_offsets,
                      &ctx->flat_points, &ctx->in_verbs,   &ctx->in_points,   &ctx->in_offsets,
                      &ctx->in_options, &ctx->order, &ctx->svg_counts, &ctx->svg_diag,
                      &ctx->svg_off64, &ctx->svg_off32, &ctx->svg_verbs, &ctx->svg_points,
                      &ctx->svg_widths, &ctx->slot_status[0],
                      &ctx->slot_status[1], &ctx->path_class, &ctx->class_counters,
                      &ctx->in_widths, &ctx->out_sources, &ctx->out_attrs, &ctx->in_attrs,
                      &ctx->src_counts, &ctx->src_offsets, &ctx->src_scratch,
                      &ctx->out_source_offsets, &ctx->arc_counts, &ctx->arc_status,
                      &ctx->arc_offsets, &ctx->arc_points, &ctx->arc_t, &ctx->arc_order,
                      &ctx->hatch_bound,
                      &ctx->hatch_edge_count, &ctx->hatch_counts, &ctx->hatch_status,
                      &ctx->hatch_offsets, &ctx->hatch_scratch, &ctx->hatch_out,
                      &ctx->hatch_order};
    for (DevBuf* b : bufs) free_buf(*b);
    lg::fill_free(ctx->fill);
    HostBuf* hb[] = {&ctx->h_verbs, &ctx->h_points, &ctx->h_out_v,  &ctx->h_out_i,
                     &ctx->h_small, &ctx->h_offs,   &ctx->h_status, &ctx->h_out_src,
                     &ctx->h_out_attrs, &ctx->h_out_soff};
    for (HostBuf* b : hb) free_host(*b);
    for (int i = 0; i < 4; ++i)
        if (ctx->ev[i]) cudaEventDestroy(ctx->ev[i]);
    for (int i = 0; i < 2; ++i)
        if (ctx->slot_done[i]) cudaEventDestroy(ctx->slot_done[i]);
    if (ctx->emitted) cudaEventDestroy(ctx->emitted);
    if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

void* lyon_gpu_stream(lyon_gpu_context* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

const char* lyon_gpu_last_error(lyon_gpu_context* ctx) {
    return ctx ? ctx->last_error.c_str() : "null context";
}

int lyon_gpu_set_stroke_tuning(lyon_gpu_context* ctx, const lyon_gpu_stroke_tuning* t) {
    if (!ctx || !t) return LYON_ERR_INVALID_ARGUMENT;
    if (t->short_path_points > lg::CLASSIFY_MAX_SHORT_POINTS) {
        ctx->last_error = "short_path_points above 64";
        return LYON_ERR_INVALID_ARGUMENT;
    }
    ctx->long_path_points = t->long_path_points;
    ctx->blocks_per_sm = t->blocks_per_sm;
    ctx->short_path_points = t->short_path_points;
    return LYON_OK;
}

int lyon_gpu_get_stroke_tuning(lyon_gpu_context* ctx, lyon_gpu_stroke_tuning* t) {
    if (!ctx || !t) return LYON_ERR_INVALID_ARGUMENT;
    t->long_path_points = ctx->long_path_points;
    t->blocks_per_sm = ctx->blocks_per_sm;
    t->short_path_points = ctx->short_path_points;
    return LYON_OK;
}

int lyon_gpu_autotune_stroke(lyon_gpu_context* ctx, const lyon_path_batch* batch,
                             const lyon_stroke_options* options, uint32_t num_options,
                             uint32_t sample_paths, lyon_gpu_stroke_tuning* best,
                             float* times_ms, uint32_t* num_candidates) {
    if (!ctx || !batch || !options || (num_options != 1 && num_options != batch->num_paths))
        return LYON_ERR_INVALID_ARGUMENT;
    static const uint32_t kPoints[] = {0u, 256u, 1024u, 8192u};
    static const uint32_t kBlocks[] = {0u, 1u};
    static const uint32_t kShort[] = {0u, 32u};
    const uint32_t nc = 16;
    if (num_candidates) *num_candidates = nc;
    lyon_path_batch sample = *batch;
    if (sample_paths > 0 && sample_paths < batch->num_paths) sample.num_paths = sample_paths;
    const uint32_t sopts = num_options > 1 ? sample.num_paths : 1;
    lyon_gpu_stroke_tuning saved;
    lyon_gpu_get_stroke_tuning(ctx, &saved);
    const bool saved_timing = ctx->timing;
    ctx->timing = false;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best_ms = -1.0f;
    lyon_gpu_stroke_tuning b = saved;
    int rc = LYON_OK;
    for (uint32_t c = 0; c < nc && rc == LYON_OK; ++c) {
        ctx->long_path_points = kPoints[c % 4];
        ctx->blocks_per_sm = kBlocks[(c / 4) % 2];
        ctx->short_path_points = kShort[c / 8];
        lyon_gpu_batch_output out;
        rc = batched_device(ctx, KIND_STROKE, &sample, options, sopts, 32, LYON_INDEX_PER_PATH, 0,
                            &out);  // warm-up (and buffer growth)
        if (rc != LYON_OK) break;
        float ms = 0.0f;
        for (int rep = 0; rep < 2 && rc == LYON_OK; ++rep) {
            cudaEventRecord(e0, ctx->stream);
            rc = batched_device(ctx, KIND_STROKE, &sample, options, sopts, 32,
                                LYON_INDEX_PER_PATH, 0, &out);
            cudaEventRecord(e1, ctx->stream);
            cudaEventSynchronize(e1);
            float m = 0.0f;
            cudaEventElapsedTime(&m, e0, e1);
            ms += m;
        }
        ms *= 0.5f;
        if (times_ms) times_ms[c] = ms;
        if (best_ms < 0.0f || ms < best_ms) {
            best_ms = ms;
            lyon_gpu_get_stroke_tuning(ctx, &b);
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    ctx->timing = saved_timing;
    if (rc != LYON_OK) {
        lyon_gpu_set_stroke_tuning(ctx, &saved);
        return rc;
    }
    lyon_gpu_set_stroke_tuning(ctx, &b);
    if (best) *best = b;
    return LYON_OK;
}

int lyon_gpu_set_fill_tuning(lyon_gpu_context* ctx, const lyon_gpu_fill_tuning* t) {
    if (!ctx || !t || t->lanes > 32 || t->blocks_per_sm > 64) return LYON_ERR_INVALID_ARGUMENT;
    ctx->fill.blocks_per_sm_cap = t->blocks_per_sm;
    ctx->fill.lanes = t->lanes;
    return LYON_OK;
}

int lyon_gpu_get_fill_tuning(lyon_gpu_context* ctx, lyon_gpu_fill_tuning* t) {
    if (!ctx || !t) return LYON_ERR_INVALID_ARGUMENT;
    t->blocks_per_sm = ctx->fill.blocks_per_sm_cap;
    t->lanes = ctx->fill.lanes;
    return LYON_OK;
}

int lyon_gpu_autotune_fill(lyon_gpu_context* ctx, const lyon_path_batch* batch,
                           const lyon_fill_options* options, uint32_t num_options,
                           uint32_t sample_paths, lyon_gpu_fill_tuning* best, float* times_ms,
                           uint32_t* num_candidates) {
    if (!ctx || !batch || !options || (num_options != 1 && num_options != batch->num_paths))
        return LYON_ERR_INVALID_ARGUMENT;
    static const uint32_t kBlocks[] = {16u, 8u};
    static const uint32_t kLanes[] = {1u, 4u, 8u, 12u, 16u};
    const uint32_t nc = 10;
    if (num_candidates) *num_candidates = nc;
    lyon_path_batch sample = *batch;
    if (sample_paths > 0 && sample_paths < batch->num_paths) sample.num_paths = sample_paths;
    const uint32_t sopts = num_options > 1 ? sample.num_paths : 1;
    lyon_gpu_fill_tuning saved;
    lyon_gpu_get_fill_tuning(ctx, &saved);
    const bool saved_timing = ctx->timing;
    ctx->timing = false;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best_ms = -1.0f;
    lyon_gpu_fill_tuning b = saved;
    int rc = LYON_OK;
    for (uint32_t c = 0; c < nc && rc == LYON_OK; ++c) {
        lyon_gpu_fill_tuning t{kBlocks[c / 5], kLanes[c % 5]};
        lyon_gpu_set_fill_tuning(ctx, &t);
        lyon_gpu_batch_output out;
        rc = batched_device(ctx, KIND_FILL, &sample, options, sopts, 32, LYON_INDEX_PER_PATH, 0,
                            &out);  // warm-up (and heap growth)
        if (rc != LYON_OK) break;
        cudaEventRecord(e0, ctx->stream);
        rc = batched_device(ctx, KIND_FILL, &sample, options, sopts, 32, LYON_INDEX_PER_PATH, 0,
                            &out);
        cudaEventRecord(e1, ctx->stream);
        cudaEventSynchronize(e1);
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (times_ms) times_ms[c] = ms;
        if (best_ms < 0.0f || ms < best_ms) {
            best_ms = ms;
            b = t;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    ctx->timing = saved_timing;
    if (rc != LYON_OK) {
        lyon_gpu_set_fill_tuning(ctx, &saved);
        return rc;
    }
    lyon_gpu_set_fill_tuning(ctx, &b);
    if (best) *best = b;
    return LYON_OK;
}

int lyon_gpu_synchronize(lyon_gpu_context* ctx) {
    if (!ctx) return LYON_ERR_INVALID_ARGUMENT;
    return set_err(ctx, "cudaStreamSynchronize", cudaStreamSynchronize(ctx->stream))
               ? LYON_OK
               : LYON_ERR_CUDA;
}

void lyon_gpu_set_timing(lyon_gpu_context* ctx, int enabled) {
    if (ctx) ctx->timing = enabled != 0;
}

int lyon_gpu_last_timings(lyon_gpu_context* ctx, float* ms4) {
    if (!ctx || !ms4) return LYON_ERR_INVALID_ARGUMENT;
    for (int i = 0; i < 4; ++i) ms4[i] = ctx->last_ms[i];
    return LYON_OK;
}

int lyon_gpu_query_sizes(lyon_gpu_context* ctx, int kind, const lyon_path_batch* batch,
                         const void* options, uint32_t num_options, int index_bits,
                         int index_mode, uint32_t vertex_offset, uint64_t* total_vertices,
                         uint64_t* total_indices, uint32_t* num_failed_paths) {
    if (!ctx || (kind != KIND_STROKE && kind != KIND_FILL) || !total_vertices ||
        !total_indices || !valid_args(ctx, batch, options, num_options, index_bits, index_mode))
        return LYON_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    ctx->query.valid = false;
    uint64_t tv = 0, ti = 0;
    uint32_t failed = 0;
    int r = pipeline_count(ctx, kind, batch, options, num_options, index_bits, index_mode,
                           vertex_offset, &tv, &ti, &failed);
    if (r != LYON_OK) return r;
    *total_vertices = tv;
    *total_indices = ti;
    if (num_failed_paths) *num_failed_paths = failed;
    ctx->query.valid = true;
    ctx->query.kind = kind;
    ctx->query.index_bits = index_bits;
    ctx->query.index_mode = index_mode;
    ctx->query.verbs = batch->verbs;
    ctx->query.num_paths = batch->num_paths;
    ctx->query.vertex_offset = vertex_offset;
    ctx->query.tv = tv;
    ctx->query.ti = ti;
    ctx->query.failed = failed;
    return LYON_OK;
}

int lyon_gpu_emit_into(lyon_gpu_context* ctx, int kind, const lyon_path_batch* batch,
                       const void* options, uint32_t num_options, int index_bits, int index_mode,
                       uint32_t vertex_offset, float* vertices, void* indices,
                       lyon_gpu_batch_output* out) {
    if (!ctx || !out || !batch || !ctx->query.valid || ctx->query.kind != kind ||
        ctx->query.index_bits != index_bits || ctx->query.index_mode != index_mode ||
        ctx->query.verbs != batch->verbs || ctx->query.num_paths != batch->num_paths ||
        ctx->query.vertex_offset != vertex_offset ||
        (ctx->query.tv > 0 && !vertices) || (ctx->query.ti > 0 && !indices)) {
        if (ctx) ctx->last_error = "lyon_gpu_emit_into without a matching lyon_gpu_query_sizes";
        return LYON_ERR_INVALID_ARGUMENT;
    }
    cudaSetDevice(ctx->device);
    ctx->query.valid = false;
    memset(out, 0, sizeof(*out));
    int r = pipeline_emit(ctx, kind, batch, options, num_options, index_bits, index_mode,
                          vertex_offset, vertices, indices, ctx->query.tv);
    if (r != LYON_OK) return r;
    out->vertices = vertices;
    out->indices = indices;
    out->vertex_offsets = as<uint64_t>(ctx->vtx_offsets);
    out->index_offsets = as<uint64_t>(ctx->idx_offsets);
    out->status = as<int32_t>(ctx->status);
    out->total_vertices = ctx->query.tv;
    out->total_indices = ctx->query.ti;
    out->num_failed_paths = ctx->query.failed;
    return LYON_OK;
}

int lyon_gpu_stroke_paths(lyon_gpu_context* ctx, const lyon_path_batch* batch,
                          const lyon_stroke_options* options, uint32_t num_options,
                          int index_bits, int index_mode, uint32_t vertex_offset,
                          lyon_gpu_batch_output* out) {
    return batched_device(ctx, KIND_STROKE, batch, options, num_options, index_bits, index_mode,
                          vertex_offset, out);
}

int lyon_gpu_stroke_paths_each(lyon_gpu_context* ctx, const lyon_path_batch* batch,
                               const lyon_stroke_options* options, uint32_t num_options,
                               int index_bits, uint32_t first, uint32_t count,
                               uint64_t* total_vertices) {
    if (!ctx || !batch || !options || !total_vertices || num_options == 0 ||
        (num_options != 1 && num_options != batch->num_paths) || first > batch->num_paths ||
        count > batch->num_paths - first)
        return LYON_ERR_INVALID_ARGUMENT;
    uint64_t tv = 0;
    for (uint32_t p = first; p < first + count; ++p) {
        // A one-path view of the batch (offsets stay absolute).
        lyon_path_batch one = *batch;
        one.verb_offsets = batch->verb_offsets + p;
        one.point_offsets = batch->point_offsets + p;
        one.num_paths = 1;
        lyon_gpu_batch_output out;
        const int r = batched_device(ctx, KIND_STROKE, &one, options + (num_options > 1 ? p : 0),
                                     1, index_bits, LYON_INDEX_PER_PATH, 0, &out);
        if (r != LYON_OK) return r;
        tv += out.total_vertices;
    }
    *total_vertices = tv;
    return LYON_OK;
}

int lyon_gpu_svg_parse_paths(lyon_gpu_context* ctx, const char* text,
                             const uint64_t* string_offsets, uint32_t num_strings,
                             const lyon_svg_parse_options* options, lyon_gpu_svg_output* out) {
    if (!ctx || !out || (num_strings && (!text || !string_offsets)) || num_strings > 0x7FFFFFFEu)
        return LYON_ERR_INVALID_ARGUMENT;
    const uint32_t num_attributes = options ? options->num_attributes : 0;
    if (num_attributes > 1) return LYON_ERR_UNSUPPORTED;
    const long long stop_at = options ? options->stop_at : -1;
    cudaSetDevice(ctx->device);
    memset(out, 0, sizeof(*out));
    const uint32_t n = num_strings;
    cudaStream_t s = ctx->stream;
    if (!ensure(ctx, ctx->svg_counts, (size_t)n * 8 + 16) ||
        !ensure(ctx, ctx->svg_diag, (size_t)n * 12 + 16) ||
        !ensure(ctx, ctx->svg_off64, ((size_t)n + 1) * 16) ||
        !ensure(ctx, ctx->svg_off32, ((size_t)n + 1) * 8) ||
        !ensure(ctx, ctx->scan_state, 2 * lg::scan_tile_count(n) * 8 + 16))
        return LYON_ERR_OUT_OF_MEMORY;
    uint32_t* vc = as<uint32_t>(ctx->svg_counts);
    uint32_t* pc = vc + n;
    int32_t* st = as<int32_t>(ctx->svg_diag);
    int32_t* el = st + n;
    int32_t* ec = el + n;
    uint64_t* voff = as<uint64_t>(ctx->svg_off64);
    uint64_t* poff = voff + n + 1;
    uint32_t* sw = small_words(ctx);
    if (!set_err(ctx, "svg count",
                 lg::launch_svg_parse(text, string_offsets, n, num_attributes, stop_at, false, vc,
                                      pc, st, el, ec, nullptr, nullptr, nullptr, nullptr,
                                      nullptr, ctx->num_sms, s)))
        return LYON_ERR_CUDA;
    cudaMemsetAsync(sw + 2, 0, 8, s);
    if (!set_err(ctx, "svg scan",
                 lg::launch_scan_pairs(vc, pc, voff, poff, n,
                                       as<unsigned long long>(ctx->scan_state), sw + 1,
                                       reinterpret_cast<int*>(sw + 2), s)) ||
        !set_err(ctx, "svg failures",
                 lg::launch_per_path_limit(vc, pc, st, n, 0, ~0ull, sw + 3, s)))
        return LYON_ERR_CUDA;
    uint64_t h[3] = {0, 0, 0};
    cudaMemcpyAsync(&h[0], voff + n, 8, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(&h[1], poff + n, 8, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(&h[2], sw + 2, 8, cudaMemcpyDeviceToHost, s);
    if (!set_err(ctx, "sync", cudaStreamSynchronize(s))) return LYON_ERR_CUDA;
    if ((uint32_t)h[2] != 0) {
        ctx->last_error = "scan look-back wait exceeded its bound";
        return LYON_ERR_CUDA;
    }
    if (h[0] > 0xFFFFFFFFull || h[1] > 0xFFFFFFFFull) return LYON_ERR_UNSUPPORTED;
    if (!ensure(ctx, ctx->svg_verbs, h[0] + 16) || !ensure(ctx, ctx->svg_points, h[1] * 8 + 16) ||
        (num_attributes && !ensure(ctx, ctx->svg_widths, h[1] * 4 + 16)))
        return LYON_ERR_OUT_OF_MEMORY;
    uint32_t* voff32 = as<uint32_t>(ctx->svg_off32);
    uint32_t* poff32 = voff32 + n + 1;
    float* widths = num_attributes ? as<float>(ctx->svg_widths) : nullptr;
    if (!set_err(ctx, "svg write",
                 lg::launch_svg_parse(text, string_offsets, n, num_attributes, stop_at, true,
                                      nullptr, nullptr, nullptr, nullptr, nullptr, voff, poff,
                                      as<uint8_t>(ctx->svg_verbs), as<float>(ctx->svg_points),
                                      widths, ctx->num_sms, s)) ||
        !set_err(ctx, "svg offsets", lg::launch_narrow_u64(voff, voff32, n + 1, s)) ||
        !set_err(ctx, "svg offsets", lg::launch_narrow_u64(poff, poff32, n + 1, s)))
        return LYON_ERR_CUDA;
    out->batch.verbs = as<uint8_t>(ctx->svg_verbs);
    out->batch.points = as<float>(ctx->svg_points);
    out->batch.verb_offsets = voff32;
    out->batch.point_offsets = poff32;
    out->batch.num_paths = n;
    out->widths = widths;
    out->status = st;
    out->error_line = el;
    out->error_column = ec;
    out->total_verbs = h[0];
    out->total_points = h[1];
    out->num_failed = (uint32_t)(h[2] >> 32);
    return LYON_OK;
}

int lyon_gpu_stroke_paths_attributes(lyon_gpu_context* ctx, const lyon_path_batch* batch,
                                     const lyon_stroke_options* options, uint32_t num_options,
                                     int index_bits, int index_mode, uint32_t vertex_offset,
                                     lyon_gpu_batch_output* out) {
    if (!ctx) return LYON_ERR_INVALID_ARGUMENT;
    ctx->vertex_attrs = true;
    int r = batched_device(ctx, KIND_STROKE, batch, options, num_options, index_bits, index_mode,
                           vertex_offset, out);
    ctx->vertex_attrs = false;
    return r;
}

int lyon_gpu_stroke_paths_variable_width(lyon_gpu_context* ctx, const lyon_path_batch* batch,
                                         const float* widths,
                                         const lyon_stroke_options* options,
                                         uint32_t num_options, int index_bits, int index_mode,
                                         uint32_t vertex_offset, int vertex_attributes,
                                         lyon_gpu_batch_output* out) {
    if (!ctx || (!widths && batch && batch->num_paths > 0)) return LYON_ERR_INVALID_ARGUMENT;
    ctx->vertex_attrs = vertex_attributes != 0;
    ctx->vw_widths = widths;
    int r = batched_device(ctx, KIND_STROKE, batch, options, num_options, index_bits, index_mode,
                           vertex_offset, out);
    ctx->vertex_attrs = false;
    ctx->vw_widths = nullptr;
    return r;
}

int lyon_gpu_fill_shapes(lyon_gpu_context* ctx, int shape_kind, const float* params,
                         uint32_t num_shapes, const lyon_fill_options* options,
                         uint32_t num_options, int index_bits, int index_mode,
                         uint32_t vertex_offset, lyon_gpu_batch_output* out) {
    const uint32_t n = num_shapes;
    const bool circles = shape_kind == LYON_SHAPE_CIRCLE;
    if (!ctx || !out || (shape_kind != LYON_SHAPE_RECTANGLE && !circles) || (n && !params) ||
        (index_bits != 16 && index_bits != 32) ||
        (index_mode != LYON_INDEX_GLOBAL && index_mode != LYON_INDEX_PER_PATH) ||
        (circles && (!options || (num_options != 1 && num_options != n)))) {
        if (ctx) ctx->last_error = "invalid argument";
        return LYON_ERR_INVALID_ARGUMENT;
    }
    cudaSetDevice(ctx->device);
    memset(out, 0, sizeof(*out));
    if (!alloc_path_arrays(ctx, n)) return LYON_ERR_OUT_OF_MEMORY;
    cudaStream_t s = ctx->stream;
    lg::ShapeArgs a;
    memset(&a, 0, sizeof a);
    a.kind = shape_kind;
    a.params = params;
    a.n = n;
    a.options = options;
    a.num_options = num_options;
    a.vtx_counts = as<uint32_t>(ctx->vtx_counts);
    a.idx_counts = as<uint32_t>(ctx->idx_counts);
    a.status = as<int32_t>(ctx->status);
    a.index_bits = index_bits;
    a.index_mode = index_mode;
    a.vertex_offset = vertex_offset;
    mark(ctx, 0);
    if (!set_err(ctx, "shapes count", lg::launch_shapes(a, false, s))) return LYON_ERR_CUDA;
    mark(ctx, 1);
    uint64_t tv = 0, ti = 0;
    uint32_t failed = 0;
    if (!finish_counts(ctx, n, index_bits, index_mode, vertex_offset, &tv, &ti, &failed))
        return LYON_ERR_CUDA;
    mark(ctx, 2);
    if (!ensure(ctx, ctx->out_vertices, tv * 8 + 16) ||
        !ensure(ctx, ctx->out_indices, ti * (index_bits / 8) + 16))
        return LYON_ERR_OUT_OF_MEMORY;
    a.vtx_offsets = as<uint64_t>(ctx->vtx_offsets);
    a.idx_offsets = as<uint64_t>(ctx->idx_offsets);
    a.vertices = as<float>(ctx->out_vertices);
    a.indices = ctx->out_indices.ptr;
    if (tv > 0 && !set_err(ctx, "shapes emit", lg::launch_shapes(a, true, s)))
        return LYON_ERR_CUDA;
    mark(ctx, 3);
    if (ctx->timing) {
        cudaEventSynchronize(ctx->ev[3]);
        cudaEventElapsedTime(&ctx->last_ms[0], ctx->ev[0], ctx->ev[1]);
        cudaEventElapsedTime(&ctx->last_ms[1], ctx->ev[1], ctx->ev[2]);
        cudaEventElapsedTime(&ctx->last_ms[2], ctx->ev[2], ctx->ev[3]);
        cudaEventElapsedTime(&ctx->last_ms[3], ctx->ev[0], ctx->ev[3]);
    }
    out->vertices = as<float>(ctx->out_vertices);
    out->indices = ctx->out_indices.ptr;
    out->vertex_offsets = as<uint64_t>(ctx->vtx_offsets);
    out->index_offsets = as<uint64_t>(ctx->idx_offsets);
    out->status = as<int32_t>(ctx->status);
    out->total_vertices = tv;
    out->total_indices = ti;
    out->num_failed_paths = failed;
    return LYON_OK;
}

int lyon_gpu_fill_paths(lyon_gpu_context* ctx, const lyon_path_batch* batch,
                        const lyon_fill_options* options, uint32_t num_options, int index_bits,
                        int index_mode, uint32_t vertex_offset, lyon_gpu_batch_output* out) {
    return batched_device(ctx, KIND_FILL, batch, options, num_options, index_bits, index_mode,
                          vertex_offset, out);
}

int lyon_gpu_stroke_paths_host(lyon_gpu_context* ctx, const lyon_path_batch* batch,
                               const lyon_stroke_options* options, uint32_t num_options,
                               int index_bits, int index_mode, uint32_t vertex_offset,
                               float* vertices, uint64_t vertex_capacity, void* indices,
                               uint64_t index_capacity, int32_t* status,
                               uint64_t* total_vertices, uint64_t* total_indices) {
    return batched_host(ctx, KIND_STROKE, batch, options, sizeof(lyon_stroke_options),
                        num_options, index_bits, index_mode, vertex_offset, vertices,
                        vertex_capacity, indices, index_capacity, status, total_vertices,
                        total_indices);
}

int lyon_gpu_fill_paths_host(lyon_gpu_context* ctx, const lyon_path_batch* batch,
                             const lyon_fill_options* options, uint32_t num_options,
                             int index_bits, int index_mode, uint32_t vertex_offset,
                             float* vertices, uint64_t vertex_capacity, void* indices,
                             uint64_t index_capacity, int32_t* status, uint64_t* total_vertices,
                             uint64_t* total_indices) {
    return batched_host(ctx, KIND_FILL, batch, options, sizeof(lyon_fill_options), num_options,
                        index_bits, index_mode, vertex_offset, vertices, vertex_capacity,
                        indices, index_capacity, status, total_vertices, total_indices);
}

int lyon_gpu_stroke_path(lyon_gpu_context* ctx, const uint8_t* verbs, uint32_t num_verbs,
                         const float* points, uint32_t num_points,
                         const lyon_stroke_options* options, int index_bits, uint32_t index_base,
                         lyon_gpu_result* result) {
    return single_path(ctx, KIND_STROKE, verbs, num_verbs, points, num_points, options,
                       sizeof(lyon_stroke_options), index_bits, index_base, result);
}

int lyon_gpu_stroke_path_attributes(lyon_gpu_context* ctx, const uint8_t* verbs,
                                    uint32_t num_verbs, const float* points, uint32_t num_points,
                                    const lyon_stroke_options* options, int index_bits,
                                    uint32_t index_base, lyon_gpu_result* result) {
    if (!ctx) return LYON_ERR_INVALID_ARGUMENT;
    ctx->vertex_attrs = true;
    int r = single_path(ctx, KIND_STROKE, verbs, num_verbs, points, num_points, options,
                        sizeof(lyon_stroke_options), index_bits, index_base, result);
    ctx->vertex_attrs = false;
    return r;
}

int lyon_gpu_stroke_path_variable_width(lyon_gpu_context* ctx, const uint8_t* verbs,
                                        uint32_t num_verbs, const float* points,
                                        uint32_t num_points, const float* widths,
                                        const lyon_stroke_options* options, int index_bits,
                                        uint32_t index_base, int vertex_attributes,
                                        lyon_gpu_result* result) {
    if (!ctx || (num_points && !widths)) return LYON_ERR_INVALID_ARGUMENT;
    static const float kNoPoints = 1.0f;
    ctx->vertex_attrs = vertex_attributes != 0;
    int r = single_path(ctx, KIND_STROKE, verbs, num_verbs, points, num_points, options,
                        sizeof(lyon_stroke_options), index_bits, index_base, result,
                        num_points ? widths : &kNoPoints);
    ctx->vertex_attrs = false;
    ctx->vw_widths = nullptr;
    ctx->width_stride = 1;
    return r;
}

int lyon_gpu_stroke_paths_custom(lyon_gpu_context* ctx, const lyon_path_batch* batch,
                                 const float* attributes, uint32_t num_attributes,
                                 int32_t width_attribute, const lyon_stroke_options* options,
                                 uint32_t num_options, int index_bits, int index_mode,
                                 uint32_t vertex_offset, int vertex_attributes,
                                 lyon_gpu_batch_output* out, lyon_gpu_custom_output* custom) {
    if (!ctx || !custom || width_attribute < -1 ||
        (width_attribute >= 0 && (uint32_t)width_attribute >= num_attributes) ||
        (num_attributes > 0 && !attributes && batch && batch->num_paths > 0))
        return LYON_ERR_INVALID_ARGUMENT;
    memset(custom, 0, sizeof(*custom));
    ctx->vertex_attrs = vertex_attributes != 0;
    ctx->vw_widths = width_attribute >= 0 ? attributes + width_attribute : nullptr;
    ctx->width_stride = num_attributes ? num_attributes : 1;
    ctx->want_sources = true;
    int r = batched_device(ctx, KIND_STROKE, batch, options, num_options, index_bits, index_mode,
                           vertex_offset, out);
    ctx->vertex_attrs = false;
    ctx->vw_widths = nullptr;
    ctx->width_stride = 1;
    ctx->want_sources = false;
    if (r != LYON_OK) return r;
    custom->sources = as<lyon_vertex_source>(ctx->out_sources);
    if (num_attributes > 0 && out->total_vertices > 0) {
        if (!ensure(ctx, ctx->out_attrs, out->total_vertices * num_attributes * 4 + 16))
            return LYON_ERR_OUT_OF_MEMORY;
        // The sources come from the batch's own points: every id is in range.
        if (!set_err(ctx, "interpolate",
                     lg::launch_interpolate(custom->sources, out->total_vertices, attributes,
                                            num_attributes, ~0ull, as<float>(ctx->out_attrs),
                                            ctx->num_sms, ctx->stream)))
            return LYON_ERR_CUDA;
        custom->attributes = as<float>(ctx->out_attrs);
    }
    return LYON_OK;
}

int lyon_gpu_interpolate_attributes(lyon_gpu_context* ctx, const lyon_vertex_source* sources,
                                    uint64_t num_vertices, const float* attributes,
                                    uint32_t num_attributes, uint64_t num_endpoints, float* out) {
    if (!ctx || (num_vertices && num_attributes && (!sources || !attributes || !out)))
        return LYON_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    if (!set_err(ctx, "interpolate",
                 lg::launch_interpolate(sources, num_vertices, attributes, num_attributes,
                                        num_endpoints, out, ctx->num_sms, ctx->stream)))
        return LYON_ERR_CUDA;
    return LYON_OK;
}

int lyon_gpu_stroke_path_custom(lyon_gpu_context* ctx, const uint8_t* verbs, uint32_t num_verbs,
                                const float* points, uint32_t num_points,
                                const float* attributes, uint32_t num_attributes,
                                int32_t width_attribute, const lyon_stroke_options* options,
                                int index_bits, uint32_t index_base, int vertex_attributes,
                                lyon_gpu_result* result, const lyon_vertex_source** sources,
                                const float** vertex_attribute_values) {
    if (!ctx || width_attribute < -1 ||
        (width_attribute >= 0 && (uint32_t)width_attribute >= num_attributes) ||
        (num_attributes > 0 && num_points > 0 && !attributes))
        return LYON_ERR_INVALID_ARGUMENT;
    if (sources) *sources = nullptr;
    if (vertex_attribute_values) *vertex_attribute_values = nullptr;
    // A path without points still stages one (unread) float per attribute.
    static const float kNoPoints[1] = {1.0f};
    const float* pf = num_attributes == 0 ? nullptr : (num_points ? attributes : kNoPoints);
    const uint32_t fpp = num_attributes == 0 ? 1 : (num_points ? num_attributes : 1);
    ctx->vertex_attrs = vertex_attributes != 0;
    ctx->want_sources = true;
    int r = single_path(ctx, KIND_STROKE, verbs, num_verbs, points, num_points, options,
                        sizeof(lyon_stroke_options), index_bits, index_base, result, pf, fpp,
                        num_points ? width_attribute : (width_attribute >= 0 ? 0 : -1));
    ctx->vertex_attrs = false;
    ctx->want_sources = false;
    ctx->vw_widths = nullptr;
    ctx->width_stride = 1;
    if (r == LYON_OK) {
        if (sources) *sources = reinterpret_cast<const lyon_vertex_source*>(ctx->h_out_src.ptr);
        if (vertex_attribute_values && num_attributes)
            *vertex_attribute_values = reinterpret_cast<const float*>(ctx->h_out_attrs.ptr);
    }
    return r;
}

int lyon_gpu_fill_paths_custom(lyon_gpu_context* ctx, const lyon_path_batch* batch,
                               const float* attributes, uint32_t num_attributes,
                               const lyon_fill_options* options, uint32_t num_options,
                               int index_bits, int index_mode, uint32_t vertex_offset,
                               lyon_gpu_batch_output* out, lyon_gpu_fill_custom_output* custom) {
    if (!ctx || !custom || (num_attributes > 0 && !attributes && batch && batch->num_paths > 0))
        return LYON_ERR_INVALID_ARGUMENT;
    memset(custom, 0, sizeof(*custom));
    ctx->want_sources = true;
    int r = batched_device(ctx, KIND_FILL, batch, options, num_options, index_bits, index_mode,
                           vertex_offset, out);
    ctx->want_sources = false;
    if (r != LYON_OK) return r;
    custom->sources = as<lyon_vertex_source>(ctx->out_sources);
    custom->source_offsets = as<uint64_t>(ctx->out_source_offsets);
    custom->total_sources = ctx->total_sources;
    if (num_attributes > 0 && out->total_vertices > 0) {
        if (!ensure(ctx, ctx->out_attrs, out->total_vertices * num_attributes * 4 + 16))
            return LYON_ERR_OUT_OF_MEMORY;
        // The sources come from the batch's own points: every id is in range.
        if (!set_err(ctx, "interpolate",
                     lg::launch_interpolate_fill(custom->sources, custom->source_offsets,
                                                 out->total_vertices, attributes,
                                                 num_attributes, ~0ull,
                                                 as<float>(ctx->out_attrs), ctx->num_sms,
                                                 ctx->stream)))
            return LYON_ERR_CUDA;
        custom->attributes = as<float>(ctx->out_attrs);
    }
    return LYON_OK;
}

int lyon_gpu_interpolate_fill_attributes(lyon_gpu_context* ctx,
                                         const lyon_vertex_source* sources,
                                         const uint64_t* source_offsets, uint64_t num_vertices,
                                         const float* attributes, uint32_t num_attributes,
                                         uint64_t num_endpoints, float* out) {
    if (!ctx || (num_vertices && num_attributes &&
                 (!sources || !source_offsets || !attributes || !out)))
        return LYON_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    if (!set_err(ctx, "interpolate",
                 lg::launch_interpolate_fill(sources, source_offsets, num_vertices, attributes,
                                             num_attributes, num_endpoints, out, ctx->num_sms,
                                             ctx->stream)))
        return LYON_ERR_CUDA;
    return LYON_OK;
}

int lyon_gpu_fill_path_custom(lyon_gpu_context* ctx, const uint8_t* verbs, uint32_t num_verbs,
                              const float* points, uint32_t num_points, const float* attributes,
                              uint32_t num_attributes, const lyon_fill_options* options,
                              int index_bits, uint32_t index_base, lyon_gpu_result* result,
                              const lyon_vertex_source** sources,
                              const uint64_t** source_offsets,
                              const float** vertex_attribute_values) {
    if (!ctx || (num_attributes > 0 && num_points > 0 && !attributes))
        return LYON_ERR_INVALID_ARGUMENT;
    if (sources) *sources = nullptr;
    if (source_offsets) *source_offsets = nullptr;
    if (vertex_attribute_values) *vertex_attribute_values = nullptr;
    static const float kNoPoints[1] = {0.0f};
    const float* pf = num_attributes == 0 ? nullptr : (num_points ? attributes : kNoPoints);
    const uint32_t fpp = num_attributes == 0 ? 1 : (num_points ? num_attributes : 1);
    ctx->want_sources = true;
    int r = single_path(ctx, KIND_FILL, verbs, num_verbs, points, num_points, options,
                        sizeof(lyon_fill_options), index_bits, index_base, result, pf, fpp, -1);
    ctx->want_sources = false;
    if (r == LYON_OK) {
        if (sources) *sources = reinterpret_cast<const lyon_vertex_source*>(ctx->h_out_src.ptr);
        if (source_offsets)
            *source_offsets = reinterpret_cast<const uint64_t*>(ctx->h_out_soff.ptr);
        if (vertex_attribute_values && num_attributes)
            *vertex_attribute_values = reinterpret_cast<const float*>(ctx->h_out_attrs.ptr);
    }
    return r;
}

int lyon_gpu_fill_path(lyon_gpu_context* ctx, const uint8_t* verbs, uint32_t num_verbs,
                       const float* points, uint32_t num_points, const lyon_fill_options* options,
                       int index_bits, uint32_t index_base, lyon_gpu_result* result) {
    return single_path(ctx, KIND_FILL, verbs, num_verbs, points, num_points, options,
                       sizeof(lyon_fill_options), index_bits, index_base, result);
}

int lyon_gpu_flatten_counts(lyon_gpu_context* ctx, const lyon_path_batch* batch, float tolerance,
                            uint32_t* counts) {
    if (!ctx || !batch || !counts) return LYON_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    if (batch->num_paths == 0) return LYON_OK;
    lg::FlattenArgs a;
    memset(&a, 0, sizeof a);
    a.verbs = batch->verbs;
    a.points = batch->points;
    a.verb_offsets = batch->verb_offsets;
    a.point_offsets = batch->point_offsets;
    a.num_paths = batch->num_paths;
    a.tolerance = tolerance;
    a.counts = counts;
    return set_err(ctx, "flatten counts",
                   lg::launch_flatten(a, false, ctx->num_sms * 8, ctx->stream))
               ? LYON_OK
               : LYON_ERR_CUDA;
}

namespace {

// Exclusive scan of n u32 counts into n + 1 u64 offsets (the second scan output is scratch);
// returns the total through *total (one synchronisation).
int scan_counts(lyon_gpu_context* ctx, const uint32_t* counts, uint64_t* offsets,
                uint64_t* scratch, uint32_t n, uint64_t* total) {
    cudaStream_t s = ctx->stream;
    *total = 0;
    if (!ensure(ctx, ctx->scan_state, 2 * lg::scan_tile_count(n) * 8 + 16) ||
        !ensure(ctx, ctx->small, 64) || !ensure_host(ctx, ctx->h_small, 64))
        return LYON_ERR_OUT_OF_MEMORY;
    if (n == 0) {
        cudaMemsetAsync(offsets, 0, 8, s);
        return LYON_OK;
    }
    uint32_t* sw = small_words(ctx);
    cudaMemsetAsync(sw + 2, 0, 4, s);
    if (!set_err(ctx, "scan",
                 lg::launch_scan_pairs(counts, counts, offsets, scratch, n,
                                       as<unsigned long long>(ctx->scan_state), sw + 1,
                                       reinterpret_cast<int*>(sw + 2), s)))
        return LYON_ERR_CUDA;
    uint64_t* hs = reinterpret_cast<uint64_t*>(ctx->h_small.ptr);
    cudaMemcpyAsync(hs, offsets + n, 8, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(hs + 1, sw + 2, 4, cudaMemcpyDeviceToHost, s);
    if (!set_err(ctx, "sync", cudaStreamSynchronize(s))) return LYON_ERR_CUDA;
    if (reinterpret_cast<uint32_t*>(hs + 1)[0] != 0) {
        ctx->last_error = "scan look-back wait exceeded its bound";
        return LYON_ERR_CUDA;
    }
    *total = hs[0];
    return LYON_OK;
}

int hatch_impl(lyon_gpu_context* ctx, const lyon_path_batch* batch,
               const lyon_hatching_options* o, bool dots, lyon_gpu_hatch_output* out) {
    if (!ctx || !batch || !o || !out) return LYON_ERR_INVALID_ARGUMENT;
    memset(out, 0, sizeof(*out));
    cudaSetDevice(ctx->device);
    cudaStream_t s = ctx->stream;
    const uint32_t n = batch->num_paths;
    lg::HatchArgs a;
    memset(&a, 0, sizeof a);
    a.verbs = batch->verbs;
    a.points = batch->points;
    a.verb_offsets = batch->verb_offsets;
    a.point_offsets = batch->point_offsets;
    a.num_paths = n;
    a.tolerance = o->tolerance;
    // Rotation::new(angle) and Rotation::new(-angle) (euclid: f32 cos and sin).
    a.c = cosf(o->angle);
    a.s = sinf(o->angle);
    a.ci = cosf(-o->angle);
    a.si = sinf(-o->angle);
    a.uv_x = o->uv_origin_x;
    a.uv_y = o->uv_origin_y;
    a.interval = o->interval;
    a.column_interval = o->column_interval;
    a.compute_tangents = dots ? 0 : (o->compute_tangents != 0);
    a.dots = dots ? 1 : 0;
    if (!ensure(ctx, ctx->hatch_bound, (size_t)n * 4 + 16) ||
        !ensure(ctx, ctx->hatch_edge_count, (size_t)n * 4 + 16) ||
        !ensure(ctx, ctx->hatch_counts, (size_t)n * 4 + 16) ||
        !ensure(ctx, ctx->hatch_status, (size_t)n * 4 + 16) ||
        !ensure(ctx, ctx->hatch_offsets, ((size_t)n + 1) * 8 * 3 + 16))
        return LYON_ERR_OUT_OF_MEMORY;
    a.edge_bound = as<uint32_t>(ctx->hatch_bound);
    a.edge_count = as<uint32_t>(ctx->hatch_edge_count);
    a.counts = as<uint32_t>(ctx->hatch_counts);
    a.status = as<int32_t>(ctx->hatch_status);
    uint64_t* scr_off = as<uint64_t>(ctx->hatch_offsets);
    uint64_t* out_off = scr_off + n + 1;
    uint64_t* tmp_off = out_off + n + 1;
    if (!set_err(ctx, "hatch bound", lg::launch_hatch(a, 0, ctx->num_sms, s)))
        return LYON_ERR_CUDA;
    uint64_t edges = 0, total = 0;
    int r = scan_counts(ctx, a.edge_bound, scr_off, tmp_off, n, &edges);
    if (r != LYON_OK) return r;
    if (!ensure(ctx, ctx->hatch_scratch, edges * 16 * 3 + 16) ||
        !ensure(ctx, ctx->hatch_order, (size_t)n * 5 + lg::SIZE_ORDER_BINS * 8 + 16))
        return LYON_ERR_OUT_OF_MEMORY;
    a.scratch_offsets = scr_off;
    a.scratch_total = edges;
    a.scratch = ctx->hatch_scratch.ptr;
    // One thread per path: both passes take the paths largest first (by edge count, then by
    // output count), so that the 32 paths of a warp take similar times.
    uint32_t* order = as<uint32_t>(ctx->hatch_order);
    uint32_t* counters = order + n;
    uint8_t* cls = reinterpret_cast<uint8_t*>(counters + 2 * lg::SIZE_ORDER_BINS);
    a.order = order;
    if (!set_err(ctx, "hatch order",
                 lg::launch_size_order(nullptr, n, cls, order, counters, s, a.edge_bound)) ||
        !set_err(ctx, "hatch count", lg::launch_hatch(a, 1, ctx->num_sms, s)))
        return LYON_ERR_CUDA;
    r = scan_counts(ctx, a.counts, out_off, tmp_off, n, &total);
    if (r != LYON_OK) return r;
    const size_t rec = dots ? sizeof(lyon_dot) : sizeof(lyon_hatch_segment);
    if (!ensure(ctx, ctx->hatch_out, total * rec + 16)) return LYON_ERR_OUT_OF_MEMORY;
    a.out_offsets = out_off;
    if (total > 0 &&
        !set_err(ctx, "hatch order",
                 lg::launch_size_order(nullptr, n, cls, order, counters, s, a.counts)))
        return LYON_ERR_CUDA;
    a.segments = reinterpret_cast<lyon_hatch_segment*>(ctx->hatch_out.ptr);
    a.dot_out = reinterpret_cast<lyon_dot*>(ctx->hatch_out.ptr);
    if (total > 0 && !set_err(ctx, "hatch emit", lg::launch_hatch(a, 2, ctx->num_sms, s)))
        return LYON_ERR_CUDA;
    out->segments = dots ? nullptr : a.segments;
    out->dots = dots ? a.dot_out : nullptr;
    out->offsets = out_off;
    out->status = a.status;
    out->total = total;
    return LYON_OK;
}

}  // namespace

int lyon_gpu_hatch_paths(lyon_gpu_context* ctx, const lyon_path_batch* batch,
                         const lyon_hatching_options* options, lyon_gpu_hatch_output* out) {
    return hatch_impl(ctx, batch, options, false, out);
}

int lyon_gpu_dot_paths(lyon_gpu_context* ctx, const lyon_path_batch* batch,
                       const lyon_hatching_options* options, lyon_gpu_hatch_output* out) {
    return hatch_impl(ctx, batch, options, true, out);
}

int lyon_gpu_flatten_arcs(lyon_gpu_context* ctx, const lyon_arc* arcs, uint32_t num_arcs,
                          float tolerance, lyon_gpu_arc_output* out) {
    if (!ctx || !out || (num_arcs && !arcs)) return LYON_ERR_INVALID_ARGUMENT;
    memset(out, 0, sizeof(*out));
    cudaSetDevice(ctx->device);
    cudaStream_t s = ctx->stream;
    const uint32_t n = num_arcs;
    if (!ensure(ctx, ctx->arc_counts, (size_t)n * 4 + 16) ||
        !ensure(ctx, ctx->arc_status, (size_t)n * 4 + 16) ||
        !ensure(ctx, ctx->arc_offsets, ((size_t)n + 1) * 8 * 2 + 16) ||
        !ensure(ctx, ctx->scan_state, 2 * lg::scan_tile_count(n) * 8 + 16) ||
        !ensure(ctx, ctx->small, 64) || !ensure_host(ctx, ctx->h_small, 64))
        return LYON_ERR_OUT_OF_MEMORY;
    uint64_t* offs = as<uint64_t>(ctx->arc_offsets);
    uint64_t total = 0;
    if (!ensure(ctx, ctx->arc_order, (size_t)n * 5 + lg::SIZE_ORDER_BINS * 8 + 16))
        return LYON_ERR_OUT_OF_MEMORY;
    // Both passes take the arcs largest first (the count pass by an estimate, the emit pass by
    // the counts), so that the 32 arcs of a warp take similar numbers of steps.
    uint32_t* order = as<uint32_t>(ctx->arc_order);
    uint32_t* counters = order + n;
    uint8_t* cls = reinterpret_cast<uint8_t*>(counters + 2 * lg::SIZE_ORDER_BINS);
    if (n > 0) {
        if (!set_err(ctx, "arcs estimate",
                     lg::launch_arcs_estimate(arcs, n, tolerance, as<uint32_t>(ctx->arc_counts),
                                              ctx->num_sms, s)) ||
            !set_err(ctx, "arcs order",
                     lg::launch_size_order(nullptr, n, cls, order, counters, s,
                                           as<uint32_t>(ctx->arc_counts))) ||
            !set_err(ctx, "arcs count",
                     lg::launch_arcs(arcs, n, tolerance, as<uint32_t>(ctx->arc_counts),
                                     as<int32_t>(ctx->arc_status), nullptr, nullptr, nullptr,
                                     ctx->num_sms, s, order)))
            return LYON_ERR_CUDA;
        uint32_t* sw = small_words(ctx);
        cudaMemsetAsync(sw + 2, 0, 4, s);
        if (!set_err(ctx, "scan",
                     lg::launch_scan_pairs(as<uint32_t>(ctx->arc_counts),
                                           as<uint32_t>(ctx->arc_counts), offs, offs + n + 1, n,
                                           as<unsigned long long>(ctx->scan_state), sw + 1,
                                           reinterpret_cast<int*>(sw + 2), s)))
            return LYON_ERR_CUDA;
        uint64_t* hs = reinterpret_cast<uint64_t*>(ctx->h_small.ptr);
        cudaMemcpyAsync(hs, offs + n, 8, cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(hs + 1, sw + 2, 4, cudaMemcpyDeviceToHost, s);
        if (!set_err(ctx, "sync", cudaStreamSynchronize(s))) return LYON_ERR_CUDA;
        if (reinterpret_cast<uint32_t*>(hs + 1)[0] != 0) {
            ctx->last_error = "scan look-back wait exceeded its bound";
            return LYON_ERR_CUDA;
        }
        total = hs[0];
    } else {
        cudaMemsetAsync(offs, 0, 8, s);
    }
    if (!ensure(ctx, ctx->arc_points, total * 8 + 16) ||
        !ensure(ctx, ctx->arc_t, total * 4 + 16))
        return LYON_ERR_OUT_OF_MEMORY;
    if (n > 0 && total > 0 &&
        (!set_err(ctx, "arcs order",
                  lg::launch_size_order(nullptr, n, cls, order, counters, s,
                                        as<uint32_t>(ctx->arc_counts))) ||
         !set_err(ctx, "arcs emit",
                  lg::launch_arcs(arcs, n, tolerance, nullptr, as<int32_t>(ctx->arc_status),
                                  offs, as<float>(ctx->arc_points), as<float>(ctx->arc_t),
                                  ctx->num_sms, s, order))))
        return LYON_ERR_CUDA;
    out->points = as<float>(ctx->arc_points);
    out->t = as<float>(ctx->arc_t);
    out->offsets = offs;
    out->status = as<int32_t>(ctx->arc_status);
    out->total_points = total;
    return LYON_OK;
}

int lyon_gpu_flatten_paths(lyon_gpu_context* ctx, const lyon_path_batch* batch, float tolerance,
                           float** out_points, uint32_t** out_offsets, uint64_t* total_points) {
    if (!ctx || !batch || !out_points || !out_offsets || !total_points)
        return LYON_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    cudaStream_t s = ctx->stream;
    uint32_t nv = 0;
    if (!ensure_host(ctx, ctx->h_small, 64)) return LYON_ERR_OUT_OF_MEMORY;
    if (batch->num_paths > 0) {
        if (!set_err(ctx, "D2H verb count",
                     cudaMemcpyAsync(ctx->h_small.ptr, batch->verb_offsets + batch->num_paths, 4,
                                     cudaMemcpyDeviceToHost, s)) ||
            !set_err(ctx, "sync", cudaStreamSynchronize(s)))
            return LYON_ERR_CUDA;
        nv = *reinterpret_cast<uint32_t*>(ctx->h_small.ptr);
    }
    if (!ensure(ctx, ctx->flat_counts, (size_t)nv * 4 + 16) ||
        !ensure(ctx, ctx->flat_offsets, ((size_t)nv + 1) * 8 * 2 + 16) ||
        !ensure(ctx, ctx->scan_state, 2 * lg::scan_tile_count(nv) * 8 + 16))
        return LYON_ERR_OUT_OF_MEMORY;
    int r = lyon_gpu_flatten_counts(ctx, batch, tolerance, as<uint32_t>(ctx->flat_counts));
    if (r != LYON_OK) return r;
    uint64_t* offs = as<uint64_t>(ctx->flat_offsets);
    uint64_t* offs2 = offs + nv + 1;
    uint32_t* sw = small_words(ctx);
    cudaMemsetAsync(sw + 2, 0, 4, s);
    if (!set_err(ctx, "scan",
                 lg::launch_scan_pairs(as<uint32_t>(ctx->flat_counts),
                                       as<uint32_t>(ctx->flat_counts), offs, offs2, nv,
                                       as<unsigned long long>(ctx->scan_state), sw + 1,
                                       reinterpret_cast<int*>(sw + 2), s)))
        return LYON_ERR_CUDA;
    cudaMemcpyAsync(ctx->h_small.ptr, offs + nv, 8, cudaMemcpyDeviceToHost, s);
    if (!set_err(ctx, "sync", cudaStreamSynchronize(s))) return LYON_ERR_CUDA;
    uint64_t total = *reinterpret_cast<uint64_t*>(ctx->h_small.ptr);
    if (!ensure(ctx, ctx->flat_points, total * 8 + 16)) return LYON_ERR_OUT_OF_MEMORY;
    lg::FlattenArgs a;
    memset(&a, 0, sizeof a);
    a.verbs = batch->verbs;
    a.points = batch->points;
    a.verb_offsets = batch->verb_offsets;
    a.point_offsets = batch->point_offsets;
    a.num_paths = batch->num_paths;
    a.tolerance = tolerance;
    a.offsets = offs;
    a.out_points = as<float>(ctx->flat_points);
    if (batch->num_paths > 0 &&
        !set_err(ctx, "flatten points", lg::launch_flatten(a, true, ctx->num_sms * 8, s)))
        return LYON_ERR_CUDA;
    *out_points = as<float>(ctx->flat_points);
    *out_offsets = reinterpret_cast<uint32_t*>(offs2);
    if (!set_err(ctx, "narrow offsets",
                 lg::launch_narrow_u64(offs, reinterpret_cast<uint32_t*>(offs2), nv + 1, s)))
        return LYON_ERR_CUDA;
    *total_points = total;
    return LYON_OK;
}

}  // extern "C"
