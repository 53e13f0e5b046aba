// fill.cu — batched fill tessellation: lyon's sweep-line FillTessellator, one thread per path
// (several per warp).
//
// Pipeline (per batched call):
//   1. fill_sweep_kernel: a persistent grid of sweeper threads (several per warp) takes paths
//      from an atomic counter. Each sweeper builds the path's event queue (event_queue.rs:
//      441-905: downward-oriented edges, curves flattened with their t ranges, vertex events
//      at local maxima), sorts it with lyon's linked-list merge sort (event_queue.rs:301-384,
//      same recursion so equal positions form the same sibling chains), runs the sweep
//      (fill.rs:749-2151) and the monotone tessellators (monotone.rs), writing vertices and
//      triangles (path-relative ids) into its private heap; at the end it reserves room in a
//      staging pool with one atomic add and copies them there.
//   2. the caller's index-range check and look-back scan turn the per-path counts into offsets;
//   3. fill_emit_kernel: one warp per path copies the staged vertices to their final place and
//      the indices with the path's id base added (u16 or u32).
// A path whose heap or staging room ran out is re-run, alone with the other such paths, with
// more room; after the last attempt it fails with LYON_ERR_CAPACITY.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "fill.h"
#include "kernels.h"
#include "fill_sweep.cuh"

namespace lg {
namespace fillk {

constexpr int32_t STATUS_RETRY = -1;

#ifndef LG_FILL_SWEEPERS_PER_SM
#define LG_FILL_SWEEPERS_PER_SM 16
#endif
#ifndef LG_FILL_MIN_BLOCKS
#define LG_FILL_MIN_BLOCKS 16
#endif
#ifndef LG_FILL_LANES
#define LG_FILL_LANES 12
#endif
// 32-thread blocks per SM; the first `lanes` threads of each block are sweepers, each with its
// own path and heap: as many lanes as the launch has paths per block (rounded down), between 1
// and LG_FILL_LANES (LYON_GB300_FILL_LANES forces a lane count, 1 to 32, for every launch). On
// 200,000 glyph paths the non-zero sweep took 1800 / 1717 / 1551 / 1643 / 2400 ms with 1 / 4 /
// 8 / 16 / 32 lanes at 32 blocks per SM (64 registers, small spills): diverged lanes run one
// after another, so more than 8 loses again. With 96 registers and no spills, 20 blocks per SM
// took 1462 / 1491 / 1443 ms with 8 / 12 / 16 lanes, 24 blocks (80 registers) 1442 ms with 8,
// and 16 blocks 1487 / 1310 ms with 8 / 12 lanes (192 sweepers per SM, 7.5 GB of heaps).
constexpr uint32_t FILL_SWEEPERS_PER_SM = LG_FILL_SWEEPERS_PER_SM;
// Heaps of all sweepers together stay under this many bytes (fewer blocks when larger).
constexpr size_t FILL_HEAP_POOL_BYTES = 16ull << 30;

struct SweepArgs {
    const uint8_t* verbs;
    const float* points;
    const uint32_t* verb_offsets;
    const uint32_t* point_offsets;
    const lyon_fill_options* options;
    uint32_t num_options;
    const uint32_t* order;  // null: item = path
    uint32_t num_items;
    uint32_t lanes;         // sweepers per block (its first threads)
    uint32_t* counters;     // [0] work, [1] retry count, [2] paths whose heap ran out
    unsigned long long* stage_tops;  // [0] vertices, [1] indices
    uint32_t* heaps;
    uint32_t heap_words;
    float2* stage_v;
    uint32_t* stage_i;
    unsigned long long stage_v_cap, stage_i_cap;
    unsigned long long* stage_off;  // per path: vertex base, index base
    uint32_t* vtx_counts;
    uint32_t* idx_counts;
    int32_t* status;
    uint32_t* retry_list;
    int final_attempt;
    // vertex sources (null src_counts: not requested)
    uint32_t* src_counts;
    uint32_t* stage_s;
    uint32_t* stage_sfirst;
    unsigned long long stage_s_cap;  // in sources
    unsigned long long* stage_soff;
};

template <bool SRC>
__global__ void __launch_bounds__(32, LG_FILL_MIN_BLOCKS) fill_sweep_kernel(SweepArgs A) {
    // Each of the block's first `lanes` threads sweeps its own paths with its own heap. The
    // sweep's control flow depends on the path, so lanes diverge; where they run the same code
    // (the event loop's common steps) one instruction fetch serves several paths.
    if (threadIdx.x >= A.lanes) return;
    const uint32_t wid = blockIdx.x * A.lanes + threadIdx.x;
    FillerT<SRC> f;
    f.h.w = A.heaps + (size_t)wid * A.heap_words;
    f.h.cap = A.heap_words;
    for (;;) {
        const uint32_t item = atomicAdd(&A.counters[0], 1u);
        if (item >= A.num_items) break;
        const uint32_t path = A.order ? A.order[item] : item;
        const uint32_t v0 = A.verb_offsets[path], v1 = A.verb_offsets[path + 1];
        const uint32_t p0 = A.point_offsets[path], p1 = A.point_offsets[path + 1];
        const lyon_fill_options o = A.options[A.num_options > 1 ? path : 0];
        f.h.reset();
        f.tessellate(A.verbs + v0, v1 - v0, A.points + 2 * (size_t)p0, p1 - p0, o);
        int32_t st = f.err;
        uint32_t nv = 0, ni = 0, ns = 0;
        if (st == LYON_OK) {
            nv = f.out_v.n;
            ni = f.out_i.n;
            ns = f.out_src.n / 3;
            const unsigned long long vb = atomicAdd(&A.stage_tops[0], (unsigned long long)nv);
            const unsigned long long ib = atomicAdd(&A.stage_tops[1], (unsigned long long)ni);
            unsigned long long sb = 0;
            if (SRC) sb = atomicAdd(&A.stage_tops[2], (unsigned long long)ns);
            if (vb + nv > A.stage_v_cap || ib + ni > A.stage_i_cap ||
                (SRC && sb + ns > A.stage_s_cap)) {
                st = STATUS_RETRY;
            } else {
                if (SRC) {
                    const uint32_t* ss = f.out_src.p(f.h);
                    for (uint32_t i = 0; i < 3 * ns; ++i) A.stage_s[3 * sb + i] = ss[i];
                    const uint32_t* sf = f.out_sfirst.p(f.h);
                    for (uint32_t i = 0; i < nv; ++i) A.stage_sfirst[vb + i] = sf[i];
                    A.stage_soff[path] = sb;
                }
                const V2* sv = f.out_v.p(f.h);
                for (uint32_t i = 0; i < nv; ++i) A.stage_v[vb + i] = make_float2(sv[i].x, sv[i].y);
                const uint32_t* si = f.out_i.p(f.h);
                for (uint32_t i = 0; i < ni; ++i) A.stage_i[ib + i] = si[i];
                A.stage_off[2 * (size_t)path] = vb;
                A.stage_off[2 * (size_t)path + 1] = ib;
            }
        } else if (st == FILL_ERR_HEAP) {
            st = STATUS_RETRY;
            atomicAdd(&A.counters[2], 1u);
        }
        if (st == STATUS_RETRY) {
            if (A.final_attempt) {
                st = LYON_ERR_CAPACITY;
            } else {
                const uint32_t r = atomicAdd(&A.counters[1], 1u);
                A.retry_list[r] = path;
            }
        }
        A.vtx_counts[path] = st == LYON_OK ? nv : 0u;
        A.idx_counts[path] = st == LYON_OK ? ni : 0u;
        if (SRC) A.src_counts[path] = st == LYON_OK ? ns : 0u;
        A.status[path] = st;
    }
}

// One warp per path: the staged sources of a successful path to their final offsets (ids made
// batch-global) and every vertex's first source.
__global__ void fill_emit_sources_kernel(uint32_t n, const uint32_t* vtx_counts,
                                         const int32_t* status,
                                         const unsigned long long* stage_off,
                                         const unsigned long long* stage_soff,
                                         const uint32_t* stage_s, const uint32_t* stage_sfirst,
                                         const uint64_t* vtx_offsets, FillSourceArgs S) {
    const uint32_t warps = gridDim.x * (blockDim.x / 32);
    const uint32_t lane = threadIdx.x & 31;
    for (uint32_t p = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32; p < n; p += warps) {
        if (status[p] != LYON_OK) continue;
        const uint32_t nv = vtx_counts[p];
        const uint64_t so = S.src_offsets[p];
        const uint32_t ns = (uint32_t)(S.src_offsets[p + 1] - so);
        const unsigned long long sb = stage_soff[p], vb = stage_off[2 * (size_t)p];
        const uint32_t base = S.point_offsets[p];
        for (uint32_t k = lane; k < ns; k += 32) {
            const uint32_t* w = stage_s + 3 * (sb + k);
            const uint32_t to = w[1];
            S.sources[so + k] = lyon_vertex_source{w[0] + base,
                                                   to == LYON_NO_ENDPOINT ? to : to + base,
                                                   __uint_as_float(w[2])};
        }
        const uint64_t vo = vtx_offsets[p];
        for (uint32_t i = lane; i < nv; i += 32) S.source_offsets[vo + i] = so + stage_sfirst[vb + i];
    }
}

// One warp per path: staged output to the final buffers, ids rebased.
__global__ void fill_emit_kernel(uint32_t n, const uint32_t* vtx_counts,
                                 const uint32_t* idx_counts, const int32_t* status,
                                 const unsigned long long* stage_off, const float2* stage_v,
                                 const uint32_t* stage_i, const uint64_t* vtx_offsets,
                                 const uint64_t* idx_offsets, float2* vertices, void* indices,
                                 int index_bits, int index_mode, uint32_t vertex_offset,
                                 const uint32_t* request_first) {
    const uint32_t warps = gridDim.x * (blockDim.x / 32);
    const uint32_t lane = threadIdx.x & 31;
    for (uint32_t p = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32; p < n; p += warps) {
        if (status[p] != LYON_OK) continue;
        const uint32_t nv = vtx_counts[p], ni = idx_counts[p];
        const unsigned long long sv = stage_off[2 * (size_t)p], si = stage_off[2 * (size_t)p + 1];
        const uint64_t vo = vtx_offsets[p], io = idx_offsets[p];
        const uint64_t rb = request_first ? vtx_offsets[request_first[p]] : 0ull;
        const uint32_t base =
            vertex_offset + (index_mode == LYON_INDEX_GLOBAL ? (uint32_t)(vo - rb) : 0u);
        for (uint32_t i = lane; i < nv; i += 32) vertices[vo + i] = stage_v[sv + i];
        if (index_bits == 16) {
            uint16_t* d = reinterpret_cast<uint16_t*>(indices) + io;
            for (uint32_t i = lane; i < ni; i += 32) d[i] = (uint16_t)(stage_i[si + i] + base);
        } else {
            uint32_t* d = reinterpret_cast<uint32_t*>(indices) + io;
            for (uint32_t i = lane; i < ni; i += 32) d[i] = stage_i[si + i] + base;
        }
    }
}

}  // namespace fillk

namespace {

// With a pool the old buffer is freed in stream order, without waiting for the device.
bool grow(void** p, size_t* cap, size_t bytes, size_t keep_bytes, cudaStream_t s,
          cudaMemPool_t pool) {
    if (bytes <= *cap && *p) return true;
    void* np = nullptr;
    size_t nc = bytes + bytes / 4 + 256;
    const cudaError_t e = pool ? cudaMallocFromPoolAsync(&np, nc, pool, s) : cudaMalloc(&np, nc);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (*p) {
        if (keep_bytes) cudaMemcpyAsync(np, *p, keep_bytes, cudaMemcpyDeviceToDevice, s);
        if (pool) {
            cudaFreeAsync(*p, s);
        } else {
            cudaStreamSynchronize(s);
            cudaFree(*p);
        }
    }
    *p = np;
    *cap = nc;
    return true;
}

}  // namespace

int fill_count(FillBuffers& fb, const lyon_path_batch* batch, const lyon_fill_options* options,
               uint32_t num_options, int num_sms, uint32_t* vtx_counts, uint32_t* idx_counts,
               int32_t* status, uint32_t* small_words, cudaStream_t stream, std::string* error,
               const FillSourceArgs* src) {
    const uint32_t n = batch->num_paths;
    if (n == 0) return LYON_OK;
    const bool sources = src && src->src_counts;
    // Counters: [0] work, [1] retries, [2] heap overflows; two u64 staging tops; two retry
    // lists.
    // After them: the size-order scratch (counters, one byte per path).
    const size_t ctl_bytes = 64 + (size_t)n * 8 + 2 * SIZE_ORDER_BINS * 4 + (size_t)n;
    if (!grow(&fb.work, &fb.work_cap, ctl_bytes, 0, stream, fb.pool) ||
        !grow(&fb.stage_off, &fb.stage_off_cap, (size_t)n * 16, 0, stream, fb.pool)) {
        if (error) *error = "cudaMalloc (fill control arrays)";
        return LYON_ERR_OUT_OF_MEMORY;
    }
    uint32_t* counters = reinterpret_cast<uint32_t*>(fb.work);
    unsigned long long* tops = reinterpret_cast<unsigned long long*>(
        reinterpret_cast<char*>(fb.work) + 16);
    uint32_t* lists[2] = {reinterpret_cast<uint32_t*>(reinterpret_cast<char*>(fb.work) + 64),
                          reinterpret_cast<uint32_t*>(reinterpret_cast<char*>(fb.work) + 64) + n};
    // Sweepers (one per warp) and heaps; heaps start at 64 K words (256 KB), which covers nearly
    // every glyph-sized path.
    const uint32_t per_sm =
        fb.blocks_per_sm_cap > 0 && fb.blocks_per_sm_cap < (uint32_t)fillk::FILL_SWEEPERS_PER_SM
            ? fb.blocks_per_sm_cap
            : (uint32_t)fillk::FILL_SWEEPERS_PER_SM;
    const uint32_t threads = (uint32_t)(num_sms > 0 ? num_sms : 1) * per_sm;
    if (fb.heap_words == 0) fb.heap_words = 65536;
    // Staging: start from a guess of 4 vertices and 12 indices per input point.
    if (fb.stage_v_cap == 0) {
        uint32_t npts = 0;
        cudaMemcpyAsync(&npts, batch->point_offsets + n, 4, cudaMemcpyDeviceToHost, stream);
        cudaStreamSynchronize(stream);
        const size_t guess_v = (size_t)npts * 4 + 4096;
        if (!grow(&fb.stage_v, &fb.stage_v_cap, guess_v * 8, 0, stream, fb.pool) ||
            !grow(&fb.stage_i, &fb.stage_i_cap, guess_v * 3 * 4, 0, stream, fb.pool)) {
            if (error) *error = "cudaMalloc (fill staging)";
            return LYON_ERR_OUT_OF_MEMORY;
        }
    }
    // Source staging: about one source per vertex, one first-source word per staged vertex.
    if (sources &&
        (!grow(&fb.stage_s, &fb.stage_s_cap, std::max<size_t>(fb.stage_v_cap / 8 * 12, 4096), 0,
               stream, fb.pool) ||
         !grow(&fb.stage_sfirst, &fb.stage_sfirst_cap, fb.stage_v_cap / 8 * 4 + 256, 0, stream,
               fb.pool) ||
         !grow(&fb.stage_soff, &fb.stage_soff_cap, (size_t)n * 8, 0, stream, fb.pool))) {
        if (error) *error = "cudaMalloc (fill source staging)";
        return LYON_ERR_OUT_OF_MEMORY;
    }
    cudaMemsetAsync(tops, 0, 24, stream);
    // Big paths first, so that the last paths a sweeper takes are short ones and the launch
    // does not end on one long sweep. The order lives in the second retry list, which the first
    // attempt does not write.
    uint32_t* size_counters = lists[1] + n;
    uint8_t* size_cls = reinterpret_cast<uint8_t*>(size_counters + 2 * SIZE_ORDER_BINS);
    const uint32_t* order = nullptr;
    if (launch_size_order(batch->point_offsets, n, size_cls, lists[1], size_counters, stream) ==
        cudaSuccess)
        order = lists[1];
    uint32_t items = n;
    uint32_t max_lanes = LG_FILL_LANES;
    bool forced = false;
    if (fb.lanes >= 1 && fb.lanes <= 32) max_lanes = fb.lanes, forced = true;
    if (const char* env = getenv("LYON_GB300_FILL_LANES")) {
        const long v = strtol(env, nullptr, 10);
        if (v >= 1 && v <= 32) max_lanes = (uint32_t)v, forced = true;
    }
    const int MAX_ATTEMPTS = 4;
    for (int attempt = 0; attempt < MAX_ATTEMPTS; ++attempt) {
        uint32_t nthreads = threads;
        // A lane shares its warp's issue slots with the other lanes, so a path on a shared warp
        // takes longer than alone: lanes are added only when there are two or more paths per
        // block (large batches, for throughput), never for a small launch (a served request, the
        // retry of a few paths), whose latency is one path's sweep.
        uint32_t lanes = forced ? max_lanes
                                : std::max<uint32_t>(1u, std::min<uint32_t>(max_lanes,
                                                                            items / nthreads));
        size_t heap_bytes = (size_t)fb.heap_words * 4 * nthreads * lanes;
        // Keep the heaps under the pool size: fewer blocks when each heap is large.
        while (heap_bytes > fillk::FILL_HEAP_POOL_BYTES && nthreads > 4) {
            nthreads /= 2;
            heap_bytes /= 2;
        }
        if (!grow(&fb.scratch, &fb.scratch_cap, heap_bytes, 0, stream, fb.pool)) {
            if (error) *error = "cudaMalloc (fill heaps)";
            return LYON_ERR_OUT_OF_MEMORY;
        }
        cudaMemsetAsync(counters, 0, 12, stream);
        fillk::SweepArgs a;
        a.verbs = batch->verbs;
        a.points = batch->points;
        a.verb_offsets = batch->verb_offsets;
        a.point_offsets = batch->point_offsets;
        a.options = options;
        a.num_options = num_options;
        a.order = order;
        a.num_items = items;
        a.lanes = lanes;
        a.counters = counters;
        a.stage_tops = tops;
        a.heaps = reinterpret_cast<uint32_t*>(fb.scratch);
        a.heap_words = fb.heap_words;
        a.stage_v = reinterpret_cast<float2*>(fb.stage_v);
        a.stage_i = reinterpret_cast<uint32_t*>(fb.stage_i);
        a.stage_v_cap = fb.stage_v_cap / 8;
        a.stage_i_cap = fb.stage_i_cap / 4;
        a.stage_off = reinterpret_cast<unsigned long long*>(fb.stage_off);
        a.vtx_counts = vtx_counts;
        a.idx_counts = idx_counts;
        a.status = status;
        a.retry_list = lists[attempt & 1];
        a.final_attempt = attempt == MAX_ATTEMPTS - 1;
        a.src_counts = sources ? src->src_counts : nullptr;
        a.stage_s = reinterpret_cast<uint32_t*>(fb.stage_s);
        a.stage_sfirst = reinterpret_cast<uint32_t*>(fb.stage_sfirst);
        a.stage_s_cap = fb.stage_s_cap / 12;
        a.stage_soff = reinterpret_cast<unsigned long long*>(fb.stage_soff);
        if (sources) {
            fillk::fill_sweep_kernel<true><<<nthreads, 32, 0, stream>>>(a);
        } else {
            fillk::fill_sweep_kernel<false><<<nthreads, 32, 0, stream>>>(a);
        }
        lg::note_launches(1);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) {
            if (error) *error = std::string("fill sweep: ") + cudaGetErrorString(e);
            return LYON_ERR_CUDA;
        }
        uint32_t h_ctl[3];
        unsigned long long h_tops[3];
        cudaMemcpyAsync(h_ctl, counters, 12, cudaMemcpyDeviceToHost, stream);
        cudaMemcpyAsync(h_tops, tops, 24, cudaMemcpyDeviceToHost, stream);
        e = cudaStreamSynchronize(stream);
        if (e != cudaSuccess) {
            if (error) *error = std::string("fill sweep: ") + cudaGetErrorString(e);
            return LYON_ERR_CUDA;
        }
        if (h_ctl[1] == 0) break;
        // Some paths ran out of heap or staging room: more of both, then only those paths.
        // The staging tops stay where they are (the failed reservations are abandoned).
        const bool staging_short =
            h_tops[0] > fb.stage_v_cap / 8 || h_tops[1] > fb.stage_i_cap / 4;
        if (sources && h_tops[2] > fb.stage_s_cap / 12) {
            const size_t used_s = std::min<size_t>(h_tops[2], fb.stage_s_cap / 12);
            if (!grow(&fb.stage_s, &fb.stage_s_cap, (size_t)h_tops[2] * 2 * 12 + 4096,
                      used_s * 12, stream, fb.pool)) {
                if (error) *error = "cudaMalloc (fill source staging)";
                return LYON_ERR_OUT_OF_MEMORY;
            }
        }
        if (staging_short) {
            const size_t used_v = std::min<size_t>(h_tops[0], fb.stage_v_cap / 8);
            const size_t used_i = std::min<size_t>(h_tops[1], fb.stage_i_cap / 4);
            if (!grow(&fb.stage_v, &fb.stage_v_cap, (size_t)h_tops[0] * 2 * 8 + 4096,
                      used_v * 8, stream, fb.pool) ||
                !grow(&fb.stage_i, &fb.stage_i_cap, (size_t)h_tops[1] * 2 * 4 + 4096,
                      used_i * 4, stream, fb.pool) ||
                (sources && !grow(&fb.stage_sfirst, &fb.stage_sfirst_cap,
                                  (size_t)h_tops[0] * 2 * 4 + 4096, used_v * 4, stream,
                                  fb.pool))) {
                if (error) *error = "cudaMalloc (fill staging)";
                return LYON_ERR_OUT_OF_MEMORY;
            }
        }
        if (h_ctl[2] > 0) fb.heap_words *= 4;
        order = lists[attempt & 1];
        items = h_ctl[1];
    }
    (void)small_words;
    return LYON_OK;
}

cudaError_t fill_emit(FillBuffers& fb, uint32_t n, const uint32_t* vtx_counts,
                      const uint32_t* idx_counts, const int32_t* status,
                      const uint64_t* vtx_offsets, const uint64_t* idx_offsets, float* vertices,
                      void* indices, int index_bits, int index_mode, uint32_t vertex_offset,
                      const uint32_t* request_first, cudaStream_t stream,
                      const FillSourceArgs* src) {
    if (n == 0) return cudaSuccess;
    if (src && src->sources) {
        fillk::fill_emit_sources_kernel<<<std::min<uint32_t>((n + 7) / 8, 4096u), 256, 0,
                                          stream>>>(
            n, vtx_counts, status, reinterpret_cast<const unsigned long long*>(fb.stage_off),
            reinterpret_cast<const unsigned long long*>(fb.stage_soff),
            reinterpret_cast<const uint32_t*>(fb.stage_s),
            reinterpret_cast<const uint32_t*>(fb.stage_sfirst), vtx_offsets, *src);
        lg::note_launches(1);
    }
    const uint32_t blocks = std::min<uint32_t>((n + 7) / 8, 4096u);
    fillk::fill_emit_kernel<<<blocks, 256, 0, stream>>>(
        n, vtx_counts, idx_counts, status,
        reinterpret_cast<const unsigned long long*>(fb.stage_off),
        reinterpret_cast<const float2*>(fb.stage_v), reinterpret_cast<const uint32_t*>(fb.stage_i),
        vtx_offsets, idx_offsets, reinterpret_cast<float2*>(vertices), indices, index_bits,
        index_mode, vertex_offset, request_first);
    lg::note_launches(1);
    return cudaGetLastError();
}

namespace fillk {
__global__ void zero_failed_counts_kernel(uint32_t* counts, const int32_t* status, uint32_t n) {
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x)
        if (status[p] != LYON_OK) counts[p] = 0u;
}
}  // namespace fillk

cudaError_t fill_zero_failed_source_counts(uint32_t* src_counts, const int32_t* status,
                                           uint32_t n, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    fillk::zero_failed_counts_kernel<<<std::min<uint32_t>((n + 255) / 256, 1024u), 256, 0,
                                       stream>>>(src_counts, status, n);
    lg::note_launches(1);
    return cudaGetLastError();
}

void fill_free(FillBuffers& fb) {
    void* bufs[] = {fb.scratch, fb.stage_v,      fb.stage_i,   fb.stage_off,
                    fb.work,    fb.stage_s, fb.stage_sfirst, fb.stage_soff};
    for (void* b : bufs)
        if (b) cudaFree(b);
    fb = FillBuffers();
}

}  // namespace lg
