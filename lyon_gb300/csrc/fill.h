// fill.h — launch interface of the fill sweep (fill.cu).
#pragma once

#include <cstdint>
#include <string>
#include <cuda_runtime.h>

#include "../../include/lyon_gpu.h"

namespace lg {

// Device buffers the fill pipeline keeps between its count and emit phases.
struct FillBuffers {
    void* scratch = nullptr;        // per-thread sweep heaps
    size_t scratch_cap = 0;
    void* stage_v = nullptr;        // staged vertices (f32 x2) per path
    size_t stage_v_cap = 0;
    void* stage_i = nullptr;        // staged indices (u32, path-relative) per path
    size_t stage_i_cap = 0;
    void* stage_off = nullptr;      // per path: staged vertex/index base (u64 x2)
    size_t stage_off_cap = 0;
    void* work = nullptr;           // counters, staging tops and retry lists
    size_t work_cap = 0;
    uint32_t heap_words = 0;        // per-thread sweep heap size (grows when a path needs more)
    // Most sweep blocks per SM (0: the default, FILL_SWEEPERS_PER_SM). The serving loop lowers
    // it so that stroke kernels launched meanwhile find room on every SM.
    uint32_t blocks_per_sm_cap = 0;
    // Sweepers per one-warp block (1..32); 0: chosen per launch from its paths per block.
    uint32_t lanes = 0;
    // When set, every buffer here comes from this pool in stream order (serving contexts).
    cudaMemPool_t pool = nullptr;
    // Vertex sources (FillVertex::sources), when a call asks for them:
    void* stage_s = nullptr;        // staged sources, three u32 words each, path-local ids
    size_t stage_s_cap = 0;
    void* stage_sfirst = nullptr;   // per staged vertex: its first source within its path
    size_t stage_sfirst_cap = 0;
    void* stage_soff = nullptr;     // per path: staged source base (u64)
    size_t stage_soff_cap = 0;
};

// The vertex-source side of a fill call: per-path source counts out of the sweep; at emit, the
// scanned per-path source offsets in and the final arrays out.
struct FillSourceArgs {
    uint32_t* src_counts;             // per path (sweep output)
    const uint64_t* src_offsets;      // per path (emit input)
    const uint32_t* point_offsets;    // the batch's, to make ids batch-global
    lyon_vertex_source* sources;      // emit output
    uint64_t* source_offsets;         // emit output, one per vertex
};

// Runs the sweep of every path into staging and writes per-path vertex/index counts and status.
// With `src` (src->src_counts set), every vertex's sources are staged too.
int fill_count(FillBuffers& fb, const lyon_path_batch* batch, const lyon_fill_options* options,
               uint32_t num_options, int num_sms, uint32_t* vtx_counts, uint32_t* idx_counts,
               int32_t* status, uint32_t* small_words, cudaStream_t stream,
               std::string* error, const FillSourceArgs* src = nullptr);

// Copies the staged output of every successful path to its final offsets, rebasing indices
// (`request_first`: optional per-path first path of its request, as in StrokeArgs).
cudaError_t fill_emit(FillBuffers& fb, uint32_t n, const uint32_t* vtx_counts,
                      const uint32_t* idx_counts, const int32_t* status,
                      const uint64_t* vtx_offsets, const uint64_t* idx_offsets, float* vertices,
                      void* indices, int index_bits, int index_mode, uint32_t vertex_offset,
                      const uint32_t* request_first, cudaStream_t stream,
                      const FillSourceArgs* src = nullptr);

// Source counts of paths that failed after the sweep (the index-range check) set to zero, so that
// the source scan skips them.
cudaError_t fill_zero_failed_source_counts(uint32_t* src_counts, const int32_t* status,
                                           uint32_t n, cudaStream_t stream);

void fill_free(FillBuffers& fb);

}  // namespace lg
