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
};

// Runs the sweep of every path into staging and writes per-path vertex/index counts and status.
int fill_count(FillBuffers& fb, const lyon_path_batch* batch, const lyon_fill_options* options,
               uint32_t num_options, int num_sms, uint32_t* vtx_counts, uint32_t* idx_counts,
               int32_t* status, uint32_t* small_words, cudaStream_t stream,
               std::string* error);

// Copies the staged output of every successful path to its final offsets, rebasing indices
// (`request_first`: optional per-path first path of its request, as in StrokeArgs).
cudaError_t fill_emit(FillBuffers& fb, uint32_t n, const uint32_t* vtx_counts,
                      const uint32_t* idx_counts, const int32_t* status,
                      const uint64_t* vtx_offsets, const uint64_t* idx_offsets, float* vertices,
                      void* indices, int index_bits, int index_mode, uint32_t vertex_offset,
                      const uint32_t* request_first, cudaStream_t stream);

void fill_free(FillBuffers& fb);

}  // namespace lg
