// kernels_flatten.h — launch interface of the flattening kernels.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/lyon_gpu.h"

namespace lg {

struct FlattenArgs {
    const uint8_t* verbs;
    const float* points;
    const uint32_t* verb_offsets;
    const uint32_t* point_offsets;
    uint32_t num_paths;
    float tolerance;
    uint32_t* counts;          // one per verb (count pass)
    const uint64_t* offsets;   // exclusive scan of counts (point pass)
    float* out_points;         // point pass output
};

cudaError_t launch_flatten(const FlattenArgs& a, bool write_points, int grid, cudaStream_t s);

}  // namespace lg
