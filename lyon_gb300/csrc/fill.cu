// fill.cu — fill tessellation (placeholder until the sweep kernel lands).
#include "fill.h"

namespace lg {

int fill_count(FillBuffers&, const lyon_path_batch*, const lyon_fill_options*, uint32_t, int,
               uint32_t*, uint32_t*, int32_t*, uint32_t*, cudaStream_t, std::string* error) {
    if (error) *error = "fill is not built yet";
    return LYON_ERR_UNSUPPORTED;
}

cudaError_t fill_emit(FillBuffers&, uint32_t, const uint32_t*, const uint32_t*, const int32_t*,
                      const uint64_t*, const uint64_t*, float*, void*, int, int, uint32_t,
                      cudaStream_t) {
    return cudaErrorNotSupported;
}

void fill_free(FillBuffers& fb) {
    void* bufs[] = {fb.scratch, fb.stage_v, fb.stage_i, fb.stage_off, fb.work};
    for (void* b : bufs)
        if (b) cudaFree(b);
    fb = FillBuffers();
}

}  // namespace lg
