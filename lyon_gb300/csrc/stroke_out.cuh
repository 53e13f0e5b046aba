// stroke_out.cuh — where one path's stroke output goes (shared by the warp-per-path kernel in
// stroke.cu and the sequential stepper in stroke_seq.cu).
#pragma once
#include "stroke_core.cuh"
#include "kernels.h"

namespace lg {

// Points a verb consumes in the batch layout (Close stores the sub-path's first point again).
__device__ __forceinline__ uint32_t points_of_verb(int kind) {
    switch (kind) {
        case LYON_VERB_LINE_TO: return 1;
        case LYON_VERB_QUADRATIC_TO: return 2;
        case LYON_VERB_CUBIC_TO: return 3;
        case LYON_VERB_BEGIN: return 1;
        case LYON_VERB_CLOSE: return 1;
        default: return 0;
    }
}

struct PathOut {
    uint32_t id_base;  // id of the path's first vertex
    float2* vout;      // positions; null when counting or writing attribute records
    lyon_stroke_vertex* rout;  // attribute records (the attribute output), else null
    void* iout;
    int bits;
    uint32_t vmax, imax;  // the path's counts from the count pass (write bounds when emitting)
};

__device__ __forceinline__ uint32_t cap_left(uint32_t total, uint32_t used) {
    return used < total ? total - used : 0u;
}

template <bool EMIT, bool ATTR>
__device__ __forceinline__ PathOut path_out(const StrokeArgs& A, uint32_t path) {
    PathOut po;
    po.bits = A.index_bits;
    if (EMIT) {
        const uint64_t vo = A.vtx_offsets[path];
        const uint64_t io = A.idx_offsets[path];
        po.vout = ATTR ? nullptr : reinterpret_cast<float2*>(A.vertices) + vo;
        po.rout = ATTR ? reinterpret_cast<lyon_stroke_vertex*>(A.vertices) + vo : nullptr;
        po.iout = A.index_bits == 16 ? (void*)((uint16_t*)A.indices + io)
                                     : (void*)((uint32_t*)A.indices + io);
        const uint64_t rb = A.request_first ? A.vtx_offsets[A.request_first[path]] : 0ull;
        po.id_base =
            A.vertex_offset + (A.index_mode == LYON_INDEX_GLOBAL ? (uint32_t)(vo - rb) : 0u);
        po.vmax = A.vtx_counts[path];
        po.imax = A.idx_counts[path];
    } else {
        po.vout = nullptr;
        po.rout = nullptr;
        po.iout = nullptr;
        po.id_base = 0;
        po.vmax = 0xFFFFFFFFu;
        po.imax = 0xFFFFFFFFu;
    }
    return po;
}

// Final per-path bookkeeping: the count pass records counts and status; the emit pass flags a
// path whose walk disagreed with the count pass (its writes were bounded by the path's range).
template <bool EMIT>
__device__ __forceinline__ void finish_path(const StrokeArgs& A, uint32_t path, uint32_t vc,
                                            uint32_t ic, int st, const PathOut& po) {
    if (!EMIT) {
        A.vtx_counts[path] = st == LYON_OK ? vc : 0u;
        A.idx_counts[path] = st == LYON_OK ? ic : 0u;
        A.status[path] = st;
    } else if (st != LYON_OK || vc != po.vmax || ic != po.imax) {
        A.status[path] = st != LYON_OK ? st : LYON_ERR_INTERNAL;
    }
}

}  // namespace lg
