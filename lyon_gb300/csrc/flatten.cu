// flatten.cu — path flattening: per-verb segment counts and `path.iter().flattened(tol)`.
//
// One warp per path. Verbs are handled in windows of 32 (lane = verb): a warp scan of the
// points-per-verb gives each verb its points, lyon's `flattened_segments_wang` gives each curve
// its segment count (crates/geom/src/quadratic_bezier.rs:943-974,
// crates/geom/src/cubic_bezier.rs:1369-1403). The point pass then walks the window's output
// points 32 at a time (lane = output point) and evaluates lyon's Horner polynomial at the
// accumulated parameter (crates/geom/src/quadratic_bezier.rs:1004-1033 and
// crates/geom/src/cubic_bezier.rs:1434-1459 iterators).
#include "geom.cuh"
#include "kernels.h"
#include "kernels_flatten.h"

namespace lg {

constexpr uint32_t FFULL = 0xFFFFFFFFu;

__device__ __forceinline__ uint32_t fl_incl_scan(uint32_t v, int lane) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t n = __shfl_up_sync(FFULL, v, o);
        if (lane >= o) v += n;
    }
    return v;
}

__device__ __forceinline__ uint32_t fl_points_of_verb(int kind) {
    switch (kind) {
        case LYON_VERB_LINE_TO: return 1;
        case LYON_VERB_QUADRATIC_TO: return 2;
        case LYON_VERB_CUBIC_TO: return 3;
        case LYON_VERB_BEGIN: return 1;
        case LYON_VERB_CLOSE: return 1;
        default: return 0;
    }
}

template <bool WRITE_POINTS>
__global__ void flatten_kernel(FlattenArgs A) {
    const int lane = threadIdx.x & 31;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t path = warp; path < A.num_paths; path += nwarps) {
        const uint32_t v_begin = A.verb_offsets[path], v_end = A.verb_offsets[path + 1];
        uint32_t pc = A.point_offsets[path];
        const uint32_t p_end = A.point_offsets[path + 1];
        for (uint32_t vi = v_begin; vi < v_end; vi += 32) {
            uint32_t v = vi + lane;
            bool valid = v < v_end;
            int kind = valid ? (int)A.verbs[v] : LYON_VERB_END;
            uint32_t pcount = valid ? fl_points_of_verb(kind) : 0u;
            uint32_t pincl = fl_incl_scan(pcount, lane);
            uint32_t pofs = pc + pincl - pcount;
            uint32_t n = 0;
            float nf = 1.0f;
            Poly poly;
            V2 to = V2{0.0f, 0.0f};
            bool ok = valid && pofs + pcount <= p_end && pofs >= 1;
            if (ok && kind == LYON_VERB_LINE_TO) {
                n = 1;
                to = load_pt(A.points, pofs);
            } else if (ok && kind == LYON_VERB_QUADRATIC_TO) {
                V2 from = load_pt(A.points, pofs - 1);
                V2 c = load_pt(A.points, pofs);
                to = load_pt(A.points, pofs + 1);
                nf = quad_wang(from, c, to, A.tolerance);
                n = to_u32_or1(nf);
                poly = quad_poly(from, c, to);
            } else if (ok && kind == LYON_VERB_CUBIC_TO) {
                V2 from = load_pt(A.points, pofs - 1);
                V2 c1 = load_pt(A.points, pofs);
                V2 c2 = load_pt(A.points, pofs + 1);
                to = load_pt(A.points, pofs + 2);
                nf = cubic_wang(from, c1, c2, to, A.tolerance);
                n = to_u32_or1(nf);
                poly = cubic_poly(from, c1, c2, to);
            }
            if (!WRITE_POINTS) {
                if (valid) A.counts[v] = n;
            } else {
                // Window output positions.
                uint32_t nincl = fl_incl_scan(n, lane);
                uint32_t total = __shfl_sync(FFULL, nincl, 31);
                uint64_t wbase = valid ? A.offsets[v] - (nincl - n) : 0ull;
                wbase = __shfl_sync(FFULL, (unsigned long long)wbase, 0);
                float s = 1.0f / nf;
                for (uint32_t base = 0; base < total; base += 32) {
                    uint32_t gi = base + lane;
                    bool act = gi < total;
                    uint32_t lo = 0, hi = 31;
#pragma unroll
                    for (int it = 0; it < 5; ++it) {
                        uint32_t mid = (lo + hi) >> 1;
                        uint32_t vm = __shfl_sync(FFULL, nincl, mid);
                        if (vm > gi) hi = mid; else lo = mid + 1;
                        if (lo > hi) lo = hi;
                    }
                    uint32_t j = lo;
                    uint32_t sj = __shfl_sync(FFULL, nincl, j) - __shfl_sync(FFULL, n, j);
                    uint32_t nj = __shfl_sync(FFULL, n, j);
                    float sjs = __shfl_sync(FFULL, s, j);
                    V2 toj = V2{__shfl_sync(FFULL, to.x, j), __shfl_sync(FFULL, to.y, j)};
                    Poly pj;
                    pj.a0 = V2{__shfl_sync(FFULL, poly.a0.x, j), __shfl_sync(FFULL, poly.a0.y, j)};
                    pj.a1 = V2{__shfl_sync(FFULL, poly.a1.x, j), __shfl_sync(FFULL, poly.a1.y, j)};
                    pj.a2 = V2{__shfl_sync(FFULL, poly.a2.x, j), __shfl_sync(FFULL, poly.a2.y, j)};
                    pj.a3 = V2{__shfl_sync(FFULL, poly.a3.x, j), __shfl_sync(FFULL, poly.a3.y, j)};
                    int kj = __shfl_sync(FFULL, kind, j);
                    pj.cubic = kj == LYON_VERB_CUBIC_TO;
                    if (act) {
                        uint32_t k = gi - sj + 1;  // 1-based index within the verb
                        V2 p;
                        if (kj == LYON_VERB_LINE_TO || k >= nj) {
                            p = toj;
                        } else {
                            float t = accumulate_t(sjs, 0, 0.0f, k);
                            p = poly_sample(pj, t);
                        }
                        reinterpret_cast<float2*>(A.out_points)[wbase + gi] = make_float2(p.x, p.y);
                    }
                }
            }
            pc += __shfl_sync(FFULL, pincl, 31);
        }
    }
}

cudaError_t launch_flatten(const FlattenArgs& a, bool write_points, int grid, cudaStream_t s) {
    if (write_points) {
        flatten_kernel<true><<<grid, 256, 0, s>>>(a);
        note_launches(1);
    } else {
        flatten_kernel<false><<<grid, 256, 0, s>>>(a);
        note_launches(1);
    }
    return cudaGetLastError();
}

}  // namespace lg
