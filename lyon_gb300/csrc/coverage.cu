// coverage.cu — per-sample triangle coverage on a regular grid: the fill output check of
// covered samples, applied identically to two tessellations of the same paths.
//
// For each path a G x G grid of sample points spans the path's box [x0, x1] x [y0, y1]; sample
// (i, j) sits at (x0 + (i + 0.5) (x1 - x0) / G, y0 + (j + 0.5) (y1 - y0) / G), in f64. A
// triangle covers a sample that lies strictly inside it, or on one of its edges that the tie
// rule gives to it: every edge is evaluated from its lexicographically smaller end point (so two
// triangles that share an edge compute the same value with opposite signs) and a sample exactly
// on an edge belongs to the triangle whose edge, in counter-clockwise order, points down or, if
// horizontal, right. Triangles sharing an edge therefore cover each sample on it once, and a
// tessellation that covers a region exactly once gives every sample in it a count of 1, however
// the region is cut into triangles. Degenerate (zero-area) triangles cover nothing.
//
// One block rasterises COV_ROWS rows of one path: each triangle adds +1 / -1 at the ends of its
// covered run of samples in every row (each end estimated from where an edge crosses the row,
// then settled by the exact per-sample test, which is monotone along a row), then a prefix sum
// per row gives each sample's count. Both tessellations go through the same code; the block adds to the path's
// totals the samples each one covers and the samples whose counts differ.
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/lyon_gpu.h"
#include "kernels.h"

namespace lg {
namespace {

constexpr int COV_ROWS = 4;  // rows per block
constexpr int COV_THREADS = 512;
constexpr uint32_t COV_MAX_GRID = 4096;

struct P2 {
    double x, y;
};

__device__ __forceinline__ bool lex_less(P2 a, P2 b) {
    return a.x < b.x || (a.x == b.x && a.y < b.y);
}

// Edge function of a -> b at (x, y): positive to the left of the edge. Evaluated from the
// lexicographically smaller end point, so that b -> a gives exactly the opposite value.
__device__ __forceinline__ double edge_fn(P2 a, P2 b, double x, double y) {
    if (lex_less(b, a)) {
        return -((a.x - b.x) * (y - b.y) - (a.y - b.y) * (x - b.x));
    }
    return (b.x - a.x) * (y - a.y) - (b.y - a.y) * (x - a.x);
}

// The tie rule: an edge of a counter-clockwise triangle keeps the samples on it when it points
// down, or right when horizontal. For the two directions of one edge exactly one qualifies.
__device__ __forceinline__ bool keeps_ties(P2 a, P2 b) {
    return (b.y < a.y) || (b.y == a.y && b.x > a.x);
}

struct Tri {
    P2 p[3];
    bool tie[3];
};

__device__ __forceinline__ bool covers_edge(const Tri& t, int k, double x, double y) {
    const double e = edge_fn(t.p[k], t.p[(k + 1) % 3], x, y);
    return e > 0.0 || (e == 0.0 && t.tie[k]);
}

struct Grid {
    double x0, y0, dx, dy;
    int g;
    __device__ double xs(int i) const { return x0 + ((double)i + 0.5) * dx; }
    __device__ double ys(int j) const { return y0 + ((double)j + 0.5) * dy; }
};

// The run [lo, hi) of samples of row y that triangle t covers, within [ilo, ihi). Along a row
// each edge's test is monotone in x, so each edge keeps a prefix or a suffix of the columns: its
// end is estimated from the edge's crossing of the row, then moved by the exact per-sample test
// until it sits where the test changes (the result is the same as a search over all columns).
__device__ void row_span(const Tri& t, const Grid& G, double y, int ilo, int ihi, int* lo,
                         int* hi) {
    int a = ilo, b = ihi;
    for (int k = 0; k < 3 && a < b; ++k) {
        const P2 p = t.p[k], q = t.p[(k + 1) % 3];
        // The edge function is decreasing in x when the edge goes up (q.y > p.y), increasing
        // when it goes down, constant when horizontal.
        if (q.y == p.y) {
            if (!covers_edge(t, k, G.xs(a), y)) b = a;
            continue;
        }
        const double xc = p.x + (y - p.y) * (q.x - p.x) / (q.y - p.y);
        double est = floor((xc - G.x0) / G.dx - 0.5);  // the last column left of the crossing
        if (!(est >= (double)(a - 1))) est = (double)(a - 1);
        if (est > (double)(b - 1)) est = (double)(b - 1);
        int c = (int)est;
        if (q.y > p.y) {
            // Covered columns form a prefix of [a, b): c = its last column (a - 1 if none).
            while (c + 1 < b && covers_edge(t, k, G.xs(c + 1), y)) ++c;
            while (c >= a && !covers_edge(t, k, G.xs(c), y)) --c;
            b = c + 1;
        } else {
            // Covered columns form a suffix: c + 1 = its first column.
            while (c >= a && covers_edge(t, k, G.xs(c), y)) --c;
            while (c + 1 < b && !covers_edge(t, k, G.xs(c + 1), y)) ++c;
            a = c + 1;
        }
    }
    *lo = a;
    *hi = b < a ? a : b;
}

struct CovSet {
    const float2* v;
    const uint32_t* idx;
    const uint64_t* voff;
    const uint64_t* ioff;
};

__device__ void raster_set(const CovSet& S, uint32_t path, const Grid& G, int j0, int* diff) {
    const uint64_t v0 = S.voff[path];
    const uint64_t i0 = S.ioff[path], i1 = S.ioff[path + 1];
    const uint64_t ntri = (i1 - i0) / 3;
    const double yb0 = G.ys(j0), yb1 = G.ys(j0 + COV_ROWS - 1);
    for (uint64_t tr = threadIdx.x; tr < ntri; tr += blockDim.x) {
        Tri t;
        for (int k = 0; k < 3; ++k) {
            const float2 f = S.v[v0 + S.idx[i0 + 3 * tr + k]];
            t.p[k] = P2{(double)f.x, (double)f.y};
        }
        const double area2 = (t.p[1].x - t.p[0].x) * (t.p[2].y - t.p[0].y) -
                             (t.p[1].y - t.p[0].y) * (t.p[2].x - t.p[0].x);
        if (!(area2 != 0.0)) continue;  // degenerate (or NaN): covers nothing
        if (area2 < 0.0) {
            const P2 s = t.p[1];
            t.p[1] = t.p[2];
            t.p[2] = s;
        }
        for (int k = 0; k < 3; ++k) t.tie[k] = keeps_ties(t.p[k], t.p[(k + 1) % 3]);
        const double ymin = fmin(t.p[0].y, fmin(t.p[1].y, t.p[2].y));
        const double ymax = fmax(t.p[0].y, fmax(t.p[1].y, t.p[2].y));
        if (ymax < yb0 || ymin > yb1) continue;
        const double xmin = fmin(t.p[0].x, fmin(t.p[1].x, t.p[2].x));
        const double xmax = fmax(t.p[0].x, fmax(t.p[1].x, t.p[2].x));
        // Sample columns that can lie in the triangle's box (one column of margin each side).
        double fl = floor((xmin - G.x0) / G.dx - 0.5) - 1.0;
        double fh = ceil((xmax - G.x0) / G.dx - 0.5) + 2.0;
        fl = fl < 0.0 ? 0.0 : (fl > (double)G.g ? (double)G.g : fl);
        fh = fh < 0.0 ? 0.0 : (fh > (double)G.g ? (double)G.g : fh);
        const int ilo = (int)fl, ihi = (int)fh;
        if (ilo >= ihi) continue;
        for (int r = 0; r < COV_ROWS; ++r) {
            const double y = G.ys(j0 + r);
            if (j0 + r >= G.g || y < ymin || y > ymax) continue;
            int lo, hi;
            row_span(t, G, y, ilo, ihi, &lo, &hi);
            if (hi > lo) {
                atomicAdd(&diff[r * (COV_MAX_GRID + 1) + lo], 1);
                atomicAdd(&diff[r * (COV_MAX_GRID + 1) + hi], -1);
            }
        }
    }
}

__global__ void __launch_bounds__(COV_THREADS)
    coverage_kernel(const float* boxes, uint32_t grid, CovSet A, CovSet B,
                    unsigned long long* counts) {
    extern __shared__ int smem[];
    int* da = smem;
    int* db = smem + COV_ROWS * (COV_MAX_GRID + 1);
    const uint32_t path = blockIdx.y;
    const int j0 = (int)blockIdx.x * COV_ROWS;
    const float* bx = boxes + 4 * (size_t)path;
    Grid G;
    G.x0 = bx[0];
    G.y0 = bx[1];
    G.dx = ((double)bx[2] - (double)bx[0]) / (double)grid;
    G.dy = ((double)bx[3] - (double)bx[1]) / (double)grid;
    G.g = (int)grid;
    for (int i = threadIdx.x; i < 2 * COV_ROWS * (int)(COV_MAX_GRID + 1); i += blockDim.x)
        smem[i] = 0;
    __syncthreads();
    raster_set(A, path, G, j0, da);
    raster_set(B, path, G, j0, db);
    __syncthreads();
    // Prefix sums: one warp per row, each lane a contiguous run of samples.
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned long long cov_a = 0, cov_b = 0, differ = 0;
    if (warp < COV_ROWS && j0 + warp < (int)grid) {
        const int per = ((int)grid + 31) / 32;
        const int s0 = min((int)grid, lane * per), s1 = min((int)grid, s0 + per);
        const int* ra = da + warp * (COV_MAX_GRID + 1);
        const int* rb = db + warp * (COV_MAX_GRID + 1);
        int sa = 0, sb = 0;
        for (int i = s0; i < s1; ++i) {
            sa += ra[i];
            sb += rb[i];
        }
        // Inclusive scan of the lanes' sums, then each lane's exclusive start.
        int pa = sa, pb = sb;
        for (int o = 1; o < 32; o <<= 1) {
            const int na = __shfl_up_sync(0xFFFFFFFFu, pa, o);
            const int nb = __shfl_up_sync(0xFFFFFFFFu, pb, o);
            if (lane >= o) {
                pa += na;
                pb += nb;
            }
        }
        int ca = pa - sa, cb = pb - sb;
        for (int i = s0; i < s1; ++i) {
            ca += ra[i];
            cb += rb[i];
            cov_a += ca > 0;
            cov_b += cb > 0;
            differ += ca != cb;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        cov_a += __shfl_down_sync(0xFFFFFFFFu, cov_a, o);
        cov_b += __shfl_down_sync(0xFFFFFFFFu, cov_b, o);
        differ += __shfl_down_sync(0xFFFFFFFFu, differ, o);
    }
    if (lane == 0 && warp < COV_ROWS && (cov_a | cov_b | differ)) {
        atomicAdd(&counts[3 * (size_t)path + 0], cov_a);
        atomicAdd(&counts[3 * (size_t)path + 1], cov_b);
        atomicAdd(&counts[3 * (size_t)path + 2], differ);
    }
}

}  // namespace
}  // namespace lg

extern "C" int lyon_gpu_coverage_compare(const float* boxes, uint32_t num_paths, uint32_t grid,
                                         const float* vertices_a, const uint32_t* indices_a,
                                         const uint64_t* vertex_offsets_a,
                                         const uint64_t* index_offsets_a,
                                         const float* vertices_b, const uint32_t* indices_b,
                                         const uint64_t* vertex_offsets_b,
                                         const uint64_t* index_offsets_b, uint64_t* counts,
                                         void* stream) {
    if (!boxes || !counts || grid == 0 || grid > lg::COV_MAX_GRID || num_paths > 65535 ||
        !vertex_offsets_a || !index_offsets_a || !vertex_offsets_b || !index_offsets_b ||
        !vertices_a || !indices_a || !vertices_b || !indices_b)
        return LYON_ERR_INVALID_ARGUMENT;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (num_paths == 0) return LYON_OK;
    if (cudaMemsetAsync(counts, 0, (size_t)num_paths * 3 * 8, s) != cudaSuccess)
        return LYON_ERR_CUDA;
    const size_t smem = 2 * (size_t)lg::COV_ROWS * (lg::COV_MAX_GRID + 1) * sizeof(int);
    static bool configured[64] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev >= 0 && dev < 64 && !configured[dev]) {
        cudaFuncSetAttribute(lg::coverage_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
        configured[dev] = true;
    }
    lg::CovSet A{reinterpret_cast<const float2*>(vertices_a), indices_a, vertex_offsets_a,
                 index_offsets_a};
    lg::CovSet B{reinterpret_cast<const float2*>(vertices_b), indices_b, vertex_offsets_b,
                 index_offsets_b};
    const dim3 g((grid + lg::COV_ROWS - 1) / lg::COV_ROWS, num_paths);
    lg::coverage_kernel<<<g, lg::COV_THREADS, smem, s>>>(
        boxes, grid, A, B, reinterpret_cast<unsigned long long*>(counts));
    lg::note_launches(1);
    return cudaGetLastError() == cudaSuccess ? LYON_OK : LYON_ERR_CUDA;
}
