// scan.cu — single-pass exclusive scan with decoupled look-back.
//
// Turns per-path vertex and index counts (u32) into u64 output offsets. Each block takes the
// next tile from an atomic counter (so every tile it looks back at is already running), scans it
// in shared memory, publishes its aggregate, walks back over the predecessors' published states
// until it meets an inclusive prefix, and publishes its own inclusive prefix. States pack a 2-bit
// flag with a 62-bit value in one u64 so that a single load sees a consistent pair. Waits are
// bounded: past the bound the kernel records an error and returns without hanging the GPU.
#include <atomic>

#include "kernels.h"

namespace lg {

static std::atomic<uint64_t> g_launches{0};
void note_launches(uint32_t k) { g_launches.fetch_add(k, std::memory_order_relaxed); }
uint64_t launches_total() { return g_launches.load(std::memory_order_relaxed); }

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 8;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;
constexpr unsigned long long FLAG_AGG = 1ull << 62;
constexpr unsigned long long FLAG_INC = 2ull << 62;
constexpr unsigned long long VALUE_MASK = (1ull << 62) - 1;
constexpr uint32_t SPIN_LIMIT = 1u << 24;

__host__ __device__ size_t scan_tile_count(uint32_t n) { return (n + SCAN_TILE - 1) / SCAN_TILE; }

__device__ __forceinline__ unsigned long long block_excl_scan(unsigned long long v,
                                                              unsigned long long* total) {
    __shared__ unsigned long long warp_sums[SCAN_THREADS / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    unsigned long long x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        unsigned long long n = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if (lane >= o) x += n;
    }
    if (lane == 31) warp_sums[w] = x;
    __syncthreads();
    if (w == 0) {
        unsigned long long s = lane < SCAN_THREADS / 32 ? warp_sums[lane] : 0ull;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            unsigned long long n = __shfl_up_sync(0xFFFFFFFFu, s, o);
            if (lane >= o) s += n;
        }
        if (lane < SCAN_THREADS / 32) warp_sums[lane] = s;
    }
    __syncthreads();
    unsigned long long before = w > 0 ? warp_sums[w - 1] : 0ull;
    *total = warp_sums[SCAN_THREADS / 32 - 1];
    __syncthreads();
    return before + x - v;
}

// Looks back from `tile` and returns the exclusive prefix of one channel.
__device__ __forceinline__ unsigned long long look_back(unsigned long long* state, uint32_t tile,
                                                        int* error) {
    unsigned long long prefix = 0;
    int64_t j = (int64_t)tile - 1;
    while (j >= 0) {
        unsigned long long s;
        uint32_t spins = 0;
        do {
            s = atomicAdd(&state[j], 0ull);
            if ((s >> 62) != 0) break;
            if (++spins > SPIN_LIMIT) {
                atomicExch(error, 1);
                return prefix;
            }
            __nanosleep(64);
        } while (true);
        prefix += s & VALUE_MASK;
        if ((s >> 62) == 2) break;
        --j;
    }
    return prefix;
}

__global__ void __launch_bounds__(SCAN_THREADS)
    scan_pairs_kernel(const uint32_t* __restrict__ a, const uint32_t* __restrict__ b,
                      uint64_t* __restrict__ out_a, uint64_t* __restrict__ out_b, uint32_t n,
                      unsigned long long* state, uint32_t* counter, int* error) {
    __shared__ uint32_t tile_s;
    __shared__ unsigned long long prefix_s[2];
    const uint32_t num_tiles = (uint32_t)scan_tile_count(n);
    if (threadIdx.x == 0) tile_s = atomicAdd(counter, 1u);
    __syncthreads();
    const uint32_t tile = tile_s;
    if (tile >= num_tiles) return;
    const uint64_t base = (uint64_t)tile * SCAN_TILE + (uint64_t)threadIdx.x * SCAN_ITEMS;
    uint32_t va[SCAN_ITEMS], vb[SCAN_ITEMS];
    unsigned long long sa = 0, sb = 0;
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; ++i) {
        uint64_t idx = base + i;
        va[i] = idx < n ? a[idx] : 0u;
        vb[i] = idx < n ? b[idx] : 0u;
        sa += va[i];
        sb += vb[i];
    }
    unsigned long long ta, tb;
    unsigned long long ea = block_excl_scan(sa, &ta);
    unsigned long long eb = block_excl_scan(sb, &tb);
    unsigned long long* state_a = state;
    unsigned long long* state_b = state + num_tiles;
    if (threadIdx.x == 0) {
        if (tile == 0) {
            atomicExch(&state_a[0], FLAG_INC | ta);
            atomicExch(&state_b[0], FLAG_INC | tb);
            prefix_s[0] = 0;
            prefix_s[1] = 0;
        } else {
            atomicExch(&state_a[tile], FLAG_AGG | ta);
            atomicExch(&state_b[tile], FLAG_AGG | tb);
            unsigned long long pa = look_back(state_a, tile, error);
            unsigned long long pb = look_back(state_b, tile, error);
            __threadfence();
            atomicExch(&state_a[tile], FLAG_INC | ((pa + ta) & VALUE_MASK));
            atomicExch(&state_b[tile], FLAG_INC | ((pb + tb) & VALUE_MASK));
            prefix_s[0] = pa;
            prefix_s[1] = pb;
        }
    }
    __syncthreads();
    unsigned long long ra = prefix_s[0] + ea, rb = prefix_s[1] + eb;
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; ++i) {
        uint64_t idx = base + i;
        if (idx < n) {
            out_a[idx] = ra;
            out_b[idx] = rb;
        }
        ra += va[i];
        rb += vb[i];
    }
    if (tile == num_tiles - 1 && threadIdx.x == 0) {
        out_a[n] = prefix_s[0] + ta;
        out_b[n] = prefix_s[1] + tb;
    }
}

__global__ void per_path_limit_kernel(uint32_t* vtx, uint32_t* idx, int32_t* status, uint32_t n,
                                      uint64_t vertex_offset, uint64_t max_index,
                                      uint32_t* failed) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t v = vtx[i];
    if (status[i] == LYON_OK && v > 0 && vertex_offset + v - 1 > max_index) {
        status[i] = LYON_ERR_TOO_MANY_VERTICES;
        vtx[i] = 0;
        idx[i] = 0;
    }
    if (status[i] != LYON_OK) atomicAdd(failed, 1u);
}

cudaError_t launch_scan_pairs(const uint32_t* a, const uint32_t* b, uint64_t* out_a,
                              uint64_t* out_b, uint32_t n, unsigned long long* tile_state,
                              uint32_t* counter, int* error, cudaStream_t stream) {
    size_t tiles = scan_tile_count(n);
    if (tiles == 0) {
        cudaMemsetAsync(out_a, 0, sizeof(uint64_t), stream);
        cudaMemsetAsync(out_b, 0, sizeof(uint64_t), stream);
        return cudaGetLastError();
    }
    cudaMemsetAsync(tile_state, 0, 2 * tiles * sizeof(unsigned long long), stream);
    cudaMemsetAsync(counter, 0, sizeof(uint32_t), stream);
    scan_pairs_kernel<<<(unsigned)tiles, SCAN_THREADS, 0, stream>>>(a, b, out_a, out_b, n,
                                                                   tile_state, counter, error);
    note_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_per_path_limit(uint32_t* vtx_counts, uint32_t* idx_counts, int32_t* status,
                                  uint32_t n, uint64_t vertex_offset, uint64_t max_index,
                                  uint32_t* failed, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    per_path_limit_kernel<<<(n + 255) / 256, 256, 0, stream>>>(vtx_counts, idx_counts, status, n,
                                                              vertex_offset, max_index, failed);
    note_launches(1);
    return cudaGetLastError();
}

}  // namespace lg

namespace lg {

__global__ void narrow_u64_kernel(const uint64_t* in, uint32_t* out, uint32_t n) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = (uint32_t)in[i];
}

__global__ void read_totals_kernel(const uint64_t* a_total, const uint64_t* b_total,
                                   const uint32_t* words, uint64_t* host_dst) {
    host_dst[0] = *a_total;
    host_dst[1] = *b_total;
    host_dst[2] = (uint64_t)words[0] | ((uint64_t)words[1] << 32);
}

cudaError_t launch_read_totals(const uint64_t* a_total, const uint64_t* b_total,
                               const uint32_t* words, uint64_t* host_dst, cudaStream_t s) {
    read_totals_kernel<<<1, 1, 0, s>>>(a_total, b_total, words, host_dst);
    note_launches(1);
    return cudaGetLastError();
}

// Class of a path for the processing order: 0 = more than `big_points` points (when big_points
// > 0), 2 + short_points - points for a line-only path of at most `short_points` points (when
// short_points > 0; fewer points, later), 1 = any other path.
__device__ __forceinline__ uint32_t path_class_of(const uint8_t* verbs, const uint32_t* verb_offsets,
                                                  const uint32_t* point_offsets, uint32_t i,
                                                  uint32_t big_points, uint32_t short_points) {
    const uint32_t pts = point_offsets[i + 1] - point_offsets[i];
    if (big_points && pts > big_points) return 0;
    if (short_points && pts <= short_points) {
        bool lines = true;
        for (uint32_t v = verb_offsets[i]; v < verb_offsets[i + 1] && lines; ++v) {
            const uint8_t k = verbs[v];
            lines = k == LYON_VERB_BEGIN || k == LYON_VERB_LINE_TO || k == LYON_VERB_CLOSE ||
                    k == LYON_VERB_END;
        }
        if (lines) return 2 + short_points - pts;
    }
    return 1;
}

constexpr uint32_t CLASSIFY_THREADS = 256;

__global__ void classify_count_kernel(const uint8_t* verbs, const uint32_t* verb_offsets,
                                      const uint32_t* point_offsets, uint32_t n,
                                      uint32_t big_points, uint32_t short_points,
                                      uint8_t* path_class, uint32_t* counters) {
    __shared__ uint32_t hist[CLASSIFY_MAX_BINS];
    const uint32_t nb = 3 + short_points;
    for (uint32_t b = threadIdx.x; b < nb; b += blockDim.x) hist[b] = 0;
    __syncthreads();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const uint32_t c = path_class_of(verbs, verb_offsets, point_offsets, i, big_points,
                                         short_points);
        path_class[i] = (uint8_t)c;
        atomicAdd(&hist[c], 1u);
    }
    __syncthreads();
    for (uint32_t b = threadIdx.x; b < nb; b += blockDim.x)
        if (hist[b]) atomicAdd(&counters[b], hist[b]);
}

__global__ void classify_place_kernel(const uint8_t* path_class, uint32_t n,
                                      uint32_t short_points, uint32_t* order,
                                      uint32_t* counters) {
    __shared__ uint32_t start[CLASSIFY_MAX_BINS];
    __shared__ uint32_t local[CLASSIFY_MAX_BINS];
    const uint32_t nb = 3 + short_points;
    if (threadIdx.x == 0) {
        uint32_t acc = 0;
        for (uint32_t b = 0; b < nb; ++b) {
            start[b] = acc;
            acc += counters[b];
        }
        if (blockIdx.x == 0) counters[2 * nb] = start[2];
    }
    for (uint32_t b = threadIdx.x; b < nb; b += blockDim.x) local[b] = 0;
    __syncthreads();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t c = 0, rank = 0;
    if (i < n) {
        c = path_class[i];
        rank = atomicAdd(&local[c], 1u);
    }
    __syncthreads();
    for (uint32_t b = threadIdx.x; b < nb; b += blockDim.x)
        if (local[b]) local[b] = atomicAdd(&counters[nb + b], local[b]);
    __syncthreads();
    if (i < n) order[start[c] + local[c] + rank] = i;
}

// Order by size: bin 31 - floor(log2(points)) (0 points: bin 32), so bigger paths come first.
__global__ void size_count_kernel(const uint32_t* point_offsets, const uint32_t* sizes,
                                  uint32_t n, uint8_t* cls, uint32_t* counters) {
    __shared__ uint32_t hist[SIZE_ORDER_BINS];
    for (uint32_t b = threadIdx.x; b < SIZE_ORDER_BINS; b += blockDim.x) hist[b] = 0;
    __syncthreads();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const uint32_t pts = sizes ? sizes[i] : point_offsets[i + 1] - point_offsets[i];
        const uint32_t c = pts == 0 ? 32u : (uint32_t)__clz(pts);
        cls[i] = (uint8_t)c;
        atomicAdd(&hist[c], 1u);
    }
    __syncthreads();
    for (uint32_t b = threadIdx.x; b < SIZE_ORDER_BINS; b += blockDim.x)
        if (hist[b]) atomicAdd(&counters[b], hist[b]);
}

__global__ void size_place_kernel(const uint8_t* cls, uint32_t n, uint32_t* order,
                                  uint32_t* counters) {
    __shared__ uint32_t start[SIZE_ORDER_BINS];
    __shared__ uint32_t local[SIZE_ORDER_BINS];
    if (threadIdx.x == 0) {
        uint32_t acc = 0;
        for (uint32_t b = 0; b < SIZE_ORDER_BINS; ++b) {
            start[b] = acc;
            acc += counters[b];
        }
    }
    for (uint32_t b = threadIdx.x; b < SIZE_ORDER_BINS; b += blockDim.x) local[b] = 0;
    __syncthreads();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t c = 0, rank = 0;
    if (i < n) {
        c = cls[i];
        rank = atomicAdd(&local[c], 1u);
    }
    __syncthreads();
    for (uint32_t b = threadIdx.x; b < SIZE_ORDER_BINS; b += blockDim.x)
        if (local[b]) local[b] = atomicAdd(&counters[SIZE_ORDER_BINS + b], local[b]);
    __syncthreads();
    if (i < n) order[start[c] + local[c] + rank] = i;
}

cudaError_t launch_size_order(const uint32_t* point_offsets, uint32_t n, uint8_t* cls,
                              uint32_t* order, uint32_t* counters, cudaStream_t s,
                              const uint32_t* sizes) {
    cudaMemsetAsync(counters, 0, 2 * SIZE_ORDER_BINS * sizeof(uint32_t), s);
    if (n == 0) return cudaGetLastError();
    const uint32_t blocks = (n + 255) / 256;
    size_count_kernel<<<blocks, 256, 0, s>>>(point_offsets, sizes, n, cls, counters);
    note_launches(1);
    size_place_kernel<<<blocks, 256, 0, s>>>(cls, n, order, counters);
    note_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_classify_paths(const uint8_t* verbs, const uint32_t* verb_offsets,
                                  const uint32_t* point_offsets, uint32_t n, uint32_t big_points,
                                  uint32_t short_points, uint8_t* path_class, uint32_t* order,
                                  uint32_t* counters, cudaStream_t s) {
    if (short_points > CLASSIFY_MAX_SHORT_POINTS) return cudaErrorInvalidValue;
    const uint32_t nb = 3 + short_points;
    cudaMemsetAsync(counters, 0, (2 * nb + 1) * sizeof(uint32_t), s);
    if (n == 0) return cudaGetLastError();
    const uint32_t blocks = (n + CLASSIFY_THREADS - 1) / CLASSIFY_THREADS;
    classify_count_kernel<<<blocks, CLASSIFY_THREADS, 0, s>>>(
        verbs, verb_offsets, point_offsets, n, big_points, short_points, path_class, counters);
    note_launches(1);
    classify_place_kernel<<<blocks, CLASSIFY_THREADS, 0, s>>>(path_class, n, short_points, order,
                                                             counters);
    note_launches(1);
    return cudaGetLastError();
}

__global__ void big_first_order_kernel(const uint32_t* point_offsets, uint32_t n,
                                       uint32_t big_points, uint32_t* order, uint32_t* counters) {
    // Every lane of every warp takes part in the votes (the grid is a whole number of warps).
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = i < n;
    const bool big = valid && point_offsets[i + 1] - point_offsets[i] > big_points;
    const bool small = valid && !big;
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t bmask = __ballot_sync(0xFFFFFFFFu, big);
    const uint32_t smask = __ballot_sync(0xFFFFFFFFu, small);
    // One atomic per warp and class.
    const int leader_b = bmask ? __ffs(bmask) - 1 : 0, leader_s = smask ? __ffs(smask) - 1 : 0;
    uint32_t base_b = 0, base_s = 0;
    if (bmask && (int)lane == leader_b) base_b = atomicAdd(&counters[0], __popc(bmask));
    if (smask && (int)lane == leader_s) base_s = atomicAdd(&counters[1], __popc(smask));
    base_b = __shfl_sync(0xFFFFFFFFu, base_b, leader_b);
    base_s = __shfl_sync(0xFFFFFFFFu, base_s, leader_s);
    if (!valid) return;
    const uint32_t below = (1u << lane) - 1u;
    if (big) {
        order[base_b + __popc(bmask & below)] = i;
    } else {
        order[n - 1 - (base_s + __popc(smask & below))] = i;
    }
}

cudaError_t launch_big_first_order(const uint32_t* point_offsets, uint32_t n, uint32_t big_points,
                                   uint32_t* order, uint32_t* counters, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    cudaMemsetAsync(counters, 0, 8, s);
    big_first_order_kernel<<<(n + 255) / 256, 256, 0, s>>>(point_offsets, n, big_points, order,
                                                           counters);
    note_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_narrow_u64(const uint64_t* in, uint32_t* out, uint32_t n, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    narrow_u64_kernel<<<(n + 255) / 256, 256, 0, s>>>(in, out, n);
    note_launches(1);
    return cudaGetLastError();
}

}  // namespace lg
