// noalloc.cu — lyon_gpu_stroke_paths_noalloc: the batched stroke pipeline (count kernel,
// index-range check, look-back scan, emit kernel) for callers that cannot allocate device
// memory, such as a plugin that is handed device buffers by a host application that owns
// every allocation on the GPU, or code running inside a memory pool that forbids cudaMalloc.
//
// The pipeline's scratch (per-path vertex/index counts, the scan's tile states and four
// counter words) lives in one file-scope __device__ array of NOALLOC_SCRATCH_BYTES, which
// every GPU that loads this library holds until the process exits. The call itself allocates
// nothing: no cudaMalloc, no cudaFree, no allocating library routine, no host heap.
//
// All calls on one device share that array and it keeps the previous call's contents: the
// counter words are cleared on every call and the count kernel writes every path's counts
// before anything reads them. Calls whose GPU work overlaps (different streams, or different
// host threads without ordering) race on the array and give wrong results.
#include <cstdio>
#include <cstring>
#include <mutex>

#include "kernels.h"

namespace {

constexpr uint32_t NOALLOC_MAX_PATHS = LYON_NOALLOC_MAX_PATHS;
// Layout: [0, 256) counter words | vertex counts | index counts | scan tile states.
constexpr size_t OFF_VTX = 256;
constexpr size_t OFF_IDX = OFF_VTX + (size_t)NOALLOC_MAX_PATHS * 4 + 256;
constexpr size_t OFF_SCAN = OFF_IDX + (size_t)NOALLOC_MAX_PATHS * 4 + 256;
constexpr size_t SCAN_TILES_MAX = ((size_t)NOALLOC_MAX_PATHS + 2047) / 2048;
constexpr size_t NOALLOC_SCRATCH_BYTES = OFF_SCAN + 2 * SCAN_TILES_MAX * 8 + 256;

// The scratch array. In host code `noalloc_scratch` only names the symbol; its device address
// comes from cudaGetSymbolAddress (once per device, below).
static __device__ __align__(256) unsigned char noalloc_scratch[NOALLOC_SCRATCH_BYTES];

constexpr int MAX_DEVICES = 64;

struct DeviceSetup {
    bool done = false;
    unsigned char* scratch = nullptr;
    int grid = 1;
};

std::mutex g_setup_lock;
DeviceSetup g_setup[MAX_DEVICES];

void set_text(char* text, size_t len, const char* msg) {
    if (text && len > 0) snprintf(text, len, "%s", msg);
}

// Resolves the scratch array's address and the launch grid for the current device, once.
int device_setup(DeviceSetup** out, char* text, size_t len) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        set_text(text, len, cudaGetErrorString(e));
        return LYON_ERR_CUDA;
    }
    if (dev < 0 || dev >= MAX_DEVICES) {
        set_text(text, len, "device ordinal beyond the library's table of devices");
        return LYON_ERR_INVALID_ARGUMENT;
    }
    std::lock_guard<std::mutex> g(g_setup_lock);
    DeviceSetup& d = g_setup[dev];
    if (!d.done) {
        void* ptr = nullptr;
        e = cudaGetSymbolAddress(&ptr, noalloc_scratch);
        if (e != cudaSuccess) {
            cudaGetLastError();
            char buf[256];
            snprintf(buf, sizeof buf, "cudaGetSymbolAddress(noalloc scratch): %s",
                     cudaGetErrorString(e));
            set_text(text, len, buf);
            return LYON_ERR_CUDA;
        }
        int sms = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        d.scratch = static_cast<unsigned char*>(ptr);
        d.grid = (sms > 0 ? sms : 1) * lg::stroke_blocks_per_sm();
        d.done = true;
    }
    *out = &d;
    return LYON_OK;
}

bool cuda_ok(cudaError_t e, const char* what, char* text, size_t len) {
    if (e == cudaSuccess) return true;
    char buf[256];
    snprintf(buf, sizeof buf, "%s: %s", what, cudaGetErrorString(e));
    set_text(text, len, buf);
    return false;
}

// BuffersBuilder's sequential index assignment (geometry_builder.rs:338-350, 478-481) for
// LYON_INDEX_GLOBAL when the batch overflows the index type, in fixed-size host chunks.
bool global_fixup_chunked(uint32_t* vc_d, uint32_t* ic_d, int32_t* st_d, uint32_t n,
                          uint64_t vertex_offset, uint64_t max_index, cudaStream_t s, char* text,
                          size_t len) {
    constexpr uint32_t CHUNK = 2048;
    uint32_t vc[CHUNK], ic[CHUNK];
    int32_t st[CHUNK];
    uint64_t run = 0;
    for (uint32_t c0 = 0; c0 < n; c0 += CHUNK) {
        const uint32_t cn = n - c0 < CHUNK ? n - c0 : CHUNK;
        cudaMemcpyAsync(vc, vc_d + c0, cn * 4ull, cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(ic, ic_d + c0, cn * 4ull, cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(st, st_d + c0, cn * 4ull, cudaMemcpyDeviceToHost, s);
        if (!cuda_ok(cudaStreamSynchronize(s), "overflow check (read)", text, len)) return false;
        for (uint32_t i = 0; i < cn; ++i) {
            if (st[i] != LYON_OK) continue;
            if (vc[i] > 0 && vertex_offset + run + vc[i] - 1 > max_index) {
                st[i] = LYON_ERR_TOO_MANY_VERTICES;
                vc[i] = 0;
                ic[i] = 0;
                continue;
            }
            run += vc[i];
        }
        cudaMemcpyAsync(vc_d + c0, vc, cn * 4ull, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(ic_d + c0, ic, cn * 4ull, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(st_d + c0, st, cn * 4ull, cudaMemcpyHostToDevice, s);
        if (!cuda_ok(cudaStreamSynchronize(s), "overflow check (write)", text, len)) return false;
    }
    return true;
}

}  // namespace

extern "C" int lyon_gpu_stroke_paths_noalloc(
    const lyon_path_batch* batch, const lyon_stroke_options* options, uint32_t num_options,
    int index_bits, int index_mode, uint32_t vertex_offset, float* vertices,
    uint64_t vertex_capacity, void* indices, uint64_t index_capacity, uint64_t* vertex_offsets,
    uint64_t* index_offsets, int32_t* status, uint64_t* total_vertices, uint64_t* total_indices,
    uint32_t* num_failed_paths, void* stream, char* error_text, size_t error_text_len) {
    set_text(error_text, error_text_len, "");
    if (total_vertices) *total_vertices = 0;
    if (total_indices) *total_indices = 0;
    if (num_failed_paths) *num_failed_paths = 0;
    if (!batch || !options || num_options == 0 || !vertex_offsets || !index_offsets || !status ||
        !total_vertices || !total_indices || (index_bits != 16 && index_bits != 32) ||
        (index_mode != LYON_INDEX_GLOBAL && index_mode != LYON_INDEX_PER_PATH) ||
        (num_options != 1 && num_options != batch->num_paths)) {
        set_text(error_text, error_text_len, "invalid argument");
        return LYON_ERR_INVALID_ARGUMENT;
    }
    const uint32_t n = batch->num_paths;
    if (n > NOALLOC_MAX_PATHS) {
        char buf[160];
        snprintf(buf, sizeof buf,
                 "batch of %u paths exceeds the no-allocation scratch limit of %u paths", n,
                 NOALLOC_MAX_PATHS);
        set_text(error_text, error_text_len, buf);
        return LYON_ERR_CAPACITY;
    }
    DeviceSetup* d = nullptr;
    int r = device_setup(&d, error_text, error_text_len);
    if (r != LYON_OK) return r;
    cudaStream_t s = static_cast<cudaStream_t>(stream);

    uint32_t* words = reinterpret_cast<uint32_t*>(d->scratch);  // work, scan, error, failed
    uint32_t* vc = reinterpret_cast<uint32_t*>(d->scratch + OFF_VTX);
    uint32_t* ic = reinterpret_cast<uint32_t*>(d->scratch + OFF_IDX);
    unsigned long long* scan_state = reinterpret_cast<unsigned long long*>(d->scratch + OFF_SCAN);
    const uint64_t maxi = index_bits == 16 ? 65535ull : 0xFFFFFFFEull;

    lg::StrokeArgs a;
    memset(&a, 0, sizeof a);
    a.verbs = batch->verbs;
    a.points = batch->points;
    a.verb_offsets = batch->verb_offsets;
    a.point_offsets = batch->point_offsets;
    a.num_paths = n;
    a.options = options;
    a.num_options = num_options;
    a.work_counter = words;
    a.vtx_counts = vc;
    a.idx_counts = ic;
    a.status = status;
    a.vtx_offsets = vertex_offsets;
    a.idx_offsets = index_offsets;
    a.vertices = vertices;
    a.indices = indices;
    a.index_bits = index_bits;
    a.index_mode = index_mode;
    a.vertex_offset = vertex_offset;
    const int grid = (int)((n + 3) / 4) < d->grid ? (int)((n + 3) / 4) : d->grid;

    if (!cuda_ok(cudaMemsetAsync(words, 0, 16, s), "clear counters", error_text, error_text_len))
        return LYON_ERR_CUDA;
    if (n > 0 && !cuda_ok(lg::launch_stroke(a, false, grid > 0 ? grid : 1, s), "stroke count",
                          error_text, error_text_len))
        return LYON_ERR_CUDA;
    if (!cuda_ok(lg::launch_per_path_limit(vc, ic, status, n, vertex_offset,
                                           index_mode == LYON_INDEX_PER_PATH ? maxi : ~0ull,
                                           words + 3, s),
                 "index range", error_text, error_text_len))
        return LYON_ERR_CUDA;
    uint64_t tv = 0, ti = 0;
    uint32_t flags[2] = {0, 0};
    for (int pass = 0; pass < 2; ++pass) {
        if (!cuda_ok(lg::launch_scan_pairs(vc, ic, vertex_offsets, index_offsets, n, scan_state,
                                           words + 1, reinterpret_cast<int*>(words + 2), s),
                     "scan", error_text, error_text_len))
            return LYON_ERR_CUDA;
        cudaMemcpyAsync(&tv, vertex_offsets + n, 8, cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(&ti, index_offsets + n, 8, cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(flags, words + 2, 8, cudaMemcpyDeviceToHost, s);
        if (!cuda_ok(cudaStreamSynchronize(s), "read totals", error_text, error_text_len))
            return LYON_ERR_CUDA;
        if (flags[0] != 0) {
            set_text(error_text, error_text_len, "scan look-back wait exceeded its bound");
            return LYON_ERR_CUDA;
        }
        if (pass == 0 && index_mode == LYON_INDEX_GLOBAL && tv > 0 &&
            vertex_offset + tv - 1 > maxi) {
            if (!global_fixup_chunked(vc, ic, status, n, vertex_offset, maxi, s, error_text,
                                      error_text_len))
                return LYON_ERR_CUDA;
            if (!cuda_ok(cudaMemsetAsync(words + 2, 0, 8, s), "clear counters", error_text,
                         error_text_len) ||
                !cuda_ok(lg::launch_per_path_limit(vc, ic, status, n, vertex_offset, ~0ull,
                                                   words + 3, s),
                         "count failures", error_text, error_text_len))
                return LYON_ERR_CUDA;
            continue;
        }
        break;
    }
    *total_vertices = tv;
    *total_indices = ti;
    if (num_failed_paths) *num_failed_paths = flags[1];
    if (tv > vertex_capacity || ti > index_capacity || (tv > 0 && !vertices) ||
        (ti > 0 && !indices)) {
        set_text(error_text, error_text_len,
                 "output buffers too small: *total_vertices / *total_indices hold the sizes needed");
        return LYON_ERR_CAPACITY;
    }
    if (n > 0 && tv > 0) {
        if (!cuda_ok(cudaMemsetAsync(words, 0, 4, s), "clear counters", error_text,
                     error_text_len) ||
            !cuda_ok(lg::launch_stroke(a, true, grid > 0 ? grid : 1, s), "stroke emit",
                     error_text, error_text_len))
            return LYON_ERR_CUDA;
    }
    return LYON_OK;
}
