// serve.cu — the serving loop: tessellation requests of mixed sizes, continuously batched.
//
// Requests (a scene of paths to stroke or fill, in host memory owned by the caller until the
// request completes) enter a FIFO per kind. Worker threads, each with its own context and CUDA
// stream, take the oldest requests of one kind, as many as fit in a batch and in the device
// memory budget, and run them as ONE batched launch (count, scan, emit) with one vertex id space
// per request. While one worker's batch runs, the next worker gathers the requests that arrived
// meanwhile, so their work overlaps on the device. Outputs stay resident in device slabs until
// the caller releases the request; slabs are pooled per worker and reused.
//
// Stroke requests take microseconds to milliseconds of GPU time, fill requests tens of
// milliseconds (one path's sweep runs on one thread). With stroke workers configured, the kinds
// get separate workers: stroke workers run on streams of the device's highest priority with one
// stroke block per SM, and fill sweeps keep at most `fill_blocks_per_sm` blocks per SM, so that
// a stroke launch finds room on every SM and starts while fill sweeps are running instead of
// waiting for them to end.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <random>
#include <thread>
#include <unordered_map>
#include <vector>

#include "kernels.h"

namespace lg {
int srv_count(lyon_gpu_context* ctx, int kind, const lyon_path_batch* batch, const void* options,
              uint32_t num_options, const uint32_t* request_first, uint64_t* tv, uint64_t* ti,
              uint32_t* failed);
int srv_configure(lyon_gpu_context* ctx, bool stroke_lane, uint32_t fill_blocks_per_sm,
                  cudaMemPool_t pool);
int srv_emit(lyon_gpu_context* ctx, int kind, const lyon_path_batch* batch, const void* options,
             uint32_t num_options, const uint32_t* request_first, float* vout, void* iout,
             uint64_t tv);
const uint64_t* srv_vtx_offsets(lyon_gpu_context* ctx);
const uint64_t* srv_idx_offsets(lyon_gpu_context* ctx);
const int32_t* srv_status(lyon_gpu_context* ctx);
cudaStream_t srv_stream(lyon_gpu_context* ctx);
}  // namespace lg

namespace {

using Clock = std::chrono::steady_clock;

double now_s() {
    return std::chrono::duration<double>(Clock::now().time_since_epoch()).count();
}

size_t option_size(int kind) {
    return kind == LYON_KIND_STROKE ? sizeof(lyon_stroke_options) : sizeof(lyon_fill_options);
}

// Device output of one batch, shared by its requests.
struct Slab {
    float2* v = nullptr;
    uint32_t* i = nullptr;
    uint64_t* voff = nullptr;
    uint64_t* ioff = nullptr;
    int32_t* st = nullptr;
    size_t vcap = 0, icap = 0, pcap = 0;  // vertices, indices, paths + 1
    int refs = 0;
    size_t bytes() const { return vcap * 8 + icap * 4 + pcap * 20; }
};

struct Request {
    uint64_t id;
    int kind;
    lyon_path_batch batch;  // host, borrowed
    const void* options;
    uint32_t num_options;
    uint64_t est_bytes;
    double t_arrival, t_start = 0, t_done = 0;
    bool done = false;
    int status = LYON_OK;
    uint32_t failed = 0;
    Slab* slab = nullptr;
    uint32_t path_begin = 0;
    uint64_t v_begin = 0, v_end = 0, i_begin = 0, i_end = 0;
};

// Device buffers of a worker: from the worker's own pool, in its stream order, when there is a
// pool (a plain cudaFree can wait for every kernel on the device, other workers' included).
template <class T>
bool dev_grow(T** p, size_t* cap, size_t n, cudaMemPool_t pool, cudaStream_t st) {
    if (n <= *cap && *p) return true;
    if (*p) {
        if (pool) {
            cudaFreeAsync(*p, st);
        } else {
            cudaFree(*p);
        }
    }
    *p = nullptr;
    size_t c = n + n / 2 + 64;
    void* np = nullptr;
    const cudaError_t e = pool ? cudaMallocFromPoolAsync(&np, c * sizeof(T), pool, st)
                               : cudaMalloc(&np, c * sizeof(T));
    if (e != cudaSuccess) {
        cudaGetLastError();
        *cap = 0;
        return false;
    }
    *p = reinterpret_cast<T*>(np);
    *cap = c;
    return true;
}

// Pinned staging of a worker. An outgrown buffer is retired, not freed: freeing page-locked
// memory can wait for the whole device (another worker's fill sweep included). Buffers grow by
// half each time, so the retired ones together stay below twice the final size; they are freed
// with the loop.
template <class T>
bool host_grow(T** p, size_t* cap, size_t n, std::vector<void*>* retired) {
    if (n <= *cap && *p) return true;
    if (*p) retired->push_back(*p);
    *p = nullptr;
    size_t c = n + n / 2 + 64;
    if (cudaMallocHost(reinterpret_cast<void**>(p), c * sizeof(T)) != cudaSuccess) {
        cudaGetLastError();
        *cap = 0;
        return false;
    }
    *cap = c;
    return true;
}

enum Role { ROLE_ANY = 0, ROLE_STROKE = 1, ROLE_FILL = 2 };

struct Worker {
    lyon_gpu_context* ctx = nullptr;
    int role = ROLE_ANY;
    std::thread th;
    // pinned staging and device copies of the batch inputs
    uint8_t* h_verbs = nullptr;
    float* h_points = nullptr;
    uint32_t* h_off = nullptr;  // verb offsets, point offsets, request_first
    uint8_t* h_opts = nullptr;
    uint64_t* h_res = nullptr;  // offsets read back (vertex, index) + status counts
    size_t hv_cap = 0, hp_cap = 0, ho_cap = 0, hopt_cap = 0, hres_cap = 0;
    uint8_t* d_verbs = nullptr;
    float* d_points = nullptr;
    uint32_t* d_off = nullptr;
    uint8_t* d_opts = nullptr;
    size_t dv_cap = 0, dp_cap = 0, do_cap = 0, dopt_cap = 0;
    std::vector<Slab*> slabs;
    std::vector<void*> retired_host;  // outgrown pinned staging, freed with the loop
    cudaMemPool_t pool = nullptr;     // this worker's device buffers (null: plain cudaMalloc)
    uint64_t batches = 0, batch_paths = 0;
};

}  // namespace

struct lyon_srv {
    lyon_srv_config cfg;
    std::mutex mu;
    std::condition_variable cv_work;  // queue or budget changed
    std::condition_variable cv_done;  // a request completed
    std::deque<Request*> queue[2];
    std::unordered_map<uint64_t, Request*> reqs;
    uint64_t next_id = 1;
    uint64_t held_bytes = 0;  // slabs of unreleased requests + reservations of running batches
    bool stop = false;
    std::vector<std::unique_ptr<Worker>> workers;
};

namespace {

uint64_t estimate_bytes(const Request& r) {
    // Inputs, plus an output guess from the input size (the count pass gives the real size).
    uint32_t pts = r.batch.point_offsets[r.batch.num_paths] - r.batch.point_offsets[0];
    uint32_t verbs = r.batch.verb_offsets[r.batch.num_paths] - r.batch.verb_offsets[0];
    uint64_t in = (uint64_t)pts * 8 + verbs + (uint64_t)r.batch.num_paths * 48;
    uint64_t out_guess = (uint64_t)pts * (r.kind == LYON_KIND_STROKE ? 400 : 60);
    return in + out_guess;
}

void finish(lyon_srv* s, std::vector<Request*>& batch, int status, Slab* slab, const uint64_t* hv,
            const uint64_t* hi, const int32_t* hst, uint64_t reserved) {
    std::lock_guard<std::mutex> g(s->mu);
    const double t = now_s();
    s->held_bytes -= reserved;
    if (slab) s->held_bytes += slab->bytes();
    uint32_t p = 0;
    for (Request* r : batch) {
        const uint32_t n = r->batch.num_paths;
        r->status = status;
        r->t_done = t;
        if (status == LYON_OK) {
            r->slab = slab;
            slab->refs += 1;
            r->path_begin = p;
            r->v_begin = hv[p];
            r->v_end = hv[p + n];
            r->i_begin = hi[p];
            r->i_end = hi[p + n];
            uint32_t f = 0;
            for (uint32_t k = 0; k < n; ++k) f += hst[p + k] != LYON_OK;
            r->failed = f;
        }
        p += n;
        r->done = true;
    }
    if (slab && slab->refs == 0) s->held_bytes -= slab->bytes();
    s->cv_done.notify_all();
    s->cv_work.notify_all();
}

Slab* take_slab(Worker& w, uint64_t tv, uint64_t ti, uint32_t np, cudaMemPool_t pool,
                cudaStream_t st) {
    Slab* best = nullptr;
    for (Slab* sl : w.slabs) {
        if (sl->refs == 0 && sl->vcap >= tv && sl->icap >= ti && sl->pcap >= (size_t)np + 1)
            return sl;
        if (sl->refs == 0 && !best) best = sl;
    }
    if (!best) {
        best = new Slab();
        w.slabs.push_back(best);
    }
    if (!dev_grow(&best->v, &best->vcap, (size_t)tv + 1, pool, st) ||
        !dev_grow(&best->i, &best->icap, (size_t)ti + 1, pool, st))
        return nullptr;
    if (best->pcap < (size_t)np + 1) {
        size_t c1 = best->pcap, c2 = best->pcap, c3 = best->pcap;
        if (!dev_grow(&best->voff, &c1, (size_t)np + 1, pool, st) ||
            !dev_grow(&best->ioff, &c2, (size_t)np + 1, pool, st) ||
            !dev_grow(&best->st, &c3, (size_t)np + 1, pool, st))
            return nullptr;
        best->pcap = c1;
    }
    return best;
}

// Runs one batch of requests of one kind on the worker's context.
void run_batch(lyon_srv* s, Worker& w, int kind, std::vector<Request*>& batch, uint64_t reserved) {
    const double t_start = now_s();
    {
        std::lock_guard<std::mutex> g(s->mu);
        for (Request* r : batch) r->t_start = t_start;
    }
    const size_t osz = option_size(kind);
    uint32_t np = 0;
    size_t nverbs = 0, npts = 0;
    for (Request* r : batch) {
        np += r->batch.num_paths;
        nverbs += r->batch.verb_offsets[r->batch.num_paths] - r->batch.verb_offsets[0];
        npts += r->batch.point_offsets[r->batch.num_paths] - r->batch.point_offsets[0];
    }
    if (!host_grow(&w.h_verbs, &w.hv_cap, nverbs + 16, &w.retired_host) ||
        !host_grow(&w.h_points, &w.hp_cap, npts * 2 + 16, &w.retired_host) ||
        !host_grow(&w.h_off, &w.ho_cap, (size_t)np * 3 + 3, &w.retired_host) ||
        !host_grow(&w.h_opts, &w.hopt_cap, (size_t)np * osz + osz, &w.retired_host) ||
        !host_grow(&w.h_res, &w.hres_cap, (size_t)np * 3 + 4, &w.retired_host) ||
        !dev_grow(&w.d_verbs, &w.dv_cap, nverbs + 16, w.pool, lg::srv_stream(w.ctx)) ||
        !dev_grow(&w.d_points, &w.dp_cap, npts * 2 + 16, w.pool, lg::srv_stream(w.ctx)) ||
        !dev_grow(&w.d_off, &w.do_cap, (size_t)np * 3 + 3, w.pool, lg::srv_stream(w.ctx)) ||
        !dev_grow(&w.d_opts, &w.dopt_cap, (size_t)np * osz + osz, w.pool,
                  lg::srv_stream(w.ctx))) {
        finish(s, batch, LYON_ERR_OUT_OF_MEMORY, nullptr, nullptr, nullptr, nullptr, reserved);
        return;
    }
    // Concatenate the requests: offsets rebased, options expanded to one record per path.
    uint32_t* voff = w.h_off;
    uint32_t* poff = w.h_off + np + 1;
    uint32_t* rfirst = w.h_off + 2 * (np + 1);
    size_t vc = 0, pc = 0;
    uint32_t p = 0;
    for (Request* r : batch) {
        const lyon_path_batch& b = r->batch;
        const uint32_t n = b.num_paths;
        const uint32_t v0 = b.verb_offsets[0], p0 = b.point_offsets[0];
        const uint32_t vn = b.verb_offsets[n] - v0, pn = b.point_offsets[n] - p0;
        std::memcpy(w.h_verbs + vc, b.verbs + v0, vn);
        std::memcpy(w.h_points + 2 * pc, b.points + 2 * (size_t)p0, (size_t)pn * 8);
        for (uint32_t k = 0; k < n; ++k) {
            voff[p + k] = (uint32_t)vc + (b.verb_offsets[k] - v0);
            poff[p + k] = (uint32_t)pc + (b.point_offsets[k] - p0);
            rfirst[p + k] = p;
            const uint8_t* src = reinterpret_cast<const uint8_t*>(r->options) +
                                 (r->num_options > 1 ? (size_t)k * osz : 0);
            std::memcpy(w.h_opts + (size_t)(p + k) * osz, src, osz);
        }
        vc += vn;
        pc += pn;
        p += n;
    }
    voff[np] = (uint32_t)vc;
    poff[np] = (uint32_t)pc;
    cudaStream_t st = lg::srv_stream(w.ctx);
    cudaMemcpyAsync(w.d_verbs, w.h_verbs, vc, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(w.d_points, w.h_points, pc * 8, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(w.d_off, w.h_off, ((size_t)np * 3 + 2) * 4, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(w.d_opts, w.h_opts, (size_t)np * osz, cudaMemcpyHostToDevice, st);
    lyon_path_batch db;
    db.verbs = w.d_verbs;
    db.points = w.d_points;
    db.verb_offsets = w.d_off;
    db.point_offsets = w.d_off + np + 1;
    db.num_paths = np;
    const uint32_t* d_rfirst = w.d_off + 2 * (np + 1);
    uint64_t tv = 0, ti = 0;
    uint32_t failed = 0;
    int rc = lg::srv_count(w.ctx, kind, &db, w.d_opts, np, d_rfirst, &tv, &ti, &failed);
    if (rc != LYON_OK) {
        finish(s, batch, rc, nullptr, nullptr, nullptr, nullptr, reserved);
        return;
    }
    Slab* slab;
    {
        std::lock_guard<std::mutex> g(s->mu);
        slab = take_slab(w, tv, ti, np, w.pool, st);
    }
    if (!slab) {
        finish(s, batch, LYON_ERR_OUT_OF_MEMORY, nullptr, nullptr, nullptr, nullptr, reserved);
        return;
    }
    rc = lg::srv_emit(w.ctx, kind, &db, w.d_opts, np, d_rfirst,
                      reinterpret_cast<float*>(slab->v), slab->i, tv);
    if (rc != LYON_OK) {
        finish(s, batch, rc, nullptr, nullptr, nullptr, nullptr, reserved);
        return;
    }
    cudaMemcpyAsync(slab->voff, lg::srv_vtx_offsets(w.ctx), ((size_t)np + 1) * 8,
                    cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(slab->ioff, lg::srv_idx_offsets(w.ctx), ((size_t)np + 1) * 8,
                    cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(slab->st, lg::srv_status(w.ctx), (size_t)np * 4, cudaMemcpyDeviceToDevice, st);
    uint64_t* hv = w.h_res;
    uint64_t* hi = w.h_res + np + 1;
    int32_t* hst = reinterpret_cast<int32_t*>(w.h_res + 2 * ((size_t)np + 1));
    cudaMemcpyAsync(hv, lg::srv_vtx_offsets(w.ctx), ((size_t)np + 1) * 8, cudaMemcpyDeviceToHost,
                    st);
    cudaMemcpyAsync(hi, lg::srv_idx_offsets(w.ctx), ((size_t)np + 1) * 8, cudaMemcpyDeviceToHost,
                    st);
    cudaMemcpyAsync(hst, lg::srv_status(w.ctx), (size_t)np * 4, cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) {
        cudaGetLastError();
        finish(s, batch, LYON_ERR_CUDA, nullptr, nullptr, nullptr, nullptr, reserved);
        return;
    }
    w.batches += 1;
    w.batch_paths += np;
    finish(s, batch, LYON_OK, slab, hv, hi, hst, reserved);
}

void worker_main(lyon_srv* s, Worker* w) {
    cudaSetDevice(s->cfg.device);
    for (;;) {
        std::vector<Request*> batch;
        int kind = 0;
        uint64_t reserved = 0;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            for (;;) {
                if (s->stop) return;
                const bool have0 = w->role != ROLE_FILL && !s->queue[0].empty();
                const bool have1 = w->role != ROLE_STROKE && !s->queue[1].empty();
                if (!have0 && !have1) {
                    s->cv_work.wait(lk);
                    continue;
                }
                // The kind whose oldest request arrived first.
                kind = (have0 && (!have1 || s->queue[0].front()->t_arrival <=
                                                s->queue[1].front()->t_arrival))
                           ? 0
                           : 1;
                std::deque<Request*>& q = s->queue[kind];
                const uint32_t max_paths =
                    kind == LYON_KIND_STROKE ? s->cfg.max_stroke_batch_paths : s->cfg.max_batch_paths;
                uint32_t paths = 0;
                while (!q.empty()) {
                    Request* r = q.front();
                    const bool first = batch.empty();
                    if (!first && paths + r->batch.num_paths > max_paths) break;
                    if (s->held_bytes + reserved + r->est_bytes > s->cfg.device_budget_bytes &&
                        !(first && s->held_bytes == 0))
                        break;
                    q.pop_front();
                    batch.push_back(r);
                    paths += r->batch.num_paths;
                    reserved += r->est_bytes;
                }
                if (!batch.empty()) break;
                s->cv_work.wait(lk);  // over budget: wait for releases
            }
            s->held_bytes += reserved;
        }
        run_batch(s, *w, kind, batch, reserved);
    }
}

void fill_result(const Request* r, lyon_srv_result* out) {
    std::memset(out, 0, sizeof(*out));
    out->status = r->status;
    out->num_paths = r->batch.num_paths;
    out->queue_ms = (r->t_start - r->t_arrival) * 1e3;
    out->latency_ms = (r->t_done - r->t_arrival) * 1e3;
    if (r->status != LYON_OK || !r->slab) return;
    out->num_failed_paths = r->failed;
    out->vertices = reinterpret_cast<const float*>(r->slab->v + r->v_begin);
    out->num_vertices = r->v_end - r->v_begin;
    out->indices = r->slab->i + r->i_begin;
    out->num_indices = r->i_end - r->i_begin;
    out->path_vertex_offsets = r->slab->voff + r->path_begin;
    out->path_index_offsets = r->slab->ioff + r->path_begin;
    out->path_status = r->slab->st + r->path_begin;
    out->vertex_base = r->v_begin;
    out->index_base = r->i_begin;
}

uint64_t submit_at(lyon_srv* s, int kind, const lyon_path_batch* batch, const void* options,
                   uint32_t num_options, double t_arrival) {
    if (!s || !batch || !options || (kind != LYON_KIND_STROKE && kind != LYON_KIND_FILL) ||
        batch->num_paths == 0 || (num_options != 1 && num_options != batch->num_paths))
        return 0;
    Request* r = new Request();
    r->kind = kind;
    r->batch = *batch;
    r->options = options;
    r->num_options = num_options;
    r->est_bytes = estimate_bytes(*r);
    r->t_arrival = t_arrival;
    std::lock_guard<std::mutex> g(s->mu);
    r->id = s->next_id++;
    s->reqs[r->id] = r;
    s->queue[kind].push_back(r);
    // Every worker is woken: with stroke and fill lanes a single wake-up can reach a worker of
    // the other kind, which finds nothing to take and sleeps again, leaving the request queued.
    s->cv_work.notify_all();
    return r->id;
}

}  // namespace

extern "C" {

lyon_srv* lyon_srv_create(const lyon_srv_config* config) {
    lyon_srv* s = new lyon_srv();
    lyon_srv_config c = config ? *config : lyon_srv_config{0, 0, 0, 0, 0, 0, 0};
    if (c.num_workers == 0) c.num_workers = 2;
    if (c.max_batch_paths == 0) c.max_batch_paths = 65536;
    if (c.device_budget_bytes == 0) c.device_budget_bytes = 40ull << 30;
    if (c.max_stroke_batch_paths == 0) c.max_stroke_batch_paths = c.max_batch_paths;
    // Measured with two fill and two stroke workers: 8 sweep blocks per SM gave small stroke
    // requests a p99 of 3.4 ms and fills 161-166 ms, 5 blocks 7.4-8.7 ms and 179-183 ms.
    if (c.num_stroke_workers > 0 && c.fill_blocks_per_sm == 0) c.fill_blocks_per_sm = 8;
    s->cfg = c;
    cudaSetDevice(c.device);
    const uint32_t total = c.num_workers + c.num_stroke_workers;
    for (uint32_t i = 0; i < total; ++i) {
        std::unique_ptr<Worker> w(new Worker());
        w->ctx = lyon_gpu_create(c.device);
        if (!w->ctx) {
            lyon_srv_destroy(s);
            return nullptr;
        }
        // A pool per worker: a pool shared between workers may hand one worker memory another
        // worker freed in its own stream order, and it then makes the first stream wait for the
        // second (a stroke batch would wait for a fill sweep). It keeps what is freed for reuse
        // (no release threshold), so steady-state batches allocate without the driver.
        cudaMemPoolProps props;
        std::memset(&props, 0, sizeof(props));
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = c.device;
        if (cudaMemPoolCreate(&w->pool, &props) == cudaSuccess) {
            uint64_t keep = ~0ull;
            cudaMemPoolSetAttribute(w->pool, cudaMemPoolAttrReleaseThreshold, &keep);
            int no = 0;
            cudaMemPoolSetAttribute(w->pool, cudaMemPoolReuseAllowInternalDependencies, &no);
        } else {
            cudaGetLastError();
            w->pool = nullptr;
        }
        const bool stroke_lane = i >= c.num_workers;
        w->role = c.num_stroke_workers == 0 ? ROLE_ANY : (stroke_lane ? ROLE_STROKE : ROLE_FILL);
        lg::srv_configure(w->ctx, stroke_lane, c.fill_blocks_per_sm, w->pool);
        s->workers.push_back(std::move(w));
    }
    for (auto& w : s->workers) w->th = std::thread(worker_main, s, w.get());
    return s;
}

void lyon_srv_destroy(lyon_srv* s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> g(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    for (auto& w : s->workers) {
        if (w->th.joinable()) w->th.join();
    }
    cudaSetDevice(s->cfg.device);
    for (auto& w : s->workers) {
        if (w->ctx) cudaStreamSynchronize(lg::srv_stream(w->ctx));
        for (Slab* sl : w->slabs) {
            cudaFree(sl->v);
            cudaFree(sl->i);
            cudaFree(sl->voff);
            cudaFree(sl->ioff);
            cudaFree(sl->st);
            delete sl;
        }
        cudaFreeHost(w->h_verbs);
        cudaFreeHost(w->h_points);
        cudaFreeHost(w->h_off);
        cudaFreeHost(w->h_opts);
        cudaFreeHost(w->h_res);
        for (void* h : w->retired_host) cudaFreeHost(h);
        cudaFree(w->d_verbs);
        cudaFree(w->d_points);
        cudaFree(w->d_off);
        cudaFree(w->d_opts);
        if (w->ctx) lyon_gpu_destroy(w->ctx);
        // After every buffer from it is freed (the context's included).
        if (w->pool) cudaMemPoolDestroy(w->pool);
    }
    for (auto& kv : s->reqs) delete kv.second;
    delete s;
}

int lyon_srv_get_config(const lyon_srv* s, lyon_srv_config* out) {
    if (!s || !out) return LYON_ERR_INVALID_ARGUMENT;
    *out = s->cfg;
    return LYON_OK;
}

uint64_t lyon_srv_submit(lyon_srv* s, int kind, const lyon_path_batch* batch, const void* options,
                         uint32_t num_options) {
    return submit_at(s, kind, batch, options, num_options, now_s());
}

int lyon_srv_poll(lyon_srv* s, uint64_t ticket, lyon_srv_result* out) {
    if (!s || !out) return LYON_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return LYON_ERR_INVALID_ARGUMENT;
    if (!it->second->done) return 1;
    fill_result(it->second, out);
    return LYON_OK;
}

int lyon_srv_wait(lyon_srv* s, uint64_t ticket, lyon_srv_result* out) {
    if (!s || !out) return LYON_ERR_INVALID_ARGUMENT;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return LYON_ERR_INVALID_ARGUMENT;
    Request* r = it->second;
    s->cv_done.wait(lk, [&] { return r->done; });
    fill_result(r, out);
    return LYON_OK;
}

int lyon_srv_release(lyon_srv* s, uint64_t ticket) {
    if (!s) return LYON_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end() || !it->second->done) return LYON_ERR_INVALID_ARGUMENT;
    Request* r = it->second;
    if (r->slab) {
        r->slab->refs -= 1;
        if (r->slab->refs == 0) s->held_bytes -= r->slab->bytes();
    }
    s->reqs.erase(it);
    delete r;
    s->cv_work.notify_all();
    return LYON_OK;
}

int lyon_srv_run_load(lyon_srv* s, const lyon_srv_load_item* items, uint32_t num_items,
                      double rate_per_s, double duration_s, uint64_t seed,
                      lyon_srv_load_stats* stats, double* latencies_ms, uint32_t latencies_cap) {
    if (!s || !items || num_items == 0 || rate_per_s <= 0 || duration_s <= 0 || !stats)
        return LYON_ERR_INVALID_ARGUMENT;
    std::memset(stats, 0, sizeof(*stats));
    uint64_t b0 = 0, bp0 = 0;
    for (auto& w : s->workers) {
        b0 += w->batches;
        bp0 += w->batch_paths;
    }
    std::mt19937_64 rng(seed);
    std::exponential_distribution<double> gap(rate_per_s);
    // Arrival times are drawn up front; the submitter sleeps until each one.
    std::vector<double> arrivals;
    double t = 0;
    while (true) {
        t += gap(rng);
        if (t >= duration_s) break;
        arrivals.push_back(t);
    }
    std::vector<uint64_t> tickets(arrivals.size(), 0);
    std::vector<double> lat;
    lat.reserve(arrivals.size());
    std::mutex tm;
    std::condition_variable tcv;
    size_t submitted = 0;
    const double t0 = now_s();
    std::thread submitter([&] {
        for (size_t k = 0; k < arrivals.size(); ++k) {
            const double due = t0 + arrivals[k];
            for (;;) {
                const double dt = due - now_s();
                if (dt <= 0) break;
                if (dt > 2e-4) std::this_thread::sleep_for(std::chrono::duration<double>(dt - 1e-4));
            }
            const lyon_srv_load_item& it = items[k % num_items];
            const uint64_t id = submit_at(s, it.kind, &it.batch, it.options, it.num_options, due);
            std::lock_guard<std::mutex> g(tm);
            tickets[k] = id;
            submitted = k + 1;
            tcv.notify_one();
        }
    });
    uint64_t paths = 0, verts = 0, idx = 0;
    uint32_t failed = 0;
    // Results are released as soon as they complete, in whatever order: waiting for them in
    // arrival order would let later requests that completed first hold the device-memory budget
    // while an earlier one waits for budget to run, and neither would move.
    std::vector<double> lat_k(arrivals.size(), -1.0);
    std::vector<size_t> pending;  // submitted, not yet released (arrival indices)
    size_t seen = 0, finished = 0;
    while (finished < arrivals.size()) {
        {
            std::lock_guard<std::mutex> g(tm);
            while (seen < submitted) pending.push_back(seen++);
        }
        bool progress = false;
        for (size_t j = 0; j < pending.size();) {
            const size_t k = pending[j];
            const uint64_t id = tickets[k];
            bool done = id == 0;
            if (id == 0) {
                failed++;
            } else {
                lyon_srv_result r;
                if (lyon_srv_poll(s, id, &r) == LYON_OK) {
                    done = true;
                    lat_k[k] = r.latency_ms;
                    if (r.status != LYON_OK) failed++;
                    paths += r.num_paths;
                    verts += r.num_vertices;
                    idx += r.num_indices;
                    lyon_srv_release(s, id);
                }
            }
            if (done) {
                pending[j] = pending.back();
                pending.pop_back();
                ++finished;
                progress = true;
            } else {
                ++j;
            }
        }
        if (!progress && finished < arrivals.size()) {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cv_done.wait_for(lk, std::chrono::milliseconds(1));
        }
    }
    submitter.join();
    for (size_t k = 0; k < lat_k.size(); ++k) {
        if (lat_k[k] >= 0.0) lat.push_back(lat_k[k]);
    }
    const double elapsed = now_s() - t0;
    std::vector<double> sorted = lat;
    std::sort(sorted.begin(), sorted.end());
    auto pct = [&](double q) {
        if (sorted.empty()) return 0.0;
        size_t i = (size_t)std::min<double>((double)sorted.size() - 1, q * (double)sorted.size());
        return sorted[i];
    };
    stats->submitted = (uint32_t)arrivals.size();
    stats->completed = (uint32_t)lat.size();
    stats->failed = failed;
    stats->offered_rate = rate_per_s;
    stats->elapsed_s = elapsed;
    stats->achieved_rate = lat.size() / elapsed;
    stats->paths = paths;
    stats->vertices = verts;
    stats->indices = idx;
    stats->p50_ms = pct(0.50);
    stats->p99_ms = pct(0.99);
    stats->p999_ms = pct(0.999);
    stats->max_ms = sorted.empty() ? 0.0 : sorted.back();
    uint64_t b1 = 0, bp1 = 0;
    for (auto& w : s->workers) {
        b1 += w->batches;
        bp1 += w->batch_paths;
    }
    stats->batches = b1 - b0;
    stats->mean_batch_paths = stats->batches ? (double)(bp1 - bp0) / (double)stats->batches : 0.0;
    if (latencies_ms) {
        for (size_t k = 0; k < lat.size() && k < latencies_cap; ++k) latencies_ms[k] = lat[k];
    }
    return LYON_OK;
}

}  // extern "C"
