// mmsp_gpu_server.cu -- the serving form (mmsp_gpu_server_*): a continuous
// batching request loop over the single-grid handles.
//
// Device memory: at start the server takes one block of the HBM budget and
// carves every admitted request's buffers out of it (first fit, 256-byte
// granules, freed blocks merge with their neighbours), so admission and
// retirement never call cudaMalloc or cudaFree, which synchronise the
// device.  Each admitted request gets a stream from a fixed set: requests of
// at most 2^21 values from the high-priority half (CUDA stream priorities),
// the rest from the low-priority half.
//
// One scheduler thread owns the device work and runs no rounds: it keeps up
// to two chunks of at most chunk_steps steps queued on every running
// request's stream, each followed by an event, and polls those events.
// When a request's last chunk completes it is reduced (mass, energy),
// copied to its host buffer and its block returned; queued requests are
// admitted in arrival order as soon as their footprint fits the budget and
// a block of that size is free.  Requests of different sizes therefore run
// side by side on the GPU and finish independently.  Every request runs the
// same kernels with the same step sequence as a lone mmsp_gpu_update (the
// chunking does not change a step's result), so its result does not depend
// on what else is running.  Clients only touch host structures under the
// mutex.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <new>
#include <thread>
#include <unordered_map>
#include <vector>

#include <stdio.h>
#include <string.h>

#include "MMSP.gpu.h"
#include "pf_handle.h"
#include "pf_internal.h"

namespace {

constexpr int kStreams = 128;      // streams for running requests, each given the least-used one of its priority class (half high priority)
constexpr long long kSmallValues = 1ll << 21;   // requests of at most this many values take high-priority streams
constexpr int kInFlight = 2;       // chunks queued ahead per request
constexpr size_t kGranule = 256;

struct Request {
    uint64_t id = 0;
    mmsp_gpu_desc d;
    int layout = MMSP_GPU_CELL_MAJOR;
    int steps = 0;
    std::atomic<int64_t> done{0};
    std::vector<unsigned char> host;   // initial state, then the result
    size_t footprint = 0;              // budget charge (mmsp_gpu_footprint)
    size_t block_off = 0, block_bytes = 0;
    mmsp_gpu_handle* h = nullptr;
    cudaStream_t stream = nullptr;
    int stream_index = -1;             // into the server's streams (scheduler thread)
    int state = MMSP_GPU_REQ_QUEUED;
    std::atomic<bool> cancel{false};
    int64_t queued = 0;                // steps queued on the device so far
    std::deque<std::pair<cudaEvent_t, int>> inflight;   // (event after the chunk, its steps)
    cudaEvent_t ev[kInFlight] = {nullptr, nullptr};
    int next_ev = 0;
    double submit_s = 0, admit_s = 0, finish_s = 0, mass = 0, energy = 0;
    char message[160] = {0};
};

// Keep the handle's message of a failed call.
static int note(Request* r, int rc, const char* what)
{
    if (rc && !r->message[0])
        snprintf(r->message, sizeof(r->message), "%s: %s", what, r->h ? mmsp_gpu_last_error(r->h) : mmsp_gpu_strerror(rc));
    return rc;
}

// First-fit sub-allocator over one device block.
struct Pool {
    char* base = nullptr;
    size_t size = 0;
    std::map<size_t, size_t> free;   // offset -> bytes

    bool alloc(size_t bytes, size_t* off)
    {
        bytes = (bytes + kGranule - 1) / kGranule * kGranule;
        for (auto it = free.begin(); it != free.end(); ++it)
            if (it->second >= bytes) {
                *off = it->first;
                const size_t rest = it->second - bytes;
                const size_t o = it->first + bytes;
                free.erase(it);
                if (rest) free[o] = rest;
                return true;
            }
        return false;
    }
    void release(size_t off, size_t bytes)
    {
        bytes = (bytes + kGranule - 1) / kGranule * kGranule;
        auto next = free.lower_bound(off);
        if (next != free.end() && off + bytes == next->first) {   // merge with the following block
            bytes += next->second;
            next = free.erase(next);
        }
        if (next != free.begin()) {
            auto prev = std::prev(next);
            if (prev->first + prev->second == off) {                // and with the preceding one
                prev->second += bytes;
                return;
            }
        }
        free[off] = bytes;
    }
};

using Clock = std::chrono::steady_clock;

}  // namespace

struct mmsp_gpu_server {
    int device = 0;
    size_t budget = 0, in_use = 0;
    int chunk = 200, max_active = 0;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Request*> queue;
    std::vector<Request*> active;
    std::unordered_map<uint64_t, Request*> all;
    uint64_t next_id = 1;
    bool stopping = false;
    std::thread th;
    Clock::time_point t0;
    mmsp_gpu_server_stats st;
    Pool pool;                    // the scheduler thread alone touches it
    cudaStream_t streams[kStreams] = {};   // [0, kStreams/2): high priority; the rest: low
    int stream_users[kStreams] = {};        // running requests on each stream
};

static double since(const mmsp_gpu_server* s) { return std::chrono::duration<double>(Clock::now() - s->t0).count(); }

// Called with s->mu held.
static void finish(mmsp_gpu_server* s, Request* r, int state)
{
    r->state = state;
    r->finish_s = since(s);
    if (state == MMSP_GPU_REQ_DONE) s->st.completed++;
    else if (state == MMSP_GPU_ECANCELED) s->st.cancelled++;
    else s->st.failed++;
    s->cv_done.notify_all();
}

// Scheduler thread: the request's device work is over (or never started);
// give back its handle, events and block.
static void release_request(mmsp_gpu_server* s, Request* r)
{
    if (r->stream) cudaStreamSynchronize(r->stream);
    if (r->stream_index >= 0) s->stream_users[r->stream_index]--;
    r->stream_index = -1;
    if (r->h) {
        mmsp_gpu_destroy(r->h);
        r->h = nullptr;
    }
    for (auto& e : r->ev)
        if (e) {
            cudaEventDestroy(e);
            e = nullptr;
        }
    r->inflight.clear();
    if (r->block_bytes) s->pool.release(r->block_off, r->block_bytes);
    r->block_bytes = 0;
    std::lock_guard<std::mutex> lock(s->mu);
    s->in_use -= r->footprint;
}

// Scheduler thread: queue chunks until kInFlight are in flight or the steps are all queued.
static int feed(mmsp_gpu_server* s, Request* r)
{
    while ((int)r->inflight.size() < kInFlight && r->queued < r->steps) {
        const int n = (int)std::min<int64_t>(s->chunk, r->steps - r->queued);
        int rc = note(r, mmsp_gpu_step(r->h, n), "step");
        if (rc) return rc;
        cudaEvent_t e = r->ev[r->next_ev];
        r->next_ev = (r->next_ev + 1) % kInFlight;
        if (cudaEventRecord(e, r->stream) != cudaSuccess) {
            cudaGetLastError();
            return note(r, MMSP_GPU_ECUDA, "event");
        }
        r->inflight.emplace_back(e, n);
        r->queued += n;
    }
    return MMSP_GPU_OK;
}

// Scheduler thread: device state for an admitted request (its block is set).
static int start_request(mmsp_gpu_server* s, Request* r)
{
    // Small grids run long chains of short steps; on high-priority streams the
    // block scheduler starts their kernels first whenever SMs free up, instead
    // of behind the large grids' full-GPU kernels.
    const long long values = (long long)r->d.n[0] * (r->d.dim > 1 ? r->d.n[1] : 1) * (r->d.dim > 2 ? r->d.n[2] : 1) *
                             r->d.fields;
    const int pri = values <= kSmallValues ? 0 : 1;
    // the least-used stream of the class: a stream shared with another running
    // request would make this request's synchronisations wait for its steps
    int best = pri * (kStreams / 2);
    for (int i = best + 1; i < (pri + 1) * (kStreams / 2); i++)
        if (s->stream_users[i] < s->stream_users[best]) best = i;
    s->stream_users[best]++;
    r->stream_index = best;
    r->stream = s->streams[best];
    for (auto& e : r->ev)
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
            cudaGetLastError();
            return note(r, MMSP_GPU_ECUDA, "event");
        }
    int rc = note(r, pf::create_in(&r->h, &r->d, s->pool.base + r->block_off, r->stream), "create");
    if (!rc) rc = note(r, mmsp_gpu_upload(r->h, r->host.data(), r->host.size(), r->layout), "upload");
    if (!rc) rc = feed(s, r);
    return rc;
}

static void scheduler(mmsp_gpu_server* s)
{
    cudaSetDevice(s->device);
    std::vector<Request*> admitted, running;
    while (true) {
        admitted.clear();
        {
            std::unique_lock<std::mutex> lock(s->mu);
            if (s->active.empty())
                s->cv_work.wait(lock, [&] { return s->stopping || !s->queue.empty(); });
            if (s->stopping) break;
            // admission, in arrival order, while the budget and a block allow
            while (!s->queue.empty()) {
                Request* r = s->queue.front();
                if (r->cancel) {
                    s->queue.pop_front();
                    finish(s, r, MMSP_GPU_ECANCELED);
                    continue;
                }
                if (s->max_active > 0 && (int)(s->active.size() + admitted.size()) >= s->max_active) break;
                if (s->in_use + r->footprint > s->budget) break;   // arrival order: wait for memory
                size_t off = 0;
                const size_t bytes = pf::handle_block_bytes(r->d);
                if (!s->pool.alloc(bytes, &off)) break;             // fragmented: wait for a block
                r->block_off = off;
                r->block_bytes = bytes;
                s->queue.pop_front();
                s->in_use += r->footprint;
                admitted.push_back(r);
            }
        }
        for (Request* r : admitted) {
            int rc = start_request(s, r);
            if (rc) {
                release_request(s, r);
                std::lock_guard<std::mutex> lock(s->mu);
                finish(s, r, rc);
                continue;
            }
            std::lock_guard<std::mutex> lock(s->mu);
            r->state = MMSP_GPU_REQ_RUNNING;
            r->admit_s = since(s);
            s->st.admitted++;
            s->active.push_back(r);
        }
        {
            std::lock_guard<std::mutex> lock(s->mu);
            running = s->active;
            s->st.rounds++;
        }
        // progress of every running request: completed chunks, the next ones, retirement
        bool progressed = !admitted.empty();
        for (Request* r : running) {
            int rc = MMSP_GPU_OK;
            while (!r->inflight.empty()) {
                cudaError_t q = cudaEventQuery(r->inflight.front().first);
                if (q == cudaErrorNotReady) break;
                if (q != cudaSuccess) {
                    cudaGetLastError();
                    rc = note(r, MMSP_GPU_ECUDA, "chunk");
                    break;
                }
                r->done += r->inflight.front().second;
                r->inflight.pop_front();
                progressed = true;
            }
            if (!rc && !r->cancel && r->done < r->steps) rc = feed(s, r);
            int end_state = 0;
            bool end = false;
            if (rc) {
                end = true;
                end_state = rc;
            } else if (r->cancel) {
                end = true;
                end_state = MMSP_GPU_ECANCELED;
            } else if (r->done >= r->steps) {
                mmsp_gpu_stats stt;
                rc = note(r, mmsp_gpu_synchronize(r->h), "synchronize");
                if (!rc) rc = note(r, mmsp_gpu_reduce(r->h, &stt), "reduce");
                if (!rc) rc = note(r, mmsp_gpu_download(r->h, r->host.data(), r->host.size(), r->layout), "download");
                r->mass = stt.mass;
                r->energy = stt.energy;
                end = true;
                end_state = rc ? rc : MMSP_GPU_REQ_DONE;
            }
            if (end) {
                progressed = true;
                release_request(s, r);
                std::lock_guard<std::mutex> lock(s->mu);
                for (size_t i = 0; i < s->active.size(); i++)
                    if (s->active[i] == r) {
                        s->active.erase(s->active.begin() + i);
                        break;
                    }
                finish(s, r, end_state);
            }
        }
        if (!progressed) {
            // nothing finished: wait briefly for the GPU or a new submission
            std::unique_lock<std::mutex> lock(s->mu);
            s->cv_work.wait_for(lock, std::chrono::microseconds(50));
        }
    }
    // stopping: everything not finished ends with ESTOPPED
    std::vector<Request*> left;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        left = s->active;
        s->active.clear();
    }
    for (Request* r : left) {
        release_request(s, r);
        std::lock_guard<std::mutex> lock(s->mu);
        finish(s, r, MMSP_GPU_ESTOPPED);
    }
    std::lock_guard<std::mutex> lock(s->mu);
    for (Request* r : s->queue) finish(s, r, MMSP_GPU_ESTOPPED);
    s->queue.clear();
}

static void fill_status(const Request* r, mmsp_gpu_request_status* st)
{
    st->state = r->state;
    st->steps_total = r->steps;
    st->steps_done = r->done.load();
    st->submit_s = r->submit_s;
    st->admit_s = r->admit_s;
    st->finish_s = r->finish_s;
    st->mass = r->mass;
    st->energy = r->energy;
    memcpy(st->message, r->message, sizeof(st->message));
}

static bool finished(const Request* r) { return r->state == MMSP_GPU_REQ_DONE || r->state < 0; }

extern "C" int mmsp_gpu_server_start(mmsp_gpu_server** out, const mmsp_gpu_server_config* cfg)
{
    if (!out) return MMSP_GPU_EINVAL;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
        cudaGetLastError();
        return MMSP_GPU_ENODEV;
    }
    mmsp_gpu_server* s = new (std::nothrow) mmsp_gpu_server();
    if (!s) return MMSP_GPU_ENOMEM;
    memset(&s->st, 0, sizeof(s->st));
    cudaGetDevice(&s->device);
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
        cudaGetLastError();
        delete s;
        return MMSP_GPU_ECUDA;
    }
    s->budget = (cfg && cfg->hbm_budget_bytes) ? cfg->hbm_budget_bytes : (size_t)(0.8 * (double)free_b);
    if (s->budget > free_b) s->budget = free_b;
    // the one device block requests are carved from (a little above the budget:
    // blocks are 256-byte aligned per buffer); halve it until the device grants it
    size_t want = s->budget + s->budget / 64 + (64u << 20);
    while (want >= (64u << 20) && cudaMalloc((void**)&s->pool.base, want) != cudaSuccess) {
        cudaGetLastError();
        want /= 2;
    }
    if (!s->pool.base) {
        delete s;
        return MMSP_GPU_ENOMEM;
    }
    s->pool.size = want;
    s->pool.free[0] = want;
    if (s->budget > want) s->budget = want;
    int lo_pri = 0, hi_pri = 0;
    if (cudaDeviceGetStreamPriorityRange(&lo_pri, &hi_pri) != cudaSuccess) {
        cudaGetLastError();
        lo_pri = hi_pri = 0;
    }
    for (int i = 0; i < kStreams; i++)
        if (cudaStreamCreateWithPriority(&s->streams[i], cudaStreamNonBlocking, i < kStreams / 2 ? hi_pri : lo_pri) !=
            cudaSuccess) {
            cudaGetLastError();
            for (auto& t : s->streams)
                if (t) cudaStreamDestroy(t);
            cudaFree(s->pool.base);
            delete s;
            return MMSP_GPU_ECUDA;
        }
    // multiples of 4: 2D FP32 Cahn-Hilliard handles run 4 steps per launch, and
    // chunks of whole blocks give the same launches as one call of all steps
    if (cfg && cfg->chunk_steps > 0) s->chunk = std::max(4, cfg->chunk_steps / 4 * 4);
    if (cfg && cfg->max_active > 0) s->max_active = cfg->max_active;
    s->st.device_bytes_budget = s->budget;
    s->t0 = Clock::now();
    try {
        s->th = std::thread(scheduler, s);
    } catch (...) {
        for (auto& t : s->streams)
            if (t) cudaStreamDestroy(t);
        cudaFree(s->pool.base);
        delete s;
        return MMSP_GPU_ENOMEM;
    }
    *out = s;
    return MMSP_GPU_OK;
}

extern "C" int mmsp_gpu_server_submit(mmsp_gpu_server* s, const mmsp_gpu_desc* desc, const void* host, size_t bytes,
                                      int layout, int steps, uint64_t* id)
{
    if (!s || !desc || !host || steps < 0 || !id) return MMSP_GPU_EINVAL;
    if (layout != MMSP_GPU_CELL_MAJOR && layout != MMSP_GPU_FIELD_MAJOR) return MMSP_GPU_EINVAL;
    if (desc->model == MMSP_GPU_SPARSE_GG) return MMSP_GPU_EUNSUPPORTED;   // lists, not a dense state
    size_t fp = 0;
    int rc = mmsp_gpu_footprint(desc, &fp);
    if (rc) return rc;
    size_t want = (size_t)desc->fields * (desc->dtype == MMSP_GPU_F64 ? 8 : 4);
    for (int a = 0; a < desc->dim; a++) want *= (size_t)desc->n[a];
    if (bytes != want) return MMSP_GPU_EINVAL;
    Request* r = new (std::nothrow) Request();
    if (!r) return MMSP_GPU_ENOMEM;
    r->d = *desc;
    r->layout = layout;
    r->steps = steps;
    r->footprint = fp;
    try {
        r->host.assign((const unsigned char*)host, (const unsigned char*)host + bytes);
    } catch (...) {
        delete r;
        return MMSP_GPU_ENOMEM;
    }
    std::lock_guard<std::mutex> lock(s->mu);
    if (s->stopping) {
        delete r;
        return MMSP_GPU_ESTOPPED;
    }
    if (fp > s->budget) {
        delete r;
        return MMSP_GPU_ENOMEM;   // could never be admitted
    }
    r->id = s->next_id++;
    r->submit_s = since(s);
    s->all[r->id] = r;
    s->queue.push_back(r);
    s->st.submitted++;
    *id = r->id;
    s->cv_work.notify_one();
    return MMSP_GPU_OK;
}

extern "C" int mmsp_gpu_server_poll(mmsp_gpu_server* s, uint64_t id, mmsp_gpu_request_status* st)
{
    if (!s || !st) return MMSP_GPU_EINVAL;
    std::lock_guard<std::mutex> lock(s->mu);
    auto it = s->all.find(id);
    if (it == s->all.end()) return MMSP_GPU_ENOTFOUND;
    fill_status(it->second, st);
    return MMSP_GPU_OK;
}

extern "C" int mmsp_gpu_server_wait(mmsp_gpu_server* s, uint64_t id, double timeout_s, mmsp_gpu_request_status* st)
{
    if (!s) return MMSP_GPU_EINVAL;
    std::unique_lock<std::mutex> lock(s->mu);
    auto it = s->all.find(id);
    if (it == s->all.end()) return MMSP_GPU_ENOTFOUND;
    Request* r = it->second;
    const auto deadline = Clock::now() + std::chrono::duration_cast<Clock::duration>(
                                             std::chrono::duration<double>(timeout_s < 0 ? 0 : timeout_s));
    bool ok = s->cv_done.wait_until(lock, deadline, [&] { return finished(r); });
    if (st) fill_status(r, st);
    return ok ? MMSP_GPU_OK : MMSP_GPU_ETIMEDOUT;
}

extern "C" int mmsp_gpu_server_fetch(mmsp_gpu_server* s, uint64_t id, void* host, size_t bytes, int layout)
{
    if (!s || !host) return MMSP_GPU_EINVAL;
    std::lock_guard<std::mutex> lock(s->mu);
    auto it = s->all.find(id);
    if (it == s->all.end()) return MMSP_GPU_ENOTFOUND;
    Request* r = it->second;
    if (!finished(r)) return MMSP_GPU_EINVAL;
    if (r->state != MMSP_GPU_REQ_DONE) {
        int code = r->state;
        s->all.erase(it);
        delete r;
        return code;
    }
    if (bytes != r->host.size() || layout != r->layout) return MMSP_GPU_EINVAL;
    memcpy(host, r->host.data(), bytes);
    s->all.erase(it);
    delete r;
    return MMSP_GPU_OK;
}

extern "C" int mmsp_gpu_server_cancel(mmsp_gpu_server* s, uint64_t id)
{
    if (!s) return MMSP_GPU_EINVAL;
    std::lock_guard<std::mutex> lock(s->mu);
    auto it = s->all.find(id);
    if (it == s->all.end()) return MMSP_GPU_ENOTFOUND;
    it->second->cancel = true;
    s->cv_work.notify_one();
    return MMSP_GPU_OK;
}

extern "C" int mmsp_gpu_server_get_stats(mmsp_gpu_server* s, mmsp_gpu_server_stats* st)
{
    if (!s || !st) return MMSP_GPU_EINVAL;
    std::lock_guard<std::mutex> lock(s->mu);
    *st = s->st;
    st->queued = (int)s->queue.size();
    st->active = (int)s->active.size();
    st->device_bytes_in_use = s->in_use;
    st->device_bytes_budget = s->budget;
    return MMSP_GPU_OK;
}

extern "C" int mmsp_gpu_server_stop(mmsp_gpu_server* s)
{
    if (!s) return MMSP_GPU_OK;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        s->stopping = true;
        s->cv_work.notify_all();
    }
    if (s->th.joinable()) s->th.join();
    for (auto& kv : s->all) delete kv.second;
    s->all.clear();
    for (auto& t : s->streams)
        if (t) cudaStreamDestroy(t);
    if (s->pool.base) cudaFree(s->pool.base);
    delete s;
    return MMSP_GPU_OK;
}
