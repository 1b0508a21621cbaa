// mmsp_gpu_output.cu -- the output path of include/MMSP.gpu.h: MMSP grid
// files from host values (mmsp_gpu_write_grid) and snapshots of a handle's
// device state (mmsp_gpu_output / mmsp_gpu_output_wait).
//
// A snapshot is three stages that overlap later steps:
//   1. on the handle's stream: the state is packed into a device staging
//      buffer in to_buffer order (include/MMSP.grid.cpp:1146-1157; a vector
//      cell is int32 N then N values, include/MMSP.vector.cpp:95-117), or
//      copied there as it is for scalar grids;
//   2. on a copy stream: staging -> one of two pinned host buffers;
//   3. on a writer thread: wait for that copy, compress on several threads
//      and write the file (pf_gridfile.cu).
// The staging buffer is reused: the next pack waits (on the device) for the
// previous copy out of it.  A host buffer is reused once its file is written.
#include <string.h>

#include <condition_variable>
#include <deque>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "MMSP.gpu.h"
#include "pf_gridfile.h"
#include "pf_handle.h"

namespace pf {

// Word k of the packed payload, where every cell record is `wpr` 32-bit
// words: word 0 the field count, then the cell's values in field order
// (a double as its low then high word, little-endian).  One thread per
// output word, so the writes are coalesced; the reads gather the fields of
// a cell from the field-major state.
template <typename T>
__global__ void pack_vector_cells(const T* __restrict__ src, uint32_t* __restrict__ dst, long long cells, int N)
{
    constexpr int WPV = sizeof(T) / 4;   // words per value
    const long long wpr = 1 + (long long)N * WPV;
    const long long words = cells * wpr;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < words;
         k += (long long)gridDim.x * blockDim.x) {
        const long long cell = k / wpr;
        const int r = (int)(k - cell * wpr);
        uint32_t w;
        if (r == 0) {
            w = (uint32_t)N;
        } else {
            const int f = (r - 1) / WPV;
            const T v = src[(long long)f * cells + cell];
            if constexpr (WPV == 1) {
                w = __float_as_uint(v);
            } else {
                const unsigned long long b = (unsigned long long)__double_as_longlong(v);
                w = ((r - 1) & 1) ? (uint32_t)(b >> 32) : (uint32_t)b;
            }
        }
        dst[k] = w;
    }
}

struct OutputJob {
    std::string filename;
    GridFileInfo fi;
    size_t bytes;
    int level, threads, slot;
};

struct OutputState {
    int device = 0;
    size_t cap = 0;                       // bytes of the staging and host buffers
    unsigned char* staging = nullptr;     // device
    unsigned char* host[2] = {nullptr, nullptr};
    bool busy[2] = {false, false};
    cudaEvent_t copied[2] = {nullptr, nullptr};   // host[s] holds its snapshot
    cudaEvent_t packed = nullptr;                 // staging holds a snapshot
    cudaEvent_t drained = nullptr;                // the last copy out of staging is done
    cudaStream_t copy = nullptr;
    std::thread writer;
    std::mutex m;
    std::condition_variable cv;
    std::deque<OutputJob> queue;
    int pending = 0;   // jobs queued or being written
    bool stop = false;
    int error = 0;     // first failure since the last mmsp_gpu_output_wait
    std::string why;

    void run()
    {
        cudaSetDevice(device);
        for (;;) {
            OutputJob j;
            {
                std::unique_lock<std::mutex> lk(m);
                cv.wait(lk, [&] { return stop || !queue.empty(); });
                if (queue.empty()) return;
                j = queue.front();
                queue.pop_front();
            }
            std::string w;
            int rc = MMSP_GPU_OK;
            cudaError_t e = cudaEventSynchronize(copied[j.slot]);
            if (e != cudaSuccess)
                rc = MMSP_GPU_ECUDA, w = std::string("output copy: ") + cudaGetErrorString(e);
            else   // write_grid_file throws nothing: failures come back as codes
                rc = write_grid_file(j.filename.c_str(), j.fi, host[j.slot], j.bytes, j.level, j.threads, &w);
            {
                std::lock_guard<std::mutex> lk(m);
                busy[j.slot] = false;
                pending--;
                if (rc && !error) error = rc, why = w;
            }
            cv.notify_all();
        }
    }

    void wait_idle()
    {
        std::unique_lock<std::mutex> lk(m);
        cv.wait(lk, [&] { return pending == 0; });
    }

    void free_buffers()
    {
        if (staging) cudaFree(staging);
        for (int s = 0; s < 2; s++)
            if (host[s]) cudaFreeHost(host[s]);
        staging = nullptr;
        host[0] = host[1] = nullptr;
        cap = 0;
    }

    ~OutputState()
    {
        if (writer.joinable()) {
            {
                std::lock_guard<std::mutex> lk(m);
                stop = true;
            }
            cv.notify_all();
            writer.join();
        }
        if (copy) cudaStreamSynchronize(copy);
        free_buffers();
        for (int s = 0; s < 2; s++)
            if (copied[s]) cudaEventDestroy(copied[s]);
        if (packed) cudaEventDestroy(packed);
        if (drained) cudaEventDestroy(drained);
        if (copy) cudaStreamDestroy(copy);
    }
};

void output_release(mmsp_gpu_handle* h)
{
    if (!h->out) return;
    h->out->wait_idle();
    delete h->out;
    h->out = nullptr;
}

}  // namespace pf

using pf::GridFileInfo;
using pf::OutputState;

static int out_fail(mmsp_gpu_handle* h, int code, const std::string& why)
{
    if (h) snprintf(h->err, sizeof(h->err), "%s", why.c_str());
    return code;
}

static int out_cuda(mmsp_gpu_handle* h, cudaError_t e, const char* where)
{
    cudaGetLastError();
    return out_fail(h, e == cudaErrorMemoryAllocation ? MMSP_GPU_ENOMEM : MMSP_GPU_ECUDA,
                    std::string(where) + ": " + cudaGetErrorString(e));
}

extern "C" int mmsp_gpu_output_opts_init(mmsp_gpu_output_opts* o)
{
    if (!o) return MMSP_GPU_EINVAL;
    memset(o, 0, sizeof(*o));
    o->level = 9;
    o->threads = 0;
    o->vector = -1;
    o->fields_line = -1;
    return MMSP_GPU_OK;
}

// File geometry of a descriptor; EINVAL for a shape no grid file holds.
static int file_info(const mmsp_gpu_desc* d, const mmsp_gpu_output_opts* o, GridFileInfo* fi, std::string* why)
{
    if (!d || d->dim < 1 || d->dim > 3 || d->fields < 1 || (d->dtype != MMSP_GPU_F64 && d->dtype != MMSP_GPU_F32)) {
        *why = "output: invalid descriptor";
        return MMSP_GPU_EINVAL;
    }
    if (o->level < 0 || o->level > 9) {
        *why = "output: level must be 0..9";
        return MMSP_GPU_EINVAL;
    }
    if (d->model == MMSP_GPU_SPARSE_GG) {
        *why = "output: sparse grids are not written as grid files";
        return MMSP_GPU_EUNSUPPORTED;
    }
    memset(fi, 0, sizeof(*fi));
    fi->dim = d->dim;
    fi->vector = o->vector < 0 ? d->fields > 1 : o->vector != 0;
    if (!fi->vector && d->fields != 1) {
        *why = "output: a scalar grid file holds one value per cell";
        return MMSP_GPU_EINVAL;
    }
    fi->f64 = d->dtype == MMSP_GPU_F64;
    fi->fields_line = o->fields_line >= 0 ? o->fields_line : (fi->vector ? d->fields : 0);
    for (int a = 0; a < d->dim; a++) {
        if (d->n[a] < 1) {
            *why = "output: extents must be positive";
            return MMSP_GPU_EINVAL;
        }
        fi->g0[a] = o->g0[a];
        fi->n[a] = d->n[a];
        fi->bc[a][0] = d->bc[a][0];
        fi->bc[a][1] = d->bc[a][1];
        fi->dx[a] = d->dx[a];
    }
    return MMSP_GPU_OK;
}

extern "C" int mmsp_gpu_write_grid(const char* filename, const mmsp_gpu_desc* desc, const void* host, size_t bytes,
                                   int layout, const mmsp_gpu_output_opts* opts)
{
    mmsp_gpu_output_opts def;
    mmsp_gpu_output_opts_init(&def);
    const mmsp_gpu_output_opts* o = opts ? opts : &def;
    if (!filename || !host) return MMSP_GPU_EINVAL;
    GridFileInfo fi;
    std::string why;
    int rc = file_info(desc, o, &fi, &why);
    if (rc) return rc;
    const size_t es = fi.f64 ? sizeof(double) : sizeof(float);
    size_t cells = 1;
    for (int a = 0; a < desc->dim; a++) cells *= (size_t)desc->n[a];
    const int N = desc->fields;
    if (bytes != cells * (size_t)N * es) return MMSP_GPU_EINVAL;
    if (N > 1 && layout != MMSP_GPU_CELL_MAJOR && layout != MMSP_GPU_FIELD_MAJOR) return MMSP_GPU_EINVAL;
    if (!fi.vector) return pf::write_grid_file(filename, fi, host, bytes, o->level, o->threads, &why);
    // vector cells: int32 N, then the cell's N values
    const size_t rec = sizeof(int32_t) + (size_t)N * es;
    std::vector<unsigned char> payload;
    try {
        payload.resize(cells * rec);
    } catch (...) {
        return MMSP_GPU_ENOMEM;
    }
    const unsigned char* src = static_cast<const unsigned char*>(host);
    const int32_t n32 = N;
    for (size_t i = 0; i < cells; i++) {
        unsigned char* r = payload.data() + i * rec;
        memcpy(r, &n32, sizeof(n32));
        if (N == 1 || layout == MMSP_GPU_CELL_MAJOR) {
            memcpy(r + sizeof(n32), src + i * N * es, N * es);
        } else {
            for (int f = 0; f < N; f++) memcpy(r + sizeof(n32) + f * es, src + ((size_t)f * cells + i) * es, es);
        }
    }
    return pf::write_grid_file(filename, fi, payload.data(), payload.size(), o->level, o->threads, &why);
}

// Buffers for snapshots of `bytes`; waits for running jobs before growing them.
static int ensure_output(mmsp_gpu_handle* h, size_t bytes)
{
    OutputState* s = h->out;
    cudaError_t e;
    if (!s) {
        s = new (std::nothrow) OutputState();
        if (!s) return MMSP_GPU_ENOMEM;
        s->device = h->device;
        if ((e = cudaStreamCreateWithFlags(&s->copy, cudaStreamNonBlocking)) != cudaSuccess ||
            (e = cudaEventCreateWithFlags(&s->packed, cudaEventDisableTiming)) != cudaSuccess ||
            (e = cudaEventCreateWithFlags(&s->drained, cudaEventDisableTiming)) != cudaSuccess ||
            (e = cudaEventCreateWithFlags(&s->copied[0], cudaEventDisableTiming)) != cudaSuccess ||
            (e = cudaEventCreateWithFlags(&s->copied[1], cudaEventDisableTiming)) != cudaSuccess) {
            delete s;
            return out_cuda(h, e, "output");
        }
        try {
            s->writer = std::thread([s] { s->run(); });
        } catch (...) {
            delete s;
            return out_fail(h, MMSP_GPU_ENOMEM, "output: could not start the writer thread");
        }
        h->out = s;
    }
    if (s->cap >= bytes) return MMSP_GPU_OK;
    s->wait_idle();
    cudaStreamSynchronize(s->copy);
    s->free_buffers();
    if ((e = cudaMalloc((void**)&s->staging, bytes)) != cudaSuccess ||
        (e = cudaHostAlloc((void**)&s->host[0], bytes, cudaHostAllocDefault)) != cudaSuccess ||
        (e = cudaHostAlloc((void**)&s->host[1], bytes, cudaHostAllocDefault)) != cudaSuccess) {
        s->free_buffers();
        return out_cuda(h, e, "output buffers");
    }
    s->cap = bytes;
    return MMSP_GPU_OK;
}

extern "C" int mmsp_gpu_output(mmsp_gpu_handle* h, const char* filename, const mmsp_gpu_output_opts* opts)
{
    if (!h || !filename) return MMSP_GPU_EINVAL;
    mmsp_gpu_output_opts def;
    mmsp_gpu_output_opts_init(&def);
    const mmsp_gpu_output_opts* o = opts ? opts : &def;
    GridFileInfo fi;
    std::string why;
    int rc = file_info(&h->d, o, &fi, &why);
    if (rc) return out_fail(h, rc, why);
    const size_t bytes = pf::payload_bytes(fi, h->d.fields);
    if ((rc = ensure_output(h, bytes))) return rc;
    OutputState* s = h->out;

    int slot;
    {
        std::unique_lock<std::mutex> lk(s->m);
        s->cv.wait(lk, [&] { return !s->busy[0] || !s->busy[1]; });
        slot = s->busy[0] ? 1 : 0;
    }
    cudaError_t e;
    // stage 1 (handle's stream), after the previous copy out of staging
    if ((e = cudaStreamWaitEvent(h->stream, s->drained, 0)) != cudaSuccess) return out_cuda(h, e, "output");
    const void* state = h->buf[h->cur];
    if (fi.vector) {
        const long long words = (long long)(bytes / 4);
        const int threads = 256;
        long long blocks = (words + threads - 1) / threads;
        const long long most = 8LL * pf::sm_count();   // grid-stride beyond 8 blocks per SM
        if (blocks > most) blocks = most;
        if (fi.f64)
            pf::pack_vector_cells<double><<<(int)blocks, threads, 0, h->stream>>>(
                (const double*)state, (uint32_t*)s->staging, h->g.cells, h->d.fields);
        else
            pf::pack_vector_cells<float><<<(int)blocks, threads, 0, h->stream>>>(
                (const float*)state, (uint32_t*)s->staging, h->g.cells, h->d.fields);
        e = cudaGetLastError();
    } else {
        e = cudaMemcpyAsync(s->staging, state, bytes, cudaMemcpyDeviceToDevice, h->stream);
    }
    if (e != cudaSuccess) return out_cuda(h, e, "output pack");
    // stage 2 (copy stream)
    if ((e = cudaEventRecord(s->packed, h->stream)) != cudaSuccess ||
        (e = cudaStreamWaitEvent(s->copy, s->packed, 0)) != cudaSuccess ||
        (e = cudaMemcpyAsync(s->host[slot], s->staging, bytes, cudaMemcpyDeviceToHost, s->copy)) != cudaSuccess ||
        (e = cudaEventRecord(s->copied[slot], s->copy)) != cudaSuccess ||
        (e = cudaEventRecord(s->drained, s->copy)) != cudaSuccess)
        return out_cuda(h, e, "output copy");
    // stage 3 (writer thread)
    try {
        pf::OutputJob j;
        j.filename = filename;
        j.fi = fi;
        j.bytes = bytes;
        j.level = o->level;
        j.threads = o->threads;
        j.slot = slot;
        std::lock_guard<std::mutex> lk(s->m);
        s->queue.push_back(j);
        s->busy[slot] = true;
        s->pending++;
    } catch (...) {
        cudaStreamSynchronize(s->copy);   // the copy into the slot must end before the slot is reused
        return out_fail(h, MMSP_GPU_ENOMEM, "output: out of host memory");
    }
    s->cv.notify_all();
    return MMSP_GPU_OK;
}

extern "C" int mmsp_gpu_output_wait(mmsp_gpu_handle* h)
{
    if (!h) return MMSP_GPU_EINVAL;
    OutputState* s = h->out;
    if (!s) return MMSP_GPU_OK;
    s->wait_idle();
    std::lock_guard<std::mutex> lk(s->m);
    const int rc = s->error;
    if (rc) out_fail(h, rc, s->why);
    s->error = 0;
    s->why.clear();
    return rc;
}
