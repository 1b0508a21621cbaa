// mmsp_gpu_batch.cu -- the batched form of the C ABI (mmsp_gpu_batch_*).
//
// Grids live in two device pools (ping-pong) at 256-byte aligned offsets.
// Eligible 2D Cahn-Hilliard grids are advanced by one persistent kernel per
// step (pf_batch.cu); the others keep their own step plans and kernels.  A
// step chunk of kBatchGraphSteps steps is captured once as a CUDA graph and
// replayed.  The autotuner times candidate (rows per item, block size)
// pairs on the batch itself, reading the live state and writing only the
// idle pool, and caches the winner per batch shape.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <iterator>
#include <map>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "MMSP.gpu.h"
#include "pf_batch.h"
#include "pf_internal.h"

using namespace pf;

namespace {

constexpr int kBatchGraphSteps = 64;   // even: a replay returns the state to pool 0

struct Member {
    mmsp_gpu_desc d;
    Geom g;
    Coeffs c;
    long long off;     // element offset in the pools
    size_t bytes;
    bool persistent;
    StepPlan plan;     // own kernel when not persistent
};

struct Tuning {
    int rows = 0, threads = 0;   // per-step kernel: rows per work item, block size
    int ks = 0, shape = 0;       // temporally blocked kernel: steps per launch (0: not used), region shape
};

std::mutex g_tune_mu;
std::map<std::string, Tuning> g_tune;   // batch shape -> tuning

}  // namespace

struct mmsp_gpu_batch {
    std::vector<Member> m;
    int dtype;
    size_t esize;
    long long pool_elems;
    void* pool[2];
    int cur;
    long long launches;          // persistent launches so far (counter parity)
    double* partials;
    int* counters;               // [0..1] work counters, [2] error word
    BatchInst* d_insts;
    BatchItem* d_items;
    int nitems;
    int items_cap;
    std::vector<BatchInst> insts;
    int persistent_model;
    bool unit;
    int npersistent;
    Tuning tune;
    // temporally blocked kernel (FP32 batches of persistent grids only)
    TbItem* d_tb;
    int tb_nitems, tb_cap, tb_blocks;
    bool tuned, tuned_from_cache;
    double tune_ms;
    int blocks;
    cudaStream_t own, stream;
    cudaGraphExec_t graph;
    std::string err;
};

static int bfail(mmsp_gpu_batch* b, int code, const std::string& msg)
{
    if (b) b->err = msg;
    return code;
}

static int bcuda(mmsp_gpu_batch* b, cudaError_t e, const char* where)
{
    if (b) b->err = std::string(where) + ": " + cudaGetErrorString(e);
    cudaGetLastError();
    return MMSP_GPU_ECUDA;
}

static void brelease(mmsp_gpu_batch* b)
{
    if (b->graph) cudaGraphExecDestroy(b->graph);
    for (int i = 0; i < 2; i++)
        if (b->pool[i]) cudaFree(b->pool[i]);
    if (b->partials) cudaFree(b->partials);
    if (b->counters) cudaFree(b->counters);
    if (b->d_insts) cudaFree(b->d_insts);
    if (b->d_items) cudaFree(b->d_items);
    if (b->d_tb) cudaFree(b->d_tb);
    if (b->own) cudaStreamDestroy(b->own);
}

extern "C" int mmsp_gpu_batch_create(mmsp_gpu_batch** out, int count, const mmsp_gpu_desc* descs)
{
    if (!out || count < 1 || !descs) return MMSP_GPU_EINVAL;
    *out = nullptr;
    for (int i = 0; i < count; i++) {
        int rc = mmsp_gpu_validate(&descs[i]);
        if (rc) return rc;
        if (descs[i].dtype != descs[0].dtype) return MMSP_GPU_EINVAL;
        // serve these through handles: a work grid, or a per-step noise index
        if (descs[i].model == MMSP_GPU_OSTWALD || descs[i].model == MMSP_GPU_CH_CONVEX ||
            descs[i].model == MMSP_GPU_SPARSE_GG || pf::noisy(descs[i]))
            return MMSP_GPU_EUNSUPPORTED;
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
        cudaGetLastError();
        return MMSP_GPU_ENODEV;
    }
    mmsp_gpu_batch* b = new (std::nothrow) mmsp_gpu_batch();
    if (!b) return MMSP_GPU_ENOMEM;
    b->dtype = descs[0].dtype;
    b->esize = b->dtype == MMSP_GPU_F64 ? sizeof(double) : sizeof(float);
    const long long align = 256 / (long long)b->esize;
    b->persistent_model = -1;
    b->unit = true;
    long long off = 0;
    for (int i = 0; i < count; i++) {
        Member mm;
        memset(&mm, 0, sizeof(mm));
        mm.d = descs[i];
        for (int a = mm.d.dim; a < 3; a++) mm.d.n[a] = 1;
        mm.g = make_geom(mm.d);
        mm.c = make_coeffs(mm.d);
        mm.off = off;
        mm.bytes = (size_t)mm.g.cells * mm.d.fields * b->esize;
        off += (mm.g.cells * mm.d.fields + align - 1) / align * align;
        if (batch_eligible(mm.d) && (b->persistent_model < 0 || b->persistent_model == mm.d.model)) {
            mm.persistent = true;
            b->persistent_model = mm.d.model;
            if (!mm.c.unit_w) b->unit = false;
            BatchInst bi;
            bi.off = mm.off;
            bi.n0 = mm.d.n[0];
            bi.n1 = mm.d.n[1];
            bi.w0 = mm.c.w[0];
            bi.w1 = mm.c.w[1];
            bi.kappa = mm.c.kappa;
            bi.dtm = mm.c.dtm;
            bi.neg_r = mm.c.neg_r;
            bi.u = mm.c.u;
            b->insts.push_back(bi);
        }
        b->m.push_back(mm);
    }
    b->npersistent = (int)b->insts.size();
    b->pool_elems = off;
    cudaError_t e = cudaStreamCreateWithFlags(&b->own, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        brelease(b);
        delete b;
        return MMSP_GPU_ECUDA;
    }
    b->stream = b->own;
    const size_t pool_bytes = (size_t)off * b->esize;
    bool ok = cudaMalloc(&b->pool[0], pool_bytes) == cudaSuccess && cudaMalloc(&b->pool[1], pool_bytes) == cudaSuccess &&
              cudaMalloc((void**)&b->partials, kPartialsBytes) == cudaSuccess &&
              cudaMalloc((void**)&b->counters, 256) == cudaSuccess;
    if (ok && b->npersistent > 0)
        ok = cudaMalloc((void**)&b->d_insts, sizeof(BatchInst) * b->insts.size()) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        brelease(b);
        delete b;
        return MMSP_GPU_ENOMEM;
    }
    e = cudaMemset(b->counters, 0, 256);
    if (e == cudaSuccess) e = cudaMemset(b->pool[0], 0, pool_bytes);
    if (e == cudaSuccess) e = cudaMemset(b->pool[1], 0, pool_bytes);
    if (e == cudaSuccess && b->npersistent > 0)
        e = cudaMemcpy(b->d_insts, b->insts.data(), sizeof(BatchInst) * b->insts.size(), cudaMemcpyHostToDevice);
    for (auto& mm : b->m) {
        if (mm.persistent || e != cudaSuccess) continue;
        const bool ch = mm.d.model == MMSP_GPU_CH || mm.d.model == MMSP_GPU_CH_POLY;
        e = ch ? plan_ch(mm.d, mm.g, &mm.plan) : plan_ac(mm.d, mm.g, &mm.plan);
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        brelease(b);
        delete b;
        return MMSP_GPU_EUNSUPPORTED;
    }
    *out = b;
    return MMSP_GPU_OK;
}

extern "C" int mmsp_gpu_batch_destroy(mmsp_gpu_batch* b)
{
    if (!b) return MMSP_GPU_OK;
    cudaStreamSynchronize(b->stream);
    brelease(b);
    delete b;
    return MMSP_GPU_OK;
}

extern "C" int mmsp_gpu_batch_set_stream(mmsp_gpu_batch* b, void* s)
{
    if (!b) return MMSP_GPU_EINVAL;
    cudaStream_t ns = s ? (cudaStream_t)s : b->own;
    if (ns != b->stream) {
        cudaEvent_t ev;
        cudaError_t e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
        if (e != cudaSuccess) return bcuda(b, e, "set_stream");
        cudaEventRecord(ev, b->stream);
        cudaStreamWaitEvent(ns, ev, 0);
        cudaEventDestroy(ev);
        b->stream = ns;
    }
    return MMSP_GPU_OK;
}

static int bcheck_io(mmsp_gpu_batch* b, int index, const void* p, size_t bytes, int layout)
{
    if (!b || !p || index < 0 || index >= (int)b->m.size()) return MMSP_GPU_EINVAL;
    if (bytes != b->m[index].bytes) return bfail(b, MMSP_GPU_EINVAL, "transfer size differs from the grid's state size");
    if (layout != MMSP_GPU_CELL_MAJOR && layout != MMSP_GPU_FIELD_MAJOR) return bfail(b, MMSP_GPU_EINVAL, "layout");
    return MMSP_GPU_OK;
}

// Queue grid `index`'s upload / download on the batch stream (no synchronisation).
static cudaError_t queue_upload(mmsp_gpu_batch* b, int index, const void* host, size_t bytes, int layout)
{
    const Member& mm = b->m[index];
    char* dst = (char*)b->pool[b->cur] + mm.off * b->esize;
    if (layout == MMSP_GPU_CELL_MAJOR && mm.d.fields > 1) {
        char* tmp = (char*)b->pool[b->cur ^ 1] + mm.off * b->esize;   // idle pool as staging
        cudaError_t e = cudaMemcpyAsync(tmp, host, bytes, cudaMemcpyHostToDevice, b->stream);
        if (e == cudaSuccess) e = launch_transpose(b->dtype, tmp, dst, mm.g.cells, mm.d.fields, true, b->stream);
        return e;
    }
    return cudaMemcpyAsync(dst, host, bytes, cudaMemcpyHostToDevice, b->stream);
}

static cudaError_t queue_download(mmsp_gpu_batch* b, int index, void* host, size_t bytes, int layout)
{
    const Member& mm = b->m[index];
    const char* src = (const char*)b->pool[b->cur] + mm.off * b->esize;
    cudaError_t e = cudaSuccess;
    if (layout == MMSP_GPU_CELL_MAJOR && mm.d.fields > 1) {
        char* tmp = (char*)b->pool[b->cur ^ 1] + mm.off * b->esize;
        e = launch_transpose(b->dtype, src, tmp, mm.g.cells, mm.d.fields, false, b->stream);
        src = tmp;
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(host, src, bytes, cudaMemcpyDeviceToHost, b->stream);
    return e;
}

// After a download: a step kernel's timed-out wait leaves its word set.
static int check_wait_word(mmsp_gpu_batch* b)
{
    int f = 0;
    if (cudaMemcpy(&f, b->counters + 2, sizeof(int), cudaMemcpyDeviceToHost) == cudaSuccess && f)
        return bfail(b, MMSP_GPU_ETIMEDOUT, "a step kernel's bounded wait ran out");
    return MMSP_GPU_OK;
}

extern "C" int mmsp_gpu_batch_upload(mmsp_gpu_batch* b, int index, const void* host, size_t bytes, int layout)
{
    int rc = bcheck_io(b, index, host, bytes, layout);
    if (rc) return rc;
    cudaError_t e = queue_upload(b, index, host, bytes, layout);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    return e == cudaSuccess ? MMSP_GPU_OK : bcuda(b, e, "batch upload");
}

extern "C" int mmsp_gpu_batch_download(mmsp_gpu_batch* b, int index, void* host, size_t bytes, int layout)
{
    int rc = bcheck_io(b, index, host, bytes, layout);
    if (rc) return rc;
    cudaError_t e = queue_download(b, index, host, bytes, layout);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) return bcuda(b, e, "batch download");
    return check_wait_word(b);
}

extern "C" int mmsp_gpu_batch_upload_all(mmsp_gpu_batch* b, const void* const* host, int layout)
{
    if (!b || !host) return MMSP_GPU_EINVAL;
    for (int i = 0; i < (int)b->m.size(); i++) {
        int rc = bcheck_io(b, i, host[i], b->m[i].bytes, layout);
        if (rc) return rc;
    }
    cudaError_t e = cudaSuccess;
    for (int i = 0; i < (int)b->m.size() && e == cudaSuccess; i++) e = queue_upload(b, i, host[i], b->m[i].bytes, layout);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    return e == cudaSuccess ? MMSP_GPU_OK : bcuda(b, e, "batch upload");
}

extern "C" int mmsp_gpu_batch_download_all(mmsp_gpu_batch* b, void* const* host, int layout)
{
    if (!b || !host) return MMSP_GPU_EINVAL;
    for (int i = 0; i < (int)b->m.size(); i++) {
        int rc = bcheck_io(b, i, host[i], b->m[i].bytes, layout);
        if (rc) return rc;
    }
    cudaError_t e = cudaSuccess;
    for (int i = 0; i < (int)b->m.size() && e == cudaSuccess; i++) e = queue_download(b, i, host[i], b->m[i].bytes, layout);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) return bcuda(b, e, "batch download");
    return check_wait_word(b);
}

// ---------------------------------------------------------------------------
// Work list, autotuner, steps.

static void build_items(const mmsp_gpu_batch* b, int rows, std::vector<BatchItem>& items)
{
    items.clear();
    for (int i = 0; i < (int)b->insts.size(); i++) {
        const int n0 = b->insts[i].n0;
        for (int xs = 0; xs < n0; xs += rows) items.push_back(BatchItem{i, xs, std::min(xs + rows, n0)});
    }
    // largest first (loaded rows x cells per row), so the tail is short items
    std::stable_sort(items.begin(), items.end(), [&](const BatchItem& a, const BatchItem& c) {
        const long long ca = (long long)(a.xe - a.xs + 4) * b->insts[a.inst].n1;
        const long long cc = (long long)(c.xe - c.xs + 4) * b->insts[c.inst].n1;
        return ca > cc;
    });
}

static int set_items(mmsp_gpu_batch* b, int rows, int threads)
{
    std::vector<BatchItem> items;
    build_items(b, rows, items);
    if ((int)items.size() > b->items_cap) {
        if (b->d_items) cudaFree(b->d_items);
        b->d_items = nullptr;
        b->items_cap = 0;
        if (cudaMalloc((void**)&b->d_items, sizeof(BatchItem) * items.size()) != cudaSuccess) {
            cudaGetLastError();
            return bfail(b, MMSP_GPU_ENOMEM, "work list");
        }
        b->items_cap = (int)items.size();
    }
    cudaError_t e = cudaMemcpyAsync(b->d_items, items.data(), sizeof(BatchItem) * items.size(),
                                    cudaMemcpyHostToDevice, b->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) return bcuda(b, e, "work list upload");
    b->nitems = (int)items.size();
    const void* fn = batch_kernel(b->dtype, b->persistent_model, b->unit);
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, 0);
    if (e != cudaSuccess) return bcuda(b, e, "occupancy");
    b->blocks = std::max(1, per_sm) * sm_count();
    b->tune.rows = rows;
    b->tune.threads = threads;
    if (b->graph) {   // the work list changed: recapture
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    return MMSP_GPU_OK;
}

// The temporally blocked kernel applies when every grid of an FP32 batch
// joins the persistent kernel (grids with their own plans advance one step
// per launch).
static bool tb_possible(const mmsp_gpu_batch* b)
{
    return b->dtype == MMSP_GPU_F32 && b->npersistent > 0 && b->npersistent == (int)b->m.size();
}

// Tiles of every grid for region shape `shape` and depth `ks`, largest first.
static int set_tb(mmsp_gpu_batch* b, int shape, int ks)
{
    const int H = 2 * ks;
    const int TX = kTbShapes[shape].ri - 2 * H, TZ = kTbCols - 2 * H;
    for (const auto& bi : b->insts)   // 16-byte groups: rows of a multiple of 4 cells at 16-byte aligned offsets
        if (bi.n1 % 4 || bi.off % 4) return bfail(b, MMSP_GPU_EUNSUPPORTED, "tile kernel alignment");
    std::vector<TbItem> items;
    for (int i = 0; i < (int)b->insts.size(); i++) {
        const int n0 = b->insts[i].n0, n1 = b->insts[i].n1;
        for (int x0 = 0; x0 < n0; x0 += TX)
            for (int z0 = 0; z0 < n1; z0 += TZ)
                items.push_back(TbItem{i, x0, z0, std::min(TX, n0 - x0), std::min(TZ, n1 - z0)});
    }
    std::stable_sort(items.begin(), items.end(),
                     [](const TbItem& a, const TbItem& c) { return a.tx * a.tz > c.tx * c.tz; });
    if ((int)items.size() > b->tb_cap) {
        if (b->d_tb) cudaFree(b->d_tb);
        b->d_tb = nullptr;
        b->tb_cap = 0;
        if (cudaMalloc((void**)&b->d_tb, sizeof(TbItem) * items.size()) != cudaSuccess) {
            cudaGetLastError();
            return bfail(b, MMSP_GPU_ENOMEM, "tile list");
        }
        b->tb_cap = (int)items.size();
    }
    cudaError_t e = cudaMemcpyAsync(b->d_tb, items.data(), sizeof(TbItem) * items.size(), cudaMemcpyHostToDevice,
                                    b->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) return bcuda(b, e, "tile list upload");
    const void* fn = tb_kernel(shape, ks, b->persistent_model, b->unit);
    const size_t smem = tb_smem(shape);
    if ((e = ensure_smem(fn, smem)) != cudaSuccess) return bcuda(b, e, "tile kernel shared memory");
    int per_sm = 0;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kTbShapes[shape].nt, smem)) != cudaSuccess)
        return bcuda(b, e, "occupancy");
    b->tb_blocks = std::max(1, per_sm) * sm_count();
    b->tb_nitems = (int)items.size();
    b->tune.ks = ks;
    b->tune.shape = shape;
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    return MMSP_GPU_OK;
}

// tune.ks steps of every grid from pool `in` to pool `out` in one launch.
static cudaError_t step_tb(mmsp_gpu_batch* b, cudaStream_t s, int in, int out)
{
    const int parity = (int)(b->launches & 1);
    cudaError_t e = launch_tb(tb_kernel(b->tune.shape, b->tune.ks, b->persistent_model, b->unit), b->tb_blocks,
                              kTbShapes[b->tune.shape].nt, tb_smem(b->tune.shape), b->d_insts, b->d_tb, b->tb_nitems,
                              b->pool[in], b->pool[out], b->counters, parity, s);
    b->launches++;
    return e;
}

// One step from pool `in` to pool `out`.
static cudaError_t step_once(mmsp_gpu_batch* b, cudaStream_t s, int in, int out)
{
    cudaError_t e = cudaSuccess;
    if (b->npersistent > 0) {
        const int parity = (int)(b->launches & 1);
        e = launch_batch(batch_kernel(b->dtype, b->persistent_model, b->unit), b->blocks, b->tune.threads,
                         b->d_insts, b->d_items, b->nitems, b->pool[in], b->pool[out], b->counters, parity, s);
        b->launches++;
    }
    for (auto& mm : b->m) {
        if (mm.persistent || e != cudaSuccess) continue;
        const void* src = (const char*)b->pool[in] + mm.off * b->esize;
        void* dst = (char*)b->pool[out] + mm.off * b->esize;
        const bool ch = mm.d.model == MMSP_GPU_CH || mm.d.model == MMSP_GPU_CH_POLY;
        e = ch ? launch_ch(mm.plan, mm.d, mm.g, mm.c, src, dst, b->counters + 2, s)
               : launch_ac(mm.plan, mm.d, mm.g, mm.c, src, dst, b->counters + 2, s);
    }
    return e;
}

static std::string tune_key(const mmsp_gpu_batch* b)
{
    // FNV-1a over (dtype, model, unit, SMs, sorted row shapes)
    std::vector<long long> shapes;
    for (const auto& bi : b->insts) shapes.push_back(((long long)bi.n0 << 20) | bi.n1);
    std::sort(shapes.begin(), shapes.end());
    unsigned long long h = 1469598103934665603ull;
    auto mix = [&](long long v) {
        for (int i = 0; i < 8; i++) {
            h ^= (unsigned long long)((v >> (8 * i)) & 0xff);
            h *= 1099511628211ull;
        }
    };
    mix(b->dtype);
    mix(b->persistent_model);
    mix(b->unit);
    mix(sm_count());
    for (long long s : shapes) mix(s);
    char buf[64];
    snprintf(buf, sizeof buf, "ch2batch-%016llx", h);
    return buf;
}

static void load_cache_file()
{
    static bool loaded = false;
    if (loaded) return;
    loaded = true;
    const char* path = getenv("MMSP_GPU_TUNE_CACHE");
    if (!path) return;
    FILE* f = fopen(path, "r");
    if (!f) return;
    char key[128];
    Tuning t;
    // one entry per line: "key": [rows, threads, steps per launch, region shape],
    char line[512];
    while (fgets(line, sizeof line, f))
        if (sscanf(line, " \"%127[^\"]\" : [ %d , %d , %d , %d ]", key, &t.rows, &t.threads, &t.ks, &t.shape) == 5 &&
            t.rows > 0 && t.threads > 0 && t.ks >= 0 && t.shape >= 0 && t.shape < kTbShapeCount)
            g_tune[key] = t;
    fclose(f);
}

static void save_cache_file()
{
    const char* path = getenv("MMSP_GPU_TUNE_CACHE");
    if (!path) return;
    std::string tmp = std::string(path) + ".tmp";
    FILE* f = fopen(tmp.c_str(), "w");
    if (!f) return;
    fprintf(f, "{\n");
    size_t i = 0;
    for (const auto& kv : g_tune)
        fprintf(f, "  \"%s\": [%d, %d, %d, %d]%s\n", kv.first.c_str(), kv.second.rows, kv.second.threads,
                kv.second.ks, kv.second.shape, ++i < g_tune.size() ? "," : "");
    fprintf(f, "}\n");
    fclose(f);
    rename(tmp.c_str(), path);
}

// Apply a tuning: the per-step kernel's work list always (it takes the steps
// a temporally blocked launch cannot), and the tile list when ks > 0.
static int apply_tuning(mmsp_gpu_batch* b, const Tuning& t)
{
    int rc = set_items(b, t.rows, t.threads);
    if (rc) return rc;
    b->tune.ks = 0;
    if (t.ks > 0 && tb_possible(b)) return set_tb(b, t.shape, t.ks);
    return MMSP_GPU_OK;
}

extern "C" int mmsp_gpu_batch_tune(mmsp_gpu_batch* b, int force)
{
    if (!b) return MMSP_GPU_EINVAL;
    if (b->npersistent == 0) {
        b->tuned = true;
        return MMSP_GPU_OK;
    }
    const auto t0 = std::chrono::steady_clock::now();
    const std::string key = tune_key(b);
    // MMSP_GPU_BATCH_TILE="depth,shape" fixes the temporally blocked kernel's
    // steps per launch and region shape (index into its shapes), "0,0" the
    // per-step kernel, instead of tuning
    if (const char* fix = getenv("MMSP_GPU_BATCH_TILE")) {
        Tuning t;
        t.rows = 16;
        t.threads = 128;
        if (sscanf(fix, "%d,%d", &t.ks, &t.shape) == 2 && t.shape >= 0 && t.shape < kTbShapeCount &&
            (t.ks == 0 || std::find(std::begin(kTbDepths), std::end(kTbDepths), t.ks) != std::end(kTbDepths)) &&
            4 * t.ks < std::min(kTbShapes[t.shape].ri, kTbCols)) {
            int rc = apply_tuning(b, t);
            if (rc) return rc;
            b->tuned = true;
            b->tuned_from_cache = false;
            b->tune_ms = 0.0;
            return MMSP_GPU_OK;
        }
        return bfail(b, MMSP_GPU_EINVAL, "MMSP_GPU_BATCH_TILE: expected \"depth,shape\" with depth 0, 2, 4 or 8");
    }
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        load_cache_file();
        auto it = g_tune.find(key);
        if (!force && it != g_tune.end()) {
            int rc = apply_tuning(b, it->second);
            if (rc) return rc;
            b->tuned = b->tuned_from_cache = true;
            b->tune_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
            return MMSP_GPU_OK;
        }
    }
    // Candidates: the per-step kernel's rows per work item x threads per
    // block, then (FP32 batches) the temporally blocked kernel's region shape
    // x steps per launch.  Each is timed on the live state (pool cur -> idle
    // pool, so the state is not changed) and scored per step.
    static const int kRows[] = {4, 8, 16, 32, 64};
    static const int kThreads[] = {64, 128};
    cudaEvent_t e0, e1;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        cudaGetLastError();
        return bfail(b, MMSP_GPU_ECUDA, "tune events");
    }
    const long long p0 = b->launches & 1;
    // time two launches of `one` after a warm-up one; keeps the launch-count
    // parity, which must keep matching `cur`
    auto time2 = [&](auto one, float* ms) -> cudaError_t {
        cudaError_t e = one();
        if (e == cudaSuccess) e = cudaEventRecord(e0, b->stream);
        for (int k = 0; k < 2 && e == cudaSuccess; k++) e = one();
        if (e == cudaSuccess) e = cudaEventRecord(e1, b->stream);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        if (e == cudaSuccess) e = cudaEventElapsedTime(ms, e0, e1);
        if (e == cudaSuccess && (b->launches & 1) != p0) e = one();
        return e;
    };
    float best = 1e30f;
    Tuning win;
    win.rows = 16;
    win.threads = 128;
    int rc = MMSP_GPU_OK;
    cudaError_t e = cudaSuccess;
    for (int rows : kRows)
        for (int threads : kThreads) {
            if ((rc = set_items(b, rows, threads))) goto done;
            float ms = 0;
            e = time2([&] { return step_once(b, b->stream, b->cur, b->cur ^ 1); }, &ms);
            if (e != cudaSuccess) goto done;
            if (ms / 2 < best) {
                best = ms / 2;
                win.rows = rows;
                win.threads = threads;
                win.ks = 0;
            }
        }
    if (tb_possible(b)) {
        for (int shape = 0; shape < kTbShapeCount; shape++)
            for (int ks : kTbDepths) {
                if (2 * 2 * ks >= std::min(kTbShapes[shape].ri, kTbCols)) continue;   // no interior
                if ((rc = set_tb(b, shape, ks))) goto done;
                float ms = 0;
                e = time2([&] { return step_tb(b, b->stream, b->cur, b->cur ^ 1); }, &ms);
                if (e != cudaSuccess) goto done;
                if (ms / (2 * ks) < best) {
                    best = ms / (2 * ks);
                    win.ks = ks;
                    win.shape = shape;
                }
            }
    }
done:
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) return bcuda(b, e, "tune");
    if (rc) return rc;
    if ((rc = apply_tuning(b, win))) return rc;
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        g_tune[key] = win;
        save_cache_file();
    }
    b->tuned = true;
    b->tuned_from_cache = false;
    b->tune_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return MMSP_GPU_OK;
}

// A CUDA graph of kBatchGraphSteps steps from pool 0 at counter parity 0:
// kBatchGraphSteps / ks temporally blocked launches, or one launch per step.
// Either count is even, so a replay leaves the state in pool 0.
static int build_batch_graph(mmsp_gpu_batch* b)
{
    if (b->graph) return MMSP_GPU_OK;
    cudaStream_t cs;
    cudaError_t e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
    if (e != cudaSuccess) return bcuda(b, e, "graph stream");
    e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) {
        cudaStreamDestroy(cs);
        return bcuda(b, e, "begin capture");
    }
    const long long saved = b->launches;
    b->launches = 0;   // the graph starts at counter parity 0
    cudaError_t le = cudaSuccess;
    const int per = b->tune.ks > 0 ? b->tune.ks : 1;
    for (int i = 0; i < kBatchGraphSteps / per && le == cudaSuccess; i++)
        le = b->tune.ks > 0 ? step_tb(b, cs, i & 1, (i & 1) ^ 1) : step_once(b, cs, i & 1, (i & 1) ^ 1);
    b->launches = saved;
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(cs, &g);
    cudaStreamDestroy(cs);
    if (le != cudaSuccess || e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return bcuda(b, le != cudaSuccess ? le : e, "batch capture");
    }
    e = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        b->graph = nullptr;
        return bcuda(b, e, "batch instantiate");
    }
    return MMSP_GPU_OK;
}

extern "C" int mmsp_gpu_batch_step(mmsp_gpu_batch* b, int steps)
{
    if (!b || steps < 0) return MMSP_GPU_EINVAL;
    if (steps == 0) return MMSP_GPU_OK;
    if (!b->tuned) {
        int rc = mmsp_gpu_batch_tune(b, 0);
        if (rc) return rc;
    }
    cudaError_t e;
    int left = steps;
    const int ks = b->tune.ks;
    // the counter parity moves with every launch and the pool with every
    // launch too (a blocked launch is ks steps but one pool swap)
    if (steps >= 2 * kBatchGraphSteps) {
        int rc = build_batch_graph(b);
        if (rc) return rc;
        // the graph starts from pool 0 at counter parity 0; cur and the
        // launch parity move together, so one plain step aligns both
        if (b->cur == 1) {
            if ((e = step_once(b, b->stream, 1, 0)) != cudaSuccess) return bcuda(b, e, "batch step");
            b->cur = 0;
            left--;
        }
        while (left >= kBatchGraphSteps) {
            if ((e = cudaGraphLaunch(b->graph, b->stream)) != cudaSuccess) return bcuda(b, e, "batch graph");
            if (b->npersistent > 0) b->launches += ks > 0 ? kBatchGraphSteps / ks : kBatchGraphSteps;
            left -= kBatchGraphSteps;
        }
    }
    while (ks > 0 && left >= ks) {
        if ((e = step_tb(b, b->stream, b->cur, b->cur ^ 1)) != cudaSuccess) return bcuda(b, e, "batch step");
        b->cur ^= 1;
        left -= ks;
    }
    while (left > 0) {
        if ((e = step_once(b, b->stream, b->cur, b->cur ^ 1)) != cudaSuccess) return bcuda(b, e, "batch step");
        b->cur ^= 1;
        left--;
    }
    return MMSP_GPU_OK;
}

extern "C" int mmsp_gpu_batch_synchronize(mmsp_gpu_batch* b)
{
    if (!b) return MMSP_GPU_EINVAL;
    cudaError_t e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) return bcuda(b, e, "batch synchronize");
    int f = 0;
    if (cudaMemcpy(&f, b->counters + 2, sizeof(int), cudaMemcpyDeviceToHost) == cudaSuccess && f)
        return bfail(b, MMSP_GPU_ETIMEDOUT, "a step kernel's bounded wait ran out");
    return MMSP_GPU_OK;
}

extern "C" int mmsp_gpu_batch_reduce(mmsp_gpu_batch* b, int index, mmsp_gpu_stats* st)
{
    if (!b || !st || index < 0 || index >= (int)b->m.size()) return MMSP_GPU_EINVAL;
    const Member& mm = b->m[index];
    const void* s = (const char*)b->pool[b->cur] + mm.off * b->esize;
    cudaError_t e = launch_reduce(mm.d, mm.g, mm.c, s, b->partials, b->stream);
    double res[2] = {0, 0};
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(res, b->partials + 4 * kReduceBlocks, sizeof(res), cudaMemcpyDeviceToHost, b->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) return bcuda(b, e, "batch reduce");
    st->mass = res[0];
    st->energy = res[1];
    st->gpu_ms = 0.0;
    st->steps = 0;
    return MMSP_GPU_OK;
}

extern "C" int mmsp_gpu_batch_get_info(const mmsp_gpu_batch* b, mmsp_gpu_batch_info* info)
{
    if (!b || !info) return MMSP_GPU_EINVAL;
    memset(info, 0, sizeof(*info));
    info->instances = (int)b->m.size();
    info->persistent = b->npersistent;
    info->fallback = (int)b->m.size() - b->npersistent;
    info->rows_per_item = b->tune.rows;
    info->threads_per_block = b->tune.threads;
    info->blocks = b->blocks;
    info->items = b->nitems;
    info->tuned_from_cache = b->tuned_from_cache ? 1 : 0;
    info->tune_ms = b->tune_ms;
    info->temporal_depth = b->tune.ks > 0 ? b->tune.ks : 1;
    info->tile_rows = b->tune.ks > 0 ? kTbShapes[b->tune.shape].ri : 0;
    info->tile_cols = b->tune.ks > 0 ? kTbCols : 0;
    info->tiles = b->tune.ks > 0 ? b->tb_nitems : 0;
    info->device_bytes = 2 * (size_t)b->pool_elems * b->esize + kPartialsBytes + 256 +
                         sizeof(BatchInst) * b->insts.size() + sizeof(BatchItem) * b->items_cap +
                         sizeof(TbItem) * b->tb_cap;
    return MMSP_GPU_OK;
}

extern "C" const char* mmsp_gpu_batch_last_error(const mmsp_gpu_batch* b) { return b ? b->err.c_str() : "NULL batch"; }
