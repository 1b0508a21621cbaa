// mmsp_gpu.cu -- the C ABI of include/MMSP.gpu.h: handles, validation,
// host/device transfers, CUDA-graph replay of step chunks, reductions.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <new>
#include <string>
#include <vector>

#include "MMSP.gpu.h"
#include "pf_batch.h"
#include "pf_handle.h"
#include "pf_internal.h"

using pf::Coeffs;
using pf::Geom;
using pf::StepPlan;

static const int kGraphSteps = 64;
static const int kGraphMin = 2 * kGraphSteps;   // replay only for runs this long

static int fail(mmsp_gpu_handle* h, int code, const char* fmt, const char* a = "", const char* b = "")
{
    if (h) snprintf(h->err, sizeof(h->err), fmt, a, b);
    return code;
}

static int cuda_fail(mmsp_gpu_handle* h, cudaError_t e, const char* where)
{
    if (h) snprintf(h->err, sizeof(h->err), "%s: %s", where, cudaGetErrorString(e));
    cudaGetLastError();   // clear a non-sticky error
    return MMSP_GPU_ECUDA;
}

static int check_flags(mmsp_gpu_handle* h);

extern "C" int mmsp_gpu_version(void) { return MMSP_GPU_ABI_VERSION; }

extern "C" const char* mmsp_gpu_strerror(int code)
{
    switch (code) {
    case MMSP_GPU_OK: return "ok";
    case MMSP_GPU_EINVAL: return "invalid argument";
    case MMSP_GPU_ENOMEM: return "out of device memory";
    case MMSP_GPU_ECUDA: return "CUDA error";
    case MMSP_GPU_EUNSUPPORTED: return "unsupported configuration";
    case MMSP_GPU_ETIMEDOUT: return "timed out";
    case MMSP_GPU_ENODEV: return "no suitable CUDA device";
    case MMSP_GPU_ENOTFOUND: return "unknown request";
    case MMSP_GPU_ECANCELED: return "cancelled";
    case MMSP_GPU_ESTOPPED: return "server stopped";
    case MMSP_GPU_EIO: return "grid file could not be written";
    case MMSP_GPU_ENOCONV: return "implicit solver did not converge";
    case MMSP_GPU_EOVERFLOW: return "sparse cell list outgrew its slots";
    default: return "unknown status";
    }
}

extern "C" int mmsp_gpu_desc_init(mmsp_gpu_desc* d, int dim, const int* n, int fields, int dtype, int model)
{
    if (!d || !n) return MMSP_GPU_EINVAL;
    memset(d, 0, sizeof(*d));
    d->dim = dim;
    for (int a = 0; a < 3; a++) {
        d->n[a] = (a < dim) ? n[a] : 1;
        d->dx[a] = 1.0;
        d->bc[a][0] = d->bc[a][1] = MMSP_GPU_BC_PERIODIC;
    }
    d->fields = fields;
    d->dtype = dtype;
    d->model = model;
    d->mobility = 1.0;
    d->kappa = 1.0;
    d->r = 1.0;
    d->u = 1.0;
    d->gamma = 1.0;
    switch (model) {
    case MMSP_GPU_CH: d->dt = 0.005; break;                       // 2D configuration of the CH study
    case MMSP_GPU_CH_POLY: d->dt = 0.01; break;                   // cahn-hilliard.cpp:59-63
    case MMSP_GPU_AC: d->dt = 0.05; d->kappa = 2.0; d->gamma = 1.5; break;
    case MMSP_GPU_GG: d->dt = 0.01; d->kappa = 2.0; break;        // graingrowth.cpp:84
    case MMSP_GPU_AC_POLY: d->dt = 0.01; break;                   // allen-cahn.cpp:57-61
    case MMSP_GPU_ZENER: d->dt = 0.01; d->kappa = 2.0; break;     // zener.cpp:115
    case MMSP_GPU_CH_CONVEX:   // convex_splitting/cahn-hilliard.cpp:38-67 (parametric energy)
        d->mobility = 2.0 / (0.95 - 0.05);    // D = 2/(Cb-Ca)
        d->kappa = 2.0;                       // K
        d->dt = pow(1.0, 2.0) / (d->mobility * d->kappa);
        d->aux[0] = 0.45;    // C0
        d->aux[1] = 0.05;    // Ca
        d->aux[2] = 0.95;    // Cb
        d->aux[3] = 2.0;     // A
        d->aux[4] = 1.2;     // omega
        d->aux[5] = 1.0e-14; // tolerance
        break;
    case MMSP_GPU_SPARSE_GG:                                      // sparsePF/graingrowth.cpp:77-78
        d->dt = 0.01;
        d->aux[0] = 1.0e-8;   // epsilon
        break;
    case MMSP_GPU_OSTWALD:                                        // ostwald.cpp:66-80
        d->dt = 0.001;
        d->kappa = 2.0;
        d->aux[0] = 1.0;    // D
        d->aux[1] = 0.05;   // Calpha
        d->aux[2] = 0.95;   // Cbeta
        d->aux[3] = 2.0;    // A
        d->aux[4] = 1.0;    // delta
        d->aux[5] = 3.0;    // epsilon
        break;
    default: return MMSP_GPU_EINVAL;
    }
    return mmsp_gpu_validate(d);
}

static int validate(const mmsp_gpu_desc* d, char* why, size_t nwhy)
{
#define BAD(code, ...) do { if (why) snprintf(why, nwhy, __VA_ARGS__); return code; } while (0)
    if (!d) BAD(MMSP_GPU_EINVAL, "NULL descriptor");
    if (d->dim < 1 || d->dim > 3) BAD(MMSP_GPU_EINVAL, "dim %d outside 1..3", d->dim);
    if (d->dtype != MMSP_GPU_F64 && d->dtype != MMSP_GPU_F32) BAD(MMSP_GPU_EINVAL, "dtype %d", d->dtype);
    if (d->model < MMSP_GPU_CH || d->model > MMSP_GPU_SPARSE_GG) BAD(MMSP_GPU_EINVAL, "model %d", d->model);
    long long cells = 1;
    for (int a = 0; a < d->dim; a++) {
        if (d->n[a] < 1) BAD(MMSP_GPU_EINVAL, "extent n[%d]=%d", a, d->n[a]);
        if (!(d->dx[a] > 0.0) || !isfinite(d->dx[a])) BAD(MMSP_GPU_EINVAL, "dx[%d] not positive and finite", a);
        for (int s = 0; s < 2; s++) {
            int b = d->bc[a][s];
            if (b < MMSP_GPU_BC_MIRROR || b > MMSP_GPU_BC_DIRICHLET) BAD(MMSP_GPU_EINVAL, "bc[%d][%d]=%d", a, s, b);
            if (b != MMSP_GPU_BC_PERIODIC)
                BAD(MMSP_GPU_EUNSUPPORTED, "bc[%d][%d]=%d: the device step takes periodic boundaries only", a, s, b);
        }
        cells *= d->n[a];
        if (cells > (1LL << 40)) BAD(MMSP_GPU_EINVAL, "grid too large");
    }
    bool scalar_model = d->model == MMSP_GPU_CH || d->model == MMSP_GPU_CH_POLY || d->model == MMSP_GPU_AC_POLY;
    if (scalar_model && d->fields != 1) BAD(MMSP_GPU_EINVAL, "model %d takes fields=1, got %d", d->model, d->fields);
    if (d->fields < 1) BAD(MMSP_GPU_EINVAL, "fields=%d", d->fields);
    if (d->model == MMSP_GPU_CH_CONVEX) {
        if (d->fields != 2) BAD(MMSP_GPU_EINVAL, "convex splitting takes fields=2 (c, mu), got %d", d->fields);
        if (d->dtype != MMSP_GPU_F64)
            BAD(MMSP_GPU_EUNSUPPORTED, "convex splitting runs in FP64 (its residual tolerance is below FP32)");
        for (int a = 0; a < d->dim; a++)
            if (d->n[a] % 2)
                BAD(MMSP_GPU_EUNSUPPORTED, "convex splitting needs even extents for an order-free red-black sweep, "
                                           "n[%d]=%d", a, d->n[a]);
        if (!(d->aux[4] > 0.0 && d->aux[4] < 2.0) || !(d->aux[5] > 0.0) || !(d->aux[1] != d->aux[0]))
            BAD(MMSP_GPU_EINVAL, "convex splitting: omega in (0,2), tolerance > 0 and Ca != C0");
    }
    if (d->model == MMSP_GPU_SPARSE_GG) {
        if (d->dtype != MMSP_GPU_F64) BAD(MMSP_GPU_EUNSUPPORTED, "sparse grain growth runs in FP64");
        if (!isfinite(d->aux[0])) BAD(MMSP_GPU_EINVAL, "sparse grain growth: epsilon (aux[0]) not finite");
        if (cells >= (1LL << 31)) BAD(MMSP_GPU_EUNSUPPORTED, "sparse grid of %lld cells above 2^31", cells);
    }
    if (d->model == MMSP_GPU_OSTWALD && d->fields < 2)
        BAD(MMSP_GPU_EINVAL, "Ostwald ripening takes a composition and at least one order parameter, fields=%d",
            d->fields);
    if ((d->model == MMSP_GPU_CH_POLY || d->model == MMSP_GPU_AC_POLY) &&
        (!(d->aux[0] >= 0.0) || !isfinite(d->aux[0]) || !(d->aux[1] >= 0.0) || !(d->aux[1] <= 9007199254740992.0) ||
         d->aux[1] != floor(d->aux[1])))
        BAD(MMSP_GPU_EINVAL, "noise: aux[0] (standard deviation) must be finite and >= 0, aux[1] (seed) an integer "
                             "in [0, 2^53]");
    if (d->model == MMSP_GPU_OSTWALD && (!(d->aux[2] != d->aux[1]) || !(d->aux[4] != 0.0)))
        BAD(MMSP_GPU_EINVAL, "Ostwald ripening needs Calpha != Cbeta and delta != 0");
    if (d->fields > 32) BAD(MMSP_GPU_EUNSUPPORTED, "fields=%d above 32", d->fields);
    if (d->flags & ~MMSP_GPU_FLAG_CONTRACT) BAD(MMSP_GPU_EINVAL, "unknown flags 0x%x", (unsigned)d->flags);
    long long yz = 1;
    for (int a = (d->dim >= 2 ? d->dim - 2 : 0); a < d->dim; a++) yz *= d->n[a];
    if (yz >= (1LL << 31)) BAD(MMSP_GPU_EUNSUPPORTED, "plane of %lld cells above 2^31", yz);
    if ((long long)d->n[0] >= (1LL << 31)) BAD(MMSP_GPU_EINVAL, "extent too large");
    if (!isfinite(d->dt) || !isfinite(d->kappa) || !isfinite(d->mobility) || !isfinite(d->gamma) ||
        !isfinite(d->r) || !isfinite(d->u))
        BAD(MMSP_GPU_EINVAL, "non-finite model parameter");
    return MMSP_GPU_OK;
#undef BAD
}

extern "C" int mmsp_gpu_validate(const mmsp_gpu_desc* d) { return validate(d, nullptr, 0); }

static size_t esize_of(const mmsp_gpu_desc* d) { return d->dtype == MMSP_GPU_F64 ? sizeof(double) : sizeof(float); }

static size_t state_bytes(const mmsp_gpu_desc* d)
{
    if (d->model == MMSP_GPU_SPARSE_GG) {
        long long cells = 1;
        for (int a = 0; a < d->dim; a++) cells *= d->n[a];
        return pf::sparse_layout(cells, d->fields).bytes;
    }
    size_t n = (size_t)d->fields;
    for (int a = 0; a < d->dim; a++) n *= (size_t)d->n[a];
    return n * esize_of(d);
}

// Device scratch of a model beyond the two state buffers: the Ostwald
// model's chemical-potential grid (one value per cell); for convex
// splitting, a staging copy of the state for cell-major downloads.
// FP64 Cahn-Hilliard in 2D/3D keeps the reference's temp grid (mu) between
// its two passes (pf_ch64.cu).
static bool two_pass_f64(const mmsp_gpu_desc* d)
{
    // also the FP32 stochastic 3D Cahn-Hilliard form, whose deviates are drawn once per cell in the mu pass
    // (in 2D the fused tile kernel, which redraws them on its halo, is faster)
    const bool noisy32 = d->dtype == MMSP_GPU_F32 && d->model == MMSP_GPU_CH_POLY && d->dim == 3 && pf::noisy(*d);
    return (d->dtype == MMSP_GPU_F64 || noisy32) && (d->dim == 2 || d->dim == 3) &&
           (d->model == MMSP_GPU_CH || d->model == MMSP_GPU_CH_POLY);
}

static size_t align256(size_t b) { return (b + 255) / 256 * 256; }

// 2D FP32 Cahn-Hilliard grids step in blocks of pf::kTbAnyDepth steps, each
// one launch of the temporally blocked kernel of the batched form
// (pf_batch.cu) over the grid's 64 x 128 regions: a quarter of the launches
// and of the HBM traffic of one kernel per step.  The leftover steps of a
// call (fewer than kTbAnyDepth) take the plan's per-step kernel, so a run
// split into calls of multiples of kTbAnyDepth steps equals one call.
static bool tb_handle(const mmsp_gpu_desc* d)
{
    return d->dtype == MMSP_GPU_F32 && d->dim == 2 && (d->model == MMSP_GPU_CH || d->model == MMSP_GPU_CH_POLY) &&
           !pf::noisy(*d);
}

static int tb_tile_rows() { return pf::kTbShapes[0].ri - 4 * pf::kTbAnyDepth; }
static int tb_tile_cols() { return pf::kTbCols - 4 * pf::kTbAnyDepth; }

static size_t tb_meta_bytes(const mmsp_gpu_desc* d)
{
    const long long tiles = (long long)((d->n[0] + tb_tile_rows() - 1) / tb_tile_rows()) *
                            ((d->n[1] + tb_tile_cols() - 1) / tb_tile_cols());
    return align256(sizeof(pf::BatchInst)) + align256(sizeof(pf::TbItem) * (size_t)tiles) + 256;
}

static size_t work_bytes(const mmsp_gpu_desc* d)
{
    if (tb_handle(d)) return tb_meta_bytes(d);   // the blocked kernel's instance, tiles and counters
    if (d->model == MMSP_GPU_CH_CONVEX) return state_bytes(d);   // download staging (the guess stays put)
    if (d->model != MMSP_GPU_OSTWALD && !two_pass_f64(d)) return 0;
    return state_bytes(d) / (size_t)d->fields;
}

extern "C" int mmsp_gpu_footprint(const mmsp_gpu_desc* d, size_t* bytes)
{
    int rc = mmsp_gpu_validate(d);
    if (rc) return rc;
    if (!bytes) return MMSP_GPU_EINVAL;
    *bytes = 2 * state_bytes(d) + pf::kPartialsBytes + work_bytes(d);
    return MMSP_GPU_OK;
}

static void release(mmsp_gpu_handle* h)
{
    if (h->out) pf::output_release(h);   // waits for snapshots still being written
    if (h->graph) cudaGraphExecDestroy(h->graph);
    for (int p = 0; p < 2; p++)
        if (h->cs_graph[p]) cudaGraphExecDestroy(h->cs_graph[p]);
    if (h->ev0) cudaEventDestroy(h->ev0);
    if (h->ev1) cudaEventDestroy(h->ev1);
    if (h->external) return;   // the caller's block and stream
    if (h->buf[0]) cudaFree(h->buf[0]);
    if (h->buf[1]) cudaFree(h->buf[1]);
    if (h->partials) cudaFree(h->partials);
    if (h->work) cudaFree(h->work);
    if (h->flags) cudaFree(h->flags);
    if (h->own) cudaStreamDestroy(h->own);
}

size_t pf::handle_block_bytes(const mmsp_gpu_desc& d)
{
    return 2 * align256(state_bytes(&d)) + align256(pf::kPartialsBytes) + 256 + align256(work_bytes(&d));
}

static int make_plan(mmsp_gpu_handle* h);
static int setup_tb(mmsp_gpu_handle* h);

int pf::create_in(mmsp_gpu_handle** out, const mmsp_gpu_desc* desc, void* block, cudaStream_t stream)
{
    if (!out || !block || ((uintptr_t)block & 255)) return MMSP_GPU_EINVAL;
    *out = nullptr;
    int rc = validate(desc, nullptr, 0);
    if (rc) return rc;
    mmsp_gpu_handle* h = new (std::nothrow) mmsp_gpu_handle();
    if (!h) return MMSP_GPU_ENOMEM;
    memset(h, 0, sizeof(*h));
    h->external = true;
    h->d = *desc;
    for (int a = desc->dim; a < 3; a++) h->d.n[a] = 1;
    h->g = pf::make_geom(h->d);
    h->c = pf::make_coeffs(h->d);
    cudaGetDevice(&h->device);
    h->esize = esize_of(&h->d);
    h->bytes = state_bytes(&h->d);
    h->elems = h->bytes / h->esize;
    h->own = h->stream = stream;
    char* p = static_cast<char*>(block);
    h->buf[0] = p;
    p += align256(h->bytes);
    h->buf[1] = p;
    p += align256(h->bytes);
    h->partials = reinterpret_cast<double*>(p);
    p += align256(pf::kPartialsBytes);
    h->flags = reinterpret_cast<int*>(p);
    p += 256;
    if (work_bytes(&h->d)) h->work = p;
    cudaError_t e = cudaEventCreate(&h->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&h->ev1);
    if (e == cudaSuccess) e = cudaMemsetAsync(h->flags, 0, 256, stream);
    if (e != cudaSuccess) {
        cudaGetLastError();
        release(h);
        delete h;
        return MMSP_GPU_ECUDA;
    }
    rc = make_plan(h);
    if (!rc) rc = setup_tb(h);
    if (rc) {
        release(h);
        delete h;
        return rc;
    }
    *out = h;
    return MMSP_GPU_OK;
}

static int make_plan(mmsp_gpu_handle* h)
{
    if (h->d.model == MMSP_GPU_CH_CONVEX) {   // kernels are launched directly (pf_convex.cu)
        h->plan.kind = 5;
        h->plan.ok = true;
        return MMSP_GPU_OK;
    }
    if (h->d.model == MMSP_GPU_SPARSE_GG) {   // pf_sparse.cu
        h->plan.kind = 7;
        h->plan.ok = true;
        return MMSP_GPU_OK;
    }
    bool ch = h->d.model == MMSP_GPU_CH || h->d.model == MMSP_GPU_CH_POLY;
    cudaError_t e = h->d.model == MMSP_GPU_OSTWALD ? pf::plan_ostwald(h->d, h->g, &h->plan)
                    : two_pass_f64(&h->d) && pf::ch64_eligible(h->d, h->g) ? pf::plan_ch64(h->d, h->g, &h->plan)
                    : ch ? pf::plan_ch(h->d, h->g, &h->plan) : pf::plan_ac(h->d, h->g, &h->plan);
    if (e != cudaSuccess) {
        if (!h->plan.ok && !ch) return fail(h, MMSP_GPU_EUNSUPPORTED, "%s", "too many fields for shared memory");
        return cuda_fail(h, e, "plan");
    }
    return MMSP_GPU_OK;
}

// The blocked kernel's instance and tile list, in the handle's work buffer.
static int setup_tb(mmsp_gpu_handle* h)
{
    if (!tb_handle(&h->d)) return MMSP_GPU_OK;
    const int n0 = h->d.n[0], n1 = h->d.n[1], TX = tb_tile_rows(), TZ = tb_tile_cols();
    std::vector<pf::TbItem> items;
    for (int x0 = 0; x0 < n0; x0 += TX)
        for (int z0 = 0; z0 < n1; z0 += TZ)
            items.push_back(pf::TbItem{0, x0, z0, std::min(TX, n0 - x0), std::min(TZ, n1 - z0)});
    pf::BatchInst bi;
    memset(&bi, 0, sizeof(bi));
    bi.off = 0;
    bi.n0 = n0;
    bi.n1 = n1;
    bi.w0 = h->c.w[0];
    bi.w1 = h->c.w[1];
    bi.kappa = h->c.kappa;
    bi.dtm = h->c.dtm;
    bi.neg_r = h->c.neg_r;
    bi.u = h->c.u;
    char* p = static_cast<char*>(h->work);
    h->tb_inst = reinterpret_cast<pf::BatchInst*>(p);
    p += align256(sizeof(pf::BatchInst));
    h->tb_list = reinterpret_cast<pf::TbItem*>(p);
    p += align256(sizeof(pf::TbItem) * items.size());
    h->tb_counters = reinterpret_cast<int*>(p);
    h->tb_items = (int)items.size();
    const bool aligned = n1 % 4 == 0;   // 16-byte row groups
    h->tb_fn = aligned ? pf::tb_kernel(0, pf::kTbAnyDepth, h->d.model, h->c.unit_w)
                       : pf::tb_kernel_any(h->d.model, h->c.unit_w);
    h->tb_smem = pf::tb_smem(0);
    // Queued on the handle's stream, ahead of its first launch, with no
    // synchronisation: a server request's stream may carry another request's
    // queued steps.  A copy from pageable memory has staged its source when
    // the call returns, so the host arrays may go out of scope.
    cudaError_t e = cudaMemcpyAsync(h->tb_inst, &bi, sizeof(bi), cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(h->tb_list, items.data(), sizeof(pf::TbItem) * items.size(), cudaMemcpyHostToDevice,
                            h->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(h->tb_counters, 0, 256, h->stream);
    if (e == cudaSuccess) e = pf::ensure_smem(h->tb_fn, h->tb_smem);
    int per_sm = 0;
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, h->tb_fn, pf::kTbShapes[0].nt, h->tb_smem);
    if (e != cudaSuccess) return cuda_fail(h, e, "blocked kernel setup");
    h->tb_blocks = std::max(1, std::min(per_sm * pf::sm_count(), h->tb_items));
    h->tb_launches = 0;
    h->tb = true;
    return MMSP_GPU_OK;
}

// kTbAnyDepth steps from buf[cur] in one launch of the blocked kernel.
static cudaError_t tb_launch(mmsp_gpu_handle* h, cudaStream_t s)
{
    const cudaError_t e =
        pf::launch_tb(h->tb_fn, h->tb_blocks, pf::kTbShapes[0].nt, h->tb_smem, h->tb_inst, h->tb_list, h->tb_items,
                      h->buf[h->cur], h->buf[h->cur ^ 1], h->tb_counters, (int)(h->tb_launches & 1), s);
    h->cur ^= 1;
    h->tb_launches++;
    return e;
}

extern "C" int mmsp_gpu_create(mmsp_gpu_handle** out, const mmsp_gpu_desc* desc)
{
    if (!out) return MMSP_GPU_EINVAL;
    *out = nullptr;
    int rc = validate(desc, nullptr, 0);
    if (rc) return rc;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
        cudaGetLastError();
        return MMSP_GPU_ENODEV;
    }
    mmsp_gpu_handle* h = new (std::nothrow) mmsp_gpu_handle();
    if (!h) return MMSP_GPU_ENOMEM;
    memset(h, 0, sizeof(*h));
    h->d = *desc;
    for (int a = desc->dim; a < 3; a++) h->d.n[a] = 1;
    h->g = pf::make_geom(h->d);
    h->c = pf::make_coeffs(h->d);
    cudaGetDevice(&h->device);
    h->esize = esize_of(&h->d);
    h->bytes = state_bytes(&h->d);
    h->elems = h->bytes / h->esize;
    cudaError_t e;
    if ((e = cudaStreamCreateWithFlags(&h->own, cudaStreamNonBlocking)) != cudaSuccess) goto cuda_err;
    h->stream = h->own;
    if ((e = cudaEventCreate(&h->ev0)) != cudaSuccess) goto cuda_err;
    if ((e = cudaEventCreate(&h->ev1)) != cudaSuccess) goto cuda_err;
    if (cudaMalloc(&h->buf[0], h->bytes) != cudaSuccess || cudaMalloc(&h->buf[1], h->bytes) != cudaSuccess ||
        cudaMalloc((void**)&h->partials, pf::kPartialsBytes) != cudaSuccess ||
        cudaMalloc((void**)&h->flags, 256) != cudaSuccess || cudaMemset(h->flags, 0, 256) != cudaSuccess ||
        (work_bytes(&h->d) && cudaMalloc(&h->work, work_bytes(&h->d)) != cudaSuccess)) {
        cudaGetLastError();
        release(h);
        delete h;
        return MMSP_GPU_ENOMEM;
    }
    rc = make_plan(h);
    if (!rc) rc = setup_tb(h);
    if (rc) {
        release(h);
        delete h;
        return rc;
    }
    *out = h;
    return MMSP_GPU_OK;
cuda_err:
    release(h);
    delete h;
    cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? MMSP_GPU_ENOMEM : MMSP_GPU_ECUDA;
}

extern "C" int mmsp_gpu_destroy(mmsp_gpu_handle* h)
{
    if (!h) return MMSP_GPU_OK;
    cudaStreamSynchronize(h->stream);
    release(h);
    delete h;
    return MMSP_GPU_OK;
}

extern "C" int mmsp_gpu_set_stream(mmsp_gpu_handle* h, void* s)
{
    if (!h) return MMSP_GPU_EINVAL;
    cudaStream_t ns = s ? (cudaStream_t)s : h->own;
    if (ns != h->stream) {
        // order the new stream after everything queued on the old one
        cudaEvent_t ev;
        cudaError_t e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
        if (e != cudaSuccess) return cuda_fail(h, e, "set_stream");
        cudaEventRecord(ev, h->stream);
        cudaStreamWaitEvent(ns, ev, 0);
        cudaEventDestroy(ev);
        h->stream = ns;
    }
    return MMSP_GPU_OK;
}

static int check_io(mmsp_gpu_handle* h, const void* p, size_t bytes, int layout)
{
    if (!h || !p) return MMSP_GPU_EINVAL;
    if (h->d.model == MMSP_GPU_SPARSE_GG)
        return fail(h, MMSP_GPU_EUNSUPPORTED, "%s", "sparse grids cross with mmsp_gpu_sparse_upload/_download");
    if (bytes != h->bytes) {
        char a[64], b[64];
        snprintf(a, sizeof a, "%zu", bytes);
        snprintf(b, sizeof b, "%zu", h->bytes);
        return fail(h, MMSP_GPU_EINVAL, "transfer of %s bytes, state is %s bytes", a, b);
    }
    if (layout != MMSP_GPU_CELL_MAJOR && layout != MMSP_GPU_FIELD_MAJOR) return fail(h, MMSP_GPU_EINVAL, "%s", "layout");
    return MMSP_GPU_OK;
}

static int upload(mmsp_gpu_handle* h, const void* src, size_t bytes, int layout, cudaMemcpyKind kind, bool sync)
{
    int rc = check_io(h, src, bytes, layout);
    if (rc) return rc;
    bool transpose = layout == MMSP_GPU_CELL_MAJOR && h->d.fields > 1;
    h->cur = 0;
    void* dst = transpose ? h->buf[1] : h->buf[0];
    cudaError_t e = cudaMemcpyAsync(dst, src, bytes, kind, h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "upload");
    if (transpose) {
        e = pf::launch_transpose(h->d.dtype, h->buf[1], h->buf[0], h->g.cells, h->d.fields, true, h->stream);
        if (e != cudaSuccess) return cuda_fail(h, e, "upload transpose");
    }
    if (h->d.model == MMSP_GPU_CH_CONVEX) {
        // the solver's first guess is a copy of the state (newGrid.copy(oldGrid), cahn-hilliard.cpp:283)
        e = cudaMemcpyAsync(h->buf[1], h->buf[0], h->bytes, cudaMemcpyDeviceToDevice, h->stream);
        if (e != cudaSuccess) return cuda_fail(h, e, "upload guess");
    }
    // the noise stream's step index counts from the upload
    if ((e = cudaMemsetAsync(h->flags + 4, 0, sizeof(long long), h->stream)) != cudaSuccess)
        return cuda_fail(h, e, "upload step counter");
    h->steps = 0;
    h->timed = false;
    if (sync && (e = cudaStreamSynchronize(h->stream)) != cudaSuccess) return cuda_fail(h, e, "upload sync");
    return MMSP_GPU_OK;
}

static int download(mmsp_gpu_handle* h, void* dst, size_t bytes, int layout, cudaMemcpyKind kind, bool sync)
{
    int rc = check_io(h, dst, bytes, layout);
    if (rc) return rc;
    bool transpose = layout == MMSP_GPU_CELL_MAJOR && h->d.fields > 1;
    const void* src = h->buf[h->cur];
    cudaError_t e;
    if (transpose) {
        // the other state buffer is free between steps, except for convex
        // splitting, whose next solve starts from it: that model stages in its
        // work buffer
        void* staging = h->d.model == MMSP_GPU_CH_CONVEX ? h->work : h->buf[h->cur ^ 1];
        e = pf::launch_transpose(h->d.dtype, h->buf[h->cur], staging, h->g.cells, h->d.fields, false, h->stream);
        if (e != cudaSuccess) return cuda_fail(h, e, "download transpose");
        src = staging;
    }
    e = cudaMemcpyAsync(dst, src, bytes, kind, h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "download");
    if (sync && (e = cudaStreamSynchronize(h->stream)) != cudaSuccess) return cuda_fail(h, e, "download sync");
    return sync ? check_flags(h) : MMSP_GPU_OK;
}

extern "C" int mmsp_gpu_upload(mmsp_gpu_handle* h, const void* host, size_t bytes, int layout)
{
    return upload(h, host, bytes, layout, cudaMemcpyHostToDevice, true);
}
extern "C" int mmsp_gpu_download(mmsp_gpu_handle* h, void* host, size_t bytes, int layout)
{
    return download(h, host, bytes, layout, cudaMemcpyDeviceToHost, true);
}
extern "C" int mmsp_gpu_upload_device(mmsp_gpu_handle* h, const void* dev, size_t bytes, int layout)
{
    return upload(h, dev, bytes, layout, cudaMemcpyDeviceToDevice, false);
}
extern "C" int mmsp_gpu_download_device(mmsp_gpu_handle* h, void* dev, size_t bytes, int layout)
{
    return download(h, dev, bytes, layout, cudaMemcpyDeviceToDevice, false);
}

// One step on `s`.  The stochastic forms read the index of their noise
// stream from the handle's device step counter and advance it after the
// step, so CUDA-graph replays of noisy steps draw new deviates every step.
static cudaError_t one_step(mmsp_gpu_handle* h, cudaStream_t s)
{
    bool ch = h->d.model == MMSP_GPU_CH || h->d.model == MMSP_GPU_CH_POLY;
    const void* in = h->buf[h->cur];
    void* out = h->buf[h->cur ^ 1];
    const pf::Coeffs& c = h->c;
    cudaError_t e = h->d.model == MMSP_GPU_OSTWALD ? pf::launch_ostwald(h->plan, h->d, h->g, c, in, out, h->work, h->flags, s)
                    : h->plan.kind == 6 ? pf::launch_ch64(h->plan, h->d, h->g, c, in, out, h->work, h->flags, s)
                    : h->plan.kind == 7 ? pf::launch_sparse_gg(h->d, h->g, c, in, out, h->flags, s)
                    : ch ? pf::launch_ch(h->plan, h->d, h->g, c, in, out, h->flags, s)
                         : pf::launch_ac(h->plan, h->d, h->g, c, in, out, h->flags, s);
    h->cur ^= 1;   // swap(oldGrid, newGrid), include/MMSP.grid.cpp:1913
    if (e == cudaSuccess && pf::noisy(h->d)) e = pf::launch_advance_step(h->flags, s);
    return e;
}

static int build_graph(mmsp_gpu_handle* h)
{
    if (h->graph) return MMSP_GPU_OK;   // kernel nodes do not depend on the launch stream
    // capture on a private stream so a caller's legacy/default stream works too
    cudaStream_t cs;
    cudaError_t e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cuda_fail(h, e, "graph stream");
    e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) {
        cudaStreamDestroy(cs);
        return cuda_fail(h, e, "begin capture");
    }
    const int saved = h->cur;
    const int64_t saved_launches = h->tb_launches;
    h->cur = 0;
    h->tb_launches = 0;
    cudaError_t le = cudaSuccess;
    if (h->tb)
        for (int i = 0; i < kGraphSteps / pf::kTbAnyDepth && le == cudaSuccess; i++) le = tb_launch(h, cs);
    else
        for (int i = 0; i < kGraphSteps && le == cudaSuccess; i++) le = one_step(h, cs);
    h->cur = saved;
    h->tb_launches = saved_launches;
    cudaGraph_t graph = nullptr;
    e = cudaStreamEndCapture(cs, &graph);
    cudaStreamDestroy(cs);
    if (le != cudaSuccess || e != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        return cuda_fail(h, le != cudaSuccess ? le : e, "capture");
    }
    e = cudaGraphInstantiate(&h->graph, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
        h->graph = nullptr;
        return cuda_fail(h, e, "instantiate");
    }
    return MMSP_GPU_OK;
}

// Convex-splitting Cahn-Hilliard: each step iterates red-black sweeps of
// the guess buf[cur^1] (which holds the state two steps back, as the
// example's swap leaves it) until the relative residual is at most the
// tolerance, checked after iterations 1-4 and every 5th
// (cahn-hilliard.cpp:311-388); then the guess becomes the state.
static const unsigned kCsMaxIter = 10000;    // max_iter, cahn-hilliard.cpp:55
static const unsigned kCsResidualStep = 5;   // residual_step, cahn-hilliard.cpp:54
// A step is one CUDA graph per state buffer (pf_convex.cu,
// build_convex_step_graph): its conditional `while` nodes run the checked
// iterations and decide on the device, so a call queues one graph launch per
// step and reads the loop state back once at the end.  The loop state lives
// in the handle's status block.
static pf::CsLoop* convex_loop(mmsp_gpu_handle* h) { return reinterpret_cast<pf::CsLoop*>(h->flags + 16); }

static int convex_steps(mmsp_gpu_handle* h, int steps)
{
    cudaError_t e;
    for (int p = 0; p < 2; p++)
        if (!h->cs_graph[p] &&
            (e = pf::build_convex_step_graph(h->d, h->g, h->c, h->buf[p], h->buf[p ^ 1], h->partials, convex_loop(h),
                                             kCsMaxIter, kCsResidualStep, &h->cs_graph[p])) != cudaSuccess) {
            h->cs_graph[p] = nullptr;
            return cuda_fail(h, e, "convex step graph");
        }
    for (int k = 0; k < steps; k++) {
        if ((e = cudaGraphLaunch(h->cs_graph[h->cur], h->stream)) != cudaSuccess) return cuda_fail(h, e, "convex step");
        h->cur ^= 1;   // swap(oldGrid, newGrid), cahn-hilliard.cpp:409
    }
    pf::CsLoop L;
    if ((e = cudaMemcpyAsync(&L, convex_loop(h), sizeof(L), cudaMemcpyDeviceToHost, h->stream)) != cudaSuccess ||
        (e = cudaStreamSynchronize(h->stream)) != cudaSuccess)
        return cuda_fail(h, e, "convex loop state");
    h->last_iters = L.last_iters;
    if (L.hit_max) {
        cudaMemsetAsync(&convex_loop(h)->hit_max, 0, sizeof(int), h->stream);
        char msg[64];
        snprintf(msg, sizeof(msg), "%u iterations, residual %.3g", L.last_iters, L.residual);
        return fail(h, MMSP_GPU_ENOCONV, "convex splitting stagnated within steps %s: %s",
                    (std::to_string(h->steps) + ".." + std::to_string(h->steps + steps - 1)).c_str(), msg);
    }
    return MMSP_GPU_OK;
}

extern "C" int mmsp_gpu_step(mmsp_gpu_handle* h, int steps)
{
    if (!h || steps < 0) return MMSP_GPU_EINVAL;
    if (steps == 0) return MMSP_GPU_OK;
    cudaError_t e = cudaEventRecord(h->ev0, h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "event");
    if (h->d.model == MMSP_GPU_SPARSE_GG) {
        // each call starts newGrid with empty cells, as update()'s copy-constructed newGrid
        // (sparsePF/graingrowth.cpp:67); within the call it keeps the state of two steps back
        e = cudaMemsetAsync(h->buf[h->cur ^ 1], 0, sizeof(int) * (size_t)h->g.cells, h->stream);
        if (e != cudaSuccess) return cuda_fail(h, e, "sparse newGrid");
    }
    int left = steps;
    if (h->d.model == MMSP_GPU_CH_CONVEX) {
        int rc = convex_steps(h, steps);
        if (rc) return rc;
        left = 0;
    } else if (h->tb) {
        constexpr int kTbGraph = kGraphSteps / pf::kTbAnyDepth;   // launches per graph replay (even)
        int nt = left / pf::kTbAnyDepth;
        left -= nt * pf::kTbAnyDepth;
        if (nt >= 2 * kTbGraph) {
            int rc = build_graph(h);
            if (rc) return rc;
            // the graph starts from buf[0] at an even launch count
            if (h->cur == 1 && (h->tb_launches & 1) == 1) {
                if ((e = tb_launch(h, h->stream)) != cudaSuccess) return cuda_fail(h, e, "blocked step");
                nt--;
            }
            if (h->cur == 0 && (h->tb_launches & 1) == 0)
                while (nt >= kTbGraph) {
                    if ((e = cudaGraphLaunch(h->graph, h->stream)) != cudaSuccess) return cuda_fail(h, e, "graph launch");
                    nt -= kTbGraph;
                    h->tb_launches += kTbGraph;
                }
        }
        while (nt > 0) {
            if ((e = tb_launch(h, h->stream)) != cudaSuccess) return cuda_fail(h, e, "blocked step");
            nt--;
        }
    } else if (steps >= kGraphMin) {
        int rc = build_graph(h);
        if (rc) return rc;
        if (h->cur == 1) {
            if ((e = one_step(h, h->stream)) != cudaSuccess) return cuda_fail(h, e, "step");
            left--;
        }
        while (left >= kGraphSteps) {
            if ((e = cudaGraphLaunch(h->graph, h->stream)) != cudaSuccess) return cuda_fail(h, e, "graph launch");
            left -= kGraphSteps;   // even count: the state is back in buf[0]
        }
    }
    while (left > 0) {
        if ((e = one_step(h, h->stream)) != cudaSuccess) return cuda_fail(h, e, "step");
        left--;
    }
    if ((e = cudaEventRecord(h->ev1, h->stream)) != cudaSuccess) return cuda_fail(h, e, "event");
    h->timed = true;
    h->steps += steps;
    return MMSP_GPU_OK;
}

// After a synchronisation: report (and clear) a kernel's timed-out wait
// (word 0) or a sparse list that outgrew its slots (word 1).
static int check_flags(mmsp_gpu_handle* h)
{
    int f[2] = {0, 0};
    cudaError_t e = cudaMemcpy(f, h->flags, sizeof(f), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(h, e, "flags");
    if (f[0] || f[1]) {
        cudaMemset(h->flags, 0, sizeof(f));
        if (f[0]) return fail(h, MMSP_GPU_ETIMEDOUT, "%s", "a step kernel's bounded wait ran out; the state is invalid");
        return fail(h, MMSP_GPU_EOVERFLOW, "%s", "a sparse cell's list outgrew its slots (desc.fields); "
                                                  "the state is invalid");
    }
    return MMSP_GPU_OK;
}

extern "C" int mmsp_gpu_synchronize(mmsp_gpu_handle* h)
{
    if (!h) return MMSP_GPU_EINVAL;
    cudaError_t e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "synchronize");
    return check_flags(h);
}

extern "C" int mmsp_gpu_reduce(mmsp_gpu_handle* h, mmsp_gpu_stats* st)
{
    if (!h || !st) return MMSP_GPU_EINVAL;
    if (h->d.model == MMSP_GPU_SPARSE_GG)
        return fail(h, MMSP_GPU_EUNSUPPORTED, "%s", "no reductions of sparse grids (the example reports none)");
    cudaError_t e = pf::launch_reduce(h->d, h->g, h->c, h->buf[h->cur], h->partials, h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "reduce");
    double res[2];
    e = cudaMemcpyAsync(res, h->partials + 4 * pf::kReduceBlocks, sizeof(res), cudaMemcpyDeviceToHost, h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "reduce copy");
    if ((e = cudaStreamSynchronize(h->stream)) != cudaSuccess) return cuda_fail(h, e, "reduce sync");
    int rc = check_flags(h);
    if (rc) return rc;
    st->mass = res[0];
    st->energy = res[1];
    st->steps = h->steps;
    st->solver_iterations = h->last_iters;
    st->gpu_ms = 0.0;
    if (h->timed) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, h->ev0, h->ev1) == cudaSuccess) st->gpu_ms = ms;
        else cudaGetLastError();
    }
    return MMSP_GPU_OK;
}

extern "C" int mmsp_gpu_state(mmsp_gpu_handle* h, void** p)
{
    if (!h || !p) return MMSP_GPU_EINVAL;
    *p = h->buf[h->cur];
    return MMSP_GPU_OK;
}

extern "C" const char* mmsp_gpu_last_error(const mmsp_gpu_handle* h) { return h ? h->err : "NULL handle"; }

extern "C" int mmsp_gpu_update(const mmsp_gpu_desc* desc, void* host, size_t bytes, int layout, int steps,
                               mmsp_gpu_stats* stats)
{
    if (!host || steps < 0) return MMSP_GPU_EINVAL;
    if (desc && desc->model == MMSP_GPU_SPARSE_GG) return MMSP_GPU_EUNSUPPORTED;   // lists: use a handle
    mmsp_gpu_handle* h = nullptr;
    int rc = mmsp_gpu_create(&h, desc);
    if (rc) return rc;
    rc = mmsp_gpu_upload(h, host, bytes, layout);
    if (!rc) rc = mmsp_gpu_step(h, steps);
    if (!rc && stats) rc = mmsp_gpu_reduce(h, stats);
    if (!rc) rc = mmsp_gpu_download(h, host, bytes, layout);
    mmsp_gpu_destroy(h);
    return rc;
}

// ---------------------------------------------------------------------------
// Sparse grids: host cell-major slots through a staging copy in the idle
// buffer (newGrid, which every step call clears anyway).

extern "C" int mmsp_gpu_sparse_upload(mmsp_gpu_handle* h, const int32_t* count, const int32_t* index, const void* value)
{
    if (!h || !count || !index || !value) return MMSP_GPU_EINVAL;
    if (h->d.model != MMSP_GPU_SPARSE_GG) return fail(h, MMSP_GPU_EINVAL, "%s", "not a sparse grid");
    const long long cells = h->g.cells;
    const int K = h->d.fields;
    for (long long c = 0; c < cells; c++)
        if (count[c] < 0 || count[c] > K)
            return fail(h, MMSP_GPU_EINVAL, "%s", "a cell's count is outside 0..fields");
    const pf::SparseLayout L = pf::sparse_layout(cells, K);
    char* st = static_cast<char*>(h->buf[1]);
    cudaError_t e = cudaMemcpyAsync(st, count, sizeof(int) * (size_t)cells, cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(st + L.idx_off, index, sizeof(int) * (size_t)cells * K, cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(st + L.val_off, value, sizeof(double) * (size_t)cells * K, cudaMemcpyHostToDevice,
                            h->stream);
    if (e == cudaSuccess) e = pf::launch_sparse_pack(st, h->buf[0], cells, K, h->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(st, 0, sizeof(int) * (size_t)cells, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "sparse upload");
    h->cur = 0;
    h->steps = 0;
    h->timed = false;
    return MMSP_GPU_OK;
}

extern "C" int mmsp_gpu_sparse_download(mmsp_gpu_handle* h, int32_t* count, int32_t* index, void* value)
{
    if (!h || !count || !index || !value) return MMSP_GPU_EINVAL;
    if (h->d.model != MMSP_GPU_SPARSE_GG) return fail(h, MMSP_GPU_EINVAL, "%s", "not a sparse grid");
    const long long cells = h->g.cells;
    const int K = h->d.fields;
    const pf::SparseLayout L = pf::sparse_layout(cells, K);
    char* st = static_cast<char*>(h->buf[h->cur ^ 1]);
    cudaError_t e = pf::launch_sparse_unpack(h->buf[h->cur], st, cells, K, h->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(count, st, sizeof(int) * (size_t)cells, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(index, st + L.idx_off, sizeof(int) * (size_t)cells * K, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(value, st + L.val_off, sizeof(double) * (size_t)cells * K, cudaMemcpyDeviceToHost,
                            h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "sparse download");
    return check_flags(h);
}
