// mmsp_gpu_noalloc.cu -- mmsp_gpu_step_noalloc: explicit steps with no device allocation.
//
// Some callers cannot call cudaMalloc: their device memory is owned by
// another allocator or a fixed budget, or they run hot loops where
// cudaMalloc/cudaFree (which may synchronise the device) are not allowed.
// They pass their own input and output buffers; the intermediate state of a
// multi-step run (the reference's newGrid) and the kernels' error word live
// in one file-scope device array, so this path allocates nothing.
//
// The array is process-wide and per device: every call shares it and the
// last call's contents stay in it.  The error word is cleared before each
// call's kernels; the state part needs no clearing because every step
// overwrites all of it before it is read.  Calls that overlap on the GPU
// race on the array.
//
// The caller's buffers reach the FP32 3D kernels, which stage planes with
// bulk asynchronous copies that need 16-byte-aligned global addresses, so
// both pointers must be 16-byte aligned; a pointer that is not, or an
// output that partly overlaps the input, is refused before anything is
// queued on the device.
//
// The device address of the array is looked up once per device and kept
// for the life of the process.  cudaDeviceReset (or anything else that
// unloads the library's module from the device's primary context) leaves
// the kept address stale: a process that resets a device must not call this
// entry point on that device again.
#include <mutex>

#include <stdint.h>
#include <string.h>

#include "MMSP.gpu.h"
#include "pf_internal.h"

namespace {

constexpr size_t kFlagBytes = 256;   // error word, after the state scratch

// In host code `g_noalloc_scratch` names a host-side stand-in, not device
// memory: only the address from cudaGetSymbolAddress may be given to a kernel.
static __device__ __align__(256) unsigned char g_noalloc_scratch[MMSP_GPU_NOALLOC_MAX_BYTES + kFlagBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_addr[kMaxDevices];          // device address of g_noalloc_scratch, per device

// Once per device, with that device current.
int scratch_address(int dev, void** p)
{
    if (dev < 0 || dev >= kMaxDevices) return MMSP_GPU_ENODEV;
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_addr[dev]) {
        void* a = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&a, g_noalloc_scratch);
        if (e != cudaSuccess || !a) {
            cudaGetLastError();
            return MMSP_GPU_ECUDA;
        }
        g_addr[dev] = a;
    }
    *p = g_addr[dev];
    return MMSP_GPU_OK;
}

size_t state_bytes(const mmsp_gpu_desc& d)
{
    size_t n = (size_t)d.fields * (d.dtype == MMSP_GPU_F64 ? sizeof(double) : sizeof(float));
    for (int a = 0; a < d.dim; a++) n *= (size_t)d.n[a];
    return n;
}

}  // namespace

extern "C" int mmsp_gpu_step_noalloc(const mmsp_gpu_desc* desc, const void* in, void* out, int steps,
                                     void* cuda_stream)
{
    int rc = mmsp_gpu_validate(desc);
    if (rc) return rc;
    if (!in || !out || steps < 0) return MMSP_GPU_EINVAL;
    // a work grid of its own, or a noise stream indexed by the handle's step count
    if (desc->model == MMSP_GPU_OSTWALD || desc->model == MMSP_GPU_CH_CONVEX || desc->model == MMSP_GPU_SPARSE_GG ||
        pf::noisy(*desc))
        return MMSP_GPU_EUNSUPPORTED;
    mmsp_gpu_desc d = *desc;
    for (int a = d.dim; a < 3; a++) d.n[a] = 1;
    const size_t bytes = state_bytes(d);
    // 16-byte alignment for the bulk-copy kernels; an output that overlaps
    // the input without being it would be written while still being read
    const uintptr_t pi = reinterpret_cast<uintptr_t>(in), po = reinterpret_cast<uintptr_t>(out);
    if ((pi | po) & 15u) return MMSP_GPU_EINVAL;
    const bool in_place = pi == po;
    if (!in_place && pi < po + bytes && po < pi + bytes) return MMSP_GPU_EINVAL;
    cudaStream_t s = (cudaStream_t)cuda_stream;
    if (steps == 0) {
        if (in_place) return MMSP_GPU_OK;
        cudaError_t e = cudaMemcpyAsync(out, in, bytes, cudaMemcpyDeviceToDevice, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) cudaGetLastError();
        return e == cudaSuccess ? MMSP_GPU_OK : MMSP_GPU_ECUDA;
    }
    if ((steps > 1 || in_place) && bytes > MMSP_GPU_NOALLOC_MAX_BYTES) return MMSP_GPU_ENOMEM;

    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return MMSP_GPU_ENODEV;
    }
    void* base = nullptr;
    rc = scratch_address(dev, &base);
    if (rc) return rc;
    void* scratch = base;
    int* flag = reinterpret_cast<int*>(static_cast<unsigned char*>(base) + MMSP_GPU_NOALLOC_MAX_BYTES);

    const pf::Geom g = pf::make_geom(d);
    const pf::Coeffs c = pf::make_coeffs(d);
    pf::StepPlan plan;
    memset(&plan, 0, sizeof(plan));
    const bool ch = d.model == MMSP_GPU_CH || d.model == MMSP_GPU_CH_POLY;
    cudaError_t e = ch ? pf::plan_ch(d, g, &plan) : pf::plan_ac(d, g, &plan);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return plan.ok || ch ? MMSP_GPU_ECUDA : MMSP_GPU_EUNSUPPORTED;
    }
    e = cudaMemsetAsync(flag, 0, sizeof(int), s);
    // Step k (1-based) writes `out` when steps-k is even, else the scratch, so
    // the last step lands in `out`; in place, the first step cannot write
    // `out`, so the chain starts in the scratch and ends with a copy if odd.
    const void* src = in;
    for (int k = 1; k <= steps && e == cudaSuccess; k++) {
        void* dst;
        if (in_place) dst = ((k & 1) == 1) ? scratch : out;
        else dst = ((steps - k) & 1) == 0 ? out : scratch;
        e = ch ? pf::launch_ch(plan, d, g, c, src, dst, flag, s) : pf::launch_ac(plan, d, g, c, src, dst, flag, s);
        src = dst;
    }
    if (e == cudaSuccess && src != out) e = cudaMemcpyAsync(out, src, bytes, cudaMemcpyDeviceToDevice, s);
    // the error word comes back on the same stream, so one synchronisation
    // of that stream (not of the device) covers the steps and the read
    int f = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&f, flag, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return MMSP_GPU_ECUDA;
    }
    return f ? MMSP_GPU_ETIMEDOUT : MMSP_GPU_OK;
}
