// pf_probe.cu -- mmsp_gpu_fp64_rate: the FP64 instruction rate of the current device.
//
// The FP64 forms of the step are bound by the FP64 pipe, not by HBM (GB300
// issues about two FP64 operations per clock per SM).  Their roofline is this
// measured rate: eight independent chains of fused multiply-adds per thread,
// every SM loaded with full blocks, timed with CUDA events.  An add, a
// multiply and a fused multiply-add each take one issue slot of the pipe, so
// the rate is in operations (instructions per lane) per second.
#include <cuda_runtime.h>

#include "MMSP.gpu.h"
#include "pf_internal.h"

namespace pf {

constexpr int kProbeChains = 8;
constexpr int kProbeThreads = 256;

__global__ void __launch_bounds__(kProbeThreads) fp64_probe(double* sink, int iters, double a, double b)
{
    double x[kProbeChains];
#pragma unroll
    for (int k = 0; k < kProbeChains; k++) x[k] = (double)(threadIdx.x + k) * 1e-3;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int k = 0; k < kProbeChains; k++) x[k] = fma(x[k], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < kProbeChains; k++) s += x[k];
    if (s == -1.0) sink[0] = s;   // never true for these inputs; keeps the chains live
}

}  // namespace pf

extern "C" int mmsp_gpu_fp64_rate(void* cuda_stream, double* ops_per_second)
{
    if (!ops_per_second) return MMSP_GPU_EINVAL;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
        cudaGetLastError();
        return MMSP_GPU_ENODEV;
    }
    cudaStream_t s = (cudaStream_t)cuda_stream;
    double* sink = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    const int blocks = pf::sm_count() * 8;
    const int iters = 4096;
    float best = 0.f;
    cudaError_t e = cudaMalloc((void**)&sink, sizeof(double));
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    for (int rep = 0; rep < 4 && e == cudaSuccess; rep++) {   // the first launch warms up
        e = cudaEventRecord(e0, s);
        if (e == cudaSuccess) {
            pf::fp64_probe<<<blocks, pf::kProbeThreads, 0, s>>>(sink, iters, 0.999999, 1e-7);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaEventRecord(e1, s);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        float ms = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        if (e == cudaSuccess && rep > 0 && (best == 0.f || ms < best)) best = ms;
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (sink) cudaFree(sink);
    if (e != cudaSuccess || !(best > 0.f)) {
        cudaGetLastError();
        return e == cudaErrorMemoryAllocation ? MMSP_GPU_ENOMEM : MMSP_GPU_ECUDA;
    }
    const double ops = (double)blocks * pf::kProbeThreads * pf::kProbeChains * iters;
    *ops_per_second = ops / (best * 1e-3);
    return MMSP_GPU_OK;
}
