// pf_handle.h -- the handle behind mmsp_gpu_handle*, shared by the
// translation units of the C ABI (steps in mmsp_gpu.cu, file output in
// mmsp_gpu_output.cu).
#pragma once

#include "MMSP.gpu.h"
#include "pf_internal.h"

namespace pf {
struct BatchInst;
struct TbItem;
// Device bytes of one block holding a handle's buffers (two states, the
// reduction partials, the error words, a model's work grid), each 256-byte
// aligned, for create_in.
size_t handle_block_bytes(const mmsp_gpu_desc& d);
// A handle whose device buffers are carved from `block` (handle_block_bytes
// long, 256-byte aligned) and whose work is ordered on `stream`: no device
// allocation, no stream creation.  Destroying it frees neither.
int create_in(mmsp_gpu_handle** out, const mmsp_gpu_desc* desc, void* block, cudaStream_t stream);
struct OutputState;
// Wait for the handle's snapshots still being written, then free what the
// output path allocated.
void output_release(mmsp_gpu_handle* h);
}  // namespace pf

struct mmsp_gpu_handle {
    mmsp_gpu_desc d;
    pf::Geom g;
    pf::Coeffs c;
    pf::StepPlan plan;
    int device;
    size_t esize, elems, bytes;
    void* buf[2];
    int cur;                 // buf[cur] holds the state
    double* partials;        // reduction scratch
    void* work;              // MMSP_GPU_OSTWALD: the chemical-potential grid (cells values);
                             // MMSP_GPU_CH_CONVEX: download staging (state size)
    int* flags;              // device error word: a kernel's bounded wait ran out
    cudaStream_t own;        // private stream
    cudaStream_t stream;     // stream in use
    cudaEvent_t ev0, ev1;
    bool timed;              // ev0/ev1 bracket the last step call
    bool external;           // buffers and stream belong to the caller (pf::create_in): not freed here
    int64_t steps;
    // CUDA graph of kGraphSteps steps starting from buf[0] (an even count ends in buf[0]); for
    // blocked handles, kGraphSteps / pf::kTbAnyDepth launches from buf[0] at an even launch count
    cudaGraphExec_t graph;
    pf::OutputState* out;    // snapshot writer (mmsp_gpu_output), created on first use
    unsigned last_iters;     // MMSP_GPU_CH_CONVEX: solver iterations of the last step
    cudaGraphExec_t cs_graph[2];   // MMSP_GPU_CH_CONVEX: one step (the solve's whole loop), per buf[cur]
    // 2D FP32 Cahn-Hilliard: blocks of pf::kTbAnyDepth steps per launch of the
    // temporally blocked kernel (its instance, tile list and work counters in `work`)
    bool tb;
    const void* tb_fn;
    size_t tb_smem;
    int tb_blocks, tb_items;
    int64_t tb_launches;     // launches so far: their parity picks the work counter
    pf::BatchInst* tb_inst;
    pf::TbItem* tb_list;
    int* tb_counters;
    char err[512];
};
