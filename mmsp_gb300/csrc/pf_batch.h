// pf_batch.h -- batched 2D Cahn-Hilliard: work-list types and kernel launcher.
#pragma once

#include <cuda_runtime.h>

#include "pf_internal.h"

namespace pf {

// One instance in the pool.  Parameters are per instance (the batched
// configuration draws kappa and the mean composition per grid).
struct BatchInst {
    long long off;          // element offset of the instance in the pool
    int n0, n1;             // rows (axis 0) and cells per row (axis 1, a multiple of 32, <= 512)
    double w0, w1;          // 1/(dx*dx) per axis
    double kappa, dtm, neg_r, u;
};

// A run of output rows [xs, xe) of one instance.
struct BatchItem {
    int inst, xs, xe;
};

constexpr int kBatchMaxRow = 512;

// True if a descriptor can join the persistent batched kernel.
inline bool batch_eligible(const mmsp_gpu_desc& d)
{
    if (d.dim != 2 || d.fields != 1) return false;
    if (d.model != MMSP_GPU_CH && d.model != MMSP_GPU_CH_POLY) return false;
    return d.n[1] % 32 == 0 && d.n[1] >= 32 && d.n[1] <= kBatchMaxRow && d.n[0] >= 1;
}

// A tile of one instance for the temporally blocked kernel: interior rows
// [x0, x0+tx) and columns [z0, z0+tz).
struct TbItem {
    int inst, x0, z0, tx, tz;
};

// Region shapes of the temporally blocked kernel (rows, halo included, of
// kTbCols cells, and block size), and the depths (steps per launch) it is
// built for.  Its 16-byte loads need rows of a multiple of 4 cells at 16-byte
// aligned offsets, which batch_eligible grids in the pools have.
constexpr int kTbCols = 128;
struct TbShape {
    int ri;   // region rows, halo included
    int nt;   // threads per block
};
constexpr int kTbShapeCount = 4;
extern const TbShape kTbShapes[kTbShapeCount];
constexpr int kTbDepths[] = {2, 4, 8};

const void* tb_kernel(int shape, int ks, int model, bool unit);   // FP32 only
size_t tb_smem(int shape);
// Single 2D FP32 Cahn-Hilliard grids of any row length (handles): region
// shape 0 (64 x 128 cells, 4 warps) at depth kTbAnyDepth, loads and stores
// cell by cell where rows are not a multiple of 4 cells.
constexpr int kTbAnyDepth = 4;
const void* tb_kernel_any(int model, bool unit);
cudaError_t launch_tb(const void* fn, int blocks, int threads, size_t smem, const BatchInst* insts,
                      const TbItem* items, int nitems, const void* in, void* out, int* counters, int parity,
                      cudaStream_t s);

const void* batch_kernel(int dtype, int model, bool unit);
cudaError_t launch_batch(const void* fn, int blocks, int threads, const BatchInst* insts, const BatchItem* items,
                         int nitems, const void* in, void* out, int* counters, int parity, cudaStream_t s);

}  // namespace pf
