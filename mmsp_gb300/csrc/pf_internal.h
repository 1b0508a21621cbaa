// pf_internal.h -- interfaces between the translation units of libmmsp_gpu.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "MMSP.gpu.h"

namespace pf {

// Grid geometry as the kernels see it: three padded axes X (slowest), Y, Z
// (fastest).  A grid of dim d occupies the last d axes; the leading ones
// have extent 1.  Periodic wrap is applied to every index.
struct Geom {
    int X, Y, Z;       // padded extents
    int dim;           // 1..3: number of real axes
    long long YZ;      // Y*Z
    long long cells;   // X*Y*Z
};

// Constants of the Ostwald-ripening model, derived from the descriptor as
// ostwald.cpp:67-80 derives them (Cm, B, gamma, Da, Db).
struct OstConst {
    double Cm, Ca, Cb, A, B, Da, Db, g, delta, eps, kappa;
    double dtD, dtL;   // dt*D and dt*L, as the update multiplies them (ostwald.cpp:108,117)
};

// Constants of the convex-splitting Cahn-Hilliard solve, as the example
// defines them (cahn-hilliard.cpp:38-96, :293-298, :316-318).
struct CsConst {
    double A12;         // dt*D*lapWeight
    double KL;          // K*lapWeight
    double Ddt;         // D*dt
    double K, A, C0, B, Ca, Cb;
    double QA, QB, QC, QD;
    double omega, om1;  // omega and 1 - omega
    double tol;         // residual tolerance
    double cells;       // gridSize
};

// Model constants in double; the launchers narrow them to the state type.
struct Coeffs {
    double w[3];       // 1/(dx*dx) per real axis, MMSP axis order (grid.cpp:2062)
    double wg[3];      // 1/(2 dx) per real axis (grid.cpp:2163)
    double kappa;      // gradient coefficient
    double dtm;        // dt*M (CH, AC_POLY), dt*L (AC), dt (GG)
    double gamma2;     // 2*gamma (AC)
    double neg_r, u;   // -r, u (polynomial models)
    double gamma;      // gamma (energy)
    double dV;         // cell volume
    bool unit_w;       // every w == 1.0 exactly
    OstConst ost;      // MMSP_GPU_OSTWALD
    CsConst cs;        // MMSP_GPU_CH_CONVEX
    // Thermal noise of MMSP_GPU_CH_POLY / MMSP_GPU_AC_POLY (aux[0], aux[1]):
    // standard deviation (0: none), stream seed, and the index of the step
    // being launched (steps since the last upload).
    double noise;
    unsigned long long seed;
    long long step;
};

// Noise on: the shipped polynomial models with a nonzero standard deviation.
inline bool noisy(const mmsp_gpu_desc& d)
{
    return (d.model == MMSP_GPU_CH_POLY || d.model == MMSP_GPU_AC_POLY) && d.aux[0] != 0.0;
}

Geom make_geom(const mmsp_gpu_desc& d);
int sm_count();                 // SMs of the current device
// Allow `fn` at least `bytes` of dynamic shared memory.  The attribute is
// process-wide per kernel, so it is only ever raised: lowering it for one
// plan would break launches of another plan of the same kernel.
cudaError_t ensure_smem(const void* fn, size_t bytes);
Coeffs make_coeffs(const mmsp_gpu_desc& d);

// A prepared launch of one explicit step.
struct StepPlan {
    const void* fn;    // kernel
    const void* fn2;   // second kernel of two-pass plans (FP64 Cahn-Hilliard: the update pass)
    dim3 grid, block;
    size_t smem;
    int planes;        // planes of axis X per block (3D streaming)
    int fields;
    int kind;          // 0: generic tile kernel, 1: FP32 3D CH streaming, 2: FP32 3D AC streaming,
                       // 3: FP32 CH rows of any length, 4: Ostwald ripening (two kernels),
                       // 5: convex splitting, 6: FP64 CH in two passes through a work grid,
                       // 8: FP32 3D Ostwald ripening streaming (one kernel)
    int ring;          // planes in the shared-memory ring (streaming kernels)
    bool ok;
};

// Plans; returns cudaSuccess or the error of cudaFuncSetAttribute.
cudaError_t plan_ch(const mmsp_gpu_desc& d, const Geom& g, StepPlan* p);
cudaError_t plan_ac(const mmsp_gpu_desc& d, const Geom& g, StepPlan* p);

// FP32 3D Cahn-Hilliard on whole rows (pf_ch3_stream.cu).
bool ch3_stream_eligible(const mmsp_gpu_desc& d, const Geom& g);
cudaError_t plan_ch3_stream(const mmsp_gpu_desc& d, const Geom& g, StepPlan* p);
cudaError_t launch_ch3_stream(const StepPlan& p, const Geom& g, const Coeffs& c, const void* in, void* out,
                              int* err, cudaStream_t s);

// FP64 2D/3D Cahn-Hilliard in two passes, mu into `work` (cells values),
// then the update (pf_ch64.cu).  Needs the work grid, so only handles use it.
bool ch64_eligible(const mmsp_gpu_desc& d, const Geom& g);
cudaError_t plan_ch64(const mmsp_gpu_desc& d, const Geom& g, StepPlan* p);
cudaError_t launch_ch64(const StepPlan& p, const mmsp_gpu_desc& d, const Geom& g, const Coeffs& c, const void* in,
                        void* out, void* work, int* err, cudaStream_t s);

// FP32 2D/3D Cahn-Hilliard for any row length up to 1024 (pf_rows.cu).
bool ch_rows_eligible(const mmsp_gpu_desc& d, const Geom& g);
cudaError_t plan_ch_rows(const mmsp_gpu_desc& d, const Geom& g, StepPlan* p);
cudaError_t launch_ch_rows(const StepPlan& p, const mmsp_gpu_desc& d, const Coeffs& c, const void* in, void* out,
                           int* err, cudaStream_t s);

// FP32 3D Allen-Cahn on whole rows (pf_ac3_stream.cu).
bool ac3_stream_eligible(const mmsp_gpu_desc& d, const Geom& g);
cudaError_t plan_ac3_stream(const mmsp_gpu_desc& d, const Geom& g, StepPlan* p);
cudaError_t launch_ac3_stream(const StepPlan& p, const Geom& g, const Coeffs& c, const void* in, void* out,
                              int* err, cudaStream_t s);

// A handle's device status block (256 bytes): int word 0 is set when a
// kernel's bounded wait runs out, int word 1 when a sparse list overflows;
// the 64-bit word at byte 16 counts the steps since the last upload, the
// index of the noise stream of the stochastic forms.  Launchers get the
// block as `err`.
inline const long long* step_word(const int* err) { return reinterpret_cast<const long long*>(err + 4); }
// Add one to the step word (after each noisy step, in stream order).
cudaError_t launch_advance_step(int* err, cudaStream_t s);

// One step in -> out on `s`.  `err` is a device word a kernel sets when a
// bounded wait runs out.
cudaError_t launch_ch(const StepPlan& p, const mmsp_gpu_desc& d, const Geom& g, const Coeffs& c,
                      const void* in, void* out, int* err, cudaStream_t s);
cudaError_t launch_ac(const StepPlan& p, const mmsp_gpu_desc& d, const Geom& g, const Coeffs& c,
                      const void* in, void* out, int* err, cudaStream_t s);

// Ostwald ripening (pf_ostwald.cu): the chemical potential of the
// composition into `work` (cells values), then the update of every field;
// FP32 3D grids with rows of 32, 64 or 128 cells and 2..4 fields take the
// one-kernel streaming step of pf_ost3_stream.cu instead (plan kind 8).
cudaError_t plan_ostwald(const mmsp_gpu_desc& d, const Geom& g, StepPlan* p);
cudaError_t launch_ostwald(const StepPlan& p, const mmsp_gpu_desc& d, const Geom& g, const Coeffs& c,
                           const void* in, void* out, void* work, int* err, cudaStream_t s);
bool ost3_stream_eligible(const mmsp_gpu_desc& d, const Geom& g);
cudaError_t plan_ost3_stream(const mmsp_gpu_desc& d, const Geom& g, const Coeffs& c, StepPlan* p);
cudaError_t launch_ost3_stream(const StepPlan& p, const Geom& g, const OstConst& o, const Coeffs& c,
                               const void* in, void* out, int* err, cudaStream_t s);

// Convex-splitting Cahn-Hilliard (pf_convex.cu).  One red-black sweep
// (color 1, then color 0 as the example orders them) of the guess `nw`
// given the old state; and the residual reduction into partials
// (result[0..1] = residual sum, norm of B, as launch_reduce leaves them).
cudaError_t launch_convex_sweeps(const mmsp_gpu_desc& d, const Geom& g, const Coeffs& c, const void* old,
                                 void* nw, cudaStream_t s);
cudaError_t launch_convex_residual(const mmsp_gpu_desc& d, const Geom& g, const Coeffs& c, const void* old,
                                   const void* nw, double* partials, cudaStream_t s);
// The iteration loop of one convex-splitting step in device memory: the
// iteration count and residual of the running solve, the count of the last
// finished one, and a flag set when a solve reached max_iter.
struct CsLoop {
    double residual;
    unsigned iter, last_iters;
    int hit_max, pad;
};
// One step as a CUDA graph (old -> guess nw): single iterations checked
// while iter < first_checks, then chunks of first_checks iterations checked
// at their ends, while the residual is above the tolerance and iter <
// max_iter; conditional `while` nodes decide on the device.
cudaError_t build_convex_step_graph(const mmsp_gpu_desc& d, const Geom& g, const Coeffs& c, const void* old, void* nw,
                                    double* partials, CsLoop* L, unsigned max_iter, unsigned first_checks,
                                    cudaGraphExec_t* exec);

// Sparse phase-field grain growth (pf_sparse.cu).  A state buffer holds
// count[cells] int32 at 0, index[K][cells] int32 at idx_off and
// value[K][cells] double at val_off (slot-major); a transfer staging buffer
// has the same offsets with the host's cell-major [cells][K] slots.
struct SparseLayout {
    size_t idx_off, val_off, bytes;
};
SparseLayout sparse_layout(long long cells, int K);
// One step in -> out (out holds the state of two steps back, or empty
// lists); a list that outgrows K sets err[1].
cudaError_t launch_sparse_gg(const mmsp_gpu_desc& d, const Geom& g, const Coeffs& c, const void* in, void* out,
                             int* err, cudaStream_t s);
cudaError_t launch_sparse_pack(const void* staging, void* state, long long cells, int K, cudaStream_t s);
cudaError_t launch_sparse_unpack(const void* state, void* staging, long long cells, int K, cudaStream_t s);

// Reductions: partial sums of (mass, energy) per block into `partials`
// (4 doubles per block: mass sum, mass compensation, energy sum, energy
// compensation), then a single-block pass into result[0..1] (mass, energy).
// The block count is fixed (kReduceBlocks), so results do not depend on timing.
constexpr int kReduceBlocks = 304;
constexpr size_t kPartialsBytes = sizeof(double) * 4 * (kReduceBlocks + 1);
cudaError_t launch_reduce(const mmsp_gpu_desc& d, const Geom& g, const Coeffs& c,
                          const void* state, double* partials, cudaStream_t s);

// Cell-major <-> field-major for vector grids.
cudaError_t launch_transpose(int dtype, const void* in, void* out, long long cells, int fields,
                             bool to_field_major, cudaStream_t s);

}  // namespace pf
