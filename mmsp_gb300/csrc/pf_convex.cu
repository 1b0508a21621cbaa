// pf_convex.cu -- semi-implicit convex-splitting Cahn-Hilliard, FP64.
//
// The reference (examples/phase_transitions/cahn-hilliard/convex_splitting/
// cahn-hilliard.cpp:273-463) solves, each step, the linearised system for
// (c, mu) at every cell by red-black Gauss-Seidel with over-relaxation,
// checking the relative residual of the original system after iterations
// 1-4 and every 5th one.  With a 5/7-point stencil a cell reads only cells
// of the other color, so a sweep over one color is independent of its
// visiting order once every periodic extent is even: one thread per cell of
// the color gives the serial sweep's values.  The residual is a
// Neumaier-compensated sum with a fixed launch shape (deterministic).
//
// Operations follow the example's expressions with separately rounded FP64
// operations; pow(C,2.0) is C*C and pow(C,3.0) the compensated cube.
#include "pf_device.cuh"
#include "pf_internal.h"

namespace pf {

struct CsArgs {
    CsConst q;
    double wx, wy, wz;   // 1/dx^2 of padded axes X, Y, Z
};

struct CsNb {
    long long xh, xl, yh, yl;
    int zh, zl;
};

static __device__ __forceinline__ CsNb cs_row(const Geom& g, int x, int y)
{
    CsNb n;
    n.xh = (x + 1 == g.X ? -(long long)x : 1LL) * g.YZ;
    n.xl = (x == 0 ? (long long)(g.X - 1) : -1LL) * g.YZ;
    n.yh = (y + 1 == g.Y ? -(long long)y : 1LL) * g.Z;
    n.yl = (y == 0 ? (long long)(g.Y - 1) : -1LL) * g.Z;
    n.zh = n.zl = 0;
    return n;
}

// fringe_laplacian (cahn-hilliard.cpp:155-170): sum over axes of
// weight * (yh + yl), the Laplacian without its central term.
template <int DIM>
static __device__ __forceinline__ double fringe(const double* __restrict__ f, long long i, const CsNb& n,
                                                const CsArgs& a)
{
    using A = Ar<double>;
    double s = 0.0;
    if (DIM == 3) s = plus_zero(A::mul(a.wx, A::add(f[i + n.xh], f[i + n.xl])));
    if (DIM == 3) s = A::add(s, A::mul(a.wy, A::add(f[i + n.yh], f[i + n.yl])));
    if (DIM == 2) s = plus_zero(A::mul(a.wy, A::add(f[i + n.yh], f[i + n.yl])));
    const double tz = A::mul(a.wz, A::add(f[i + n.zh], f[i + n.zl]));
    return DIM == 1 ? plus_zero(tz) : A::add(s, tz);
}

template <int DIM>
static __device__ __forceinline__ double field_lap(const double* __restrict__ f, long long i, const CsNb& n,
                                                   const CsArgs& a)
{
    return lap_ref<double, false, DIM>(twice(f[i]), f[i + n.xh], f[i + n.xl], f[i + n.yh], f[i + n.yl], f[i + n.zh],
                                       f[i + n.zl], a.wx, a.wy, a.wz);
}

// expansive_dfdc (cahn-hilliard.cpp:92-96): -A*(C-C0) - QB*pow(C,2.0) - QD
static __device__ __forceinline__ double expansive(double C, const CsConst& q)
{
    using A = Ar<double>;
    return A::sub(A::sub(A::mul(-q.A, A::sub(C, q.C0)), A::mul(q.QB, A::mul(C, C))), q.QD);
}

// One color of the red-black sweep (cahn-hilliard.cpp:325-345): cells whose
// coordinate sum has the parity `skip` are left alone, as `continue` does.
template <int DIM>
__global__ void __launch_bounds__(256)
cs_sweep(const double* __restrict__ old, double* __restrict__ nw, Geom g, CsArgs a, int skip)
{
    using A = Ar<double>;
    const CsConst& q = a.q;
    const long long rows = (long long)g.X * g.Y;
    const double* c1 = nw;              // guess, field 0
    const double* u1 = nw + g.cells;    // guess, field 1
    for (long long row = blockIdx.x; row < rows; row += gridDim.x) {
        const int x = (int)(row / g.Y), y = (int)(row - (long long)x * g.Y);
        CsNb n = cs_row(g, x, y);
        // the first z of this row with the parity that is updated
        for (int z = ((x + y + skip + 1) & 1) + 2 * threadIdx.x; z < g.Z; z += 2 * blockDim.x) {
            n.zh = z + 1 == g.Z ? -z : 1;
            n.zl = z == 0 ? g.Z - 1 : -1;
            const long long i = row * g.Z + z;
            const double cOld = old[i];
            const double cGuess = c1[i], uGuess = u1[i];
            const double nonlin = A::add(A::mul(q.QA, A::mul(cGuess, cGuess)), q.QC);   // nonlinear_coeff
            const double A21 = A::sub(-nonlin, q.KL);
            const double detA = A::sub(1.0, A::mul(q.A12, A21));
            const double B1 = A::add(cOld, A::mul(q.Ddt, fringe<DIM>(u1, i, n, a)));
            const double B2 = A::sub(expansive(cOld, q), A::mul(q.K, fringe<DIM>(c1, i, n, a)));
            const double cNew = __ddiv_rn(A::sub(B1, A::mul(B2, q.A12)), detA);
            const double uNew = __ddiv_rn(A::sub(B2, A::mul(B1, A21)), detA);
            nw[i] = A::add(A::mul(q.omega, cNew), A::mul(q.om1, cGuess));
            nw[g.cells + i] = A::add(A::mul(q.omega, uNew), A::mul(q.om1, uGuess));
        }
    }
}

struct CsNS {
    double s, c;
};

static __device__ __forceinline__ void cs_add(CsNS& a, double x)
{
    const double t = a.s + x;
    if (fabs(a.s) >= fabs(x)) a.c += (a.s - t) + x;
    else a.c += (x - t) + a.s;
    a.s = t;
}

// Residual of the original system (cahn-hilliard.cpp:353-380): per cell
// R1 = cOld - (cNew - D*dt*lap u), R2 = expansive(cOld) - (uNew -
// contractive(cNew) + K*lap c); sums of R1^2 + R2^2 and of B1^2 + B2^2.
template <int DIM>
__global__ void __launch_bounds__(256)
cs_residual(const double* __restrict__ old, const double* __restrict__ nw, Geom g, CsArgs a,
            double* __restrict__ partials)
{
    using A = Ar<double>;
    const CsConst& q = a.q;
    CsNS r{0.0, 0.0}, b{0.0, 0.0};
    const long long rows = (long long)g.X * g.Y;
    const double* c1 = nw;
    const double* u1 = nw + g.cells;
    for (long long row = blockIdx.x; row < rows; row += gridDim.x) {
        const int x = (int)(row / g.Y), y = (int)(row - (long long)x * g.Y);
        CsNb n = cs_row(g, x, y);
        for (int z = threadIdx.x; z < g.Z; z += blockDim.x) {
            n.zh = z + 1 == g.Z ? -z : 1;
            n.zl = z == 0 ? g.Z - 1 : -1;
            const long long i = row * g.Z + z;
            const double lapC = field_lap<DIM>(c1, i, n, a);
            const double lapU = field_lap<DIM>(u1, i, n, a);
            const double cOld = old[i], cNew = c1[i], uNew = u1[i];
            const double B1 = cOld;
            const double B2 = expansive(cOld, q);
            const double AX1 = A::sub(cNew, A::mul(q.Ddt, lapU));
            const double contr = A::add(A::mul(q.QA, cube(cNew)), A::mul(q.QC, cNew));   // contractive_dfdc
            const double AX2 = A::add(A::sub(uNew, contr), A::mul(q.K, lapC));
            const double R1 = A::sub(B1, AX1), R2 = A::sub(B2, AX2);
            cs_add(r, A::add(A::mul(R1, R1), A::mul(R2, R2)));
            cs_add(b, A::add(A::mul(B1, B1), A::mul(B2, B2)));
        }
    }
    // block: warp shuffles, then one thread per block in warp order
    for (int off = 16; off > 0; off >>= 1) {
        CsNS ro{__shfl_down_sync(0xffffffffu, r.s, off), __shfl_down_sync(0xffffffffu, r.c, off)};
        CsNS bo{__shfl_down_sync(0xffffffffu, b.s, off), __shfl_down_sync(0xffffffffu, b.c, off)};
        cs_add(r, ro.s);
        r.c += ro.c;
        cs_add(b, bo.s);
        b.c += bo.c;
    }
    __shared__ double sh[8][4];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) {
        sh[warp][0] = r.s;
        sh[warp][1] = r.c;
        sh[warp][2] = b.s;
        sh[warp][3] = b.c;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        CsNS br{0.0, 0.0}, bb{0.0, 0.0};
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
            cs_add(br, sh[w][0]);
            br.c += sh[w][1];
            cs_add(bb, sh[w][2]);
            bb.c += sh[w][3];
        }
        partials[blockIdx.x * 4 + 0] = br.s;
        partials[blockIdx.x * 4 + 1] = br.c;
        partials[blockIdx.x * 4 + 2] = bb.s;
        partials[blockIdx.x * 4 + 3] = bb.c;
    }
}

// One warp: lane l combines partials l, l+32, ..., then lane 0 the lane
// sums in lane order (a fixed assignment: deterministic).
__global__ void cs_residual_final(double* partials, int nblocks)
{
    if (blockIdx.x != 0 || threadIdx.x >= 32) return;
    const int lane = threadIdx.x;
    CsNS r{0.0, 0.0}, b{0.0, 0.0};
    for (int k = lane; k < nblocks; k += 32) {
        cs_add(r, partials[k * 4 + 0]);
        r.c += partials[k * 4 + 1];
        cs_add(b, partials[k * 4 + 2]);
        b.c += partials[k * 4 + 3];
    }
    CsNS tr{0.0, 0.0}, tb{0.0, 0.0};
    for (int w = 0; w < 32; w++) {
        cs_add(tr, __shfl_sync(0xffffffffu, r.s, w));
        tr.c += __shfl_sync(0xffffffffu, r.c, w);
        cs_add(tb, __shfl_sync(0xffffffffu, b.s, w));
        tb.c += __shfl_sync(0xffffffffu, b.c, w);
    }
    if (lane == 0) {
        partials[nblocks * 4 + 0] = tr.s + tr.c;
        partials[nblocks * 4 + 1] = tb.s + tb.c;
    }
}

static CsArgs cs_args(const Coeffs& c, const Geom& g)
{
    CsArgs a;
    a.q = c.cs;
    double w[3] = {1.0, 1.0, 1.0};
    for (int k = 0; k < g.dim; k++) w[3 - g.dim + k] = c.w[k];
    a.wx = w[0];
    a.wy = w[1];
    a.wz = w[2];
    return a;
}

static dim3 cs_block(const Geom& g) { return dim3(g.Z >= 512 ? 256 : ((g.Z + 1) / 2 + 31) / 32 * 32); }

cudaError_t launch_convex_sweeps(const mmsp_gpu_desc& d, const Geom& g, const Coeffs& c, const void* old, void* nw,
                                 cudaStream_t s)
{
    (void)d;
    const CsArgs a = cs_args(c, g);
    long long blocks = (long long)g.X * g.Y;
    const long long most = 16LL * sm_count();
    if (blocks > most) blocks = most;
    const dim3 bl = cs_block(g);
    for (int color = 1; color > -1; color--) {   // cahn-hilliard.cpp:321: color 1, then 0
        if (g.dim == 3) cs_sweep<3><<<(int)blocks, bl, 0, s>>>((const double*)old, (double*)nw, g, a, color);
        else if (g.dim == 2) cs_sweep<2><<<(int)blocks, bl, 0, s>>>((const double*)old, (double*)nw, g, a, color);
        else cs_sweep<1><<<(int)blocks, bl, 0, s>>>((const double*)old, (double*)nw, g, a, color);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t launch_convex_residual(const mmsp_gpu_desc& d, const Geom& g, const Coeffs& c, const void* old,
                                   const void* nw, double* partials, cudaStream_t s)
{
    (void)d;
    const CsArgs a = cs_args(c, g);
    if (g.dim == 3) cs_residual<3><<<kReduceBlocks, 256, 0, s>>>((const double*)old, (const double*)nw, g, a, partials);
    else if (g.dim == 2)
        cs_residual<2><<<kReduceBlocks, 256, 0, s>>>((const double*)old, (const double*)nw, g, a, partials);
    else cs_residual<1><<<kReduceBlocks, 256, 0, s>>>((const double*)old, (const double*)nw, g, a, partials);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    cs_residual_final<<<1, 32, 0, s>>>(partials, kReduceBlocks);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// The solve's iteration loop on the device.  The example iterates
// (cahn-hilliard.cpp:311-388) while iter < max_iter and the residual is above
// the tolerance, checking the residual after iterations 1-4 and every 5th.
// A step is one CUDA graph: begin, a `while` node of single iterations (each
// checked) while iter < 5, a gate, a `while` node of 5-iteration chunks
// (checked at the end of each), end.  The check kernels compute the same
// residual expression as a host read-back would (correctly rounded sqrt and
// division) and set the nodes' conditions, so no step waits on the host.

__global__ void cs_loop_begin(CsLoop* L)
{
    L->iter = 0;
    L->residual = 1.0;
}

// after `add` iterations: the residual of cs_residual_final's sums, and
// whether the loop node goes on (iter < limit and residual > tol)
__global__ void cs_loop_check(const double* __restrict__ partials, int nblocks, CsLoop* L, double tol, double cells,
                              unsigned add, unsigned limit, cudaGraphConditionalHandle cond)
{
    L->iter += add;
    const double r = sqrt(partials[nblocks * 4 + 0] / partials[nblocks * 4 + 1]) / (2.0 * cells);
    L->residual = r;
    cudaGraphSetConditional(cond, (L->iter < limit && r > tol) ? 1u : 0u);
}

__global__ void cs_loop_gate(const CsLoop* L, double tol, unsigned max_iter, cudaGraphConditionalHandle cond)
{
    cudaGraphSetConditional(cond, (L->iter < max_iter && L->residual > tol) ? 1u : 0u);
}

__global__ void cs_loop_end(CsLoop* L, unsigned max_iter)
{
    L->last_iters = L->iter;
    if (L->iter >= max_iter) L->hit_max = 1;
}

namespace {

// Append a `while` node on handle `h` after the capture's current
// dependencies and return its body graph; the capture continues after the node.
cudaError_t add_while(cudaStream_t cs, cudaGraphConditionalHandle h, cudaGraph_t* body)
{
    cudaStreamCaptureStatus st;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t n = 0;
    cudaError_t e = cudaStreamGetCaptureInfo(cs, &st, nullptr, &g, &deps, nullptr, &n);
    if (e != cudaSuccess) return e;
    cudaGraphNodeParams prm = {};
    prm.type = cudaGraphNodeTypeConditional;
    prm.conditional.handle = h;
    prm.conditional.type = cudaGraphCondTypeWhile;
    prm.conditional.size = 1;
    cudaGraphNode_t node;
    if ((e = cudaGraphAddNode(&node, g, deps, nullptr, n, &prm)) != cudaSuccess) return e;
    *body = prm.conditional.phGraph_out[0];
    return cudaStreamUpdateCaptureDependencies(cs, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
}

}  // namespace

cudaError_t build_convex_step_graph(const mmsp_gpu_desc& d, const Geom& g, const Coeffs& c, const void* old, void* nw,
                                    double* partials, CsLoop* L, unsigned max_iter, unsigned first_checks,
                                    cudaGraphExec_t* exec)
{
    cudaStream_t cs = nullptr, bs = nullptr;
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&bs, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    const double tol = c.cs.tol, cells = c.cs.cells;
    bool capturing = e == cudaSuccess;
    cudaGraphConditionalHandle ha = 0, hb = 0;
    cudaGraph_t body = nullptr;
    if (e == cudaSuccess) {
        // both conditions belong to the graph being captured; the gate sets hb
        cudaStreamCaptureStatus st;
        cudaGraph_t top = nullptr;
        e = cudaStreamGetCaptureInfo(cs, &st, nullptr, &top, nullptr, nullptr, nullptr);
        if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&ha, top, 1, cudaGraphCondAssignDefault);
        if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&hb, top, 0, cudaGraphCondAssignDefault);
    }
    if (e == cudaSuccess) {
        cs_loop_begin<<<1, 1, 0, cs>>>(L);
        e = cudaGetLastError();
    }
    // single checked iterations while iter < first_checks
    if (e == cudaSuccess) e = add_while(cs, ha, &body);
    if (e == cudaSuccess) e = cudaStreamBeginCaptureToGraph(bs, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        e = launch_convex_sweeps(d, g, c, old, nw, bs);
        if (e == cudaSuccess) e = launch_convex_residual(d, g, c, old, nw, partials, bs);
        if (e == cudaSuccess) {
            cs_loop_check<<<1, 1, 0, bs>>>(partials, kReduceBlocks, L, tol, cells, 1u, first_checks, ha);
            e = cudaGetLastError();
        }
        cudaGraph_t done = nullptr;
        const cudaError_t e2 = cudaStreamEndCapture(bs, &done);
        if (e == cudaSuccess) e = e2;
    }
    if (e == cudaSuccess) {
        cs_loop_gate<<<1, 1, 0, cs>>>(L, tol, max_iter, hb);
        e = cudaGetLastError();
    }
    // then chunks of first_checks iterations, checked at the end of each
    if (e == cudaSuccess) e = add_while(cs, hb, &body);
    if (e == cudaSuccess) e = cudaStreamBeginCaptureToGraph(bs, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        for (unsigned k = 0; k < first_checks && e == cudaSuccess; k++) e = launch_convex_sweeps(d, g, c, old, nw, bs);
        if (e == cudaSuccess) e = launch_convex_residual(d, g, c, old, nw, partials, bs);
        if (e == cudaSuccess) {
            cs_loop_check<<<1, 1, 0, bs>>>(partials, kReduceBlocks, L, tol, cells, first_checks, max_iter, hb);
            e = cudaGetLastError();
        }
        cudaGraph_t done = nullptr;
        const cudaError_t e2 = cudaStreamEndCapture(bs, &done);
        if (e == cudaSuccess) e = e2;
    }
    if (e == cudaSuccess) {
        cs_loop_end<<<1, 1, 0, cs>>>(L, max_iter);
        e = cudaGetLastError();
    }
    if (capturing) {
        const cudaError_t e2 = cudaStreamEndCapture(cs, &graph);
        if (e == cudaSuccess) e = e2;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(exec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    if (cs) cudaStreamDestroy(cs);
    if (bs) cudaStreamDestroy(bs);
    return e;
}

}  // namespace pf
