// pf_aux.cu -- geometry/coefficients, FP64 compensated reductions, layout transposes.
#include <math.h>

#include <map>
#include <mutex>

#include "pf_device.cuh"
#include "pf_internal.h"

namespace pf {

int sm_count()
{
    static int n = 0;
    if (!n) {
        int dev = 0, v = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) v = 152;
        n = v;
    }
    return n;
}

cudaError_t ensure_smem(const void* fn, size_t bytes)
{
    static std::mutex mu;
    static std::map<const void*, size_t> set;
    std::lock_guard<std::mutex> lock(mu);
    size_t& cur = set[fn];
    if (bytes <= cur) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess) cur = bytes;
    return e;
}

Geom make_geom(const mmsp_gpu_desc& d)
{
    Geom g;
    int e[3] = {1, 1, 1};
    for (int a = 0; a < d.dim; a++) e[3 - d.dim + a] = d.n[a];
    g.X = e[0];
    g.Y = e[1];
    g.Z = e[2];
    g.dim = d.dim;
    g.YZ = (long long)g.Y * g.Z;
    g.cells = (long long)g.X * g.YZ;
    return g;
}

Coeffs make_coeffs(const mmsp_gpu_desc& d)
{
    Coeffs c{};
    c.unit_w = true;
    c.dV = 1.0;
    for (int a = 0; a < d.dim; a++) {
        c.w[a] = 1.0 / (d.dx[a] * d.dx[a]);   // include/MMSP.grid.cpp:2062
        c.wg[a] = 1.0 / (2.0 * d.dx[a]);      // include/MMSP.grid.cpp:2163
        if (c.w[a] != 1.0) c.unit_w = false;
        c.dV *= d.dx[a];
    }
    c.kappa = d.kappa;
    c.gamma = d.gamma;
    c.gamma2 = 2.0 * d.gamma;
    c.neg_r = -d.r;
    c.u = d.u;
    c.dtm = (d.model == MMSP_GPU_GG || d.model == MMSP_GPU_ZENER || d.model == MMSP_GPU_SPARSE_GG)
                ? d.dt : d.dt * d.mobility;
    if (noisy(d)) {
        c.noise = d.aux[0];
        c.seed = (unsigned long long)d.aux[1];
    }
    if (d.model == MMSP_GPU_CH_CONVEX) {
        // cahn-hilliard.cpp (convex splitting) :38-96 and :293-298, the same expressions
        CsConst& q = c.cs;
        const double D = d.mobility, K = d.kappa, dt = d.dt;
        const double C0 = d.aux[0], Ca = d.aux[1], Cb = d.aux[2], A = d.aux[3];
        const double B = A / pow(Ca - C0, 2.0);
        double lapWeight = 0.0, gridSize = 1.0;
        for (int a = 0; a < d.dim; a++) {
            lapWeight += 2.0 / pow(d.dx[a], 2.0);
            gridSize *= (double)d.n[a];
        }
        q.A12 = dt * D * lapWeight;
        q.KL = K * lapWeight;
        q.Ddt = D * dt;
        q.K = K;
        q.A = A;
        q.C0 = C0;
        q.B = B;
        q.Ca = Ca;
        q.Cb = Cb;
        q.QA = B + Ca + Cb;
        q.QB = 3.0 * (B * C0 + Ca * Ca + Cb * Cb);
        q.QC = 3.0 * (B * C0 * C0 + pow(Ca, 3.0) + pow(Cb, 3.0));
        q.QD = B * pow(C0, 3.0) + pow(Ca, 4.0) + pow(Cb, 4.0);
        q.omega = d.aux[4];
        q.om1 = 1.0 - d.aux[4];
        q.tol = d.aux[5];
        q.cells = gridSize;
    }
    if (d.model == MMSP_GPU_OSTWALD) {
        // ostwald.cpp:67-80, with the same pow calls
        OstConst& o = c.ost;
        o.Ca = d.aux[1];
        o.Cb = d.aux[2];
        o.Cm = 0.5 * (o.Ca + o.Cb);
        o.A = d.aux[3];
        o.B = o.A / pow(o.Cb - o.Cm, 2);
        o.g = 2.0 / pow(o.Cb - o.Ca, 2);
        o.delta = d.aux[4];
        o.eps = d.aux[5];
        o.Da = o.g / pow(o.delta, 2);
        o.Db = o.g / pow(o.delta, 2);
        o.kappa = d.kappa;
        o.dtD = d.dt * d.aux[0];
        o.dtL = d.dt * d.mobility;
    }
    return c;
}

// ---------------------------------------------------------------------------
// Reductions.  Neumaier's compensated sum per thread, combined pairwise with
// the same rule across the warp (shuffles), the block (shared memory) and
// finally across blocks by one thread in block order, so the result depends
// only on the data and the fixed launch shape.

struct NS {
    double s, c;
};

static __device__ __forceinline__ void nadd(NS& a, double x)
{
    double t = a.s + x;
    if (fabs(a.s) >= fabs(x)) a.c += (a.s - t) + x;
    else a.c += (x - t) + a.s;
    a.s = t;
}

static __device__ __forceinline__ NS ncombine(NS a, NS b)
{
    nadd(a, b.s);
    a.c += b.c;
    return a;
}

struct RedArgs {
    double wg[3];          // gradient weights of padded axes X, Y, Z (0 for padding)
    double kappa, gamma, r, u;
    OstConst ost;
    CsConst cs;
    int model;
};

template <typename T>
static __device__ __forceinline__ double gsq(const T* f, const Geom& g, const RedArgs& a, int x, int y, int z)
{
    double s = 0.0;
    if (a.wg[0] != 0.0) {
        double h = (double)f[(long long)wrapi(x + 1, g.X) * g.YZ + (long long)y * g.Z + z];
        double l = (double)f[(long long)wrapi(x - 1, g.X) * g.YZ + (long long)y * g.Z + z];
        double gi = a.wg[0] * (h - l);
        s += gi * gi;
    }
    if (a.wg[1] != 0.0) {
        double h = (double)f[(long long)x * g.YZ + (long long)wrapi(y + 1, g.Y) * g.Z + z];
        double l = (double)f[(long long)x * g.YZ + (long long)wrapi(y - 1, g.Y) * g.Z + z];
        double gi = a.wg[1] * (h - l);
        s += gi * gi;
    }
    {
        double h = (double)f[(long long)x * g.YZ + (long long)y * g.Z + wrapi(z + 1, g.Z)];
        double l = (double)f[(long long)x * g.YZ + (long long)y * g.Z + wrapi(z - 1, g.Z)];
        double gi = a.wg[2] * (h - l);
        s += gi * gi;
    }
    return s;
}

template <typename T>
__global__ void __launch_bounds__(256) reduce_kernel(const T* __restrict__ st, Geom g, int N, RedArgs a,
                                                     double* __restrict__ partials)
{
    NS m{0.0, 0.0}, e{0.0, 0.0};
    const bool ch = a.model == MMSP_GPU_CH || a.model == MMSP_GPU_CH_POLY;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < g.cells;
         i += (long long)gridDim.x * blockDim.x) {
        int x = (int)(i / g.YZ);
        long long r = i - (long long)x * g.YZ;
        int y = (int)(r / g.Z);
        int z = (int)(r - (long long)y * g.Z);
        if (ch) {
            double C = (double)st[i];
            double f;
            if (a.model == MMSP_GPU_CH) {
                double omc = 1.0 - C;
                f = C * C * omc * omc;
            } else {
                double c2 = C * C;
                f = -0.5 * a.r * c2 + 0.25 * a.u * c2 * c2;
            }
            nadd(e, f + 0.5 * a.kappa * gsq(st, g, a, x, y, z));
            nadd(m, C);
        } else if (a.model == MMSP_GPU_CH_CONVEX) {
            // reportEnergy of the example (cahn-hilliard.cpp:172-200): energy_density(C)
            // + K/2 |grad C|^2 and the mass of C (field 1, the chemical potential, is not summed)
            const CsConst& q = a.cs;
            const double C = (double)st[i];
            const double d0 = C - q.C0, da = C - q.Ca, db = C - q.Cb;
            const double f = -0.5 * q.A * d0 * d0 + 0.25 * q.B * d0 * d0 * d0 * d0 + 0.25 * q.Ca * da * da * da * da +
                             0.25 * q.Cb * db * db * db * db;
            nadd(e, f + 0.5 * q.K * gsq(st, g, a, x, y, z));
            nadd(m, C);
        } else if (a.model == MMSP_GPU_OSTWALD) {
            // f = -A/2 (C-Cm)^2 + B/4 (C-Cm)^4 + Da/4 (C-Ca)^4 + Db/4 (C-Cb)^4 - g/2 (C-Ca)^2 sum e^2
            //     + delta/4 sum e^4 + eps/2 sum_{i<j} e_i^2 e_j^2 + kappa/2 sum over all fields |grad|^2,
            // whose C-derivative is the chemical potential of ostwald.cpp:97-99
            const OstConst& o = a.ost;
            const double C = (double)st[i];
            const double dm = C - o.Cm, da = C - o.Ca, db = C - o.Cb;
            double grad = gsq(st, g, a, x, y, z), sq = 0.0, quart = 0.0, pair = 0.0;
            nadd(m, C);
            for (int j = 1; j < N; j++) {
                const T* f = st + (long long)j * g.cells;
                const double p = (double)f[i];
                const double p2 = p * p;
                quart += p2 * p2;
                pair += p2 * sq;
                sq += p2;
                grad += gsq(f, g, a, x, y, z);
                nadd(m, p);
            }
            const double dm2 = dm * dm, da2 = da * da, db2 = db * db;
            nadd(e, -0.5 * o.A * dm2 + 0.25 * o.B * dm2 * dm2 + 0.25 * o.Da * da2 * da2 + 0.25 * o.Db * db2 * db2 -
                        0.5 * o.g * da2 * sq + 0.25 * o.delta * quart + 0.5 * o.eps * pair + 0.5 * o.kappa * grad);
        } else {
            double bulk = 0.0, pair = 0.0, grad = 0.0, sq = 0.0;
            for (int j = 0; j < N; j++) {
                const T* f = st + (long long)j * g.cells;
                double p = (double)f[i];
                double p2 = p * p;
                if (a.model == MMSP_GPU_AC_POLY) bulk += -0.5 * a.r * p2 + 0.25 * a.u * p2 * p2;
                else bulk += -0.5 * p2 + 0.25 * p2 * p2;
                pair += p2 * sq;
                sq += p2;
                grad += gsq(f, g, a, x, y, z);
                nadd(m, p);
            }
            nadd(e, bulk + a.gamma * pair + 0.5 * a.kappa * grad);
        }
    }
    for (int off = 16; off > 0; off >>= 1) {
        NS mo{__shfl_down_sync(0xffffffffu, m.s, off), __shfl_down_sync(0xffffffffu, m.c, off)};
        NS eo{__shfl_down_sync(0xffffffffu, e.s, off), __shfl_down_sync(0xffffffffu, e.c, off)};
        m = ncombine(m, mo);
        e = ncombine(e, eo);
    }
    __shared__ double sh[8][4];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) {
        sh[warp][0] = m.s;
        sh[warp][1] = m.c;
        sh[warp][2] = e.s;
        sh[warp][3] = e.c;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        NS bm{0.0, 0.0}, be{0.0, 0.0};
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
            bm = ncombine(bm, NS{sh[w][0], sh[w][1]});
            be = ncombine(be, NS{sh[w][2], sh[w][3]});
        }
        partials[blockIdx.x * 4 + 0] = bm.s;
        partials[blockIdx.x * 4 + 1] = bm.c;
        partials[blockIdx.x * 4 + 2] = be.s;
        partials[blockIdx.x * 4 + 3] = be.c;
    }
}

// One warp: lane l combines partials l, l+32, ... (its loads run in
// parallel with the other lanes'), then lane 0 combines the 32 lane sums in
// lane order.  The assignment is fixed, so the result is deterministic.
__global__ void reduce_final(double* partials, int nblocks, double dV)
{
    if (blockIdx.x != 0 || threadIdx.x >= 32) return;
    const int lane = threadIdx.x;
    NS m{0.0, 0.0}, e{0.0, 0.0};
    for (int b = lane; b < nblocks; b += 32) {
        m = ncombine(m, NS{partials[b * 4 + 0], partials[b * 4 + 1]});
        e = ncombine(e, NS{partials[b * 4 + 2], partials[b * 4 + 3]});
    }
    NS tm{0.0, 0.0}, te{0.0, 0.0};
    for (int w = 0; w < 32; w++) {
        const NS om{__shfl_sync(0xffffffffu, m.s, w), __shfl_sync(0xffffffffu, m.c, w)};
        const NS oe{__shfl_sync(0xffffffffu, e.s, w), __shfl_sync(0xffffffffu, e.c, w)};
        tm = ncombine(tm, om);
        te = ncombine(te, oe);
    }
    if (lane == 0) {
        partials[nblocks * 4 + 0] = dV * (tm.s + tm.c);
        partials[nblocks * 4 + 1] = dV * (te.s + te.c);
    }
}

cudaError_t launch_reduce(const mmsp_gpu_desc& d, const Geom& g, const Coeffs& c,
                          const void* state, double* partials, cudaStream_t s)
{
    RedArgs a{};
    for (int k = 0; k < d.dim; k++) a.wg[3 - d.dim + k] = c.wg[k];
    a.kappa = d.kappa;
    const bool gg = d.model == MMSP_GPU_GG || d.model == MMSP_GPU_ZENER;
    a.gamma = gg ? 1.0 : d.gamma;
    a.r = d.r;
    a.u = d.u;
    a.model = d.model;
    a.ost = c.ost;
    a.cs = c.cs;
    int N = d.fields;
    if (gg) a.kappa = 2.0;   // graingrowth.cpp:105, zener.cpp:135: lap enters as 2*lap
    if (d.dtype == MMSP_GPU_F64)
        reduce_kernel<double><<<kReduceBlocks, 256, 0, s>>>((const double*)state, g, N, a, partials);
    else
        reduce_kernel<float><<<kReduceBlocks, 256, 0, s>>>((const float*)state, g, N, a, partials);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    reduce_final<<<1, 32, 0, s>>>(partials, kReduceBlocks, c.dV);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Cell-major (grid<dim,vector<T>> order) <-> field-major (device order).

template <typename T>
__global__ void transpose_kernel(const T* __restrict__ in, T* __restrict__ out, long long cells, int N,
                                 bool to_fm)
{
    const long long total = cells * N;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < total;
         k += (long long)gridDim.x * blockDim.x) {
        long long i = k / N;
        int j = (int)(k - i * N);
        if (to_fm) out[(long long)j * cells + i] = in[k];
        else out[k] = in[(long long)j * cells + i];
    }
}

cudaError_t launch_transpose(int dtype, const void* in, void* out, long long cells, int fields,
                             bool to_field_major, cudaStream_t s)
{
    int blocks = sm_count() * 8;
    if (dtype == MMSP_GPU_F64)
        transpose_kernel<double><<<blocks, 256, 0, s>>>((const double*)in, (double*)out, cells, fields, to_field_major);
    else
        transpose_kernel<float><<<blocks, 256, 0, s>>>((const float*)in, (float*)out, cells, fields, to_field_major);
    return cudaGetLastError();
}

__global__ void advance_step_kernel(long long* step) { *step += 1; }

cudaError_t launch_advance_step(int* err, cudaStream_t s)
{
    advance_step_kernel<<<1, 1, 0, s>>>(reinterpret_cast<long long*>(err + 4));
    return cudaGetLastError();
}

}  // namespace pf
