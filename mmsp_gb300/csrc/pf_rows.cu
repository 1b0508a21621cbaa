// pf_rows.cu -- FP32 Cahn-Hilliard step for rows of any length.
//
// The precision-form kernel for 2D (rows up to 1024 cells) and 3D (up to
// 512) grids that the bulk-copy streaming kernel does not take (rows that
// are not 32..512 cells in powers of two, or too few rows).  A block owns R rows of the plane (R = 1 in 2D) over their
// full length, one thread per cell, and streams along axis 0: each thread
// keeps its column of c for planes x, x+1, x+2 (and the next plane, loaded
// one plane ahead) and of mu for x-1, x, x+1 in registers.  The Z
// neighbours of c(x+1) and of mu(x) are read from two small shared-memory
// row buffers, double-buffered by plane parity, so one barrier per plane
// orders everything.  Periodic wrap: rows and planes by index, Z by the
// neighbour indices of the first and last cell.  Plain loads work for any
// alignment, which bulk copies would not.
#include "pf_device.cuh"
#include "pf_internal.h"

namespace pf {

struct RowsGeom {
    int NX;          // planes along the streaming axis (axis 0)
    int NY;          // rows per plane (1 in 2D)
    int Z;           // cells per row
    long long plane; // NY * Z
};

struct RowsCoef {
    float wx, wy, wz, w2;   // weights of the streaming, row and cell axes; w2 = 2 * sum
    float kappa, dtm, neg_r, u;
    float noise;                 // thermal noise standard deviation (NOISE kernels)
    unsigned long long seed;     // its stream
    long long cells;
    const long long* stepp;      // the handle's step counter: the stream's step index
};

template <int MODEL>
static __device__ __forceinline__ float rows_mu(float c, float lap, const RowsCoef& q)
{
    const float fp = MODEL == MMSP_GPU_CH ? c * fmaf(fmaf(4.0f, c, -6.0f), c, 2.0f) : c * fmaf(q.u, c * c, q.neg_r);
    return fmaf(-q.kappa, lap, fp);
}

// R rows per block; H halo rows of c on each side (2 in 3D, 0 in 2D).
template <int R, int H>
struct RowsShape {
    static constexpr int RC = R + 2 * H;          // rows of c held
    static constexpr int RM = H ? R + 2 : R;      // rows of mu computed
    static constexpr int OFF = H ? 1 : 0;         // index of row 0 in the mu arrays
};

// NOISE: the stochastic forms (model_B.cpp:100-101, spinodal.cpp:95-97) add
// std * N(0,1) to mu, deviate step*cells + cell of the counter-based stream
// (pf_device.cuh), so a halo mu recomputed in a neighbouring block draws the
// same number; the step comes from the handle's device counter, so graph
// replays advance it.
template <int R, int H, int MODEL, bool NOISE>
__global__ void __launch_bounds__(H ? 512 : 1024)
ch_rows_f32(const float* __restrict__ cin, float* __restrict__ cout, RowsGeom g, RowsCoef q, int planes)
{
    using S = RowsShape<R, H>;
    constexpr int RC = S::RC, RM = S::RM, OFF = S::OFF;
    const int Z = g.Z;
    const int t = threadIdx.x;
    const bool on = t < Z;
    const int zc = on ? t : 0;
    const int zl = zc == 0 ? Z - 1 : zc - 1;
    const int zh = zc == Z - 1 ? 0 : zc + 1;
    extern __shared__ __align__(16) float sm[];
    float* cz = sm;                  // [2][RM][Z]: c(x+1) rows, for Z neighbours
    float* mz = sm + 2 * RM * Z;     // [2][R][Z]:  mu(x) rows, for Z neighbours

    const int y0 = blockIdx.x * R;
    const int xs = blockIdx.y * planes;
    const int xe = min(xs + planes, g.NX);
    if (xs >= xe) return;
    int rowoff[RC];
#pragma unroll
    for (int i = 0; i < RC; i++) rowoff[i] = wrapi(y0 - H + i, g.NY) * Z + zc;
    auto load = [&](float (&d)[RC], int pl) {
        const float* base = cin + (long long)wrapi(pl, g.NX) * g.plane;
#pragma unroll
        for (int i = 0; i < RC; i++) d[i] = __ldg(base + rowoff[i]);
    };

    const unsigned long long kstep = NOISE ? (unsigned long long)*q.stepp * (unsigned long long)q.cells : 0ull;
    float c0[RC], c1[RC], c2[RC], nx[RC];
    float m0[RM], m1[RM], m2[RM];
    load(c0, xs - 2);
    load(c1, xs - 1);
    load(nx, xs);
#pragma unroll
    for (int i = 0; i < RM; i++) m0[i] = m1[i] = 0.0f;
    const int rows = min(R, g.NY - y0);

#pragma unroll 1
    for (int x = xs - 2; x < xe; x++) {
#pragma unroll
        for (int i = 0; i < RC; i++) c2[i] = nx[i];
        if (x + 3 <= xe + 1) load(nx, x + 3);
        // publish c(x+1) for the Z neighbours of this plane's mu
        float* czp = cz + (x & 1) * RM * Z;
        if (on)
#pragma unroll
            for (int m = 0; m < RM; m++) czp[m * Z + zc] = c1[m + H - OFF];
        __syncthreads();
        // mu(x+1) on rows -1..R (3D) or the row (2D)
#pragma unroll
        for (int m = 0; m < RM; m++) {
            const int i = m + H - OFF;
            const float cc = c1[i];
            const float sx = c0[i] + c2[i];
            const float sz = czp[m * Z + zl] + czp[m * Z + zh];
            float lap;
            if constexpr (H != 0) lap = fmaf(q.wx, sx, fmaf(q.wy, c1[i - 1] + c1[i + 1], fmaf(q.wz, sz, -q.w2 * cc)));
            else lap = fmaf(q.wx, sx, fmaf(q.wz, sz, -q.w2 * cc));
            m2[m] = rows_mu<MODEL>(cc, lap, q);
            if (NOISE) {
                const long long cell = (long long)wrapi(x + 1, g.NX) * g.plane + rowoff[i];
                m2[m] += gauss_at_f(q.seed, kstep + (unsigned long long)cell) * q.noise;
            }
        }
        // c'(x) from mu(x-1), mu(x), mu(x+1); Z neighbours of mu(x) from the buffer
        if (x >= xs) {
            const float* mzp = mz + (x & 1) * R * Z;
            float* dst = cout + (long long)x * g.plane + (long long)y0 * Z + zc;
#pragma unroll
            for (int r = 0; r < R; r++) {
                const int m = r + OFF;
                const float mm = m1[m];
                const float sx = m0[m] + m2[m];
                const float sz = mzp[r * Z + zl] + mzp[r * Z + zh];
                float lap;
                if constexpr (H != 0) lap = fmaf(q.wx, sx, fmaf(q.wy, m1[m - 1] + m1[m + 1], fmaf(q.wz, sz, -q.w2 * mm)));
                else lap = fmaf(q.wx, sx, fmaf(q.wz, sz, -q.w2 * mm));
                if (on && r < rows) dst[(long long)r * Z] = fmaf(q.dtm, lap, c0[r + H]);
            }
        }
        // publish mu(x+1) rows 0..R-1 for the next plane's update
        float* mzn = mz + ((x + 1) & 1) * R * Z;
        if (on)
#pragma unroll
            for (int r = 0; r < R; r++) mzn[r * Z + zc] = m2[r + OFF];
#pragma unroll
        for (int i = 0; i < RC; i++) {
            c0[i] = c1[i];
            c1[i] = c2[i];
        }
#pragma unroll
        for (int i = 0; i < RM; i++) {
            m0[i] = m1[i];
            m1[i] = m2[i];
        }
    }
}

template <int R, int H>
static const void* rows_pick(int model, bool noise)
{
    if (noise) return (const void*)&ch_rows_f32<R, H, MMSP_GPU_CH_POLY, true>;   // only the shipped form is noisy
    return model == MMSP_GPU_CH ? (const void*)&ch_rows_f32<R, H, MMSP_GPU_CH, false>
                                : (const void*)&ch_rows_f32<R, H, MMSP_GPU_CH_POLY, false>;
}

static RowsGeom rows_geom(const mmsp_gpu_desc& d)
{
    RowsGeom r;
    r.NX = d.n[0];
    r.NY = d.dim == 3 ? d.n[1] : 1;
    r.Z = d.n[d.dim - 1];
    r.plane = (long long)r.NY * r.Z;
    return r;
}

bool ch_rows_eligible(const mmsp_gpu_desc& d, const Geom& g)
{
    (void)g;
    // 3D blocks hold more registers per thread: rows up to 512 cells there
    return d.dtype == MMSP_GPU_F32 && (d.dim == 2 || d.dim == 3) && d.n[d.dim - 1] <= (d.dim == 3 ? 512 : 1024) &&
           (d.model == MMSP_GPU_CH || d.model == MMSP_GPU_CH_POLY);
}

static int rows_r(const mmsp_gpu_desc& d)
{
    if (d.dim == 2) return 1;
    return d.n[1] >= 4 ? 4 : (d.n[1] >= 2 ? 2 : 1);
}

cudaError_t plan_ch_rows(const mmsp_gpu_desc& d, const Geom& g, StepPlan* p)
{
    const RowsGeom rg = rows_geom(d);
    const int R = rows_r(d);
    const int H = d.dim == 3 ? 2 : 0;
    const int RM = H ? R + 2 : R;
    const bool noise = noisy(d);
    if (d.dim == 2) p->fn = rows_pick<1, 0>(d.model, noise);
    else if (R == 4) p->fn = rows_pick<4, 2>(d.model, noise);
    else if (R == 2) p->fn = rows_pick<2, 2>(d.model, noise);
    else p->fn = rows_pick<1, 2>(d.model, noise);
    const int threads = (rg.Z + 31) / 32 * 32;
    p->smem = sizeof(float) * (size_t)(2 * RM + 2 * R) * rg.Z;
    p->block = dim3(threads, 1, 1);
    cudaError_t e = ensure_smem(p->fn, p->smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, p->fn, threads, p->smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    const int strips = (rg.NY + R - 1) / R;
    // fill the GPU, but keep runs of at least 8 planes so the 4-plane warm-up stays small
    long long want = (long long)sm_count() * per_sm;
    int segs = (int)((want + strips - 1) / strips);
    int maxseg = (rg.NX + 7) / 8;
    if (segs > maxseg) segs = maxseg;
    if (segs < 1) segs = 1;
    p->planes = (rg.NX + segs - 1) / segs;
    segs = (rg.NX + p->planes - 1) / p->planes;
    p->grid = dim3(strips, segs, 1);
    p->fields = 1;
    p->kind = 3;
    p->ok = true;
    (void)g;
    return cudaSuccess;
}

cudaError_t launch_ch_rows(const StepPlan& p, const mmsp_gpu_desc& d, const Coeffs& c, const void* in, void* out,
                           int* err, cudaStream_t s)
{
    RowsGeom rg = rows_geom(d);
    RowsCoef q;
    if (d.dim == 3) {
        q.wx = (float)c.w[0];
        q.wy = (float)c.w[1];
        q.wz = (float)c.w[2];
    } else {
        q.wx = (float)c.w[0];
        q.wy = 0.0f;
        q.wz = (float)c.w[1];
    }
    q.w2 = 2.0f * (q.wx + q.wy + q.wz);
    q.kappa = (float)c.kappa;
    q.dtm = (float)c.dtm;
    q.neg_r = (float)c.neg_r;
    q.u = (float)c.u;
    q.noise = (float)c.noise;
    q.seed = c.seed;
    q.cells = (long long)rg.NX * rg.plane;
    q.stepp = noisy(d) ? step_word(err) : nullptr;
    int planes = p.planes;
    void* args[] = {(void*)&in, (void*)&out, (void*)&rg, (void*)&q, (void*)&planes};
    return cudaLaunchKernel(p.fn, p.grid, p.block, args, p.smem, s);
}

}  // namespace pf
