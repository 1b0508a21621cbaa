// pf_ch64.cu -- FP64 Cahn-Hilliard step in two passes, as the reference runs it.
//
// The reference's update() (cahn-hilliard.cpp:69-79) makes two node loops per
// step: temp = mu(c) over every node, then c' = c + dt*M*lap(temp).  On GB300
// the FP64 pipe issues about two operations per clock per SM, a 64th of the
// FP32 rate, so the FP64 form is bound by its count of FP64 instructions,
// not by memory: HBM traffic is nearly free beside it.  A fused kernel has
// to recompute mu on the halo of every tile (1.2x the mu work on 256^3);
// these two kernels keep the reference's temp grid in HBM instead, so each
// mu is computed exactly once and each pass does the minimum FP64 work:
//
//   exact form       23 operations per cell (13 for mu, 10 for the update),
//                    the reference's order, every operation rounded on its
//                    own: bit-identical to the reference
//   contracted form  16 operations per cell: the six-neighbour sum once,
//                    the centre term folded into the chemical potential's
//                    polynomial and into the update's multiply-add.  Within
//                    a few ulps per step of the exact form; held to 1e-12
//                    relative against the reference after the full runs.
//
// A thread owns one (y, z) column and walks a run of X planes, carrying
// c(x-1), c(x), c(x+1) in registers; the four in-plane neighbours come
// through L1 with periodic wraps precomputed per thread.  Blocks are small
// (16 planes), so the block scheduler balances the FP64 work across SMs.
// Multiplies by 2 and the 0.0 + t of the Laplacian's first axis are done on
// the integer pipe (pf_device.cuh), and every decision about parameters
// (unit weights, kappa == 1, noise) is a template argument, so no FP64
// compare runs per cell.
#include "pf_device.cuh"
#include "pf_internal.h"

namespace pf {

constexpr int kC64Z = 32;        // block width along Z (one warp)
constexpr int kC64Y = 4;         // rows per block: 128 threads
constexpr int kC64Planes = 16;   // X planes per block (3D)

// Constants of both forms.
struct C64 {
    double wx, wy, wz;    // Laplacian weights of padded axes X, Y, Z
    double kappa, dtm, neg_r, u;
    double w2;            // 2 (wx + wy + wz) over the real axes: the centre weight
    double poly0;         // contracted mu: 2 + kappa*w2 (CH) or -r + kappa*w2 (CH_POLY)
    double upd0;          // contracted update: -dt*M*w2
    double noise;
    unsigned long long seed;
    long long step;
};

// Weighted sum of the neighbour pairs (sx, sy, sz: sums of the two
// neighbours along X, Y, Z), the contracted Laplacian without its centre term.
template <int DIM, bool UNIT>
static __device__ __forceinline__ double nsum(double sx, double sy, double sz, const C64& q)
{
    if (UNIT) return DIM == 3 ? (sx + sy) + sz : sy + sz;
    return DIM == 3 ? fma(q.wx, sx, fma(q.wy, sy, q.wz * sz)) : fma(q.wy, sy, q.wz * sz);
}

template <int DIM, int MODEL, bool UNIT, bool KONE, bool EXACT>
static __device__ __forceinline__ double mu_cell(double c, double xh, double xl, double yh, double yl, double zh,
                                                 double zl, const C64& q, const P<double>& p)
{
    if (EXACT) {
        // temp = mu(c) in the reference's order (pf_device.cuh: lap_ref, ch_mu)
        const double lap = lap_ref<double, UNIT, DIM>(twice(c), xh, xl, yh, yl, zh, zl, p.wx, p.wy, p.wz);
        P<double> pk = p;
        if (KONE) pk.kappa = 1.0;   // constant: kappa_times folds to lap
        return ch_mu<double, MODEL>(c, lap, pk);
    }
    // mu = f'(c) - kappa (S - w2 c) = c * (poly0 + ...) - kappa S
    const double s = nsum<DIM, UNIT>(xh + xl, yh + yl, zh + zl, q);
    double t;
    if (MODEL == MMSP_GPU_CH) {   // 2c(1-c)(1-2c) = c (2 + c (-6 + 4c))
        t = fma(fma(4.0, c, -6.0), c, q.poly0);
    } else {                      // -r c + u c^3 = c (-r + u c^2)
        t = fma(q.u, c * c, q.poly0);
    }
    return KONE ? t * c - s : fma(-q.kappa, s, t * c);
}

template <int DIM, int MODEL, bool UNIT, bool KONE, bool EXACT, bool NOISE>
__global__ void __launch_bounds__(kC64Z * kC64Y)
ch64_mu(const double* __restrict__ cin, double* __restrict__ mu, Geom g, C64 q, P<double> p, int planes)
{
    const int z = blockIdx.x * kC64Z + threadIdx.x;
    const int y = blockIdx.y * kC64Y + threadIdx.y;
    if (z >= g.Z || y >= g.Y) return;   // no barrier in this kernel
    const int zl = z == 0 ? g.Z - 1 : z - 1, zh = z + 1 == g.Z ? 0 : z + 1;
    const long long row = (long long)y * g.Z;
    const long long rl = (long long)(y == 0 ? g.Y - 1 : y - 1) * g.Z;
    const long long rh = (long long)(y + 1 == g.Y ? 0 : y + 1) * g.Z;
    const int xs = blockIdx.z * planes;
    const int xe = min(xs + planes, g.X);
    auto plane = [&](int x) { return cin + (long long)x * g.YZ; };
    double a = 0.0, b = __ldg(plane(xs) + row + z);
    if (DIM == 3) a = __ldg(plane(xs == 0 ? g.X - 1 : xs - 1) + row + z);
    for (int x = xs; x < xe; x++) {
        const double* pc = plane(x);
        double n = 0.0;
        if (DIM == 3) n = __ldg(plane(x + 1 == g.X ? 0 : x + 1) + row + z);
        const double vyh = __ldg(pc + rh + z), vyl = __ldg(pc + rl + z);
        const double vzh = __ldg(pc + row + zh), vzl = __ldg(pc + row + zl);
        double m = mu_cell<DIM, MODEL, UNIT, KONE, EXACT>(b, n, a, vyh, vyl, vzh, vzl, q, p);
        // thermal noise of the stochastic forms (model_B.cpp:100-101, spinodal.cpp:95-97): mu + noise
        if (NOISE) m = EXACT ? __dadd_rn(m, noise_at(p, g.cells, (long long)x * g.YZ + row + z))
                             : m + noise_at(p, g.cells, (long long)x * g.YZ + row + z);
        mu[(long long)x * g.YZ + row + z] = m;
        a = b;
        b = n;
    }
}

template <int DIM, bool UNIT, bool EXACT>
__global__ void __launch_bounds__(kC64Z * kC64Y)
ch64_update(const double* __restrict__ cin, const double* __restrict__ mu, double* __restrict__ cout, Geom g, C64 q,
            P<double> p, int planes)
{
    const int z = blockIdx.x * kC64Z + threadIdx.x;
    const int y = blockIdx.y * kC64Y + threadIdx.y;
    if (z >= g.Z || y >= g.Y) return;
    const int zl = z == 0 ? g.Z - 1 : z - 1, zh = z + 1 == g.Z ? 0 : z + 1;
    const long long row = (long long)y * g.Z;
    const long long rl = (long long)(y == 0 ? g.Y - 1 : y - 1) * g.Z;
    const long long rh = (long long)(y + 1 == g.Y ? 0 : y + 1) * g.Z;
    const int xs = blockIdx.z * planes;
    const int xe = min(xs + planes, g.X);
    auto plane = [&](int x) { return mu + (long long)x * g.YZ; };
    double a = 0.0, b = __ldg(plane(xs) + row + z);
    if (DIM == 3) a = __ldg(plane(xs == 0 ? g.X - 1 : xs - 1) + row + z);
    for (int x = xs; x < xe; x++) {
        const long long i = (long long)x * g.YZ + row + z;
        const double* pm = plane(x);
        double n = 0.0;
        if (DIM == 3) n = __ldg(plane(x + 1 == g.X ? 0 : x + 1) + row + z);
        const double myh = __ldg(pm + rh + z), myl = __ldg(pm + rl + z);
        const double mzh = __ldg(pm + row + zh), mzl = __ldg(pm + row + zl);
        const double c = __ldg(cin + i);
        double o;
        if (EXACT) {
            // newGrid(n) = GRID(n) + dt*M*lap(temp)   (cahn-hilliard.cpp:75-76)
            const double lap = lap_ref<double, UNIT, DIM>(twice(b), n, a, myh, myl, mzh, mzl, p.wx, p.wy, p.wz);
            o = __dadd_rn(c, __dmul_rn(p.dtm, lap));
        } else {
            // c + dtM (S - w2 mu) = fma(dtM, S, c - dtM w2 mu)
            const double s = nsum<DIM, UNIT>(n + a, myh + myl, mzh + mzl, q);
            o = fma(q.dtm, s, fma(q.upd0, b, c));
        }
        cout[i] = o;
        a = b;
        b = n;
    }
}

// The stochastic 3D Cahn-Hilliard form in FP32 (model B, spinodal: CH_POLY
// with noise) takes the same two passes: the noise term costs two SplitMix64
// draws, a logarithm, a cosine and a square root per cell, and a fused kernel
// would draw it again on every halo; here each deviate is drawn once, in the
// mu pass, at 8 B per cell of extra traffic (128^3 x 500 steps: 13.0 ms
// against 15.2 ms for the fused row kernel; in 2D the fused tile kernel
// stays faster, 7.1 ms against 8.3 ms on 1024^2).  Arithmetic as the FP32 form's:
// mu = c (-r + kappa w2 + u c^2) - kappa S + noise, c' = c + dtM (S_mu - w2 mu).
struct C32 {
    float wx, wy, wz, kappa, u, dtm, poly0, upd0;
};

template <int DIM, bool UNIT>
static __device__ __forceinline__ float nsum_f(float sx, float sy, float sz, const C32& q)
{
    if (UNIT) return DIM == 3 ? (sx + sy) + sz : sy + sz;
    return DIM == 3 ? fmaf(q.wx, sx, fmaf(q.wy, sy, q.wz * sz)) : fmaf(q.wy, sy, q.wz * sz);
}

template <int DIM, bool UNIT>
__global__ void __launch_bounds__(kC64Z * kC64Y)
chf_noise_mu(const float* __restrict__ cin, float* __restrict__ mu, Geom g, C32 q, P<float> p, int planes)
{
    const int z = blockIdx.x * kC64Z + threadIdx.x;
    const int y = blockIdx.y * kC64Y + threadIdx.y;
    if (z >= g.Z || y >= g.Y) return;   // no barrier in this kernel
    const int zl = z == 0 ? g.Z - 1 : z - 1, zh = z + 1 == g.Z ? 0 : z + 1;
    const long long row = (long long)y * g.Z;
    const long long rl = (long long)(y == 0 ? g.Y - 1 : y - 1) * g.Z;
    const long long rh = (long long)(y + 1 == g.Y ? 0 : y + 1) * g.Z;
    const int xs = blockIdx.z * planes;
    const int xe = min(xs + planes, g.X);
    auto plane = [&](int x) { return cin + (long long)x * g.YZ; };
    float a = 0.0f, b = __ldg(plane(xs) + row + z);
    if (DIM == 3) a = __ldg(plane(xs == 0 ? g.X - 1 : xs - 1) + row + z);
    for (int x = xs; x < xe; x++) {
        const float* pc = plane(x);
        float n = 0.0f;
        if (DIM == 3) n = __ldg(plane(x + 1 == g.X ? 0 : x + 1) + row + z);
        const float s = nsum_f<DIM, UNIT>(n + a, __ldg(pc + rh + z) + __ldg(pc + rl + z),
                                          __ldg(pc + row + zh) + __ldg(pc + row + zl), q);
        const long long i = (long long)x * g.YZ + row + z;
        const float m = fmaf(-q.kappa, s, fmaf(q.u, b * b, q.poly0) * b);
        mu[i] = m + noise_at(p, g.cells, i);
        a = b;
        b = n;
    }
}

template <int DIM, bool UNIT>
__global__ void __launch_bounds__(kC64Z * kC64Y)
chf_update(const float* __restrict__ cin, const float* __restrict__ mu, float* __restrict__ cout, Geom g, C32 q,
           int planes)
{
    const int z = blockIdx.x * kC64Z + threadIdx.x;
    const int y = blockIdx.y * kC64Y + threadIdx.y;
    if (z >= g.Z || y >= g.Y) return;
    const int zl = z == 0 ? g.Z - 1 : z - 1, zh = z + 1 == g.Z ? 0 : z + 1;
    const long long row = (long long)y * g.Z;
    const long long rl = (long long)(y == 0 ? g.Y - 1 : y - 1) * g.Z;
    const long long rh = (long long)(y + 1 == g.Y ? 0 : y + 1) * g.Z;
    const int xs = blockIdx.z * planes;
    const int xe = min(xs + planes, g.X);
    auto plane = [&](int x) { return mu + (long long)x * g.YZ; };
    float a = 0.0f, b = __ldg(plane(xs) + row + z);
    if (DIM == 3) a = __ldg(plane(xs == 0 ? g.X - 1 : xs - 1) + row + z);
    for (int x = xs; x < xe; x++) {
        const long long i = (long long)x * g.YZ + row + z;
        const float* pm = plane(x);
        float n = 0.0f;
        if (DIM == 3) n = __ldg(plane(x + 1 == g.X ? 0 : x + 1) + row + z);
        const float s = nsum_f<DIM, UNIT>(n + a, __ldg(pm + rh + z) + __ldg(pm + rl + z),
                                          __ldg(pm + row + zh) + __ldg(pm + row + zl), q);
        cout[i] = fmaf(q.dtm, s, fmaf(q.upd0, b, __ldg(cin + i)));
        a = b;
        b = n;
    }
}

bool ch64_eligible(const mmsp_gpu_desc& d, const Geom& g)
{
    // grid dimensions y and z of the launch stay within 65535 blocks
    const long long by = (g.Y + kC64Y - 1) / kC64Y;
    const long long bz = g.dim == 3 ? (g.X + kC64Planes - 1) / kC64Planes : 1;
    const bool fp64 = d.dtype == MMSP_GPU_F64 && (d.model == MMSP_GPU_CH || d.model == MMSP_GPU_CH_POLY);
    const bool noisy32 = d.dtype == MMSP_GPU_F32 && d.model == MMSP_GPU_CH_POLY && g.dim == 3 && noisy(d);
    return (fp64 || noisy32) && (g.dim == 2 || g.dim == 3) && by <= 65535 && bz <= 65535;
}

namespace {

// Kernel tables indexed by the template switches.
template <int DIM, int MODEL, bool UNIT, bool KONE, bool EXACT>
const void* mu_fn_n(bool noise)
{
    return noise ? reinterpret_cast<const void*>(&ch64_mu<DIM, MODEL, UNIT, KONE, EXACT, true>)
                 : reinterpret_cast<const void*>(&ch64_mu<DIM, MODEL, UNIT, KONE, EXACT, false>);
}
template <int DIM, int MODEL, bool UNIT, bool KONE>
const void* mu_fn_e(bool exact, bool noise)
{
    return exact ? mu_fn_n<DIM, MODEL, UNIT, KONE, true>(noise) : mu_fn_n<DIM, MODEL, UNIT, KONE, false>(noise);
}
template <int DIM, int MODEL, bool UNIT>
const void* mu_fn_k(bool kone, bool exact, bool noise)
{
    return kone ? mu_fn_e<DIM, MODEL, UNIT, true>(exact, noise) : mu_fn_e<DIM, MODEL, UNIT, false>(exact, noise);
}
template <int DIM, int MODEL>
const void* mu_fn_u(bool unit, bool kone, bool exact, bool noise)
{
    return unit ? mu_fn_k<DIM, MODEL, true>(kone, exact, noise) : mu_fn_k<DIM, MODEL, false>(kone, exact, noise);
}
template <int DIM>
const void* mu_fn_m(int model, bool unit, bool kone, bool exact, bool noise)
{
    return model == MMSP_GPU_CH ? mu_fn_u<DIM, MMSP_GPU_CH>(unit, kone, exact, noise)
                                : mu_fn_u<DIM, MMSP_GPU_CH_POLY>(unit, kone, exact, noise);
}
template <int DIM>
const void* upd_fn(bool unit, bool exact)
{
    if (unit) return exact ? reinterpret_cast<const void*>(&ch64_update<DIM, true, true>)
                           : reinterpret_cast<const void*>(&ch64_update<DIM, true, false>);
    return exact ? reinterpret_cast<const void*>(&ch64_update<DIM, false, true>)
                 : reinterpret_cast<const void*>(&ch64_update<DIM, false, false>);
}

C64 c64_of(const Coeffs& c, int dim)
{
    const P<double> p = narrow<double>(c, dim);
    C64 q;
    q.wx = p.wx;
    q.wy = p.wy;
    q.wz = p.wz;
    q.kappa = c.kappa;
    q.dtm = c.dtm;
    q.neg_r = c.neg_r;
    q.u = c.u;
    q.w2 = 2.0 * (dim == 3 ? p.wx + p.wy + p.wz : p.wy + p.wz);
    q.poly0 = 0.0;   // set by the launcher per model
    q.upd0 = -c.dtm * q.w2;
    q.noise = c.noise;
    q.seed = c.seed;
    q.step = c.step;
    return q;
}

}  // namespace

// The mu kernel goes in p->fn, the update kernel in p->fn2.
cudaError_t plan_ch64(const mmsp_gpu_desc& d, const Geom& g, StepPlan* p)
{
    const Coeffs c = make_coeffs(d);
    const bool exact = !(d.flags & MMSP_GPU_FLAG_CONTRACT);
    const bool kone = c.kappa == 1.0;
    const bool noise = noisy(d);
    if (d.dtype == MMSP_GPU_F32) {   // the noisy FP32 form, 3D only (ch64_eligible)
        p->fn = c.unit_w ? (const void*)&chf_noise_mu<3, true> : (const void*)&chf_noise_mu<3, false>;
        p->fn2 = c.unit_w ? (const void*)&chf_update<3, true> : (const void*)&chf_update<3, false>;
    } else {
        p->fn = g.dim == 3 ? mu_fn_m<3>(d.model, c.unit_w, kone, exact, noise)
                           : mu_fn_m<2>(d.model, c.unit_w, kone, exact, noise);
        p->fn2 = g.dim == 3 ? upd_fn<3>(c.unit_w, exact) : upd_fn<2>(c.unit_w, exact);
    }
    p->block = dim3(kC64Z, kC64Y, 1);
    p->planes = g.dim == 3 ? kC64Planes : 1;
    const int segs = (g.X + p->planes - 1) / p->planes;
    p->grid = dim3((g.Z + kC64Z - 1) / kC64Z, (g.Y + kC64Y - 1) / kC64Y, segs);
    p->smem = 0;
    p->fields = 1;
    p->kind = 6;
    p->ring = 0;
    p->ok = true;
    return cudaSuccess;
}

cudaError_t launch_ch64(const StepPlan& p, const mmsp_gpu_desc& d, const Geom& g, const Coeffs& c, const void* in,
                        void* out, void* work, int* err, cudaStream_t s)
{
    C64 q = c64_of(c, g.dim);
    q.poly0 = (d.model == MMSP_GPU_CH ? 2.0 : c.neg_r) + c.kappa * q.w2;
    int planes = p.planes;
    if (d.dtype == MMSP_GPU_F32) {
        C32 f;
        f.wx = (float)q.wx;
        f.wy = (float)q.wy;
        f.wz = (float)q.wz;
        f.kappa = (float)q.kappa;
        f.u = (float)q.u;
        f.dtm = (float)q.dtm;
        f.poly0 = (float)q.poly0;
        f.upd0 = (float)q.upd0;
        P<float> pf = narrow<float>(c, g.dim);
        pf.stepp = step_word(err);
        void* a1[] = {(void*)&in, (void*)&work, (void*)&g, (void*)&f, (void*)&pf, (void*)&planes};
        cudaError_t e = cudaLaunchKernel(p.fn, p.grid, p.block, a1, 0, s);
        if (e != cudaSuccess) return e;
        const void* mu = work;
        void* a2[] = {(void*)&in, (void*)&mu, (void*)&out, (void*)&g, (void*)&f, (void*)&planes};
        return cudaLaunchKernel(p.fn2, p.grid, p.block, a2, 0, s);
    }
    P<double> pp = narrow<double>(c, g.dim);
    if (noisy(d)) pp.stepp = step_word(err);
    void* a1[] = {(void*)&in, (void*)&work, (void*)&g, (void*)&q, (void*)&pp, (void*)&planes};
    cudaError_t e = cudaLaunchKernel(p.fn, p.grid, p.block, a1, 0, s);
    if (e != cudaSuccess) return e;
    const void* mu = work;
    void* a2[] = {(void*)&in, (void*)&mu, (void*)&out, (void*)&g, (void*)&q, (void*)&pp, (void*)&planes};
    return cudaLaunchKernel(p.fn2, p.grid, p.block, a2, 0, s);
}

}  // namespace pf
