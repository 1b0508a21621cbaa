// pf_ostwald.cu -- explicit Ostwald-ripening step, two kernels per step.
//
// The reference's update (examples/coarsening/ostwald_ripening/isotropic/
// phase_field/ostwald.cpp:84-122) makes two passes over the grid: the
// chemical potential of the composition C (field 0) into a scalar work grid
// (:89-100), ghostswap, then the new composition from the Laplacian of that
// grid and the new order parameters (fields 1..N-1) from their own
// Laplacians (:103-120).  Here each pass is one kernel over all cells (a
// thread walks a (y, z) column plane by plane, so a cell's coordinates need
// no division and its neighbour offsets are fixed per column), the work
// grid is a device buffer of the handle, and the periodic halo is index
// arithmetic.  Neighbour values come through the L1/L2 caches.
//
// FP64 follows the reference's operation order with separately rounded
// operations (pow(x,3) as the compensated cube of pf_device.cuh, pow(x,2)
// as x*x); FP32 uses the same expressions in float.
#include <stdlib.h>

#include "pf_device.cuh"
#include "pf_internal.h"

namespace pf {

template <typename T> struct OstP {
    T wx, wy, wz;
    T Cm, Ca, Cb, negA, B, Da, Db, g, neg_g, delta, eps, kappa, dtD, dtL;
};

template <typename T>
static OstP<T> ost_narrow(const Coeffs& c, int dim)
{
    const P<T> w = narrow<T>(c, dim);
    const OstConst& o = c.ost;
    OstP<T> p;
    p.wx = w.wx;
    p.wy = w.wy;
    p.wz = w.wz;
    p.Cm = (T)o.Cm;
    p.Ca = (T)o.Ca;
    p.Cb = (T)o.Cb;
    p.negA = (T)(-o.A);
    p.B = (T)o.B;
    p.Da = (T)o.Da;
    p.Db = (T)o.Db;
    p.g = (T)o.g;
    p.neg_g = (T)(-o.g);
    p.delta = (T)o.delta;
    p.eps = (T)o.eps;
    p.kappa = (T)o.kappa;
    p.dtD = (T)o.dtD;
    p.dtL = (T)o.dtL;
    return p;
}

// A thread owns one (y, z) column of the padded axes X, Y, Z and walks it
// plane by plane.  In-plane offsets are 32-bit (a plane holds fewer than
// 2^31 cells) and fixed per column, the plane pointers advance once per
// plane, and the values of the planes either side along X roll through
// registers, so each Laplacian reads 5 values per cell instead of 7.
struct Col {
    int o, yh, yl, zh, zl;   // offsets in a plane: the cell and its four in-plane neighbours
};

static __device__ __forceinline__ Col column_of(const Geom& g, int y, int z)
{
    Col c;
    const int ry = y * g.Z;
    c.o = ry + z;
    c.yh = (y + 1 == g.Y ? 0 : y + 1) * g.Z + z;
    c.yl = (y == 0 ? g.Y - 1 : y - 1) * g.Z + z;
    c.zh = ry + (z + 1 == g.Z ? 0 : z + 1);
    c.zl = ry + (z == 0 ? g.Z - 1 : z - 1);
    return c;
}

// The Laplacian at plane pointer pc from the rolled X neighbours xh, xl
// (the reference's operand order: lap_ref).
template <typename T, int DIM, bool UNIT>
static __device__ __forceinline__ T lap_col(const T* __restrict__ pc, T c, T xh, T xl, const Col& k, const OstP<T>& p)
{
    return lap_ref<T, UNIT, DIM>(twice(c), xh, xl, __ldg(pc + k.yh), __ldg(pc + k.yl), __ldg(pc + k.zh),
                                 __ldg(pc + k.zl), p.wx, p.wy, p.wz);
}

// sum_{j>=1} pow(e_j,2), ostwald.cpp:91-93 (0.0 + x == x for x >= 0), at
// offset o of plane offset xo.  NF: the field count when it is a
// compile-time constant (loops unroll), 0 when it is taken from N.
template <typename T, int NF>
static __device__ __forceinline__ T order_sum(const T* __restrict__ s, long long xo, int o, long long cells, int N)
{
    using A = Ar<T>;
    const int n = NF ? NF : N;
    T sum = T(0);
#pragma unroll(NF ? NF : 1)
    for (int j = 1; j < (NF ? NF : 64); j++) {
        if (!NF && j >= n) break;
        const T e = __ldg(s + (long long)j * cells + xo + o);
        sum = j == 1 ? A::mul(e, e) : A::add(sum, A::mul(e, e));
    }
    return sum;
}

// Both passes run on (y, z) columns: a block of kOstZ x kOstY threads over a
// run of kOstPlanes X planes (coalesced rows, no per-cell division).
constexpr int kOstZ = 32, kOstY = 4, kOstPlanes = 8;

// Pass 1, ostwald.cpp:95-99:
//   w = -A*(C-Cm) + B*pow(C-Cm,3) + Da*pow(C-Ca,3) + Db*pow(C-Cb,3) - g*(C-Ca)*sum - kappa*lap C
template <typename T, int DIM, bool UNIT, int NF>
__global__ void __launch_bounds__(kOstZ * kOstY)
ostwald_mu(const T* __restrict__ s, T* __restrict__ w, Geom g, OstP<T> p, int N)
{
    using A = Ar<T>;
    const int z = blockIdx.x * kOstZ + threadIdx.x;
    const int y = blockIdx.y * kOstY + threadIdx.y;
    if (z >= g.Z || y >= g.Y) return;
    const Col k = column_of(g, y, z);
    const int xs = blockIdx.z * kOstPlanes, xe = min(xs + kOstPlanes, g.X);
    const long long YZ = g.YZ;
    const T* pc = s + (long long)xs * YZ;
    T cl = __ldg(s + (long long)(xs == 0 ? g.X - 1 : xs - 1) * YZ + k.o);   // C(x-1)
    T cc = __ldg(pc + k.o);                                                  // C(x)
    for (int x = xs; x < xe; x++) {
        const T* ph = s + (long long)(x + 1 == g.X ? 0 : x + 1) * YZ;
        const T ch = __ldg(ph + k.o);
        const long long xo = (long long)x * YZ;
        const T sum = order_sum<T, NF>(s, xo, k.o, g.cells, N);
        const T C = cc;
        const T lap = lap_col<T, DIM, UNIT>(pc, cc, ch, cl, k, p);
        const T dm = A::sub(C, p.Cm), da = A::sub(C, p.Ca), db = A::sub(C, p.Cb);
        T v = A::mul(p.negA, dm);
        v = A::add(v, A::mul(p.B, cube(dm)));
        v = A::add(v, A::mul(p.Da, cube(da)));
        v = A::add(v, A::mul(p.Db, cube(db)));
        v = A::sub(v, A::mul(A::mul(p.g, da), sum));
        w[xo + k.o] = A::sub(v, kappa_times(p.kappa, lap));
        cl = cc;
        cc = ch;
        pc = ph;
    }
}

// Pass 2, ostwald.cpp:103-120:
//   C'   = C + dt*D*lap w
//   e_j' = e_j - dt*L*(-g*pow(C-Ca,2) + delta*pow(e_j,3) + eps*e_j*(sum - pow(e_j,2)) - kappa*lap e_j)
// The work grid and, for a compile-time field count, every order parameter
// roll their X neighbours through registers.
template <typename T, int DIM, bool UNIT, int NF>
__global__ void __launch_bounds__(kOstZ * kOstY)
ostwald_update(const T* __restrict__ s, const T* __restrict__ w, T* __restrict__ out, Geom g, OstP<T> p, int N)
{
    using A = Ar<T>;
    constexpr int NE = NF ? NF - 1 : 1;   // order parameters rolled (none when NF is 0)
    const int z = blockIdx.x * kOstZ + threadIdx.x;
    const int y = blockIdx.y * kOstY + threadIdx.y;
    if (z >= g.Z || y >= g.Y) return;
    const Col k = column_of(g, y, z);
    const int xs = blockIdx.z * kOstPlanes, xe = min(xs + kOstPlanes, g.X);
    const long long YZ = g.YZ, cells = g.cells;
    const long long xlo = (long long)(xs == 0 ? g.X - 1 : xs - 1) * YZ;
    const T* wc_p = w + (long long)xs * YZ;
    T wl = __ldg(w + xlo + k.o), wc = __ldg(wc_p + k.o);
    T el[NE], ec[NE];
    if (NF) {
#pragma unroll
        for (int j = 0; j < NE; j++) {
            el[j] = __ldg(s + (long long)(j + 1) * cells + xlo + k.o);
            ec[j] = __ldg(s + (long long)(j + 1) * cells + (long long)xs * YZ + k.o);
        }
    }
    for (int x = xs; x < xe; x++) {
        const long long xo = (long long)x * YZ;
        const long long xho = (long long)(x + 1 == g.X ? 0 : x + 1) * YZ;
        const T wh = __ldg(w + xho + k.o);
        const T C = __ldg(s + xo + k.o);
        out[xo + k.o] = A::add(C, A::mul(p.dtD, lap_col<T, DIM, UNIT>(wc_p, wc, wh, wl, k, p)));
        const T sum = order_sum<T, NF>(s, xo, k.o, cells, N);
        const T da = A::sub(C, p.Ca);
        const T t1 = A::mul(p.neg_g, A::mul(da, da));
        if (NF) {
#pragma unroll
            for (int j = 0; j < NE; j++) {
                const T* f = s + (long long)(j + 1) * cells;
                const T e = ec[j];
                const T eh = __ldg(f + xho + k.o);
                T v = A::add(t1, A::mul(p.delta, cube(e)));
                v = A::add(v, A::mul(A::mul(p.eps, e), A::sub(sum, A::mul(e, e))));
                v = A::sub(v, kappa_times(p.kappa, lap_col<T, DIM, UNIT>(f + xo, e, eh, el[j], k, p)));
                out[(long long)(j + 1) * cells + xo + k.o] = A::sub(e, A::mul(p.dtL, v));
                el[j] = e;
                ec[j] = eh;
            }
        } else {
            const long long xlo2 = (long long)(x == 0 ? g.X - 1 : x - 1) * YZ;
            for (int j = 1; j < N; j++) {
                const T* f = s + (long long)j * cells;
                const T e = __ldg(f + xo + k.o);
                T v = A::add(t1, A::mul(p.delta, cube(e)));
                v = A::add(v, A::mul(A::mul(p.eps, e), A::sub(sum, A::mul(e, e))));
                v = A::sub(v, kappa_times(p.kappa, lap_col<T, DIM, UNIT>(f + xo, e, __ldg(f + xho + k.o),
                                                                        __ldg(f + xlo2 + k.o), k, p)));
                out[(long long)j * cells + xo + k.o] = A::sub(e, A::mul(p.dtL, v));
            }
        }
        wl = wc;
        wc = wh;
        wc_p = w + xho;
    }
}

template <typename T, int DIM, bool UNIT, int NF>
static void ost_fns(const void** mu, const void** up)
{
    *mu = (const void*)&ostwald_mu<T, DIM, UNIT, NF>;
    *up = (const void*)&ostwald_update<T, DIM, UNIT, NF>;
}

template <typename T, int DIM, bool UNIT>
static void ost_pick_n(int N, const void** mu, const void** up)
{
    if (N == 2) ost_fns<T, DIM, UNIT, 2>(mu, up);
    else if (N == 3) ost_fns<T, DIM, UNIT, 3>(mu, up);
    else if (N == 4) ost_fns<T, DIM, UNIT, 4>(mu, up);
    else ost_fns<T, DIM, UNIT, 0>(mu, up);
}

template <typename T>
static void ost_pick(int dim, bool unit, int N, const void** mu, const void** up)
{
    if (dim == 3) unit ? ost_pick_n<T, 3, true>(N, mu, up) : ost_pick_n<T, 3, false>(N, mu, up);
    else if (dim == 2) unit ? ost_pick_n<T, 2, true>(N, mu, up) : ost_pick_n<T, 2, false>(N, mu, up);
    else unit ? ost_pick_n<T, 1, true>(N, mu, up) : ost_pick_n<T, 1, false>(N, mu, up);
}

cudaError_t plan_ostwald(const mmsp_gpu_desc& d, const Geom& g, StepPlan* p)
{
    const Coeffs c = make_coeffs(d);
    if (ost3_stream_eligible(d, g) && !getenv("MMSP_GPU_OST_TWO_KERNELS")) return plan_ost3_stream(d, g, c, p);
    const void* up = nullptr;
    if (d.dtype == MMSP_GPU_F64) ost_pick<double>(g.dim, c.unit_w, d.fields, &p->fn, &up);
    else ost_pick<float>(g.dim, c.unit_w, d.fields, &p->fn, &up);
    // (y, z) columns of kOstZ x kOstY threads over runs of kOstPlanes planes
    p->grid = dim3((g.Z + kOstZ - 1) / kOstZ, (g.Y + kOstY - 1) / kOstY, (g.X + kOstPlanes - 1) / kOstPlanes);
    p->block = dim3(kOstZ, kOstY, 1);
    if (p->grid.y > 65535 || p->grid.z > 65535) return cudaErrorInvalidConfiguration;
    p->smem = 0;
    p->planes = 1;
    p->fields = d.fields;
    p->kind = 4;
    p->ring = 0;
    p->ok = true;
    return cudaSuccess;
}

cudaError_t launch_ostwald(const StepPlan& p, const mmsp_gpu_desc& d, const Geom& g, const Coeffs& c,
                           const void* in, void* out, void* work, int* err, cudaStream_t s)
{
    if (p.kind == 8) return launch_ost3_stream(p, g, c.ost, c, in, out, err, s);
    const void* mu = nullptr;
    const void* up = nullptr;
    int n = d.fields;
    Geom gg = g;
    cudaError_t e;
    if (d.dtype == MMSP_GPU_F64) {
        ost_pick<double>(g.dim, c.unit_w, d.fields, &mu, &up);
        OstP<double> q = ost_narrow<double>(c, g.dim);
        void* a1[] = {(void*)&in, (void*)&work, (void*)&gg, (void*)&q, (void*)&n};
        if ((e = cudaLaunchKernel(mu, p.grid, p.block, a1, 0, s)) != cudaSuccess) return e;
        void* a2[] = {(void*)&in, (void*)&work, (void*)&out, (void*)&gg, (void*)&q, (void*)&n};
        return cudaLaunchKernel(up, p.grid, p.block, a2, 0, s);
    }
    ost_pick<float>(g.dim, c.unit_w, d.fields, &mu, &up);
    OstP<float> q = ost_narrow<float>(c, g.dim);
    void* a1[] = {(void*)&in, (void*)&work, (void*)&gg, (void*)&q, (void*)&n};
    if ((e = cudaLaunchKernel(mu, p.grid, p.block, a1, 0, s)) != cudaSuccess) return e;
    void* a2[] = {(void*)&in, (void*)&work, (void*)&out, (void*)&gg, (void*)&q, (void*)&n};
    return cudaLaunchKernel(up, p.grid, p.block, a2, 0, s);
}

}  // namespace pf
