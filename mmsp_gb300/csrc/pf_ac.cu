// pf_ac.cu -- explicit multi-order-parameter Allen-Cahn step.
//
// One pass per step as in graingrowth.cpp:91-107: per cell, the sum of
// squares over the N order parameters, then each field's new value from its
// own Laplacian.  The device layout is field-major (SoA, [field][x][y][z])
// instead of the reference's array of per-cell heap vectors, so every field
// is a contiguous, coalesced stream.  Shared memory holds the tile plus a
// halo of 1 for all N fields; 3D grids stream along axis X with a ring of 4
// planes (one barrier per plane).  Periodic wrap is index arithmetic, as in
// the Cahn-Hilliard kernel.
#include "pf_device.cuh"
#include "pf_internal.h"

namespace pf {

constexpr int kTZ = 32;
constexpr int kThreadsY = 8;

template <int TY>
struct AcTile {
    static constexpr int CW = kTZ + 2, CH = TY + 2, CP = CW * CH;
    static size_t smem(int dim, int fields, size_t esize)
    {
        int nc = dim == 3 ? 4 : 1;
        return esize * (size_t)nc * fields * CP + sizeof(int) * (CH + CW);
    }
};

template <typename T, int DIM, int MODEL, int TY, bool UNIT_W>
__global__ void __launch_bounds__(256)
ac_step_kernel(const T* __restrict__ ein, T* __restrict__ eout, Geom g, P<T> p, int planes, int N)
{
    using A = Ar<T>;
    using TL = AcTile<TY>;
    constexpr int CW = TL::CW, CH = TL::CH, CP = TL::CP;
    constexpr int NC = DIM == 3 ? 4 : 1;

    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* es = reinterpret_cast<T*>(smem_raw);   // [slot][field][CP]
    int* yoff = reinterpret_cast<int*>(es + (size_t)NC * N * CP);
    int* zoff = yoff + CH;

    const int tid = threadIdx.x + threadIdx.y * kTZ;
    const int z0 = blockIdx.x * kTZ;
    const int y0 = blockIdx.y * TY;
    for (int i = tid; i < CH; i += 256) yoff[i] = wrapi(y0 - 1 + i, g.Y) * g.Z;
    for (int i = tid; i < CW; i += 256) zoff[i] = wrapi(z0 - 1 + i, g.Z);
    __syncthreads();

    const long long cells = g.cells;
    auto load = [&](int slot, int gx) {
        const T* src = ein + (long long)wrapi(gx, g.X) * g.YZ;
        T* dst = es + (size_t)slot * N * CP;
        const int total = N * CP;
        for (int e = tid; e < total; e += 256) {
            int f = e / CP, r = e - f * CP;
            int ly = r / CW, lz = r - ly * CW;
            dst[e] = __ldg(src + f * cells + yoff[ly] + zoff[lz]);
        }
    };
    auto out_plane = [&](int gx, int sl, int sc, int sh) {
        const int lz = threadIdx.x, gz = z0 + lz;
        if (gz >= g.Z) return;
        const T* L = es + (size_t)sl * N * CP;
        const T* C = es + (size_t)sc * N * CP;
        const T* H = es + (size_t)sh * N * CP;
        for (int ly = threadIdx.y; ly < TY; ly += kThreadsY) {
            int gy = y0 + ly;
            if (gy >= g.Y) break;
            int ci = (ly + 1) * CW + (lz + 1);
            // sum of squares in field order (graingrowth.cpp:98-101); 0.0 + p0^2 == p0^2
            T sum = A::mul(C[ci], C[ci]);
            for (int f = 1; f < N; f++) sum = A::add(sum, A::mul(C[f * CP + ci], C[f * CP + ci]));
            T* dst = eout + (long long)gx * g.YZ + (long long)gy * g.Z + gz;
            for (int f = 0; f < N; f++) {
                const int o = f * CP + ci;
                T y = C[o];
                T y2 = twice(y);
                T lap = lap_ref<T, UNIT_W, DIM>(y2, H[o], L[o], C[o + CW], C[o - CW], C[o + 1], C[o - 1], p.wx, p.wy,
                                                p.wz);
                if (MODEL == MMSP_GPU_AC_POLY && p.noise != 0.0) {
                    // model_A.cpp:99-100: p - dt*M*(-r p + u pow(p,3) - K lap + noise)
                    T e = A::sub(A::add(A::mul(p.neg_r, y), A::mul(p.u, cube(y))), kappa_times(p.kappa, lap));
                    e = A::add(e, noise_at(p, cells, (long long)gx * g.YZ + (long long)gy * g.Z + gz));
                    dst[f * cells] = A::sub(y, A::mul(p.dtm, e));
                    continue;
                }
                // Zener pinning: the particles (field 0) have zero mobility (zener.cpp:134)
                dst[f * cells] = (MODEL == MMSP_GPU_ZENER && f == 0) ? y : ac_new<T, MODEL>(y, sum, lap, p);
            }
        }
    };

    if (DIM < 3) {
        load(0, 0);
        __syncthreads();
        out_plane(0, 0, 0, 0);
        return;
    }
    const int xs = blockIdx.z * planes;
    const int xe = min(xs + planes, g.X);
    if (xs >= xe) return;
    auto sl = [&](int x) { return (x - xs + 1) & 3; };
    load(sl(xs - 1), xs - 1);
    load(sl(xs), xs);
    for (int x = xs; x < xe; x++) {
        load(sl(x + 1), x + 1);  // overwrites plane x-3, last read before the previous barrier
        __syncthreads();
        out_plane(x, sl(x - 1), sl(x), sl(x + 1));
    }
}

template <typename T, int DIM, int MODEL, int TY>
static const void* ac_pick_w(bool unit)
{
    return unit ? reinterpret_cast<const void*>(&ac_step_kernel<T, DIM, MODEL, TY, true>)
                : reinterpret_cast<const void*>(&ac_step_kernel<T, DIM, MODEL, TY, false>);
}

template <typename T, int DIM, int MODEL>
static const void* ac_pick_ty(int ty, bool unit)
{
    return ty == 8 ? ac_pick_w<T, DIM, MODEL, 8>(unit) : ac_pick_w<T, DIM, MODEL, 4>(unit);
}

template <typename T, int DIM>
static const void* ac_pick_model(int model, int ty, bool unit)
{
    if (model == MMSP_GPU_AC) return ac_pick_ty<T, DIM, MMSP_GPU_AC>(ty, unit);
    if (model == MMSP_GPU_GG) return ac_pick_ty<T, DIM, MMSP_GPU_GG>(ty, unit);
    if (model == MMSP_GPU_ZENER) return ac_pick_ty<T, DIM, MMSP_GPU_ZENER>(ty, unit);
    return ac_pick_ty<T, DIM, MMSP_GPU_AC_POLY>(ty, unit);
}

template <typename T>
static const void* ac_pick(int dim, int model, int ty, bool unit)
{
    if (dim == 3) return ac_pick_model<T, 3>(model, ty, unit);
    if (dim == 2) return ac_pick_model<T, 2>(model, ty, unit);
    return ac_pick_model<T, 1>(model, ty, unit);
}

cudaError_t plan_ac(const mmsp_gpu_desc& d, const Geom& g, StepPlan* p)
{
    // the stochastic form takes the tile kernel, which adds the noise term
    if (!noisy(d) && ac3_stream_eligible(d, g)) return plan_ac3_stream(d, g, p);
    Coeffs c = make_coeffs(d);
    bool dbl = d.dtype == MMSP_GPU_F64;
    size_t es = dbl ? sizeof(double) : sizeof(float);
    int ty = 8;
    if (AcTile<8>::smem(g.dim, d.fields, es) > 200 * 1024 || g.Y < 8) ty = 4;
    p->smem = ty == 8 ? AcTile<8>::smem(g.dim, d.fields, es) : AcTile<4>::smem(g.dim, d.fields, es);
    if (p->smem > 227 * 1024) {
        p->ok = false;
        return cudaErrorInvalidValue;
    }
    p->fn = dbl ? ac_pick<double>(g.dim, d.model, ty, c.unit_w) : ac_pick<float>(g.dim, d.model, ty, c.unit_w);
    p->block = dim3(kTZ, kThreadsY, 1);
    cudaError_t e = ensure_smem(p->fn, p->smem);
    if (e != cudaSuccess) return e;
    int tz = (g.Z + kTZ - 1) / kTZ, tyn = (g.Y + ty - 1) / ty;
    int segs = 1;
    p->planes = 1;
    if (g.dim == 3) {
        int per_sm = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, p->fn, 256, p->smem);
        if (e != cudaSuccess) return e;
        if (per_sm < 1) per_sm = 1;
        long long want = (long long)sm_count() * per_sm;
        long long cols = (long long)tz * tyn;
        segs = (int)((want + cols - 1) / cols);
        int maxseg = (g.X + 7) / 8;
        if (segs > maxseg) segs = maxseg;
        if (segs < 1) segs = 1;
        p->planes = (g.X + segs - 1) / segs;
        segs = (g.X + p->planes - 1) / p->planes;
    }
    p->grid = dim3(tz, tyn, segs);
    p->fields = d.fields;
    p->kind = 0;
    p->ok = true;
    return cudaSuccess;
}

cudaError_t launch_ac(const StepPlan& p, const mmsp_gpu_desc& d, const Geom& g, const Coeffs& c,
                      const void* in, void* out, int* err, cudaStream_t s)
{
    if (p.kind == 2) return launch_ac3_stream(p, g, c, in, out, err, s);
    int planes = p.planes, n = d.fields;
    if (d.dtype == MMSP_GPU_F64) {
        P<double> q = narrow<double>(c, g.dim);
        if (noisy(d)) q.stepp = step_word(err);
        void* args[] = {(void*)&in, (void*)&out, (void*)&g, (void*)&q, (void*)&planes, (void*)&n};
        return cudaLaunchKernel(p.fn, p.grid, p.block, args, p.smem, s);
    } else {
        P<float> q = narrow<float>(c, g.dim);
        if (noisy(d)) q.stepp = step_word(err);
        void* args[] = {(void*)&in, (void*)&out, (void*)&g, (void*)&q, (void*)&planes, (void*)&n};
        return cudaLaunchKernel(p.fn, p.grid, p.block, args, p.smem, s);
    }
}

}  // namespace pf
