// pf_ch.cu -- explicit Cahn-Hilliard step, fused into one kernel per step.
//
// The reference runs two node loops per step (cahn-hilliard.cpp:69-76):
// temp = mu(c) over every node, ghostswap(temp), then c' = c + dt*M*lap(temp).
// Here one kernel does both on a shared-memory tile: c is staged with a
// halo of 2, mu is evaluated on the tile plus a halo of 1 (so every mu the
// update reads is computed in the block), and the update is written out.
// Each mu value is computed with the same operations as the reference's
// pass 1, so recomputing it in two neighbouring blocks changes no bit.
//
// 3D grids stream along axis X (the slowest, plane-contiguous axis): a
// block owns a TY x TZ column of the (Y, Z) plane and a run of X planes,
// and keeps a ring of 4 c planes and 3 mu planes in shared memory, so each
// plane is read from global memory once per block instead of once per
// 7-point stencil.  2D and 1D grids are a single plane.
//
// Periodic halos (ghostswap + check_boundary) are index arithmetic: the
// per-block tables yoff/zoff hold the wrapped row offsets and columns of
// the staged tile.
#include "pf_device.cuh"
#include "pf_internal.h"

namespace pf {

constexpr int kTZ = 32;       // tile width along Z = one warp
constexpr int kThreadsY = 8;  // 32 x 8 = 256 threads

template <typename T, int TY>
struct ChTile {
    static constexpr int CW = kTZ + 4, CH = TY + 4, CP = CW * CH;   // c with halo 2
    static constexpr int MW = kTZ + 2, MH = TY + 2, MP = MW * MH;   // mu with halo 1
    static size_t smem(int dim)
    {
        int nc = dim == 3 ? 4 : 1, nm = dim == 3 ? 3 : 1;
        return sizeof(T) * (size_t)(nc * CP + nm * MP) + sizeof(int) * (CH + CW);
    }
};

template <typename T, int DIM, int MODEL, int TY, bool UNIT_W>
__global__ void __launch_bounds__(256)
ch_step_kernel(const T* __restrict__ cin, T* __restrict__ cout, Geom g, P<T> p, int planes)
{
    using A = Ar<T>;
    using TL = ChTile<T, TY>;
    constexpr int CW = TL::CW, CH = TL::CH, CP = TL::CP, MW = TL::MW, MP = TL::MP;
    constexpr int NC = DIM == 3 ? 4 : 1, NM = DIM == 3 ? 3 : 1;

    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* cs = reinterpret_cast<T*>(smem_raw);
    T* ms = cs + NC * CP;
    int* yoff = reinterpret_cast<int*>(ms + NM * MP);
    int* zoff = yoff + CH;

    const int tid = threadIdx.x + threadIdx.y * kTZ;
    const int z0 = blockIdx.x * kTZ;
    const int y0 = blockIdx.y * TY;
    for (int i = tid; i < CH; i += 256) yoff[i] = wrapi(y0 - 2 + i, g.Y) * g.Z;
    for (int i = tid; i < CW; i += 256) zoff[i] = wrapi(z0 - 2 + i, g.Z);
    __syncthreads();

    auto load = [&](int slot, int gx) {
        const T* src = cin + (long long)wrapi(gx, g.X) * g.YZ;
        T* dst = cs + slot * CP;
        for (int e = tid; e < CP; e += 256) {
            int ly = e / CW, lz = e - ly * CW;
            dst[e] = __ldg(src + yoff[ly] + zoff[lz]);
        }
    };
    // mu on the (TY+2) x (TZ+2) plane from c planes below / at / above it
    auto mu_plane = [&](int mslot, int cl, int cc, int chh, int gx) {
        const long long pbase = (long long)wrapi(gx, g.X) * g.YZ;
        const T* C = cs + cc * CP;
        const T* L = cs + cl * CP;
        const T* H = cs + chh * CP;
        T* M = ms + mslot * MP;
        for (int e = tid; e < MP; e += 256) {
            int my = e / MW, mz = e - my * MW;
            int ci = (my + 1) * CW + (mz + 1);
            T y = C[ci];
            T y2 = twice(y);
            T lap = lap_ref<T, UNIT_W, DIM>(y2, H[ci], L[ci], C[ci + CW], C[ci - CW], C[ci + 1], C[ci - 1], p.wx,
                                            p.wy, p.wz);
            T mu = ch_mu<T, MODEL>(y, lap, p);
            // thermal noise of the stochastic forms (model_B.cpp:100-101, spinodal.cpp:95-97): mu + noise
            if (p.noise != 0.0) mu = A::add(mu, noise_at(p, g.cells, pbase + yoff[my + 1] + zoff[mz + 1]));
            M[e] = mu;
        }
    };
    // c' = c + dt*M*lap(mu) on the TY x TZ tile of plane gx
    auto out_plane = [&](int gx, int cc, int ml, int mc, int mh) {
        const T* M = ms + mc * MP;
        const T* ML = ms + ml * MP;
        const T* MH = ms + mh * MP;
        const T* C = cs + cc * CP;
        const int lz = threadIdx.x, gz = z0 + lz;
        if (gz >= g.Z) return;
        for (int ly = threadIdx.y; ly < TY; ly += kThreadsY) {
            int gy = y0 + ly;
            if (gy >= g.Y) break;
            int mi = (ly + 1) * MW + (lz + 1);
            T y = M[mi];
            T y2 = twice(y);
            T lap = lap_ref<T, UNIT_W, DIM>(y2, MH[mi], ML[mi], M[mi + MW], M[mi - MW], M[mi + 1], M[mi - 1], p.wx,
                                            p.wy, p.wz);
            T c = C[(ly + 2) * CW + (lz + 2)];
            cout[(long long)gx * g.YZ + (long long)gy * g.Z + gz] = A::add(c, A::mul(p.dtm, lap));
        }
    };

    if (DIM < 3) {
        load(0, 0);
        __syncthreads();
        mu_plane(0, 0, 0, 0, 0);
        __syncthreads();
        out_plane(0, 0, 0, 0, 0);
        return;
    }

    const int xs = blockIdx.z * planes;
    const int xe = min(xs + planes, g.X);
    if (xs >= xe) return;
    // ring slots: c plane x -> (x - xs + 2) & 3, mu plane x -> (x - xs + 1) % 3
    auto csl = [&](int x) { return (x - xs + 2) & 3; };
    auto msl = [&](int x) { return (x - xs + 1) % 3; };
    for (int x = xs - 2; x <= xs + 1; x++) load(csl(x), x);
    __syncthreads();
    mu_plane(msl(xs - 1), csl(xs - 2), csl(xs - 1), csl(xs), xs - 1);
    mu_plane(msl(xs), csl(xs - 1), csl(xs), csl(xs + 1), xs);
    __syncthreads();
    for (int x = xs; x < xe; x++) {
        load(csl(x + 2), x + 2);  // overwrites c(x-2): its last readers were before the previous syncs
        __syncthreads();
        mu_plane(msl(x + 1), csl(x), csl(x + 1), csl(x + 2), x + 1);
        __syncthreads();
        out_plane(x, csl(x), msl(x - 1), msl(x), msl(x + 1));
    }
}

template <typename T, int DIM, int MODEL, int TY, bool UNIT_W>
static const void* ch_fn()
{
    return reinterpret_cast<const void*>(&ch_step_kernel<T, DIM, MODEL, TY, UNIT_W>);
}

template <typename T, int DIM, int MODEL, int TY>
static const void* ch_pick_w(bool unit) { return unit ? ch_fn<T, DIM, MODEL, TY, true>() : ch_fn<T, DIM, MODEL, TY, false>(); }

template <typename T, int DIM, int MODEL>
static const void* ch_pick_ty(int ty, bool unit)
{
    return ty == 16 ? ch_pick_w<T, DIM, MODEL, 16>(unit) : ch_pick_w<T, DIM, MODEL, 8>(unit);
}

template <typename T, int DIM>
static const void* ch_pick_model(int model, int ty, bool unit)
{
    return model == MMSP_GPU_CH ? ch_pick_ty<T, DIM, MMSP_GPU_CH>(ty, unit)
                                : ch_pick_ty<T, DIM, MMSP_GPU_CH_POLY>(ty, unit);
}

template <typename T>
static const void* ch_pick(int dim, int model, int ty, bool unit)
{
    if (dim == 3) return ch_pick_model<T, 3>(model, ty, unit);
    if (dim == 2) return ch_pick_model<T, 2>(model, ty, unit);
    return ch_pick_model<T, 1>(model, ty, unit);
}

cudaError_t plan_ch(const mmsp_gpu_desc& d, const Geom& g, StepPlan* p)
{
    // the stochastic forms take the rows kernel in 3D and the tile kernel
    // otherwise (a 2D rows block holds a whole row: 1024-thread blocks leave
    // the noise arithmetic short of warps), both of which add the noise term
    if (!noisy(d) && ch3_stream_eligible(d, g)) return plan_ch3_stream(d, g, p);
    if (ch_rows_eligible(d, g) && (!noisy(d) || g.dim == 3)) return plan_ch_rows(d, g, p);
    p->kind = 0;
    Coeffs c = make_coeffs(d);
    int ty = g.Y >= 16 ? 16 : 8;
    bool dbl = d.dtype == MMSP_GPU_F64;
    p->fn = dbl ? ch_pick<double>(g.dim, d.model, ty, c.unit_w) : ch_pick<float>(g.dim, d.model, ty, c.unit_w);
    p->smem = dbl ? (ty == 16 ? ChTile<double, 16>::smem(g.dim) : ChTile<double, 8>::smem(g.dim))
                  : (ty == 16 ? ChTile<float, 16>::smem(g.dim) : ChTile<float, 8>::smem(g.dim));
    p->block = dim3(kTZ, kThreadsY, 1);
    int tz = (g.Z + kTZ - 1) / kTZ, tyn = (g.Y + ty - 1) / ty;
    int segs = 1;
    p->planes = 1;
    if (g.dim == 3) {
        cudaError_t e = ensure_smem(p->fn, p->smem);
        if (e != cudaSuccess) return e;
        int per_sm = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, p->fn, 256, p->smem);
        if (e != cudaSuccess) return e;
        if (per_sm < 1) per_sm = 1;
        // Enough X segments to fill every SM, each at least 16 planes long so
        // the 4-plane warm-up of the ring stays a small share of the loads.
        long long want = (long long)sm_count() * per_sm;
        long long cols = (long long)tz * tyn;
        segs = (int)((want + cols - 1) / cols);
        int maxseg = (g.X + 15) / 16;
        if (segs > maxseg) segs = maxseg;
        if (segs < 1) segs = 1;
        p->planes = (g.X + segs - 1) / segs;
        segs = (g.X + p->planes - 1) / p->planes;
    } else {
        cudaError_t e = ensure_smem(p->fn, p->smem);
        if (e != cudaSuccess) return e;
    }
    p->grid = dim3(tz, tyn, segs);
    p->fields = 1;
    p->ok = true;
    return cudaSuccess;
}

cudaError_t launch_ch(const StepPlan& p, const mmsp_gpu_desc& d, const Geom& g, const Coeffs& c,
                      const void* in, void* out, int* err, cudaStream_t s)
{
    if (p.kind == 1) return launch_ch3_stream(p, g, c, in, out, err, s);
    if (p.kind == 3) return launch_ch_rows(p, d, c, in, out, err, s);
    int planes = p.planes;
    if (d.dtype == MMSP_GPU_F64) {
        P<double> q = narrow<double>(c, g.dim);
        if (noisy(d)) q.stepp = step_word(err);
        void* args[] = {(void*)&in, (void*)&out, (void*)&g, (void*)&q, (void*)&planes};
        return cudaLaunchKernel(p.fn, p.grid, p.block, args, p.smem, s);
    } else {
        P<float> q = narrow<float>(c, g.dim);
        if (noisy(d)) q.stepp = step_word(err);
        void* args[] = {(void*)&in, (void*)&out, (void*)&g, (void*)&q, (void*)&planes};
        return cudaLaunchKernel(p.fn, p.grid, p.block, args, p.smem, s);
    }
}

}  // namespace pf
