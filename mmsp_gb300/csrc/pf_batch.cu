// pf_batch.cu -- one persistent kernel advancing many 2D Cahn-Hilliard grids.
//
// The batched form: instances of uneven sizes and parameters live in one
// pool (per-instance offsets), and a single launch advances all of them by
// one explicit step.  The work list holds (instance, run of rows) items,
// largest first; warps take items from a global counter until none is left,
// so uneven instances balance across the whole GPU.
//
// A warp owns whole rows: lane l holds cells l*V .. l*V+V-1 of a row of
// n1 = 32*V cells, so the periodic Z neighbours of its first and last cell
// are one shuffle away (lane 0 wraps to lane 31) and no shared memory or
// block barrier is needed.  The warp streams down its run of rows (axis 0)
// keeping c for rows x, x+1, x+2 and mu for x-1, x, x+1 in registers, with
// the next row's load issued one row ahead.
//
// FP64 instances use the reference's operation order (bit-identical to the
// single-grid kernels and the oracle); FP32 instances use ordinary operators.
#include "pf_async.cuh"
#include "pf_batch.h"
#include "pf_device.cuh"

namespace pf {

template <typename T, int N>
static __device__ __forceinline__ void ld_row(T (&dst)[N], const T* __restrict__ src)
{
    if constexpr (sizeof(T) == 4 && N % 4 == 0) {
#pragma unroll
        for (int i = 0; i < N; i += 4) {
            const float4 v = __ldg(reinterpret_cast<const float4*>(src) + i / 4);
            dst[i] = v.x, dst[i + 1] = v.y, dst[i + 2] = v.z, dst[i + 3] = v.w;
        }
    } else if constexpr (N % 2 == 0) {
        using V2 = typename std::conditional<sizeof(T) == 4, float2, double2>::type;
#pragma unroll
        for (int i = 0; i < N; i += 2) {
            const V2 v = __ldg(reinterpret_cast<const V2*>(src) + i / 2);
            dst[i] = v.x, dst[i + 1] = v.y;
        }
    } else {
#pragma unroll
        for (int i = 0; i < N; i++) dst[i] = __ldg(src + i);
    }
}

template <typename T, int N>
static __device__ __forceinline__ void st_row(T* __restrict__ dst, const T (&v)[N])
{
    if constexpr (sizeof(T) == 4 && N % 4 == 0) {
#pragma unroll
        for (int i = 0; i < N; i += 4)
            reinterpret_cast<float4*>(dst)[i / 4] = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
    } else if constexpr (N % 2 == 0) {
        using V2 = typename std::conditional<sizeof(T) == 4, float2, double2>::type;
#pragma unroll
        for (int i = 0; i < N; i += 2) {
            V2 t;
            t.x = v[i];
            t.y = v[i + 1];
            reinterpret_cast<V2*>(dst)[i / 2] = t;
        }
    } else {
#pragma unroll
        for (int i = 0; i < N; i++) dst[i] = v[i];
    }
}

// 2D Laplacian at cell j of a lane's row segment, reference order: axis 0
// (rows) then axis 1 (cells of a row).
template <typename T, int V, bool UNIT>
static __device__ __forceinline__ T lap2(const T (&lo)[V], const T (&ce)[V], const T (&hi)[V], T left, T right,
                                         int j, T w0, T w1)
{
    using A = Ar<T>;
    const T y = ce[j];
    const T zl = j == 0 ? left : ce[j - 1];
    const T zh = j == V - 1 ? right : ce[j + 1];
    if constexpr (sizeof(T) == 4) {
        // precision form: neighbour sums, one multiply-add per axis
        if (UNIT) return fmaf(-4.0f, y, (hi[j] + lo[j]) + (zh + zl));
        return fmaf(w0, hi[j] + lo[j], fmaf(w1, zh + zl, -2.0f * (w0 + w1) * y));
    } else {
        const T y2 = twice(y);
        T lap = lap_axis<T, UNIT, true>(T(0), hi[j], y2, lo[j], w0);
        return lap_axis<T, UNIT>(lap, zh, y2, zl, w1);
    }
}

// mu of the Cahn-Hilliard models; Horner's form in the precision form.
template <typename T, int MODEL>
static __device__ __forceinline__ T mu2(T c, T lap, const P<T>& p)
{
    if constexpr (sizeof(T) == 4) {
        const float fp = MODEL == MMSP_GPU_CH ? c * fmaf(fmaf(4.0f, c, -6.0f), c, 2.0f) : c * fmaf(p.u, c * c, p.neg_r);
        return fmaf(-p.kappa, lap, fp);
    } else {
        return ch_mu<T, MODEL>(c, lap, p);
    }
}

template <typename T, int V, int MODEL, bool UNIT>
static __device__ void run_rows(const BatchInst& bi, int xs, int xe, const T* __restrict__ in, T* __restrict__ out,
                                int lane)
{
    using A = Ar<T>;
    const int n0 = bi.n0, n1 = bi.n1;
    const T* base_in = in + bi.off + lane * V;
    T* base_out = out + bi.off + lane * V;
    P<T> p;
    p.kappa = (T)bi.kappa;
    p.dtm = (T)bi.dtm;
    p.neg_r = (T)bi.neg_r;
    p.u = (T)bi.u;
    p.gamma2 = T(0);
    const T w0 = (T)bi.w0, w1 = (T)bi.w1;
    const unsigned FULL = 0xffffffffu;
    const int lm = (lane + 31) & 31, lp = (lane + 1) & 31;

    // c0 = c(x), c1 = c(x+1), c2 = c(x+2); m0 = mu(x-1), m1 = mu(x), m2 = mu(x+1).
    // The rotation is register moves rather than a three-way unrolled body:
    // the kernel holds 16 row widths, and a smaller body keeps them in the
    // instruction cache.
    T c0[V], c1[V], c2[V], nx[V];
    T m0[V], m1[V], m2[V];
    ld_row<T, V>(c0, base_in + (long long)wrapi(xs - 2, n0) * n1);
    ld_row<T, V>(c1, base_in + (long long)wrapi(xs - 1, n0) * n1);
    ld_row<T, V>(nx, base_in + (long long)wrapi(xs, n0) * n1);
#pragma unroll
    for (int j = 0; j < V; j++) m0[j] = m1[j] = T(0);
#pragma unroll 1
    for (int x = xs - 2; x < xe; x++) {
#pragma unroll
        for (int j = 0; j < V; j++) c2[j] = nx[j];
        if (x + 3 <= xe + 1) ld_row<T, V>(nx, base_in + (long long)wrapi(x + 3, n0) * n1);
        const T bl = __shfl_sync(FULL, c1[V - 1], lm);
        const T br = __shfl_sync(FULL, c1[0], lp);
#pragma unroll
        for (int j = 0; j < V; j++) m2[j] = mu2<T, MODEL>(c1[j], lap2<T, V, UNIT>(c0, c1, c2, bl, br, j, w0, w1), p);
        if (x >= xs) {
            const T ml = __shfl_sync(FULL, m1[V - 1], lm);
            const T mr = __shfl_sync(FULL, m1[0], lp);
            T o[V];
#pragma unroll
            for (int j = 0; j < V; j++) o[j] = A::add(c0[j], A::mul(p.dtm, lap2<T, V, UNIT>(m0, m1, m2, ml, mr, j, w0, w1)));
            st_row<T, V>(base_out + (long long)x * n1, o);
        }
#pragma unroll
        for (int j = 0; j < V; j++) {
            c0[j] = c1[j];
            c1[j] = c2[j];
            m0[j] = m1[j];
            m1[j] = m2[j];
        }
    }
}

template <typename T, int MODEL, bool UNIT>
__global__ void __launch_bounds__(128)
ch2_batch_kernel(const BatchInst* __restrict__ insts, const BatchItem* __restrict__ items, int nitems,
                 const T* __restrict__ in, T* __restrict__ out, int* __restrict__ counters, int parity)
{
    const int lane = threadIdx.x & 31;
    if (blockIdx.x == 0 && threadIdx.x == 0) counters[parity ^ 1] = 0;   // for the next launch
    while (true) {
        int k = 0;
        if (lane == 0) k = atomicAdd(&counters[parity], 1);
        k = __shfl_sync(0xffffffffu, k, 0);
        if (k >= nitems) break;
        const BatchItem it = items[k];
        const BatchInst bi = insts[it.inst];
        switch (bi.n1 >> 5) {
#define PF_BATCH_CASE(v) \
    case v: run_rows<T, v, MODEL, UNIT>(bi, it.xs, it.xe, in, out, lane); break;
            PF_BATCH_CASE(1)
            PF_BATCH_CASE(2)
            PF_BATCH_CASE(3)
            PF_BATCH_CASE(4)
            PF_BATCH_CASE(5)
            PF_BATCH_CASE(6)
            PF_BATCH_CASE(7)
            PF_BATCH_CASE(8)
            PF_BATCH_CASE(9)
            PF_BATCH_CASE(10)
            PF_BATCH_CASE(11)
            PF_BATCH_CASE(12)
            PF_BATCH_CASE(13)
            PF_BATCH_CASE(14)
            PF_BATCH_CASE(15)
            PF_BATCH_CASE(16)
#undef PF_BATCH_CASE
        default: break;
        }
    }
}

const void* batch_kernel(int dtype, int model, bool unit)
{
    if (dtype == MMSP_GPU_F64) {
        if (model == MMSP_GPU_CH)
            return unit ? (const void*)&ch2_batch_kernel<double, MMSP_GPU_CH, true>
                        : (const void*)&ch2_batch_kernel<double, MMSP_GPU_CH, false>;
        return unit ? (const void*)&ch2_batch_kernel<double, MMSP_GPU_CH_POLY, true>
                    : (const void*)&ch2_batch_kernel<double, MMSP_GPU_CH_POLY, false>;
    }
    if (model == MMSP_GPU_CH)
        return unit ? (const void*)&ch2_batch_kernel<float, MMSP_GPU_CH, true>
                    : (const void*)&ch2_batch_kernel<float, MMSP_GPU_CH, false>;
    return unit ? (const void*)&ch2_batch_kernel<float, MMSP_GPU_CH_POLY, true>
                : (const void*)&ch2_batch_kernel<float, MMSP_GPU_CH_POLY, false>;
}

cudaError_t launch_batch(const void* fn, int blocks, int threads, const BatchInst* insts, const BatchItem* items,
                         int nitems, const void* in, void* out, int* counters, int parity, cudaStream_t s)
{
    void* args[] = {(void*)&insts, (void*)&items, (void*)&nitems, (void*)&in, (void*)&out, (void*)&counters,
                    (void*)&parity};
    return cudaLaunchKernel(fn, dim3(blocks), dim3(threads), args, 0, s);
}


// ---------------------------------------------------------------------------
// Temporal blocking: KS steps per launch on shared-memory tiles.
//
// A work item is a tile of one FP32 instance: an interior of tx x tz cells
// whose region, widened by a halo of H = 2*KS cells on every side (the
// Cahn-Hilliard step reads two cells deep: mu of the neighbours), is loaded
// once into shared memory with periodic wraps.  Each of the KS steps then
// computes mu on the region minus one more ring and the update on the region
// minus two, in place, so after KS steps the interior holds the state KS
// steps later and goes back to HBM.  HBM traffic per step falls by about KS
// times; the price is the halo work, which the autotuner weighs against it.
//
// The region is RI x CI floats (compile-time); in the passes a block of NT
// (256 or 512) threads sees it as CI/2 column pairs x (2 NT / CI) row groups, each thread
// walking a run of rows of one pair with the pairs above and below in
// registers, so a pair-step costs 3 shared loads and 1 store per pass, and
// the arithmetic runs in packed FP32x2 instructions.  Per cell it is the
// batched kernel's FP32 form.
// Two adjacent cells per thread in packed FP32x2 arithmetic (one
// instruction for both cells, and one 8-byte shared access for both).
static __device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }
static __device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }
static __device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
static __device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
static __device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

template <int MODEL>
static __device__ __forceinline__ float2 tb_mu(float2 c, float2 lap, float kappa, float neg_r, float u)
{
    const float2 fp = MODEL == MMSP_GPU_CH ? mul2(c, fma2(fma2(f2(4.0f), c, f2(-6.0f)), c, f2(2.0f)))
                                           : mul2(c, fma2(f2(u), mul2(c, c), f2(neg_r)));
    return fma2(f2(-kappa), lap, fp);
}

// lap of cells (y.x, y.y) from the pairs above and below and the cells just
// left (l) and right (r) of the pair
template <bool UNIT>
static __device__ __forceinline__ float2 tb_lap(float2 y, float2 up, float2 dn, float l, float r, float w0, float w1)
{
    const float2 hz = add2(f2(l, y.x), f2(y.y, r));
    if (UNIT) return fma2(f2(-4.0f), y, add2(add2(dn, up), hz));
    return fma2(f2(w0), add2(dn, up), fma2(f2(w1), hz, mul2(f2(-2.0f * (w0 + w1)), y)));
}

template <int RI, int CI, int KS, int NT, int MODEL, bool UNIT>
__global__ void __launch_bounds__(NT)
ch2_tb_kernel(const BatchInst* __restrict__ insts, const TbItem* __restrict__ items, int nitems,
              const float* __restrict__ in, float* __restrict__ out, int* __restrict__ counters, int parity)
{
    constexpr int H = 2 * KS;
    constexpr int RG = NT / CI;          // row groups of the loads and stores (one cell per thread)
    constexpr int PG = 2 * NT / CI;      // row groups of the passes (a pair of cells per thread)
    static_assert(CI % 32 == 0 && NT % CI == 0 && RI > 2 * H && CI > 2 * H, "tile shape");
    extern __shared__ __align__(16) float tb_sm[];
    float* C = tb_sm;              // c, updated in place
    float* M = tb_sm + RI * CI;    // mu
    __shared__ int s_item;
    const int t = threadIdx.x;
    const int col = t % CI, rg = t / CI;                    // loads and stores
    const int pc = 2 * (t % (CI / 2)), pg = t / (CI / 2);  // passes: cells pc, pc+1
    const int pl = pc == 0 ? 0 : pc - 1;                    // left of the pair (column 0 is never computed)
    const int pr = pc + 2 == CI ? CI - 1 : pc + 2;          // right of the pair
    if (blockIdx.x == 0 && t == 0) counters[parity ^ 1] = 0;   // for the next launch
    while (true) {
        if (t == 0) s_item = atomicAdd(&counters[parity], 1);
        __syncthreads();
        const int k = s_item;
        if (k >= nitems) break;
        const TbItem it = items[k];
        const BatchInst bi = insts[it.inst];
        const int rows = it.tx + 2 * H, cols = it.tz + 2 * H;
        const float kappa = (float)bi.kappa, dtm = (float)bi.dtm, neg_r = (float)bi.neg_r, u = (float)bi.u;
        const float w0 = (float)bi.w0, w1 = (float)bi.w1;
        const float* src = in + bi.off;
        // the region with periodic wraps (rows of axis 0, columns of axis 1)
        // (4-byte asynchronous copies: every load of the region is in flight at once)
        if (col < cols) {
            const int gz = wrapi(it.z0 - H + col, bi.n1);
            int gx = wrapi(it.x0 - H + rg, bi.n0);   // row of region row r, advanced without a division
            for (int r = rg; r < rows; r += RG) {
                cp_async4(&C[r * CI + col], src + (long long)gx * bi.n1 + gz);
                gx += RG;
                while (gx >= bi.n0) gx -= bi.n0;     // more than once only for grids smaller than a tile
            }
        }
        cp_async_wait_all();
        __syncthreads();
        // A pass computes both cells of every pair that meets its column
        // range; a cell just outside it gets a value that no later cell of
        // the range reads (the ranges shrink by one cell per pass).
        for (int j = 0; j < KS; j++) {
            // mu on rows [2j+1, rows-2j-1) x cols [2j+1, cols-2j-1)
            {
                const int a = 2 * j + 1, b = rows - 2 * j - 1;
                const int h = (b - a + PG - 1) / PG;
                const int r0 = a + pg * h, r1 = min(b, r0 + h);
                if (pc + 1 >= a && pc < cols - 2 * j - 1 && r0 < r1) {
                    float2 up = *reinterpret_cast<const float2*>(&C[(r0 - 1) * CI + pc]);
                    float2 cc = *reinterpret_cast<const float2*>(&C[r0 * CI + pc]);
                    for (int r = r0; r < r1; r++) {
                        const float2 dn = *reinterpret_cast<const float2*>(&C[(r + 1) * CI + pc]);
                        const float2 lap = tb_lap<UNIT>(cc, up, dn, C[r * CI + pl], C[r * CI + pr], w0, w1);
                        *reinterpret_cast<float2*>(&M[r * CI + pc]) = tb_mu<MODEL>(cc, lap, kappa, neg_r, u);
                        up = cc;
                        cc = dn;
                    }
                }
            }
            __syncthreads();
            // c' = c + dt*M*lap(mu) on rows [2j+2, rows-2j-2) x cols [2j+2, cols-2j-2), in place
            {
                const int a = 2 * j + 2, b = rows - 2 * j - 2;
                const int h = (b - a + PG - 1) / PG;
                const int r0 = a + pg * h, r1 = min(b, r0 + h);
                if (pc + 1 >= a && pc < cols - 2 * j - 2 && r0 < r1) {
                    float2 up = *reinterpret_cast<const float2*>(&M[(r0 - 1) * CI + pc]);
                    float2 mm = *reinterpret_cast<const float2*>(&M[r0 * CI + pc]);
                    for (int r = r0; r < r1; r++) {
                        const float2 dn = *reinterpret_cast<const float2*>(&M[(r + 1) * CI + pc]);
                        const float2 lap = tb_lap<UNIT>(mm, up, dn, M[r * CI + pl], M[r * CI + pr], w0, w1);
                        float2* cp = reinterpret_cast<float2*>(&C[r * CI + pc]);
                        *cp = fma2(f2(dtm), lap, *cp);
                        up = mm;
                        mm = dn;
                    }
                }
            }
            __syncthreads();
        }
        // the interior back to HBM
        if (col >= H && col < H + it.tz) {
            float* dst = out + bi.off + (it.z0 - H + col);
            for (int r = H + rg; r < H + it.tx; r += RG) dst[(long long)(it.x0 - H + r) * bi.n1] = C[r * CI + col];
        }
        __syncthreads();   // the region is reloaded by the next item
    }
}

namespace {
template <int RI, int CI, int KS, int NT, int MODEL>
const void* tb_unit(bool unit)
{
    return unit ? (const void*)&ch2_tb_kernel<RI, CI, KS, NT, MODEL, true>
                : (const void*)&ch2_tb_kernel<RI, CI, KS, NT, MODEL, false>;
}
template <int RI, int CI, int KS, int NT>
const void* tb_model(int model, bool unit)
{
    return model == MMSP_GPU_CH ? tb_unit<RI, CI, KS, NT, MMSP_GPU_CH>(unit)
                                : tb_unit<RI, CI, KS, NT, MMSP_GPU_CH_POLY>(unit);
}
template <int RI, int CI, int NT>
const void* tb_depth(int ks, int model, bool unit)
{
    switch (ks) {
    case 2: return tb_model<RI, CI, 2, NT>(model, unit);
    case 4: return tb_model<RI, CI, 4, NT>(model, unit);
    case 8: return tb_model<RI, CI, 8, NT>(model, unit);
    default: return nullptr;
    }
}
}  // namespace

const TbShape kTbShapes[kTbShapeCount] = {{64, 128, 256}, {96, 128, 256}, {128, 64, 256},
                                          {64, 128, 512}, {96, 128, 512}, {128, 64, 512}};

const void* tb_kernel(int shape, int ks, int model, bool unit)
{
    switch (shape) {
    case 0: return tb_depth<64, 128, 256>(ks, model, unit);
    case 1: return tb_depth<96, 128, 256>(ks, model, unit);
    case 2: return tb_depth<128, 64, 256>(ks, model, unit);
    case 3: return tb_depth<64, 128, 512>(ks, model, unit);
    case 4: return tb_depth<96, 128, 512>(ks, model, unit);
    case 5: return tb_depth<128, 64, 512>(ks, model, unit);
    default: return nullptr;
    }
}

size_t tb_smem(int shape) { return sizeof(float) * 2 * (size_t)kTbShapes[shape].ri * kTbShapes[shape].ci; }

cudaError_t launch_tb(const void* fn, int blocks, int threads, size_t smem, const BatchInst* insts,
                      const TbItem* items, int nitems, const void* in, void* out, int* counters, int parity,
                      cudaStream_t s)
{
    void* args[] = {(void*)&insts, (void*)&items, (void*)&nitems, (void*)&in, (void*)&out, (void*)&counters,
                    (void*)&parity};
    return cudaLaunchKernel(fn, dim3(blocks), dim3(threads), args, smem, s);
}

}  // namespace pf
