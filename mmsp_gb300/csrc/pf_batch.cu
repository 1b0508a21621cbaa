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
// once into shared memory with periodic wraps.  KS steps then run there in
// place, each valid on two fewer rings of the region, so after KS steps the
// interior holds the state KS steps later and goes back to HBM.  HBM traffic
// per step falls by about KS times; the price is the halo work, which the
// autotuner weighs against it.
//
// The region is RI x 128 floats.  A warp spans a whole region row, 4 cells
// per lane (16-byte shared accesses); its left and right neighbours come from
// the adjacent lanes by shuffle.  The warps of a block split the rows of the
// step's update range into bands; a warp walks its band downwards with c of
// rows r, r+1 and mu of rows r-1, r in registers: per row it loads c(r+2),
// computes mu(r+1) and writes c'(r) = c + dt*M*lap(mu) over c(r), so mu never
// goes to shared memory and is computed twice only on the two rows that
// border each band.  The two rows on either side of a band belong to the
// neighbouring bands, which overwrite them, so each warp reads them into
// registers before a barrier at the start of the step.  Columns are computed
// over the full width: the outermost column of each side reads a neighbour
// from the wrong side (lane 0's left, lane 31's right) or a column beyond the
// tile, and like every cell of the halo this garbage moves inwards by two
// cells per step, so after KS steps it has not reached the interior
// [2*KS, cols - 2*KS).  Rows outside the shrinking update range are not
// written and hold values of earlier steps or tiles, which again only halo
// cells read.  Loads and stores are 16-byte: batched grids have rows of a
// multiple of 32 cells at 256-byte aligned offsets, and tile columns start at
// multiples of 4, so a group of 4 cells never straddles a periodic wrap.
// Per cell the arithmetic is the batched kernel's FP32 form, in packed FP32x2
// instructions (one instruction for two cells).
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

// lap of a lane's 4 cells from the rows above and below; the horizontal
// neighbour sums are formed by scalar adds (no register pairs to build), the
// rest in packed FP32x2
template <bool UNIT>
static __device__ __forceinline__ void tb_lap4(float4 up, float4 cc, float4 dn, float w0, float w1, float2& l01,
                                               float2& l23)
{
    const float left = __shfl_up_sync(0xffffffffu, cc.w, 1);
    const float right = __shfl_down_sync(0xffffffffu, cc.x, 1);
    const float2 h01 = f2(left + cc.y, cc.x + cc.z), h23 = f2(cc.y + cc.w, cc.z + right);
    const float2 v01 = add2(f2(up.x, up.y), f2(dn.x, dn.y)), v23 = add2(f2(up.z, up.w), f2(dn.z, dn.w));
    const float2 c01 = f2(cc.x, cc.y), c23 = f2(cc.z, cc.w);
    if (UNIT) {
        l01 = fma2(f2(-4.0f), c01, add2(v01, h01));
        l23 = fma2(f2(-4.0f), c23, add2(v23, h23));
    } else {
        const float2 k = f2(-2.0f * (w0 + w1));
        l01 = fma2(f2(w0), v01, fma2(f2(w1), h01, mul2(k, c01)));
        l23 = fma2(f2(w0), v23, fma2(f2(w1), h23, mul2(k, c23)));
    }
}

template <int MODEL, bool UNIT>
static __device__ __forceinline__ float4 tb_mu4(float4 up, float4 cc, float4 dn, float w0, float w1, float kappa,
                                                float neg_r, float u)
{
    float2 l01, l23;
    tb_lap4<UNIT>(up, cc, dn, w0, w1, l01, l23);
    const float2 m01 = tb_mu<MODEL>(f2(cc.x, cc.y), l01, kappa, neg_r, u);
    const float2 m23 = tb_mu<MODEL>(f2(cc.z, cc.w), l23, kappa, neg_r, u);
    return make_float4(m01.x, m01.y, m23.x, m23.y);
}

template <bool UNIT>
static __device__ __forceinline__ float4 tb_update4(float4 c, float4 up, float4 mm, float4 dn, float w0, float w1,
                                                    float dtm)
{
    float2 l01, l23;
    tb_lap4<UNIT>(up, mm, dn, w0, w1, l01, l23);
    const float2 n01 = fma2(f2(dtm), l01, f2(c.x, c.y)), n23 = fma2(f2(dtm), l23, f2(c.z, c.w));
    return make_float4(n01.x, n01.y, n23.x, n23.y);
}

template <int RI, int KS, int NW, int MODEL, bool UNIT, bool ALIGNED>
__global__ void __launch_bounds__(NW * 32)
ch2_tb_kernel(const BatchInst* __restrict__ insts, const TbItem* __restrict__ items, int nitems,
              const float* __restrict__ in, float* __restrict__ out, int* __restrict__ counters, int parity)
{
    constexpr int CI = kTbCols;          // 32 lanes x 4 cells
    constexpr int H = 2 * KS;
    constexpr int NT = NW * 32;
    constexpr int RG = NT / (CI / 4);    // row groups of the 16-byte loads and stores
    static_assert(RI > 2 * H && CI > 2 * H && NT % (CI / 4) == 0, "tile shape");
    extern __shared__ __align__(16) float tb_sm[];
    float* C = tb_sm;
    __shared__ int s_item;
    const int t = threadIdx.x;
    const int lane = t & 31, warp = t >> 5;
    const int g = t % (CI / 4), rg = t / (CI / 4);   // loads and stores: cells 4g..4g+3 of rows rg + k*RG
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
        // the region with periodic wraps (rows of axis 0, columns of axis 1),
        // every copy in flight at once: 16-byte groups (ALIGNED), else cell by cell
        if (4 * g < cols) {
            int gx = wrapi(it.x0 - H + rg, bi.n0);   // row of region row r, advanced without a division
            if (ALIGNED) {
                const int gz = wrapi(it.z0 - H + 4 * g, bi.n1);
                for (int r = rg; r < rows; r += RG) {
                    cp_async16(&C[r * CI + 4 * g], src + (long long)gx * bi.n1 + gz);
                    gx += RG;
                    while (gx >= bi.n0) gx -= bi.n0;     // more than once only for grids smaller than a tile
                }
            } else {
                int gz[4];
#pragma unroll
                for (int q = 0; q < 4; q++) gz[q] = wrapi(it.z0 - H + 4 * g + q, bi.n1);
                for (int r = rg; r < rows; r += RG) {
                    const float* row = src + (long long)gx * bi.n1;
#pragma unroll
                    for (int q = 0; q < 4; q++)
                        if (4 * g + q < cols) cp_async4(&C[r * CI + 4 * g + q], row + gz[q]);
                    gx += RG;
                    while (gx >= bi.n0) gx -= bi.n0;
                }
            }
        }
        cp_async_wait_all();
        __syncthreads();
        for (int j = 0; j < KS; j++) {
            const int a = 2 * j + 2, b = rows - 2 * j - 2;   // update rows of step j
            const int h = (b - a + NW - 1) / NW;
            const int r0 = a + warp * h, r1 = min(b, r0 + h);
            auto ld = [&](int r) { return *reinterpret_cast<const float4*>(&C[r * CI + 4 * lane]); };
            auto put = [&](int r, float4 v) { *reinterpret_cast<float4*>(&C[r * CI + 4 * lane]) = v; };
            float4 ca, cb, f0, f1;   // c of the two rows above and the two rows below the band
            if (r0 < r1) {
                ca = ld(r0 - 2);
                cb = ld(r0 - 1);
                f0 = ld(r1);
                f1 = ld(r1 + 1);
            }
            __syncthreads();
            if (r0 < r1) {   // warp-uniform: the shuffles see the whole warp
                auto row = [&](int r) { return r < r1 ? ld(r) : r == r1 ? f0 : f1; };
                // c(r), c(r+1), mu(r-1), mu(r) in registers at row r
                float4 cA = row(r0), cB = row(r0 + 1);
                float4 mA = tb_mu4<MODEL, UNIT>(ca, cb, cA, w0, w1, kappa, neg_r, u);
                float4 mB = tb_mu4<MODEL, UNIT>(cb, cA, cB, w0, w1, kappa, neg_r, u);
                int r = r0;
                // three rows per iteration (the register roles come back to
                // the same places, so no copies), while the rows read are in the band
                for (; r + 5 <= r1; r += 3) {
                    const float4 c2 = ld(r + 2);
                    const float4 m2 = tb_mu4<MODEL, UNIT>(cA, cB, c2, w0, w1, kappa, neg_r, u);
                    put(r, tb_update4<UNIT>(cA, mA, mB, m2, w0, w1, dtm));
                    const float4 c3 = ld(r + 3);
                    const float4 m3 = tb_mu4<MODEL, UNIT>(cB, c2, c3, w0, w1, kappa, neg_r, u);
                    put(r + 1, tb_update4<UNIT>(cB, mB, m2, m3, w0, w1, dtm));
                    const float4 c4 = ld(r + 4);
                    const float4 m4 = tb_mu4<MODEL, UNIT>(c2, c3, c4, w0, w1, kappa, neg_r, u);
                    put(r + 2, tb_update4<UNIT>(c2, m2, m3, m4, w0, w1, dtm));
                    cA = c3;
                    cB = c4;
                    mA = m3;
                    mB = m4;
                }
                for (; r < r1; r++) {   // the last rows: at most four
                    const float4 c2 = row(r + 2);
                    const float4 m2 = tb_mu4<MODEL, UNIT>(cA, cB, c2, w0, w1, kappa, neg_r, u);
                    put(r, tb_update4<UNIT>(cA, mA, mB, m2, w0, w1, dtm));
                    cA = cB;
                    cB = c2;
                    mA = mB;
                    mB = m2;
                }
            }
            __syncthreads();
        }
        // the interior back to HBM
        if (ALIGNED) {
            if (4 * g >= H && 4 * g < H + it.tz) {
                float* dst = out + bi.off + (it.z0 - H + 4 * g);
                for (int r = H + rg; r < H + it.tx; r += RG)
                    *reinterpret_cast<float4*>(dst + (long long)(it.x0 - H + r) * bi.n1) =
                        *reinterpret_cast<const float4*>(&C[r * CI + 4 * g]);
            }
        } else if (4 * g + 3 >= H && 4 * g < H + it.tz) {
            float* dst = out + bi.off + (it.z0 - H + 4 * g);
            for (int r = H + rg; r < H + it.tx; r += RG) {
                float* drow = dst + (long long)(it.x0 - H + r) * bi.n1;
#pragma unroll
                for (int q = 0; q < 4; q++)
                    if (4 * g + q >= H && 4 * g + q < H + it.tz) drow[q] = C[r * CI + 4 * g + q];
            }
        }
        __syncthreads();   // the region is reloaded by the next item
    }
}

namespace {
template <int RI, int KS, int NW, bool AL>
const void* tb_model_al(int model, bool unit)
{
    if (model == MMSP_GPU_CH)
        return unit ? (const void*)&ch2_tb_kernel<RI, KS, NW, MMSP_GPU_CH, true, AL>
                    : (const void*)&ch2_tb_kernel<RI, KS, NW, MMSP_GPU_CH, false, AL>;
    return unit ? (const void*)&ch2_tb_kernel<RI, KS, NW, MMSP_GPU_CH_POLY, true, AL>
                : (const void*)&ch2_tb_kernel<RI, KS, NW, MMSP_GPU_CH_POLY, false, AL>;
}
template <int RI, int KS, int NW>
const void* tb_model(int model, bool unit)
{
    return tb_model_al<RI, KS, NW, true>(model, unit);
}
template <int RI, int NW>
const void* tb_depth(int ks, int model, bool unit)
{
    switch (ks) {
    case 2: return tb_model<RI, 2, NW>(model, unit);
    case 4: return tb_model<RI, 4, NW>(model, unit);
    case 8: return tb_model<RI, 8, NW>(model, unit);
    default: return nullptr;
    }
}
}  // namespace

const TbShape kTbShapes[kTbShapeCount] = {{64, 128}, {96, 128}, {128, 256}, {128, 128}};

const void* tb_kernel(int shape, int ks, int model, bool unit)
{
    switch (shape) {
    case 0: return tb_depth<64, 4>(ks, model, unit);
    case 1: return tb_depth<96, 4>(ks, model, unit);
    case 2: return tb_depth<128, 8>(ks, model, unit);
    case 3: return tb_depth<128, 4>(ks, model, unit);
    default: return nullptr;
    }
}

size_t tb_smem(int shape) { return sizeof(float) * (size_t)kTbShapes[shape].ri * kTbCols; }

const void* tb_kernel_any(int model, bool unit) { return tb_model_al<64, kTbAnyDepth, 4, false>(model, unit); }

cudaError_t launch_tb(const void* fn, int blocks, int threads, size_t smem, const BatchInst* insts,
                      const TbItem* items, int nitems, const void* in, void* out, int* counters, int parity,
                      cudaStream_t s)
{
    void* args[] = {(void*)&insts, (void*)&items, (void*)&nitems, (void*)&in, (void*)&out, (void*)&counters,
                    (void*)&parity};
    return cudaLaunchKernel(fn, dim3(blocks), dim3(threads), args, smem, s);
}

}  // namespace pf
