// pf_ac3_stream.cu -- FP32 3D multi-order Allen-Cahn step, streaming along X.
//
// The precision-form kernel for 3D grids with rows (axis Z) of up to 256
// cells.  A block owns R rows (axis Y) of full Z extent and a run of X
// planes, with one or two threads per cell of a row (each over R or R/2
// rows).  For every plane the block's R+2 rows (one halo row each side,
// wrapped periodically) of all N fields arrive in shared memory on a D-deep
// mbarrier ring: by cp.async.bulk (one copy per field, two where the rows
// wrap) when rows are 16-byte multiples, by per-thread 4-byte cp.async
// otherwise.  With D = 3 the copy of plane x+2 is issued as soon as plane
// x-1 is released; the copies of the several blocks resident on an SM
// overlap each other's computation.  Per cell the sum of squares over the
// fields comes first, then each field's new value from its own 7-point
// Laplacian; Y neighbours are registers, X and Z neighbours are read from
// shared memory (Z wraps across the row).  There is no Z halo, and the Y
// halo costs 2 extra rows per R-row strip in reads only.
#include <algorithm>
#include <cstdio>
#include <cstdlib>

#include "pf_async.cuh"
#include "pf_device.cuh"
#include "pf_internal.h"

namespace pf {

struct AcF32 {
    float wx, wy, wz, w2;
    float kappa, dtm, gamma2, neg_r, u;
};

template <int MODEL>
static __device__ __forceinline__ float ac_new_f32(float c, float sum, float lap, const AcF32& q)
{
    const float c2 = c * c;
    if (MODEL == MMSP_GPU_AC) {
        // -c + c^3 + 2 gamma c (sum - c^2) - kappa lap
        const float df = c * fmaf(q.gamma2, sum - c2, c2 - 1.0f);
        return fmaf(-q.dtm, fmaf(-q.kappa, lap, df), c);
    } else if (MODEL == MMSP_GPU_GG || MODEL == MMSP_GPU_ZENER) {
        // -c - c^3 + 2 (c sum - lap)
        const float e = fmaf(2.0f, fmaf(c, sum, -lap), -c * fmaf(c, c, 1.0f));
        return fmaf(-q.dtm, e, c);
    } else {
        // -r c + u c^3 - K lap
        const float e = fmaf(-q.kappa, lap, c * fmaf(q.u, c2, q.neg_r));
        return fmaf(-q.dtm, e, c);
    }
}

static size_t ac3_smem(int R, int Z, int N, int D)
{
    return sizeof(float) * (((size_t)D * N * (R + 2) * Z + 1) & ~(size_t)1) + sizeof(uint64_t) * D;
}

#ifndef PF_AC3_FUNROLL
#define PF_AC3_FUNROLL 2
#endif
constexpr int kAcFieldUnroll = PF_AC3_FUNROLL;   // fields updated per loop trip

// A block is Zt x TY threads (Zt = Z rounded up to a warp), R = RT * TY rows:
// thread (z, ty) owns cell z of rows ty*RT .. ty*RT+RT-1 of the strip.  ZT is
// the row length when it is a compile-time constant (shared-memory and store
// offsets become immediates), 0 when it is taken from the grid.  Shared
// offsets are 32-bit.
//
// BULK: rows are a multiple of 16 bytes, and thread 0 stages each field's
// rows with cp.async.bulk (transaction-counted mbarrier, one arrival).
// Otherwise every thread copies cells with 4-byte cp.async and arrives on
// the mbarrier when they land (one arrival per thread).
template <int RT, int TY, int ZT, int MODEL, bool BULK>
__global__ void __launch_bounds__(256)
ac3_stream_f32(const float* __restrict__ ein, float* __restrict__ eout, Geom g, AcF32 q, int planes, int N, int D,
               int* __restrict__ err)
{
    constexpr int R = RT * TY, RR = R + 2;
    const int Z = ZT ? ZT : g.Z;
    const int t = threadIdx.x, ty = TY > 1 ? threadIdx.y : 0;
    const int tid = t + ty * blockDim.x;
    const bool on = t < Z;
    const int z = on ? t : 0;
    extern __shared__ __align__(128) unsigned char sm[];
    float* slots = reinterpret_cast<float*>(sm);
    const int chunk = RR * Z;   // floats of one field's rows in a slot
    const int slot_elems = N * chunk;
    uint64_t* bars = reinterpret_cast<uint64_t*>(slots + ((D * slot_elems + 1) & ~1));

    const int y0 = blockIdx.x * R;
    const int xs = blockIdx.y * planes;
    const int xe = min(xs + planes, g.X);
    if (xs >= xe) return;
    const int dl = z == 0 ? Z - 1 : -1;          // offset of the low Z neighbour
    const int dh = z == Z - 1 ? 1 - Z : 1;       // offset of the high Z neighbour
    const int x_first = xs - 1, x_last = xe;     // planes read from global memory
    const long long cells = g.cells;
    const int nrows = min(RT, g.Y - y0 - ty * RT);   // rows of this thread inside the grid (may be <= 0)
    const int me = z + ty * RT * Z;              // this thread's cell in the halo row above its rows

    // BULK: called by thread 0 only; otherwise by every thread
    auto fill = [&](int pl) {
        const int k = pl - x_first, s = k % D;
        uint64_t* bar = &bars[s];
        float* dst0 = slots + s * slot_elems;
        const long long plane = (long long)wrapi(pl, g.X) * g.YZ;
        if constexpr (BULK) {
            const uint32_t row = (uint32_t)Z * sizeof(float);
            fence_proxy_async();
            mbar_expect_tx(bar, (uint32_t)N * RR * row);
            const int a = y0 - 1, b = y0 + R + 1;
            for (int f = 0; f < N; f++) {
                const float* base = ein + (long long)f * cells + plane;
                float* dst = dst0 + f * chunk;
                if (a >= 0 && b <= g.Y) {
                    bulk_g2s(dst, base + (long long)a * Z, RR * row, bar);
                } else if (a < 0) {
                    bulk_g2s(dst, base + (long long)(g.Y - 1) * Z, row, bar);
                    bulk_g2s(dst + Z, base, (RR - 1) * row, bar);
                } else {
                    const int n1 = g.Y - a;
                    bulk_g2s(dst, base + (long long)a * Z, n1 * row, bar);
                    bulk_g2s(dst + n1 * Z, base, (RR - n1) * row, bar);
                }
            }
        } else {
            if (on)
                for (int f = 0; f < N; f++) {
                    const float* base = ein + (long long)f * cells + plane + z;
                    float* dst = dst0 + f * chunk + z;
                    for (int r = ty; r < RR; r += TY)   // (g.Y >= R + 2)
                        cp_async4(dst + r * Z, base + (long long)wrap_near(y0 - 1 + r, g.Y) * Z);
                }
            cp_async_arrive(bar);
        }
    };
    auto slot_of = [&](int pl) -> const float* { return slots + ((pl - x_first) % D) * slot_elems; };
    auto arrived = [&](int pl) {
        const int k = pl - x_first;
        return mbar_wait(&bars[k % D], (uint32_t)(k / D) & 1u);
    };
    const bool producer = !BULK || tid == 0;

    if (tid == 0) {
        for (int s = 0; s < D; s++) mbar_init(&bars[s], BULK ? 1 : blockDim.x * blockDim.y);
        mbar_fence_init();
    }
    __syncthreads();
    int issued = min(x_first + D - 1, x_last);   // last plane whose fill was issued
    if (producer)
        for (int pl = x_first; pl <= issued; pl++) fill(pl);
    bool bad = !arrived(x_first);
    bad |= !arrived(x_first + 1);
    // The decision to stop is taken block-wide (__syncthreads_or), so every
    // thread leaves the loop at the same barrier.
    bool stop = __syncthreads_or(bad);

    for (int x = xs; x < xe && !stop; x++) {
        bad = !arrived(x + 1);
        const float* SL = slot_of(x - 1) + me + Z;   // centre rows of the planes either side
        const float* SH = slot_of(x + 1) + me + Z;
        const float* SC = slot_of(x) + me;           // rows ty*RT .. ty*RT+RT+1 of plane x
        float sum[RT];
#pragma unroll
        for (int i = 0; i < RT; i++) sum[i] = 0.0f;
#pragma unroll 1
        for (int f = 0; f < N; f++) {
            const float* c = SC + f * chunk + Z;
#pragma unroll
            for (int i = 0; i < RT; i++) sum[i] = fmaf(c[i * Z], c[i * Z], sum[i]);
        }
        float* dst = eout + (long long)x * g.YZ + (long long)(y0 + ty * RT) * Z + z;
#pragma unroll kAcFieldUnroll
        for (int f = 0; f < N; f++) {
            const int fo = f * chunk;
            float col[RT + 2];
#pragma unroll
            for (int i = 0; i < RT + 2; i++) col[i] = SC[fo + i * Z];
#pragma unroll
            for (int i = 0; i < RT; i++) {
                const int o = fo + i * Z;
                const float cc = col[i + 1];
                const float sx = SL[o] + SH[o];
                const float sy = col[i] + col[i + 2];
                const float sz = SC[o + Z + dl] + SC[o + Z + dh];
                const float lap = fmaf(q.wx, sx, fmaf(q.wy, sy, fmaf(q.wz, sz, -q.w2 * cc)));
                // Zener pinning: the particles (field 0) have zero mobility
                const float v = (MODEL == MMSP_GPU_ZENER && f == 0) ? cc : ac_new_f32<MODEL>(cc, sum[i], lap, q);
                if (on && i < nrows) dst[(long long)f * cells + i * Z] = v;
            }
        }
        stop = __syncthreads_or(bad);
        if (!stop && x - 1 + D <= x_last) {   // the slot of x-1 is free now
            if (producer) fill(x - 1 + D);
            issued = x - 1 + D;
        }
    }
    if (stop) {
        if (tid == 0) atomicExch(err, 1);
        // leave no copy in flight: wait (bounded) for the last fill of every slot
        for (int pl = max(x_first, issued - D + 1); pl <= issued; pl++) arrived(pl);
    }
}

// Rows of Z = 32*V cells (64, 128, 256): a warp spans a row, V adjacent cells
// per lane.  The ring, its copies and the strip geometry are those of the
// kernel above (bulk copies: such rows are 16-byte multiples), with TY rows
// per strip and FG warps per row that take every FG-th field (each sums the
// squares of all fields of its cells): FG times the warps at the same shared
// memory, to hide the latency of each warp's dependent loads and arithmetic.
// Shared reads are V-wide vectors, the Z
// neighbours at a lane's ends come from the adjacent lanes by shuffle (lane 0
// and lane 31 are neighbours: the periodic wrap of the row), and the
// arithmetic runs on pairs of cells in packed FP32x2 instructions; the
// in-row neighbour sums are scalar adds, which need no pairs built.
static __device__ __forceinline__ float2 v2(float a, float b) { return make_float2(a, b); }
static __device__ __forceinline__ float2 v2(float a) { return make_float2(a, a); }

// The update of ac_new_f32 on a pair of cells, with the polynomial terms
// regrouped into fewer multiply-adds (FP32 rounding differs in the last bits).
template <int MODEL>
static __device__ __forceinline__ float2 ac_new_f32x2(float2 c, float2 sum, float2 lap, const AcF32& q)
{
    const float2 c2 = __fmul2_rn(c, c);
    if (MODEL == MMSP_GPU_AC) {
        // c' = c - dt L (c (gamma2 sum + (1 - gamma2) c^2 - 1) - kappa lap)
        const float2 df = __fmul2_rn(c, __ffma2_rn(v2(q.gamma2), sum, __ffma2_rn(v2(1.0f - q.gamma2), c2, v2(-1.0f))));
        return __ffma2_rn(v2(-q.dtm), __ffma2_rn(v2(-q.kappa), lap, df), c);
    } else if (MODEL == MMSP_GPU_GG || MODEL == MMSP_GPU_ZENER) {
        // c' = c - dt L (2 (c sum - lap) - c (c^2 + 1))
        const float2 t = __ffma2_rn(c, sum, __fmul2_rn(lap, v2(-1.0f)));
        const float2 m = __fmul2_rn(c, __fadd2_rn(c2, v2(1.0f)));
        return __ffma2_rn(v2(q.dtm), m, __ffma2_rn(v2(-2.0f * q.dtm), t, c));
    } else {
        // c' = c - dt L (c (u c^2 - r) - kappa lap)
        const float2 e = __ffma2_rn(v2(-q.kappa), lap, __fmul2_rn(c, __ffma2_rn(v2(q.u), c2, v2(q.neg_r))));
        return __ffma2_rn(v2(-q.dtm), e, c);
    }
}

template <int V>
static __device__ __forceinline__ void ldv(const float* p, float (&v)[V])
{
    if constexpr (V == 2) {
        const float2 a = *reinterpret_cast<const float2*>(p);
        v[0] = a.x;
        v[1] = a.y;
    } else {
#pragma unroll
        for (int k = 0; k < V; k += 4) {
            const float4 a = *reinterpret_cast<const float4*>(p + k);
            v[k] = a.x;
            v[k + 1] = a.y;
            v[k + 2] = a.z;
            v[k + 3] = a.w;
        }
    }
}

template <int V>
static __device__ __forceinline__ void stv(float* p, const float (&v)[V])
{
    if constexpr (V == 2) {
        *reinterpret_cast<float2*>(p) = make_float2(v[0], v[1]);
    } else {
#pragma unroll
        for (int k = 0; k < V; k += 4) *reinterpret_cast<float4*>(p + k) = make_float4(v[k], v[k + 1], v[k + 2], v[k + 3]);
    }
}

template <int V, int TY, int FG, int MODEL>
__global__ void __launch_bounds__(32 * TY * FG)
ac3_vec_f32(const float* __restrict__ ein, float* __restrict__ eout, Geom g, AcF32 q, int planes, int N, int D,
            int* __restrict__ err)
{
    constexpr int Z = 32 * V, R = TY, RR = R + 2;
    const int lane = threadIdx.x, w = threadIdx.y, fg = FG > 1 ? threadIdx.z : 0;
    const int tid = lane + 32 * (w + TY * fg);
    extern __shared__ __align__(128) unsigned char sm[];
    float* slots = reinterpret_cast<float*>(sm);
    const int chunk = RR * Z;   // floats of one field's rows in a slot
    const int slot_elems = N * chunk;
    uint64_t* bars = reinterpret_cast<uint64_t*>(slots + ((D * slot_elems + 1) & ~1));

    const int y0 = blockIdx.x * R;
    const int xs = blockIdx.y * planes;
    const int xe = min(xs + planes, g.X);
    if (xs >= xe) return;
    const int x_first = xs - 1, x_last = xe;   // planes read from global memory
    const long long cells = g.cells;
    const bool row_on = y0 + w < g.Y;           // this warp's row is inside the grid

    auto fill = [&](int pl) {   // thread 0 only
        const int k = pl - x_first, s = k % D;
        uint64_t* bar = &bars[s];
        float* dst0 = slots + s * slot_elems;
        const long long plane = (long long)wrapi(pl, g.X) * g.YZ;
        const uint32_t row = (uint32_t)Z * sizeof(float);
        fence_proxy_async();
        mbar_expect_tx(bar, (uint32_t)N * RR * row);
        const int a = y0 - 1, b = y0 + R + 1;
        for (int f = 0; f < N; f++) {
            const float* base = ein + (long long)f * cells + plane;
            float* dst = dst0 + f * chunk;
            if (a >= 0 && b <= g.Y) {
                bulk_g2s(dst, base + (long long)a * Z, RR * row, bar);
            } else if (a < 0) {
                bulk_g2s(dst, base + (long long)(g.Y - 1) * Z, row, bar);
                bulk_g2s(dst + Z, base, (RR - 1) * row, bar);
            } else {
                const int n1 = g.Y - a;
                bulk_g2s(dst, base + (long long)a * Z, n1 * row, bar);
                bulk_g2s(dst + n1 * Z, base, (RR - n1) * row, bar);
            }
        }
    };
    auto slot_of = [&](int pl) -> const float* { return slots + ((pl - x_first) % D) * slot_elems; };
    auto arrived = [&](int pl) {
        const int k = pl - x_first;
        return mbar_wait(&bars[k % D], (uint32_t)(k / D) & 1u);
    };

    if (tid == 0) {
        for (int s = 0; s < D; s++) mbar_init(&bars[s], 1);
        mbar_fence_init();
    }
    __syncthreads();
    int issued = min(x_first + D - 1, x_last);   // last plane whose fill was issued
    if (tid == 0)
        for (int pl = x_first; pl <= issued; pl++) fill(pl);
    bool bad = !arrived(x_first);
    bad |= !arrived(x_first + 1);
    bool stop = __syncthreads_or(bad);   // every thread leaves the loop at the same barrier

    const int lo = (lane + 31) & 31, hi = (lane + 1) & 31;
    for (int x = xs; x < xe && !stop; x++) {
        bad = !arrived(x + 1);
        const float* SL = slot_of(x - 1) + (w + 1) * Z + V * lane;   // own row of the plane below
        const float* SH = slot_of(x + 1) + (w + 1) * Z + V * lane;   // and above
        const float* SC = slot_of(x) + w * Z + V * lane;             // the row above the own row of plane x
        // two accumulators (even and odd fields): two independent chains
        float2 sum[V / 2], sum1[V / 2];
#pragma unroll
        for (int k = 0; k < V / 2; k++) sum[k] = sum1[k] = v2(0.0f);
        int f0 = 0;
#pragma unroll 2
        for (; f0 + 1 < N; f0 += 2) {
            float c[V], e[V];
            ldv<V>(SC + f0 * chunk + Z, c);
            ldv<V>(SC + (f0 + 1) * chunk + Z, e);
#pragma unroll
            for (int k = 0; k < V / 2; k++) {
                sum[k] = __ffma2_rn(v2(c[2 * k], c[2 * k + 1]), v2(c[2 * k], c[2 * k + 1]), sum[k]);
                sum1[k] = __ffma2_rn(v2(e[2 * k], e[2 * k + 1]), v2(e[2 * k], e[2 * k + 1]), sum1[k]);
            }
        }
        if (f0 < N) {
            float c[V];
            ldv<V>(SC + f0 * chunk + Z, c);
#pragma unroll
            for (int k = 0; k < V / 2; k++) sum[k] = __ffma2_rn(v2(c[2 * k], c[2 * k + 1]), v2(c[2 * k], c[2 * k + 1]), sum[k]);
        }
#pragma unroll
        for (int k = 0; k < V / 2; k++) sum[k] = __fadd2_rn(sum[k], sum1[k]);
        float* dst = eout + (long long)x * g.YZ + (long long)(y0 + w) * Z + V * lane;
#pragma unroll 2
        for (int f = fg; f < N; f += FG) {
            const int fo = f * chunk;
            float up[V], cc[V], dn[V], xl[V], xh[V], out[V];
            ldv<V>(SC + fo, up);
            ldv<V>(SC + fo + Z, cc);
            ldv<V>(SC + fo + 2 * Z, dn);
            ldv<V>(SL + fo, xl);
            ldv<V>(SH + fo, xh);
            const float left = __shfl_sync(0xffffffffu, cc[V - 1], lo);
            const float right = __shfl_sync(0xffffffffu, cc[0], hi);
#pragma unroll
            for (int k = 0; k < V; k += 2) {
                const float2 c2 = v2(cc[k], cc[k + 1]);
                const float2 sz = v2((k == 0 ? left : cc[k - 1]) + cc[k + 1], cc[k] + (k + 2 == V ? right : cc[k + 2]));
                const float2 sx = __fadd2_rn(v2(xl[k], xl[k + 1]), v2(xh[k], xh[k + 1]));
                const float2 sy = __fadd2_rn(v2(up[k], up[k + 1]), v2(dn[k], dn[k + 1]));
                const float2 lap = __ffma2_rn(v2(q.wx), sx, __ffma2_rn(v2(q.wy), sy,
                                              __ffma2_rn(v2(q.wz), sz, __fmul2_rn(v2(-q.w2), c2))));
                // Zener pinning: the particles (field 0) have zero mobility
                const float2 nv = (MODEL == MMSP_GPU_ZENER && f == 0) ? c2 : ac_new_f32x2<MODEL>(c2, sum[k / 2], lap, q);
                out[k] = nv.x;
                out[k + 1] = nv.y;
            }
            if (row_on) stv<V>(dst + (long long)f * cells, out);
        }
        stop = __syncthreads_or(bad);
        if (!stop && x - 1 + D <= x_last) {   // the slot of x-1 is free now
            if (tid == 0) fill(x - 1 + D);
            issued = x - 1 + D;
        }
    }
    if (stop) {
        if (tid == 0) atomicExch(err, 1);
        // leave no copy in flight: wait (bounded) for the last fill of every slot
        for (int pl = max(x_first, issued - D + 1); pl <= issued; pl++) arrived(pl);
    }
}

// The same computation with the ring run as a producer/consumer pipeline
// and no block-wide barrier in the plane loop: warp TY*FG (lane 0) issues
// the plane copies, each slot with a "full" barrier (the copy's bytes) and
// an "empty" barrier on which every computing warp arrives once it is done
// with the plane; the producer refills a slot when its "empty" phase
// completes.  A computing warp that finishes a plane goes on to the next as
// soon as that plane has arrived, instead of waiting for the slowest warp.
// Every wait is bounded; a warp whose wait runs out sets the error word and
// leaves, the others then run out too, and the producer waits (bounded) for
// its last copies before it leaves.
template <int V, int TY, int FG, int MODEL>
__global__ void __launch_bounds__(32 * (TY * FG + 1))
ac3_ws_f32(const float* __restrict__ ein, float* __restrict__ eout, Geom g, AcF32 q, int planes, int N, int D,
           int* __restrict__ err)
{
    constexpr int Z = 32 * V, R = TY, RR = R + 2, CW = TY * FG;   // CW computing warps
    const int lane = threadIdx.x, cw = threadIdx.y;
    const int w = cw % TY, fg = cw / TY;
    extern __shared__ __align__(128) unsigned char sm[];
    float* slots = reinterpret_cast<float*>(sm);
    const int chunk = RR * Z;
    const int slot_elems = N * chunk;
    uint64_t* full = reinterpret_cast<uint64_t*>(slots + ((D * slot_elems + 1) & ~1));
    uint64_t* empty = full + D;

    const int y0 = blockIdx.x * R;
    const int xs = blockIdx.y * planes;
    const int xe = min(xs + planes, g.X);
    if (xs >= xe) return;
    const int x_first = xs - 1, x_last = xe;
    const long long cells = g.cells;

    if (cw == 0 && lane == 0) {
        for (int s = 0; s < D; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], CW);
        }
        mbar_fence_init();
    }
    __syncthreads();   // the only block-wide barrier

    if (cw == CW) {   // the producer warp
        if (lane != 0) return;
        const uint32_t row = (uint32_t)Z * sizeof(float);
        int pl = x_first;
        for (; pl <= x_last; pl++) {
            const int k = pl - x_first, s = k % D;
            if (k >= D && !mbar_wait(&empty[s], (uint32_t)(k / D - 1) & 1u)) {
                atomicExch(err, 1);
                break;
            }
            float* dst0 = slots + s * slot_elems;
            const long long plane = (long long)wrapi(pl, g.X) * g.YZ;
            fence_proxy_async();
            mbar_expect_tx(&full[s], (uint32_t)N * RR * row);
            const int a = y0 - 1, b = y0 + R + 1;
            for (int f = 0; f < N; f++) {
                const float* base = ein + (long long)f * cells + plane;
                float* dst = dst0 + f * chunk;
                if (a >= 0 && b <= g.Y) {
                    bulk_g2s(dst, base + (long long)a * Z, RR * row, &full[s]);
                } else if (a < 0) {
                    bulk_g2s(dst, base + (long long)(g.Y - 1) * Z, row, &full[s]);
                    bulk_g2s(dst + Z, base, (RR - 1) * row, &full[s]);
                } else {
                    const int n1 = g.Y - a;
                    bulk_g2s(dst, base + (long long)a * Z, n1 * row, &full[s]);
                    bulk_g2s(dst + n1 * Z, base, (RR - n1) * row, &full[s]);
                }
            }
        }
        // leave no copy in flight: wait (bounded) for the last fill of every slot
        for (int p2 = max(x_first, pl - D); p2 < pl; p2++) {
            const int k = p2 - x_first;
            mbar_wait(&full[k % D], (uint32_t)(k / D) & 1u);
        }
        return;
    }

    auto slot_of = [&](int pl) -> const float* { return slots + ((pl - x_first) % D) * slot_elems; };
    auto arrived = [&](int pl) {
        const int k = pl - x_first;
        return mbar_wait(&full[k % D], (uint32_t)(k / D) & 1u);
    };
    const bool row_on = y0 + w < g.Y;
    const int lo = (lane + 31) & 31, hi = (lane + 1) & 31;
    bool ok = arrived(x_first) && arrived(x_first + 1);
    for (int x = xs; x < xe && ok; x++) {
        if (!arrived(x + 1)) {
            ok = false;
            break;
        }
        const float* SL = slot_of(x - 1) + (w + 1) * Z + V * lane;
        const float* SH = slot_of(x + 1) + (w + 1) * Z + V * lane;
        const float* SC = slot_of(x) + w * Z + V * lane;
        float2 sum[V / 2], sum1[V / 2];
#pragma unroll
        for (int k = 0; k < V / 2; k++) sum[k] = sum1[k] = v2(0.0f);
        int f0 = 0;
#pragma unroll 2
        for (; f0 + 1 < N; f0 += 2) {
            float c[V], e[V];
            ldv<V>(SC + f0 * chunk + Z, c);
            ldv<V>(SC + (f0 + 1) * chunk + Z, e);
#pragma unroll
            for (int k = 0; k < V / 2; k++) {
                sum[k] = __ffma2_rn(v2(c[2 * k], c[2 * k + 1]), v2(c[2 * k], c[2 * k + 1]), sum[k]);
                sum1[k] = __ffma2_rn(v2(e[2 * k], e[2 * k + 1]), v2(e[2 * k], e[2 * k + 1]), sum1[k]);
            }
        }
        if (f0 < N) {
            float c[V];
            ldv<V>(SC + f0 * chunk + Z, c);
#pragma unroll
            for (int k = 0; k < V / 2; k++) sum[k] = __ffma2_rn(v2(c[2 * k], c[2 * k + 1]), v2(c[2 * k], c[2 * k + 1]), sum[k]);
        }
#pragma unroll
        for (int k = 0; k < V / 2; k++) sum[k] = __fadd2_rn(sum[k], sum1[k]);
        float* dst = eout + (long long)x * g.YZ + (long long)(y0 + w) * Z + V * lane;
#pragma unroll 2
        for (int f = fg; f < N; f += FG) {
            const int fo = f * chunk;
            float up[V], cc[V], dn[V], xl[V], xh[V], out[V];
            ldv<V>(SC + fo, up);
            ldv<V>(SC + fo + Z, cc);
            ldv<V>(SC + fo + 2 * Z, dn);
            ldv<V>(SL + fo, xl);
            ldv<V>(SH + fo, xh);
            const float left = __shfl_sync(0xffffffffu, cc[V - 1], lo);
            const float right = __shfl_sync(0xffffffffu, cc[0], hi);
#pragma unroll
            for (int k = 0; k < V; k += 2) {
                const float2 c2 = v2(cc[k], cc[k + 1]);
                const float2 sz = v2((k == 0 ? left : cc[k - 1]) + cc[k + 1], cc[k] + (k + 2 == V ? right : cc[k + 2]));
                const float2 sx = __fadd2_rn(v2(xl[k], xl[k + 1]), v2(xh[k], xh[k + 1]));
                const float2 sy = __fadd2_rn(v2(up[k], up[k + 1]), v2(dn[k], dn[k + 1]));
                const float2 lap = __ffma2_rn(v2(q.wx), sx, __ffma2_rn(v2(q.wy), sy,
                                              __ffma2_rn(v2(q.wz), sz, __fmul2_rn(v2(-q.w2), c2))));
                const float2 nv = (MODEL == MMSP_GPU_ZENER && f == 0) ? c2 : ac_new_f32x2<MODEL>(c2, sum[k / 2], lap, q);
                out[k] = nv.x;
                out[k + 1] = nv.y;
            }
            if (row_on) stv<V>(dst + (long long)f * cells, out);
        }
        // this warp is done with plane x-1
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[(x - 1 - x_first) % D]);
    }
    if (!ok && lane == 0) atomicExch(err, 1);
}

// Thread rows per block for a strip of R rows of Z cells and N fields.
// Measured on 128^3 grids: two thread rows (twice the warps at the same
// shared memory) win from 8 fields up (47 -> 41 us per step at N = 8,
// 196 -> 142 us at N = 16) but lose at N = 4 and with per-thread copies
// (rows that are not 16-byte multiples).
static void ac3_threads(int R, int Z, int N, int* RT, int* TY)
{
    const int zt = (Z + 31) / 32 * 32;
#ifdef PF_AC3_TY
    int ty = PF_AC3_TY;
    (void)N;
#else
    int ty = (N > 4 && Z % 4 == 0) ? 2 : 1;
#endif
    if (R % ty || zt * ty > 256) ty = 1;
    *TY = ty;
    *RT = R / ty;
}

template <int RT, int TY, int ZT, bool BULK>
static const void* ac3_pick_model(int model)
{
    if (model == MMSP_GPU_AC) return (const void*)&ac3_stream_f32<RT, TY, ZT, MMSP_GPU_AC, BULK>;
    if (model == MMSP_GPU_GG) return (const void*)&ac3_stream_f32<RT, TY, ZT, MMSP_GPU_GG, BULK>;
    if (model == MMSP_GPU_ZENER) return (const void*)&ac3_stream_f32<RT, TY, ZT, MMSP_GPU_ZENER, BULK>;
    return (const void*)&ac3_stream_f32<RT, TY, ZT, MMSP_GPU_AC_POLY, BULK>;
}

template <int RT, int TY>
static const void* ac3_pick_z(int Z, int model)
{
    if (Z % 4) return ac3_pick_model<RT, TY, 0, false>(model);
    if (Z == 64) return ac3_pick_model<RT, TY, 64, true>(model);
    if (Z == 128) return ac3_pick_model<RT, TY, 128, true>(model);
    if (Z == 256) return ac3_pick_model<RT, TY, 256, true>(model);
    return ac3_pick_model<RT, TY, 0, true>(model);
}

// nullptr for a shape without an instantiation
static const void* ac3_pick(int RT, int TY, int Z, int model)
{
    if (TY == 2 && RT == 2) return ac3_pick_z<2, 2>(Z, model);
    if (TY == 2 && RT == 1) return ac3_pick_z<1, 2>(Z, model);
    if (TY != 1) return nullptr;
    if (RT == 4) return ac3_pick_z<4, 1>(Z, model);
    if (RT == 2) return ac3_pick_z<2, 1>(Z, model);
    if (RT == 1) return ac3_pick_z<1, 1>(Z, model);
    return nullptr;
}

constexpr size_t kAcSmemCap = 200 * 1024;

// Blocks of `smem` bytes that fit the 228 KB of shared memory of an SM
// (1 KB of each block's share is reserved by the hardware).
static int ac3_blocks_per_sm(size_t smem) { return (int)((228u * 1024u) / (smem + 1024u)); }

// Rows per strip and ring depth: the tallest strip (4, 2, 1 rows) whose
// 3-slot ring fits.  4-row strips beat 2-row ones everywhere measured (the
// Y halo is read twice as often with 2 rows), and more resident blocks beat
// a deeper ring unless the ring already limits the SM to 2 blocks or fewer.
static bool ac3_shape(const Geom& g, int N, int* R, int* D)
{
#if defined(PF_AC3_FORCE_R) && defined(PF_AC3_FORCE_D)
    if (g.Y >= PF_AC3_FORCE_R + 2 && ac3_smem(PF_AC3_FORCE_R, g.Z, N, PF_AC3_FORCE_D) <= kAcSmemCap) {
        *R = PF_AC3_FORCE_R;
        *D = PF_AC3_FORCE_D;
        return true;
    }
#endif
    static const int kR[] = {4, 2, 1};
    for (int i = 0; i < 3; i++)
        if (g.Y >= kR[i] + 2 && ac3_smem(kR[i], g.Z, N, 3) <= kAcSmemCap) {
            *R = kR[i];
            *D = 3;
            // A fourth slot (one plane of copy lead per block) pays where the
            // 3-slot ring already leaves at most 2 blocks per SM: measured
            // 142 -> 129 us at 128^3 x 16 and 65 -> 53 us at 96x200x200 x 6,
            // but 41 -> 43 us at 128^3 x 8 (3 blocks per SM with 3 slots).
            if (ac3_blocks_per_sm(ac3_smem(kR[i], g.Z, N, 3)) <= 2 && ac3_smem(kR[i], g.Z, N, 4) <= kAcSmemCap)
                *D = 4;
            return true;
        }
    return false;
}


template <int V, int TY, int FG>
static const void* acw_pick_model(int model)
{
    if (model == MMSP_GPU_AC) return (const void*)&ac3_ws_f32<V, TY, FG, MMSP_GPU_AC>;
    if (model == MMSP_GPU_GG) return (const void*)&ac3_ws_f32<V, TY, FG, MMSP_GPU_GG>;
    if (model == MMSP_GPU_ZENER) return (const void*)&ac3_ws_f32<V, TY, FG, MMSP_GPU_ZENER>;
    return (const void*)&ac3_ws_f32<V, TY, FG, MMSP_GPU_AC_POLY>;
}

template <int V, int TY, int FG>
static const void* acv_pick_model(int model)
{
    if (model == MMSP_GPU_AC) return (const void*)&ac3_vec_f32<V, TY, FG, MMSP_GPU_AC>;
    if (model == MMSP_GPU_GG) return (const void*)&ac3_vec_f32<V, TY, FG, MMSP_GPU_GG>;
    if (model == MMSP_GPU_ZENER) return (const void*)&ac3_vec_f32<V, TY, FG, MMSP_GPU_ZENER>;
    return (const void*)&ac3_vec_f32<V, TY, FG, MMSP_GPU_AC_POLY>;
}

template <int V, int TY>
static const void* acv_pick_fg(int fg, bool ws, int model)
{
    if (ws) return fg == 4 ? acw_pick_model<V, TY, 4>(model) : fg == 2 ? acw_pick_model<V, TY, 2>(model)
                                                              : acw_pick_model<V, TY, 1>(model);
    if (fg == 4) return acv_pick_model<V, TY, 4>(model);
    if (fg == 2) return acv_pick_model<V, TY, 2>(model);
    return acv_pick_model<V, TY, 1>(model);
}

template <int V>
static const void* acv_pick_ty(int ty, int fg, bool ws, int model)
{
    if (ty == 4) return acv_pick_fg<V, 4>(fg, ws, model);
    if (ty == 2) return acv_pick_fg<V, 2>(fg, ws, model);
    return nullptr;
}

// The warp-per-row kernel for rows of 64, 128 or 256 cells: 4-row strips
// (2 where 4 do not fit) and a ring of 3 slots, or 4 where the 3-slot ring
// already limits an SM to 3 blocks or fewer and the fourth slot keeps 2
// blocks, or loses none; two warps per row from 8 fields up; the
// producer/consumer form (4 slots) from 12 fields up and for 256-cell rows.
// Measured, us per step: 128^3 x 8 fields 35.1 (3 slots), 32.9 (4 slots),
// 31.9 (4 slots, 2 warps per row), 32.2 (the same, producer/consumer);
// 128^3 x 16: 114.5, 100.7, 87.0, 75.7; 128^3 x 3: 10.1 (3 slots), 10.6 (4),
// 14.6 (3 slots, 2 warps per row), 12.7 (producer/consumer); 96x64x256 x 6:
// 28.1 against 24.4 (producer/consumer).  MMSP_GPU_AC3_SHAPE=
// "rows,depth[,warps per row[,1]]" (rows 2 or 4, depth 3 to 6, warps 1, 2
// or 4, 1: the producer/consumer form) replaces the choice, "0,0" selects
// the kernel above.
static const void* acv_plan(const mmsp_gpu_desc& d, const Geom& g, int* R, int* D, int* FG, bool* WS)
{
    if (g.Z != 64 && g.Z != 128 && g.Z != 256) return nullptr;
    int ty = 4, dd = 0, fg = d.fields >= 8 ? 2 : 1;
    bool ws = false;
    if (const char* e = getenv("MMSP_GPU_AC3_SHAPE")) {
        int a = 0, b = 0, c = 0, w = 0;
        const int n = sscanf(e, "%d,%d,%d,%d", &a, &b, &c, &w);
        if (n >= 2) {
            if (a == 0) return nullptr;
            if ((a == 2 || a == 4) && b >= 3 && b <= 6) {
                ty = a;
                dd = b;
                fg = n >= 3 && (c == 1 || c == 2 || c == 4) ? c : 1;
                ws = n == 4 && w == 1;
            }
        }
    }
    const int fix = dd;
    // large slots (many fields, or 256-cell rows): the producer/consumer form
    // with two warps per row on a 4-slot ring
    if (!fix && (d.fields >= 12 || g.Z == 256)) {
        ws = true;
        fg = d.fields >= 2 ? 2 : 1;
    }
    if (!fix) dd = 3;
    while (ty > 2 && (g.Y < ty + 2 || ac3_smem(ty, g.Z, d.fields, dd) > kAcSmemCap)) ty /= 2;
    if (g.Y < ty + 2 || ac3_smem(ty, g.Z, d.fields, dd) > kAcSmemCap) return nullptr;
    if (!fix && ac3_smem(ty, g.Z, d.fields, 4) <= kAcSmemCap) {
        const int b3 = ac3_blocks_per_sm(ac3_smem(ty, g.Z, d.fields, 3));
        const int b4 = ac3_blocks_per_sm(ac3_smem(ty, g.Z, d.fields, 4));
        if (ws || (b3 <= 3 && (b4 >= 2 || b4 == b3))) dd = 4;
    }
    *R = ty;
    *D = dd;
    const int V = g.Z / 32;
    *FG = fg;
    *WS = ws;
    return V == 2 ? acv_pick_ty<2>(ty, fg, ws, d.model) : V == 4 ? acv_pick_ty<4>(ty, fg, ws, d.model)
                  : acv_pick_ty<8>(ty, fg, ws, d.model);
}

bool ac3_stream_eligible(const mmsp_gpu_desc& d, const Geom& g)
{
    int R, D, FG;
    bool WS;
    return d.dtype == MMSP_GPU_F32 && g.dim == 3 && g.Z <= 256 &&
           (d.model == MMSP_GPU_AC || d.model == MMSP_GPU_GG || d.model == MMSP_GPU_AC_POLY ||
            d.model == MMSP_GPU_ZENER) &&
           (acv_plan(d, g, &R, &D, &FG, &WS) || ac3_shape(g, d.fields, &R, &D));
}

cudaError_t plan_ac3_stream(const mmsp_gpu_desc& d, const Geom& g, StepPlan* p)
{
    int R = 4, D = 4, FG = 1;
    bool WS = false;
    int threads;
    if ((p->fn = acv_plan(d, g, &R, &D, &FG, &WS))) {
        // the pipelined form: computing warps along y, then the producer warp
        threads = WS ? 32 * (R * FG + 1) : 32 * R * FG;
        p->block = WS ? dim3(32, R * FG + 1, 1) : dim3(32, R, FG);
    } else {
        ac3_shape(g, d.fields, &R, &D);
        int RT, TY;
        ac3_threads(R, g.Z, d.fields, &RT, &TY);
        const int zt = (g.Z + 31) / 32 * 32;
        threads = zt * TY;
        p->fn = ac3_pick(RT, TY, g.Z, d.model);   // bulk copies when rows are 16-byte multiples
        if (!p->fn) return cudaErrorInvalidConfiguration;
        p->block = dim3(zt, TY, 1);
    }
    p->smem = ac3_smem(R, g.Z, d.fields, D) + (WS ? sizeof(uint64_t) * D : 0);   // + the "empty" barriers
    cudaError_t e = ensure_smem(p->fn, p->smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, p->fn, threads, p->smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    const int strips = (g.Y + R - 1) / R;
    long long slots = (long long)sm_count() * per_sm;
    int segs = (int)(slots / strips);
    if (segs < 1) segs = 1;
    if (segs > g.X) segs = g.X;
    p->planes = (g.X + segs - 1) / segs;
    segs = (g.X + p->planes - 1) / p->planes;
    p->grid = dim3(strips, segs, 1);
    p->fields = d.fields;
    p->kind = 2;
    p->ring = D;
    p->ok = true;
    return cudaSuccess;
}

cudaError_t launch_ac3_stream(const StepPlan& p, const Geom& g, const Coeffs& c, const void* in, void* out, int* err,
                              cudaStream_t s)
{
    AcF32 q;
    q.wx = (float)c.w[0];
    q.wy = (float)c.w[1];
    q.wz = (float)c.w[2];
    q.w2 = 2.0f * (q.wx + q.wy + q.wz);
    q.kappa = (float)c.kappa;
    q.dtm = (float)c.dtm;
    q.gamma2 = (float)c.gamma2;
    q.neg_r = (float)c.neg_r;
    q.u = (float)c.u;
    int planes = p.planes, n = p.fields, ring = p.ring;
    void* args[] = {(void*)&in, (void*)&out, (void*)&g, (void*)&q, (void*)&planes, (void*)&n, (void*)&ring, (void*)&err};
    return cudaLaunchKernel(p.fn, p.grid, p.block, args, p.smem, s);
}

}  // namespace pf
