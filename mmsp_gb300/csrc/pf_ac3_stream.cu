// pf_ac3_stream.cu -- FP32 3D multi-order Allen-Cahn step, streaming along X.
//
// The precision-form kernel for 3D grids with rows (axis Z) of up to 256
// cells.  A block owns R rows (axis Y) of full Z extent, one
// thread per cell of a row, and a run of X planes.  For every plane the
// block's R+2 rows (one halo row each side, wrapped periodically) of all N
// fields arrive in shared memory through cp.async.bulk (one copy per field,
// two where the rows wrap) on a D-deep mbarrier ring.  With D = 3 the copy
// of plane x+2 is issued as soon as plane x-1 is released; the copies of the
// several blocks resident on an SM overlap each other's computation.  Per
// cell the sum of squares over the fields comes first, then each field's
// new value from its own
// 7-point Laplacian; Y neighbours are registers, X and Z neighbours are read
// from shared memory (Z wraps across the row).  There is no Z halo, and the
// Y halo costs 2 extra rows per R-row strip in reads only.
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
    } else if (MODEL == MMSP_GPU_GG) {
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

// BULK: rows are a multiple of 16 bytes, and thread 0 stages each field's
// rows with cp.async.bulk (transaction-counted mbarrier, one arrival).
// Otherwise every thread copies its own cells with 4-byte cp.async and
// arrives on the mbarrier when they land (one arrival per thread).
template <int R, int MODEL, bool BULK>
__global__ void __launch_bounds__(256)
ac3_stream_f32(const float* __restrict__ ein, float* __restrict__ eout, Geom g, AcF32 q, int planes, int N, int D,
               int* __restrict__ err)
{
    constexpr int RR = R + 2;
    const int Z = g.Z;
    const int t = threadIdx.x;
    const bool on = t < Z;
    const int z = on ? t : 0;
    extern __shared__ __align__(128) unsigned char sm[];
    float* slots = reinterpret_cast<float*>(sm);
    const size_t slot_elems = (size_t)N * RR * Z;
    uint64_t* bars = reinterpret_cast<uint64_t*>(slots + (((size_t)D * slot_elems + 1) & ~(size_t)1));

    const int y0 = blockIdx.x * R;
    const int xs = blockIdx.y * planes;
    const int xe = min(xs + planes, g.X);
    if (xs >= xe) return;
    const int zl = z == 0 ? Z - 1 : z - 1;
    const int zh = z == Z - 1 ? 0 : z + 1;
    const int x_first = xs - 1, x_last = xe;   // planes read from global memory
    const long long cells = g.cells;

    // BULK: called by thread 0 only; otherwise by every thread
    auto fill = [&](int pl) {
        const int k = pl - x_first, s = k % D;
        uint64_t* bar = &bars[s];
        float* dst0 = slots + (size_t)s * slot_elems;
        const long long plane = (long long)wrapi(pl, g.X) * g.YZ;
        if constexpr (BULK) {
            const uint32_t row = (uint32_t)Z * sizeof(float);
            fence_proxy_async();
            mbar_expect_tx(bar, (uint32_t)N * RR * row);
            const int a = y0 - 1, b = y0 + R + 1;
            for (int f = 0; f < N; f++) {
                const float* base = ein + (long long)f * cells + plane;
                float* dst = dst0 + (size_t)f * RR * Z;
                if (a >= 0 && b <= g.Y) {
                    bulk_g2s(dst, base + (long long)a * Z, RR * row, bar);
                } else if (a < 0) {
                    bulk_g2s(dst, base + (long long)(g.Y - 1) * Z, row, bar);
                    bulk_g2s(dst + Z, base, (RR - 1) * row, bar);
                } else {
                    const int n1 = g.Y - a;
                    bulk_g2s(dst, base + (long long)a * Z, n1 * row, bar);
                    bulk_g2s(dst + (size_t)n1 * Z, base, (RR - n1) * row, bar);
                }
            }
        } else {
            if (on)
                for (int f = 0; f < N; f++) {
                    const float* base = ein + (long long)f * cells + plane + z;
                    float* dst = dst0 + (size_t)f * RR * Z + z;
#pragma unroll
                    for (int r = 0; r < RR; r++) cp_async4(dst + r * Z, base + (long long)wrapi(y0 - 1 + r, g.Y) * Z);
                }
            cp_async_arrive(bar);
        }
    };
    auto slot_of = [&](int pl) -> const float* { return slots + (size_t)((pl - x_first) % D) * slot_elems; };
    auto arrived = [&](int pl) {
        const int k = pl - x_first;
        return mbar_wait(&bars[k % D], (uint32_t)(k / D) & 1u);
    };

    if (t == 0) {
        for (int s = 0; s < D; s++) mbar_init(&bars[s], BULK ? 1 : blockDim.x);
        mbar_fence_init();
    }
    __syncthreads();
    int issued = min(x_first + D - 1, x_last);   // last plane whose fill was issued
    if (!BULK || t == 0)
        for (int pl = x_first; pl <= issued; pl++) fill(pl);
    bool bad = !arrived(x_first);
    bad |= !arrived(x_first + 1);
    // The decision to stop is taken block-wide (__syncthreads_or), so every
    // thread leaves the loop at the same barrier.
    bool stop = __syncthreads_or(bad);

    for (int x = xs; x < xe && !stop; x++) {
        bad = !arrived(x + 1);
        const float* SL = slot_of(x - 1);
        const float* SC = slot_of(x);
        const float* SH = slot_of(x + 1);
        float sum[R];
#pragma unroll
        for (int r = 0; r < R; r++) sum[r] = 0.0f;
#pragma unroll 1
        for (int f = 0; f < N; f++) {
            const float* c = SC + (size_t)f * RR * Z + z;
#pragma unroll
            for (int r = 0; r < R; r++) {
                const float v = c[(r + 1) * Z];
                sum[r] = fmaf(v, v, sum[r]);
            }
        }
        const int rows = min(R, g.Y - y0);
#pragma unroll 1
        for (int f = 0; f < N; f++) {
            const size_t fo = (size_t)f * RR * Z;
            float col[RR];
#pragma unroll
            for (int r = 0; r < RR; r++) col[r] = SC[fo + r * Z + z];
            float* dst = eout + (long long)f * cells + (long long)x * g.YZ + (long long)y0 * Z + z;
#pragma unroll
            for (int r = 0; r < R; r++) {
                const size_t o = fo + (size_t)(r + 1) * Z;
                const float cc = col[r + 1];
                const float sx = SL[o + z] + SH[o + z];
                const float sy = col[r] + col[r + 2];
                const float sz = SC[o + zl] + SC[o + zh];
                const float lap = fmaf(q.wx, sx, fmaf(q.wy, sy, fmaf(q.wz, sz, -q.w2 * cc)));
                if (on && r < rows) dst[(long long)r * Z] = ac_new_f32<MODEL>(cc, sum[r], lap, q);
            }
        }
        stop = __syncthreads_or(bad);
        if (!stop && x - 1 + D <= x_last) {   // the slot of x-1 is free now
            if (!BULK || t == 0) fill(x - 1 + D);
            issued = x - 1 + D;
        }
    }
    if (stop) {
        if (t == 0) atomicExch(err, 1);
        // leave no copy in flight: wait (bounded) for the last fill of every slot
        for (int pl = max(x_first, issued - D + 1); pl <= issued; pl++) arrived(pl);
    }
}

template <int R, bool BULK>
static const void* ac3_pick_model(int model)
{
    if (model == MMSP_GPU_AC) return (const void*)&ac3_stream_f32<R, MMSP_GPU_AC, BULK>;
    if (model == MMSP_GPU_GG) return (const void*)&ac3_stream_f32<R, MMSP_GPU_GG, BULK>;
    return (const void*)&ac3_stream_f32<R, MMSP_GPU_AC_POLY, BULK>;
}

static const void* ac3_pick(int R, bool bulk, int model)
{
    if (R == 4) return bulk ? ac3_pick_model<4, true>(model) : ac3_pick_model<4, false>(model);
    if (R == 2) return bulk ? ac3_pick_model<2, true>(model) : ac3_pick_model<2, false>(model);
    return bulk ? ac3_pick_model<1, true>(model) : ac3_pick_model<1, false>(model);
}

constexpr size_t kAcSmemCap = 200 * 1024;

// Rows per strip and ring depth: the first pair whose shared memory fits.
// Measured on 128^3 grids (N = 4, 8, 16 fields), more resident blocks beat a
// deeper ring: a 3-plane ring (no plane in flight beyond the three being
// read) with 4-row strips was fastest wherever it fit.
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
    static const int kD[] = {3, 3, 3};
    for (int i = 0; i < 3; i++)
        if (g.Y >= kR[i] + 2 && ac3_smem(kR[i], g.Z, N, kD[i]) <= kAcSmemCap) {
            *R = kR[i];
            *D = kD[i];
            return true;
        }
    return false;
}

bool ac3_stream_eligible(const mmsp_gpu_desc& d, const Geom& g)
{
    int R, D;
    return d.dtype == MMSP_GPU_F32 && g.dim == 3 && g.Z <= 256 &&
           (d.model == MMSP_GPU_AC || d.model == MMSP_GPU_GG || d.model == MMSP_GPU_AC_POLY) &&
           ac3_shape(g, d.fields, &R, &D);
}

cudaError_t plan_ac3_stream(const mmsp_gpu_desc& d, const Geom& g, StepPlan* p)
{
    int R = 4, D = 4;
    ac3_shape(g, d.fields, &R, &D);
    const bool bulk = g.Z % 4 == 0;   // 16-byte rows
    const int threads = (g.Z + 31) / 32 * 32;
    p->fn = ac3_pick(R, bulk, d.model);
    p->smem = ac3_smem(R, g.Z, d.fields, D);
    p->block = dim3(threads, 1, 1);
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
