// pf_ac3_stream.cu -- FP32 3D multi-order Allen-Cahn step, streaming along X.
//
// The precision-form kernel for 3D grids whose rows (axis Z) hold 32, 64,
// 128 or 256 cells.  A block owns R rows (axis Y) of full Z extent, one
// thread per cell of a row, and a run of X planes.  For every plane the
// block's R+2 rows (one halo row each side, wrapped periodically) of all N
// fields arrive in shared memory through cp.async.bulk (one copy per field,
// two where the rows wrap) on a D-deep mbarrier ring.  With D = 3 the copy
// of plane x+2 is issued as soon as plane x-1 is released; the copies of the
// several blocks resident on an SM overlap each other's computation.  Per cell the sum of squares
// over the fields comes first, then each field's new value from its own
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

static size_t ac3_smem(int R, int Z, int N, int D) { return sizeof(float) * (size_t)D * N * (R + 2) * Z + sizeof(uint64_t) * D; }

template <int R, int Z, int MODEL>
__global__ void __launch_bounds__(Z)
ac3_stream_f32(const float* __restrict__ ein, float* __restrict__ eout, Geom g, AcF32 q, int planes, int N, int D,
               int* __restrict__ err)
{
    constexpr int RR = R + 2;
    const int z = threadIdx.x;
    extern __shared__ __align__(128) unsigned char sm[];
    float* slots = reinterpret_cast<float*>(sm);
    const size_t slot_elems = (size_t)N * RR * Z;
    uint64_t* bars = reinterpret_cast<uint64_t*>(slots + (size_t)D * slot_elems);
    __shared__ int s_err;

    const int y0 = blockIdx.x * R;
    const int xs = blockIdx.y * planes;
    const int xe = min(xs + planes, g.X);
    if (xs >= xe) return;
    const int zl = z == 0 ? Z - 1 : z - 1;
    const int zh = z == Z - 1 ? 0 : z + 1;
    const int x_first = xs - 1, x_last = xe;   // planes read from global memory
    const long long cells = g.cells;

    auto fill = [&](int pl) {
        const int k = pl - x_first, s = k % D;
        uint64_t* bar = &bars[s];
        float* dst0 = slots + (size_t)s * slot_elems;
        const long long plane = (long long)wrapi(pl, g.X) * g.YZ;
        constexpr uint32_t row = (uint32_t)Z * sizeof(float);
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
    };
    auto slot_of = [&](int pl) -> const float* { return slots + (size_t)((pl - x_first) % D) * slot_elems; };
    auto wait_plane = [&](int pl) {
        const int k = pl - x_first;
        if (!mbar_wait(&bars[k % D], (uint32_t)(k / D) & 1u)) {
            s_err = 1;
            atomicExch(err, 1);
        }
    };

    if (z == 0) {
        for (int s = 0; s < D; s++) mbar_init(&bars[s], 1);
        mbar_fence_init();
        s_err = 0;
    }
    __syncthreads();
    if (z == 0)
        for (int pl = x_first; pl < x_first + D && pl <= x_last; pl++) fill(pl);
    wait_plane(x_first);
    wait_plane(x_first + 1);

    int x = xs;
    for (; x < xe && !s_err; x++) {
        wait_plane(x + 1);
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
                const int o = (int)fo + (r + 1) * Z;
                const float cc = col[r + 1];
                const float sx = SL[o + z] + SH[o + z];
                const float sy = col[r] + col[r + 2];
                const float sz = SC[o + zl] + SC[o + zh];
                const float lap = fmaf(q.wx, sx, fmaf(q.wy, sy, fmaf(q.wz, sz, -q.w2 * cc)));
                if (r < rows) dst[(long long)r * Z] = ac_new_f32<MODEL>(cc, sum[r], lap, q);
            }
        }
        __syncthreads();
        if (z == 0 && !s_err && x - 1 + D <= x_last) fill(x - 1 + D);   // slot of x-1 is free now
    }
    if (s_err && z == 0) {
        for (int pl = max(x - 1, x_first); pl <= min(x - 1 + D, x_last); pl++) {
            const int k = pl - x_first;
            mbar_wait(&bars[k % D], (uint32_t)(k / D) & 1u);
        }
    }
}

template <int R, int Z>
static const void* ac3_pick_model(int model)
{
    if (model == MMSP_GPU_AC) return (const void*)&ac3_stream_f32<R, Z, MMSP_GPU_AC>;
    if (model == MMSP_GPU_GG) return (const void*)&ac3_stream_f32<R, Z, MMSP_GPU_GG>;
    return (const void*)&ac3_stream_f32<R, Z, MMSP_GPU_AC_POLY>;
}

template <int R>
static const void* ac3_pick_z(int Z, int model)
{
    switch (Z) {
    case 32: return ac3_pick_model<R, 32>(model);
    case 64: return ac3_pick_model<R, 64>(model);
    case 128: return ac3_pick_model<R, 128>(model);
    default: return ac3_pick_model<R, 256>(model);
    }
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
    static const int kR[] = {4, 2, 2, 2};
    static const int kD[] = {3, 3, 3, 3};
    for (int i = 0; i < 4; i++)
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
    const bool rows = g.Z == 32 || g.Z == 64 || g.Z == 128 || g.Z == 256;
    return d.dtype == MMSP_GPU_F32 && g.dim == 3 && rows &&
           (d.model == MMSP_GPU_AC || d.model == MMSP_GPU_GG || d.model == MMSP_GPU_AC_POLY) &&
           ac3_shape(g, d.fields, &R, &D);
}

cudaError_t plan_ac3_stream(const mmsp_gpu_desc& d, const Geom& g, StepPlan* p)
{
    int R = 4, D = 4;
    ac3_shape(g, d.fields, &R, &D);
    p->fn = R == 4 ? ac3_pick_z<4>(g.Z, d.model) : ac3_pick_z<2>(g.Z, d.model);
    p->smem = ac3_smem(R, g.Z, d.fields, D);
    p->block = dim3(g.Z, 1, 1);
    cudaError_t e = ensure_smem(p->fn, p->smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, p->fn, g.Z, p->smem);
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
