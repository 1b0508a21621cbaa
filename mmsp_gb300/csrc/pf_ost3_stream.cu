// pf_ost3_stream.cu -- FP32 3D Ostwald-ripening step in one kernel,
// streaming along X.
//
// The reference's update (examples/coarsening/ostwald_ripening/isotropic/
// phase_field/ostwald.cpp:84-122) makes two passes: the chemical potential
// w of the composition C (field 0) over the whole grid (:89-100), then the
// new composition from the Laplacian of w and the new order parameters
// e_j (fields 1..N-1) from their own Laplacians (:103-120).  Here one
// kernel does both for rows (axis Z) of 32, 64 or 128 cells: a block owns R
// rows (axis Y) of full Z extent and walks a run of X planes.
//
// * Every plane's R+4 rows (2 halo rows each side, wrapped periodically) of
//   all fields arrive in shared memory on an mbarrier ring by cp.async.bulk
//   (rows are 16-byte multiples), D planes deep: planes x-1 .. x+2 are in
//   use while plane x is updated, the rest are copies in flight.
// * A warp owns RT consecutive rows of the strip.  For plane x it computes
//   w(x+1) on its rows and one row either side (the neighbouring warps
//   compute those rows again), then updates plane x from w(x-1), w(x),
//   w(x+1), which stay in its registers, and the staged fields.  w never
//   goes to shared or global memory, the warps meet only at one barrier per
//   plane (the release of a ring slot), and each step reads the state once
//   (plus halo re-reads that hit L2) and writes it once.
// * A warp spans a row, V = Z/32 adjacent cells per lane; Z neighbours at a
//   lane's ends come from the adjacent lanes by shuffle (lane 0 and lane 31
//   are neighbours: the periodic wrap of the row).
//
// FP32 arithmetic is regrouped for throughput (neighbour sums before the
// weights) and runs on pairs of cells in packed FP32x2 instructions; the
// result is checked against the FP64 oracle with a tolerance, not bitwise.  Every wait is bounded: a wait that runs out sets
// the error word, and the block waits (bounded) for its copies in flight
// and leaves.
#include "pf_async.cuh"
#include "pf_device.cuh"
#include "pf_internal.h"

namespace pf {

struct OstF32 {
    float wx, wy, wz, w2;   // Laplacian weights, w2 = 2(wx+wy+wz)
    float Cm, Ca, Cb, negA, B, Da, Db, g, neg_g, delta, eps, kappa, dtD, dtL;
};

// A lane's V cells as NP packs: float2 pairs (V = 2, 4), whose arithmetic
// runs in packed FP32x2 instructions (one instruction for both cells), or
// one float (V = 1).
template <int V> struct Pack { using T = float2; static constexpr int NP = V / 2; };
template <> struct Pack<1> { using T = float; static constexpr int NP = 1; };

static __device__ __forceinline__ float padd(float a, float b) { return a + b; }
static __device__ __forceinline__ float2 padd(float2 a, float2 b) { return __fadd2_rn(a, b); }
static __device__ __forceinline__ float pmul(float a, float b) { return a * b; }
static __device__ __forceinline__ float2 pmul(float2 a, float2 b) { return __fmul2_rn(a, b); }
static __device__ __forceinline__ float pfma(float a, float b, float c) { return fmaf(a, b, c); }
static __device__ __forceinline__ float2 pfma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
template <typename T> static __device__ __forceinline__ T splat(float k);
template <> __device__ __forceinline__ float splat<float>(float k) { return k; }
template <> __device__ __forceinline__ float2 splat<float2>(float k) { return make_float2(k, k); }

template <int V>
static __device__ __forceinline__ void ldp(const float* p, typename Pack<V>::T (&v)[Pack<V>::NP])
{
    if constexpr (V == 4) {
        const float4 t = *reinterpret_cast<const float4*>(p);
        v[0] = make_float2(t.x, t.y);
        v[1] = make_float2(t.z, t.w);
    } else if constexpr (V == 2) {
        v[0] = *reinterpret_cast<const float2*>(p);
    } else {
        v[0] = *p;
    }
}

template <int V>
static __device__ __forceinline__ void stp(float* p, const typename Pack<V>::T (&v)[Pack<V>::NP])
{
    if constexpr (V == 4) *reinterpret_cast<float4*>(p) = make_float4(v[0].x, v[0].y, v[1].x, v[1].y);
    else if constexpr (V == 2) *reinterpret_cast<float2*>(p) = v[0];
    else *p = v[0];
}

// Sums of the two Z neighbours of each of a lane's V cells (the row wraps
// across lanes 31 and 0).  Scalar adds, so no pairs are built before them.
template <int V>
static __device__ __forceinline__ void zsum(const typename Pack<V>::T (&c)[Pack<V>::NP], int lane,
                                            typename Pack<V>::T (&s)[Pack<V>::NP])
{
    constexpr int NP = Pack<V>::NP;
    if constexpr (V == 1) {
        const float left = __shfl_sync(0xffffffffu, c[0], (lane + 31) & 31);
        const float right = __shfl_sync(0xffffffffu, c[0], (lane + 1) & 31);
        s[0] = left + right;
    } else {
        const float left = __shfl_sync(0xffffffffu, c[NP - 1].y, (lane + 31) & 31);
        const float right = __shfl_sync(0xffffffffu, c[0].x, (lane + 1) & 31);
#pragma unroll
        for (int i = 0; i < NP; i++) {
            const float lo = i == 0 ? left : c[i - 1].y;
            const float hi = i == NP - 1 ? right : c[i + 1].x;
            s[i] = make_float2(lo + c[i].y, c[i].x + hi);
        }
    }
}

// wx*sx + wy*sy + wz*sz - 2(wx+wy+wz)*c from the neighbour sums along each axis
template <bool UNIT, typename T>
static __device__ __forceinline__ T lap3(T sx, T sy, T sz, T c, const OstF32& q)
{
    if (UNIT) return pfma(splat<T>(-6.0f), c, padd(padd(sx, sy), sz));
    return pfma(splat<T>(q.wx), sx, pfma(splat<T>(q.wy), sy, pfma(splat<T>(q.wz), sz, pmul(splat<T>(-q.w2), c))));
}

// V = Z/32 cells per lane, TY warps, RT update rows per warp (R = TY*RT rows
// per strip), NF fields, D ring slots (D >= 5: four planes in use).
template <int V, int TY, int RT, int NF, int D, bool UNIT>
__global__ void __launch_bounds__(32 * TY)
ost3_stream_f32(const float* __restrict__ sin, float* __restrict__ sout, Geom g, OstF32 q, int planes,
                int* __restrict__ err)
{
    constexpr int Z = 32 * V, R = TY * RT, RR = R + 4;
    constexpr int FS = RR * Z;        // floats of one field's rows in a slot
    constexpr int SS = NF * FS;       // floats of a slot
    constexpr int NP = Pack<V>::NP;
    using T = typename Pack<V>::T;
    static_assert(D >= 5 && NF >= 2, "ring depth, fields");
    extern __shared__ __align__(128) unsigned char sm[];
    float* ring = reinterpret_cast<float*>(sm);
    uint64_t* bars = reinterpret_cast<uint64_t*>(ring + D * SS);

    const int t = threadIdx.x, lane = t & 31, ty = t >> 5;
    const int z0 = lane * V;
    const int r0 = ty * RT;           // this warp's first row of the strip
    const int y0 = blockIdx.x * R;
    const int xs = blockIdx.y * planes, xe = min(xs + planes, g.X);
    if (xs >= xe) return;
    const int x_first = xs - 2, x_last = xe + 1;   // planes read from global memory
    const long long cells = g.cells;

    // thread 0: stage plane pl (wrapped) of every field into its slot; slot
    // row i holds strip row i-2
    auto fill = [&](int pl) {
        const int k = pl - x_first, s = k % D;
        uint64_t* bar = &bars[s];
        float* dst0 = ring + s * SS;
        const long long plane = (long long)wrapi(pl, g.X) * g.YZ;
        constexpr uint32_t row = Z * sizeof(float);
        fence_proxy_async();
        mbar_expect_tx(bar, (uint32_t)(NF * RR) * row);
        const int a = y0 - 2, b = y0 + R + 2;
#pragma unroll
        for (int f = 0; f < NF; f++) {
            const float* base = sin + (long long)f * cells + plane;
            float* dst = dst0 + f * FS;
            if (a >= 0 && b <= g.Y) {
                bulk_g2s(dst, base + (long long)a * Z, RR * row, bar);
            } else if (a < 0) {   // rows Y-2, Y-1, then 0 ..
                bulk_g2s(dst, base + (long long)(g.Y + a) * Z, -a * row, bar);
                bulk_g2s(dst + (-a) * Z, base, (RR + a) * row, bar);
            } else {              // rows a .. Y-1, then 0 ..
                const int n1 = g.Y - a;
                bulk_g2s(dst, base + (long long)a * Z, n1 * row, bar);
                bulk_g2s(dst + n1 * Z, base, (RR - n1) * row, bar);
            }
        }
    };
    auto slot = [&](int pl) -> const float* { return ring + ((pl - x_first) % D) * SS; };
    auto arrived = [&](int pl) {
        const int k = pl - x_first;
        return mbar_wait(&bars[k % D], (uint32_t)(k / D) & 1u);
    };

    // w(xp) on this warp's rows r0-1 .. r0+RT (ostwald.cpp:95-99), into w:
    //   w = -A*(C-Cm) + B*(C-Cm)^3 + Da*(C-Ca)^3 + Db*(C-Cb)^3 - g*(C-Ca)*sum - kappa*lap C
    // with sum the squares of the order parameters; planes xp-1, xp, xp+1
    // staged.  The rows either side of the warp's own are computed again by
    // the neighbouring warps, so w never leaves registers.
    auto compute_w = [&](int xp, T (&w)[RT + 2][NP]) {
        const float* sl = slot(xp - 1);
        const float* sc = slot(xp);
        const float* sh = slot(xp + 1);
        T c[RT + 4][NP];   // C(xp) on rows r0-2 .. r0+RT+1 (slot rows r0 .. r0+RT+3)
#pragma unroll
        for (int k = 0; k < RT + 4; k++) ldp<V>(sc + (r0 + k) * Z + z0, c[k]);
#pragma unroll
        for (int k = 0; k < RT + 2; k++) {   // row r0-1+k
            const int o = (r0 + 1 + k) * Z + z0;
            T xh[NP], xl[NP], sz[NP], sum[NP], e[NP];
            ldp<V>(sl + o, xl);
            ldp<V>(sh + o, xh);
            ldp<V>(sc + FS + o, e);
#pragma unroll
            for (int i = 0; i < NP; i++) sum[i] = pmul(e[i], e[i]);
#pragma unroll
            for (int j = 2; j < NF; j++) {
                ldp<V>(sc + j * FS + o, e);
#pragma unroll
                for (int i = 0; i < NP; i++) sum[i] = pfma(e[i], e[i], sum[i]);
            }
            zsum<V>(c[k + 1], lane, sz);
#pragma unroll
            for (int i = 0; i < NP; i++) {
                const T cc = c[k + 1][i];
                const T lap = lap3<UNIT>(padd(xh[i], xl[i]), padd(c[k][i], c[k + 2][i]), sz[i], cc, q);
                const T dm = padd(cc, splat<T>(-q.Cm)), da = padd(cc, splat<T>(-q.Ca)), db = padd(cc, splat<T>(-q.Cb));
                T r = pfma(pmul(splat<T>(q.B), dm), pmul(dm, dm), pmul(splat<T>(q.negA), dm));
                r = pfma(pmul(splat<T>(q.Da), da), pmul(da, da), r);
                r = pfma(pmul(splat<T>(q.Db), db), pmul(db, db), r);
                r = pfma(pmul(splat<T>(-q.g), da), sum[i], r);
                w[k][i] = pfma(splat<T>(-q.kappa), lap, r);
            }
        }
    };

    // Plane x on this warp's rows r0 .. r0+RT-1 (ostwald.cpp:103-120), from
    // wa = w(x-1), wb = w(x), wc = w(x+1):
    //   C'   = C + dt*D*lap w
    //   e_j' = e_j - dt*L*(-g*(C-Ca)^2 + delta*e_j^3 + eps*e_j*(sum - e_j^2) - kappa*lap e_j)
    auto update = [&](int x, const T (&wa)[RT + 2][NP], const T (&wb)[RT + 2][NP], const T (&wc)[RT + 2][NP]) {
        const float* sl = slot(x - 1);
        const float* sc = slot(x);
        const float* sh = slot(x + 1);
        // every order parameter at plane x on rows r0-1 .. r0+RT
        T ec[NF - 1][RT + 2][NP];
#pragma unroll
        for (int k = 0; k < RT + 2; k++)
#pragma unroll
            for (int j = 1; j < NF; j++) ldp<V>(sc + j * FS + (r0 + k + 1) * Z + z0, ec[j - 1][k]);
        float* dst = sout + (long long)x * g.YZ + (long long)(y0 + r0) * Z + z0;
#pragma unroll
        for (int k = 0; k < RT; k++) {
            const bool inside = y0 + r0 + k < g.Y;
            const int o = (r0 + k + 2) * Z + z0;   // slot row of row r0+k
            T a[NP], b[NP], sz[NP], C[NP], out[NP], sum[NP], t1[NP];
            ldp<V>(sc + o, C);
            zsum<V>(wb[k + 1], lane, sz);
#pragma unroll
            for (int i = 0; i < NP; i++) {
                const T lap = lap3<UNIT>(padd(wa[k + 1][i], wc[k + 1][i]), padd(wb[k][i], wb[k + 2][i]), sz[i],
                                         wb[k + 1][i], q);
                out[i] = pfma(splat<T>(q.dtD), lap, C[i]);
            }
            if (inside) stp<V>(dst + (long long)k * Z, out);
#pragma unroll
            for (int i = 0; i < NP; i++) {
                sum[i] = pmul(ec[0][k + 1][i], ec[0][k + 1][i]);
#pragma unroll
                for (int j = 1; j < NF - 1; j++) sum[i] = pfma(ec[j][k + 1][i], ec[j][k + 1][i], sum[i]);
                const T da = padd(C[i], splat<T>(-q.Ca));
                t1[i] = pmul(splat<T>(q.neg_g), pmul(da, da));
            }
#pragma unroll
            for (int j = 1; j < NF; j++) {
                const T(&e)[NP] = ec[j - 1][k + 1];
                ldp<V>(sl + j * FS + o, a);
                ldp<V>(sh + j * FS + o, b);
                zsum<V>(e, lane, sz);
#pragma unroll
                for (int i = 0; i < NP; i++) {
                    const T lap = lap3<UNIT>(padd(a[i], b[i]), padd(ec[j - 1][k][i], ec[j - 1][k + 2][i]), sz[i], e[i], q);
                    const T e2 = pmul(e[i], e[i]);
                    T r = pfma(pmul(splat<T>(q.delta), e[i]), e2, t1[i]);
                    r = pfma(pmul(splat<T>(q.eps), e[i]), pfma(splat<T>(-1.0f), e2, sum[i]), r);
                    r = pfma(splat<T>(-q.kappa), lap, r);
                    out[i] = pfma(splat<T>(-q.dtL), r, e[i]);
                }
                if (inside) stp<V>(dst + (long long)j * cells + (long long)k * Z, out);
            }
        }
    };

    if (t == 0) {
        for (int s = 0; s < D; s++) mbar_init(&bars[s], 1);
        mbar_fence_init();
    }
    __syncthreads();
    int issued = min(x_first + D - 1, x_last);   // thread 0: the last plane whose fill was issued
    if (t == 0)
        for (int pl = x_first; pl <= issued; pl++) fill(pl);
    // warm-up: w(xs-1) and w(xs) from planes xs-2 .. xs+1.  Whether to stop
    // is decided block-wide at a barrier (__syncthreads_or), so every thread
    // leaves the loop at the same point.
    T wA[RT + 2][NP], wB[RT + 2][NP], wC[RT + 2][NP];
    bool bad = false;
    for (int pl = x_first; pl <= xs + 1; pl++) bad |= !arrived(pl);
    compute_w(xs - 1, wA);
    compute_w(xs, wB);
    bool stop = __syncthreads_or(bad);
    if (!stop && t == 0 && x_first + D <= x_last) fill(issued = x_first + D);   // the slot of xs-2 is free

    // One plane: w(x+1) into wc, then plane x.  (A failed wait computes and
    // stores garbage for this plane; the error word reports the step.)
    auto iter = [&](int x, const T (&wa)[RT + 2][NP], const T (&wb)[RT + 2][NP], T (&wc)[RT + 2][NP]) {
        const bool late = !arrived(x + 2);
        compute_w(x + 1, wc);
        update(x, wa, wb, wc);
        if (__syncthreads_or(late)) return false;
        // the slot of plane x-1 is free now
        if (t == 0 && x - 1 + D <= x_last) fill(issued = x - 1 + D);
        return true;
    };
    int x = xs;
    while (!stop) {
        if (x >= xe) break;
        if (!iter(x, wA, wB, wC)) { stop = true; break; }
        if (++x >= xe) break;
        if (!iter(x, wB, wC, wA)) { stop = true; break; }
        if (++x >= xe) break;
        if (!iter(x, wC, wA, wB)) { stop = true; break; }
        ++x;
    }
    if (stop && t == 0) {
        atomicExch(err, 1);
        // leave no copy in flight: wait (bounded) for every fill not yet consumed
        for (int pl = max(x_first, issued - D + 1); pl <= issued; pl++) arrived(pl);
    }
}

// The instance for rows of 32*V cells and N fields: warps, rows per warp and
// ring depth of its shape.
struct OstKernel {
    const void* fn;
    int ty, rt, d;
};

template <int V, int TY, int RT, int D>
static OstKernel ost3_k(int N, bool unit)
{
    OstKernel k{nullptr, TY, RT, D};
    if (N == 2) k.fn = unit ? (const void*)&ost3_stream_f32<V, TY, RT, 2, D, true>
                            : (const void*)&ost3_stream_f32<V, TY, RT, 2, D, false>;
    if (N == 3) k.fn = unit ? (const void*)&ost3_stream_f32<V, TY, RT, 3, D, true>
                            : (const void*)&ost3_stream_f32<V, TY, RT, 3, D, false>;
    if (N == 4) k.fn = unit ? (const void*)&ost3_stream_f32<V, TY, RT, 4, D, true>
                            : (const void*)&ost3_stream_f32<V, TY, RT, 4, D, false>;
    return k;
}

// Measured on 256x128x64 x 2 fields (us per step; warps, rows per warp,
// ring depth): 10.7 (4, 4, 6), 10.9 (4, 4, 5), 11.0 (8, 4, 5) and (4, 8, 5),
// 12.1 (8, 2, 6), 12.6 (2, 8, 6), 15.6 (8, 1, 6); the same step with w in a
// shared-memory ring and a barrier between the two halves: 12.5.
static OstKernel ost3_pick(int V, int N, bool unit)
{
    if (V == 1) return ost3_k<1, 8, 2, 6>(N, unit);
    if (V == 4) return ost3_k<4, 4, 2, 5>(N, unit);
    return ost3_k<2, 4, 4, 6>(N, unit);
}

bool ost3_stream_eligible(const mmsp_gpu_desc& d, const Geom& g)
{
    if (d.dtype != MMSP_GPU_F32 || g.dim != 3 || d.fields < 2 || d.fields > 4) return false;
    if (g.Z != 32 && g.Z != 64 && g.Z != 128) return false;
    const OstKernel k = ost3_pick(g.Z / 32, d.fields, true);
    return g.Y >= k.ty * k.rt + 4 && g.X >= 4;
}

cudaError_t plan_ost3_stream(const mmsp_gpu_desc& d, const Geom& g, const Coeffs& c, StepPlan* p)
{
    const int V = g.Z / 32;
    const int N = d.fields;
    const OstKernel k = ost3_pick(V, N, c.unit_w);
    if (!k.fn) return cudaErrorInvalidConfiguration;
    const int R = k.ty * k.rt;
    p->fn = k.fn;
    p->smem = sizeof(float) * (size_t)k.d * N * (R + 4) * g.Z + sizeof(uint64_t) * k.d;
    p->block = dim3(32 * k.ty, 1, 1);
    cudaError_t e = ensure_smem(p->fn, p->smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, p->fn, (int)p->block.x, p->smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    const int strips = (g.Y + R - 1) / R;
    // one wave: strips * segments <= resident blocks, segments >= 1
    const long long slots = (long long)sm_count() * per_sm;
    int segs = (int)(slots / strips);
    if (segs < 1) segs = 1;
    if (segs > g.X) segs = g.X;
    p->planes = (g.X + segs - 1) / segs;
    segs = (g.X + p->planes - 1) / p->planes;
    p->grid = dim3(strips, segs, 1);
    p->fields = N;
    p->kind = 8;
    p->ring = 0;
    p->ok = true;
    return cudaSuccess;
}

cudaError_t launch_ost3_stream(const StepPlan& p, const Geom& g, const OstConst& o, const Coeffs& c,
                               const void* in, void* out, int* err, cudaStream_t s)
{
    OstF32 q;
    q.wx = (float)c.w[0];
    q.wy = (float)c.w[1];
    q.wz = (float)c.w[2];
    q.w2 = 2.0f * (q.wx + q.wy + q.wz);
    q.Cm = (float)o.Cm;
    q.Ca = (float)o.Ca;
    q.Cb = (float)o.Cb;
    q.negA = (float)(-o.A);
    q.B = (float)o.B;
    q.Da = (float)o.Da;
    q.Db = (float)o.Db;
    q.g = (float)o.g;
    q.neg_g = (float)(-o.g);
    q.delta = (float)o.delta;
    q.eps = (float)o.eps;
    q.kappa = (float)o.kappa;
    q.dtD = (float)o.dtD;
    q.dtL = (float)o.dtL;
    int planes = p.planes;
    Geom gg = g;
    void* args[] = {(void*)&in, (void*)&out, (void*)&gg, (void*)&q, (void*)&planes, (void*)&err};
    return cudaLaunchKernel(p.fn, p.grid, p.block, args, p.smem, s);
}

}  // namespace pf
