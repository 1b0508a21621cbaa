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
// * For plane x the block first computes w(x+1) on rows -1..R into a ring of
//   three w planes in shared memory, then updates plane x from w(x-1),
//   w(x), w(x+1) and the staged fields.  w never goes to global memory:
//   each step reads the state once (plus halo re-reads that hit L2) and
//   writes it once.
// * A warp spans a row, V = Z/32 adjacent cells per lane; Z neighbours at a
//   lane's ends come from the adjacent lanes by shuffle (lane 0 and lane 31
//   are neighbours: the periodic wrap of the row).  Warps take w rows in
//   turn and RT consecutive rows of the update, whose Y neighbours stay in
//   registers.
//
// FP32 arithmetic is regrouped for throughput (neighbour sums before the
// weights); the result is checked against the FP64 oracle with a
// tolerance, not bitwise.  Every wait is bounded: a wait that runs out sets
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

template <int V>
static __device__ __forceinline__ void ldv(const float* p, float (&v)[V])
{
    if constexpr (V == 4) {
        const float4 t = *reinterpret_cast<const float4*>(p);
        v[0] = t.x, v[1] = t.y, v[2] = t.z, v[3] = t.w;
    } else if constexpr (V == 2) {
        const float2 t = *reinterpret_cast<const float2*>(p);
        v[0] = t.x, v[1] = t.y;
    } else {
        v[0] = *p;
    }
}

template <int V>
static __device__ __forceinline__ void stv(float* p, const float (&v)[V])
{
    if constexpr (V == 4) *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
    else if constexpr (V == 2) *reinterpret_cast<float2*>(p) = make_float2(v[0], v[1]);
    else *p = v[0];
}

// sums of the two Z neighbours of each of a lane's V cells (the row wraps
// across lanes 31 and 0)
template <int V>
static __device__ __forceinline__ void zsum(const float (&c)[V], int lane, float (&s)[V])
{
    const float left = __shfl_sync(0xffffffffu, c[V - 1], (lane + 31) & 31);
    const float right = __shfl_sync(0xffffffffu, c[0], (lane + 1) & 31);
#pragma unroll
    for (int v = 0; v < V; v++) s[v] = (v == 0 ? left : c[v - 1]) + (v == V - 1 ? right : c[v + 1]);
}

// wx*sx + wy*sy + wz*sz - 2(wx+wy+wz)*c from the neighbour sums along each axis
template <bool UNIT>
static __device__ __forceinline__ float lap3(float sx, float sy, float sz, float c, const OstF32& q)
{
    if (UNIT) return fmaf(-6.0f, c, (sx + sy) + sz);
    return fmaf(q.wx, sx, fmaf(q.wy, sy, fmaf(q.wz, sz, -q.w2 * c)));
}

// V = Z/32 cells per lane, TY warps, RT update rows per warp (R = TY*RT rows
// per strip), NF fields, D ring slots (D >= 5: four planes in use).
template <int V, int TY, int RT, int NF, int D, bool UNIT>
__global__ void __launch_bounds__(32 * TY)
ost3_stream_f32(const float* __restrict__ sin, float* __restrict__ sout, Geom g, OstF32 q, int planes,
                int* __restrict__ err)
{
    constexpr int Z = 32 * V, R = TY * RT, RR = R + 4, WR = R + 2;
    constexpr int FS = RR * Z;        // floats of one field's rows in a slot
    constexpr int SS = NF * FS;       // floats of a slot
    static_assert(D >= 5 && NF >= 2, "ring depth, fields");
    extern __shared__ __align__(128) unsigned char sm[];
    float* ring = reinterpret_cast<float*>(sm);
    float* wring = ring + D * SS;
    uint64_t* bars = reinterpret_cast<uint64_t*>(wring + 3 * WR * Z);

    const int t = threadIdx.x, lane = t & 31, ty = t >> 5;
    const int z0 = lane * V;
    const int y0 = blockIdx.x * R;
    const int xs = blockIdx.y * planes, xe = min(xs + planes, g.X);
    if (xs >= xe) return;
    const int x_first = xs - 2, x_last = xe + 1;   // planes read from global memory
    const long long cells = g.cells;

    // thread 0: stage plane pl (wrapped) of every field into its slot
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
    auto wslot = [&](int xp) -> float* { return wring + ((xp - x_first) % 3) * WR * Z; };
    auto arrived = [&](int pl) {
        const int k = pl - x_first;
        return mbar_wait(&bars[k % D], (uint32_t)(k / D) & 1u);
    };

    // w(xp) on rows -1..R (ostwald.cpp:95-99):
    //   w = -A*(C-Cm) + B*(C-Cm)^3 + Da*(C-Ca)^3 + Db*(C-Cb)^3 - g*(C-Ca)*sum - kappa*lap C
    // with sum the squares of the order parameters; planes xp-1, xp, xp+1 staged.
    auto compute_w = [&](int xp) {
        const float* sl = slot(xp - 1);
        const float* sc = slot(xp);
        const float* sh = slot(xp + 1);
        float* wd = wslot(xp);
        for (int r = ty - 1; r <= R; r += TY) {
            const int o = (r + 2) * Z + z0;
            float c[V], cu[V], cd[V], xh[V], xl[V], sz[V], sum[V];
            ldv<V>(sc + o, c);
            ldv<V>(sc + o - Z, cd);
            ldv<V>(sc + o + Z, cu);
            ldv<V>(sl + o, xl);
            ldv<V>(sh + o, xh);
            {
                float e[V];
                ldv<V>(sc + FS + o, e);
#pragma unroll
                for (int v = 0; v < V; v++) sum[v] = e[v] * e[v];
#pragma unroll
                for (int j = 2; j < NF; j++) {
                    ldv<V>(sc + j * FS + o, e);
#pragma unroll
                    for (int v = 0; v < V; v++) sum[v] = fmaf(e[v], e[v], sum[v]);
                }
            }
            zsum<V>(c, lane, sz);
            float w[V];
#pragma unroll
            for (int v = 0; v < V; v++) {
                const float lap = lap3<UNIT>(xh[v] + xl[v], cu[v] + cd[v], sz[v], c[v], q);
                const float dm = c[v] - q.Cm, da = c[v] - q.Ca, db = c[v] - q.Cb;
                float s = fmaf(q.B * dm, dm * dm, q.negA * dm);
                s = fmaf(q.Da * da, da * da, s);
                s = fmaf(q.Db * db, db * db, s);
                s = fmaf(-q.g * da, sum[v], s);
                w[v] = fmaf(-q.kappa, lap, s);
            }
            stv<V>(wd + (r + 1) * Z + z0, w);
        }
    };

    // Plane x, rows ty*RT .. ty*RT+RT-1 (ostwald.cpp:103-120):
    //   C'   = C + dt*D*lap w
    //   e_j' = e_j - dt*L*(-g*(C-Ca)^2 + delta*e_j^3 + eps*e_j*(sum - e_j^2) - kappa*lap e_j)
    auto update = [&](int x) {
        const float* sl = slot(x - 1);
        const float* sc = slot(x);
        const float* sh = slot(x + 1);
        const float* wm = wslot(x - 1);
        const float* w0 = wslot(x);
        const float* wp = wslot(x + 1);
        const int r0 = ty * RT;
        // columns of rows r0-1 .. r0+RT: w(x) and every order parameter at plane x
        float wc[RT + 2][V], ec[NF - 1][RT + 2][V];
#pragma unroll
        for (int k = 0; k < RT + 2; k++) {
            ldv<V>(w0 + (r0 + k) * Z + z0, wc[k]);
#pragma unroll
            for (int j = 1; j < NF; j++) ldv<V>(sc + j * FS + (r0 + k + 1) * Z + z0, ec[j - 1][k]);
        }
        float* dst = sout + (long long)x * g.YZ + (long long)(y0 + r0) * Z + z0;
#pragma unroll
        for (int k = 0; k < RT; k++) {
            const bool inside = y0 + r0 + k < g.Y;
            const int o = (r0 + k + 2) * Z + z0;   // ring row of update row r0+k
            float a[V], b[V], sz[V], C[V], out[V];
            ldv<V>(wm + (r0 + k + 1) * Z + z0, a);
            ldv<V>(wp + (r0 + k + 1) * Z + z0, b);
            ldv<V>(sc + o, C);
            zsum<V>(wc[k + 1], lane, sz);
#pragma unroll
            for (int v = 0; v < V; v++) {
                const float lap = lap3<UNIT>(a[v] + b[v], wc[k][v] + wc[k + 2][v], sz[v], wc[k + 1][v], q);
                out[v] = fmaf(q.dtD, lap, C[v]);
            }
            if (inside) stv<V>(dst + (long long)k * Z, out);
            float sum[V], t1[V];
#pragma unroll
            for (int v = 0; v < V; v++) {
                sum[v] = ec[0][k + 1][v] * ec[0][k + 1][v];
#pragma unroll
                for (int j = 1; j < NF - 1; j++) sum[v] = fmaf(ec[j][k + 1][v], ec[j][k + 1][v], sum[v]);
                const float da = C[v] - q.Ca;
                t1[v] = q.neg_g * (da * da);
            }
#pragma unroll
            for (int j = 1; j < NF; j++) {
                const float(&e)[V] = ec[j - 1][k + 1];
                ldv<V>(sl + j * FS + o, a);
                ldv<V>(sh + j * FS + o, b);
                zsum<V>(e, lane, sz);
#pragma unroll
                for (int v = 0; v < V; v++) {
                    const float lap =
                        lap3<UNIT>(a[v] + b[v], ec[j - 1][k][v] + ec[j - 1][k + 2][v], sz[v], e[v], q);
                    float s = fmaf(q.delta * e[v], e[v] * e[v], t1[v]);
                    s = fmaf(q.eps * e[v], fmaf(-e[v], e[v], sum[v]), s);
                    s = fmaf(-q.kappa, lap, s);
                    out[v] = fmaf(-q.dtL, s, e[v]);
                }
                if (inside) stv<V>(dst + (long long)j * cells + (long long)k * Z, out);
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
    bool bad = false;
    for (int pl = x_first; pl <= xs + 1; pl++) bad |= !arrived(pl);
    compute_w(xs - 1);
    compute_w(xs);
    bool stop = __syncthreads_or(bad);
    if (!stop && t == 0 && x_first + D <= x_last) fill(issued = x_first + D);   // the slot of xs-2 is free
    for (int x = xs; x < xe && !stop; x++) {
        bad = !arrived(x + 2);
        compute_w(x + 1);
        stop = __syncthreads_or(bad);
        if (stop) break;
        update(x);
        __syncthreads();
        // the slot of plane x-1 and the w plane of x-1 are free now
        if (t == 0 && x - 1 + D <= x_last) fill(issued = x - 1 + D);
    }
    if (stop && t == 0) {
        atomicExch(err, 1);
        // leave no copy in flight: wait (bounded) for every fill not yet consumed
        for (int pl = max(x_first, issued - D + 1); pl <= issued; pl++) arrived(pl);
    }
}

// Kernel shapes per row length: rows per warp and warps, ring depth.
template <int V> struct OstShape;
template <> struct OstShape<1> { static constexpr int TY = 8, RT = 2, D = 6; };
template <> struct OstShape<2> { static constexpr int TY = 8, RT = 2, D = 6; };
template <> struct OstShape<4> { static constexpr int TY = 8, RT = 1, D = 5; };

template <int V, int NF>
static const void* ost3_fn(bool unit)
{
    using S = OstShape<V>;
    return unit ? (const void*)&ost3_stream_f32<V, S::TY, S::RT, NF, S::D, true>
                : (const void*)&ost3_stream_f32<V, S::TY, S::RT, NF, S::D, false>;
}

template <int V>
static const void* ost3_pick_n(int N, bool unit)
{
    if (N == 2) return ost3_fn<V, 2>(unit);
    if (N == 3) return ost3_fn<V, 3>(unit);
    if (N == 4) return ost3_fn<V, 4>(unit);
    return nullptr;
}

template <int V>
static size_t ost3_smem(int N)
{
    using S = OstShape<V>;
    constexpr int Z = 32 * V, R = S::TY * S::RT;
    return sizeof(float) * ((size_t)S::D * N * (R + 4) * Z + 3 * (R + 2) * Z) + sizeof(uint64_t) * S::D;
}

static int ost3_rows(int V)
{
    if (V == 1) return OstShape<1>::TY * OstShape<1>::RT;
    if (V == 2) return OstShape<2>::TY * OstShape<2>::RT;
    return OstShape<4>::TY * OstShape<4>::RT;
}

bool ost3_stream_eligible(const mmsp_gpu_desc& d, const Geom& g)
{
    if (d.dtype != MMSP_GPU_F32 || g.dim != 3 || d.fields < 2 || d.fields > 4) return false;
    if (g.Z != 32 && g.Z != 64 && g.Z != 128) return false;
    return g.Y >= ost3_rows(g.Z / 32) + 4 && g.X >= 4;
}

cudaError_t plan_ost3_stream(const mmsp_gpu_desc& d, const Geom& g, const Coeffs& c, StepPlan* p)
{
    const int V = g.Z / 32;
    const int N = d.fields;
    p->fn = V == 1 ? ost3_pick_n<1>(N, c.unit_w) : V == 2 ? ost3_pick_n<2>(N, c.unit_w) : ost3_pick_n<4>(N, c.unit_w);
    p->smem = V == 1 ? ost3_smem<1>(N) : V == 2 ? ost3_smem<2>(N) : ost3_smem<4>(N);
    p->block = dim3(32 * (V == 1 ? OstShape<1>::TY : V == 2 ? OstShape<2>::TY : OstShape<4>::TY), 1, 1);
    if (!p->fn) return cudaErrorInvalidConfiguration;
    cudaError_t e = ensure_smem(p->fn, p->smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, p->fn, (int)p->block.x, p->smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    const int R = ost3_rows(V);
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
