// pf_sparse.cu -- isotropic sparse phase-field grain growth (the sparsePF example).
//
// The reference keeps, per cell, a list of (grain index, value) items in
// insertion order (class sparse, include/MMSP.sparse.h:19; set() overwrites
// an item or appends one, operator[] reads 0 for an absent index), and its
// update (examples/coarsening/grain_growth/isotropic/sparsePF/graingrowth.cpp:58-120)
// works per cell on the union of the indices of the cell and its 2*dim face
// neighbours.
//
// Device format: a state buffer holds the lists slot-major, so that slot h
// of neighbouring cells is one coalesced line:
//   count[cells]           int32 items per cell
//   index[K][cells]        int32 grain index of slot h
//   value[K][cells]        T value of slot h
// with K = mmsp_gpu_desc.fields slots per cell.  A list that would outgrow K
// sets the overflow word and leaves that item out (the host reports
// MMSP_GPU_EOVERFLOW; the state is then invalid).
//
// One thread per cell.  The example's newGrid starts with empty cells and is
// never cleared: after swap() the buffer written at step s holds the state of
// step s-2, and set() keeps the items it does not overwrite.  The ping-pong
// buffers do the same (the host clears the idle buffer's counts at the start
// of each step call, as each update() call builds a fresh newGrid), so the
// stale items that enter later neighbour sets and sums are the reference's.
//
// Arithmetic: the sparse Laplacian (include/MMSP.grid.cpp:2110-2128) adds and
// subtracts item lists through sparse operator+/- that start each index at 0;
// where an index is absent each operation is exact, so its value is the
// dense weight*((yh - 2y) + yl) summed from 0.0 over axes with absent items
// read as 0 -- computed here in that order with every operation rounded on
// its own.  pow(phi,3) is the compensated cube of pf_device.cuh (within the
// C library's 1 ulp), so values are held to 1e-12 relative and counts and
// indices exactly.
#include "pf_device.cuh"
#include "pf_internal.h"

namespace pf {

constexpr int kSparseSet = 64;   // largest neighbour set (union of 2*dim+1 lists)

struct SpView {
    int* cnt;
    int* idx;        // idx[h * cells + c]
    double* val;     // val[h * cells + c]
};

SparseLayout sparse_layout(long long cells, int K)
{
    SparseLayout L;
    auto pad = [](size_t b) { return (b + 255) / 256 * 256; };
    L.idx_off = pad(sizeof(int) * (size_t)cells);
    L.val_off = L.idx_off + pad(sizeof(int) * (size_t)cells * K);
    L.bytes = L.val_off + sizeof(double) * (size_t)cells * K;
    return L;
}

static SpView view_of(void* buf, long long cells, int K)
{
    const SparseLayout L = sparse_layout(cells, K);
    SpView v;
    v.cnt = static_cast<int*>(buf);
    v.idx = reinterpret_cast<int*>(static_cast<char*>(buf) + L.idx_off);
    v.val = reinterpret_cast<double*>(static_cast<char*>(buf) + L.val_off);
    return v;
}

// Value of index i in cell c's list (0 when absent), as sparse::operator[].
static __device__ __forceinline__ double sp_get(const SpView& s, long long cells, long long c, int i)
{
    const int n = __ldg(s.cnt + c);
    for (int h = 0; h < n; h++)
        if (__ldg(s.idx + h * cells + c) == i) return __ldg(s.val + h * cells + c);
    return 0.0;
}

struct SpConst {
    double w[3];     // 1/(dx*dx) per real axis
    double eps;      // epsilon: values at or below it are not stored
    P<double> p;     // dtm = dt for the update expression
};

template <int DIM, bool UNIT>
__global__ void __launch_bounds__(128)
sparse_gg_step(SpView in, SpView out, Geom g, SpConst q, int K, int* __restrict__ err)
{
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.cells) return;
    const long long cells = g.cells;
    // padded coordinates and the periodic face neighbours of the real axes,
    // in the reference's axis order (real axis 0 first)
    const int x = (int)(c / g.YZ);
    const int r = (int)(c - (long long)x * g.YZ);
    const int y = r / g.Z;
    const int z = r - y * g.Z;
    long long lo[3], hi[3];
    {
        const int xl = x == 0 ? g.X - 1 : x - 1, xh = x + 1 == g.X ? 0 : x + 1;
        const int yl = y == 0 ? g.Y - 1 : y - 1, yh = y + 1 == g.Y ? 0 : y + 1;
        const int zl = z == 0 ? g.Z - 1 : z - 1, zh = z + 1 == g.Z ? 0 : z + 1;
        const long long px[3] = {c + (long long)(xl - x) * g.YZ, c + (long long)(yl - y) * g.Z, c + (zl - z)};
        const long long qx[3] = {c + (long long)(xh - x) * g.YZ, c + (long long)(yh - y) * g.Z, c + (zh - z)};
        for (int ra = 0; ra < DIM; ra++) {
            lo[ra] = px[3 - DIM + ra];
            hi[ra] = qx[3 - DIM + ra];
        }
    }
    // nonzero fields of the neighbourhood, in the example's visiting order:
    // per axis the low neighbour, the cell itself, the high neighbour
    int S[kSparseSet];
    int ns = 0;
    bool ovf = false;
#pragma unroll
    for (int ra = 0; ra < DIM; ra++) {
        for (int k = 0; k < 3; k++) {
            const long long nc = k == 0 ? lo[ra] : k == 1 ? c : hi[ra];
            const int n = __ldg(in.cnt + nc);
            for (int h = 0; h < n; h++) {
                const int i = __ldg(in.idx + h * cells + nc);
                bool seen = false;
                for (int s = 0; s < ns; s++) seen |= S[s] == i;
                if (!seen) {
                    if (ns == kSparseSet) ovf = true;
                    else S[ns++] = i;
                }
            }
        }
    }
    const int own = __ldg(in.cnt + c);
    if (ns < 2) {
        // newGrid(n) = oldGrid(n): the whole list
        out.cnt[c] = own;
        for (int h = 0; h < own; h++) {
            out.idx[h * cells + c] = __ldg(in.idx + h * cells + c);
            out.val[h * cells + c] = __ldg(in.val + h * cells + c);
        }
    } else {
        double sum = 0.0;
        for (int h = 0; h < own; h++) {
            const double phi = __ldg(in.val + h * cells + c);
            sum = __dadd_rn(sum, __dmul_rn(phi, phi));
        }
        // newGrid(n) as it stands: the state of two steps back
        int dn = out.cnt[c];
        for (int s = 0; s < ns; s++) {
            const int i = S[s];
            const double phi = sp_get(in, cells, c, i);
            const double y2 = twice(phi);
            double lap = 0.0;
#pragma unroll
            for (int ra = 0; ra < DIM; ra++) {
                double t = __dadd_rn(__dsub_rn(sp_get(in, cells, hi[ra], i), y2), sp_get(in, cells, lo[ra], i));
                if (!UNIT) t = __dmul_rn(q.w[ra], t);
                lap = ra == 0 ? plus_zero(t) : __dadd_rn(lap, t);
            }
            const double v = ac_new<double, MMSP_GPU_GG>(phi, sum, lap, q.p);
            if (v > q.eps) {
                int h = 0;
                while (h < dn && out.idx[h * cells + c] != i) h++;
                if (h == dn) {
                    if (dn == K) {
                        ovf = true;
                        continue;
                    }
                    out.idx[h * cells + c] = i;
                    dn++;
                }
                out.val[h * cells + c] = v;
            }
        }
        out.cnt[c] = dn;
    }
    if (ovf) atomicExch(err, 1);
}

// Host cell-major slots (count[cells], index[cells*K], value[cells*K]) <->
// the device's slot-major buffer, through a staging buffer that holds the
// three host arrays at the offsets of sparse_layout.
__global__ void sparse_pack(const int* __restrict__ hcnt, const int* __restrict__ hidx, const double* __restrict__ hval,
                            SpView d, long long cells, int K)
{
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cells) return;
    const int n = min(max(hcnt[c], 0), K);   // the host has checked 0 <= n <= K
    d.cnt[c] = n;
    for (int h = 0; h < K; h++) {
        d.idx[h * cells + c] = h < n ? hidx[c * K + h] : 0;
        d.val[h * cells + c] = h < n ? hval[c * K + h] : 0.0;
    }
}

__global__ void sparse_unpack(SpView d, int* __restrict__ hcnt, int* __restrict__ hidx, double* __restrict__ hval,
                              long long cells, int K)
{
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cells) return;
    const int n = d.cnt[c];
    hcnt[c] = n;
    for (int h = 0; h < K; h++) {
        hidx[c * K + h] = h < n ? d.idx[h * cells + c] : 0;
        hval[c * K + h] = h < n ? d.val[h * cells + c] : 0.0;
    }
}

static unsigned blocks_for(long long cells) { return (unsigned)((cells + 127) / 128); }

cudaError_t launch_sparse_gg(const mmsp_gpu_desc& d, const Geom& g, const Coeffs& c, const void* in, void* out,
                             int* err, cudaStream_t s)
{
    const int K = d.fields;
    SpView vi = view_of(const_cast<void*>(in), g.cells, K), vo = view_of(out, g.cells, K);
    SpConst q;
    for (int a = 0; a < 3; a++) q.w[a] = a < d.dim ? c.w[a] : 1.0;
    q.eps = d.aux[0];
    q.p = narrow<double>(c, g.dim);
    const void* fn;
    if (g.dim == 3) fn = c.unit_w ? (const void*)&sparse_gg_step<3, true> : (const void*)&sparse_gg_step<3, false>;
    else if (g.dim == 2) fn = c.unit_w ? (const void*)&sparse_gg_step<2, true> : (const void*)&sparse_gg_step<2, false>;
    else fn = c.unit_w ? (const void*)&sparse_gg_step<1, true> : (const void*)&sparse_gg_step<1, false>;
    int* ovf = err + 1;
    void* args[] = {(void*)&vi, (void*)&vo, (void*)&g, (void*)&q, (void*)&K, (void*)&ovf};
    return cudaLaunchKernel(fn, dim3(blocks_for(g.cells)), dim3(128), args, 0, s);
}

cudaError_t launch_sparse_pack(const void* staging, void* state, long long cells, int K, cudaStream_t s)
{
    const SpView h = view_of(const_cast<void*>(staging), cells, K);
    sparse_pack<<<blocks_for(cells), 128, 0, s>>>(h.cnt, h.idx, h.val, view_of(state, cells, K), cells, K);
    return cudaGetLastError();
}

cudaError_t launch_sparse_unpack(const void* state, void* staging, long long cells, int K, cudaStream_t s)
{
    const SpView h = view_of(staging, cells, K);
    sparse_unpack<<<blocks_for(cells), 128, 0, s>>>(view_of(const_cast<void*>(state), cells, K), h.cnt, h.idx, h.val,
                                                    cells, K);
    return cudaGetLastError();
}

}  // namespace pf
