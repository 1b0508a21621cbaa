// MMSP.gpu.hpp -- drop-in GB300 update() for MMSP grids.
//
// Include after MMSP.hpp and link libmmsp_gpu.so.  A plugin keeps MMSP's
// contract (include/MMSP.main.hpp:5-26): it defines generate() and
//
//     template <int dim, typename T> void update(MMSP::grid<dim,T>& g, int steps)
//
// and forwards the body to MMSP::gpu::update with the model it integrates,
// e.g. for the explicit Cahn-Hilliard example
// (examples/phase_transitions/cahn-hilliard/explicit/cahn-hilliard.cpp:47-81):
//
//     template <int dim, typename T> void update(MMSP::grid<dim,T>& g, int steps)
//     { MMSP::gpu::update(g, steps, MMSP::gpu::cahn_hilliard(1.0, 1.0, 0.005)); }
//
// and for isotropic phase-field grain growth
// (examples/coarsening/grain_growth/isotropic/phase_field/graingrowth.cpp:73-111):
//
//     template <int dim, typename T> void update(MMSP::grid<dim,MMSP::vector<T> >& g, int steps)
//     { MMSP::gpu::update(g, steps, MMSP::gpu::grain_growth_shipped(0.01)); }
//
// The grid is read once, advanced `steps` explicit steps on the device and
// written back, like the reference's update() which swaps its result into the
// caller's grid (cahn-hilliard.cpp:78).  grid<dim,double> runs the FP64 plain
// form (the reference's operation order, bit-identical results);
// grid<dim,float> runs the FP32 precision form.  Output, file format and
// main() stay the reference's own.
//
// Errors follow the reference: a message on std::cerr and MMSP::Abort(code)
// (include/MMSP.utility.cpp:30-36).  gpu::try_update returns the code instead.
//
// The wrapper uses only MMSP's free grid functions (nodes, fields, g0, g1,
// x0, x1, b0, b1, dx) and operator()(int), so any container with that
// interface works.
#ifndef MMSP_GPU_HPP
#define MMSP_GPU_HPP

#include <iostream>
#include <string>
#include <vector>

#include <cmath>

#include "MMSP.gpu.h"

namespace MMSP {

// MMSP's sparse cell type (include/MMSP.sparse.h:19), declared so that the
// sparse grid overloads below can name it; the caller's MMSP headers define it.
template <typename T> class sparse;

namespace gpu {

struct Model {
    int model;
    double dt, kappa, mobility, gamma, r, u;
    double aux[6];   // further parameters (mmsp_gpu_desc.aux); zero unless the model takes them
    int flags;       // MMSP_GPU_FLAG_* (mmsp_gpu_desc.flags)
    int slots;       // sparse grids: item slots per cell on the device (mmsp_gpu_desc.fields; 0: 16)
};

// The same model with the FP64 Cahn-Hilliard step contracted (fused
// multiply-adds, 16 instead of 23 FP64 operations per cell): within 1e-12
// relative of the reference instead of bit-identical.
inline Model contracted(Model m)
{
    m.flags |= MMSP_GPU_FLAG_CONTRACT;
    return m;
}

// f = c^2(1-c)^2: mu = 2c(1-c)(1-2c) - kappa*lap c; dc/dt = M lap mu
inline Model cahn_hilliard(double kappa, double M, double dt)
{
    Model m = {MMSP_GPU_CH, dt, kappa, M, 0.0, 0.0, 0.0};
    return m;
}
// cahn-hilliard.cpp:59-76 as shipped: mu = -r c + u c^3 - K lap c
inline Model cahn_hilliard_shipped(double r, double u, double K, double M, double dt)
{
    Model m = {MMSP_GPU_CH_POLY, dt, K, M, 0.0, r, u};
    return m;
}
// f = sum(-e^2/2 + e^4/4) + gamma sum_{i<j} e_i^2 e_j^2, de/dt = -L (df/de - kappa lap e)
inline Model allen_cahn(double gamma, double kappa, double L, double dt)
{
    Model m = {MMSP_GPU_AC, dt, kappa, L, gamma, 0.0, 0.0};
    return m;
}
// graingrowth.cpp:84-106 as shipped
inline Model grain_growth_shipped(double dt)
{
    Model m = {MMSP_GPU_GG, dt, 2.0, 1.0, 1.0, 0.0, 0.0};
    return m;
}
// examples/coarsening/zener_pinning/isotropic/phase_field/zener.cpp:113-138 as shipped:
// grain growth with field 0 (the particles) held fixed
inline Model zener_pinning_shipped(double dt)
{
    Model m = {MMSP_GPU_ZENER, dt, 2.0, 1.0, 1.0, 0.0, 0.0};
    return m;
}
// examples/coarsening/ostwald_ripening/isotropic/phase_field/ostwald.cpp:56-123 as shipped,
// on grid<dim,vector<T> > with field 0 the composition and fields 1.. the order parameters
inline Model ostwald_ripening_shipped(double dt = 0.001, double L = 1.0, double D = 1.0, double Calpha = 0.05,
                                      double Cbeta = 0.95, double A = 2.0, double delta = 1.0,
                                      double epsilon = 3.0, double kappa = 2.0)
{
    Model m = {MMSP_GPU_OSTWALD, dt, kappa, L, 1.0, 0.0, 0.0, {D, Calpha, Cbeta, A, delta, epsilon}};
    return m;
}
// examples/phase_transitions/model_A/model_A.cpp:74-107: scalar Allen-Cahn with thermal noise
// of standard deviation sqrt(2 kT/(dt dV)) from stream `seed`
inline Model model_A(double r = 1.0, double u = 1.0, double K = 1.0, double M = 1.0, double dt = 0.01,
                     double kT = 0.01, double dV = 1.0, double seed = 0.0)
{
    Model m = {MMSP_GPU_AC_POLY, dt, K, M, 0.0, r, u, {std::sqrt(2.0 * kT / (dt * dV)), seed, 0.0, 0.0, 0.0, 0.0}};
    return m;
}
// examples/phase_transitions/model_B/model_B.cpp:74-112: Cahn-Hilliard with thermal noise in mu
inline Model model_B(double r = 1.0, double u = 1.0, double K = 1.0, double M = 1.0, double dt = 0.01,
                     double kT = 0.01, double dV = 1.0, double seed = 0.0)
{
    Model m = {MMSP_GPU_CH_POLY, dt, K, M, 0.0, r, u, {std::sqrt(2.0 * kT / (dt * dV)), seed, 0.0, 0.0, 0.0, 0.0}};
    return m;
}
// examples/phase_transitions/spinodal/spinodal.cpp:95-102: mu = -c + c^3 - lap c + noise of standard
// deviation sqrt(epsilon dt/dV); c' = c + dt/(2 dV) lap mu
inline Model spinodal(double dt = 0.01, double dV = 1.0, double epsilon = 0.05, double seed = 0.0)
{
    Model m = {MMSP_GPU_CH_POLY, dt, 1.0, 1.0 / (2.0 * dV), 0.0, 1.0, 1.0,
               {std::sqrt(epsilon * dt / dV), seed, 0.0, 0.0, 0.0, 0.0}};
    return m;
}
// examples/phase_transitions/cahn-hilliard/convex_splitting/cahn-hilliard.cpp:273-463 as shipped
// (parametric energy), on grid<dim,vector<double> > with fields c and mu, FP64, even extents
inline Model cahn_hilliard_convex_splitting(double C0 = 0.45, double Ca = 0.05, double Cb = 0.95, double A = 2.0,
                                            double K = 2.0, double omega = 1.2, double tolerance = 1.0e-14)
{
    const double D = 2.0 / (Cb - Ca);
    Model m = {MMSP_GPU_CH_CONVEX, 1.0 / (D * K), K, D, 1.0, 0.0, 0.0, {C0, Ca, Cb, A, omega, tolerance}};
    return m;
}
// examples/coarsening/grain_growth/isotropic/sparsePF/graingrowth.cpp:58-120 as shipped, on
// grid<dim,sparse<double> >: at most `slots` items per cell on the device (MMSP_GPU_EOVERFLOW beyond)
inline Model sparse_grain_growth_shipped(double dt = 0.01, double epsilon = 1.0e-8, int slots = 16)
{
    Model m = {MMSP_GPU_SPARSE_GG, dt, 1.0, 1.0, 1.0, 0.0, 0.0, {epsilon, 0.0, 0.0, 0.0, 0.0, 0.0}, 0, slots};
    return m;
}
// allen-cahn.cpp:57-70 as shipped (scalar grid)
inline Model allen_cahn_shipped(double r, double u, double K, double M, double dt)
{
    Model m = {MMSP_GPU_AC_POLY, dt, K, M, 0.0, r, u};
    return m;
}

template <typename T> struct dtype_of;
template <> struct dtype_of<double> { static const int value = MMSP_GPU_F64; };
template <> struct dtype_of<float> { static const int value = MMSP_GPU_F32; };

template <class G>
int describe(const G& g, int dim, int fields, int dtype, const Model& m, mmsp_gpu_desc* d)
{
    int n[3] = {1, 1, 1};
    for (int a = 0; a < dim; a++) {
        // one serial domain covering the whole grid (no MPI decomposition)
        if (x0(g, a) != g0(g, a) || x1(g, a) != g1(g, a)) return MMSP_GPU_EUNSUPPORTED;
        n[a] = g1(g, a) - g0(g, a);
    }
    int rc = mmsp_gpu_desc_init(d, dim, n, fields, dtype, m.model);
    if (rc == MMSP_GPU_EINVAL) return rc;
    for (int a = 0; a < dim; a++) {
        d->dx[a] = dx(g, a);
        d->bc[a][0] = b0(g, a);
        d->bc[a][1] = b1(g, a);
    }
    d->dt = m.dt;
    d->kappa = m.kappa;
    d->mobility = m.mobility;
    d->gamma = m.gamma;
    d->r = m.r;
    d->u = m.u;
    for (int k = 0; k < 6; k++) d->aux[k] = m.aux[k];
    d->flags = m.flags;
    return mmsp_gpu_validate(d);
}

inline int report(int rc, const char* what)
{
    if (rc != MMSP_GPU_OK)
        std::cerr << "MMSP::gpu::update: " << what << ": " << mmsp_gpu_strerror(rc) << " (" << rc << ")" << std::endl;
    return rc;
}

// Scalar grids: grid<dim,double> (plain form) and grid<dim,float> (precision form).
template <template <int, typename> class Grid, int dim, typename T>
int try_update(Grid<dim, T>& g, int steps, const Model& m, mmsp_gpu_stats* stats = 0)
{
    mmsp_gpu_desc d;
    int rc = describe(g, dim, 1, dtype_of<T>::value, m, &d);
    if (rc) return report(rc, "descriptor");
    const int n = nodes(g);
    std::vector<T> buf((size_t)n);
    for (int i = 0; i < n; i++) buf[i] = g(i);
    rc = mmsp_gpu_update(&d, &buf[0], buf.size() * sizeof(T), MMSP_GPU_CELL_MAJOR, steps, stats);
    if (rc) return report(rc, "device step");
    for (int i = 0; i < n; i++) g(i) = buf[i];
    return MMSP_GPU_OK;
}

// Vector grids: grid<dim,vector<double>> / grid<dim,vector<float>>.  Values
// are gathered cell-major (to_buffer order without the per-cell length).
template <template <int, typename> class Grid, template <typename> class Vec, int dim, typename T>
int try_update(Grid<dim, Vec<T> >& g, int steps, const Model& m, mmsp_gpu_stats* stats = 0)
{
    const int N = fields(g);
    mmsp_gpu_desc d;
    int rc = describe(g, dim, N, dtype_of<T>::value, m, &d);
    if (rc) return report(rc, "descriptor");
    const int n = nodes(g);
    std::vector<T> buf((size_t)n * N);
    for (int i = 0; i < n; i++)
        for (int j = 0; j < N; j++) buf[(size_t)i * N + j] = g(i)[j];
    rc = mmsp_gpu_update(&d, &buf[0], buf.size() * sizeof(T), MMSP_GPU_CELL_MAJOR, steps, stats);
    if (rc) return report(rc, "device step");
    for (int i = 0; i < n; i++)
        for (int j = 0; j < N; j++) g(i)[j] = buf[(size_t)i * N + j];
    return MMSP_GPU_OK;
}

// Sparse grids: grid<dim,sparse<double> > (the sparsePF example).  Each
// cell's items travel in their stored order (length/index/value of
// include/MMSP.sparse.h:82-103) and come back through set(), so the host
// grid ends as the reference's update() leaves it.
template <template <int, typename> class Grid, int dim, typename T>
int try_update(Grid<dim, sparse<T> >& g, int steps, const Model& m, mmsp_gpu_stats* stats = 0)
{
    (void)stats;   // the example reports no reductions
    const int K = m.slots > 0 ? m.slots : 16;
    mmsp_gpu_desc d;
    int rc = describe(g, dim, K, dtype_of<T>::value, m, &d);
    if (rc) return report(rc, "descriptor");
    const int n = nodes(g);
    std::vector<int32_t> count((size_t)n), index((size_t)n * K, 0);
    std::vector<double> value((size_t)n * K, 0.0);
    for (int i = 0; i < n; i++) {
        const int len = length(g(i));
        if (len > K) return report(MMSP_GPU_EOVERFLOW, "sparse cell longer than the slots");
        count[i] = len;
        for (int h = 0; h < len; h++) {
            index[(size_t)i * K + h] = MMSP::index(g(i), h);
            value[(size_t)i * K + h] = MMSP::value(g(i), h);
        }
    }
    mmsp_gpu_handle* hd = 0;
    rc = mmsp_gpu_create(&hd, &d);
    if (rc) return report(rc, "create");
    rc = mmsp_gpu_sparse_upload(hd, &count[0], &index[0], &value[0]);
    if (!rc) rc = mmsp_gpu_step(hd, steps);
    if (!rc) rc = mmsp_gpu_sparse_download(hd, &count[0], &index[0], &value[0]);
    if (rc) std::cerr << "MMSP::gpu::update: " << mmsp_gpu_last_error(hd) << std::endl;
    mmsp_gpu_destroy(hd);
    if (rc) return report(rc, "device step");
    for (int i = 0; i < n; i++) {
        g(i) = sparse<T>();
        for (int h = 0; h < count[i]; h++) MMSP::set(g(i), index[(size_t)i * K + h]) = value[(size_t)i * K + h];
    }
    return MMSP_GPU_OK;
}

// The plugin-facing call: aborts like the reference on failure.
template <class G>
void update(G& g, int steps, const Model& m)
{
    int rc = try_update(g, steps, m);
    if (rc) MMSP::Abort(rc);
}

// The run loop of MMSP.main.hpp with the state kept on the device.  The
// reference's main() (include/MMSP.main.hpp:277-300, repeated for 2D and 3D)
// calls update(grid, increment) and then output(grid, name) for
// i = start, start + increment, ... < steps, the name being base, then
// i + increment zero-padded to the digits of `steps`, then suffix.  Through
// gpu::update every increment would copy the grid in and out; here the grid
// goes to the device once, each snapshot is written by mmsp_gpu_output while
// the next increment runs, and the host grid holds the final state at the end.
// Files are the reference's format (grid::output, one block, zlib level 9).
inline int run_buffer(const mmsp_gpu_desc& d, void* buf, size_t bytes, mmsp_gpu_output_opts& o, int start, int steps,
                      int increment, const std::string& base, const std::string& suffix, mmsp_gpu_stats* stats)
{
    if (increment < 1) return MMSP_GPU_EINVAL;
    mmsp_gpu_handle* h = 0;
    int rc = mmsp_gpu_create(&h, &d);
    if (rc) return report(rc, "create");
    rc = mmsp_gpu_upload(h, buf, bytes, MMSP_GPU_CELL_MAJOR);
    const size_t width = std::to_string(steps).size();
    for (int i = start; rc == MMSP_GPU_OK && i < steps; i += increment) {
        rc = mmsp_gpu_step(h, increment);
        std::string num = std::to_string(i + increment);
        if (num.size() < width) num = std::string(width - num.size(), '0') + num;
        if (rc == MMSP_GPU_OK) rc = mmsp_gpu_output(h, (base + num + suffix).c_str(), &o);
    }
    int wrc = mmsp_gpu_output_wait(h);
    if (rc == MMSP_GPU_OK) rc = wrc;
    if (rc == MMSP_GPU_OK) rc = mmsp_gpu_download(h, buf, bytes, MMSP_GPU_CELL_MAJOR);
    if (rc == MMSP_GPU_OK && stats) rc = mmsp_gpu_reduce(h, stats);
    if (rc) std::cerr << "MMSP::gpu::run: " << mmsp_gpu_last_error(h) << std::endl;
    mmsp_gpu_destroy(h);
    return report(rc, "run");
}

template <template <int, typename> class Grid, int dim, typename T>
int try_run(Grid<dim, T>& g, int start, int steps, int increment, const std::string& base, const std::string& suffix,
            const Model& m, mmsp_gpu_stats* stats = 0)
{
    mmsp_gpu_desc d;
    int rc = describe(g, dim, 1, dtype_of<T>::value, m, &d);
    if (rc) return report(rc, "descriptor");
    const int n = nodes(g);
    std::vector<T> buf((size_t)n);
    for (int i = 0; i < n; i++) buf[i] = g(i);
    mmsp_gpu_output_opts o;
    mmsp_gpu_output_opts_init(&o);
    o.vector = 0;
    o.fields_line = fields(g);
    for (int a = 0; a < dim; a++) o.g0[a] = g0(g, a);
    rc = run_buffer(d, &buf[0], buf.size() * sizeof(T), o, start, steps, increment, base, suffix, stats);
    if (rc) return rc;
    for (int i = 0; i < n; i++) g(i) = buf[i];
    return MMSP_GPU_OK;
}

template <template <int, typename> class Grid, template <typename> class Vec, int dim, typename T>
int try_run(Grid<dim, Vec<T> >& g, int start, int steps, int increment, const std::string& base,
            const std::string& suffix, const Model& m, mmsp_gpu_stats* stats = 0)
{
    const int N = fields(g);
    mmsp_gpu_desc d;
    int rc = describe(g, dim, N, dtype_of<T>::value, m, &d);
    if (rc) return report(rc, "descriptor");
    const int n = nodes(g);
    std::vector<T> buf((size_t)n * N);
    for (int i = 0; i < n; i++)
        for (int j = 0; j < N; j++) buf[(size_t)i * N + j] = g(i)[j];
    mmsp_gpu_output_opts o;
    mmsp_gpu_output_opts_init(&o);
    o.vector = 1;
    o.fields_line = N;
    for (int a = 0; a < dim; a++) o.g0[a] = g0(g, a);
    rc = run_buffer(d, &buf[0], buf.size() * sizeof(T), o, start, steps, increment, base, suffix, stats);
    if (rc) return rc;
    for (int i = 0; i < n; i++)
        for (int j = 0; j < N; j++) g(i)[j] = buf[(size_t)i * N + j];
    return MMSP_GPU_OK;
}

// The main()-facing call: aborts like the reference on failure.
template <class G>
void run(G& g, int start, int steps, int increment, const std::string& base, const std::string& suffix,
         const Model& m)
{
    int rc = try_run(g, start, steps, increment, base, suffix, m);
    if (rc) MMSP::Abort(rc);
}

}  // namespace gpu
}  // namespace MMSP

#endif
