/* pf_oracle.c -- CPU oracle for the explicit phase-field step (TEST INFRASTRUCTURE).
 *
 * See pf_oracle.h for what each function restates and where in the
 * reference it comes from.  Build with -ffp-contract=off (oracle/Makefile).
 */
#include "pf_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

/* check_boundary (include/MMSP.utility.cpp:42-57, serial build) for a local
 * domain [0, n).  Returns the mapped coordinate. */
static int map_coord(int x, int n, int b0, int b1)
{
    if (x < 0) {
        if (b0 == PFO_NEUMANN || b0 == PFO_DIRICHLET) x = 0;
        else if (b0 == PFO_PERIODIC) x = n - (0 - x);
        else if (b0 == PFO_MIRROR) x = 2 * 0 - x;
    } else if (x >= n) {
        if (b1 == PFO_NEUMANN || b1 == PFO_DIRICHLET) x = n - 1;
        else if (b1 == PFO_PERIODIC) x = 0 + (x - n);
        else if (b1 == PFO_MIRROR) x = 2 * (n - 1) - x;
    }
    return x;
}

/* The grid seen as three padded axes; the real axes are the last `dim`. */
typedef struct {
    int dim;
    int n[3];          /* padded extents (leading 1s) */
    long st[3];        /* strides, last axis fastest */
    double w[3];       /* 1/(dx*dx) of each real axis, in real-axis order */
    double wg[3];      /* 1/(2*dx), for gradient() */
    int* lo[3];        /* mapped x-1 per padded axis */
    int* hi[3];        /* mapped x+1 per padded axis */
    long cells;
} geo;

static void geo_free(geo* q)
{
    for (int a = 0; a < 3; a++) {
        free(q->lo[a]);
        free(q->hi[a]);
        q->lo[a] = q->hi[a] = NULL;
    }
}

static int geo_init(geo* q, const pfo_grid* g)
{
    memset(q, 0, sizeof(*q));
    if (!g || g->dim < 1 || g->dim > 3) return -1;
    q->dim = g->dim;
    int off = 3 - g->dim;
    for (int a = 0; a < 3; a++) q->n[a] = 1;
    for (int a = 0; a < g->dim; a++) {
        if (g->n[a] < 1) return -1;
        q->n[off + a] = g->n[a];
        /* grid.cpp:2062 (scalar and vector overloads use dx*dx) */
        q->w[a] = 1.0 / (g->dx[a] * g->dx[a]);
        q->wg[a] = 1.0 / (2.0 * g->dx[a]);
    }
    q->st[2] = 1;
    q->st[1] = q->n[2];
    q->st[0] = (long)q->n[1] * q->n[2];
    q->cells = (long)q->n[0] * q->st[0];
    for (int a = 0; a < 3; a++) {
        int n = q->n[a];
        q->lo[a] = (int*)malloc(sizeof(int) * (size_t)n);
        q->hi[a] = (int*)malloc(sizeof(int) * (size_t)n);
        if (!q->lo[a] || !q->hi[a]) { geo_free(q); return -1; }
        int ra = a - off; /* real axis index, <0 for padding */
        for (int x = 0; x < n; x++) {
            if (ra < 0) { q->lo[a][x] = q->hi[a][x] = x; continue; }
            int l = map_coord(x - 1, n, g->bc[ra][0], g->bc[ra][1]);
            int h = map_coord(x + 1, n, g->bc[ra][0], g->bc[ra][1]);
            /* a mapping that leaves the domain (mirror on n=1, "parallel"
             * in a serial grid) is undefined in the reference: refuse it. */
            if (l < 0 || l >= n || h < 0 || h >= n) { geo_free(q); return -1; }
            q->lo[a][x] = l;
            q->hi[a][x] = h;
        }
    }
    return 0;
}

long pfo_nodes(const pfo_grid* g)
{
    long c = 1;
    for (int a = 0; a < g->dim; a++) c *= g->n[a];
    return c;
}

/* Offsets of the low/high neighbour of cell (i0,i1,i2) along padded axis a. */
#define NB_LO(q, a, x) (((long)(q)->lo[a][x] - (x)) * (q)->st[a])
#define NB_HI(q, a, x) (((long)(q)->hi[a][x] - (x)) * (q)->st[a])

/* MMSP::laplacian, scalar (grid.cpp:2049-2066): lap starts at 0.0 and adds
 * weight*(yh - 2.0*y + yl) for axes 0..dim-1.  Field j of a cell-major
 * vector grid with N values per cell when N > 1 (grid.cpp:2068-2088). */
static inline double lap_at(const geo* q, const double* f, long idx, int N, int j,
                            const int xc[3])
{
    double lap = 0.0;
    const double y = f[idx * N + j];
    int off = 3 - q->dim;
    for (int ra = 0; ra < q->dim; ra++) {
        int a = off + ra;
        const double yh = f[(idx + NB_HI(q, a, xc[a])) * N + j];
        const double yl = f[(idx + NB_LO(q, a, xc[a])) * N + j];
        double weight = q->w[ra];
        lap += weight * (yh - 2.0 * y + yl);
    }
    return lap;
}

static int nthreads(int t)
{
#ifdef _OPENMP
    if (t <= 0) t = omp_get_max_threads();
    return t;
#else
    (void)t;
    return 1;
#endif
}

int pfo_laplacian(const pfo_grid* g, const double* in, double* out)
{
    geo q;
    if (geo_init(&q, g) || !in || !out) return -1;
    for (int i0 = 0; i0 < q.n[0]; i0++)
        for (int i1 = 0; i1 < q.n[1]; i1++)
            for (int i2 = 0; i2 < q.n[2]; i2++) {
                int xc[3] = {i0, i1, i2};
                long idx = i0 * q.st[0] + i1 * q.st[1] + i2;
                out[idx] = lap_at(&q, in, idx, 1, 0, xc);
            }
    geo_free(&q);
    return 0;
}

/* Value j of the SplitMix64 stream `seed` (Steele, Lea and Flood, OOPSLA
 * 2014), as mmsp_gb300/inputs.py and the device compute it. */
static uint64_t splitmix64_at(uint64_t seed, uint64_t j)
{
    uint64_t z = seed + (j + 1u) * 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

/* Standard normal deviate k of stream `seed`: Box-Muller on uniforms 2k and
 * 2k+1 (top 53 bits).  Stands in for the examples' gaussian()
 * (model_A.cpp:13-40), whose rand()-driven polar method depends on the
 * serial visiting order of the cells. */
double pfo_gaussian(uint64_t seed, uint64_t k)
{
    const double u1 = (double)(splitmix64_at(seed, 2u * k) >> 11) * 0x1.0p-53;
    const double u2 = (double)(splitmix64_at(seed, 2u * k + 1u) >> 11) * 0x1.0p-53;
    return sqrt(-2.0 * log(1.0 - u1)) * cos(6.283185307179586 * u2);
}

/* gaussian(0.0, std) of cell i in step `step`, as ave + u*std (model_A.cpp:31) */
static inline double noise_at(double nstd, uint64_t seed, long long step, long cells, long i)
{
    return 0.0 + pfo_gaussian(seed, (uint64_t)step * (uint64_t)cells + (uint64_t)i) * nstd;
}

/* Two-pass explicit Cahn-Hilliard in the structure of cahn-hilliard.cpp:65-80.
 * form 0: the configured free energy f = c^2 (1-c)^2, form 1: the shipped
 * polynomial. */
static int ch_run(const pfo_grid* g, double* c, int steps, int form,
                  double r, double u, double K, double M, double dt, int threads,
                  double nstd, uint64_t seed, long long step0)
{
    geo q;
    if (geo_init(&q, g) || !c || steps < 0) return -1;
    double* temp = (double*)malloc(sizeof(double) * (size_t)q.cells);
    double* nw = (double*)malloc(sizeof(double) * (size_t)q.cells);
    if (!temp || !nw) { free(temp); free(nw); geo_free(&q); return -1; }
    double* old = c;
    int nt = nthreads(threads);
    (void)nt;
    for (int step = 0; step < steps; step++) {
        #pragma omp parallel for schedule(static) num_threads(nt)
        for (int i0 = 0; i0 < q.n[0]; i0++)
            for (int i1 = 0; i1 < q.n[1]; i1++)
                for (int i2 = 0; i2 < q.n[2]; i2++) {
                    int xc[3] = {i0, i1, i2};
                    long i = i0 * q.st[0] + i1 * q.st[1] + i2;
                    double phi = old[i];
                    if (form == 0)
                        temp[i] = 2.0 * phi * (1.0 - phi) * (1.0 - 2.0 * phi) - K * lap_at(&q, old, i, 1, 0, xc);
                    else
                        temp[i] = -r * phi + u * pow(phi, 3) - K * lap_at(&q, old, i, 1, 0, xc);
                    /* model_B.cpp:100-101, spinodal.cpp:95-97: the mu pass takes + noise */
                    if (nstd != 0.0) temp[i] = temp[i] + noise_at(nstd, seed, step0 + step, q.cells, i);
                }
        #pragma omp parallel for schedule(static) num_threads(nt)
        for (int i0 = 0; i0 < q.n[0]; i0++)
            for (int i1 = 0; i1 < q.n[1]; i1++)
                for (int i2 = 0; i2 < q.n[2]; i2++) {
                    int xc[3] = {i0, i1, i2};
                    long i = i0 * q.st[0] + i1 * q.st[1] + i2;
                    nw[i] = old[i] + dt * M * lap_at(&q, temp, i, 1, 0, xc);
                }
        /* swap(oldGrid,newGrid), cahn-hilliard.cpp:78 */
        double* t = old;
        old = nw;
        nw = t;
    }
    if (old != c) {
        memcpy(c, old, sizeof(double) * (size_t)q.cells);
        nw = old;
    }
    free(temp);
    free(nw);
    geo_free(&q);
    return 0;
}

int pfo_ch_baseline(const pfo_grid* g, double* c, int steps,
                    double kappa, double M, double dt, int threads)
{
    return ch_run(g, c, steps, 0, 0.0, 0.0, kappa, M, dt, threads, 0.0, 0, 0);
}

int pfo_ch_shipped(const pfo_grid* g, double* c, int steps,
                   double r, double u, double K, double M, double dt, int threads)
{
    return ch_run(g, c, steps, 1, r, u, K, M, dt, threads, 0.0, 0, 0);
}

int pfo_ch_shipped_noise(const pfo_grid* g, double* c, int steps, double r, double u, double K, double M,
                         double dt, double nstd, uint64_t seed, long long step0, int threads)
{
    return ch_run(g, c, steps, 1, r, u, K, M, dt, threads, nstd, seed, step0);
}

/* Single-pass multi-field Allen-Cahn in the structure of graingrowth.cpp:86-110.
 * form 0: the configured free energy with gamma; form 1: graingrowth.cpp:105 as
 * shipped; form 2: allen-cahn.cpp:70 as shipped (N must be 1); form 3:
 * isotropic phase-field Zener pinning as shipped
 * (examples/coarsening/zener_pinning/isotropic/phase_field/zener.cpp:121-138):
 * form 1 with field 0 (the particles) copied unchanged. */
static int ac_run(const pfo_grid* g, int N, double* eta, int steps, int form,
                  double gamma, double kappa, double L, double r, double u,
                  double dt, int threads, double nstd, uint64_t seed, long long step0)
{
    geo q;
    if (N < 1 || N > 64 || geo_init(&q, g) || !eta || steps < 0) return -1;
    if (form == 2 && N != 1) { geo_free(&q); return -1; }
    double* nw = (double*)malloc(sizeof(double) * (size_t)q.cells * (size_t)N);
    if (!nw) { geo_free(&q); return -1; }
    double* old = eta;
    int nt = nthreads(threads);
    (void)nt;
    for (int step = 0; step < steps; step++) {
        #pragma omp parallel for schedule(static) num_threads(nt)
        for (int i0 = 0; i0 < q.n[0]; i0++)
            for (int i1 = 0; i1 < q.n[1]; i1++)
                for (int i2 = 0; i2 < q.n[2]; i2++) {
                    int xc[3] = {i0, i1, i2};
                    long i = i0 * q.st[0] + i1 * q.st[1] + i2;
                    const double* phi = old + i * N;
                    double* out = nw + i * N;
                    double lap[64];
                    for (int j = 0; j < N; j++) lap[j] = lap_at(&q, old, i, N, j, xc);
                    if (form == 2) {
                        double p = phi[0];
                        if (nstd != 0.0) /* model_A.cpp:99-100 */
                            out[0] = p - dt * L * (-r * p + u * pow(p, 3) - kappa * lap[0]
                                                   + noise_at(nstd, seed, step0 + step, q.cells, i));
                        else
                            out[0] = p - dt * L * (-r * p + u * pow(p, 3) - kappa * lap[0]);
                        continue;
                    }
                    /* sum of squares, graingrowth.cpp:97-101 */
                    double sum = 0.0;
                    for (int j = 0; j < N; j++) sum += phi[j] * phi[j];
                    if (form == 0) {
                        for (int j = 0; j < N; j++)
                            out[j] = phi[j] - dt * L * (-phi[j] + phi[j] * phi[j] * phi[j]
                                     + 2.0 * gamma * phi[j] * (sum - phi[j] * phi[j])
                                     - kappa * lap[j]);
                    } else {
                        for (int j = 0; j < N; j++)
                            out[j] = phi[j] - dt * (-phi[j] - pow(phi[j], 3) + 2.0 * (phi[j] * sum - lap[j]));
                        if (form == 3) out[0] = phi[0];   /* particles have zero mobility (zener.cpp:134) */
                    }
                }
        double* t = old;
        old = nw;
        nw = t;
    }
    if (old != eta) {
        memcpy(eta, old, sizeof(double) * (size_t)q.cells * (size_t)N);
        nw = old;
    }
    free(nw);
    geo_free(&q);
    return 0;
}

int pfo_ac_baseline(const pfo_grid* g, int N, double* eta, int steps,
                    double gamma, double kappa, double L, double dt, int threads)
{
    return ac_run(g, N, eta, steps, 0, gamma, kappa, L, 0.0, 0.0, dt, threads, 0.0, 0, 0);
}

int pfo_ac_graingrowth(const pfo_grid* g, int N, double* eta, int steps,
                       double dt, int threads)
{
    return ac_run(g, N, eta, steps, 1, 0.0, 0.0, 1.0, 0.0, 0.0, dt, threads, 0.0, 0, 0);
}

int pfo_ac_zener(const pfo_grid* g, int N, double* eta, int steps, double dt, int threads)
{
    return ac_run(g, N, eta, steps, 3, 0.0, 0.0, 1.0, 0.0, 0.0, dt, threads, 0.0, 0, 0);
}

int pfo_ac_scalar_shipped(const pfo_grid* g, double* phi, int steps,
                          double r, double u, double K, double M, double dt,
                          int threads)
{
    return ac_run(g, 1, phi, steps, 2, 0.0, K, M, r, u, dt, threads, 0.0, 0, 0);
}

int pfo_ac_scalar_noise(const pfo_grid* g, double* phi, int steps, double r, double u, double K, double M,
                        double dt, double nstd, uint64_t seed, long long step0, int threads)
{
    return ac_run(g, 1, phi, steps, 2, 0.0, K, M, r, u, dt, threads, nstd, seed, step0);
}

/* Isotropic phase-field Ostwald ripening, ostwald.cpp:84-121: field 0 the
 * composition C, fields 1..N-1 the order parameters.  Pass 1 writes the
 * chemical potential into a scalar work grid (:89-100); pass 2 updates C
 * from its Laplacian and each order parameter from its own (:103-120).
 * The derived constants follow :67-80 with the same pow calls. */
int pfo_ostwald(const pfo_grid* g, int N, double* eta, int steps, double dt, double L, double D,
                double Calpha, double Cbeta, double A, double delta, double epsilon, double kappa,
                int threads)
{
    geo q;
    if (N < 2 || N > 64 || geo_init(&q, g) || !eta || steps < 0) return -1;
    const double Cmatrix = 0.5 * (Calpha + Cbeta);
    const double B = A / pow(Cbeta - Cmatrix, 2);
    const double gamma = 2.0 / pow(Cbeta - Calpha, 2);
    const double Dalpha = gamma / pow(delta, 2);
    const double Dbeta = gamma / pow(delta, 2);
    double* nw = (double*)malloc(sizeof(double) * (size_t)q.cells * (size_t)N);
    double* w = (double*)malloc(sizeof(double) * (size_t)q.cells);
    if (!nw || !w) { free(nw); free(w); geo_free(&q); return -1; }
    double* old = eta;
    int nt = nthreads(threads);
    (void)nt;
    for (int step = 0; step < steps; step++) {
        #pragma omp parallel for schedule(static) num_threads(nt)
        for (int i0 = 0; i0 < q.n[0]; i0++)
            for (int i1 = 0; i1 < q.n[1]; i1++)
                for (int i2 = 0; i2 < q.n[2]; i2++) {
                    int xc[3] = {i0, i1, i2};
                    long i = i0 * q.st[0] + i1 * q.st[1] + i2;
                    const double* phi = old + i * N;
                    double sum = 0.0;
                    for (int j = 1; j < N; j++) sum += pow(phi[j], 2);
                    double C = phi[0];
                    double lap = lap_at(&q, old, i, N, 0, xc);
                    w[i] = -A * (C - Cmatrix) + B * pow(C - Cmatrix, 3)
                           + Dalpha * pow(C - Calpha, 3) + Dbeta * pow(C - Cbeta, 3)
                           - gamma * (C - Calpha) * sum - kappa * lap;
                }
        #pragma omp parallel for schedule(static) num_threads(nt)
        for (int i0 = 0; i0 < q.n[0]; i0++)
            for (int i1 = 0; i1 < q.n[1]; i1++)
                for (int i2 = 0; i2 < q.n[2]; i2++) {
                    int xc[3] = {i0, i1, i2};
                    long i = i0 * q.st[0] + i1 * q.st[1] + i2;
                    const double* phi = old + i * N;
                    double* out = nw + i * N;
                    double lap = lap_at(&q, w, i, 1, 0, xc);
                    double C = phi[0];
                    out[0] = C + dt * D * lap;
                    double sum = 0.0;
                    for (int j = 1; j < N; j++) sum += pow(phi[j], 2);
                    for (int j = 1; j < N; j++) {
                        double value = phi[j];
                        double vlap = lap_at(&q, old, i, N, j, xc);
                        out[j] = value - dt * L * (-gamma * pow(C - Calpha, 2) + delta * pow(value, 3)
                                                   + epsilon * value * (sum - pow(value, 2)) - kappa * vlap);
                    }
                }
        double* t = old;
        old = nw;
        nw = t;
    }
    if (old != eta) {
        memcpy(eta, old, sizeof(double) * (size_t)q.cells * (size_t)N);
        nw = old;
    }
    free(nw);
    free(w);
    geo_free(&q);
    return 0;
}

/* Convex-splitting Cahn-Hilliard, update() of
 * examples/phase_transitions/cahn-hilliard/convex_splitting/cahn-hilliard.cpp:273-463
 * with the parametric free energy (:38-96) and the constants as arguments.
 * cm is cell-major (c, mu).  Serial red-black sweeps in cell order, the
 * residual of :353-388 after iterations 1-4 and every 5th, the guess of the
 * next step being the state two steps back (newGrid after swap).  Returns
 * -2 when a step reaches max_iter; *iters receives the iterations of the
 * last step. */
int pfo_ch_convex(const pfo_grid* g, double* cm, int steps, double dt, double D, double K, double C0,
                  double Ca, double Cb, double A, double omega, double tolerance, int* iters)
{
    geo q;
    if (geo_init(&q, g) || !cm || steps < 0) return -1;
    const double B = A / pow(Ca - C0, 2.0);
    const double QA = B + Ca + Cb;
    const double QB = 3.0 * (B * C0 + Ca * Ca + Cb * Cb);
    const double QC = 3.0 * (B * C0 * C0 + pow(Ca, 3.0) + pow(Cb, 3.0));
    const double QD = B * pow(C0, 3.0) + pow(Ca, 4.0) + pow(Cb, 4.0);
    const unsigned residual_step = 5, max_iter = 10000;
    double lapWeight = 0.0;
    for (int a = 0; a < q.dim; a++) lapWeight += 2.0 / pow(g->dx[a], 2.0);
    const double gridSize = (double)q.cells;
    double* nw = (double*)malloc(sizeof(double) * 2 * (size_t)q.cells);
    if (!nw) { geo_free(&q); return -1; }
    memcpy(nw, cm, sizeof(double) * 2 * (size_t)q.cells);   /* newGrid.copy(oldGrid) */
    double* old = cm;
    int rc = 0;
    for (int step = 0; step < steps && rc == 0; step++) {
        double residual = 1.0;
        unsigned iter = 0;
        while (iter < max_iter && residual > tolerance) {
            for (int color = 1; color > -1; color--)
                for (int i0 = 0; i0 < q.n[0]; i0++)
                    for (int i1 = 0; i1 < q.n[1]; i1++)
                        for (int i2 = 0; i2 < q.n[2]; i2++) {
                            if ((i0 + i1 + i2) % 2 == color) continue;
                            int xc[3] = {i0, i1, i2};
                            long i = i0 * q.st[0] + i1 * q.st[1] + i2;
                            double cOld = old[2 * i];
                            double cGuess = nw[2 * i];
                            double uGuess = nw[2 * i + 1];
                            double A12 = dt * D * lapWeight;
                            double A21 = -(QA * pow(nw[2 * i], 2.0) + QC) - K * lapWeight;
                            double detA = 1.0 - (A12 * A21);
                            /* fringe_laplacian (:155-170) of fields 1 and 0 */
                            double f1 = 0.0, f0 = 0.0;
                            int off = 3 - q.dim;
                            for (int ra = 0; ra < q.dim; ra++) {
                                int a = off + ra;
                                double weight = 1.0 / pow(g->dx[ra], 2.0);
                                long hi = i + NB_HI(&q, a, xc[a]), lo = i + NB_LO(&q, a, xc[a]);
                                f1 += weight * (nw[2 * hi + 1] + nw[2 * lo + 1]);
                                f0 += weight * (nw[2 * hi] + nw[2 * lo]);
                            }
                            double B1 = cOld + D * dt * f1;
                            double B2 = (-A * (cOld - C0) - QB * pow(cOld, 2.0) - QD) - K * f0;
                            double cNew = (B1 - B2 * A12) / detA;
                            double uNew = (B2 - B1 * A21) / detA;
                            nw[2 * i] = omega * cNew + (1.0 - omega) * cGuess;
                            nw[2 * i + 1] = omega * uNew + (1.0 - omega) * uGuess;
                        }
            iter++;
            if (iter < residual_step || iter % residual_step == 0) {
                double normB = 0.0;
                residual = 0.0;
                for (int i0 = 0; i0 < q.n[0]; i0++)
                    for (int i1 = 0; i1 < q.n[1]; i1++)
                        for (int i2 = 0; i2 < q.n[2]; i2++) {
                            int xc[3] = {i0, i1, i2};
                            long i = i0 * q.st[0] + i1 * q.st[1] + i2;
                            double lapC = lap_at(&q, nw, i, 2, 0, xc);
                            double lapU = lap_at(&q, nw, i, 2, 1, xc);
                            double cOld = old[2 * i], cNew = nw[2 * i], uNew = nw[2 * i + 1];
                            double B1 = cOld;
                            double B2 = -A * (cOld - C0) - QB * pow(cOld, 2.0) - QD;
                            double AX1 = cNew - D * dt * lapU;
                            double AX2 = uNew - (QA * pow(cNew, 3.0) + QC * cNew) + K * lapC;
                            double R1 = B1 - AX1;
                            double R2 = B2 - AX2;
                            residual += R1 * R1 + R2 * R2;
                            normB += B1 * B1 + B2 * B2;
                        }
                residual = sqrt(residual / normB) / (2.0 * gridSize);
            }
        }
        if (iters) *iters = (int)iter;
        if (iter == max_iter) rc = -2;
        double* t = old;   /* swap(oldGrid,newGrid) */
        old = nw;
        nw = t;
    }
    if (old != cm) {
        memcpy(cm, old, sizeof(double) * 2 * (size_t)q.cells);
        nw = old;
    }
    free(nw);
    geo_free(&q);
    return rc;
}

/* Neumaier's improvement of Kahan summation. */
typedef struct { double s, c; } nsum;
static inline void nadd(nsum* a, double x)
{
    double t = a->s + x;
    if (fabs(a->s) >= fabs(x)) a->c += (a->s - t) + x;
    else a->c += (x - t) + a->s;
    a->s = t;
}
static inline double nval(const nsum* a) { return a->s + a->c; }

/* |grad f_j|^2 at a cell with gradient() of grid.cpp:2154-2170:
 * g_i = (1/(2 dx_i)) * (yh - yl), summed as g_i*g_i over axes. */
static inline double gradsq_at(const geo* q, const double* f, long idx, int N, int j,
                               const int xc[3])
{
    double s = 0.0;
    int off = 3 - q->dim;
    for (int ra = 0; ra < q->dim; ra++) {
        int a = off + ra;
        const double yh = f[(idx + NB_HI(q, a, xc[a])) * N + j];
        const double yl = f[(idx + NB_LO(q, a, xc[a])) * N + j];
        double gi = q->wg[ra] * (yh - yl);
        s += gi * gi;
    }
    return s;
}

static double cell_volume(const pfo_grid* g)
{
    double dV = 1.0;
    for (int a = 0; a < g->dim; a++) dV *= g->dx[a];
    return dV;
}

int pfo_ch_mass_energy(const pfo_grid* g, const double* c, double kappa,
                       double* mass, double* energy)
{
    geo q;
    if (geo_init(&q, g) || !c) return -1;
    nsum m = {0, 0}, e = {0, 0};
    for (int i0 = 0; i0 < q.n[0]; i0++)
        for (int i1 = 0; i1 < q.n[1]; i1++)
            for (int i2 = 0; i2 < q.n[2]; i2++) {
                int xc[3] = {i0, i1, i2};
                long i = i0 * q.st[0] + i1 * q.st[1] + i2;
                double C = c[i];
                double omc = 1.0 - C;
                double f = C * C * omc * omc;
                nadd(&e, f + 0.5 * kappa * gradsq_at(&q, c, i, 1, 0, xc));
                nadd(&m, C);
            }
    double dV = cell_volume(g);
    if (mass) *mass = dV * nval(&m);
    if (energy) *energy = dV * nval(&e);
    geo_free(&q);
    return 0;
}

int pfo_ac_mass_energy(const pfo_grid* g, int N, const double* eta,
                       double gamma, double kappa, double* mass, double* energy)
{
    geo q;
    if (N < 1 || N > 64 || geo_init(&q, g) || !eta) return -1;
    nsum e = {0, 0};
    nsum m[64];
    for (int j = 0; j < N; j++) m[j].s = m[j].c = 0.0;
    for (int i0 = 0; i0 < q.n[0]; i0++)
        for (int i1 = 0; i1 < q.n[1]; i1++)
            for (int i2 = 0; i2 < q.n[2]; i2++) {
                int xc[3] = {i0, i1, i2};
                long i = i0 * q.st[0] + i1 * q.st[1] + i2;
                const double* p = eta + i * N;
                double bulk = 0.0, pair = 0.0, grad = 0.0, sq = 0.0;
                for (int j = 0; j < N; j++) {
                    double p2 = p[j] * p[j];
                    bulk += -0.5 * p2 + 0.25 * p2 * p2;
                    pair += p2 * sq;          /* sum_{k<j} e_k^2 e_j^2 */
                    sq += p2;
                    grad += gradsq_at(&q, eta, i, N, j, xc);
                    nadd(&m[j], p[j]);
                }
                nadd(&e, bulk + gamma * pair + 0.5 * kappa * grad);
            }
    double dV = cell_volume(g);
    if (mass)
        for (int j = 0; j < N; j++) mass[j] = dV * nval(&m[j]);
    if (energy) *energy = dV * nval(&e);
    geo_free(&q);
    return 0;
}

void pfo_pow3(const double* x, double* y, long n)
{
    for (long i = 0; i < n; i++) y[i] = pow(x[i], 3);
}

/* ---- isotropic sparse phase-field grain growth ------------------------------------------------
 * examples/coarsening/grain_growth/isotropic/sparsePF/graingrowth.cpp:58-120 over
 * grid<dim,sparse<double>> (include/MMSP.sparse.h:19, MMSP.sparse.cpp).  A cell is a list of
 * (index, value) items in insertion order; set() overwrites an item or appends one
 * (MMSP.sparse.cpp set), operator[] reads 0 for an absent index.  Here a list lives in K slots:
 * cnt[c] items, idx[c*K + h], val[c*K + h].
 *
 * The sparse Laplacian (include/MMSP.grid.cpp:2110-2128) combines the items of yh, 2.0*y and yl
 * through sparse operator+/- (MMSP.sparse.cpp), which start every index at 0 and add or
 * subtract; each operation is exact where an index is absent, so its value for index i is the
 * dense expression weight*((yh_i - 2.0*y_i) + yl_i), summed over axes from 0.0, with absent
 * items read as 0.  Only the sign of an exact zero can differ, and the update below cannot
 * carry it into a stored value.
 *
 * update() builds newGrid by the copy constructor, whose cells start empty, and never clears
 * it: after swap() the grid written at step s holds the state of step s-2, and set() leaves
 * the items it does not overwrite.  Those stale items are part of the state (they enter the
 * neighbour sets, the sum of squares and the Laplacians), so this restatement keeps them too:
 * buffer B starts empty on every call, as each update() call's newGrid does. */
static inline int sp_find(const int* cnt, const int* idx, int K, long c, int i)
{
    const int n = cnt[c];
    const int* ix = idx + c * K;
    for (int h = 0; h < n; h++)
        if (ix[h] == i) return h;
    return -1;
}

static inline double sp_get(const int* cnt, const int* idx, const double* val, int K, long c, int i)
{
    const int h = sp_find(cnt, idx, K, c, i);
    return h < 0 ? 0.0 : val[c * K + h];
}

#define PFO_SPARSE_SET 256   /* largest neighbour set (union of 2*dim+1 lists) */

int pfo_sparse_gg(const pfo_grid* g, int K, int* cnt, int* idx, double* val, int steps, double dt, double eps,
                  int threads, int* longest)
{
    geo q;
    if (K < 1 || K > 64 || steps < 0 || !cnt || !idx || !val || geo_init(&q, g) != 0) return -1;
    const long cells = q.cells;
    int* bc = (int*)calloc((size_t)cells, sizeof(int));
    int* bi = (int*)calloc((size_t)cells * K, sizeof(int));
    double* bv = (double*)calloc((size_t)cells * K, sizeof(double));
    if (!bc || !bi || !bv) {
        free(bc); free(bi); free(bv); geo_free(&q);
        return -1;
    }
    int *ac = cnt, *ai = idx, *xc_ = bc, *xi = bi;
    double *av = val, *xv = bv;
    int overflow = 0, maxlen = 0;
    for (long c = 0; c < cells; c++) {
        if (cnt[c] < 0 || cnt[c] > K) overflow = 1;
        if (cnt[c] > maxlen) maxlen = cnt[c];
    }
    const int off = 3 - q.dim;
    const int nt = nthreads(threads);
    for (int step = 0; step < steps && !overflow; step++) {
        int ovf = 0, mx = 0;
#ifdef _OPENMP
#pragma omp parallel for num_threads(nt) schedule(static) reduction(| : ovf) reduction(max : mx)
#endif
        for (long c = 0; c < cells; c++) {
            int xc[3];
            xc[0] = (int)(c / q.st[0]);
            xc[1] = (int)((c / q.st[1]) % q.n[1]);
            xc[2] = (int)(c % q.n[2]);
            /* nonzero fields of the neighbourhood, in the example's visiting order:
             * per axis the low neighbour, the cell itself, the high neighbour */
            int S[PFO_SPARSE_SET];
            int ns = 0;
            for (int ra = 0; ra < q.dim; ra++) {
                const int a = off + ra;
                for (int k = -1; k <= 1; k++) {
                    const long nc = k < 0 ? c + NB_LO(&q, a, xc[a]) : k > 0 ? c + NB_HI(&q, a, xc[a]) : c;
                    for (int h = 0; h < ac[nc]; h++) {
                        const int i = ai[nc * K + h];
                        int seen = 0;
                        for (int s = 0; s < ns; s++)
                            if (S[s] == i) { seen = 1; break; }
                        if (!seen) {
                            if (ns == PFO_SPARSE_SET) { ovf = 1; break; }
                            S[ns++] = i;
                        }
                    }
                }
            }
            if (ns < 2) {
                /* newGrid(n) = oldGrid(n): the whole list */
                xc_[c] = ac[c];
                for (int h = 0; h < ac[c]; h++) {
                    xi[c * K + h] = ai[c * K + h];
                    xv[c * K + h] = av[c * K + h];
                }
            } else {
                double sum = 0.0;
                for (int h = 0; h < ac[c]; h++) {
                    const double phi = av[c * K + h];
                    sum += phi * phi;
                }
                for (int s = 0; s < ns; s++) {
                    const int i = S[s];
                    const double phi = sp_get(ac, ai, av, K, c, i);
                    double lap = 0.0;
                    for (int ra = 0; ra < q.dim; ra++) {
                        const int a = off + ra;
                        const double yh = sp_get(ac, ai, av, K, c + NB_HI(&q, a, xc[a]), i);
                        const double yl = sp_get(ac, ai, av, K, c + NB_LO(&q, a, xc[a]), i);
                        lap += q.w[ra] * (yh - 2.0 * phi + yl);
                    }
                    const double value = phi - dt * (-phi - pow(phi, 3) + 2.0 * (phi * sum - lap));
                    if (value > eps) {
                        int h = sp_find(xc_, xi, K, c, i);
                        if (h < 0) {
                            if (xc_[c] == K) { ovf = 1; continue; }
                            h = xc_[c]++;
                            xi[c * K + h] = i;
                        }
                        xv[c * K + h] = value;
                    }
                }
            }
            if (xc_[c] > mx) mx = xc_[c];
        }
        overflow |= ovf;
        if (mx > maxlen) maxlen = mx;
        /* swap(oldGrid, newGrid) */
        int* t = ac; ac = xc_; xc_ = t;
        t = ai; ai = xi; xi = t;
        double* tv = av; av = xv; xv = tv;
    }
    if (ac != cnt) {
        memcpy(cnt, ac, sizeof(int) * (size_t)cells);
        memcpy(idx, ai, sizeof(int) * (size_t)cells * K);
        memcpy(val, av, sizeof(double) * (size_t)cells * K);
    }
    free(bc); free(bi); free(bv);
    geo_free(&q);
    if (longest) *longest = maxlen;
    return overflow ? -3 : 0;
}
