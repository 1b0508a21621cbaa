/* pf_oracle.h -- CPU oracle for the explicit phase-field step (TEST INFRASTRUCTURE).
 *
 * This is the checker, not the product.  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline legs may load it.  It restates, in plain C, the
 * arithmetic of MMSP's serial explicit-Euler update() loops:
 *
 *   MMSP::laplacian            include/MMSP.grid.cpp:2049-2066 (scalar),
 *                              :2068-2088 (vector<T>), index overloads :2130-2140
 *   check_boundary             include/MMSP.utility.cpp:42-57 (serial build)
 *   explicit Cahn-Hilliard     examples/phase_transitions/cahn-hilliard/explicit/cahn-hilliard.cpp:47-81
 *   isotropic PF grain growth  examples/coarsening/grain_growth/isotropic/phase_field/graingrowth.cpp:73-111
 *   scalar Allen-Cahn          examples/phase_transitions/allen-cahn/allen-cahn.cpp:47-75
 *   mass / free energy         examples/phase_transitions/cahn-hilliard/convex_splitting/cahn-hilliard.cpp:179-213
 *                              with gradient() include/MMSP.grid.cpp:2154-2170
 *
 * The operation order of every expression is the reference's own (left to
 * right, no reassociation); the file must be compiled with -ffp-contract=off
 * so that no multiply-add is fused.  The cell loops run in the reference's
 * node order; the optional OpenMP threads split independent cells only, so a
 * threaded run is bit-identical to a serial one.  Reductions are serial.
 *
 * Parity pin: tests/golden/ holds outputs of the reference's own grid,
 * laplacian and swap, compiled from the reference headers by
 * oracle/ref_api/ref_update.cpp; tests/test_oracle_golden.py checks this file
 * against them bit for bit.
 *
 * Layout: row-major, last index fastest, data[(x0*n1 + x1)*n2 + x2]
 * (include/MMSP.grid.cpp:306-313).  Vector-valued grids are cell-major
 * (value j of cell i at i*N + j), the order of grid<dim,vector<T>>::to_buffer
 * without the per-cell length prefix.
 */
#ifndef PF_ORACLE_H
#define PF_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Boundary-condition codes of include/MMSP.utility.h:23-29. */
enum { PFO_MIRROR = 0, PFO_NEUMANN = 1, PFO_PERIODIC = 2, PFO_PARALLEL = 3, PFO_DIRICHLET = 4 };

typedef struct {
    int dim;        /* 1, 2 or 3 */
    int n[3];       /* extents, axis 0 slowest; unused axes ignored */
    double dx[3];   /* cell spacing per axis */
    int bc[3][2];   /* lower / upper boundary condition per axis */
} pfo_grid;

/* Number of cells. */
long pfo_nodes(const pfo_grid* g);

/* Cahn-Hilliard with f(c)=c^2(1-c)^2, two passes as cahn-hilliard.cpp:69-76:
 *   temp = 2c(1-c)(1-2c) - kappa*lap(c);  c' = c + dt*M*lap(temp).
 * Returns 0, or -1 on bad arguments. */
int pfo_ch_baseline(const pfo_grid* g, double* c, int steps,
                    double kappa, double M, double dt, int threads);

/* Cahn-Hilliard exactly as shipped (cahn-hilliard.cpp:71,76):
 *   temp = -r*c + u*pow(c,3) - K*lap(c);  c' = c + dt*M*lap(temp). */
int pfo_ch_shipped(const pfo_grid* g, double* c, int steps,
                   double r, double u, double K, double M, double dt, int threads);

/* Multi-order-parameter Allen-Cahn with
 *   f = sum(-e^2/2 + e^4/4) + gamma*sum_{i<j} e_i^2 e_j^2,
 * single pass in the structure of graingrowth.cpp:91-107:
 *   sum = sum_j e_j*e_j
 *   e_j' = e_j - dt*L*(-e_j + e_j*e_j*e_j + 2*gamma*e_j*(sum - e_j*e_j) - kappa*lap_j).
 * eta is cell-major with N values per cell. */
int pfo_ac_baseline(const pfo_grid* g, int N, double* eta, int steps,
                    double gamma, double kappa, double L, double dt, int threads);

/* Grain growth exactly as shipped (graingrowth.cpp:104-106):
 *   e_j' = e_j - dt*(-e_j - pow(e_j,3) + 2*(e_j*sum - lap_j)). */
int pfo_ac_graingrowth(const pfo_grid* g, int N, double* eta, int steps,
                       double dt, int threads);

/* Isotropic phase-field Zener pinning exactly as shipped
 * (examples/coarsening/zener_pinning/isotropic/phase_field/zener.cpp:121-138):
 * grain growth with field 0, the particles, held fixed; the sum of squares
 * still runs over every field. */
int pfo_ac_zener(const pfo_grid* g, int N, double* eta, int steps, double dt, int threads);

/* Isotropic phase-field Ostwald ripening exactly as shipped
 * (examples/coarsening/ostwald_ripening/isotropic/phase_field/ostwald.cpp:84-121),
 * with the constants of :66-80 as arguments.  eta is cell-major with N >= 2
 * values per cell: the composition first, then the order parameters. */
int pfo_ostwald(const pfo_grid* g, int N, double* eta, int steps, double dt, double L, double D,
                double Calpha, double Cbeta, double A, double delta, double epsilon, double kappa,
                int threads);

/* Stochastic forms.  The examples add gaussian(0.0, std) to the
 * polynomial models' mu (model_A.cpp:99-100 on the scalar Allen-Cahn update,
 * model_B.cpp:100-101 and spinodal.cpp:95-97 on the Cahn-Hilliard mu pass), drawn
 * from rand() in cell order.  These restatements draw the same term from a
 * counter-based stream instead: deviate (step0 + step) * cells + cell of
 * pfo_gaussian(seed, .), times std.  std = 0 reproduces the deterministic
 * functions bit for bit. */
double pfo_gaussian(uint64_t seed, uint64_t k);
int pfo_ch_shipped_noise(const pfo_grid* g, double* c, int steps, double r, double u, double K, double M,
                         double dt, double nstd, uint64_t seed, long long step0, int threads);
int pfo_ac_scalar_noise(const pfo_grid* g, double* phi, int steps, double r, double u, double K, double M,
                        double dt, double nstd, uint64_t seed, long long step0, int threads);

/* Convex-splitting Cahn-Hilliard exactly as shipped
 * (examples/phase_transitions/cahn-hilliard/convex_splitting/cahn-hilliard.cpp:273-463,
 * parametric free energy), serial; cm cell-major (c, mu).  Returns -2 when a
 * step reaches 10000 iterations; *iters gets the last step's iterations. */
int pfo_ch_convex(const pfo_grid* g, double* cm, int steps, double dt, double D, double K, double C0,
                  double Ca, double Cb, double A, double omega, double tolerance, int* iters);

/* Scalar Allen-Cahn exactly as shipped (allen-cahn.cpp:70):
 *   p' = p - dt*M*(-r*p + u*pow(p,3) - K*lap(p)). */
int pfo_ac_scalar_shipped(const pfo_grid* g, double* phi, int steps,
                          double r, double u, double K, double M, double dt,
                          int threads);

/* One application of the scalar Laplacian to every cell (grid.cpp:2049-2066). */
int pfo_laplacian(const pfo_grid* g, const double* in, double* out);

/* Compensated (Neumaier) FP64 sums in node order:
 *   mass   = dV * sum c
 *   energy = dV * sum [ c^2 (1-c)^2 + kappa/2 |grad c|^2 ]
 * with the central-difference gradient of grid.cpp:2154-2170. */
int pfo_ch_mass_energy(const pfo_grid* g, const double* c, double kappa,
                       double* mass, double* energy);

/* Per-field masses (dV * sum e_j, N values into mass[]) and the free energy
 *   dV * sum [ sum_j(-e_j^2/2 + e_j^4/4) + gamma*sum_{i<j} e_i^2 e_j^2
 *              + kappa/2 sum_j |grad e_j|^2 ]. */
int pfo_ac_mass_energy(const pfo_grid* g, int N, const double* eta,
                       double gamma, double kappa, double* mass, double* energy);

/* Isotropic sparse phase-field grain growth exactly as shipped
 * (examples/coarsening/grain_growth/isotropic/sparsePF/graingrowth.cpp:58-120) on
 * grid<dim,sparse<double>> (include/MMSP.sparse.h:19): per cell a list of (index, value)
 * items in insertion order, in K slots: cnt[c] items at idx[c*K + h], val[c*K + h].  One call
 * is one update() call: its newGrid starts with empty cells and keeps the stale items of two
 * steps back, as the example's does.  *longest gets the longest list seen.  Returns -3 when
 * a list would exceed K items. */
int pfo_sparse_gg(const pfo_grid* g, int K, int* cnt, int* idx, double* val, int steps, double dt, double eps,
                  int threads, int* longest);

/* pow(x,3) through the C library, for checking a device cube routine. */
void pfo_pow3(const double* x, double* y, long n);

#ifdef __cplusplus
}
#endif
#endif
