/* MMSP.gpu.h -- C ABI of the GB300 explicit phase-field step (libmmsp_gpu.so).
 *
 * This is the drop-in boundary for MMSP's explicit-Euler update() of
 * Cahn-Hilliard and multi-order-parameter Allen-Cahn grids.  Each entry point
 * replaces a piece of the reference's serial path:
 *
 *   mmsp_gpu_update    the whole plugin call update(grid&, steps):
 *                      examples/phase_transitions/cahn-hilliard/explicit/cahn-hilliard.cpp:47-81,
 *                      examples/coarsening/grain_growth/isotropic/phase_field/graingrowth.cpp:73-111,
 *                      examples/phase_transitions/allen-cahn/allen-cahn.cpp:47-75
 *   mmsp_gpu_create    the scratch grids newGrid/temp of update() (copy-ctor,
 *                      include/MMSP.grid.cpp:71-99) and the grid geometry
 *                      (setup, include/MMSP.grid.cpp:141-327)
 *   mmsp_gpu_upload / mmsp_gpu_download
 *                      the host grid's storage, read as grid<dim,T>::to_buffer
 *                      order (include/MMSP.grid.cpp:1146-1157) without the
 *                      per-cell vector length
 *   mmsp_gpu_step      the step loop of update(): laplacian
 *                      (include/MMSP.grid.cpp:2049-2088), the model's pointwise
 *                      update, swap (include/MMSP.grid.cpp:1913-1991) and the
 *                      periodic halo of ghostswap (include/MMSP.grid.cpp:414-515)
 *                      as serial check_boundary wraps it (include/MMSP.utility.cpp:42-57)
 *   mmsp_gpu_reduce    mass and free energy of a snapshot, as reportEnergy()
 *                      sums them (examples/phase_transitions/cahn-hilliard/
 *                      convex_splitting/cahn-hilliard.cpp:179-213), in FP64
 *                      with compensated accumulation
 *
 * All functions return MMSP_GPU_OK (0) or a negative MMSP_GPU_E* code; none
 * throws, exits or prints.  The reference reports the same failures with
 * exit()/MMSP::Abort() (include/MMSP.utility.cpp:30-36); the C++ wrapper
 * MMSP.gpu.hpp maps a failure to std::cerr + MMSP::Abort(code).
 *
 * Threading: calls on one handle must not overlap; different handles are
 * independent.  Device work of a handle is ordered on that handle's stream.
 */
#ifndef MMSP_GPU_H
#define MMSP_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MMSP_GPU_ABI_VERSION 3

/* Status codes. */
#define MMSP_GPU_OK            0
#define MMSP_GPU_EINVAL       -1  /* argument out of range, size mismatch, NULL pointer */
#define MMSP_GPU_ENOMEM       -2  /* device allocation failed or memory budget exceeded */
#define MMSP_GPU_ECUDA        -3  /* CUDA runtime error (message in mmsp_gpu_last_error) */
#define MMSP_GPU_EUNSUPPORTED -4  /* valid MMSP input that the device path does not handle */
#define MMSP_GPU_ETIMEDOUT    -5  /* a bounded wait ran out */
#define MMSP_GPU_ENODEV       -6  /* no CUDA device, or not an sm_103 device */
#define MMSP_GPU_ENOTFOUND    -7  /* unknown request id (server) */
#define MMSP_GPU_ECANCELED    -8  /* request cancelled (server) */
#define MMSP_GPU_ESTOPPED     -9  /* server stopped */
#define MMSP_GPU_EIO         -10  /* a grid file could not be opened or written */
#define MMSP_GPU_ENOCONV     -11  /* an implicit solve reached its iteration limit (the reference aborts) */
#define MMSP_GPU_EOVERFLOW   -12  /* a sparse cell's item list outgrew its slots (mmsp_gpu_desc.fields) */

/* Boundary-condition codes, identical to include/MMSP.utility.h:23-29. */
#define MMSP_GPU_BC_MIRROR    0
#define MMSP_GPU_BC_NEUMANN   1
#define MMSP_GPU_BC_PERIODIC  2
#define MMSP_GPU_BC_PARALLEL  3
#define MMSP_GPU_BC_DIRICHLET 4

/* Storage type of the state (and the arithmetic of the step). */
#define MMSP_GPU_F64 0   /* plain form: reference operation order, no fused multiply-add */
#define MMSP_GPU_F32 1   /* precision form: FP32 state and arithmetic, FP64 reductions */

/* mmsp_gpu_desc.flags */
#define MMSP_GPU_FLAG_CONTRACT 1  /* FP64 Cahn-Hilliard (MMSP_GPU_CH, MMSP_GPU_CH_POLY) in 2D and 3D:
                                     fused multiply-adds and a regrouped Laplacian (16 FP64 operations
                                     per cell instead of the reference order's 23); results within
                                     1e-12 relative of the reference instead of bit-identical.  Other
                                     models, dims and FP32 ignore it. */

/* Models.  Parameters are read from mmsp_gpu_desc as noted. */
#define MMSP_GPU_CH       0  /* Cahn-Hilliard, f=c^2(1-c)^2: mu = 2c(1-c)(1-2c) - kappa*lap c;
                                c' = c + dt*mobility*lap mu                                   */
#define MMSP_GPU_CH_POLY  1  /* Cahn-Hilliard as shipped (cahn-hilliard.cpp:71):
                                mu = -r c + u c^3 - kappa*lap c                              */
#define MMSP_GPU_AC       2  /* multi-order Allen-Cahn, f = sum(-e^2/2+e^4/4) + gamma*sum_{i<j} e_i^2 e_j^2:
                                e' = e - dt*mobility*(-e + e^3 + 2 gamma e (sum e^2 - e^2) - kappa*lap e) */
#define MMSP_GPU_GG       3  /* grain growth as shipped (graingrowth.cpp:105):
                                e' = e - dt*(-e - e^3 + 2 (e sum e^2 - lap e))                */
#define MMSP_GPU_AC_POLY  4  /* scalar Allen-Cahn as shipped (allen-cahn.cpp:70), fields=1:
                                p' = p - dt*mobility*(-r p + u p^3 - kappa*lap p)             */
#define MMSP_GPU_ZENER    5  /* isotropic phase-field Zener pinning as shipped
                                (examples/coarsening/zener_pinning/isotropic/phase_field/zener.cpp:121-138):
                                MMSP_GPU_GG with field 0 (the particles) held fixed; the sum of
                                squares still runs over every field                            */
#define MMSP_GPU_OSTWALD  6  /* isotropic phase-field Ostwald ripening as shipped
                                (examples/coarsening/ostwald_ripening/isotropic/phase_field/ostwald.cpp:56-123),
                                fields >= 2: field 0 the composition C, fields 1.. the order
                                parameters e_i; two passes per step:
                                w   = -A(C-Cm) + B(C-Cm)^3 + Da(C-Ca)^3 + Db(C-Cb)^3
                                      - g (C-Ca) sum e_i^2 - kappa lap C
                                C'  = C + dt*D*lap w
                                e_i'= e_i - dt*L*(-g (C-Ca)^2 + delta e_i^3 + eps e_i (sum - e_i^2)
                                      - kappa lap e_i)
                                with Cm = (Ca+Cb)/2, B = A/(Cb-Cm)^2, g = 2/(Cb-Ca)^2,
                                Da = Db = g/delta^2 (ostwald.cpp:67-80); L = mobility;
                                D, Ca, Cb, A, delta, eps in aux[0..5]                         */
#define MMSP_GPU_CH_CONVEX 7 /* semi-implicit convex-splitting Cahn-Hilliard as shipped
                                (examples/phase_transitions/cahn-hilliard/convex_splitting/
                                cahn-hilliard.cpp:273-463, parametric free energy), FP64, fields = 2
                                (c, mu), even extents: each step solves the linearised system by
                                red-black successive over-relaxation until the relative residual
                                falls below the tolerance (checked after iterations 1-4 and every
                                5th), starting from the state two steps back as the example does.
                                mobility = D, kappa = K; aux = {C0, Ca, Cb, A, omega, tolerance};
                                at most 10000 iterations per step (MMSP_GPU_ENOCONV beyond)    */
#define MMSP_GPU_SPARSE_GG 8 /* isotropic sparse phase-field grain growth as shipped
                                (examples/coarsening/grain_growth/isotropic/sparsePF/graingrowth.cpp:58-120)
                                on grid<dim,sparse<double> > (include/MMSP.sparse.h:19), FP64: each
                                cell a list of (grain index, value) items in insertion order, at most
                                `fields` items (1..32, MMSP_GPU_EOVERFLOW beyond); over the union S
                                of the indices of the cell and its face neighbours, for |S| >= 2:
                                e_i' = e_i - dt*(-e_i - e_i^3 + 2 (e_i sum e^2 - lap e_i)), stored
                                when above epsilon = aux[0]; |S| < 2 copies the list.  As in the
                                example, the grid written each step starts as the state of two steps
                                back (empty at the start of each mmsp_gpu_step call, as each update()
                                call's newGrid is), so items below epsilon keep their old values.
                                State crosses with mmsp_gpu_sparse_upload / _download only. */

/* Host/device layouts of vector-valued grids (fields > 1). */
#define MMSP_GPU_CELL_MAJOR  0  /* value j of cell i at i*fields + j (grid<dim,vector<T>> order) */
#define MMSP_GPU_FIELD_MAJOR 1  /* value j of cell i at j*cells + i (the device layout)          */

typedef struct mmsp_gpu_desc {
    int dim;          /* 1, 2 or 3 */
    int n[3];         /* extents per axis (x1-x0), axis 0 slowest; unused axes ignored */
    int fields;       /* values per cell: 1 for grid<dim,T>, N for grid<dim,vector<T>> */
    int dtype;        /* MMSP_GPU_F64 or MMSP_GPU_F32 */
    int model;        /* MMSP_GPU_CH ... MMSP_GPU_SPARSE_GG */
    int bc[3][2];     /* lower/upper boundary per axis; the device path takes periodic only */
    int flags;        /* MMSP_GPU_FLAG_* (0: none); mmsp_gpu_desc_init clears it.  Added in ABI
                         version 3 in what was padding, so the layout of the other members is
                         that of version 2 */
    double dx[3];     /* cell spacing per axis */
    double dt;        /* time step */
    double kappa;     /* gradient coefficient (K of the shipped examples) */
    double mobility;  /* M (Cahn-Hilliard) or L (Allen-Cahn) */
    double gamma;     /* grain-boundary coupling (MMSP_GPU_AC) */
    double r, u;      /* polynomial coefficients (MMSP_GPU_CH_POLY, MMSP_GPU_AC_POLY) */
    double aux[6];    /* further model parameters: MMSP_GPU_OSTWALD takes D, Ca, Cb, A, delta, eps;
                         MMSP_GPU_CH_POLY and MMSP_GPU_AC_POLY take a thermal noise standard
                         deviation (aux[0], 0: none) and stream seed (aux[1], an integer <= 2^53):
                         the stochastic forms of model_A.cpp:99-100 (AC_POLY), model_B.cpp:100-106
                         and spinodal.cpp:95-102 (CH_POLY) add gaussian(0, aux[0]) to mu.  The examples
                         draw it from rand() in cell order; here deviate step*cells + cell of a
                         SplitMix64 / Box-Muller stream, step counting from the last upload.
                         Noisy grids are stepped without graph replay and are refused by batches
                         and mmsp_gpu_step_noalloc (EUNSUPPORTED). */
} mmsp_gpu_desc;

typedef struct mmsp_gpu_stats {
    double mass;      /* dV * sum of all values (all fields) */
    double energy;    /* dV * sum of the model's free-energy density + kappa/2 |grad|^2 */
    double gpu_ms;    /* device time of the last mmsp_gpu_step call, CUDA events on the handle's stream */
    int64_t steps;    /* steps advanced since the last upload */
    int64_t solver_iterations;  /* MMSP_GPU_CH_CONVEX: red-black iterations of the last step's solve */
} mmsp_gpu_stats;

typedef struct mmsp_gpu_handle mmsp_gpu_handle;

/* Library ABI version (MMSP_GPU_ABI_VERSION). */
int mmsp_gpu_version(void);

/* Text for a status code. */
const char* mmsp_gpu_strerror(int code);

/* Fill *desc with the defaults of a periodic grid of the given model: dx=1,
 * dt/kappa/mobility/gamma of the shipped example for that model. */
int mmsp_gpu_desc_init(mmsp_gpu_desc* desc, int dim, const int* n, int fields,
                       int dtype, int model);

/* Validate a descriptor without touching the device (0, EINVAL or EUNSUPPORTED). */
int mmsp_gpu_validate(const mmsp_gpu_desc* desc);

/* Device bytes a handle for this descriptor allocates. */
int mmsp_gpu_footprint(const mmsp_gpu_desc* desc, size_t* bytes);

/* Create a handle: validates the descriptor, allocates two state buffers
 * (the grid and its newGrid) and the reduction scratch on the current device,
 * and a private non-blocking stream. */
int mmsp_gpu_create(mmsp_gpu_handle** out, const mmsp_gpu_desc* desc);

/* Free the handle's device memory and stream. NULL is accepted. */
int mmsp_gpu_destroy(mmsp_gpu_handle* h);

/* Order the handle's work on an external cudaStream_t (NULL: back to the
 * private stream).  Stream-ordered with previously queued work on the old stream. */
int mmsp_gpu_set_stream(mmsp_gpu_handle* h, void* cuda_stream);

/* Copy a host grid in (pageable or pinned memory); bytes must equal
 * cells*fields*sizeof(T).  Resets the step counter.  Synchronous. */
int mmsp_gpu_upload(mmsp_gpu_handle* h, const void* host, size_t bytes, int layout);

/* Copy the current state out to host memory.  Synchronous. */
int mmsp_gpu_download(mmsp_gpu_handle* h, void* host, size_t bytes, int layout);

/* Same as upload/download with a device pointer, stream-ordered (asynchronous). */
int mmsp_gpu_upload_device(mmsp_gpu_handle* h, const void* dev, size_t bytes, int layout);
int mmsp_gpu_download_device(mmsp_gpu_handle* h, void* dev, size_t bytes, int layout);

/* Advance the state by `steps` explicit-Euler steps (asynchronous; CUDA
 * graphs replay long runs).  steps == 0 is a no-op.  2D FP32 Cahn-Hilliard
 * grids (noise-free) take whole blocks of 4 steps per launch of a
 * temporally blocked kernel and the call's last steps % 4 steps one launch
 * each; the two round differently in FP32, so runs split into calls of
 * multiples of 4 steps equal one call, bit for bit. */
int mmsp_gpu_step(mmsp_gpu_handle* h, int steps);

/* Wait for the handle's queued work. */
int mmsp_gpu_synchronize(mmsp_gpu_handle* h);

/* Mass and free energy of the current state (FP64, compensated), plus the
 * device time of the last step call and the step counter.  Synchronous. */
int mmsp_gpu_reduce(mmsp_gpu_handle* h, mmsp_gpu_stats* stats);

/* Device pointer of the current state (field-major), valid until the next step. */
int mmsp_gpu_state(mmsp_gpu_handle* h, void** dev_ptr);

/* Message of the last failure on this handle ("" if none). */
const char* mmsp_gpu_last_error(const mmsp_gpu_handle* h);

/* FP64 operations per second of the current device: a probe of independent
 * fused multiply-add chains on every SM (about 20 ms, on `cuda_stream`,
 * NULL: the legacy default stream).  Each add, multiply or fused
 * multiply-add counts one operation.  The FP64 forms of the step are bound
 * by this rate on GB300, not by memory; it is their roofline.  No
 * counterpart in the reference (it runs on the CPU). */
int mmsp_gpu_fp64_rate(void* cuda_stream, double* ops_per_second);

/* Sparse grids (MMSP_GPU_SPARSE_GG).  Replaces the storage of
 * grid<dim,sparse<T> > (include/MMSP.sparse.h:19-60: per cell a list of
 * item{int index; T value} in insertion order, to_buffer/from_buffer
 * include/MMSP.sparse.cpp:140-163).  Host arrays, K = desc.fields slots per
 * cell in node order: count[cells] items per cell (0..K), index[cells*K] and
 * value[cells*K] (double) with the first count[c] slots of cell c in the
 * list's order; the other slots are ignored on upload and zero on download.
 * Upload checks the counts (MMSP_GPU_EINVAL), resets the step counter and is
 * synchronous; download is synchronous and reports MMSP_GPU_EOVERFLOW if a
 * list outgrew its slots.  The dense transfers, reductions, grid-file output,
 * batches, the server and mmsp_gpu_step_noalloc refuse sparse grids
 * (MMSP_GPU_EUNSUPPORTED). */
int mmsp_gpu_sparse_upload(mmsp_gpu_handle* h, const int32_t* count, const int32_t* index, const void* value);
int mmsp_gpu_sparse_download(mmsp_gpu_handle* h, int32_t* count, int32_t* index, void* value);

/* One call per update(grid&, steps): create, upload `host`, advance `steps`,
 * download into `host`, destroy.  `stats` may be NULL. */
int mmsp_gpu_update(const mmsp_gpu_desc* desc, void* host, size_t bytes, int layout,
                    int steps, mmsp_gpu_stats* stats);

/* ---------------------------------------------------------------------------
 * Output path: MMSP grid files.
 *
 * Replaces grid::output (include/MMSP.grid.cpp:1358-1402), write_buffer
 * (include/MMSP.grid.cpp:1818-1909) and to_buffer (:1146-1157) of a serial
 * run: the same ASCII header, one block, zlib payload, so the reference's
 * grid::input (and mmsp2png / mmsp2tsv) read the files.  Payloads up to
 * 1 MiB are compressed by one compress2 call as the reference does and are
 * byte-identical to its files; larger payloads are deflated in 1 MiB pieces
 * on several host threads and joined into one zlib stream (same data, other
 * compressed bytes; independent of the thread count). */
typedef struct mmsp_gpu_output_opts {
    int level;        /* zlib level 1..9 (the reference writes 9); 0: uncompressed,
                         as the reference's RAW build writes */
    int threads;      /* host threads compressing one file; <= 0: every hardware thread */
    int vector;       /* 1: grid<dim,vector<T>> cells (int32 N, then N values);
                         0: scalar cells; < 0: vector when fields > 1 */
    int fields_line;  /* the header's "fields" value; < 0: N for vector grids, 0 for
                         scalar ones (the examples' generate() builds those with 0) */
    int g0[3];        /* global lower corner per axis; the upper corner is g0 + n */
} mmsp_gpu_output_opts;

/* Defaults: level 9, all threads, vector when fields > 1, g0 = 0. */
int mmsp_gpu_output_opts_init(mmsp_gpu_output_opts* opts);

/* Write host values (layout as for mmsp_gpu_upload) as a grid file of
 * `desc`'s shape, spacing and boundary codes.  Needs no device.  `opts`
 * may be NULL.  Synchronous. */
int mmsp_gpu_write_grid(const char* filename, const mmsp_gpu_desc* desc, const void* host, size_t bytes,
                        int layout, const mmsp_gpu_output_opts* opts);

/* Snapshot the handle's state, as ordered after the work queued so far,
 * into `filename`.  The device packs the cells in to_buffer order (vector
 * grids get their per-cell length) into a staging buffer on the handle's
 * stream; the copy to pinned host memory runs on a second stream and the
 * compression and file write on a host thread, so later steps overlap
 * them.  Returns once the snapshot is queued; it blocks only while two
 * earlier snapshots are still being written.  Allocates the staging buffer
 * and two pinned host buffers on first use (held until mmsp_gpu_destroy). */
int mmsp_gpu_output(mmsp_gpu_handle* h, const char* filename, const mmsp_gpu_output_opts* opts);

/* Wait until every queued snapshot is on disk; returns the first failure
 * among them (message in mmsp_gpu_last_error). */
int mmsp_gpu_output_wait(mmsp_gpu_handle* h);

/* ---------------------------------------------------------------------------
 * Batched form: many independent grids of uneven sizes and parameters
 * advanced together.  The reference has no batched path (one update() per
 * grid, cahn-hilliard.cpp:47-81); this replaces a loop of those calls.
 *
 * MMSP_GPU_OSTWALD, MMSP_GPU_CH_CONVEX and noisy grids are not batched
 * (EUNSUPPORTED); handles and the server take them.
 * 2D Cahn-Hilliard grids (MMSP_GPU_CH / MMSP_GPU_CH_POLY, fields=1) whose
 * rows hold a multiple of 32 cells up to 512 share one persistent kernel per
 * step: a work list of (grid, run of rows) items is drained by all warps of
 * the GPU.  Other grids in the batch are advanced by their own kernels in
 * the same step.  All grids share one dtype.  Step chunks replay a CUDA
 * graph.  FP32 batches whose grids all join the persistent kernel can also
 * advance by temporal blocking: each launch loads tiles of every grid with a
 * halo of 2 cells per step into shared memory, takes 2, 4 or 8 steps there
 * and writes the tiles back, cutting HBM traffic per step by about that
 * factor for some redundant halo work.  The run of rows per work item and
 * the block size of the per-step kernel, and the tile region and steps per
 * launch of the blocked one (or none), are chosen by an autotuner on the
 * first step (or mmsp_gpu_batch_tune) and cached per batch shape, in memory
 * and, when the environment variable MMSP_GPU_TUNE_CACHE names a file, in
 * that JSON file.  The environment variable MMSP_GPU_BATCH_TILE="depth,shape"
 * replaces the tuning: depth 2, 4 or 8 steps per blocked launch on region
 * shape 0 (64 x 128 cells, 4 warps), 1 (96 x 128, 4 warps), 2 (128 x 128,
 * 8 warps) or 3 (128 x 128, 4 warps), or "0,0" for the per-step kernel.
 * Results do not depend on the choice beyond FP32 rounding (the blocked
 * kernel contracts the update into one multiply-add). */
typedef struct mmsp_gpu_batch mmsp_gpu_batch;

typedef struct mmsp_gpu_batch_info {
    int instances;          /* grids in the batch */
    int persistent;         /* grids advanced by the persistent kernel */
    int fallback;           /* grids advanced by their own kernels */
    int rows_per_item;      /* autotuned rows per work item (0 before tuning) */
    int threads_per_block;  /* autotuned block size of the persistent kernel */
    int blocks;             /* persistent grid size */
    int items;              /* work items per step */
    int tuned_from_cache;   /* 1 when the tuning came from the cache */
    double tune_ms;         /* wall time spent autotuning */
    size_t device_bytes;    /* device memory the batch holds */
    int temporal_depth;     /* steps per launch of the persistent kernel: 1, or the autotuned depth of
                               the temporally blocked kernel (shared-memory tiles, FP32) */
    int tile_rows, tile_cols;   /* its tile region (halo included), 0 when not used */
    int tiles;              /* its work items per launch */
} mmsp_gpu_batch_info;

int mmsp_gpu_batch_create(mmsp_gpu_batch** out, int count, const mmsp_gpu_desc* descs);
int mmsp_gpu_batch_destroy(mmsp_gpu_batch* b);
int mmsp_gpu_batch_set_stream(mmsp_gpu_batch* b, void* cuda_stream);
/* Copy grid `index` in/out (synchronous), as mmsp_gpu_upload/download. */
int mmsp_gpu_batch_upload(mmsp_gpu_batch* b, int index, const void* host, size_t bytes, int layout);
int mmsp_gpu_batch_download(mmsp_gpu_batch* b, int index, void* host, size_t bytes, int layout);
/* Every grid in one call: host[i] is grid i's buffer of its state size (as
 * mmsp_gpu_batch_upload/download); the copies are queued back to back and
 * the call synchronises once.  Synchronous. */
int mmsp_gpu_batch_upload_all(mmsp_gpu_batch* b, const void* const* host, int layout);
int mmsp_gpu_batch_download_all(mmsp_gpu_batch* b, void* const* host, int layout);
/* Advance every grid by `steps` steps (asynchronous). */
int mmsp_gpu_batch_step(mmsp_gpu_batch* b, int steps);
int mmsp_gpu_batch_synchronize(mmsp_gpu_batch* b);
/* Mass and free energy of grid `index` (synchronous). */
int mmsp_gpu_batch_reduce(mmsp_gpu_batch* b, int index, mmsp_gpu_stats* stats);
/* Run the autotuner now; force != 0 ignores the cache. */
int mmsp_gpu_batch_tune(mmsp_gpu_batch* b, int force);
int mmsp_gpu_batch_get_info(const mmsp_gpu_batch* b, mmsp_gpu_batch_info* info);
const char* mmsp_gpu_batch_last_error(const mmsp_gpu_batch* b);

/* ---------------------------------------------------------------------------
 * Serving form: a request loop for mixed solves.  The reference has no
 * counterpart (its driver runs one grid per process, MMSP.main.hpp:273-350).
 *
 * Clients submit (descriptor, initial state, steps) from any thread.  A
 * scheduler thread admits queued requests in arrival order while their
 * device footprint (mmsp_gpu_footprint) fits the HBM budget, carving their
 * buffers from one device block taken at start, and keeps two chunks of at
 * most chunk_steps steps (rounded down to a multiple of 4) queued on every
 * admitted request's stream, so requests overlap on the GPU and finish
 * independently; small grids run on high-priority streams.  Finished
 * requests are reduced (mass, energy), copied to the host and their block
 * returned at once.  Each request runs the same kernels with the same step
 * sequence as a lone mmsp_gpu_update, so its result does not depend on what
 * else is running.  A serving process should set CUDA_DEVICE_MAX_CONNECTIONS
 * to 32 before it creates its CUDA context (the requests' streams then do
 * not share the default 8 hardware work queues). */
typedef struct mmsp_gpu_server mmsp_gpu_server;

typedef struct mmsp_gpu_server_config {
    size_t hbm_budget_bytes;   /* device bytes for request state (0: 80% of free memory) */
    int chunk_steps;           /* steps per queued chunk, a multiple of 4 (0: 200) */
    int max_active;            /* requests resident at once (0: no limit but the budget) */
} mmsp_gpu_server_config;

/* Request states. */
#define MMSP_GPU_REQ_QUEUED  0
#define MMSP_GPU_REQ_RUNNING 1
#define MMSP_GPU_REQ_DONE    2   /* negative values: the request failed with that status */

typedef struct mmsp_gpu_request_status {
    int state;                 /* MMSP_GPU_REQ_* or a negative MMSP_GPU_E* code */
    int steps_total;
    int64_t steps_done;
    double submit_s, admit_s, finish_s;   /* seconds since the server started */
    double mass, energy;       /* of the result (state DONE) */
    char message[160];         /* what failed, for a negative state */
} mmsp_gpu_request_status;

typedef struct mmsp_gpu_server_stats {
    int64_t submitted, admitted, completed, failed, cancelled;
    int queued, active;
    size_t device_bytes_in_use, device_bytes_budget;
    int64_t rounds;
} mmsp_gpu_server_stats;

int mmsp_gpu_server_start(mmsp_gpu_server** out, const mmsp_gpu_server_config* cfg);
/* Queue a request; `host` is copied before the call returns.  A request whose
 * footprint exceeds the whole budget is refused with MMSP_GPU_ENOMEM. */
int mmsp_gpu_server_submit(mmsp_gpu_server* s, const mmsp_gpu_desc* desc, const void* host, size_t bytes,
                           int layout, int steps, uint64_t* request_id);
/* Status without blocking; MMSP_GPU_ENOTFOUND for an unknown or fetched id. */
int mmsp_gpu_server_poll(mmsp_gpu_server* s, uint64_t request_id, mmsp_gpu_request_status* status);
/* Block until the request is done or failed, or `timeout_s` passes
 * (MMSP_GPU_ETIMEDOUT; the request keeps running). */
int mmsp_gpu_server_wait(mmsp_gpu_server* s, uint64_t request_id, double timeout_s,
                         mmsp_gpu_request_status* status);
/* Copy a finished request's state to `host` and forget the request. */
int mmsp_gpu_server_fetch(mmsp_gpu_server* s, uint64_t request_id, void* host, size_t bytes, int layout);
/* Cancel a queued or running request (it ends with MMSP_GPU_ECANCELED). */
int mmsp_gpu_server_cancel(mmsp_gpu_server* s, uint64_t request_id);
int mmsp_gpu_server_get_stats(mmsp_gpu_server* s, mmsp_gpu_server_stats* stats);
/* Stop the scheduler; requests not finished end with MMSP_GPU_ESTOPPED.
 * Frees all device memory and the server. */
int mmsp_gpu_server_stop(mmsp_gpu_server* s);

/* Largest state (bytes) mmsp_gpu_step_noalloc can advance by more than one
 * step or in place: the size of the library's fixed device scratch array. */
#define MMSP_GPU_NOALLOC_MAX_BYTES (16u << 20)

/* Advance a device-resident grid without allocating any memory.
 *
 * No counterpart in the reference: MMSP's update() allocates its scratch
 * grids on every call (cahn-hilliard.cpp:56-57).  This entry point is for
 * callers that must not call cudaMalloc: code whose device memory belongs to
 * another allocator or a fixed budget (a framework's memory pool, a serving
 * loop that has committed its HBM), and hot loops that cannot afford
 * cudaMalloc/cudaFree, which may synchronise the whole device.
 *
 * `in` and `out` are device pointers to field-major state of
 * desc->fields * cells values of the descriptor's type (there is no layout
 * argument: vector grids must already be field-major), both 16-byte
 * aligned; `out` may equal `in` but must not otherwise overlap it.  A
 * misaligned or partly overlapping pointer returns MMSP_GPU_EINVAL before
 * any device work is queued.  The intermediate steps live in one file-scope device array of
 * MMSP_GPU_NOALLOC_MAX_BYTES shared by every call in the process; a state
 * larger than that returns MMSP_GPU_ENOMEM when steps > 1 or out == in
 * (one step from in to a distinct out needs no scratch).  Work is queued on
 * `cuda_stream` (NULL: the legacy default stream) and the call returns once
 * it has finished, with MMSP_GPU_ETIMEDOUT if a kernel's bounded wait ran
 * out.  The first call on a device looks up the array's device address
 * with that device current; make that first call before any stream capture.
 * The address is kept for the life of the process: after cudaDeviceReset on
 * a device, do not call this entry point on that device again.
 * Calls that overlap on the GPU (from several threads or streams) share the
 * scratch array and race: serialise them.  MMSP_GPU_OSTWALD (its step needs a
 * work grid beside the state, except on the FP32 3D grids of its one-kernel
 * step), MMSP_GPU_CH_CONVEX (an iterative solve per
 * step) and the noisy polynomial forms return MMSP_GPU_EUNSUPPORTED. */
int mmsp_gpu_step_noalloc(const mmsp_gpu_desc* desc, const void* in, void* out, int steps,
                          void* cuda_stream);

#ifdef __cplusplus
}
#endif
#endif /* MMSP_GPU_H */
