/*
 * cufoam_gb300.h -- C ABI of the GB300 sparse-solve library.
 *
 * This is the drop-in boundary for the reference's solver library
 * (libGIS.so, gis/gis.h:1-95) and for the host work its OpenFOAM plugins do
 * before calling it (gis/ldu2csr.h:7-40, cuFoam<X>/cuFoam<X>.C).  Every
 * function is extern "C", takes plain pointers and sizes, never exits the
 * process and never throws: failures come back as a cf_status plus a
 * message from cf_context_last_error().
 *
 * Pointers tagged with a `memory` argument/field are host pointers when it
 * is CF_MEM_HOST and device pointers (on the context's device) when it is
 * CF_MEM_DEVICE.  All device memory the library needs is owned by the
 * context or the matrix; nothing is allocated per solver iteration.
 *
 * Thread safety: one context may be used by one host thread at a time.
 * Work is ordered on the context's CUDA stream (cf_context_set_stream).
 */
#ifndef CUFOAM_GB300_H
#define CUFOAM_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CF_ABI_VERSION 1

typedef enum cf_status {
    CF_OK = 0,
    CF_NOT_CONVERGED = 1, /* max_iter reached with the residual above tolerance */
    CF_BREAKDOWN = 2,     /* BiCG: |xi| < int_bound (SolverSingleGPU.h:629-630) */
    CF_NONFINITE = 3,     /* a NaN/Inf residual or scalar stopped the loop */
    CF_BAD_INPUT = 4,     /* invalid sizes, addressing or arguments */
    CF_CUDA_ERROR = 5,    /* a CUDA runtime call failed (message has details) */
    CF_TIMEOUT = 6,       /* the device loop guard or the time limit stopped the solve */
    CF_NO_DEVICE = 7,     /* no usable CUDA device */
    CF_UNSUPPORTED = 8,   /* option combination not implemented */
    CF_OUT_OF_MEMORY = 9
} cf_status;

/* Solver selection: the eight cuFoam plugins (fvSolution `solver cuFoamX;`),
 * plus a Jacobi-preconditioned CG (CF_PCG) the reference announces in its
 * roadmap (README.md:71-73) but does not have. */
typedef enum cf_solver {
    CF_CG = 0,         /* cuFoamCG         -> gis.h:11-17  CG */
    CF_BICG = 1,       /* cuFoamBiCG       -> gis.h:28-36  BiCG(A, At) */
    CF_JACOBI = 2,     /* cuFoamJacobi     -> gis.h:56-62  Jacobi */
    CF_MR = 3,         /* cuFoamMR         -> gis.h:48-54  MR */
    CF_MRJACOBI = 4,   /* cuFoamMRJacobi   -> gis.h:64-70  MRJacobi */
    CF_MRS = 5,        /* cuFoamMRS        -> gis.h:80-87  MRS with invM = D^-1 */
    CF_JMR = 6,        /* cuFoamJMR        -> gis.h:72-78  JMR */
    CF_RICHARDSON = 7, /* cuFoamRichardson -> gis.h:38-46  Richardson */
    CF_PCG = 8         /* cuFoamPCG: CG preconditioned by D^-1 (no reference
                          counterpart; fast reduction order, FP64 only) */
} cf_solver;

enum { CF_MEM_HOST = 0, CF_MEM_DEVICE = 1 };

/* Arithmetic of the solve. */
enum {
    CF_PREC_FP64 = 0,  /* FP64 values, vectors and reductions (the reference's) */
    CF_PREC_MIXED = 1  /* FP32 matrix/vectors/accumulation inside an FP64
                          iterative-refinement loop (CG, BiCG, MR, MRJacobi,
                          MRS and JMR) */
};

/* Summation order of FP64 solves (row sums and dot products). */
enum {
    CF_REDUCE_FAST = 0,      /* each row one FMA chain, dot products in a
                                deterministic tree over an occupancy-sized grid */
    CF_REDUCE_REFERENCE = 1, /* the reference's order on this GPU: rows in
                                its 8-lane tree, grid = maxThreadsPerSM/256 *
                                SMs blocks of 256, sequential sum of block
                                partials; gives the reference algorithm's
                                exact bits */
    CF_REDUCE_AUTO = 2       /* the default (cf_controls_init): REFERENCE for
                                BiCG, FAST for the other solvers.  BiCG's
                                iterates follow the summation order
                                chaotically on non-symmetric systems (on a
                                48^3 convection-diffusion system at cell
                                Peclet 3 two correct summation orders take
                                350 and 377 steps; at 256^3 the fast order
                                broke down where the reference order
                                converges), so its default is the
                                reference's bits */
};

/* normFactor flavour reported in cf_perf and used for the tolerance. */
enum {
    CF_NORM_REFERENCE_L2 = 0, /* gis/gis.cu:106-123 (the reference's) */
    CF_NORM_OPENFOAM_L1 = 1   /* OpenFOAM's lduMatrix::normFactor (sum of |.|) */
};

typedef struct cf_context cf_context;
typedef struct cf_matrix cf_matrix;

/* An OpenFOAM lduMatrix: n_cells diagonal entries, n_faces lower/upper
 * coefficients, owner (lowerAddr) / neighbour (upperAddr) per face, faces
 * sorted by owner with owner < neighbour.  losort, losort_start and
 * owner_start are lduAddressing's losortAddr/losortStartAddr/ownerStartAddr;
 * pass NULL for all three to have them computed on the device. */
typedef struct cf_ldu_view {
    int32_t n_cells;
    int32_t n_faces;
    const double *diag;
    const double *lower;
    const double *upper;
    const int32_t *lower_addr;
    const int32_t *upper_addr;
    const int32_t *losort;
    const int32_t *losort_start;
    const int32_t *owner_start;
    int32_t memory;
} cf_ldu_view;

typedef struct cf_controls {
    double tolerance;        /* tolerance_ (absolute, in normFactor units) */
    double rel_tol;          /* relTol_; 0 = ignore (the reference ignores it) */
    int32_t max_iter;        /* maxIter_; <= 0 means unlimited, as the reference */
    int32_t min_iter;        /* minIter_; 0 = none (the reference ignores it) */
    int32_t precision;       /* CF_PREC_* */
    int32_t reduction;       /* CF_REDUCE_* (FP64 only; default AUTO) */
    int32_t memory;          /* where source and psi live: CF_MEM_* */
    int32_t norm_type;       /* CF_NORM_* */
    double bicg_int_bound;   /* BiCG breakdown bound, default 1e-10 */
    double richardson_omega; /* 0 = estimate by the power method (default) */
    int32_t power_max_steps; /* power-method steps for Richardson, default 30 */
    int32_t mixed_max_outer; /* mixed: refinement sweeps limit, default 50 */
    double mixed_inner_rtol; /* mixed: inner FP32 relative tolerance; 0 (the
                                default) = 1e-6 for CG (batched too), 1e-4 for
                                BiCG and the MR family, the fastest measured */
    double *history;         /* optional HOST buffer: absolute ||r||_2 per step */
    int32_t history_capacity;
    int32_t use_graph;       /* 1 (default): device-driven loop in a CUDA graph */
    double time_limit_s;     /* > 0: stop with CF_TIMEOUT after this wall time */
    int32_t profile_kernels; /* 1: host-driven loop with CUDA events around every
                                body kernel; fills cf_perf.kernel_ms */
    int32_t transpose;       /* 1: solve A^T psi = source (the adjoint system) */
    int32_t absolute_tolerance; /* 1: tolerance is an absolute ||r||_2 threshold
                                   (libGIS's `error` argument), no normFactor scaling */
    int32_t history_time;    /* 1: history holds seconds since the initial residual
                                at the end of each step (device clock), the
                                reference's DetailType::Time, instead of ||r||_2 */
    int32_t mixed_inner_max; /* mixed: FP32 steps per refinement sweep; 0 = no
                                limit (to the inner tolerance).  A sweep that
                                raises the FP64 residual is undone and retried
                                with half as many steps as it took (the solve
                                stops as not converged below 8); an inner
                                breakdown before the first step ends it with
                                CF_BREAKDOWN.  Mixed BiCG's FP32 inner solver
                                is BiCGStab. */
    int32_t reserved[3];
} cf_controls;

/* solverPerformance plus diagnostics. */
typedef struct cf_perf {
    double initial_residual;     /* ||r_0|| / normFactor  (OpenFOAM convention) */
    double final_residual;       /* ||r_end|| / normFactor */
    double initial_residual_abs; /* ||r_0||_2, what libGIS records */
    double final_residual_abs;
    double norm_factor;
    double true_residual;        /* FP64 ||b - A x|| / normFactor at exit */
    double omega;                /* Richardson: relaxation factor used */
    double solve_ms;             /* device time of the solve (CUDA events) */
    int32_t n_iterations;        /* solver steps (inner steps for mixed) */
    int32_t n_outer;             /* mixed: refinement sweeps */
    int32_t status;              /* cf_status of the solve */
    int32_t history_length;      /* entries written to controls->history */
    /* with profile_kernels: summed device time and launch count of
       [0] the SpMV body kernel, [1] the update body kernel,
       [2] the element-wise prep body kernel, [3] set-up (normFactor,
       power method, initial residual) */
    double kernel_ms[4];
    int32_t kernel_launches[4];
    int32_t reserved[6];
} cf_perf;

typedef struct cf_device_info {
    int32_t device;
    int32_t sm_count;
    int32_t cc_major, cc_minor;
    int32_t max_threads_per_sm;
    int32_t reference_grid;      /* the reference's LaunchConfig grid here */
    int64_t l2_bytes;
    int64_t global_mem_bytes;
    char name[128];
} cf_device_info;

/* ---- library / context ------------------------------------------------- */
int32_t cf_abi_version(void);
const char *cf_status_string(int32_t status);
/* Name of a plugin ("cuFoamCG", "CG", ...) -> cf_solver.  Mirrors the
 * run-time selection by name in fvSolution (cuFoamCG/cuFoamCG.C:11-15). */
cf_status cf_solver_from_name(const char *name, int32_t *solver);
void cf_controls_init(cf_controls *c);

cf_status cf_context_create(int32_t device, cf_context **out);
/* Also releases the device memory of the matrices and batches made on the
 * context.  Their handles stay valid for cf_matrix_destroy /
 * cf_batch_destroy only (any order; every other call on them returns
 * CF_BAD_INPUT), so a garbage collector may free handles after their
 * context. */
void cf_context_destroy(cf_context *ctx);
/* Orders the context's work on `cuda_stream` (a cudaStream_t the caller
 * keeps alive; cudaStreamLegacy and cudaStreamPerThread are accepted), or on
 * a private non-blocking stream of the library when it is NULL. */
cf_status cf_context_set_stream(cf_context *ctx, void *cuda_stream);
const char *cf_context_last_error(const cf_context *ctx);
cf_status cf_device_query(cf_context *ctx, cf_device_info *out);

/* ---- matrices ---------------------------------------------------------- */
/* A matrix given as a square CSR matrix (host or device arrays; copied).
 * The diagonal is found as the reference's FindDiag does
 * (gis/SparseSystem/kernels.h:447-464).  The transpose solve and BiCG need
 * a structurally symmetric pattern.  Replaces the SingleGPU::SparseCSR
 * upload of a CPU::SparseCSR (gis/SparseSystem/SparseSingleGPU.h:51-80). */
cf_status cf_matrix_create_csr(cf_context *ctx, int32_t n, int64_t nnz, const int32_t *row_offsets,
                               const int32_t *cols, const double *vals, int32_t memory, cf_matrix **out);
/* Uploads an LDU matrix and converts it on the device to the reference's
 * CSR (replaces getSparseCSRMat, gis/ldu2csr.h:7-40, plus the
 * SingleGPU::SparseCSR upload, gis/SparseSystem/SparseSingleGPU.h:51-80). */
cf_status cf_matrix_create_ldu(cf_context *ctx, const cf_ldu_view *ldu, cf_matrix **out);
/* New coefficients, same addressing (time-step / Ux,Uy,Uz reuse). */
cf_status cf_matrix_update_values(cf_matrix *m, const double *diag, const double *lower,
                                  const double *upper, int32_t memory);
/* New values, same pattern, for a matrix made by cf_matrix_create_csr
 * (vals[nnz] in its entry order; host or device memory).  No reference
 * counterpart: the reference converts and uploads its CSR on every solve
 * (cuFoamCG/cuFoamCG.C:48-62); the plugin uses this for the coupled
 * matrices of meshes with cyclic patches. */
cf_status cf_matrix_update_csr_values(cf_matrix *m, const double *vals, int32_t memory);
void cf_matrix_destroy(cf_matrix *m);
/* Storage the fast (CF_REDUCE_FAST) kernels read the matrix from.  AUTO
 * (the default) picks SELL-32 -- slices of 32 rows padded to their longest
 * row, entry-major, read with coalesced loads and no staging -- when the
 * padding adds at most 20% to nnz and rows average at most 32 entries, and
 * the CSR arrays with warp-chunk staging otherwise.  SELL-32 stores each
 * slot's column as a one-byte code (CF_FORMAT_SELL_C8) when the pattern has
 * at most 32 distinct column offsets col - row (a structured mesh has one
 * per stencil point), else as a 32-bit index (CF_FORMAT_SELL); a code costs
 * 1 byte instead of 4, i.e. 9 instead of 12 bytes per FP64 entry and 5
 * instead of 8 per FP32 entry.  With AUTO the codes are read by the
 * product (cf_spmv) and the FP32 sweeps of mixed-precision solves; the FP64
 * solver loops keep the 32-bit columns (GB300's FP64 issue rate, not HBM,
 * bounds them).  SELL and SELL_C8 may be asked for: SELL_C8 makes every
 * fast pass read the codes, and fails with CF_UNSUPPORTED on a pattern with
 * more offsets.  A pattern with more offsets, all in [-32768, 32767] (an
 * unstructured mesh in a bandwidth-reducing order), gets 16-bit column
 * deltas instead (CF_FORMAT_SELL_D16: column = row + delta; 10 bytes per
 * FP64 entry, 6 per FP32 entry), read where the codes would be; asked for
 * on a pattern outside that range it fails with CF_UNSUPPORTED.  Every format
 * sums each row in entry order, so results do not depend on the choice.
 * The reference-order kernels read the 32-bit columns.  No reference
 * counterpart (the reference has CSR only). */
enum { CF_FORMAT_AUTO = 0, CF_FORMAT_CSR = 1, CF_FORMAT_SELL = 2, CF_FORMAT_SELL_C8 = 3, CF_FORMAT_SELL_D16 = 4 };
cf_status cf_matrix_set_format(cf_matrix *m, int32_t format);
/* The format the fast kernels use now (CF_FORMAT_CSR, CF_FORMAT_SELL,
 * CF_FORMAT_SELL_C8 or CF_FORMAT_SELL_D16; decides AUTO first) and the
 * stored entries including padding. */
cf_status cf_matrix_format(cf_matrix *m, int32_t *format, int64_t *stored_entries);
cf_status cf_matrix_shape(const cf_matrix *m, int32_t *n_rows, int32_t *n_faces, int64_t *nnz);
/* CSR arrays of A (transpose = 0) or A^T (transpose = 1; the reference's
 * Transpose, gis/gis.h:10-11).  row_offsets[n+1], cols[nnz], vals[nnz]. */
cf_status cf_matrix_export_csr(cf_matrix *m, int32_t transpose, int32_t *row_offsets,
                               int32_t *cols, double *vals, int32_t memory);

/* One-shot device ldu2csr into caller buffers (gis/ldu2csr.h:7-40). */
cf_status cf_ldu2csr(cf_context *ctx, const cf_ldu_view *ldu, int32_t *row_offsets,
                     int32_t *cols, double *vals, int32_t memory);

/* ---- operations -------------------------------------------------------- */
/* y = A x (transpose = 0) or A^T x (SpMv, SolverSingleGPU.h:173-184).
 * row_order CF_REDUCE_REFERENCE sums each row in the reference's 8-lane
 * order (SpMvKernel, gis/SparseSystem/kernels.h:206-237); CF_REDUCE_FAST
 * sums it as one FMA chain. */
cf_status cf_spmv(cf_matrix *m, int32_t transpose, const double *x, double *y, int32_t memory,
                  int32_t row_order);
/* The same on device pointers, enqueued on the context's stream without
 * waiting for it (for callers that chain their own kernels or time the
 * SpMV with events).  No reference counterpart (SpMv is internal to libGIS). */
cf_status cf_spmv_async(cf_matrix *m, int32_t transpose, const double *x, double *y, int32_t row_order);
/* normFactor(source, psi) (gis/gis.cu:106-123 for CF_NORM_REFERENCE_L2). */
cf_status cf_norm_factor(cf_matrix *m, const double *source, const double *psi,
                         int32_t memory, int32_t norm_type, int32_t reduction, double *out);
/* cuFoam<X>::solve(psi, source): normFactor, then the solver at
 * tolerance*normFactor, psi updated in place, performance in *perf.
 * (cuFoamCG/cuFoamCG.C:38-90 and its seven siblings.) */
cf_status cf_solve(cf_matrix *m, int32_t solver, const cf_controls *controls,
                   const double *source, double *psi, cf_perf *perf);

/* ---- decomposed cases (processor patches) ------------------------------- */
/* The reference has no counterpart: its solvers take OpenFOAM's interface
 * lists and ignore them (cuFoamCG/cuFoamCG.C:19-35), so a decomposed run
 * solves every subdomain alone.  Here `m` is this rank's subdomain and the
 * processor patches couple it to the others as OpenFOAM's lduMatrix::Amul
 * does (initMatrixInterfaces / updateMatrixInterfaces): after the local
 * product, row face_cells[f] loses coeffs[f] * (the neighbouring rank's
 * value of the cell across face f), coeffs being interfaceBouCoeffs.
 * Faces are listed patch after patch in the order every rank agrees on;
 * the faces of one cell are applied in that order.
 *
 * The caller moves the data; the library never talks to another process.
 *   exchange(user, send, recv, count): send[f] is this rank's value of
 *     face_cells[f]; fill recv[f] with the neighbour's value of the cell on
 *     the other side of face f.  Called once per product, by every rank,
 *     also with count 0 on a rank without processor faces.
 *   allreduce_sum(user, values, count): replace values[0..count) by their
 *     sums over all ranks -- the same bits on every rank (the ranks take
 *     their stopping decisions on them).
 *   allreduce_max(user, values, count): the same with the maximum; only
 *     Richardson without a given relaxation factor needs it (the smallest
 *     |a_ii| of the whole mesh), and may be NULL otherwise.
 * They return 0 on success; anything else ends the solve with
 * CF_BAD_INPUT.  Buffers are host memory and valid during the call only. */
typedef struct cf_comm {
    void *user;
    int32_t (*exchange)(void *user, const double *send, double *recv, int32_t count);
    int32_t (*allreduce_sum)(void *user, double *values, int32_t count);
    int32_t (*allreduce_max)(void *user, double *values, int32_t count);
} cf_comm;

typedef struct cf_interfaces {
    int32_t n_faces;            /* processor-patch faces of this subdomain */
    const int32_t *face_cells;  /* [n_faces] host: local cell of each face */
    const double *coeffs;       /* [n_faces] host: interfaceBouCoeffs */
} cf_interfaces;

/* cuFoam<X>::solve on a decomposed case: normFactor and every inner
 * product summed over all ranks, the product coupled through the
 * interfaces (A^T's, for BiCG, through the neighbours' coefficients of the
 * same faces, exchanged once).  All nine solvers, FP64, the fast summation
 * order, no transpose; history, time_limit_s, norm_type, min/max_iter,
 * rel_tol, bicg_int_bound, richardson_omega and power_max_steps as in
 * cf_solve.  The loop is host-driven: per step one exchange per product
 * (BiCG two) and one or two all-reduces. */
cf_status cf_solve_decomposed(cf_matrix *m, int32_t solver, const cf_controls *controls,
                              const cf_interfaces *interfaces, const cf_comm *comm,
                              const double *source, double *psi, cf_perf *perf);

/* Gradient of a loss L through A x = b with respect to the LDU
 * coefficients, from the forward solution x and the adjoint solution
 * lambda of A^T lambda = dL/dx (solve with controls.transpose = 1):
 * d_diag[i] = -lambda_i x_i, d_upper[f] = -lambda_owner x_neighbour,
 * d_lower[f] = -lambda_neighbour x_owner (dL/dsource is lambda itself).
 * Any output may be NULL.  No counterpart in the reference, which has no
 * differentiable path; it is the backward of the torch.autograd.Function
 * in cufoam_gb300/autograd.py. */
cf_status cf_adjoint_gradients(cf_matrix *m, const double *lambda, const double *x,
                               double *d_diag, double *d_lower, double *d_upper,
                               int32_t memory);

/* ---- allocation-free normFactor ------------------------------------------ */
/* No counterpart in the reference.  normFactor (the reference's L2 form,
 * gis/gis.cu:106-123) of a CSR matrix the caller already holds on the
 * device, for callers that must not allocate device memory: an application
 * whose own memory pool owns the GPU and forbids driver allocations after
 * start-up, or a latency-critical loop where a cudaMalloc/cudaFree (which
 * can synchronise the whole device) is not acceptable.  It allocates nothing.
 *
 * All pointers are device pointers on the current device (cudaSetDevice);
 * the result is written to *norm_factor (device memory) by work enqueued on
 * `cuda_stream`, which must belong to the current device (CF_BAD_INPUT
 * otherwise; NULL is the legacy default stream); the call does not wait
 * for it.  The matrix arrays are read only inside [0, nnz).
 * Scratch: one fixed array of about 33 KB inside the library, which every
 * GPU that loads the library keeps until the process exits.  All calls
 * share it and it keeps the last call's contents (the call restarts its
 * counters itself): calls whose work overlaps on the GPU race -- order them,
 * e.g. on one stream.  The first call on a device looks up the array's
 * device address on that device; make that first call before any stream
 * capture.
 * reduction: CF_REDUCE_FAST, or CF_REDUCE_REFERENCE (the reference's grid of
 * maxThreadsPerSM/256 * SMs blocks) -- rejected with CF_UNSUPPORTED when
 * that grid needs more than the 2048 block partials the scratch holds.
 * CF_BAD_INPUT for n_rows <= 0 or a null pointer. */
cf_status cf_norm_factor_noalloc(int32_t n_rows, const int32_t *row_offsets, const int32_t *cols,
                                 const double *vals, const double *source, const double *psi,
                                 int32_t reduction, double *norm_factor, void *cuda_stream);

/* ---- files (host only; no context) --------------------------------------
 * The reference's formats (gis/SparseSystem/SparseCPU.h): a name ending in
 * ".rb" is a Rutherford-Boeing matrix (real / integer, assembled;
 * unsymmetric, symmetric or skew; :149-297), anything else the binary CSR
 * file of CPU::SparseCSR::load/save (:105-147: int32 rows, cols, nnz; f64
 * values; int32 row offsets without the last; int32 columns).  Vectors: a
 * name ending in ".mtx" is a Matrix Market array (:661-678), anything else
 * the binary file of CPU::Vector::load/save (int32 size, f64 values).
 * _info gives the sizes, _read fills caller arrays of those sizes. */
cf_status cf_csr_file_info(const char *path, int32_t *rows, int32_t *cols, int64_t *nnz);
cf_status cf_csr_file_read(const char *path, int32_t *row_offsets, int32_t *cols, double *vals);
cf_status cf_csr_file_save(const char *path, int32_t rows, int32_t cols, int64_t nnz,
                           const int32_t *row_offsets, const int32_t *cols_idx, const double *vals);
cf_status cf_vector_file_info(const char *path, int32_t *size);
cf_status cf_vector_file_read(const char *path, double *values);
cf_status cf_vector_file_save(const char *path, int32_t size, const double *values);
/* The message of the last failed file call of this thread. */
const char *cf_file_last_error(void);

/* ---- batched solves ---------------------------------------------------- */
/* Many independent LDU systems, each with n_rhs right-hand sides sharing its
 * matrix (OpenFOAM solves Ux, Uy, Uz with one matrix, calling solve() per
 * component), solved by CG in ONE persistent kernel launch inside a CUDA
 * graph.  No counterpart in the reference, whose plugins solve one system
 * and one component per call (cuFoamCG/cuFoamCG.C:38-90). */
typedef struct cf_batch cf_batch;

typedef struct cf_batch_config {
    int32_t cluster_size;   /* CTAs cooperating on one system: 1, 2, 4, 8, 16 (0 = 16 where it
                               fits on the device, else 8) */
    int32_t threads;        /* threads per CTA: 128, 256, 512 (0 = 256) */
    int32_t order;          /* 0 = largest system first, 1 = given order */
    int32_t max_clusters;   /* 0 = one full wave */
    int32_t reserved[4];
} cf_batch_config;

typedef struct cf_batch_result {
    double initial_residual; /* normalised by normFactor */
    double final_residual;
    double norm_factor;
    int32_t n_iterations;
    int32_t status;
} cf_batch_result;

cf_status cf_batch_create(cf_context *ctx, int32_t n_systems, const cf_ldu_view *systems,
                          cf_batch **out);
void cf_batch_destroy(cf_batch *b);
/* total rows and, if row_offsets is not NULL, each system's first row in
 * the batch vectors (length n_systems). */
cf_status cf_batch_shape(const cf_batch *b, int32_t *n_systems, int64_t *total_rows,
                         int64_t *row_offsets);
/* sources / psi: [total_rows][n_rhs] (the n_rhs components of a cell are
 * adjacent), psi updated in place; results[n_systems * n_rhs].  solver must
 * be CF_CG; controls->precision CF_PREC_FP64, or CF_PREC_MIXED for FP32 CG
 * sweeps inside FP64 refinement (controls->mixed_inner_rtol, mixed_max_outer). */
cf_status cf_batch_solve(cf_batch *b, int32_t solver, const cf_controls *controls,
                         const cf_batch_config *config, int32_t n_rhs, const double *sources,
                         double *psi, cf_batch_result *results, double *device_ms);

#ifdef __cplusplus
}
#endif
#endif /* CUFOAM_GB300_H */
