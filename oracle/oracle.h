/*
 * oracle.h -- CPU oracle for the cuFoam sparse solve path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links, loads or
 * calls this code; it is the checker used by tests/, by the smoke test and
 * by the CPU-baseline leg of bench.py.
 *
 * It is a plain-C restatement of the reference's algorithms:
 *   - OpenFOAM lduAddressing (losort / losortStart / ownerStart),
 *   - gis/ldu2csr.h:7-40  getSparseCSRMat,
 *   - gis/gis.cu:106-123  NormFactor,
 *   - gis/SparseSystem/SolverSingleGPU.h  CG, BiCG(A,At), Richardson
 *     (+OptimizePower, FindDiagAbsMin), MR, Jacobi, MRJacobi,
 *     PreconditionedMRJacobi (JMR), MRS,
 * in the floating-point order the reference's kernels use on a GPU whose
 * LaunchConfig grid is G blocks of 256 threads (gis/SparseSystem/launch.h:
 * 116-139): per-thread grid-stride FMA partials, a 256-wide block tree, and
 * a sequential host sum of the G block partials; an 8-lane per-row SpMV tree
 * (gis/SparseSystem/kernels.h:206-237).  All arithmetic that the reference
 * compiles to fused multiply-add is written here with fma() and the file is
 * compiled with -ffp-contract=off, so results are identical on x86 and Arm.
 *
 * Parity status: ldu2csr is pinned against the reference's own
 * gis/ldu2csr.h compiled from its sources (oracle/refstub).  The solver
 * restatement's arithmetic is pinned on the GPU: the same drivers run once
 * on the CPU emulation and once on the reference's own kernels
 * (gis/SparseSystem/kernels.h, compiled from its sources into a cubin by
 * oracle/build.py and launched by oracle/refgpu/ref_gpu.c), and the two
 * must agree bit for bit (tests/test_gpu_refgpu.py).  The host-side
 * sequencing of each driver is restated from SolverSingleGPU.h line by
 * line; the reference ships no tests or golden vectors of its own.
 */
#ifndef CUFOAM_ORACLE_H
#define CUFOAM_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- OpenFOAM lduAddressing and ldu2csr -------------------------------- */
int32_t orc_ldu_addressing(int32_t n, int32_t f, const int32_t *lower_addr,
                           const int32_t *upper_addr, int32_t *losort,
                           int32_t *losort_start, int32_t *owner_start);
void orc_ldu2csr(int32_t n, int32_t f, const double *diag, const double *lower,
                 const double *upper, const int32_t *lower_addr,
                 const int32_t *upper_addr, const int32_t *losort,
                 const int32_t *losort_start, const int32_t *owner_start,
                 int32_t *row_offsets, int32_t *cols, double *vals);

/* ---- reference-order primitives ---------------------------------------- */
typedef struct orc_csr {
    int32_t n;
    int32_t nnz;
    const int32_t *row_offsets;
    const int32_t *cols;
    const double *vals;
} orc_csr;

void orc_set_threads(int32_t n);
int32_t orc_get_threads(void);
double orc_ref_dot(const double *a, const double *b, int32_t n, int32_t grid);
double orc_ref_sum(const double *a, int32_t n, int32_t grid);
double orc_ref_distance(const double *a, const double *b, int32_t n, int32_t grid);
void orc_ref_spmv(const orc_csr *A, const double *x, double *y);
void orc_ref_residual(const orc_csr *A, const double *b, const double *x, double *r);

/* The primitives the drivers below run on.  By default they are the CPU
 * emulation above; a backend replaces them (all or none), e.g. with the
 * reference's own kernels launched on a GPU (oracle/refgpu/ref_gpu.c), so
 * that the same drivers run once through each and their bits compare. */
typedef struct orc_backend {
    /* kind 0: sum a*b (DotKernel), 1: sum a (ReductionKernel), 2: sum
     * (a-b)^2 (DistanceKernel); G blocks, host sum of the partials */
    double (*reduce)(int kind, const double *a, const double *b, int32_t n, int32_t grid);
    void (*spmv)(const orc_csr *A, const double *x, double *y);                     /* SpMvKernel */
    void (*residual)(const orc_csr *A, const double *b, const double *x, double *r); /* ResidualKernel */
    void (*add)(double *res, const double *v1, const double *v2, double alpha, int32_t n); /* AddKernel1 */
    void (*hadamard)(double *res, const double *v1, const double *v2, int32_t n);   /* HadamardKernel */
    void (*scale)(double *res, const double *v, double alpha, int32_t n);           /* ScaleKernel */
    void (*fill)(double *res, double val, int32_t n);                               /* FillKernel */
    /* mode 0: a_ii (FindDiag), 1: 1/a_ii (FindDiagInv), 2: sqrt(1/a_ii)
     * (FindDiagInvSqrt); only rows with a diagonal entry are defined */
    void (*diag)(const orc_csr *A, double *d, int mode);
    double (*diag_abs_min)(const orc_csr *A);                                       /* FindDiagAbsMin */
} orc_backend;

/* NULL restores the CPU emulation.  Not thread-safe: set it between solves. */
void orc_set_backend(const orc_backend *backend);

/* compensated (double-double) true residual norm ||b - A x||_2 */
double orc_true_residual_norm(const orc_csr *A, const double *b, const double *x);

/* ---- solvers ----------------------------------------------------------- */
enum {
    ORC_CG = 0, ORC_BICG = 1, ORC_JACOBI = 2, ORC_MR = 3, ORC_MRJACOBI = 4,
    ORC_MRS = 5, ORC_JMR = 6, ORC_RICHARDSON = 7
};

typedef struct orc_result {
    int32_t n_hist;      /* entries written to history (initial + one per step) */
    int32_t breakdown;   /* BiCG: 1 when |xi| < int_bound stopped the loop */
    double omega;        /* Richardson: relaxation factor used */
    double lambda_max;   /* Richardson: power-method eigenvalue estimate */
    double diag_abs_min; /* Richardson: min |a_ii| */
} orc_result;

double orc_norm_factor(const orc_csr *A, const double *b, const double *x,
                       int32_t grid);
/* A_t may be NULL except for BiCG.  history must hold max_steps+1 entries
 * (or hist_cap entries; the loop also stops when it is full). */
int32_t orc_solve(int32_t kind, const orc_csr *A, const orc_csr *At,
                  const double *b, double *x, double error, int32_t max_steps,
                  int32_t grid, double int_bound, double omega,
                  int32_t power_max_steps, double *history, int32_t hist_cap,
                  orc_result *res);

#ifdef __cplusplus
}
#endif
#endif
