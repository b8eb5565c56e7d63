/*
 * oracle.c -- CPU oracle for the cuFoam sparse solve path.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle.h).  Compiled with -ffp-contract=off:
 * every fused multiply-add the reference's CUDA kernels perform is written
 * as fma() below, every other operation is a single IEEE operation, so the
 * same inputs give the same bits on x86 and on Arm.
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <limits.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ======================================================================= */
/* lduAddressing and ldu2csr                                               */
/* ======================================================================= */

/* OpenFOAM lduAddressing semantics, restated:
 *   ownerStart[c]  = first face whose owner (lowerAddr) is >= c, [n] = F;
 *   losort         = face indices stably sorted by neighbour (upperAddr);
 *   losortStart[c] = first losort position whose neighbour is >= c, [n] = F.
 * Returns 0, or -1 when lowerAddr is not sorted or an index is out of
 * range or a face is not strictly upper-triangular. */
int32_t orc_ldu_addressing(int32_t n, int32_t f, const int32_t *lower_addr,
                           const int32_t *upper_addr, int32_t *losort,
                           int32_t *losort_start, int32_t *owner_start)
{
    if (n < 0 || f < 0) return -1;
    for (int32_t i = 0; i < f; ++i) {
        if (lower_addr[i] < 0 || lower_addr[i] >= n) return -1;
        if (upper_addr[i] < 0 || upper_addr[i] >= n) return -1;
        if (upper_addr[i] <= lower_addr[i]) return -1;
        if (i > 0 && lower_addr[i] < lower_addr[i - 1]) return -1;
    }
    /* ownerStart */
    int32_t fi = 0;
    for (int32_t c = 0; c <= n; ++c) {
        while (fi < f && lower_addr[fi] < c) ++fi;
        owner_start[c] = fi;
    }
    /* losort: counting sort by neighbour, stable in face order */
    int32_t *cnt = (int32_t *)calloc((size_t)(uint32_t)n + 1u, sizeof(int32_t));
    for (int32_t i = 0; i < f; ++i) cnt[upper_addr[i] + 1]++;
    for (int32_t c = 0; c < n; ++c) cnt[c + 1] += cnt[c];
    for (int32_t c = 0; c <= n; ++c) losort_start[c] = cnt[c];
    for (int32_t i = 0; i < f; ++i) losort[cnt[upper_addr[i]]++] = i;
    free(cnt);
    return 0;
}

/* Restatement of getSparseCSRMat (gis/ldu2csr.h:7-40): row c holds the
 * lower coefficients of the faces whose neighbour is c, in losort order,
 * then the diagonal, then the upper coefficients of the faces c owns, in
 * face order. */
void orc_ldu2csr(int32_t n, int32_t f, const double *diag, const double *lower,
                 const double *upper, const int32_t *lower_addr,
                 const int32_t *upper_addr, const int32_t *losort,
                 const int32_t *losort_start, const int32_t *owner_start,
                 int32_t *row_offsets, int32_t *cols, double *vals)
{
    (void)f;
    int32_t e = 0;
    for (int32_t c = 0; c < n; ++c) {
        row_offsets[c] = e;
        for (int32_t idx = losort_start[c]; idx < losort_start[c + 1]; ++idx) {
            int32_t face = losort[idx];
            cols[e] = lower_addr[face];
            vals[e] = lower[face];
            ++e;
        }
        cols[e] = c;
        vals[e] = diag[c];
        ++e;
        for (int32_t face = owner_start[c]; face < owner_start[c + 1]; ++face) {
            cols[e] = upper_addr[face];
            vals[e] = upper[face];
            ++e;
        }
    }
    row_offsets[n] = e;
}

/* ======================================================================= */
/* reference-order primitives                                              */
/* ======================================================================= */
#define REF_BLOCK 256

void orc_set_threads(int32_t n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

int32_t orc_get_threads(void)
{
#ifdef _OPENMP
    return (int32_t)omp_get_max_threads();
#else
    return 1;
#endif
}

/* 256-wide shared-memory tree of the reference's reduction kernels
 * (gis/SparseSystem/kernels.h:100-145): strides 128, 64, then the
 * warp-synchronous 32..1 steps, each t[i] = t[i] + t[i+s]. */
static double block_tree(double *t)
{
    for (int s = REF_BLOCK / 2; s > 0; s >>= 1)
        for (int i = 0; i < s; ++i) t[i] = t[i] + t[i + s];
    return t[0];
}

static const orc_backend *g_backend = NULL;

void orc_set_backend(const orc_backend *backend)
{
    g_backend = backend;
}

/* kind: 0 dot (fma(a,b,t)), 1 sum (t + a), 2 distance (fma(d,d,t), d=a-b) */
static double ref_reduce(int kind, const double *a, const double *b, int32_t n,
                         int32_t grid)
{
    if (g_backend) return g_backend->reduce(kind, a, b, n, grid);
    if (grid <= 0) grid = 1;
    /* blocks whose first index is past n hold exact +0 partials */
    const int32_t busy = (int32_t)(((int64_t)n + REF_BLOCK - 1) / REF_BLOCK) < grid
                             ? (int32_t)(((int64_t)n + REF_BLOCK - 1) / REF_BLOCK)
                             : grid;
    double *partial = (double *)malloc(sizeof(double) * (size_t)(busy > 0 ? busy : 1));
    const int64_t stride = (int64_t)grid * REF_BLOCK;
#pragma omp parallel for schedule(static) if (n > 65536)
    for (int32_t blk = 0; blk < busy; ++blk) {
        double t[REF_BLOCK];
        for (int i = 0; i < REF_BLOCK; ++i) t[i] = 0.0;
        for (int64_t base = (int64_t)blk * REF_BLOCK; base < n; base += stride) {
            int64_t lim = n - base < REF_BLOCK ? n - base : REF_BLOCK;
            const double *pa = a + base;
            if (kind == 0) {
                const double *pb = b + base;
                for (int64_t i = 0; i < lim; ++i) t[i] = fma(pa[i], pb[i], t[i]);
            } else if (kind == 1) {
                for (int64_t i = 0; i < lim; ++i) t[i] = t[i] + pa[i];
            } else {
                const double *pb = b + base;
                for (int64_t i = 0; i < lim; ++i) { double d = pa[i] - pb[i]; t[i] = fma(d, d, t[i]); }
            }
        }
        partial[blk] = block_tree(t);
    }
    double sum = 0.0; /* host-side sequential sum of the block partials */
    for (int32_t blk = 0; blk < busy; ++blk) sum += partial[blk];
    if (busy < grid) sum += 0.0; /* the remaining all-zero partials */
    free(partial);
    return sum;
}

double orc_ref_dot(const double *a, const double *b, int32_t n, int32_t grid)
{
    return ref_reduce(0, a, b, n, grid);
}

double orc_ref_sum(const double *a, int32_t n, int32_t grid)
{
    return ref_reduce(1, a, NULL, n, grid);
}

double orc_ref_distance(const double *a, const double *b, int32_t n, int32_t grid)
{
    return sqrt(ref_reduce(2, a, b, n, grid));
}

/* One row of the reference SpMV (gis/SparseSystem/kernels.h:206-237):
 * 8 lanes accumulate the entries j = start+lane+8m with FMA, then the
 * warp-synchronous tree ((t0+t4)+(t2+t6)) + ((t1+t5)+(t3+t7)). */
static inline double ref_row(const orc_csr *A, const double *x, int32_t row)
{
    const int32_t s = A->row_offsets[row], e = A->row_offsets[row + 1];
    double t[8];
    for (int l = 0; l < 8; ++l) {
        double acc = 0.0;
        for (int32_t j = s + l; j < e; j += 8) acc = fma(A->vals[j], x[A->cols[j]], acc);
        t[l] = acc;
    }
    return ((t[0] + t[4]) + (t[2] + t[6])) + ((t[1] + t[5]) + (t[3] + t[7]));
}

void orc_ref_spmv(const orc_csr *A, const double *x, double *y)
{
    if (g_backend) { g_backend->spmv(A, x, y); return; }
#pragma omp parallel for schedule(static) if (A->n > 16384)
    for (int32_t i = 0; i < A->n; ++i) y[i] = ref_row(A, x, i);
}

void orc_ref_residual(const orc_csr *A, const double *b, const double *x, double *r)
{
    if (g_backend) { g_backend->residual(A, b, x, r); return; }
#pragma omp parallel for schedule(static) if (A->n > 16384)
    for (int32_t i = 0; i < A->n; ++i) r[i] = b[i] - ref_row(A, x, i);
}

/* Element-wise kernels (gis/SparseSystem/kernels.h:318-402). */
static void v_add(double *res, const double *v1, const double *v2, double alpha, int32_t n)
{   /* AddKernel1: v1 + alpha*v2, contracted to fma */
    if (g_backend) { g_backend->add(res, v1, v2, alpha, n); return; }
#pragma omp parallel for schedule(static) if (n > 65536)
    for (int32_t i = 0; i < n; ++i) res[i] = fma(alpha, v2[i], v1[i]);
}

static void v_hadamard(double *res, const double *v1, const double *v2, int32_t n)
{
    if (g_backend) { g_backend->hadamard(res, v1, v2, n); return; }
#pragma omp parallel for schedule(static) if (n > 65536)
    for (int32_t i = 0; i < n; ++i) res[i] = v1[i] * v2[i];
}

static void v_scale(double *res, const double *v, double alpha, int32_t n)
{
    if (g_backend) { g_backend->scale(res, v, alpha, n); return; }
#pragma omp parallel for schedule(static) if (n > 65536)
    for (int32_t i = 0; i < n; ++i) res[i] = alpha * v[i];
}

static void v_fill(double *res, double val, int32_t n)
{
    if (g_backend) { g_backend->fill(res, val, n); return; }
#pragma omp parallel for schedule(static) if (n > 65536)
    for (int32_t i = 0; i < n; ++i) res[i] = val;
}

static void v_copy(double *res, const double *v, int32_t n)
{
    memcpy(res, v, sizeof(double) * (size_t)n);
}

/* diagonal entry of each row (FindDiag, gis/SparseSystem/kernels.h:447-464):
 * the entry with column == row; rows without one read as 0 (the reference
 * leaves them unset).  mode 1 gives 1/a_ii (FindDiagInv, :563-580), mode 2
 * sqrt(1/a_ii) (FindDiagInvSqrt, :586-603). */
static void diag_vec(const orc_csr *A, double *d, int mode)
{
    if (g_backend) { g_backend->diag(A, d, mode); return; }
#pragma omp parallel for schedule(static)
    for (int32_t i = 0; i < A->n; ++i) {
        double v = 0.0;
        for (int32_t j = A->row_offsets[i]; j < A->row_offsets[i + 1] && A->cols[j] <= i; ++j)
            if (A->cols[j] == i) v = A->vals[j];
        d[i] = mode == 0 ? v : mode == 1 ? 1.0 / v : sqrt(1.0 / v);
    }
}

/* ---- compensated true residual ---------------------------------------- */
static inline void two_sum(double a, double b, double *s, double *e)
{
    double x = a + b, bb = x - a;
    *s = x;
    *e = (a - (x - bb)) + (b - bb);
}

double orc_true_residual_norm(const orc_csr *A, const double *b, const double *x)
{
    double hi = 0.0, lo = 0.0;
#pragma omp parallel
    {
        double th = 0.0, tl = 0.0;
#pragma omp for schedule(static)
        for (int32_t i = 0; i < A->n; ++i) {
            double sh = b[i], sl = 0.0;
            for (int32_t j = A->row_offsets[i]; j < A->row_offsets[i + 1]; ++j) {
                double p = A->vals[j] * x[A->cols[j]];
                double pe = fma(A->vals[j], x[A->cols[j]], -p);
                double s, e;
                two_sum(sh, -p, &s, &e);
                sh = s;
                sl = sl + (e - pe);
            }
            double r = sh + sl;
            double r2 = r * r, r2e = fma(r, r, -r2);
            double s, e;
            two_sum(th, r2, &s, &e);
            th = s;
            tl = tl + (e + r2e);
        }
#pragma omp critical
        {
            double s, e;
            two_sum(hi, th, &s, &e);
            hi = s;
            lo = lo + (e + tl);
        }
    }
    return sqrt(hi + lo);
}

/* ======================================================================= */
/* NormFactor and solvers                                                  */
/* ======================================================================= */

/* gis/gis.cu:106-123 */
double orc_norm_factor(const orc_csr *A, const double *b, const double *x, int32_t grid)
{
    const int32_t N = A->n;
    double x_bar = orc_ref_sum(x, N, grid) / N;
    double *X_bar = (double *)malloc(sizeof(double) * (size_t)(N > 0 ? N : 1));
    double *Y = (double *)malloc(sizeof(double) * (size_t)(N > 0 ? N : 1));
    double *Y_bar = (double *)malloc(sizeof(double) * (size_t)(N > 0 ? N : 1));
    v_fill(X_bar, x_bar, N);
    orc_ref_spmv(A, x, Y);
    orc_ref_spmv(A, X_bar, Y_bar);
    double nf = orc_ref_distance(Y, Y_bar, N, grid) + orc_ref_distance(b, Y_bar, N, grid) + 1e-20;
    free(X_bar); free(Y); free(Y_bar);
    return nf;
}

typedef struct {
    double *hist;
    int32_t cap;
    int32_t len;
} histbuf;

static int hist_push(histbuf *h, double v)
{
    if (h->len < h->cap) { h->hist[h->len++] = v; return 1; }
    return 0;
}

#define VEC(name) double *name = (double *)calloc((size_t)(N > 0 ? N : 1), sizeof(double))

/* SolverSingleGPU.h:366-445 */
static void solve_cg(const orc_csr *A, const double *b, double *x, double error,
                     int32_t max_steps, int32_t G, histbuf *h)
{
    const int32_t N = A->n;
    VEC(r); VEC(p); VEC(q);
    orc_ref_residual(A, b, x, r);
    v_copy(p, r, N);
    double rho0 = orc_ref_dot(r, r, N, G), rho1 = 0.0;
    double norm_r = sqrt(rho0);
    if (max_steps <= 0) max_steps = INT_MAX;
    hist_push(h, norm_r);
    for (int32_t k = 1; k <= max_steps && norm_r > error; ++k) {
        if (k > 1) v_add(p, r, p, rho0 / rho1, N);
        orc_ref_spmv(A, p, q);
        double xi = rho0 / orc_ref_dot(p, q, N, G);
        v_add(x, x, p, xi, N);
        v_add(r, r, q, -xi, N);
        rho1 = rho0;
        rho0 = orc_ref_dot(r, r, N, G);
        norm_r = sqrt(rho0);
        if (!hist_push(h, norm_r)) break;
        if (k == INT_MAX) break;
    }
    free(r); free(p); free(q);
}

/* SolverSingleGPU.h:568-675 (BiCG with an explicit transpose) */
static int solve_bicg(const orc_csr *A, const orc_csr *At, const double *b, double *x,
                      double error, int32_t max_steps, double int_bound, int32_t G,
                      histbuf *h)
{
    const int32_t N = A->n;
    VEC(r); VEC(rs); VEC(p); VEC(ps); VEC(q); VEC(qs);
    int broke = 0;
    orc_ref_residual(A, b, x, r);
    v_copy(rs, r, N);
    v_copy(p, r, N);
    v_copy(ps, rs, N);
    double rho0 = orc_ref_dot(r, rs, N, G), rho1 = 0.0;
    double norm_r = sqrt(orc_ref_dot(r, r, N, G));
    if (max_steps <= 0) max_steps = INT_MAX;
    hist_push(h, norm_r);
    for (int32_t k = 1; k <= max_steps; ++k) {
        orc_ref_spmv(A, p, q);
        double xi = rho0 / orc_ref_dot(ps, q, N, G);
        if (xi > -int_bound && xi < int_bound) { broke = 1; break; }
        v_add(x, x, p, xi, N);
        v_add(r, r, q, -xi, N);
        norm_r = sqrt(orc_ref_dot(r, r, N, G));
        if (!hist_push(h, norm_r)) break;
        if (norm_r < error) break;
        orc_ref_spmv(At, ps, qs);
        v_add(rs, rs, qs, -xi, N);
        rho1 = rho0;
        rho0 = orc_ref_dot(r, rs, N, G);
        double theta = rho0 / rho1;
        v_add(p, r, p, theta, N);
        v_add(ps, rs, ps, theta, N);
        if (k == INT_MAX) break;
    }
    free(r); free(rs); free(p); free(ps); free(q); free(qs);
    return broke;
}

/* FindDiagAbsMin, SolverSingleGPU.h:686-720 */
static double diag_abs_min(const orc_csr *A)
{
    if (g_backend) return g_backend->diag_abs_min(A);
    const int32_t N = A->n;
    VEC(d);
    diag_vec(A, d, 0);
    double m = HUGE_VAL;
    for (int32_t i = 0; i < N; ++i) { double a = fabs(d[i]); if (a < m) m = a; }
    free(d);
    return m;
}

/* OptimizePower, SolverSingleGPU.h:723-752 */
static double optimize_power(const orc_csr *A, int32_t max_steps, int32_t G,
                             double *lmax, double *dmin)
{
    const int32_t N = A->n;
    VEC(x1); VEC(x2); VEC(Av);
    v_fill(x1, 0.0, N);
    v_fill(x2, 1.0 / N, N);
    for (int32_t s = 0; s < max_steps; ++s) {
        v_copy(x1, x2, N);
        orc_ref_spmv(A, x1, x2);
        double norm_x2 = sqrt(orc_ref_dot(x2, x2, N, G));
        v_scale(x2, x2, 1 / norm_x2, N);
    }
    orc_ref_spmv(A, x2, Av);
    double max_eigenvalue = orc_ref_dot(x2, Av, N, G);
    double min_eigenvalue = diag_abs_min(A);
    free(x1); free(x2); free(Av);
    *lmax = max_eigenvalue;
    *dmin = min_eigenvalue;
    return 2.0 / (max_eigenvalue + min_eigenvalue);
}

/* SolverSingleGPU.h:762-819 */
static void solve_richardson(const orc_csr *A, const double *b, double *x, double error,
                             double omega, int32_t power_max_steps, int32_t max_steps,
                             int32_t G, histbuf *h, orc_result *res)
{
    const int32_t N = A->n;
    res->lambda_max = 0.0;
    res->diag_abs_min = 0.0;
    if (-1e-15 < omega && omega < 1e-15)
        omega = optimize_power(A, power_max_steps, G, &res->lambda_max, &res->diag_abs_min);
    res->omega = omega;
    VEC(r);
    orc_ref_residual(A, b, x, r);
    double norm_r = sqrt(orc_ref_dot(r, r, N, G));
    if (max_steps <= 0) max_steps = INT_MAX;
    hist_push(h, norm_r);
    int64_t k = 1;
    while (k++ <= max_steps && norm_r > error) {
        v_add(x, x, r, omega, N);
        orc_ref_residual(A, b, x, r);
        norm_r = sqrt(orc_ref_dot(r, r, N, G));
        if (!hist_push(h, norm_r)) break;
    }
    free(r);
}

/* SolverSingleGPU.h:825-890 */
static void solve_mr(const orc_csr *A, const double *b, double *x, double error,
                     int32_t max_steps, int32_t G, histbuf *h)
{
    const int32_t N = A->n;
    VEC(r); VEC(Ar);
    orc_ref_residual(A, b, x, r);
    double norm_r = sqrt(orc_ref_dot(r, r, N, G));
    if (max_steps <= 0) max_steps = INT_MAX;
    hist_push(h, norm_r);
    int64_t k = 1;
    while (k++ <= max_steps && norm_r > error) {
        orc_ref_spmv(A, r, Ar);
        double omega = orc_ref_dot(r, Ar, N, G) / orc_ref_dot(Ar, Ar, N, G);
        v_add(x, x, r, omega, N);
        v_add(r, r, Ar, -omega, N);
        norm_r = sqrt(orc_ref_dot(r, r, N, G));
        if (!hist_push(h, norm_r)) break;
    }
    free(r); free(Ar);
}

/* SolverSingleGPU.h:924-994 (Jacobi in residual form) */
static void solve_jacobi(const orc_csr *A, const double *b, double *x, double error,
                         int32_t max_steps, int32_t G, histbuf *h)
{
    const int32_t N = A->n;
    VEC(r); VEC(D_1); VEC(D_1r); VEC(AD_1r);
    orc_ref_residual(A, b, x, r);
    double norm_r = sqrt(orc_ref_dot(r, r, N, G));
    diag_vec(A, D_1, 1); /* FindDiagInv */
    if (max_steps <= 0) max_steps = INT_MAX;
    hist_push(h, norm_r);
    int64_t k = 1;
    while (k++ <= max_steps && norm_r > error) {
        v_hadamard(D_1r, D_1, r, N);
        orc_ref_spmv(A, D_1r, AD_1r);
        v_add(x, x, D_1r, 1.0, N);
        v_add(r, r, AD_1r, -1.0, N);
        norm_r = sqrt(orc_ref_dot(r, r, N, G));
        if (!hist_push(h, norm_r)) break;
    }
    free(r); free(D_1); free(D_1r); free(AD_1r);
}

/* SolverSingleGPU.h:1000-1073 */
static void solve_mrjacobi(const orc_csr *A, const double *b, double *x, double error,
                           int32_t max_steps, int32_t G, histbuf *h)
{
    const int32_t N = A->n;
    VEC(r); VEC(D_1); VEC(D_1r); VEC(AD_1r);
    orc_ref_residual(A, b, x, r);
    double norm_r = sqrt(orc_ref_dot(r, r, N, G));
    diag_vec(A, D_1, 1); /* FindDiagInv */
    if (max_steps <= 0) max_steps = INT_MAX;
    hist_push(h, norm_r);
    int64_t k = 1;
    while (k++ <= max_steps && norm_r > error) {
        v_hadamard(D_1r, D_1, r, N);
        orc_ref_spmv(A, D_1r, AD_1r);
        double alpha = orc_ref_dot(r, AD_1r, N, G) / orc_ref_dot(AD_1r, AD_1r, N, G);
        v_add(x, x, D_1r, alpha, N);
        v_add(r, r, AD_1r, -alpha, N);
        norm_r = sqrt(orc_ref_dot(r, r, N, G));
        if (!hist_push(h, norm_r)) break;
    }
    free(r); free(D_1); free(D_1r); free(AD_1r);
}

/* PreconditionedMRJacobi (JMR), SolverSingleGPU.h:1079-1155 */
static void solve_jmr(const orc_csr *A, const double *b, double *x, double error,
                      int32_t max_steps, int32_t G, histbuf *h)
{
    const int32_t N = A->n;
    VEC(sD); VEC(r); VEC(sDr); VEC(z);
    diag_vec(A, sD, 2); /* FindDiagInvSqrt */
    orc_ref_residual(A, b, x, r);
    v_hadamard(r, sD, r, N);
    double norm_r = sqrt(orc_ref_dot(r, r, N, G));
    if (max_steps <= 0) max_steps = INT_MAX;
    hist_push(h, norm_r);
    int64_t k = 1;
    while (k++ <= max_steps && norm_r > error) {
        v_hadamard(sDr, sD, r, N);
        orc_ref_spmv(A, sDr, z);
        v_hadamard(z, sD, z, N);
        double alpha = orc_ref_dot(r, z, N, G) / orc_ref_dot(z, z, N, G);
        v_add(x, x, sDr, alpha, N);
        v_add(r, r, z, -alpha, N);
        norm_r = sqrt(orc_ref_dot(r, r, N, G));
        if (!hist_push(h, norm_r)) break;
    }
    free(sD); free(r); free(sDr); free(z);
}

/* MRS, SolverSingleGPU.h:1236-1303, with invM = JacobiPrecondition()
 * (gis/SparseSystem/SparseCPU.h:428-446): a diagonal CSR of 1/a_ii,
 * applied through the SpMV. */
static void solve_mrs(const orc_csr *A, const double *b, double *x, double error,
                      int32_t max_steps, int32_t G, histbuf *h)
{
    const int32_t N = A->n;
    int32_t *mro = (int32_t *)malloc(sizeof(int32_t) * ((size_t)N + 1));
    int32_t *mcol = (int32_t *)malloc(sizeof(int32_t) * (size_t)(N > 0 ? N : 1));
    double *mval = (double *)malloc(sizeof(double) * (size_t)(N > 0 ? N : 1));
    mro[0] = 0;
    for (int32_t i = 0; i < N; ++i) {
        int32_t j = A->row_offsets[i];
        while (j < A->row_offsets[i + 1] && A->cols[j] < i) ++j;
        mval[i] = (j < A->row_offsets[i + 1] && A->cols[j] == i) ? 1 / A->vals[j] : NAN;
        mcol[i] = i;
        mro[i + 1] = i + 1;
    }
    orc_csr invM = {N, N, mro, mcol, mval};
    VEC(r); VEC(Mr); VEC(AMr);
    orc_ref_residual(A, b, x, r);
    double norm_r = sqrt(orc_ref_dot(r, r, N, G));
    if (max_steps <= 0) max_steps = INT_MAX;
    hist_push(h, norm_r);
    int64_t k = 1;
    while (k++ <= max_steps && norm_r > error) {
        orc_ref_spmv(&invM, r, Mr);
        orc_ref_spmv(A, Mr, AMr);
        double alpha = orc_ref_dot(r, AMr, N, G) / orc_ref_dot(AMr, AMr, N, G);
        v_add(x, x, Mr, alpha, N);
        v_add(r, r, AMr, -alpha, N);
        norm_r = sqrt(orc_ref_dot(r, r, N, G));
        if (!hist_push(h, norm_r)) break;
    }
    free(r); free(Mr); free(AMr); free(mro); free(mcol); free(mval);
}

int32_t orc_solve(int32_t kind, const orc_csr *A, const orc_csr *At,
                  const double *b, double *x, double error, int32_t max_steps,
                  int32_t grid, double int_bound, double omega,
                  int32_t power_max_steps, double *history, int32_t hist_cap,
                  orc_result *res)
{
    histbuf h = {history, hist_cap, 0};
    orc_result local;
    if (!res) res = &local;
    memset(res, 0, sizeof(*res));
    switch (kind) {
    case ORC_CG: solve_cg(A, b, x, error, max_steps, grid, &h); break;
    case ORC_BICG:
        if (!At) return -1;
        res->breakdown = solve_bicg(A, At, b, x, error, max_steps, int_bound, grid, &h);
        break;
    case ORC_JACOBI: solve_jacobi(A, b, x, error, max_steps, grid, &h); break;
    case ORC_MR: solve_mr(A, b, x, error, max_steps, grid, &h); break;
    case ORC_MRJACOBI: solve_mrjacobi(A, b, x, error, max_steps, grid, &h); break;
    case ORC_MRS: solve_mrs(A, b, x, error, max_steps, grid, &h); break;
    case ORC_JMR: solve_jmr(A, b, x, error, max_steps, grid, &h); break;
    case ORC_RICHARDSON:
        solve_richardson(A, b, x, error, omega, power_max_steps, max_steps, grid, &h, res);
        break;
    default: return -1;
    }
    res->n_hist = h.len;
    return 0;
}
