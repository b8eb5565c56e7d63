// solve_fp64.cu -- FP64 solvers of the eight cuFoam plugins as fused
// row-sweep kernels with device-side loop control.
//
// Each reference iteration (gis/SparseSystem/SolverSingleGPU.h) becomes one
// or two kernels.  Kernels that need A*v stage a warp's 32 consecutive CSR
// rows in shared memory with 16-byte loads and form v on the fly from the
// vectors it is built of (p = r + beta*p_old, D^-1 r, x + omega*r, ...), so
// the element-wise steps cost no extra pass.  Dot products are reduced in
// the same pass; the last block to finish computes the step scalars, the
// stopping test and the CUDA-graph loop condition.  Every scalar and every
// vector element is formed with the reference's operations (FMA where the
// reference's kernels contract to FMA), and with CF_REDUCE_REFERENCE the
// dot products also follow the reference's grid and summation order, so the
// solve reproduces the reference algorithm's bits.
#include "solver_common.cuh"

#include <algorithm>
#include <chrono>
#include <climits>
#include <cmath>
#include <thread>

namespace cf {

// ---------------------------------------------------------------------------
// normFactor (gis/gis.cu:106-123; OpenFOAM's L1 form as an option)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kBlock) k_nf_sum(const SolveArgs *__restrict__ a)
{
    const int n = a->n;
    const double *x = a->x;
    double acc[1] = {0.0};
    CF_FOR_ELEMS(i, n) acc[0] = acc[0] + x[i]; // ReductionKernel: t += v[i]
    double tot[1];
    if (grid_reduce<1, double>(acc, a->partials, a->partial_stride, &a->st->counters[SLOT_NF1],
                               a->ref_order, tot) && threadIdx.x == 0)
        a->st->xbar = tot[0] / n;
}

__global__ void __launch_bounds__(kBlock) k_nf_dist(const SolveArgs *__restrict__ a, int l1)
{
    const int n = a->n, cap = a->stage_cap;
    CF_STAGE(double, cap);
    const double *x = a->x, *b = a->b;
    const double xbar = ld_cg(&a->st->xbar);
    double acc[2] = {0.0, 0.0};
    CF_FOR_CHUNKS(base, n) {
        const RefRow R(a, base, cap, sv_, sc_);
        const int row = base + (threadIdx.x & 31);
        const double Y = R.product([&](int c) { return x[c]; });
        double Yb;
        if (!l1) Yb = R.product([&](int) { return xbar; });
        else Yb = __dmul_rn(R.product([&](int) { return 1.0; }), xbar);
        if (row < n) {
            const double d1 = Y - Yb, d2 = b[row] - Yb;
            if (!l1) {
                acc[0] = fma_t(d1, d1, acc[0]); // DistanceKernel
                acc[1] = fma_t(d2, d2, acc[1]);
            } else {
                acc[0] = acc[0] + (fabs(d1) + fabs(d2));
            }
        }
        __syncwarp();
    }
    double tot[2];
    if (grid_reduce<2, double>(acc, a->partials, a->partial_stride, &a->st->counters[SLOT_NF2],
                               a->ref_order, tot) && threadIdx.x == 0) {
        DevState *st = a->st;
        const double nf = l1 ? tot[0] + 1e-20 : sqrt(tot[0]) + sqrt(tot[1]) + 1e-20;
        st->nf = nf;
        st->tol = (st->flags & kFlagAbsTol) ? st->tolerance : st->tolerance * nf;
    }
}

// ---------------------------------------------------------------------------
// initial residual r = b - A x (ResidualKernel), ||r||
// mode 0: plain; 1: JMR (r = D^-1/2 (b - A x)); 2: BiCG (also r* = r)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kBlock) k_res_init(const SolveArgs *__restrict__ a, int mode)
{
    const int n = a->n, cap = a->stage_cap;
    CF_STAGE(double, cap);
    const double *x = a->x, *b = a->b, *sD = a->dinv_sqrt, *dinv = a->dinv;
    double *r = a->r[0], *rs = a->rs;
    double acc[2] = {0.0, 0.0};
    CF_FOR_CHUNKS(base, n) {
        const RefRow R(a, base, cap, sv_, sc_);
        const int row = base + (threadIdx.x & 31);
        const double t = R.product([&](int c) { return x[c]; });
        if (row < n) {
            double ri = b[row] - t;
            if (mode == 1) ri = __dmul_rn(sD[row], ri);
            r[row] = ri;
            if (mode == 2) rs[row] = ri;
            if (mode == 4) a->w[1][row] = __dmul_rn(dinv[row], ri); // z = D^-1 r
            acc[0] = fma_t(ri, ri, acc[0]);
            if (mode == 3) acc[1] = fma_t(ri, __dmul_rn(dinv[row], ri), acc[1]);
        }
        __syncwarp();
    }
    double tot[2];
    if (grid_reduce<2, double>(acc, a->partials, a->partial_stride, &a->st->counters[SLOT_INIT],
                               a->ref_order, tot) && threadIdx.x == 0) {
        finish_init(a, a->st, tot[0], mode == 2);
        if (mode == 3) a->st->rho0 = tot[1]; // PCG: (r, D^-1 r)
    }
}

// ---------------------------------------------------------------------------
// CG (SolverSingleGPU.h:366-445)
//   K1: p_k = r + beta p_{k-1} (on the fly), q = A p_k, (p_k, q);
//       also applies the deferred x += xi_{k-1} p_{k-1}
//   K2: r -= xi q, (r, r), stopping test
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kBlock) k_cg_spmv(const SolveArgs *__restrict__ a)
{
    DevState *st = a->st;
    CF_EXIT_IF_DONE(a, st, false);
    const int n = a->n, cap = a->stage_cap;
    CF_STAGE(double, cap);
    const int k = ld_cg(&st->k) + 1;
    const bool first = (k == 1);
    const double beta = first ? 0.0 : ld_cg(&st->beta); // rho0 / rho1, formed once
    const double xi_prev = ld_cg(&st->xi);
    const bool xpend = ld_cg(&st->x_pending) != 0;
    const double *pin = a->p[(k + 1) & 1];
    double *pout = a->p[k & 1];
    const double *r = a->r[0];
    double *x = a->x, *q = a->q;
    auto g = [&](int c) { return first ? r[c] : fma_t(beta, pin[c], r[c]); };
    double acc[1] = {0.0};
    CF_FOR_CHUNKS(base, n) {
        const RefRow R(a, base, cap, sv_, sc_);
        const int row = base + (threadIdx.x & 31);
        const double y = R.product(g);
        if (row < n) {
            const double pi = g(row);
            pout[row] = pi;
            q[row] = y;
            if (xpend) x[row] = fma_t(xi_prev, pin[row], x[row]);
            acc[0] = fma_t(pi, y, acc[0]);
        }
        __syncwarp();
    }
    double tot[1];
    if (grid_reduce<1, double>(acc, a->partials, a->partial_stride, &st->counters[SLOT_A],
                               a->ref_order, tot) && threadIdx.x == 0) {
        st->xi = st->rho0 / tot[0];
        st->x_pending = 0;
    }
}

__global__ void __launch_bounds__(kBlock) k_cg_update(const SolveArgs *__restrict__ a)
{
    DevState *st = a->st;
    CF_EXIT_IF_DONE(a, st, true);
    const int n = a->n;
    const double xi = ld_cg(&st->xi);
    double *r = a->r[0];
    const double *q = a->q;
    double acc[1] = {0.0};
    CF_FOR_ELEMS(i, n) {
        const double ri = fma_t(-xi, q[i], r[i]);
        r[i] = ri;
        acc[0] = fma_t(ri, ri, acc[0]);
    }
    double tot[1];
    if (grid_reduce<1, double>(acc, a->partials, a->partial_stride, &st->counters[SLOT_B],
                               a->ref_order, tot) && threadIdx.x == 0) {
        st->rho1 = st->rho0;
        st->rho0 = tot[0];
        st->beta = st->rho0 / st->rho1;
        st->x_pending = 1;
        finish_step(a, st, sqrt(tot[0]));
    }
}

// x += xi * p_k for the last step (deferred update of CG and BiCG).
__global__ void __launch_bounds__(kBlock) k_flush_x(const SolveArgs *__restrict__ a)
{
    DevState *st = a->st;
    if (!ld_cg(&st->x_pending)) return;
    const int n = a->n;
    const int k = ld_cg(&st->k);
    const double xi = ld_cg(&st->xi);
    const double *p = a->p[k & 1];
    double *x = a->x;
    CF_FOR_ELEMS(i, n) x[i] = fma_t(xi, p[i], x[i]);
}

__global__ void k_clear_pending(DevState *st)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) st->x_pending = 0;
}

// ---------------------------------------------------------------------------
// BiCG with A^T (SolverSingleGPU.h:568-675)
//   K1: p, p* updates on the fly; q = A p and q* = A^T p* in one pass over
//       the shared pattern; (p*, q); breakdown test on xi
//   K2: r -= xi q, r* -= xi q*, ||r||, (r, r*), stopping test, theta
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kBlock) k_bicg_spmv(const SolveArgs *__restrict__ a)
{
    DevState *st = a->st;
    CF_EXIT_IF_DONE(a, st, false);
    const int n = a->n, cap = a->stage_cap;
    CF_STAGE(double, cap);
    const int k = ld_cg(&st->k) + 1;
    const bool first = (k == 1);
    const double theta = ld_cg(&st->theta);
    const double xi_prev = ld_cg(&st->xi);
    const bool xpend = ld_cg(&st->x_pending) != 0;
    const double *pin = a->p[(k + 1) & 1], *psin = a->ps[(k + 1) & 1];
    double *pout = a->p[k & 1], *psout = a->ps[k & 1];
    const double *r = a->r[0], *rs = a->rs;
    double *x = a->x, *q = a->q, *qs = a->qs;
    auto gp = [&](int c) { return first ? r[c] : fma_t(theta, pin[c], r[c]); };
    auto gps = [&](int c) { return first ? rs[c] : fma_t(theta, psin[c], rs[c]); };
    double acc[1] = {0.0};
    CF_FOR_CHUNKS(base, n) {
        const RefRow R(a, base, cap, sv_, sc_);
        const int row = base + (threadIdx.x & 31);
        double y1, y2;
        R.product2(gp, gps, y1, y2);
        if (row < n) {
            const double pi = gp(row), psi = gps(row);
            pout[row] = pi;
            psout[row] = psi;
            q[row] = y1;
            qs[row] = y2;
            if (xpend) x[row] = fma_t(xi_prev, pin[row], x[row]);
            acc[0] = fma_t(psi, y1, acc[0]);
        }
        __syncwarp();
    }
    double tot[1];
    if (grid_reduce<1, double>(acc, a->partials, a->partial_stride, &st->counters[SLOT_A],
                               a->ref_order, tot) && threadIdx.x == 0) {
        const double xi = st->rho0 / tot[0];
        st->x_pending = 0;
        const double bound = st->int_bound;
        if (xi > -bound && xi < bound) { // breakdown: the reference returns here
            st->done = 1;
            st->status = CF_BREAKDOWN;
        } else {
            st->xi = xi;
        }
    }
}

__global__ void __launch_bounds__(kBlock) k_bicg_update(const SolveArgs *__restrict__ a)
{
    DevState *st = a->st;
    CF_EXIT_IF_DONE(a, st, true);
    const int n = a->n;
    const double xi = ld_cg(&st->xi);
    double *r = a->r[0], *rs = a->rs;
    const double *q = a->q, *qs = a->qs;
    double acc[2] = {0.0, 0.0};
    CF_FOR_ELEMS(i, n) {
        const double ri = fma_t(-xi, q[i], r[i]);
        const double rsi = fma_t(-xi, qs[i], rs[i]);
        r[i] = ri;
        rs[i] = rsi;
        acc[0] = fma_t(ri, ri, acc[0]);
        acc[1] = fma_t(ri, rsi, acc[1]);
    }
    double tot[2];
    if (grid_reduce<2, double>(acc, a->partials, a->partial_stride, &st->counters[SLOT_B],
                               a->ref_order, tot) && threadIdx.x == 0) {
        const double norm = sqrt(tot[0]);
        const int k = st->k + 1;
        st->k = k;
        st->norm = norm;
        st->x_pending = 1;
        record_hist(a, st, k, norm);
        bool cont = true;
        int status = CF_NOT_CONVERGED;
        if (norm < st->tol && k >= st->min_steps) { cont = false; status = CF_OK; }
        else if (k >= st->max_steps) { cont = false; status = CF_NOT_CONVERGED; }
        else if (!isfinite(norm)) { cont = false; status = CF_NONFINITE; }
        st->body_count += 1;
        if (st->body_count > k + 2 || (a->abort_flag && *a->abort_flag)) { cont = false; status = CF_TIMEOUT; }
        if (cont) {
            st->rho1 = st->rho0;
            st->rho0 = tot[1];
            st->theta = st->rho0 / st->rho1;
        } else {
            st->done = 1;
            st->status = status;
        }
        set_loop_condition(a, cont);
    }
}

// ---------------------------------------------------------------------------
// Richardson (SolverSingleGPU.h:723-819): power method for omega, then
//   x_k = x_{k-1} + omega r_{k-1}; r_k = b - A x_k  (one kernel per step:
//   x and r are double-buffered, the new x is formed on the fly)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kBlock) k_pow_step(const SolveArgs *__restrict__ a, int s)
{
    const int n = a->n, cap = a->stage_cap;
    CF_STAGE(double, cap);
    DevState *st = a->st;
    const double inv_n = 1.0 / n;
    const double sc = ld_cg(&st->pow_inv);
    const double *yprev = a->w[(s + 1) & 1];
    double *y = a->w[s & 1];
    auto g = [&](int c) { return s == 0 ? inv_n : __dmul_rn(sc, yprev[c]); };
    double acc[1] = {0.0};
    CF_FOR_CHUNKS(base, n) {
        const RefRow R(a, base, cap, sv_, sc_);
        const int row = base + (threadIdx.x & 31);
        const double v = R.product(g);
        if (row < n) {
            y[row] = v;
            acc[0] = fma_t(v, v, acc[0]);
        }
        __syncwarp();
    }
    double tot[1];
    if (grid_reduce<1, double>(acc, a->partials, a->partial_stride, &st->counters[SLOT_POW],
                               a->ref_order, tot) && threadIdx.x == 0)
        st->pow_inv = 1 / sqrt(tot[0]);
}

__global__ void __launch_bounds__(kBlock) k_pow_final(const SolveArgs *__restrict__ a, int steps)
{
    const int n = a->n, cap = a->stage_cap;
    CF_STAGE(double, cap);
    DevState *st = a->st;
    const double inv_n = 1.0 / n;
    const double sc = ld_cg(&st->pow_inv);
    const double *ylast = a->w[(steps + 1) & 1];
    auto g = [&](int c) { return steps == 0 ? inv_n : __dmul_rn(sc, ylast[c]); };
    double acc[1] = {0.0};
    CF_FOR_CHUNKS(base, n) {
        const RefRow R(a, base, cap, sv_, sc_);
        const int row = base + (threadIdx.x & 31);
        const double av = R.product(g);
        if (row < n) acc[0] = fma_t(g(row), av, acc[0]);
        __syncwarp();
    }
    double tot[1];
    if (grid_reduce<1, double>(acc, a->partials, a->partial_stride, &st->counters[SLOT_POW],
                               a->ref_order, tot) && threadIdx.x == 0) {
        st->lambda_max = tot[0];
        st->omega = 2.0 / (tot[0] + st->diag_abs_min);
    }
}

__global__ void __launch_bounds__(kBlock) k_rich_step(const SolveArgs *__restrict__ a)
{
    DevState *st = a->st;
    CF_EXIT_IF_DONE(a, st, true);
    const int n = a->n, cap = a->stage_cap;
    CF_STAGE(double, cap);
    const int k = ld_cg(&st->k) + 1;
    const double omega = ld_cg(&st->omega);
    const double *xold = (k & 1) ? a->x : a->w[1];
    double *xnew = (k & 1) ? a->w[1] : a->x;
    const double *rold = a->r[(k + 1) & 1];
    double *rnew = a->r[k & 1];
    const double *b = a->b;
    auto g = [&](int c) { return fma_t(omega, rold[c], xold[c]); };
    double acc[1] = {0.0};
    CF_FOR_CHUNKS(base, n) {
        const RefRow R(a, base, cap, sv_, sc_);
        const int row = base + (threadIdx.x & 31);
        const double t = R.product(g);
        if (row < n) {
            const double ri = b[row] - t;
            xnew[row] = g(row);
            rnew[row] = ri;
            acc[0] = fma_t(ri, ri, acc[0]);
        }
        __syncwarp();
    }
    double tot[1];
    if (grid_reduce<1, double>(acc, a->partials, a->partial_stride, &st->counters[SLOT_A],
                               a->ref_order, tot) && threadIdx.x == 0)
        finish_step(a, st, sqrt(tot[0]));
}

// After Richardson: the latest x is in w[1] when an odd number of steps ran.
__global__ void __launch_bounds__(kBlock) k_rich_finish(const SolveArgs *__restrict__ a)
{
    if (!(ld_cg(&a->st->k) & 1)) return;
    const int n = a->n;
    const double *src = a->w[1];
    double *x = a->x;
    CF_FOR_ELEMS(i, n) x[i] = src[i];
}

// ---------------------------------------------------------------------------
// Jacobi in residual form (SolverSingleGPU.h:924-994), one kernel per step:
//   d = D^-1 r (on the fly); r_new = r - A d; x += d
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kBlock) k_jacobi_step(const SolveArgs *__restrict__ a)
{
    DevState *st = a->st;
    CF_EXIT_IF_DONE(a, st, true);
    const int n = a->n, cap = a->stage_cap;
    CF_STAGE(double, cap);
    const int k = ld_cg(&st->k) + 1;
    const double *rold = a->r[(k + 1) & 1];
    double *rnew = a->r[k & 1];
    const double *dinv = a->dinv;
    double *x = a->x;
    auto g = [&](int c) { return __dmul_rn(dinv[c], rold[c]); };
    double acc[1] = {0.0};
    CF_FOR_CHUNKS(base, n) {
        const RefRow R(a, base, cap, sv_, sc_);
        const int row = base + (threadIdx.x & 31);
        const double y = R.product(g);
        if (row < n) {
            const double d = g(row);
            x[row] = fma_t(1.0, d, x[row]);
            const double ri = fma_t(-1.0, y, rold[row]);
            rnew[row] = ri;
            acc[0] = fma_t(ri, ri, acc[0]);
        }
        __syncwarp();
    }
    double tot[1];
    if (grid_reduce<1, double>(acc, a->partials, a->partial_stride, &st->counters[SLOT_A],
                               a->ref_order, tot) && threadIdx.x == 0)
        finish_step(a, st, sqrt(tot[0]));
}

// ---------------------------------------------------------------------------
// MR family: y = A M r (M = I for MR, D^-1 for MRJacobi/MRS, and the
// symmetric D^-1/2 scaling for JMR), alpha = (r, y)/(y, y), then
// x += alpha M r, r -= alpha y.
// kind 0 MR (:825-890), 1 MRJacobi (:1000-1073), 2 MRS (:1236-1303,
// invM r through a diagonal SpMV, i.e. D^-1 r with -0 -> +0),
// 3 JMR (:1079-1155)
// ---------------------------------------------------------------------------
template <int KIND>
__device__ __forceinline__ double mr_apply(const double *dinv, const double *sD, const double *r, int c)
{
    if (KIND == 0) return r[c];
    if (KIND == 1) return __dmul_rn(dinv[c], r[c]);
    if (KIND == 2) return __dadd_rn(__dmul_rn(dinv[c], r[c]), 0.0);
    return __dmul_rn(sD[c], r[c]);
}

template <int KIND>
__global__ void __launch_bounds__(kBlock) k_mr_spmv(const SolveArgs *__restrict__ a)
{
    DevState *st = a->st;
    CF_EXIT_IF_DONE(a, st, false);
    const int n = a->n, cap = a->stage_cap;
    CF_STAGE(double, cap);
    const double *r = a->r[0], *dinv = a->dinv, *sD = a->dinv_sqrt;
    double *y = a->w[0];
    auto g = [&](int c) { return mr_apply<KIND>(dinv, sD, r, c); };
    double acc[2] = {0.0, 0.0};
    CF_FOR_CHUNKS(base, n) {
        const RefRow R(a, base, cap, sv_, sc_);
        const int row = base + (threadIdx.x & 31);
        double v = R.product(g);
        if (row < n) {
            if (KIND == 3) v = __dmul_rn(sD[row], v);
            y[row] = v;
            acc[0] = fma_t(r[row], v, acc[0]);
            acc[1] = fma_t(v, v, acc[1]);
        }
        __syncwarp();
    }
    double tot[2];
    if (grid_reduce<2, double>(acc, a->partials, a->partial_stride, &st->counters[SLOT_A],
                               a->ref_order, tot) && threadIdx.x == 0)
        st->omega = tot[0] / tot[1];
}

template <int KIND>
__global__ void __launch_bounds__(kBlock) k_mr_update(const SolveArgs *__restrict__ a)
{
    DevState *st = a->st;
    CF_EXIT_IF_DONE(a, st, true);
    const int n = a->n;
    const double alpha = ld_cg(&st->omega);
    double *r = a->r[0], *x = a->x;
    const double *y = a->w[0], *dinv = a->dinv, *sD = a->dinv_sqrt;
    double acc[1] = {0.0};
    CF_FOR_ELEMS(i, n) {
        const double m = mr_apply<KIND>(dinv, sD, r, i);
        x[i] = fma_t(alpha, m, x[i]);
        const double ri = fma_t(-alpha, y[i], r[i]);
        r[i] = ri;
        acc[0] = fma_t(ri, ri, acc[0]);
    }
    double tot[1];
    if (grid_reduce<1, double>(acc, a->partials, a->partial_stride, &st->counters[SLOT_B],
                               a->ref_order, tot) && threadIdx.x == 0)
        finish_step(a, st, sqrt(tot[0]));
}

// ---------------------------------------------------------------------------
// host driver
// ---------------------------------------------------------------------------
static Kernels body_kernels(int solver, bool sell)
{
    Kernels k;
    switch (solver) {
    case CF_CG: k.k1 = (const void *)k_cg_spmv; k.k1_spmv = true; k.k2 = (const void *)k_cg_update; break;
    case CF_BICG: k.k1 = (const void *)k_bicg_spmv; k.k1_spmv = true; k.k2 = (const void *)k_bicg_update; break;
    case CF_JACOBI: k.k1 = (const void *)k_jacobi_step; k.k1_spmv = true; break;
    case CF_RICHARDSON: k.k1 = (const void *)k_rich_step; k.k1_spmv = true; break;
    case CF_MR: k.k1 = (const void *)k_mr_spmv<0>; k.k1_spmv = true; k.k2 = (const void *)k_mr_update<0>; break;
    case CF_MRJACOBI: k.k1 = (const void *)k_mr_spmv<1>; k.k1_spmv = true; k.k2 = (const void *)k_mr_update<1>; break;
    case CF_MRS: k.k1 = (const void *)k_mr_spmv<2>; k.k1_spmv = true; k.k2 = (const void *)k_mr_update<2>; break;
    case CF_JMR: k.k1 = (const void *)k_mr_spmv<3>; k.k1_spmv = true; k.k2 = (const void *)k_mr_update<3>; break;
    default: break;
    }
    // rows read from the SELL-32 copy stage nothing in shared memory
    if (sell) k.k1_spmv = false;
    return k;
}

static size_t vec_bytes(int n) { return sizeof(double) * ((size_t)n + 8); }

// Systems up to this many rows solve CG (fast order, FP64, no history) in one
// cluster-persistent launch instead of the multi-kernel loop: at 64^2 8.7 us
// per step against 16.7; from ~14k rows on (24^3: 17.4 against 17-20 us)
// the loop's full-GPU passes are as fast, and at 40^3 the single cluster is
// 2.5x slower.
#ifndef CF_SMALL_CG_ROWS
#define CF_SMALL_CG_ROWS 8192
#endif
constexpr int kSmallCgRows = CF_SMALL_CG_ROWS;

// normFactor alone (cf_norm_factor): b, x are device pointers.
double norm_factor(Matrix *m, const double *b, const double *x, int norm_type, bool ref)
{
    Context *ctx = m->ctx;
    require(m->n > 0, CF_BAD_INPUT, "empty matrix");
    const GridCap small(ctx, m->n);
    const int cap = stage_cap_for(m);
    const int stride = std::max(ctx->ref_grid, ctx->sm_count * 8);
    ctx->partials.ensure(sizeof(double) * kMaxNV * (size_t)stride);
    SolveArgs &A = *ctx->h_args;
    A = SolveArgs{};
    A.n = m->n;
    A.stage_cap = cap;
    A.ro = m->ro.as<int32_t>();
    A.col = m->col.as<int32_t>();
    A.val = m->val.as<double>();
    A.x = const_cast<double *>(x);
    A.b = b;
    const bool sell = matrix_ensure_sell(m, false, false);
    if (sell) {
        A.n_slices = m->n_slices;
        A.has_long = m->has_long ? 1 : 0;
        A.s_off = m->s_off.as<int32_t>();
        A.s_col = m->s_col.as<int32_t>();
        A.s_val = m->s_val.as<double>();
    }
    A.partials = ctx->partials.as<double>();
    A.partial_stride = stride;
    A.ref_order = ref ? 1 : 0;
    A.st = ctx->state.as<DevState>();
    DevState &S = *ctx->h_state;
    S = DevState{};
    S.tolerance = 1.0;
    SolveArgs *d_args = ctx->args.as<SolveArgs>();
    CF_CUDA(cudaMemcpyAsync(d_args, &A, sizeof(SolveArgs), cudaMemcpyHostToDevice, ctx->stream));
    CF_CUDA(cudaMemcpyAsync(A.st, &S, sizeof(DevState), cudaMemcpyHostToDevice, ctx->stream));
    void *args1[] = {&d_args};
    launch(ctx, ctx->stream, (const void *)k_nf_sum, launch_cfg(ctx, (const void *)k_nf_sum, false, cap, ref), args1);
    int l1 = norm_type == CF_NORM_OPENFOAM_L1 ? 1 : 0;
    void *a2[] = {&d_args, &l1};
    launch(ctx, ctx->stream, (const void *)k_nf_dist, launch_cfg(ctx, (const void *)k_nf_dist, !sell, cap, ref), a2);
    CF_CUDA(cudaMemcpyAsync(ctx->h_state, A.st, sizeof(DevState), cudaMemcpyDeviceToHost, ctx->stream));
    CF_CUDA(cudaStreamSynchronize(ctx->stream));
    return ctx->h_state->nf;
}

void solve(Matrix *m, int solver, const cf_controls &c, const double *b_in, double *x_io,
           cf_perf *perf)
{
    Context *ctx = m->ctx;
    require(solver >= CF_CG && solver <= CF_PCG, CF_BAD_INPUT, "unknown solver");
    require(b_in && x_io, CF_BAD_INPUT, "source and psi must not be null");
    require(c.memory == CF_MEM_HOST || c.memory == CF_MEM_DEVICE, CF_BAD_INPUT, "bad memory kind");
    require(c.reduction == CF_REDUCE_FAST || c.reduction == CF_REDUCE_REFERENCE ||
                c.reduction == CF_REDUCE_AUTO, CF_BAD_INPUT, "bad reduction");
    // AUTO: the reference order for BiCG, whose iterates follow the
    // summation order chaotically (see CF_REDUCE_AUTO), the fast one else
    const int reduction = c.reduction != CF_REDUCE_AUTO ? c.reduction
                          : (solver == CF_BICG ? CF_REDUCE_REFERENCE : CF_REDUCE_FAST);
    const int n = m->n;
    require(n > 0, CF_BAD_INPUT, "empty matrix");
    const GridCap small(ctx, n);
    const bool mixed = c.precision == CF_PREC_MIXED;
    require(c.precision == CF_PREC_FP64 || mixed, CF_BAD_INPUT, "bad precision");
    require(!mixed || mixed_supported(solver), CF_UNSUPPORTED,
            "mixed precision is implemented for CG, BiCG, MR, MRJacobi, MRS and JMR");
    require(solver != CF_PCG || (!mixed && c.transpose == 0), CF_UNSUPPORTED,
            "the preconditioned CG is FP64 only");
    require(solver != CF_PCG || reduction == CF_REDUCE_FAST, CF_UNSUPPORTED,
            "the preconditioned CG has no reference summation order (no reference counterpart)");
    const bool ref = reduction == CF_REDUCE_REFERENCE && !mixed;
    const int cap = stage_cap_for(m);
    const bool tr = c.transpose != 0;
    if (solver == CF_BICG || tr) matrix_ensure_transpose(m);
    if (solver == CF_RICHARDSON) matrix_ensure_dmin(m);
    // both orders read the SELL-32 copy when the pattern suits it (FP32
    // values too for the mixed inner solve); the reference order takes its
    // 8-lane row sums from the SELL slots (RefRow), the same bits as from CSR
    // (the mixed MR family's FP32 values are a scaled matrix, made per solve)
    const bool fp32_copy = mixed && (solver == CF_CG || solver == CF_BICG || solver == CF_MR);
    const bool sell = matrix_ensure_sell(m, solver == CF_BICG || tr, fp32_copy);

    // ---- vectors -------------------------------------------------------
    double *x, *b;
    if (c.memory == CF_MEM_HOST) {
        ctx->vec[0].ensure(vec_bytes(n));
        ctx->vec[1].ensure(vec_bytes(n));
        x = ctx->vec[0].as<double>();
        b = ctx->vec[1].as<double>();
        upload(ctx, x, x_io, sizeof(double) * n, CF_MEM_HOST);
        upload(ctx, b, b_in, sizeof(double) * n, CF_MEM_HOST);
    } else {
        x = x_io;
        b = const_cast<double *>(b_in);
    }
    for (int i = 2; i < 14; ++i) ctx->vec[i].ensure(vec_bytes(n));
    const int stride = std::max(ctx->ref_grid, ctx->sm_count * 8);
    ctx->partials.ensure(sizeof(double) * kMaxNV * (size_t)stride);
    const bool want_hist = c.history && c.history_capacity > 0;
    const int hist_cap = want_hist ? c.history_capacity : 0;
    if (want_hist) ctx->hist.ensure(sizeof(double) * (size_t)hist_cap);
    const bool hist_time = want_hist && c.history_time != 0;
    if (hist_time) ctx->hist_t.ensure(sizeof(unsigned long long) * (size_t)hist_cap);

    // ---- a small system: one cluster-persistent launch -----------------
    // (kernel boundaries, not bytes, set a small system's step time; CG runs
    // in the batched kernel, Jacobi, Richardson and the MR family in
    // k_small_solve, the whole solve behind hardware cluster barriers)
    const bool small_kind = solver == CF_CG || solver == CF_JACOBI || solver == CF_RICHARDSON ||
                            solver == CF_MR || solver == CF_MRJACOBI || solver == CF_MRS || solver == CF_JMR;
    if (small_kind && !ref && !mixed && !tr && n <= kSmallCgRows && !want_hist &&
        c.time_limit_s <= 0 && c.profile_kernels == 0 && c.rel_tol == 0 && c.min_iter <= 0 &&
        c.norm_type == CF_NORM_REFERENCE_L2 && !c.absolute_tolerance && c.use_graph != 0 && small_cg_ok(ctx)) {
        const SmallSolveResult R =
            solver == CF_CG
                ? solve_cg_single_cluster(m, c, b, x, ctx->vec[2].as<double>(), ctx->vec[4].as<double>(),
                                          ctx->vec[6].as<double>())
                : solve_small_single_cluster(m, solver, c, b, x, ctx->vec[2].as<double>(),
                                             ctx->vec[4].as<double>(), ctx->vec[6].as<double>());
        if (c.memory == CF_MEM_HOST) download(ctx, x_io, x, sizeof(double) * n, CF_MEM_HOST);
        CF_CUDA(cudaStreamSynchronize(ctx->stream));
        if (perf) {
            *perf = cf_perf{};
            perf->norm_factor = R.nf;
            perf->initial_residual_abs = R.norm0;
            perf->final_residual_abs = R.norm;
            perf->initial_residual = R.norm0 / R.nf;
            perf->final_residual = R.norm / R.nf;
            perf->n_iterations = R.iters;
            perf->status = R.status;
            perf->solve_ms = R.ms;
            perf->true_residual = -1.0;
            perf->omega = R.omega;
        }
        return;
    }

    SolveArgs &A = *ctx->h_args;
    A = SolveArgs{};
    A.n = n;
    A.stage_cap = cap;
    A.ro = m->ro.as<int32_t>();
    A.col = m->col.as<int32_t>();
    A.val = m->val.as<double>();
    A.valT = m->have_valT ? m->valT.as<double>() : nullptr;
    if (sell) {
        A.n_slices = m->n_slices;
        A.has_long = m->has_long ? 1 : 0;
        A.s_off = m->s_off.as<int32_t>();
        A.s_col = m->s_col.as<int32_t>();
        A.s_val = m->s_val.as<double>();
        A.s_valT = m->have_svalT ? m->s_valT.as<double>() : nullptr;
        // one-byte column codes (or 16-bit column deltas): read by the FP32
        // sweeps, and by the FP64 fast passes when asked for
        // (CF_FORMAT_SELL_C8, CF_FORMAT_SELL_D16).  Those passes are
        // bound by FP64 issue on GB300 (8 FP64 instructions per row of the CG
        // SpMV), so saving bytes does not shorten them (128^3 CG step 71.2 us
        // either way); the FP32 MR step at 256^3 drops from 237 to 214 us.
        if (m->n_codes > 0 && !ref && (mixed || m->format_request == CF_FORMAT_SELL_C8)) {
            A.s_code = m->s_code.as<uint8_t>();
            A.s_dtab = m->s_dtab.as<int32_t>();
        } else if (m->has_d16 && !ref && (mixed || m->format_request == CF_FORMAT_SELL_D16)) {
            A.s_d16 = m->s_d16.as<int16_t>();   // 16-bit column deltas, read by the same passes
        }
    }
    if (tr) {
        std::swap(A.val, A.valT); // A^T on the same pattern; its transpose is A
        std::swap(A.s_val, A.s_valT);
    }
    A.diag = m->diag.as<double>();
    A.dinv = m->dinv.as<double>();
    A.dinv_sqrt = m->dinv_sqrt.as<double>();
    A.x = x;
    A.b = b;
    A.r[0] = ctx->vec[2].as<double>();
    A.r[1] = ctx->vec[3].as<double>();
    A.p[0] = ctx->vec[4].as<double>();
    A.p[1] = ctx->vec[5].as<double>();
    A.q = ctx->vec[6].as<double>();
    A.rs = ctx->vec[7].as<double>();
    A.ps[0] = ctx->vec[8].as<double>();
    A.ps[1] = ctx->vec[9].as<double>();
    A.qs = ctx->vec[10].as<double>();
    A.w[0] = ctx->vec[11].as<double>();
    A.w[1] = ctx->vec[12].as<double>();
    A.partials = ctx->partials.as<double>();
    A.partial_stride = stride;
    A.ref_order = ref ? 1 : 0;
    A.st = ctx->state.as<DevState>();
    A.hist = want_hist ? ctx->hist.as<double>() : nullptr;
    A.hist_t = hist_time ? ctx->hist_t.as<unsigned long long>() : nullptr;
    A.power_steps = c.power_max_steps;
    A.abort_flag = (c.time_limit_s > 0) ? ctx->d_abort : nullptr;

    if (mixed) mixed_prepare(ctx, m, solver, A);
    // fast order: JMR runs as MR on the scaled matrix D^-1/2 A D^-1/2,
    // Jacobi as one pass over A D^-1 (MRJacobi and MRS gather z = D^-1 r)
    if (!ref && !mixed && (solver == CF_JMR || solver == CF_JACOBI))
        A.sc_val = scaled_values<double>(ctx, m, A, solver, tr, m->sc64, &A.corr_scale);

    DevState &S = *ctx->h_state;
    S = DevState{};
    S.tolerance = c.tolerance;
    S.rel_tol = c.rel_tol;
    S.max_steps = c.max_iter <= 0 ? INT_MAX : c.max_iter;
    S.min_steps = c.min_iter > 0 ? c.min_iter : 0;
    S.int_bound = c.bicg_int_bound;
    S.hist_cap = hist_cap;
    S.diag_abs_min = m->diag_abs_min;
    S.omega = c.richardson_omega;
    S.flags = c.absolute_tolerance ? kFlagAbsTol : 0;

    const bool prof = c.profile_kernels != 0;
    bool use_graph = c.use_graph != 0 && ctx->graphs_ok && !prof;
    GraphEntry *ge = nullptr;
    const int fmt = solve_format(A);
    const Kernels kk = ref ? body_kernels(solver, sell) : fast_body_kernels(solver, fmt);
    SolveArgs *d_args = ctx->args.as<SolveArgs>();
    if (use_graph && !mixed) {
        try {
            ge = loop_graph(ctx, kk, solver, CF_PREC_FP64, cap, ref, d_args, fmt);
        } catch (const Error &) {
            ctx->graphs_ok = false; // fall back to host-driven launches
            use_graph = false;
        }
    }
    A.use_cond = (use_graph && !mixed) ? 1 : 0;
    A.cond = (use_graph && !mixed) ? ge->cond : 0;
    *ctx->h_abort = 0;
    CF_CUDA(cudaMemcpyAsync(d_args, &A, sizeof(SolveArgs), cudaMemcpyHostToDevice, ctx->stream));
    CF_CUDA(cudaMemcpyAsync(A.st, &S, sizeof(DevState), cudaMemcpyHostToDevice, ctx->stream));

    void *args1[] = {&d_args};
    CF_CUDA(cudaEventRecord(ctx->ev_start, ctx->stream));
    // ---- normFactor -> tolerance * normFactor --------------------------
    {
        launch(ctx, ctx->stream, (const void *)k_nf_sum,
               launch_cfg(ctx, (const void *)k_nf_sum, false, cap, ref), args1);
        int l1 = (c.norm_type == CF_NORM_OPENFOAM_L1) ? 1 : 0;
        void *a2[] = {&d_args, &l1};
        launch(ctx, ctx->stream, (const void *)k_nf_dist,
               launch_cfg(ctx, (const void *)k_nf_dist, !sell, cap, ref), a2);
    }
    // ---- Richardson relaxation factor -----------------------------------
    if (solver == CF_RICHARDSON && !mixed) {
        const double om = c.richardson_omega;
        if (-1e-15 < om && om < 1e-15) {
            int steps = c.power_max_steps;
            for (int s = 0; s < steps; ++s) {
                void *a2[] = {&d_args, &s};
                launch(ctx, ctx->stream, (const void *)k_pow_step,
                       launch_cfg(ctx, (const void *)k_pow_step, !sell, cap, ref), a2);
            }
            void *a3[] = {&d_args, &steps};
            launch(ctx, ctx->stream, (const void *)k_pow_final,
                   launch_cfg(ctx, (const void *)k_pow_final, !sell, cap, ref), a3);
        }
    }
    // ---- initial residual ----------------------------------------------
    {
        // (the mixed JMR loop keeps the scaled residual as well)
        int mode = solver == CF_JMR ? 1 : mixed ? 0 : (solver == CF_BICG ? 2 : (solver == CF_PCG ? 3 : 0));
        if (!ref && !mixed && (solver == CF_MRJACOBI || solver == CF_MRS)) mode = 4;
        void *a2[] = {&d_args, &mode};
        launch(ctx, ctx->stream, (const void *)k_res_init,
               launch_cfg(ctx, (const void *)k_res_init, !sell, cap, ref), a2);
    }
    // ---- iterations: device-driven while loop, or host-driven chunks ----
    CF_CUDA(cudaEventRecord(ctx->ev_mid, ctx->stream));
    auto wall0 = std::chrono::steady_clock::now();
    double kms[3] = {0.0, 0.0, 0.0};
    int klaunch[3] = {0, 0, 0};
    MixedResult mres;
    if (mixed) {
        mres = run_mixed(ctx, m, solver, c, d_args, cap, use_graph);
    } else if (use_graph) {
        CF_CUDA(cudaGraphLaunch(ge->exec, ctx->stream));
    } else {
        const int chunk = 16;
        const Launch l0 = kk.k0 ? launch_cfg(ctx, kk.k0, false, cap, ref) : Launch{};
        const Launch l1 = launch_cfg(ctx, kk.k1, kk.k1_spmv, cap, ref);
        const Launch l2 = kk.k2 ? launch_cfg(ctx, kk.k2, kk.k2_spmv, cap, ref) : Launch{};
        if (prof) {
            while (ctx->prof_events.size() < 4 * chunk) {
                cudaEvent_t e;
                CF_CUDA(cudaEventCreate(&e));
                ctx->prof_events.push_back(e);
            }
        }
        int k_before = 0;
        for (;;) {
            for (int i = 0; i < chunk; ++i) {
                cudaEvent_t *ev = prof ? &ctx->prof_events[4 * i] : nullptr;
                if (prof) CF_CUDA(cudaEventRecord(ev[0], ctx->stream));
                if (kk.k0) launch(ctx, ctx->stream, kk.k0, l0, args1, !prof);
                if (prof) CF_CUDA(cudaEventRecord(ev[1], ctx->stream));
                launch(ctx, ctx->stream, kk.k1, l1, args1, !prof);
                if (prof) CF_CUDA(cudaEventRecord(ev[2], ctx->stream));
                if (kk.k2) launch(ctx, ctx->stream, kk.k2, l2, args1, !prof);
                if (prof) CF_CUDA(cudaEventRecord(ev[3], ctx->stream));
            }
            CF_CUDA(cudaMemcpyAsync(ctx->h_state, A.st, sizeof(DevState), cudaMemcpyDeviceToHost,
                                    ctx->stream));
            CF_CUDA(cudaStreamSynchronize(ctx->stream));
            const int k_now = ctx->h_state->k;
            if (prof) {
                for (int i = 0; i < chunk; ++i) {
                    if (k_before + i + 1 > k_now) break; // launches after the loop ended
                    cudaEvent_t *ev = &ctx->prof_events[4 * i];
                    float t = 0.f;
                    if (kk.k0) {
                        CF_CUDA(cudaEventElapsedTime(&t, ev[0], ev[1]));
                        kms[2] += t;
                        klaunch[2] += 1;
                    }
                    CF_CUDA(cudaEventElapsedTime(&t, ev[1], ev[2]));
                    kms[0] += t;
                    klaunch[0] += 1;
                    if (kk.k2) {
                        CF_CUDA(cudaEventElapsedTime(&t, ev[2], ev[3]));
                        kms[1] += t;
                        klaunch[1] += 1;
                    }
                }
            }
            k_before = k_now;
            if (ctx->h_state->done) break;
            if (c.time_limit_s > 0) {
                const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - wall0).count();
                if (el > c.time_limit_s) *ctx->h_abort = 1;
            }
        }
    }
    // ---- deferred updates ------------------------------------------------
    if ((solver == CF_CG || solver == CF_BICG || solver == CF_PCG) && !mixed) {
        const void *flush = ref ? (const void *)k_flush_x : fast_flush_kernel();
        launch(ctx, ctx->stream, flush, launch_cfg(ctx, flush, false, cap, false), args1);
        k_clear_pending<<<1, 32, 0, ctx->stream>>>(A.st);
        CF_CHECK_LAUNCH();
    }
    if (solver == CF_RICHARDSON && !mixed && ref) {
        launch(ctx, ctx->stream, (const void *)k_rich_finish,
               launch_cfg(ctx, (const void *)k_rich_finish, false, cap, false), args1);
    }
    CF_CUDA(cudaEventRecord(ctx->ev_stop, ctx->stream));
    CF_CUDA(cudaMemcpyAsync(ctx->h_state, A.st, sizeof(DevState), cudaMemcpyDeviceToHost, ctx->stream));
    if (c.time_limit_s > 0 && use_graph) {
        while (cudaEventQuery(ctx->ev_stop) == cudaErrorNotReady) {
            const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - wall0).count();
            if (el > c.time_limit_s) *ctx->h_abort = 1;
            std::this_thread::sleep_for(std::chrono::microseconds(200));
        }
    }
    CF_CUDA(cudaStreamSynchronize(ctx->stream));
    const DevState R = *ctx->h_state;
    if (c.memory == CF_MEM_HOST) {
        download(ctx, x_io, x, sizeof(double) * n, CF_MEM_HOST);
    }
    int hist_len = 0;
    if (want_hist) {
        hist_len = std::min(R.k + 1, hist_cap);
        if (hist_time) {
            std::vector<unsigned long long> t((size_t)hist_len);
            download(ctx, t.data(), A.hist_t, sizeof(unsigned long long) * (size_t)hist_len, CF_MEM_HOST);
            CF_CUDA(cudaStreamSynchronize(ctx->stream));
            for (int i = 0; i < hist_len; ++i) c.history[i] = 1e-9 * (double)(t[(size_t)i] - t[0]);
        } else {
            download(ctx, c.history, A.hist, sizeof(double) * (size_t)hist_len, CF_MEM_HOST);
        }
    }
    CF_CUDA(cudaStreamSynchronize(ctx->stream));
    float ms = 0.f;
    CF_CUDA(cudaEventElapsedTime(&ms, ctx->ev_start, ctx->ev_stop));
    if (perf) {
        *perf = cf_perf{};
        perf->norm_factor = R.nf;
        perf->initial_residual_abs = R.norm0;
        perf->final_residual_abs = R.norm;
        perf->initial_residual = R.norm0 / R.nf;
        perf->final_residual = R.norm / R.nf;
        perf->omega = (solver == CF_RICHARDSON) ? R.omega : 0.0;
        perf->n_iterations = mixed ? mres.inner_iterations : R.k;
        perf->n_outer = mixed ? mres.outer : 0;
        perf->status = mixed ? mres.status : R.status;
        perf->history_length = hist_len;
        perf->solve_ms = ms;
        perf->true_residual = -1.0;
        if (prof) {
            float setup = 0.f;
            CF_CUDA(cudaEventElapsedTime(&setup, ctx->ev_start, ctx->ev_mid));
            perf->kernel_ms[0] = kms[0];
            perf->kernel_ms[1] = kms[1];
            perf->kernel_ms[2] = kms[2];
            perf->kernel_ms[3] = setup;
            perf->kernel_launches[0] = klaunch[0];
            perf->kernel_launches[1] = klaunch[1];
            perf->kernel_launches[2] = klaunch[2];
            perf->kernel_launches[3] = 1;
        }
    }
}

} // namespace cf
