// solve_fast.cu -- the default (fast) FP64 iteration kernels.
//
// GB300 executes FP64 at 2 FMA per cycle per SM (ncu:
// sm__sass_thread_inst_executed_op_dfma peak), so a fused kernel that forms
// the SpMV input on the fly (one FP64 op per matrix entry) and sums rows in
// the reference's 8-lane tree (seven more adds per row) runs out of FP64
// issue slots before HBM bandwidth.  These kernels keep the reference's
// operations per vector element but
//   * sum each row as one FMA chain (one FP64 instruction per entry),
//   * form the SpMV input vector once per element in a light element-wise
//     pass ("prep") instead of once per matrix entry,
// which costs a few bytes per row and halves the FP64 work: CG needs 12
// FP64 ops per row and iteration instead of 26.  Dot products use the
// deterministic fast reduction order.  The loop structure, stopping tests
// and scalars are those of the reference drivers (SolverSingleGPU.h).
#include "solver_common.cuh"

#include <algorithm>

namespace cf {

// ---------------------------------------------------------------------------
// CG (SolverSingleGPU.h:366-445) in three passes:
//   prep:   x += xi_{k-1} p_{k-1} (deferred);  p_k = r + beta p_{k-1}  (p_1 = r)
//   spmv:   q = A p_k, (p_k, q) -> xi_k
//   update: r -= xi_k q, (r, r) -> stopping test, beta
// ---------------------------------------------------------------------------
// Element-wise passes process four elements per thread per step, loading
// all inputs before any store, so each thread keeps several independent
// loads in flight.
#define CF_X4_LOOP(i, n)                                                   \
    const int stride_ = gridDim.x * kBlock;                                \
    int i = blockIdx.x * kBlock + threadIdx.x;                             \
    for (; i + 3 * stride_ < (n); i += 4 * stride_)
#define CF_X4_IDX(i, u) ((i) + (u) * stride_)
#define CF_X4_TAIL(i, n) for (; i < (n); i += stride_)

__global__ void __launch_bounds__(kBlock) k_f_cg_prep(const SolveArgs *__restrict__ a)
{
    DevState *st = a->st;
    const int n = a->n;
    double *__restrict__ p = a->p[0];
    const double *__restrict__ r = a->r[0];
    double *__restrict__ x = a->x;
    const bool pairs = (((uintptr_t)x | (uintptr_t)p | (uintptr_t)r) & 15) == 0;
    const int np = n >> 1;
    const int stride = gridDim.x * kBlock;
    int j = blockIdx.x * kBlock + threadIdx.x;
    double2 *__restrict__ x2 = reinterpret_cast<double2 *>(x);
    double2 *__restrict__ p2 = reinterpret_cast<double2 *>(p);
    // p and x were last written by the previous step's prep, which completed
    // before the update this launch follows could start: the first pair is
    // loaded before the wait for the update (r, written by it, after)
    double2 pv = make_double2(0.0, 0.0), xv = pv, rv = pv;
    if (pairs && j < np) {
        pv = p2[j];
        xv = x2[j];
    }
    CF_EXIT_IF_DONE(a, st, false);
    const int k = ld_cg(&st->k) + 1;
    if (k == 1) {
        CF_FOR_ELEMS(i, n) p[i] = r[i];
        return;
    }
    const double beta = ld_cg(&st->beta);
    const double xi = ld_cg(&st->xi);
    if (pairs) {
        // element pairs as 16-byte loads; each thread loads its next pair
        // before computing the current one, so the FP64 work of one pair
        // overlaps the loads of the next (measured 12.4 -> 10.4 us at 128^3
        // with L2-resident vectors)
        const double2 *__restrict__ r2 = reinterpret_cast<const double2 *>(r);
        if (j < np) rv = r2[j];
        for (; j < np; j += stride) {
            const int jn = j + stride;
            double2 pn = make_double2(0.0, 0.0), xn = pn, rn = pn;
            if (jn < np) {
                pn = p2[jn];
                xn = x2[jn];
                rn = r2[jn];
            }
            x2[j] = make_double2(fma_t(xi, pv.x, xv.x), fma_t(xi, pv.y, xv.y));
            p2[j] = make_double2(fma_t(beta, pv.x, rv.x), fma_t(beta, pv.y, rv.y));
            pv = pn;
            xv = xn;
            rv = rn;
        }
        if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) {
            const int i = n - 1;
            const double pi = p[i];
            x[i] = fma_t(xi, pi, x[i]);
            p[i] = fma_t(beta, pi, r[i]);
        }
        return;
    }
    CF_X4_LOOP(i, n) {
        double pv[4], xv[4], rv[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            pv[u] = p[CF_X4_IDX(i, u)];
            xv[u] = x[CF_X4_IDX(i, u)];
            rv[u] = r[CF_X4_IDX(i, u)];
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            x[CF_X4_IDX(i, u)] = fma_t(xi, pv[u], xv[u]);
            p[CF_X4_IDX(i, u)] = fma_t(beta, pv[u], rv[u]);
        }
    }
    CF_X4_TAIL(i, n) {
        const double pi = p[i];
        x[i] = fma_t(xi, pi, x[i]);
        p[i] = fma_t(beta, pi, r[i]);
    }
}

template <int FMT>
__global__ void __launch_bounds__(kBlock, CF_SPMV_MIN_BLOCKS) k_f_cg_spmv(const SolveArgs *__restrict__ a)
{
    DevState *st = a->st;
    sell_prefetch<FMT>(a, a->s_val);
    CF_EXIT_IF_DONE(a, st, false);
    const double *__restrict__ p = a->p[0];
    double *__restrict__ q = a->q;
    double acc[1] = {0.0};
    for_rows<FMT, double>(a, a->val, a->s_val, [&](int c) { return p[c]; }, [&](int row, double y) {
        q[row] = y;
        acc[0] = fma_t(p[row], y, acc[0]);
    });
    double tot[1];
    if (grid_reduce<1, double>(acc, a->partials, a->partial_stride, &st->counters[SLOT_A], false, tot) &&
        threadIdx.x == 0) {
        st->xi = st->rho0 / tot[0];
        st->x_pending = 0;
    }
}

// resident blocks per SM asked of nvcc for the update pass (five: 71.95 us
// per 128^3 CG step against 72.8 us with six)
#ifndef CF_CG_UPDATE_MIN_BLOCKS
#define CF_CG_UPDATE_MIN_BLOCKS 5
#endif

// r -= xi q, (r, r)
__global__ void __launch_bounds__(kBlock, CF_CG_UPDATE_MIN_BLOCKS) k_f_cg_update(const SolveArgs *__restrict__ a)
{
    DevState *st = a->st;
    const int n = a->n;
    double *__restrict__ r = a->r[0];
    const double *__restrict__ q = a->q;
    const int stride = gridDim.x * kBlock;
    int i = blockIdx.x * kBlock + threadIdx.x;
    // r was last written by the previous step's update, which completed
    // before the SpMV this launch follows could start: its first loads are
    // issued before the wait for the SpMV, and each step loads the next r
    // group before its FP64 work
    double rv[4];
    if (i + 3 * stride < n) {
#pragma unroll
        for (int u = 0; u < 4; ++u) rv[u] = r[i + u * stride];
    }
    CF_EXIT_IF_DONE(a, st, true);
    const double xi = ld_cg(&st->xi);
    // one accumulator: the FP64 unit, not the FMA latency, limits this pass
    // on GB300, and combining four partials cost 12% more FP64 instructions
    double acc[1] = {0.0};
    for (; i + 3 * stride < n; i += 4 * stride) {
        double qv[4], rn[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) qv[u] = q[i + u * stride];
        const int in = i + 4 * stride;
        if (in + 3 * stride < n) {
#pragma unroll
            for (int u = 0; u < 4; ++u) rn[u] = r[in + u * stride];
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const double ri = fma_t(-xi, qv[u], rv[u]);
            r[i + u * stride] = ri;
            acc[0] = fma_t(ri, ri, acc[0]);
            rv[u] = rn[u];
        }
    }
    for (; i < n; i += stride) {
        const double ri = fma_t(-xi, q[i], r[i]);
        r[i] = ri;
        acc[0] = fma_t(ri, ri, acc[0]);
    }
    double tot[1];
    if (grid_reduce<1, double>(acc, a->partials, a->partial_stride, &st->counters[SLOT_B], false, tot) &&
        threadIdx.x == 0) {
        st->rho1 = st->rho0;
        st->rho0 = tot[0];
        st->beta = st->rho0 / st->rho1;
        st->x_pending = 1;
        finish_step(a, st, sqrt(tot[0]));
    }
}

__global__ void __launch_bounds__(kBlock) k_f_flush_x(const SolveArgs *__restrict__ a)
{
    DevState *st = a->st;
    if (!ld_cg(&st->x_pending)) return;
    const int n = a->n;
    const double xi = ld_cg(&st->xi);
    const double *p = a->p[0];
    double *x = a->x;
    CF_FOR_ELEMS(i, n) x[i] = fma_t(xi, p[i], x[i]);
}

// ---------------------------------------------------------------------------
// Jacobi-preconditioned CG (no reference counterpart): CG on the same three
// passes with z = D^-1 r formed where it is used --
//   prep:   x += xi_{k-1} p_{k-1} (deferred);  p_k = z + beta p_{k-1}
//   spmv:   k_f_cg_spmv (q = A p_k, (p_k, q) -> xi_k = (r, z) / (p, q))
//   update: r -= xi_k q, (r, r) for the stopping test, (r, z) -> beta
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kBlock) k_f_pcg_prep(const SolveArgs *__restrict__ a)
{
    DevState *st = a->st;
    CF_EXIT_IF_DONE(a, st, false);
    const int n = a->n;
    const int k = ld_cg(&st->k) + 1;
    double *__restrict__ p = a->p[0];
    const double *__restrict__ r = a->r[0];
    const double *__restrict__ dinv = a->dinv;
    double *__restrict__ x = a->x;
    if (k == 1) {
        CF_FOR_ELEMS(i, n) p[i] = __dmul_rn(dinv[i], r[i]);
        return;
    }
    const double beta = ld_cg(&st->beta);
    const double xi = ld_cg(&st->xi);
    CF_X4_LOOP(i, n) {
        double pv[4], xv[4], rv[4], dv[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            pv[u] = p[CF_X4_IDX(i, u)];
            xv[u] = x[CF_X4_IDX(i, u)];
            rv[u] = r[CF_X4_IDX(i, u)];
            dv[u] = dinv[CF_X4_IDX(i, u)];
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            x[CF_X4_IDX(i, u)] = fma_t(xi, pv[u], xv[u]);
            p[CF_X4_IDX(i, u)] = fma_t(beta, pv[u], __dmul_rn(dv[u], rv[u]));
        }
    }
    CF_X4_TAIL(i, n) {
        const double pi = p[i];
        x[i] = fma_t(xi, pi, x[i]);
        p[i] = fma_t(beta, pi, __dmul_rn(dinv[i], r[i]));
    }
}

__global__ void __launch_bounds__(kBlock) k_f_pcg_update(const SolveArgs *__restrict__ a)
{
    DevState *st = a->st;
    CF_EXIT_IF_DONE(a, st, true);
    const int n = a->n;
    const double xi = ld_cg(&st->xi);
    double *__restrict__ r = a->r[0];
    const double *__restrict__ q = a->q;
    const double *__restrict__ dinv = a->dinv;
    double rr[4] = {0.0, 0.0, 0.0, 0.0}, rz[4] = {0.0, 0.0, 0.0, 0.0};
    CF_X4_LOOP(i, n) {
        double qv[4], rv[4], dv[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            qv[u] = q[CF_X4_IDX(i, u)];
            rv[u] = r[CF_X4_IDX(i, u)];
            dv[u] = dinv[CF_X4_IDX(i, u)];
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const double ri = fma_t(-xi, qv[u], rv[u]);
            r[CF_X4_IDX(i, u)] = ri;
            rr[u] = fma_t(ri, ri, rr[u]);
            rz[u] = fma_t(ri, __dmul_rn(dv[u], ri), rz[u]);
        }
    }
    CF_X4_TAIL(i, n) {
        const double ri = fma_t(-xi, q[i], r[i]);
        r[i] = ri;
        rr[0] = fma_t(ri, ri, rr[0]);
        rz[0] = fma_t(ri, __dmul_rn(dinv[i], ri), rz[0]);
    }
    double acc[2] = {(rr[0] + rr[1]) + (rr[2] + rr[3]), (rz[0] + rz[1]) + (rz[2] + rz[3])};
    double tot[2];
    if (grid_reduce<2, double>(acc, a->partials, a->partial_stride, &st->counters[SLOT_B], false, tot) &&
        threadIdx.x == 0) {
        st->rho1 = st->rho0;
        st->rho0 = tot[1];
        st->beta = st->rho0 / st->rho1;
        st->x_pending = 1;
        finish_step(a, st, sqrt(tot[0]));
    }
}

// ---------------------------------------------------------------------------
// BiCG with A^T (SolverSingleGPU.h:568-675):
//   prep:   x += xi p (deferred); p = r + theta p; p* = r* + theta p*
//   spmv:   q = A p, q* = A^T p* (one pass over the shared pattern),
//           (p*, q) -> xi, breakdown test
//   update: k_bicg_update (r, r* updates, ||r||, (r, r*), theta)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kBlock) k_f_bicg_prep(const SolveArgs *__restrict__ a)
{
    DevState *st = a->st;
    CF_EXIT_IF_DONE(a, st, false);
    const int n = a->n;
    const int k = ld_cg(&st->k) + 1;
    double *__restrict__ p = a->p[0];
    double *__restrict__ ps = a->ps[0];
    const double *__restrict__ r = a->r[0];
    const double *__restrict__ rs = a->rs;
    double *__restrict__ x = a->x;
    if (k == 1) {
        CF_FOR_ELEMS(i, n) {
            p[i] = r[i];
            ps[i] = rs[i];
        }
        return;
    }
    const double theta = ld_cg(&st->theta);
    const double xi = ld_cg(&st->xi);
    const bool xpend = ld_cg(&st->x_pending) != 0;
    CF_X4_LOOP(i, n) {
        double pv[4], rv[4], psv[4], rsv[4], xv[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            pv[u] = p[CF_X4_IDX(i, u)];
            rv[u] = r[CF_X4_IDX(i, u)];
            psv[u] = ps[CF_X4_IDX(i, u)];
            rsv[u] = rs[CF_X4_IDX(i, u)];
            xv[u] = xpend ? x[CF_X4_IDX(i, u)] : 0.0;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            if (xpend) x[CF_X4_IDX(i, u)] = fma_t(xi, pv[u], xv[u]);
            p[CF_X4_IDX(i, u)] = fma_t(theta, pv[u], rv[u]);
            ps[CF_X4_IDX(i, u)] = fma_t(theta, psv[u], rsv[u]);
        }
    }
    CF_X4_TAIL(i, n) {
        const double pi = p[i];
        if (xpend) x[i] = fma_t(xi, pi, x[i]);
        p[i] = fma_t(theta, pi, r[i]);
        ps[i] = fma_t(theta, ps[i], rs[i]);
    }
}

template <int FMT>
__global__ void __launch_bounds__(kBlock, CF_BICG_SPMV_MIN_BLOCKS) k_f_bicg_spmv(const SolveArgs *__restrict__ a)
{
    DevState *st = a->st;
    sell_prefetch<FMT>(a, a->s_val);
    sell_prefetch<FMT>(a, a->s_valT);
    CF_EXIT_IF_DONE(a, st, false);
    const double *__restrict__ p = a->p[0];
    const double *__restrict__ ps = a->ps[0];
    double *__restrict__ q = a->q;
    double *__restrict__ qs = a->qs;
    double acc[1] = {0.0};
    for_rows2<FMT, double>(a, a->val, a->valT, a->s_val, a->s_valT, [&](int c) { return p[c]; },
                   [&](int c) { return ps[c]; }, [&](int row, double y1, double y2) {
                       q[row] = y1;
                       qs[row] = y2;
                       acc[0] = fma_t(ps[row], y1, acc[0]);
                   });
    double tot[1];
    if (grid_reduce<1, double>(acc, a->partials, a->partial_stride, &st->counters[SLOT_A], false, tot) &&
        threadIdx.x == 0) {
        const double xi = st->rho0 / tot[0];
        st->x_pending = 0;
        const double bound = st->int_bound;
        if (xi > -bound && xi < bound) {
            st->done = 1;
            st->status = CF_BREAKDOWN;
        } else {
            st->xi = xi;
        }
    }
}

// ---------------------------------------------------------------------------
// Jacobi (SolverSingleGPU.h:924-994): x += D^-1 r, r -= A D^-1 r, ||r||.
// One pass per step over the scaled matrix A D^-1 (a->sc_val, cached on the
// matrix): the residual alternates between r[0] and r[1] (step k reads
// r[(k + 1) & 1], writes r[k & 1]), so every row gathers the old residual
// while its own row writes the new one; x += D^-1 r is row-local.
// ---------------------------------------------------------------------------
template <int FMT>
__global__ void __launch_bounds__(kBlock, CF_SPMV_MIN_BLOCKS) k_f_jac_step(const SolveArgs *__restrict__ a)
{
    DevState *st = a->st;
    sell_prefetch<FMT>(a, a->sc_val);
    CF_EXIT_IF_DONE(a, st, true);
    const int k = ld_cg(&st->k) + 1;
    const double *__restrict__ rin = a->r[(k + 1) & 1];
    double *__restrict__ rout = a->r[k & 1];
    const double *__restrict__ dinv = a->dinv;
    double *__restrict__ x = a->x;
    double acc[1] = {0.0};
    for_rows<FMT, double>(a, a->sc_val, a->sc_val, [&](int c) { return rin[c]; }, [&](int row, double y) {
        const double r0 = rin[row];
        x[row] = fma_t(1.0, __dmul_rn(dinv[row], r0), x[row]);
        const double ri = fma_t(-1.0, y, r0);
        rout[row] = ri;
        acc[0] = fma_t(ri, ri, acc[0]);
    });
    double tot[1];
    if (grid_reduce<1, double>(acc, a->partials, a->partial_stride, &st->counters[SLOT_A], false, tot) &&
        threadIdx.x == 0)
        finish_step(a, st, sqrt(tot[0]));
}

// ---------------------------------------------------------------------------
// Richardson (SolverSingleGPU.h:762-819): prep x += omega r; spmv r = b - A x
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kBlock) k_f_rich_prep(const SolveArgs *__restrict__ a)
{
    DevState *st = a->st;
    CF_EXIT_IF_DONE(a, st, false);
    const int n = a->n;
    const double omega = ld_cg(&st->omega);
    const double *__restrict__ r = a->r[0];
    double *__restrict__ x = a->x;
    CF_X4_LOOP(i, n) {
        double rv[4], xv[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            rv[u] = r[CF_X4_IDX(i, u)];
            xv[u] = x[CF_X4_IDX(i, u)];
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) x[CF_X4_IDX(i, u)] = fma_t(omega, rv[u], xv[u]);
    }
    CF_X4_TAIL(i, n) x[i] = fma_t(omega, r[i], x[i]);
}

template <int FMT>
__global__ void __launch_bounds__(kBlock, CF_SPMV_MIN_BLOCKS) k_f_rich_spmv(const SolveArgs *__restrict__ a)
{
    DevState *st = a->st;
    sell_prefetch<FMT>(a, a->s_val);
    CF_EXIT_IF_DONE(a, st, true);
    const double *__restrict__ x = a->x;
    const double *__restrict__ b = a->b;
    double *__restrict__ r = a->r[0];
    double acc[1] = {0.0};
    for_rows<FMT, double>(a, a->val, a->s_val, [&](int c) { return x[c]; }, [&](int row, double t) {
        const double ri = b[row] - t;
        r[row] = ri;
        acc[0] = fma_t(ri, ri, acc[0]);
    });
    double tot[1];
    if (grid_reduce<1, double>(acc, a->partials, a->partial_stride, &st->counters[SLOT_A], false, tot) &&
        threadIdx.x == 0)
        finish_step(a, st, sqrt(tot[0]));
}

// ---------------------------------------------------------------------------
// MR family.  FORM kMrPlain: MR; kMrScaled: JMR as MR on D^-1/2 A D^-1/2
// (a->sc_val, see scaled_values), which needs no prep pass; kMrZ: MRJacobi
// and MRS in the reference's arithmetic (SolverSingleGPU.h:1000-1073), the
// SpMV gathering z = D^-1 r, which the previous update wrote.
//   spmv:   y = A r (A z, or L A R r), (r, y), (y, y) -> step
//   update: x += alpha d, r -= alpha y, ||r|| with d = r (MR), R r (JMR:
//           R = a->corr_scale = D^-1/2) or z (MRJacobi, MRS, which also
//           write the next z = D^-1 r)
// MRJacobi on a scaled A D^-1 -- one rounding of a_ij / a_jj in the
// matrix instead of one of r_j / a_jj in the vector -- converged in 282-330
// steps instead of the reference's 277 on a 32^3 lognormal system, outside
// the 254-277 the reference itself takes when one source entry moves by
// one ulp, while every unscaled summation order stayed inside; JMR's
// scaled form stayed at the reference's count.
// ---------------------------------------------------------------------------
enum { kMrPlain = 0, kMrScaled = 1, kMrZ = 2 };

template <int FORM, int FMT>
__global__ void __launch_bounds__(kBlock, CF_SPMV_MIN_BLOCKS) k_f_mr_spmv(const SolveArgs *__restrict__ a)
{
    DevState *st = a->st;
    sell_prefetch<FMT>(a, FORM == kMrScaled ? a->sc_val : a->s_val);
    CF_EXIT_IF_DONE(a, st, false);
    const double *__restrict__ r = a->r[0];
    const double *__restrict__ gv = FORM == kMrZ ? a->w[1] : a->r[0];
    const double *val = FORM == kMrScaled ? a->sc_val : a->val;
    const double *sval = FORM == kMrScaled ? a->sc_val : a->s_val;
    double *__restrict__ y = a->w[0];
    double acc[2] = {0.0, 0.0};
    for_rows<FMT, double>(a, val, sval, [&](int c) { return gv[c]; }, [&](int row, double v) {
        y[row] = v;
        acc[0] = fma_t(r[row], v, acc[0]);
        acc[1] = fma_t(v, v, acc[1]);
    });
    double tot[2];
    if (grid_reduce<2, double>(acc, a->partials, a->partial_stride, &st->counters[SLOT_A], false, tot) &&
        threadIdx.x == 0)
        st->omega = tot[0] / tot[1];
}

// BiCG update: r -= xi q, r* -= xi q*, ||r||, (r, r*); the step logic of
// SolverSingleGPU.h:632-671 (stop when ||r|| < tol, theta = rho0 / rho1).
__global__ void __launch_bounds__(kBlock) k_f_bicg_update(const SolveArgs *__restrict__ a)
{
    DevState *st = a->st;
    CF_EXIT_IF_DONE(a, st, true);
    const int n = a->n;
    const double xi = ld_cg(&st->xi);
    double *__restrict__ r = a->r[0];
    double *__restrict__ rs = a->rs;
    const double *__restrict__ q = a->q;
    const double *__restrict__ qs = a->qs;
    double p0[4] = {0.0, 0.0, 0.0, 0.0}, p1[4] = {0.0, 0.0, 0.0, 0.0};
    CF_X4_LOOP(i, n) {
        double qv[4], rv[4], qsv[4], rsv[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            qv[u] = q[CF_X4_IDX(i, u)];
            rv[u] = r[CF_X4_IDX(i, u)];
            qsv[u] = qs[CF_X4_IDX(i, u)];
            rsv[u] = rs[CF_X4_IDX(i, u)];
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const double ri = fma_t(-xi, qv[u], rv[u]);
            const double rsi = fma_t(-xi, qsv[u], rsv[u]);
            r[CF_X4_IDX(i, u)] = ri;
            rs[CF_X4_IDX(i, u)] = rsi;
            p0[u] = fma_t(ri, ri, p0[u]);
            p1[u] = fma_t(ri, rsi, p1[u]);
        }
    }
    CF_X4_TAIL(i, n) {
        const double ri = fma_t(-xi, q[i], r[i]);
        const double rsi = fma_t(-xi, qs[i], rs[i]);
        r[i] = ri;
        rs[i] = rsi;
        p0[0] = fma_t(ri, ri, p0[0]);
        p1[0] = fma_t(ri, rsi, p1[0]);
    }
    double acc[2] = {(p0[0] + p0[1]) + (p0[2] + p0[3]), (p1[0] + p1[1]) + (p1[2] + p1[3])};
    double tot[2];
    if (grid_reduce<2, double>(acc, a->partials, a->partial_stride, &st->counters[SLOT_B], false, tot) &&
        threadIdx.x == 0) {
        const double norm = sqrt(tot[0]);
        const int k = st->k + 1;
        st->k = k;
        st->norm = norm;
        st->x_pending = 1;
        record_hist(a, st, k, norm);
        bool cont = true;
        int status = CF_NOT_CONVERGED;
        if (norm < st->tol && k >= st->min_steps) { cont = false; status = CF_OK; }
        else if (k >= st->max_steps) { cont = false; }
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

template <int FORM>
__global__ void __launch_bounds__(kBlock) k_f_mr_update(const SolveArgs *__restrict__ a)
{
    DevState *st = a->st;
    CF_EXIT_IF_DONE(a, st, true);
    const int n = a->n;
    const double alpha = ld_cg(&st->omega);
    double *__restrict__ r = a->r[0];
    double *__restrict__ x = a->x;
    const double *__restrict__ y = a->w[0];
    const double *__restrict__ R = FORM == kMrZ ? a->dinv : a->corr_scale;
    double *__restrict__ z = a->w[1];
    double part[4] = {0.0, 0.0, 0.0, 0.0};
    CF_X4_LOOP(i, n) {
        double rv[4], xv[4], yv[4], dv[4], sv[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            rv[u] = r[CF_X4_IDX(i, u)];
            xv[u] = x[CF_X4_IDX(i, u)];
            yv[u] = y[CF_X4_IDX(i, u)];
            if (FORM == kMrZ) {
                dv[u] = z[CF_X4_IDX(i, u)];
                sv[u] = R[CF_X4_IDX(i, u)];
            } else {
                dv[u] = FORM == kMrScaled ? __dmul_rn(R[CF_X4_IDX(i, u)], rv[u]) : rv[u];
            }
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            x[CF_X4_IDX(i, u)] = fma_t(alpha, dv[u], xv[u]);
            const double ri = fma_t(-alpha, yv[u], rv[u]);
            r[CF_X4_IDX(i, u)] = ri;
            if (FORM == kMrZ) z[CF_X4_IDX(i, u)] = __dmul_rn(sv[u], ri);
            part[u] = fma_t(ri, ri, part[u]);
        }
    }
    CF_X4_TAIL(i, n) {
        const double ri0 = r[i];
        const double di = FORM == kMrZ ? z[i] : FORM == kMrScaled ? __dmul_rn(R[i], ri0) : ri0;
        x[i] = fma_t(alpha, di, x[i]);
        const double ri = fma_t(-alpha, y[i], ri0);
        r[i] = ri;
        if (FORM == kMrZ) z[i] = __dmul_rn(R[i], ri);
        part[0] = fma_t(ri, ri, part[0]);
    }
    double acc[1] = {(part[0] + part[1]) + (part[2] + part[3])};
    double tot[1];
    if (grid_reduce<1, double>(acc, a->partials, a->partial_stride, &st->counters[SLOT_B], false, tot) &&
        threadIdx.x == 0)
        finish_step(a, st, sqrt(tot[0]));
}

// ---------------------------------------------------------------------------
template <int FMT>
static Kernels fast_kernels(int solver)
{
    Kernels k;
    switch (solver) {
    case CF_CG:
        k.k0 = (const void *)k_f_cg_prep;
        k.k1 = (const void *)k_f_cg_spmv<FMT>;
        k.k2 = (const void *)k_f_cg_update;
        break;
    case CF_BICG:
        k.k0 = (const void *)k_f_bicg_prep;
        k.k1 = (const void *)k_f_bicg_spmv<FMT>;
        k.k2 = (const void *)k_f_bicg_update;
        break;
    case CF_JACOBI: // on A D^-1 (scaled_values), set up by the caller
        k.k1 = (const void *)k_f_jac_step<FMT>;
        break;
    case CF_PCG:
        k.k0 = (const void *)k_f_pcg_prep;
        k.k1 = (const void *)k_f_cg_spmv<FMT>;
        k.k2 = (const void *)k_f_pcg_update;
        break;
    case CF_RICHARDSON:
        k.k0 = (const void *)k_f_rich_prep;
        k.k1 = (const void *)k_f_rich_spmv<FMT>;
        break;
    case CF_MR:
        k.k1 = (const void *)k_f_mr_spmv<kMrPlain, FMT>;
        k.k2 = (const void *)k_f_mr_update<kMrPlain>;
        break;
    case CF_MRJACOBI:
    case CF_MRS: // z = D^-1 r of the initial residual written by k_res_init
        k.k1 = (const void *)k_f_mr_spmv<kMrZ, FMT>;
        k.k2 = (const void *)k_f_mr_update<kMrZ>;
        break;
    case CF_JMR: // MR on D^-1/2 A D^-1/2 (scaled_values), set up by the caller
        k.k1 = (const void *)k_f_mr_spmv<kMrScaled, FMT>;
        k.k2 = (const void *)k_f_mr_update<kMrScaled>;
        break;
    default: break;
    }
    // the SELL-32 passes stage nothing (no dynamic shared memory)
    k.k1_spmv = FMT == kCsr;
    return k;
}

Kernels fast_body_kernels(int solver, int format)
{
    return format == kSellC ? fast_kernels<kSellC>(solver)
           : format == kSellD ? fast_kernels<kSellD>(solver)
           : format == kSell  ? fast_kernels<kSell>(solver)
                              : fast_kernels<kCsr>(solver);
}

const void *fast_flush_kernel() { return (const void *)k_f_flush_x; }

} // namespace cf
