// mixed.cu -- mixed-precision solves: FP32 matrix values, FP32 Krylov
// vectors and FP32 accumulation in the inner solver, inside an FP64
// iterative-refinement loop that owns the true residual b - A x, the
// normFactor and the stopping test.
//
// Outer step j:  r = b - A x (FP64);  solve A d = r / ||r|| in FP32 to a
// relative tolerance eta (CG and MR: the same fused passes as FP64 with
// float data; MRJacobi, MRS, JMR: MR on a diagonally scaled matrix; BiCG:
// BiCGStab, see below);  x += ||r|| d (FP64).  The loop stops when the FP64
// residual reaches tolerance * normFactor, so the answer carries the FP64
// tolerance.
// FP32 halves the bytes of every vector stream and cuts the matrix from 12
// to 8 bytes per entry.
#include "solver_common.cuh"

#include <algorithm>
#include <climits>
#include <cmath>

// Resident blocks per SM the FP32 SpMV passes ask for: the MR one six
// (the 256^3 upwind MR inner solve with batches of eight: 238 us per step
// against 242 us with five and 258 us with four), the BiCGStab ones five,
// and the CG one four (49.2 us per step at 128^3 against 53.0 us with
// five; its on-the-fly direction update needs the registers).
#ifndef CF_MX_MIN_BLOCKS
#define CF_MX_MIN_BLOCKS 6
#endif
#ifndef CF_MX_BCS_MIN_BLOCKS
#define CF_MX_BCS_MIN_BLOCKS 5
#endif
#ifndef CF_MX_CG_MIN_BLOCKS
#define CF_MX_CG_MIN_BLOCKS 4
#endif
// SELL entries per thread and batch in the two BiCGStab SpMV passes (8: the
// 256^3 convection-diffusion BiCGStab step took 735 us against 989 us with
// 4 and 1,039 us with 2).
#ifndef CF_BCS_SELL_BATCH
#define CF_BCS_SELL_BATCH 8
#endif

namespace cf {

// ---------------------------------------------------------------------------
// FP64 pieces of the outer loop
// ---------------------------------------------------------------------------
// x += s * d with s = ||r|| of the residual the inner system was scaled by
// (MR family: x += s * R d, R the column scaling of the inner matrix).
__global__ void __launch_bounds__(kBlock) k_mx_correct(const SolveArgs *__restrict__ a)
{
    const int n = a->n;
    const double s = ld_cg(&a->st->norm);
    const float *d = a->fx;
    const double *R = a->corr_scale;
    double *x = a->x;
    CF_FOR_ELEMS(i, n) {
        double di = (double)d[i];
        if (R) di *= R[i];
        x[i] = fma_t(s, di, x[i]);
    }
}

// r = b - A x, ||r|| (FP64); records the outer step.  SCALED (JMR, whose
// residual is the symmetrically scaled one): r = D^-1/2 (b - A x).
template <int FMT, bool SCALED>
__global__ void __launch_bounds__(kBlock, CF_SPMV_MIN_BLOCKS) k_mx_residual(const SolveArgs *__restrict__ a)
{
    const double *x = a->x, *b = a->b, *sD = a->dinv_sqrt;
    double *r = a->r[0];
    double acc[1] = {0.0};
    for_rows<FMT, double>(a, a->val, a->s_val, [&](int c) { return x[c]; }, [&](int row, double t) {
        double ri = b[row] - t;
        if (SCALED) ri = __dmul_rn(sD[row], ri);
        r[row] = ri;
        acc[0] = fma_t(ri, ri, acc[0]);
    });
    double tot[1];
    if (grid_reduce<1, double>(acc, a->partials, a->partial_stride, &a->st->counters[SLOT_MISC],
                               false, tot) && threadIdx.x == 0) {
        DevState *st = a->st;
        const double norm = sqrt(tot[0]);
        const int k = st->k + 1; // outer steps
        st->k = k;
        st->norm = norm;
        record_hist(a, st, k, norm);
        if (!isfinite(norm)) {
            st->done = 1;
            st->status = CF_NONFINITE;
        } else if (norm <= st->tol) {
            st->done = 1;
            st->status = CF_OK;
        }
    }
}

// ---------------------------------------------------------------------------
// FP32 inner solve
// ---------------------------------------------------------------------------
// r32 = float(r64 / ||r64||), d = 0 (, r*32 = r32 for BiCG); inner state.
__global__ void __launch_bounds__(kBlock) k_mx_setup(const SolveArgs *__restrict__ a, int bicg)
{
    const int n = a->n;
    DevState *si = a->st_in;
    const double inv = 1.0 / ld_cg(&a->st->norm);
    const double *r64 = a->r[0];
    float *fr = a->fr, *fd = a->fx, *frs = a->frs;
    float acc[1] = {0.f};
    CF_FOR_ELEMS(i, n) {
        const float v = (float)(r64[i] * inv);
        fr[i] = v;
        fd[i] = 0.f;
        if (bicg) frs[i] = v;
        acc[0] = fma_t(v, v, acc[0]);
    }
    float tot[1];
    if (grid_reduce<1, float>(acc, a->partials32, a->partial_stride, &si->counters[SLOT_INIT], false,
                              tot) && threadIdx.x == 0) {
        const float rr = tot[0];
        const double norm0 = sqrtf(rr);
        si->rho0 = rr;
        si->rho1 = 0.0;
        si->norm0 = norm0;
        si->norm = norm0;
        si->tol = si->tolerance * norm0;
        si->k = 0;
        si->x_pending = 0;
        si->body_count = 0;
        const bool finite = isfinite(norm0);
        bool cont = finite && si->max_steps >= 1 && (bicg || norm0 > si->tol);
        si->done = cont ? 0 : 1;
        si->status = finite ? CF_OK : CF_NONFINITE;
    }
}

// CG: K1 p = r + beta p_old (on the fly), q = A32 p, (p, q); deferred d update
template <int FMT>
__global__ void __launch_bounds__(kBlock, CF_MX_CG_MIN_BLOCKS) k_mx_cg_spmv(const SolveArgs *__restrict__ a)
{
    DevState *st = a->st_in;
    sell_prefetch<FMT>(a, a->s_val32);
    CF_EXIT_IF_DONE(a, st, false);
    const int k = ld_cg(&st->k) + 1;
    const bool first = (k == 1);
    const float beta = first ? 0.f : (float)ld_cg(&st->rho0) / (float)ld_cg(&st->rho1);
    const float xi_prev = (float)ld_cg(&st->xi);
    const bool xpend = ld_cg(&st->x_pending) != 0;
    const float *pin = a->fp[(k + 1) & 1];
    float *pout = a->fp[k & 1];
    const float *r = a->fr;
    float *d = a->fx, *q = a->fq;
    auto g = [&](int c) { return first ? r[c] : fma_t(beta, pin[c], r[c]); };
    float acc[1] = {0.f};
    for_rows<FMT, float>(a, a->val32, a->s_val32, g, [&](int row, float y) {
        const float pi = g(row);
        pout[row] = pi;
        q[row] = y;
        if (xpend) d[row] = fma_t(xi_prev, pin[row], d[row]);
        acc[0] = fma_t(pi, y, acc[0]);
    });
    float tot[1];
    if (grid_reduce<1, float>(acc, a->partials32, a->partial_stride, &st->counters[SLOT_A], false,
                              tot) && threadIdx.x == 0) {
        st->xi = (float)st->rho0 / tot[0];
        st->x_pending = 0;
    }
}

__global__ void __launch_bounds__(kBlock) k_mx_cg_update(const SolveArgs *__restrict__ a)
{
    DevState *st = a->st_in;
    CF_EXIT_IF_DONE(a, st, true);
    const int n = a->n;
    const float xi = (float)ld_cg(&st->xi);
    float *r = a->fr;
    const float *q = a->fq;
    float acc[1] = {0.f};
    CF_FOR_ELEMS(i, n) {
        const float ri = fma_t(-xi, q[i], r[i]);
        r[i] = ri;
        acc[0] = fma_t(ri, ri, acc[0]);
    }
    float tot[1];
    if (grid_reduce<1, float>(acc, a->partials32, a->partial_stride, &st->counters[SLOT_B], false,
                              tot) && threadIdx.x == 0) {
        st->rho1 = st->rho0;
        st->rho0 = tot[0];
        st->x_pending = 1;
        finish_step(a, st, sqrtf(tot[0]));
    }
}

__global__ void __launch_bounds__(kBlock) k_mx_flush(const SolveArgs *__restrict__ a)
{
    DevState *st = a->st_in;
    if (!ld_cg(&st->x_pending)) return;
    const int n = a->n;
    const int k = ld_cg(&st->k);
    const float xi = (float)ld_cg(&st->xi);
    const float *p = a->fp[k & 1];
    float *d = a->fx;
    CF_FOR_ELEMS(i, n) d[i] = fma_t(xi, p[i], d[i]);
}

// BiCG's FP32 inner solver is BiCGStab (van der Vorst): FP32 BiCG loses
// the bi-orthogonality of its two sequences and diverges on the
// convection-diffusion systems where FP64 BiCG converges, BiCGStab in FP32
// reaches the inner tolerance.  The outer FP64 loop is BiCG's own stopping
// test on the true residual.  One step is four passes:
//   K0  p = r + beta (p - omega v)                       (first step: p = r)
//   K1  v = A p, alpha = rho / (r^, v)
//   K2  s = r - alpha v (formed for every gathered column), t = A s,
//       omega = (t, s) / (t, t)
//   K3  d += alpha p + omega s, r = s - omega t, rho' = (r^, r), ||r||
// with r^ the fixed shadow residual (the scaled r of the sweep's start).
__global__ void __launch_bounds__(kBlock) k_mx_bcs_prep(const SolveArgs *__restrict__ a)
{
    DevState *st = a->st_in;
    CF_EXIT_IF_DONE(a, st, false);
    const int n = a->n;
    const int k = ld_cg(&st->k) + 1;
    const float *__restrict__ r = a->fr;
    float *__restrict__ p = a->fp[0];
    if (k == 1) {
        CF_FOR_ELEMS(i, n) p[i] = r[i];
        return;
    }
    const float beta = (float)ld_cg(&st->theta);
    const float w = (float)ld_cg(&st->omega);
    const float *__restrict__ v = a->fq;
    CF_FOR_ELEMS(i, n) p[i] = fma_t(beta, fma_t(-w, v[i], p[i]), r[i]);
}

template <int FMT>
__global__ void __launch_bounds__(kBlock, CF_MX_BCS_MIN_BLOCKS) k_mx_bcs_spmv1(const SolveArgs *__restrict__ a)
{
    DevState *st = a->st_in;
    sell_prefetch<FMT>(a, a->s_val32);
    CF_EXIT_IF_DONE(a, st, false);
    const float *__restrict__ p = a->fp[0];
    const float *__restrict__ rh = a->frs;
    float *__restrict__ v = a->fq;
    float acc[1] = {0.f};
    for_rows<FMT, float, CF_BCS_SELL_BATCH>(a, a->val32, a->s_val32, [&](int c) { return p[c]; }, [&](int row, float y) {
        v[row] = y;
        acc[0] = fma_t(rh[row], y, acc[0]);
    });
    float tot[1];
    if (grid_reduce<1, float>(acc, a->partials32, a->partial_stride, &st->counters[SLOT_A], false,
                              tot) && threadIdx.x == 0) {
        const float alpha = (float)st->rho0 / tot[0];
        if (isfinite(alpha) && tot[0] != 0.f) {
            st->xi = alpha;
        } else {
            st->done = 1;
            st->status = tot[0] == 0.f ? CF_BREAKDOWN : CF_NONFINITE;
        }
    }
}

template <int FMT>
__global__ void __launch_bounds__(kBlock, CF_MX_BCS_MIN_BLOCKS) k_mx_bcs_spmv2(const SolveArgs *__restrict__ a)
{
    DevState *st = a->st_in;
    sell_prefetch<FMT>(a, a->s_val32);
    CF_EXIT_IF_DONE(a, st, false);
    const float alpha = (float)ld_cg(&st->xi);
    const float *__restrict__ r = a->fr;
    const float *__restrict__ v = a->fq;
    float *__restrict__ sv = a->fp[1];
    float *__restrict__ t = a->fqs;
    auto g = [&](int c) { return fma_t(-alpha, v[c], r[c]); };
    float acc[2] = {0.f, 0.f};
    for_rows<FMT, float, CF_BCS_SELL_BATCH>(a, a->val32, a->s_val32, g, [&](int row, float y) {
        const float si = g(row);
        sv[row] = si;
        t[row] = y;
        acc[0] = fma_t(y, si, acc[0]);
        acc[1] = fma_t(y, y, acc[1]);
    });
    float tot[2];
    if (grid_reduce<2, float>(acc, a->partials32, a->partial_stride, &st->counters[SLOT_C], false,
                              tot) && threadIdx.x == 0)
        st->omega = tot[1] > 0.f ? tot[0] / tot[1] : 0.f;
}

__global__ void __launch_bounds__(kBlock) k_mx_bcs_update(const SolveArgs *__restrict__ a)
{
    DevState *st = a->st_in;
    CF_EXIT_IF_DONE(a, st, true);
    const int n = a->n;
    const float alpha = (float)ld_cg(&st->xi);
    const float w = (float)ld_cg(&st->omega);
    const float *__restrict__ p = a->fp[0];
    const float *__restrict__ sv = a->fp[1];
    const float *__restrict__ t = a->fqs;
    const float *__restrict__ rh = a->frs;
    float *__restrict__ r = a->fr;
    float *__restrict__ d = a->fx;
    float acc[2] = {0.f, 0.f};
    CF_FOR_ELEMS(i, n) {
        const float si = sv[i];
        d[i] = fma_t(w, si, fma_t(alpha, p[i], d[i]));
        const float ri = fma_t(-w, t[i], si);
        r[i] = ri;
        acc[0] = fma_t(ri, ri, acc[0]);
        acc[1] = fma_t(rh[i], ri, acc[1]);
    }
    float tot[2];
    if (grid_reduce<2, float>(acc, a->partials32, a->partial_stride, &st->counters[SLOT_B], false,
                              tot) && threadIdx.x == 0) {
        const double norm = sqrtf(tot[0]);
        const int k = st->k + 1;
        st->k = k;
        st->norm = norm;
        bool cont = true;
        int status = CF_NOT_CONVERGED;
        if (norm < st->tol) { cont = false; status = CF_OK; }
        else if (k >= st->max_steps) { cont = false; }
        else if (!isfinite(norm)) { cont = false; status = CF_NONFINITE; }
        else if (tot[1] == 0.f || w == 0.f) { cont = false; status = CF_BREAKDOWN; }
        st->body_count += 1;
        if (st->body_count > k + 2 || (a->abort_flag && *a->abort_flag)) { cont = false; status = CF_TIMEOUT; }
        if (cont) {
            st->rho1 = st->rho0;
            st->rho0 = tot[1];
            st->theta = ((float)st->rho0 / (float)st->rho1) * (alpha / w);
        } else {
            st->done = 1;
            st->status = status;
        }
        set_loop_condition(a, cont);
    }
}

// MR: K1 y = A32 r, (r, y), (y, y); K2 d += w r, r -= w y, ||r||.  (A
// single kernel that forms r - w y on the fly for every gathered column
// measured slower at 256^3: two gathers per entry cost more than the
// separate element-wise pass.)
template <int FMT>
__global__ void __launch_bounds__(kBlock, CF_MX_MIN_BLOCKS) k_mx_mr_spmv(const SolveArgs *__restrict__ a)
{
    DevState *st = a->st_in;
    sell_prefetch<FMT>(a, a->s_val32);
    CF_EXIT_IF_DONE(a, st, false);
    const float *__restrict__ r = a->fr;
    float *__restrict__ y = a->fq;
    float acc[2] = {0.f, 0.f};
    for_rows<FMT, float>(a, a->val32, a->s_val32, [&](int c) { return r[c]; }, [&](int row, float v) {
        y[row] = v;
        acc[0] = fma_t(r[row], v, acc[0]);
        acc[1] = fma_t(v, v, acc[1]);
    });
    float tot[2];
    if (grid_reduce<2, float>(acc, a->partials32, a->partial_stride, &st->counters[SLOT_A], false,
                              tot) && threadIdx.x == 0)
        st->omega = tot[0] / tot[1];
}

// four consecutive elements per thread and step (16-byte loads)
__global__ void __launch_bounds__(kBlock) k_mx_mr_update(const SolveArgs *__restrict__ a)
{
    DevState *st = a->st_in;
    CF_EXIT_IF_DONE(a, st, true);
    const int n = a->n;
    const float w = (float)ld_cg(&st->omega);
    float *__restrict__ r = a->fr;
    float *__restrict__ d = a->fx;
    const float *__restrict__ y = a->fq;
    float4 *r4 = reinterpret_cast<float4 *>(r);
    float4 *d4 = reinterpret_cast<float4 *>(d);
    const float4 *y4 = reinterpret_cast<const float4 *>(y);
    float acc[1] = {0.f};
    const int n4 = n >> 2;
    CF_FOR_ELEMS(i, n4) {
        const float4 rv = r4[i], dv = d4[i], yv = y4[i];
        float4 dn, rn;
        dn.x = fma_t(w, rv.x, dv.x);
        dn.y = fma_t(w, rv.y, dv.y);
        dn.z = fma_t(w, rv.z, dv.z);
        dn.w = fma_t(w, rv.w, dv.w);
        rn.x = fma_t(-w, yv.x, rv.x);
        rn.y = fma_t(-w, yv.y, rv.y);
        rn.z = fma_t(-w, yv.z, rv.z);
        rn.w = fma_t(-w, yv.w, rv.w);
        d4[i] = dn;
        r4[i] = rn;
        acc[0] = fma_t(rn.x, rn.x, fma_t(rn.y, rn.y, fma_t(rn.z, rn.z, fma_t(rn.w, rn.w, acc[0]))));
    }
    for (int i = 4 * n4 + blockIdx.x * kBlock + threadIdx.x; i < n; i += gridDim.x * kBlock) {
        d[i] = fma_t(w, r[i], d[i]);
        const float ri = fma_t(-w, y[i], r[i]);
        r[i] = ri;
        acc[0] = fma_t(ri, ri, acc[0]);
    }
    float tot[1];
    if (grid_reduce<1, float>(acc, a->partials32, a->partial_stride, &st->counters[SLOT_B], false,
                              tot) && threadIdx.x == 0)
        finish_step(a, st, sqrtf(tot[0]));
}

// ---------------------------------------------------------------------------
// host driver of the refinement loop
// ---------------------------------------------------------------------------
template <int FMT>
static Kernels inner_kernels_t(int solver)
{
    Kernels k;
    k.value_bytes = sizeof(float);
    switch (solver) {
    case CF_CG: k.k1 = (const void *)k_mx_cg_spmv<FMT>; k.k2 = (const void *)k_mx_cg_update; break;
    case CF_BICG:
        k.k0 = (const void *)k_mx_bcs_prep;
        k.k1 = (const void *)k_mx_bcs_spmv1<FMT>;
        k.k2 = (const void *)k_mx_bcs_spmv2<FMT>;
        k.k3 = (const void *)k_mx_bcs_update;
        k.k2_spmv = FMT == kCsr;
        break;
    case CF_MR:
    case CF_MRJACOBI: // the preconditioned MR solvers run MR on a scaled matrix
    case CF_MRS:
    case CF_JMR: k.k1 = (const void *)k_mx_mr_spmv<FMT>; k.k2 = (const void *)k_mx_mr_update; break;
    default: break;
    }
    k.k1_spmv = FMT == kCsr;   // the SELL passes stage nothing
    return k;
}

static Kernels inner_kernels(int solver, int format)
{
    return format == kSellC ? inner_kernels_t<kSellC>(solver)
           : format == kSellD ? inner_kernels_t<kSellD>(solver)
           : format == kSell  ? inner_kernels_t<kSell>(solver)
                              : inner_kernels_t<kCsr>(solver);
}

template <int FMT>
static const void *residual_kernel(bool scaled)
{
    return scaled ? (const void *)k_mx_residual<FMT, true> : (const void *)k_mx_residual<FMT, false>;
}

bool mixed_supported(int solver)
{
    return solver == CF_CG || solver == CF_BICG || solver == CF_MR || mr_scaled_solver(solver);
}

void mixed_prepare(Context *ctx, Matrix *m, int solver, SolveArgs &A)
{
    require(mixed_supported(solver), CF_UNSUPPORTED,
            "mixed precision is implemented for CG, BiCG, MR, MRJacobi, MRS and JMR");
    const bool tr = A.val != m->val.as<double>(); // transposed solve
    const bool scaled = mr_scaled_solver(solver);
    if (!scaled) {
        matrix_ensure_fp32(m, false);
        if (solver == CF_BICG || tr) matrix_ensure_fp32(m, true);
    }
    const size_t fb = sizeof(float) * ((size_t)m->n + 16);
    for (int i = 14; i < 24; ++i) ctx->vec[i].ensure(fb);
    const int stride = std::max(ctx->ref_grid, ctx->sm_count * 8);
    ctx->partials32.ensure(sizeof(float) * kMaxNV * (size_t)stride);
    ctx->state_in.ensure(sizeof(DevState));
    A.corr_scale = nullptr;
    if (scaled) {
        // FP32 L A R of the solved matrix in the layout in use
        const float *v = scaled_values<float>(ctx, m, A, solver, tr, m->sc32, &A.corr_scale);
        A.val32 = A.n_slices > 0 ? nullptr : v;
        A.s_val32 = A.n_slices > 0 ? v : nullptr;
        A.valT32 = A.s_valT32 = nullptr;
    } else {
        A.val32 = m->val32.as<float>();
        A.valT32 = m->have_T32 ? m->valT32.as<float>() : nullptr;
        if (tr) std::swap(A.val32, A.valT32);
        if (A.n_slices > 0) { // SELL-32 copies (FP32 values filled by the caller's matrix_ensure_sell)
            A.s_val32 = m->s_val32.as<float>();
            A.s_valT32 = m->have_svalT32 ? m->s_valT32.as<float>() : nullptr;
            if (tr) std::swap(A.s_val32, A.s_valT32);
        }
    }
    A.fx = ctx->vec[14].as<float>();
    A.fr = ctx->vec[15].as<float>();
    A.fp[0] = ctx->vec[16].as<float>();
    A.fp[1] = ctx->vec[17].as<float>();
    A.fq = ctx->vec[18].as<float>();
    A.frs = ctx->vec[19].as<float>();
    A.fps[0] = ctx->vec[20].as<float>();
    A.fps[1] = ctx->vec[21].as<float>();
    A.fqs = ctx->vec[22].as<float>();
    A.partials32 = ctx->partials32.as<float>();
    A.st_in = ctx->state_in.as<DevState>();
}

// Fraction of the remaining FP64 reduction the last refinement sweep aims
// for (the FP32 recursive residual tracks the FP64 one to ~1e-6 relative).
constexpr double kLastSweepMargin = 0.8;

// Runs after the FP64 normFactor and initial residual (st holds ||r_0||,
// tol = tolerance * normFactor).  Returns the total inner iterations.
MixedResult run_mixed(Context *ctx, Matrix *m, int solver, const cf_controls &c, SolveArgs *d_args,
                      int cap, bool use_graph_in)
{
    MixedResult res;
    SolveArgs &A = *ctx->h_args;
    void *args1[] = {&d_args};
    const bool sell = A.n_slices > 0;
    const int fmt = solve_format(A);
    const Kernels kk = inner_kernels(solver, fmt);
    const bool scaled = solver == CF_JMR;
    const void *k_residual = fmt == kSellC ? residual_kernel<kSellC>(scaled)
                             : fmt == kSellD ? residual_kernel<kSellD>(scaled)
                             : fmt == kSell  ? residual_kernel<kSell>(scaled)
                                             : residual_kernel<kCsr>(scaled);
    bool use_graph = use_graph_in;
    GraphEntry *ge = nullptr;
    if (use_graph) {
        try {
            ge = loop_graph(ctx, kk, solver, CF_PREC_MIXED, cap, false, d_args, fmt);
        } catch (const Error &) {
            ctx->graphs_ok = false;
            use_graph = false;
        }
    }
    if (use_graph) {
        // the loop handle travels in the device-resident arguments
        A.use_cond = 1;
        A.cond = ge->cond;
        CF_CUDA(cudaMemcpyAsync(d_args, &A, sizeof(SolveArgs), cudaMemcpyHostToDevice, ctx->stream));
    }
    CF_CUDA(cudaMemcpyAsync(ctx->h_state, A.st, sizeof(DevState), cudaMemcpyDeviceToHost, ctx->stream));
    CF_CUDA(cudaStreamSynchronize(ctx->stream));
    const int64_t max_total = c.max_iter <= 0 ? INT_MAX : c.max_iter;
    const int max_outer = c.mixed_max_outer > 0 ? c.mixed_max_outer : 50;
    // default inner tolerance per solver, the fastest measured on GB300: CG
    // at 128^3 27.5 ms with 1e-6 against 32.4 ms with 1e-4 (fewer restarts of
    // the Krylov space); BiCG and MR on C3 within 3% for 1e-4 .. 1e-6
    const double eta = (c.mixed_inner_rtol > 0 && c.mixed_inner_rtol < 1) ? c.mixed_inner_rtol
                                                                          : (solver == CF_CG ? 1e-6 : 1e-4);
    // every inner sweep runs to the inner tolerance unless capped
    int inner_cap = c.mixed_inner_max > 0 ? c.mixed_inner_max : INT_MAX;
    // x and r before each correction, to undo a sweep that made things worse
    // (workspace vectors 12 and 13: unused by the mixed path otherwise)
    const size_t vb = sizeof(double) * (size_t)m->n;
    ctx->vec[12].ensure(vb);
    ctx->vec[13].ensure(vb);
    double *x_keep = ctx->vec[12].as<double>(), *r_keep = ctx->vec[13].as<double>();
    double prev_norm = ctx->h_state->norm;
    int64_t total = 0;
    int outer = 0;
    int status = ctx->h_state->done ? ctx->h_state->status : CF_NOT_CONVERGED;
    DevState &SI = *ctx->h_state_in;
    while (!ctx->h_state->done && outer < max_outer && total < max_total) {
        SI = DevState{};
        // the last sweep only has to reach the FP64 target (with a margin
        // for the FP32 / FP64 residual gap), not eta below it
        SI.tolerance = std::max(eta, std::min(0.5, kLastSweepMargin * ctx->h_state->tol / prev_norm));
        SI.max_steps = (int)std::min<int64_t>(std::min<int64_t>(max_total - total, (int64_t)inner_cap), INT_MAX);
        SI.int_bound = c.bicg_int_bound;
        SI.hist_cap = 0;
        CF_CUDA(cudaMemcpyAsync(A.st_in, &SI, sizeof(DevState), cudaMemcpyHostToDevice, ctx->stream));
        int bicg = solver == CF_BICG ? 1 : 0;
        void *a2[] = {&d_args, &bicg};
        launch(ctx, ctx->stream, (const void *)k_mx_setup,
               launch_cfg(ctx, (const void *)k_mx_setup, false, cap, false), a2);
        if (use_graph) {
            CF_CUDA(cudaGraphLaunch(ge->exec, ctx->stream));
        } else {
            for (;;) {
                for (int i = 0; i < 16; ++i) launch_body(ctx, ctx->stream, kk, cap, false, d_args);
                CF_CUDA(cudaMemcpyAsync(&SI, A.st_in, sizeof(DevState), cudaMemcpyDeviceToHost, ctx->stream));
                CF_CUDA(cudaStreamSynchronize(ctx->stream));
                if (SI.done) break;
            }
        }
        if (solver == CF_CG || solver == CF_BICG)
            launch(ctx, ctx->stream, (const void *)k_mx_flush,
                   launch_cfg(ctx, (const void *)k_mx_flush, false, cap, false), args1);
        CF_CUDA(cudaMemcpyAsync(x_keep, A.x, vb, cudaMemcpyDeviceToDevice, ctx->stream));
        CF_CUDA(cudaMemcpyAsync(r_keep, A.r[0], vb, cudaMemcpyDeviceToDevice, ctx->stream));
        launch(ctx, ctx->stream, (const void *)k_mx_correct,
               launch_cfg(ctx, (const void *)k_mx_correct, false, cap, false), args1);
        launch(ctx, ctx->stream, k_residual, launch_cfg(ctx, k_residual, !sell, cap, false), args1);
        CF_CUDA(cudaMemcpyAsync(&SI, A.st_in, sizeof(DevState), cudaMemcpyDeviceToHost, ctx->stream));
        CF_CUDA(cudaMemcpyAsync(ctx->h_state, A.st, sizeof(DevState), cudaMemcpyDeviceToHost, ctx->stream));
        CF_CUDA(cudaStreamSynchronize(ctx->stream));
        total += SI.k;
        ++outer;
        const double nrm = ctx->h_state->norm;
        if (ctx->h_state->done && ctx->h_state->status == CF_OK) {
            status = CF_OK;
            break;
        }
        if (SI.status == CF_BREAKDOWN && SI.k == 0) {
            // the inner solver broke down before its first step: x is
            // unchanged, so a retry would repeat the same breakdown
            status = CF_BREAKDOWN;
            break;
        }
        if (!(nrm < prev_norm)) {
            // The FP32 sweep raised the FP64 residual (a non-finite inner
            // solve included): undo it and retry with a sweep half as long
            // as the one just undone (the sweep is deterministic, so a
            // retry of the same length would repeat it).
            CF_CUDA(cudaMemcpyAsync(A.x, x_keep, vb, cudaMemcpyDeviceToDevice, ctx->stream));
            CF_CUDA(cudaMemcpyAsync(A.r[0], r_keep, vb, cudaMemcpyDeviceToDevice, ctx->stream));
            DevState &S = *ctx->h_state;
            S.norm = prev_norm;
            S.done = 0;
            S.status = CF_NOT_CONVERGED;
            CF_CUDA(cudaMemcpyAsync(A.st, &S, sizeof(DevState), cudaMemcpyHostToDevice, ctx->stream));
            CF_CUDA(cudaStreamSynchronize(ctx->stream));
            inner_cap = SI.k / 2;
            if (inner_cap < 8) {
                status = CF_NOT_CONVERGED;
                break;
            }
            continue;
        }
        if (ctx->h_state->done) {
            status = ctx->h_state->status;
            break;
        }
        prev_norm = nrm;
    }
    if (!ctx->h_state->done && status == CF_NOT_CONVERGED) status = CF_NOT_CONVERGED;
    res.inner_iterations = (int)std::min<int64_t>(total, INT_MAX);
    res.outer = outer;
    res.status = ctx->h_state->done ? ctx->h_state->status : status;
    return res;
}

} // namespace cf
