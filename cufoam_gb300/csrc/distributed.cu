// distributed.cu -- the solvers on one subdomain of a decomposed case (one
// rank per subdomain, OpenFOAM's processor patches).
//
// OpenFOAM's lduMatrix::Amul on a decomposed mesh forms the local product
// and then, per processor patch, subtracts interfaceBouCoeffs[f] times the
// neighbouring rank's value of the cell on the far side of face f from the
// product's row faceCells[f] (initMatrixInterfaces /
// updateMatrixInterfaces); its dot products and normFactor sum over all
// ranks.  This is OpenFOAM's semantics restated (its sources are not
// available here, and the reference ignores interfaces altogether --
// cuFoamCG/cuFoamCG.C:19-35).  The solve here:
//   * before every product, the values of the product's input at the patch
//     faces' cells are gathered on the device, handed to the caller's
//     exchange callback, and the neighbours' values come back as ghosts;
//   * the product is the local SpMV (fast order) followed by one pass that
//     subtracts coeff * ghost per face, the faces of a cell in the order
//     given (patch order, then face order, as OpenFOAM loops);
//   * A^T (BiCG) couples through the neighbour's coefficient of the same
//     face -- the global matrix's (neighbour row, own column) entry --
//     which one exchange of the coefficients provides at the start;
//   * every dot product is a local deterministic sum handed to the caller's
//     all-reduce callback.
// The loops are host-paced and follow the reference's drivers
// (SolverSingleGPU.h: CG 366-445, BiCG 568-675, Richardson 762-819 with
// OptimizePower 723-752, MR 825-890, Jacobi 924-994, MRJacobi 1000-1073,
// JMR 1079-1155, MRS 1236-1303) and the library's Jacobi-preconditioned
// CG, with the library's stopping rule: continue while ||r||_2 >
// tolerance * normFactor (or fewer than minIter steps) and fewer than
// maxIter steps.
#include "solver_common.cuh"

#include <algorithm>
#include <chrono>
#include <climits>
#include <cmath>
#include <vector>

namespace cf {

namespace {

__global__ void __launch_bounds__(kBlock) k_dd_gather(int m, const int32_t *__restrict__ cells,
                                                      const double *__restrict__ x, double *__restrict__ send)
{
    CF_FOR_ELEMS(i, m) send[i] = x[cells[i]];
}

// y[cell] -= coeff[f] * ghost[f] for the faces of each coupled cell, in order
__global__ void __launch_bounds__(kBlock) k_dd_iface(int nc, const int32_t *__restrict__ cell,
                                                     const int32_t *__restrict__ start,
                                                     const int32_t *__restrict__ face,
                                                     const double *__restrict__ coeff,
                                                     const double *__restrict__ ghost, double *__restrict__ y)
{
    CF_FOR_ELEMS(i, nc) {
        const int c = cell[i];
        double v = y[c];
        for (int k = start[i]; k < start[i + 1]; ++k) {
            const int f = face[k];
            v = fma_t(-coeff[f], ghost[f], v);
        }
        y[c] = v;
    }
}

__global__ void __launch_bounds__(kBlock) k_dd_fill(int n, double v, double *__restrict__ x)
{
    CF_FOR_ELEMS(i, n) x[i] = v;
}

// o = w .* v (w given) or s * v
__global__ void __launch_bounds__(kBlock) k_dd_scale(int n, const double *__restrict__ w, double s,
                                                     const double *__restrict__ v, double *__restrict__ o)
{
    CF_FOR_ELEMS(i, n) o[i] = w ? __dmul_rn(w[i], v[i]) : __dmul_rn(s, v[i]);
}

// x += s p
__global__ void __launch_bounds__(kBlock) k_dd_axpy(int n, double s, const double *__restrict__ p,
                                                    double *__restrict__ x)
{
    CF_FOR_ELEMS(i, n) x[i] = fma_t(s, p[i], x[i]);
}

// p = r + beta p (p = r on the first step); the same for (ps, rs) if given
__global__ void __launch_bounds__(kBlock) k_dd_dir(int n, int first, double beta, const double *__restrict__ r,
                                                   double *__restrict__ p, const double *__restrict__ rs,
                                                   double *__restrict__ ps)
{
    CF_FOR_ELEMS(i, n) {
        p[i] = first ? r[i] : fma_t(beta, p[i], r[i]);
        if (ps) ps[i] = first ? rs[i] : fma_t(beta, ps[i], rs[i]);
    }
}

// local sums in the fast reduction order; out[0..NV) in device memory
enum SumMode {
    kSum = 0,        // sum a
    kDot = 1,        // (a, b)
    kNfL2 = 2,       // sum (a - b)^2, sum (c - b)^2                     (NV 2)
    kResidual = 3,   // c = a - b; (c, c)
    kUpdate = 4,     // x += s p; r -= s q; (r, r)
    kNfL1 = 5,       // sum |a - s b| + |c - s b|
    kDot2 = 6,       // (a, b), (b, b)                                   (NV 2)
    kBicgRho = 7,    // c -= s b; (a, c)
    kPcgUpdate = 8,  // x += s p; r -= s q; c = w .* r; (r, r), (r, c)   (NV 2)
    kScaledRes = 9,  // c = w .* (a - b); (c, c)
};

struct DdArgs {
    int n, mode;
    double s;
    const double *a, *b, *w;
    double *c, *x, *r;
    const double *p, *q;
    double *partials;
    int stride;
    uint32_t *counter;
    double *out;
};

template <int NV>
__global__ void __launch_bounds__(kBlock) k_dd_sum(DdArgs d)
{
    double acc[NV];
#pragma unroll
    for (int i = 0; i < NV; ++i) acc[i] = 0.0;
    CF_FOR_ELEMS(i, d.n) {
        switch (d.mode) {
        case kSum: acc[0] += d.a[i]; break;
        case kDot: acc[0] = fma_t(d.a[i], d.b[i], acc[0]); break;
        case kNfL2: {
            const double u = d.a[i] - d.b[i], v = d.c[i] - d.b[i];
            acc[0] = fma_t(u, u, acc[0]);
            acc[NV - 1] = fma_t(v, v, acc[NV - 1]);
            break;
        }
        case kResidual: {
            const double ri = d.a[i] - d.b[i];
            d.c[i] = ri;
            acc[0] = fma_t(ri, ri, acc[0]);
            break;
        }
        case kUpdate: {
            d.x[i] = fma_t(d.s, d.p[i], d.x[i]);
            const double ri = fma_t(-d.s, d.q[i], d.r[i]);
            d.r[i] = ri;
            acc[0] = fma_t(ri, ri, acc[0]);
            break;
        }
        case kNfL1: {
            const double yb = __dmul_rn(d.b[i], d.s);
            acc[0] = acc[0] + (fabs(d.a[i] - yb) + fabs(d.c[i] - yb));
            break;
        }
        case kDot2: {
            const double bi = d.b[i];
            acc[0] = fma_t(d.a[i], bi, acc[0]);
            acc[NV - 1] = fma_t(bi, bi, acc[NV - 1]);
            break;
        }
        case kBicgRho: {
            const double ci = fma_t(-d.s, d.b[i], d.c[i]);
            d.c[i] = ci;
            acc[0] = fma_t(d.a[i], ci, acc[0]);
            break;
        }
        case kPcgUpdate: {
            d.x[i] = fma_t(d.s, d.p[i], d.x[i]);
            const double ri = fma_t(-d.s, d.q[i], d.r[i]);
            d.r[i] = ri;
            const double zi = __dmul_rn(d.w[i], ri);
            d.c[i] = zi;
            acc[0] = fma_t(ri, ri, acc[0]);
            acc[NV - 1] = fma_t(ri, zi, acc[NV - 1]);
            break;
        }
        default: {   // kScaledRes
            const double ri = __dmul_rn(d.w[i], d.a[i] - d.b[i]);
            d.c[i] = ri;
            acc[0] = fma_t(ri, ri, acc[0]);
            break;
        }
        }
    }
    double tot[NV];
    if (grid_reduce<NV, double>(acc, d.partials, d.stride, d.counter, false, tot) && threadIdx.x == 0)
#pragma unroll
        for (int i = 0; i < NV; ++i) d.out[i] = tot[i];
}

// One decomposed solve: the subdomain's matrix, its interfaces, the
// caller's transfers, and the device workspace of the call.
class Decomposed {
public:
    // workspace vectors
    enum { kR, kP, kQ, kRs, kPs, kQs, kZ, kNf0, kNf1, kNf2, kNVec };

    Decomposed(Matrix *m, const cf_interfaces &ifc, const cf_comm &comm)
        : m_(m), ctx_(m->ctx), comm_(comm), n_(m->n), nfi_(ifc.n_faces)
    {
        require(n_ > 0 && nfi_ >= 0, CF_BAD_INPUT, "bad sizes");
        require(nfi_ == 0 || (ifc.face_cells && ifc.coeffs), CF_BAD_INPUT, "interface arrays are null");
        // coupled cells and their faces, in the order given
        std::vector<std::vector<int32_t>> faces_of((size_t)n_);
        for (int f = 0; f < nfi_; ++f) {
            const int cc = ifc.face_cells[f];
            require(cc >= 0 && cc < n_, CF_BAD_INPUT, "interface face cell out of range");
            faces_of[(size_t)cc].push_back(f);
        }
        std::vector<int32_t> h_cell, h_start(1, 0), h_face;
        for (int cc = 0; cc < n_; ++cc) {
            if (faces_of[(size_t)cc].empty()) continue;
            h_cell.push_back(cc);
            for (int32_t f : faces_of[(size_t)cc]) h_face.push_back(f);
            h_start.push_back((int32_t)h_face.size());
        }
        nc_ = (int)h_cell.size();
        const size_t mb = sizeof(double) * ((size_t)nfi_ + 1);
        fcells_.ensure(sizeof(int32_t) * ((size_t)nfi_ + 1));
        coeff_.ensure(mb);
        coeffT_.ensure(mb);
        ghost_.ensure(mb);
        send_.ensure(mb);
        cell_.ensure(sizeof(int32_t) * ((size_t)nc_ + 1));
        start_.ensure(sizeof(int32_t) * ((size_t)nc_ + 2));
        face_.ensure(sizeof(int32_t) * ((size_t)nfi_ + 1));
        stride_ = ctx_->sm_count * 8;
        partials_.ensure(sizeof(double) * kMaxNV * (size_t)stride_);
        counter_.ensure(sizeof(uint32_t) * 4);
        out_.ensure(sizeof(double) * 4);
        CF_CUDA(cudaMemsetAsync(counter_.ptr, 0, sizeof(uint32_t) * 4, ctx_->stream));
        if (nfi_ > 0) {
            upload(ctx_, fcells_.ptr, ifc.face_cells, sizeof(int32_t) * nfi_, CF_MEM_HOST);
            upload(ctx_, coeff_.ptr, ifc.coeffs, sizeof(double) * nfi_, CF_MEM_HOST);
            upload(ctx_, face_.ptr, h_face.data(), sizeof(int32_t) * nfi_, CF_MEM_HOST);
        }
        if (nc_ > 0) {
            upload(ctx_, cell_.ptr, h_cell.data(), sizeof(int32_t) * nc_, CF_MEM_HOST);
            upload(ctx_, start_.ptr, h_start.data(), sizeof(int32_t) * (nc_ + 1), CF_MEM_HOST);
        }
        h_send_.assign((size_t)nfi_ + 1, 0.0);
        h_recv_.assign((size_t)nfi_ + 1, 0.0);
        h_coeff_.assign(ifc.coeffs, ifc.coeffs + nfi_);
        h_coeff_.push_back(0.0);
        grid_ = ctx_->fast_grid((const void *)k_dd_sum<2>, 0);
        egrid_ = ctx_->fast_grid((const void *)k_dd_dir, 0);
        for (DeviceBuffer &v : vec_) v.ensure(sizeof(double) * ((size_t)n_ + 8));
    }

    double *vec(int i) { return vec_[i].as<double>(); }
    int egrid() const { return egrid_; }
    cudaStream_t stream() const { return ctx_->stream; }

    void allreduce(double *v, int cnt) { check(comm_.allreduce_sum(comm_.user, v, cnt), "all-reduce"); }

    double allreduce_max(double v)
    {
        require(comm_.allreduce_max != nullptr, CF_UNSUPPORTED,
                "this solve needs a maximum over the ranks: cf_comm.allreduce_max is not set");
        check(comm_.allreduce_max(comm_.user, &v, 1), "maximum");
        return v;
    }

    // the local sums of one pass, summed over the ranks
    void sums(DdArgs d, int nv, double *h)
    {
        d.n = n_;
        d.partials = partials_.as<double>();
        d.stride = stride_;
        d.counter = counter_.as<uint32_t>();
        d.out = out_.as<double>();
        if (nv == 1) k_dd_sum<1><<<grid_, kBlock, 0, ctx_->stream>>>(d);
        else k_dd_sum<2><<<grid_, kBlock, 0, ctx_->stream>>>(d);
        CF_CHECK_LAUNCH();
        CF_CUDA(cudaMemcpyAsync(h, out_.ptr, sizeof(double) * nv, cudaMemcpyDeviceToHost, ctx_->stream));
        CF_CUDA(cudaStreamSynchronize(ctx_->stream));
        allreduce(h, nv);
    }

    double dot(const double *u, const double *v)
    {
        DdArgs d{};
        d.mode = kDot;
        d.a = u;
        d.b = v;
        double s = 0.0;
        sums(d, 1, &s);
        return s;
    }

    // the neighbours' coefficients of the same faces: A^T's coupling
    void prepare_transpose()
    {
        if (have_T_) return;
        check(comm_.exchange(comm_.user, h_coeff_.data(), h_recv_.data(), nfi_), "exchange");
        if (nfi_ > 0) upload(ctx_, coeffT_.ptr, h_recv_.data(), sizeof(double) * nfi_, CF_MEM_HOST);
        have_T_ = true;
    }

    // o = A v (or A^T v) with the interface terms: the ghosts are the
    // neighbours' values of v (exchange) or, for a constant vector, the
    // constant itself (no exchange)
    void apply(const double *v, double *o, bool transpose = false, bool constant = false, double cval = 0.0)
    {
        if (nfi_ > 0) {
            if (constant) {
                k_dd_fill<<<egrid_, kBlock, 0, ctx_->stream>>>(nfi_, cval, ghost_.as<double>());
            } else {
                k_dd_gather<<<egrid_, kBlock, 0, ctx_->stream>>>(nfi_, fcells_.as<int32_t>(), v,
                                                                  send_.as<double>());
                CF_CHECK_LAUNCH();
                CF_CUDA(cudaMemcpyAsync(h_send_.data(), send_.ptr, sizeof(double) * nfi_, cudaMemcpyDeviceToHost,
                                        ctx_->stream));
                CF_CUDA(cudaStreamSynchronize(ctx_->stream));
                check(comm_.exchange(comm_.user, h_send_.data(), h_recv_.data(), nfi_), "exchange");
                upload(ctx_, ghost_.ptr, h_recv_.data(), sizeof(double) * nfi_, CF_MEM_HOST);
            }
            CF_CHECK_LAUNCH();
        } else if (!constant) {
            // a rank without processor faces still takes part in every exchange
            check(comm_.exchange(comm_.user, h_send_.data(), h_recv_.data(), 0), "exchange");
        }
        spmv(m_, transpose, v, o, false);
        if (nc_ > 0) {
            k_dd_iface<<<egrid_, kBlock, 0, ctx_->stream>>>(nc_, cell_.as<int32_t>(), start_.as<int32_t>(),
                                                             face_.as<int32_t>(),
                                                             (transpose ? coeffT_ : coeff_).as<double>(),
                                                             ghost_.as<double>(), o);
            CF_CHECK_LAUNCH();
        }
    }

    // normFactor of the whole mesh (gis/gis.cu:106-123; OpenFOAM's L1 form
    // as an option) and the whole mesh's row count
    double norm_factor(const double *x, const double *b, bool l1, double *n_global)
    {
        double sx[2] = {0.0, (double)n_};
        {
            DdArgs d{};
            d.mode = kSum;
            d.a = x;
            d.n = n_;
            d.partials = partials_.as<double>();
            d.stride = stride_;
            d.counter = counter_.as<uint32_t>();
            d.out = out_.as<double>();
            k_dd_sum<1><<<grid_, kBlock, 0, ctx_->stream>>>(d);
            CF_CHECK_LAUNCH();
            CF_CUDA(cudaMemcpyAsync(sx, out_.ptr, sizeof(double), cudaMemcpyDeviceToHost, ctx_->stream));
            CF_CUDA(cudaStreamSynchronize(ctx_->stream));
            allreduce(sx, 2);
        }
        *n_global = sx[1];
        const double xbar = sx[0] / sx[1];
        double *y = vec(kNf0), *ybar = vec(kNf1), *cv = vec(kNf2);
        apply(x, y);                                        // A x
        // L2: A (xbar 1); L1: (A 1) xbar
        const double cval = l1 ? 1.0 : xbar;
        k_dd_fill<<<egrid_, kBlock, 0, ctx_->stream>>>(n_, cval, cv);
        CF_CHECK_LAUNCH();
        apply(cv, ybar, false, true, cval);
        double dd[2] = {0.0, 0.0};
        DdArgs d{};
        d.mode = l1 ? kNfL1 : kNfL2;
        d.s = xbar;
        d.a = y;
        d.b = ybar;
        d.c = const_cast<double *>(b);
        sums(d, l1 ? 1 : 2, dd);
        return l1 ? dd[0] + 1e-20 : std::sqrt(dd[0]) + std::sqrt(dd[1]) + 1e-20;
    }

private:
    static void check(int32_t rc, const char *what)
    {
        require(rc == 0, CF_BAD_INPUT, std::string("the ") + what + " callback failed");
    }

    Matrix *m_;
    Context *ctx_;
    cf_comm comm_;
    int n_, nfi_, nc_ = 0, stride_ = 0, grid_ = 0, egrid_ = 0;
    bool have_T_ = false;
    DeviceBuffer fcells_, coeff_, coeffT_, ghost_, send_, cell_, start_, face_, partials_, counter_, out_;
    DeviceBuffer vec_[kNVec];
    std::vector<double> h_send_, h_recv_, h_coeff_;
};

// The stopping rule of the library's loops (finish_init / finish_step):
// continue while ||r|| > tol (or fewer than min_iter steps) and fewer than
// max steps; the time limit ends the loop with CF_TIMEOUT.
struct Loop {
    const cf_controls &c;
    double tol;
    int max_steps, min_steps;
    int hist_len = 0;
    int k = 0;
    bool timed_out = false;
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();

    Loop(const cf_controls &cc, double tol_) : c(cc), tol(tol_)
    {
        max_steps = c.max_iter <= 0 ? INT_MAX : c.max_iter;
        min_steps = c.min_iter > 0 ? c.min_iter : 0;
    }
    void record(double norm)
    {
        if (c.history && c.history_capacity > 0 && hist_len < c.history_capacity) c.history[hist_len++] = norm;
    }
    bool more(double norm) const { return std::isfinite(norm) && (norm > tol || k < min_steps); }
    bool go(double norm)
    {
        if (c.time_limit_s > 0 &&
            std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count() > c.time_limit_s) {
            timed_out = true;
            return false;
        }
        return k < max_steps && more(norm);
    }
    int status(double norm, bool breakdown) const
    {
        if (timed_out) return CF_TIMEOUT;
        if (breakdown) return CF_BREAKDOWN;
        return !std::isfinite(norm) ? CF_NONFINITE : (norm > tol ? CF_NOT_CONVERGED : CF_OK);
    }
};

} // namespace

void solve_distributed(Matrix *m, int solver, const cf_controls &c, const cf_interfaces &ifc,
                       const cf_comm &comm, const double *b_in, double *x_io, cf_perf *perf)
{
    Context *ctx = m->ctx;
    require(solver >= CF_CG && solver <= CF_PCG, CF_BAD_INPUT, "unknown solver");
    require(b_in && x_io, CF_BAD_INPUT, "source and psi must not be null");
    require(comm.allreduce_sum && comm.exchange, CF_BAD_INPUT, "the communication callbacks are required");
    require(c.memory == CF_MEM_HOST || c.memory == CF_MEM_DEVICE, CF_BAD_INPUT, "bad memory kind");
    require(c.precision == CF_PREC_FP64, CF_UNSUPPORTED, "decomposed solves are FP64 only");
    require(!c.transpose, CF_UNSUPPORTED, "decomposed solves of A^T are not implemented");
    const int n = m->n;
    const GridCap small(ctx, n);
    Decomposed D(m, ifc, comm);
    const int eg = D.egrid();
    cudaStream_t st = D.stream();
    DeviceBuffer dx, db;
    double *x, *b;
    if (c.memory == CF_MEM_HOST) {
        dx.ensure(sizeof(double) * ((size_t)n + 8));
        db.ensure(sizeof(double) * ((size_t)n + 8));
        x = dx.as<double>();
        b = db.as<double>();
        upload(ctx, x, x_io, sizeof(double) * n, CF_MEM_HOST);
        upload(ctx, b, b_in, sizeof(double) * n, CF_MEM_HOST);
    } else {
        x = x_io;
        b = const_cast<double *>(b_in);
    }
    const double *dinv = m->dinv.as<double>();
    const double *dsq = m->dinv_sqrt.as<double>();
    double *r = D.vec(Decomposed::kR), *p = D.vec(Decomposed::kP), *q = D.vec(Decomposed::kQ);
    double *rs = D.vec(Decomposed::kRs), *ps = D.vec(Decomposed::kPs), *qs = D.vec(Decomposed::kQs);
    double *z = D.vec(Decomposed::kZ);

    CF_CUDA(cudaEventRecord(ctx->ev_start, st));
    double n_global = 0.0;
    const double nf = D.norm_factor(x, b, c.norm_type == CF_NORM_OPENFOAM_L1, &n_global);
    Loop L(c, c.absolute_tolerance ? c.tolerance : c.tolerance * nf);

    // r = b - A x (JMR: r = D^-1/2 (b - A x)); returns (r, r)
    auto residual = [&]() {
        D.apply(x, q);
        DdArgs d{};
        d.mode = solver == CF_JMR ? kScaledRes : kResidual;
        d.a = b;
        d.b = q;
        d.c = r;
        d.w = dsq;
        double rr = 0.0;
        D.sums(d, 1, &rr);
        return rr;
    };
    double omega_used = 0.0;
    if (solver == CF_RICHARDSON) {
        double omega = c.richardson_omega;
        if (omega > -1e-15 && omega < 1e-15) {
            // OptimizePower on the whole mesh: x2 = 1/N, then x2 = A x1 / ||A x1||
            double *x1 = p, *x2 = q;
            k_dd_fill<<<eg, kBlock, 0, st>>>(n, 1.0 / n_global, x2);
            CF_CHECK_LAUNCH();
            const int steps = c.power_max_steps > 0 ? c.power_max_steps : 30;
            for (int s = 0; s < steps; ++s) {
                std::swap(x1, x2);
                D.apply(x1, x2);
                const double nx2 = std::sqrt(D.dot(x2, x2));
                k_dd_scale<<<eg, kBlock, 0, st>>>(n, nullptr, 1 / nx2, x2, x2);
                CF_CHECK_LAUNCH();
            }
            D.apply(x2, z);
            const double lmax = D.dot(x2, z);
            matrix_ensure_dmin(m);
            const double dmin = -D.allreduce_max(-m->diag_abs_min);
            omega = 2.0 / (lmax + dmin);
        }
        omega_used = omega;
    }
    double norm = std::sqrt(residual());
    if (c.rel_tol > 0.0) L.tol = std::max(L.tol, c.rel_tol * norm);
    const double norm0 = norm;
    L.record(norm);
    bool breakdown = false;

    if (solver == CF_CG || solver == CF_PCG) {
        const bool pcg = solver == CF_PCG;
        double rho0 = norm * norm, rho1 = 0.0;
        if (pcg) {
            k_dd_scale<<<eg, kBlock, 0, st>>>(n, dinv, 0.0, r, z);
            CF_CHECK_LAUNCH();
            rho0 = D.dot(r, z);
        }
        while (L.go(norm)) {
            ++L.k;
            k_dd_dir<<<eg, kBlock, 0, st>>>(n, L.k == 1, L.k == 1 ? 0.0 : rho0 / rho1, pcg ? z : r, p, nullptr,
                                            nullptr);
            CF_CHECK_LAUNCH();
            D.apply(p, q);
            const double xi = rho0 / D.dot(p, q);
            DdArgs d{};
            d.mode = pcg ? kPcgUpdate : kUpdate;
            d.s = xi;
            d.x = x;
            d.r = r;
            d.p = p;
            d.q = q;
            d.w = dinv;
            d.c = z;
            double t[2] = {0.0, 0.0};
            D.sums(d, pcg ? 2 : 1, t);
            rho1 = rho0;
            rho0 = pcg ? t[1] : t[0];
            norm = std::sqrt(t[0]);
            L.record(norm);
        }
    } else if (solver == CF_BICG) {
        D.prepare_transpose();
        CF_CUDA(cudaMemcpyAsync(rs, r, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
        CF_CUDA(cudaMemcpyAsync(p, r, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
        CF_CUDA(cudaMemcpyAsync(ps, r, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
        double rho0 = D.dot(r, rs);
        const double bound = c.bicg_int_bound > 0 ? c.bicg_int_bound : 1e-10;
        // the first step always runs (SolverSingleGPU.h:568-675)
        bool first = L.max_steps >= 1 && std::isfinite(norm);
        while (first || L.go(norm)) {
            first = false;
            ++L.k;
            D.apply(p, q);
            const double xi = rho0 / D.dot(ps, q);
            if (xi > -bound && xi < bound) {
                breakdown = true;
                break;
            }
            DdArgs d{};
            d.mode = kUpdate;
            d.s = xi;
            d.x = x;
            d.r = r;
            d.p = p;
            d.q = q;
            double t = 0.0;
            D.sums(d, 1, &t);
            norm = std::sqrt(t);
            L.record(norm);
            if (!L.more(norm) || L.k >= L.max_steps) break;
            D.apply(ps, qs, true);
            DdArgs e{};
            e.mode = kBicgRho;
            e.s = xi;
            e.a = r;
            e.b = qs;
            e.c = rs;
            const double rho1 = rho0;
            D.sums(e, 1, &rho0);
            k_dd_dir<<<eg, kBlock, 0, st>>>(n, 0, rho0 / rho1, r, p, rs, ps);
            CF_CHECK_LAUNCH();
        }
    } else if (solver == CF_RICHARDSON) {
        while (L.go(norm)) {
            ++L.k;
            k_dd_axpy<<<eg, kBlock, 0, st>>>(n, omega_used, r, x);
            CF_CHECK_LAUNCH();
            norm = std::sqrt(residual());
            L.record(norm);
        }
    } else {
        // the MR family and Jacobi: d = R r, y = A d (JMR: y = D^-1/2 A d),
        // alpha = (r, y) / (y, y) (Jacobi: 1), x += alpha d, r -= alpha y
        const double *w = solver == CF_MR ? nullptr : (solver == CF_JMR ? dsq : dinv);
        while (L.go(norm)) {
            ++L.k;
            k_dd_scale<<<eg, kBlock, 0, st>>>(n, w, 1.0, r, p);
            CF_CHECK_LAUNCH();
            D.apply(p, q);
            if (solver == CF_JMR) {
                k_dd_scale<<<eg, kBlock, 0, st>>>(n, dsq, 0.0, q, q);
                CF_CHECK_LAUNCH();
            }
            double alpha = 1.0;
            if (solver != CF_JACOBI) {
                DdArgs d{};
                d.mode = kDot2;
                d.a = r;
                d.b = q;
                double t[2] = {0.0, 0.0};
                D.sums(d, 2, t);
                alpha = t[0] / t[1];
            }
            DdArgs d{};
            d.mode = kUpdate;
            d.s = alpha;
            d.x = x;
            d.r = r;
            d.p = p;
            d.q = q;
            double t = 0.0;
            D.sums(d, 1, &t);
            norm = std::sqrt(t);
            L.record(norm);
        }
    }
    const int status = L.status(norm, breakdown);
    CF_CUDA(cudaEventRecord(ctx->ev_stop, st));
    if (c.memory == CF_MEM_HOST) download(ctx, x_io, x, sizeof(double) * n, CF_MEM_HOST);
    CF_CUDA(cudaStreamSynchronize(st));
    float ms = 0.f;
    CF_CUDA(cudaEventElapsedTime(&ms, ctx->ev_start, ctx->ev_stop));
    if (perf) {
        *perf = cf_perf{};
        perf->norm_factor = nf;
        perf->initial_residual_abs = norm0;
        perf->final_residual_abs = norm;
        perf->initial_residual = norm0 / nf;
        perf->final_residual = norm / nf;
        perf->n_iterations = L.k;
        perf->status = status;
        perf->history_length = L.hist_len;
        perf->solve_ms = ms;
        perf->true_residual = -1.0;
        perf->omega = omega_used;
    }
}

} // namespace cf
