// distributed.cu -- CG on one subdomain of a decomposed case (one rank per
// GPU, OpenFOAM's processor patches).
//
// OpenFOAM's lduMatrix::Amul on a decomposed mesh forms the local product
// and then, per processor patch, subtracts interfaceBouCoeffs[f] times the
// neighbouring rank's value of the cell on the far side of face f from the
// product's row faceCells[f] (initMatrixInterfaces /
// updateMatrixInterfaces); its dot products and normFactor sum over all
// ranks.  This is OpenFOAM's semantics restated (its sources are not
// available here, and the reference ignores interfaces altogether --
// cuFoamCG/cuFoamCG.C:27-33).  The solve here:
//   * before every product, the values of the product's input at the patch
//     faces' cells are gathered on the device, handed to the caller's
//     exchange callback, and the neighbours' values come back as ghosts;
//   * the product is the local SpMV (fast order) followed by one pass that
//     subtracts coeff * ghost per face, the faces of a cell in the order
//     given (patch order, then face order, as OpenFOAM loops);
//   * every dot product is a local deterministic sum handed to the caller's
//     all-reduce callback.
// The driver is host-paced: three host round trips per CG step (exchange
// and two reductions), which a decomposed run pays in its communication
// anyway.  The loop follows the reference's CG (SolverSingleGPU.h:366-445):
// stop when ||r||_2 <= tolerance * normFactor or after maxIter steps.
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

// local sums in the fast reduction order; out[0..NV) in device memory
//   mode 0: sum a;  1: (a, b);  2: sum (a - b)^2, sum (c - b)^2
//   3: r = a - b (into c), (r, r);  4: x += s p, r -= s q, (r, r)
//   5: sum |a - s b| + |c - s b|  (OpenFOAM's L1 normFactor)
struct DdArgs {
    int n, mode;
    double s;
    const double *a, *b;
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
        if (d.mode == 0) {
            acc[0] += d.a[i];
        } else if (d.mode == 1) {
            acc[0] = fma_t(d.a[i], d.b[i], acc[0]);
        } else if (d.mode == 2) {
            const double u = d.a[i] - d.b[i], v = d.c[i] - d.b[i];
            acc[0] = fma_t(u, u, acc[0]);
            if (NV > 1) acc[NV - 1] = fma_t(v, v, acc[NV - 1]);
        } else if (d.mode == 5) {
            const double yb = __dmul_rn(d.b[i], d.s);
            acc[0] = acc[0] + (fabs(d.a[i] - yb) + fabs(d.c[i] - yb));
        } else if (d.mode == 3) {
            const double ri = d.a[i] - d.b[i];
            d.c[i] = ri;
            acc[0] = fma_t(ri, ri, acc[0]);
        } else {
            d.x[i] = fma_t(d.s, d.p[i], d.x[i]);
            const double ri = fma_t(-d.s, d.q[i], d.r[i]);
            d.r[i] = ri;
            acc[0] = fma_t(ri, ri, acc[0]);
        }
    }
    double tot[NV];
    if (grid_reduce<NV, double>(acc, d.partials, d.stride, d.counter, false, tot) && threadIdx.x == 0)
#pragma unroll
        for (int i = 0; i < NV; ++i) d.out[i] = tot[i];
}

// p = r (first step) or p = r + beta p
__global__ void __launch_bounds__(kBlock) k_dd_dir(int n, int first, double beta, const double *__restrict__ r,
                                                   double *__restrict__ p)
{
    CF_FOR_ELEMS(i, n) p[i] = first ? r[i] : fma_t(beta, p[i], r[i]);
}

} // namespace

void solve_distributed(Matrix *m, int solver, const cf_controls &c, const cf_interfaces &ifc,
                       const cf_comm &comm, const double *b_in, double *x_io, cf_perf *perf)
{
    Context *ctx = m->ctx;
    require(solver == CF_CG, CF_UNSUPPORTED,
            "decomposed (processor-patch) solves are implemented for CG only");
    require(b_in && x_io, CF_BAD_INPUT, "source and psi must not be null");
    require(comm.allreduce_sum && comm.exchange, CF_BAD_INPUT, "the communication callbacks are required");
    require(c.memory == CF_MEM_HOST || c.memory == CF_MEM_DEVICE, CF_BAD_INPUT, "bad memory kind");
    require(c.precision == CF_PREC_FP64, CF_UNSUPPORTED, "decomposed solves are FP64 only");
    require(!c.transpose, CF_UNSUPPORTED, "decomposed solves of A^T are not implemented");
    const int n = m->n;
    const int nfi = ifc.n_faces;
    require(n > 0 && nfi >= 0, CF_BAD_INPUT, "bad sizes");
    require(nfi == 0 || (ifc.face_cells && ifc.coeffs), CF_BAD_INPUT, "interface arrays are null");

    // ---- coupled cells and their faces, in the order given --------------
    std::vector<std::vector<int32_t>> faces_of((size_t)n);
    for (int f = 0; f < nfi; ++f) {
        const int cc = ifc.face_cells[f];
        require(cc >= 0 && cc < n, CF_BAD_INPUT, "interface face cell out of range");
        faces_of[(size_t)cc].push_back(f);
    }
    std::vector<int32_t> h_cell, h_start(1, 0), h_face;
    for (int cc = 0; cc < n; ++cc) {
        if (faces_of[(size_t)cc].empty()) continue;
        h_cell.push_back(cc);
        for (int32_t f : faces_of[(size_t)cc]) h_face.push_back(f);
        h_start.push_back((int32_t)h_face.size());
    }
    const int nc = (int)h_cell.size();

    // ---- workspace (per call; nothing per step) ---------------------------
    const size_t vb = sizeof(double) * ((size_t)n + 8);
    DeviceBuffer dx, db, dr, dp, dq, dy, dt, fcells, coeff, ghost, send, cell, start, face, partials, counter, out;
    for (DeviceBuffer *v : {&dr, &dp, &dq, &dy, &dt}) v->ensure(vb);
    const size_t mb = sizeof(double) * ((size_t)nfi + 1);
    fcells.ensure(sizeof(int32_t) * ((size_t)nfi + 1));
    coeff.ensure(mb);
    ghost.ensure(mb);
    send.ensure(mb);
    cell.ensure(sizeof(int32_t) * ((size_t)nc + 1));
    start.ensure(sizeof(int32_t) * ((size_t)nc + 2));
    face.ensure(sizeof(int32_t) * ((size_t)nfi + 1));
    const int stride = ctx->sm_count * 8;
    partials.ensure(sizeof(double) * kMaxNV * (size_t)stride);
    counter.ensure(sizeof(uint32_t) * 4);
    out.ensure(sizeof(double) * 4);
    CF_CUDA(cudaMemsetAsync(counter.ptr, 0, sizeof(uint32_t) * 4, ctx->stream));
    if (nfi > 0) {
        upload(ctx, fcells.ptr, ifc.face_cells, sizeof(int32_t) * nfi, CF_MEM_HOST);
        upload(ctx, coeff.ptr, ifc.coeffs, sizeof(double) * nfi, CF_MEM_HOST);
        upload(ctx, face.ptr, h_face.data(), sizeof(int32_t) * nfi, CF_MEM_HOST);
    }
    if (nc > 0) {
        upload(ctx, cell.ptr, h_cell.data(), sizeof(int32_t) * nc, CF_MEM_HOST);
        upload(ctx, start.ptr, h_start.data(), sizeof(int32_t) * (nc + 1), CF_MEM_HOST);
    }
    double *x, *b;
    if (c.memory == CF_MEM_HOST) {
        dx.ensure(vb);
        db.ensure(vb);
        x = dx.as<double>();
        b = db.as<double>();
        upload(ctx, x, x_io, sizeof(double) * n, CF_MEM_HOST);
        upload(ctx, b, b_in, sizeof(double) * n, CF_MEM_HOST);
    } else {
        x = x_io;
        b = const_cast<double *>(b_in);
    }
    std::vector<double> h_send((size_t)nfi + 1), h_recv((size_t)nfi + 1);
    const GridCap small(ctx, n);
    const int grid = ctx->fast_grid((const void *)k_dd_sum<2>, 0);
    const int egrid = ctx->fast_grid((const void *)k_dd_dir, 0);

    auto check_comm = [](int32_t rc, const char *what) {
        require(rc == 0, CF_BAD_INPUT, std::string("the ") + what + " callback failed");
    };
    auto allreduce = [&](double *v, int cnt) { check_comm(comm.allreduce_sum(comm.user, v, cnt), "all-reduce"); };
    auto local_sums = [&](DdArgs d, int nv, double *h) {
        d.n = n;
        d.partials = partials.as<double>();
        d.stride = stride;
        d.counter = counter.as<uint32_t>();
        d.out = out.as<double>();
        if (nv == 1) k_dd_sum<1><<<grid, kBlock, 0, ctx->stream>>>(d);
        else k_dd_sum<2><<<grid, kBlock, 0, ctx->stream>>>(d);
        CF_CHECK_LAUNCH();
        CF_CUDA(cudaMemcpyAsync(h, out.ptr, sizeof(double) * nv, cudaMemcpyDeviceToHost, ctx->stream));
        CF_CUDA(cudaStreamSynchronize(ctx->stream));
    };
    auto global_dot = [&](const double *u, const double *v) {
        DdArgs d{};
        d.mode = 1;
        d.a = u;
        d.b = v;
        double s = 0.0;
        local_sums(d, 1, &s);
        allreduce(&s, 1);
        return s;
    };
    // out = A v with the interface terms: the ghosts are the neighbours'
    // values of v (exchange) or, for the constant vector of normFactor, the
    // constant itself
    auto apply = [&](const double *v, double *o, bool constant, double cval) {
        if (nfi > 0) {
            if (constant) {
                k_dd_fill<<<egrid, kBlock, 0, ctx->stream>>>(nfi, cval, ghost.as<double>());
            } else {
                k_dd_gather<<<egrid, kBlock, 0, ctx->stream>>>(nfi, fcells.as<int32_t>(), v, send.as<double>());
                CF_CHECK_LAUNCH();
                CF_CUDA(cudaMemcpyAsync(h_send.data(), send.ptr, sizeof(double) * nfi, cudaMemcpyDeviceToHost,
                                        ctx->stream));
                CF_CUDA(cudaStreamSynchronize(ctx->stream));
                check_comm(comm.exchange(comm.user, h_send.data(), h_recv.data(), nfi), "exchange");
                upload(ctx, ghost.ptr, h_recv.data(), sizeof(double) * nfi, CF_MEM_HOST);
            }
            CF_CHECK_LAUNCH();
        } else if (!constant) {
            // a rank without processor faces still takes part in every exchange
            check_comm(comm.exchange(comm.user, h_send.data(), h_recv.data(), 0), "exchange");
        }
        spmv(m, false, v, o, false);
        if (nc > 0) {
            k_dd_iface<<<egrid, kBlock, 0, ctx->stream>>>(nc, cell.as<int32_t>(), start.as<int32_t>(),
                                                           face.as<int32_t>(), coeff.as<double>(),
                                                           ghost.as<double>(), o);
            CF_CHECK_LAUNCH();
        }
    };

    CF_CUDA(cudaEventRecord(ctx->ev_start, ctx->stream));
    // ---- normFactor over all ranks (gis/gis.cu:106-123 on the whole mesh) --
    double sx[2] = {0.0, (double)n};
    {
        DdArgs d{};
        d.mode = 0;
        d.a = x;
        local_sums(d, 1, sx);
        allreduce(sx, 2);
    }
    const double xbar = sx[0] / sx[1];
    const bool l1 = c.norm_type == CF_NORM_OPENFOAM_L1;
    double *y = dy.as<double>(), *ybar = dt.as<double>();
    apply(x, y, false, 0.0);                                   // A x
    // L2 (gis/gis.cu:106-123): A (xbar 1); L1: (A 1) xbar
    const double cval = l1 ? 1.0 : xbar;
    k_dd_fill<<<egrid, kBlock, 0, ctx->stream>>>(n, cval, dq.as<double>());
    CF_CHECK_LAUNCH();
    apply(dq.as<double>(), ybar, true, cval);
    double dd[2] = {0.0, 0.0};
    {
        DdArgs d{};
        d.mode = l1 ? 5 : 2;
        d.s = xbar;
        d.a = y;
        d.b = ybar;
        d.c = b;
        local_sums(d, l1 ? 1 : 2, dd);
        allreduce(dd, l1 ? 1 : 2);
    }
    const double nf = l1 ? dd[0] + 1e-20 : std::sqrt(dd[0]) + std::sqrt(dd[1]) + 1e-20;
    double tol = c.absolute_tolerance ? c.tolerance : c.tolerance * nf;

    // ---- CG (SolverSingleGPU.h:366-445) ------------------------------------
    double *r = dr.as<double>(), *p = dp.as<double>(), *q = dq.as<double>();
    double rho0 = 0.0;
    {
        DdArgs d{};
        d.mode = 3;
        d.a = b;
        d.b = y;   // r = b - A x
        d.c = r;
        local_sums(d, 1, &rho0);
        allreduce(&rho0, 1);
    }
    const double norm0 = std::sqrt(rho0);
    if (c.rel_tol > 0.0) tol = std::max(tol, c.rel_tol * norm0);
    const int max_steps = c.max_iter <= 0 ? INT_MAX : c.max_iter;
    const bool want_hist = c.history && c.history_capacity > 0;
    if (want_hist) c.history[0] = norm0;
    int hist_len = want_hist ? 1 : 0;
    double norm = norm0, rho1 = 0.0;
    int k = 0, status = std::isfinite(norm0) ? CF_NOT_CONVERGED : CF_NONFINITE;
    auto wall0 = std::chrono::steady_clock::now();
    while (std::isfinite(norm) && k < max_steps && (norm > tol || k < c.min_iter)) {
        ++k;
        k_dd_dir<<<egrid, kBlock, 0, ctx->stream>>>(n, k == 1 ? 1 : 0, k == 1 ? 0.0 : rho0 / rho1, r, p);
        CF_CHECK_LAUNCH();
        apply(p, q, false, 0.0);
        const double xi = rho0 / global_dot(p, q);
        double rr = 0.0;
        {
            DdArgs d{};
            d.mode = 4;
            d.s = xi;
            d.x = x;
            d.r = r;
            d.p = p;
            d.q = q;
            local_sums(d, 1, &rr);
            allreduce(&rr, 1);
        }
        rho1 = rho0;
        rho0 = rr;
        norm = std::sqrt(rr);
        if (want_hist && hist_len < c.history_capacity) c.history[hist_len++] = norm;
        if (c.time_limit_s > 0 &&
            std::chrono::duration<double>(std::chrono::steady_clock::now() - wall0).count() > c.time_limit_s) {
            status = CF_TIMEOUT;
            break;
        }
    }
    if (status != CF_TIMEOUT)
        status = !std::isfinite(norm) ? CF_NONFINITE : (norm <= tol ? CF_OK : CF_NOT_CONVERGED);
    CF_CUDA(cudaEventRecord(ctx->ev_stop, ctx->stream));
    if (c.memory == CF_MEM_HOST) download(ctx, x_io, x, sizeof(double) * n, CF_MEM_HOST);
    CF_CUDA(cudaStreamSynchronize(ctx->stream));
    float ms = 0.f;
    CF_CUDA(cudaEventElapsedTime(&ms, ctx->ev_start, ctx->ev_stop));
    if (perf) {
        *perf = cf_perf{};
        perf->norm_factor = nf;
        perf->initial_residual_abs = norm0;
        perf->final_residual_abs = norm;
        perf->initial_residual = norm0 / nf;
        perf->final_residual = norm / nf;
        perf->n_iterations = k;
        perf->status = status;
        perf->history_length = hist_len;
        perf->solve_ms = ms;
        perf->true_residual = -1.0;
    }
}

} // namespace cf
