// adjoint.cu -- gradient of a loss through A x = b with respect to the LDU
// coefficients, given the forward solution x and the adjoint solution
// lambda of A^T lambda = dL/dx:
//     dL/d diag[i]  = -lambda_i x_i
//     dL/d upper[f] = -lambda_own x_nbr      (upper[f] = A[own][nbr])
//     dL/d lower[f] = -lambda_nbr x_own      (lower[f] = A[nbr][own])
//     dL/d source   =  lambda
// One thread per face / per cell, each output written once: no atomics, so
// the result is deterministic.
#include "device.cuh"

namespace cf {

__global__ void __launch_bounds__(kBlock) k_adjoint_faces(int nf, const int32_t *__restrict__ la,
                                                          const int32_t *__restrict__ ua,
                                                          const double *__restrict__ lam,
                                                          const double *__restrict__ x,
                                                          double *d_lower, double *d_upper)
{
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < nf; f += gridDim.x * blockDim.x) {
        const int o = la[f], u = ua[f];
        if (d_upper) d_upper[f] = -(lam[o] * x[u]);
        if (d_lower) d_lower[f] = -(lam[u] * x[o]);
    }
}

__global__ void __launch_bounds__(kBlock) k_adjoint_cells(int n, const double *__restrict__ lam,
                                                          const double *__restrict__ x,
                                                          double *d_diag)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        d_diag[i] = -(lam[i] * x[i]);
}

void adjoint_gradients(Matrix *m, const double *lam, const double *x, double *d_diag,
                       double *d_lower, double *d_upper)
{
    Context *ctx = m->ctx;
    require(!m->from_csr, CF_UNSUPPORTED, "gradients need an LDU matrix (this one was created from CSR)");
    const int g = ctx->sm_count * 8;
    if (m->nf > 0 && (d_lower || d_upper)) {
        k_adjoint_faces<<<g, kBlock, 0, ctx->stream>>>(m->nf, m->la.as<int32_t>(), m->ua.as<int32_t>(),
                                                       lam, x, d_lower, d_upper);
        CF_CHECK_LAUNCH();
    }
    if (m->n > 0 && d_diag) {
        k_adjoint_cells<<<g, kBlock, 0, ctx->stream>>>(m->n, lam, x, d_diag);
        CF_CHECK_LAUNCH();
    }
}

} // namespace cf
