// gis_harness.cpp -- drives a libGIS.so through the gis.h interface the way
// the cuFoam plugins do (device SparseCSR / Vector containers built with
// cudaMalloc + cudaMemcpy, then one solver call), behind extern "C" entry
// points with plain host arrays so that tests can call it with ctypes.
// Built against SingleGPUCompat.h; the same source compiled against the
// reference's gis.h links to the same symbols.
#include <cuda_runtime.h>

#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#ifdef GH_REFERENCE_HEADER
#include "gis.h"
#else
#include "SingleGPUCompat.h"
#endif

namespace {

using CSR = SingleGPU::SparseCSR<ValueType, IndexType>;
using Vec = SingleGPU::Vector<ValueType, IndexType>;

thread_local std::string g_err;

void ck(cudaError_t e, const char *what)
{
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

template <class T> T *dev_copy(const T *h, size_t n)
{
    T *d = nullptr;
    ck(cudaMalloc(&d, sizeof(T) * (n ? n : 1)), "cudaMalloc");
    if (n) ck(cudaMemcpy(d, h, sizeof(T) * n, cudaMemcpyHostToDevice), "cudaMemcpy");
    return d;
}

void fill_csr(CSR &A, int n_rows, int n_cols, int nnz, const int *ro, const int *col, const double *val)
{
    A.num_rows = n_rows;
    A.num_cols = n_cols;
    A.num_entries = nnz;
    A.row_offsets = dev_copy(ro, (size_t)n_rows + 1);
    A.column_indices = dev_copy(col, (size_t)nnz);
    A.values = dev_copy(val, (size_t)nnz);
}

void fill_vec(Vec &v, int n, const double *h)
{
    v.size = n;
    v.capacity = n;
    v.values = dev_copy(h, (size_t)n);
}

template <class F> int guarded(F f)
{
    try {
        f();
        return 0;
    } catch (const std::invalid_argument &e) {
        g_err = e.what();
        return 2;
    } catch (const std::exception &e) {
        g_err = e.what();
        return 1;
    }
}

} // namespace

extern "C" {

const char *gh_last_error() { return g_err.c_str(); }

// Layout of the containers as this translation unit sees them:
// out[0..5] = sizeof(CSR), offsets of values, row_offsets, column_indices,
// num_rows, num_entries; out[6..8] = sizeof(Vec), offsets of size, capacity.
void gh_layout(long *out)
{
    out[0] = (long)sizeof(CSR);
    out[1] = (long)offsetof(CSR, values);
    out[2] = (long)offsetof(CSR, row_offsets);
    out[3] = (long)offsetof(CSR, column_indices);
    out[4] = (long)offsetof(CSR, num_rows);
    out[5] = (long)offsetof(CSR, num_entries);
    out[6] = (long)sizeof(Vec);
    out[7] = (long)offsetof(Vec, size);
    out[8] = (long)offsetof(Vec, capacity);
}

// name: CG BiCG BiCGAt Richardson MR Jacobi MRJacobi JMR MRS.  nb / nx:
// lengths of b and x (the containers get these sizes, so a mismatch with n
// reaches the library).  p_real: BiCG int_bound / Richardson omega; p_int:
// Richardson power steps.  detail_type: -1 none, 0 Error, 1 Time.
// *flag = BiCG's return value.
int gh_solve(const char *name, int n, int nnz, const int *ro, const int *col, const double *val,
             int nb, const double *b, int nx, double *x, double error, int max_steps, double p_real,
             int p_int, int detail_type, double *detail, int detail_cap, int *detail_len, int *flag)
{
    return guarded([&] {
        CSR A;
        fill_csr(A, n, n, nnz, ro, col, val);
        Vec vb, vx;
        fill_vec(vb, nb, b);
        fill_vec(vx, nx, x);
        std::vector<double> det;
        std::vector<double> *dp = detail_type >= 0 ? &det : nullptr;
        const DetailType dt = detail_type == 1 ? DetailType::Time : DetailType::Error;
        bool f = false;
        const std::string s(name);
        if (s == "CG") CG(&vx, A, vb, error, max_steps, dp, dt);
        else if (s == "BiCG") f = BiCG(&vx, A, vb, error, max_steps, p_real, dp, dt);
        else if (s == "BiCGAt") {
            CSR At = Transpose(A);
            f = BiCG(&vx, A, At, vb, error, max_steps, p_real, dp, dt);
        } else if (s == "Richardson") Richardson(&vx, A, vb, error, p_real, p_int, max_steps, dp, dt);
        else if (s == "MR") MR(&vx, A, vb, error, max_steps, dp, dt);
        else if (s == "Jacobi") Jacobi(&vx, A, vb, error, max_steps, dp, dt);
        else if (s == "MRJacobi") MRJacobi(&vx, A, vb, error, max_steps, dp, dt);
        else if (s == "JMR") JMR(&vx, A, vb, error, max_steps, dp, dt);
        else if (s == "MRS") {
            // the inverse diagonal as a CSR matrix, as cuFoamMRS builds it
            std::vector<int> iro((size_t)n + 1), icol((size_t)n);
            std::vector<double> iv((size_t)n, 0.0);
            for (int i = 0; i < n; ++i) {
                iro[(size_t)i] = i;
                icol[(size_t)i] = i;
                for (int j = ro[i]; j < ro[i + 1]; ++j)
                    if (col[j] == i) iv[(size_t)i] = 1.0 / val[j];
            }
            iro[(size_t)n] = n;
            CSR M;
            fill_csr(M, n, n, n, iro.data(), icol.data(), iv.data());
            MRS(&vx, A, vb, M, error, max_steps, dp, dt);
        } else throw std::invalid_argument("unknown solver " + s);
        ck(cudaMemcpy(x, vx.values, sizeof(double) * (size_t)nx, cudaMemcpyDeviceToHost), "cudaMemcpy");
        if (flag) *flag = f ? 1 : 0;
        if (detail_len) *detail_len = (int)det.size();
        if (detail)
            for (size_t i = 0; i < det.size() && (int)i < detail_cap; ++i) detail[i] = det[i];
    });
}

int gh_transpose(int n_rows, int n_cols, int nnz, const int *ro, const int *col, const double *val,
                 int *roT, int *colT, double *valT, int *shape)
{
    return guarded([&] {
        CSR A;
        fill_csr(A, n_rows, n_cols, nnz, ro, col, val);
        CSR T = Transpose(A);
        shape[0] = T.num_rows;
        shape[1] = T.num_cols;
        shape[2] = T.num_entries;
        ck(cudaMemcpy(roT, T.row_offsets, sizeof(int) * ((size_t)T.num_rows + 1), cudaMemcpyDeviceToHost),
           "cudaMemcpy");
        ck(cudaMemcpy(colT, T.column_indices, sizeof(int) * (size_t)nnz, cudaMemcpyDeviceToHost), "cudaMemcpy");
        ck(cudaMemcpy(valT, T.values, sizeof(double) * (size_t)nnz, cudaMemcpyDeviceToHost), "cudaMemcpy");
    });
}

int gh_norm_factor(int n, int nnz, const int *ro, const int *col, const double *val, const double *b,
                   const double *x, double *out)
{
    return guarded([&] {
        CSR A;
        fill_csr(A, n, n, nnz, ro, col, val);
        Vec vb, vx;
        fill_vec(vb, n, b);
        fill_vec(vx, n, x);
        *out = NormFactor(A, vb, vx);
    });
}

} // extern "C"
