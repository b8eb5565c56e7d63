// gis_compat.cu -- a stand-in for the reference's solver library libGIS.so.
//
// Exports the non-template functions of gis/gis.h (gis/gis.cu:3-123) with
// the reference's C++ signatures, argument meaning and results, implemented
// on this library's device solvers, so that the unmodified cuFoam plugins
// (cuFoamCG/cuFoamCG.C and siblings) link against it in place of
// libGIS.so.  Their SparseCSR / Vector arguments hold device pointers
// (SingleGPUCompat.h gives the layouts).
//
//   * `error` is an absolute ||r||_2 threshold and `max_steps <= 0` means
//     no limit, as in the reference drivers (SolverSingleGPU.h).
//   * `detail` receives ||r||_2 before the first step and after every step
//     (DetailType::Error) or the seconds since the initial residual at the
//     end of every step, taken from the device clock (DetailType::Time).
//     At most 2^22 + 1 entries are kept.
//   * BiCG returns true when it stopped on the reference's breakdown test
//     (|xi| < int_bound), false otherwise.
//   * MRS takes invM as a matrix; the reference's plugin passes the inverse
//     diagonal (cuFoamMRS/cuFoamMRS.C), which is what this library solves
//     with -- any other pattern throws std::invalid_argument.
//   * Transpose returns A^T with its rows in ascending column order of A
//     (the reference's stable sort by column); arrays are cudaMalloc'd and
//     owned by the returned object.
//   * Reductions use the fast deterministic order; CUFOAM_GIS_REDUCTION=
//     reference selects the reference's summation order instead.
//   * Errors are thrown as std::invalid_argument (bad arguments) or
//     std::runtime_error (CUDA failures), like the reference's checks.
//
// Work runs on one stream per device and host thread, after the legacy
// default stream (where the plugins' own copies run) has drained; every
// call returns with its results in place.
#include "SingleGPUCompat.h"

#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>

#include "internal.h"

namespace {

using CSR = SingleGPU::SparseCSR<ValueType, IndexType>;
using Vec = SingleGPU::Vector<ValueType, IndexType>;

constexpr int kMaxDetail = (1 << 22) + 1;

// One context per (host thread, device), alive until the process exits:
// contexts are never destroyed, so no teardown runs after the CUDA runtime
// has shut down.
cf::Context *shim_context()
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        throw std::runtime_error("libGIS (cufoam_gb300): no CUDA device");
    }
    thread_local std::map<int, cf::Context *> ctxs;
    auto it = ctxs.find(dev);
    if (it != ctxs.end()) return it->second;
    cf::Context *c = cf::context_create(dev);
    ctxs[dev] = c;
    return c;
}

int reduction_order()
{
    const char *e = std::getenv("CUFOAM_GIS_REDUCTION");
    if (e && std::strcmp(e, "reference") == 0) return CF_REDUCE_REFERENCE;
    if (e && std::strcmp(e, "fast") == 0) return CF_REDUCE_FAST;
    return CF_REDUCE_AUTO;
}

[[noreturn]] void rethrow(const cf::Error &e)
{
    const std::string msg = "libGIS (cufoam_gb300): " + e.msg;
    if (e.status == CF_BAD_INPUT || e.status == CF_UNSUPPORTED) throw std::invalid_argument(msg);
    throw std::runtime_error(msg);
}

void check_system(const CSR &A, const Vec &b, const Vec *x)
{
    if (!x) throw std::invalid_argument("libGIS (cufoam_gb300): x must not be null");
    if (A.num_rows <= 0 || A.num_rows != A.num_cols)
        throw std::invalid_argument("libGIS (cufoam_gb300): A must be square and non-empty");
    if (b.size != A.num_rows || x->size != A.num_rows)
        throw std::invalid_argument("libGIS (cufoam_gb300): vector sizes do not match A");
    if (!A.values || !A.row_offsets || !A.column_indices || !b.values || !x->values)
        throw std::invalid_argument("libGIS (cufoam_gb300): null device array");
}

std::unique_ptr<cf::Matrix> device_matrix(cf::Context *ctx, const CSR &A)
{
    CF_CUDA(cudaStreamSynchronize(cudaStreamLegacy));
    return std::unique_ptr<cf::Matrix>(cf::matrix_from_csr(ctx, A.num_rows, A.num_entries, A.row_offsets,
                                                           A.column_indices, A.values));
}

struct SolveSpec {
    int solver = CF_CG;
    const CSR *At = nullptr;
    const CSR *invM = nullptr;
    double int_bound = 1e-10;
    double omega = 0.0;
    int power_steps = 30;
};

int run(const SolveSpec &s, Vec *x, const CSR &A, const Vec &b, double error, int max_steps,
        std::vector<double> *detail, DetailType detail_type)
{
    check_system(A, b, x);
    if (detail && detail_type != DetailType::Error && detail_type != DetailType::Time)
        throw std::runtime_error{"detail type must be one of Time and Error!"};
    try {
        cf::Context *ctx = shim_context();
        std::unique_ptr<cf::Matrix> m = device_matrix(ctx, A);
        if (s.At) {
            if (s.At->num_rows != A.num_cols || s.At->num_cols != A.num_rows ||
                s.At->num_entries != A.num_entries)
                throw std::invalid_argument("libGIS (cufoam_gb300): At is not the shape of A^T");
            cf::matrix_set_transpose_csr(m.get(), s.At->row_offsets, s.At->column_indices, s.At->values);
        }
        if (s.invM) {
            const CSR &M = *s.invM;
            if (M.num_rows != A.num_rows || M.num_cols != A.num_rows || M.num_entries != A.num_rows)
                throw std::invalid_argument("libGIS (cufoam_gb300): MRS needs a diagonal invM");
            std::vector<int32_t> ro((size_t)M.num_rows + 1), col((size_t)M.num_rows);
            CF_CUDA(cudaMemcpy(ro.data(), M.row_offsets, sizeof(int32_t) * ro.size(), cudaMemcpyDeviceToHost));
            CF_CUDA(cudaMemcpy(col.data(), M.column_indices, sizeof(int32_t) * col.size(),
                               cudaMemcpyDeviceToHost));
            for (int i = 0; i < M.num_rows; ++i)
                if (ro[(size_t)i] != i || col[(size_t)i] != i)
                    throw std::invalid_argument("libGIS (cufoam_gb300): MRS needs a diagonal invM");
            cf::matrix_set_inverse_diagonal(m.get(), M.values);
        }
        cf_controls c;
        cf_controls_init(&c);
        c.tolerance = error;
        c.absolute_tolerance = 1;
        c.max_iter = max_steps;
        c.memory = CF_MEM_DEVICE;
        c.reduction = reduction_order();
        c.bicg_int_bound = s.int_bound;
        c.richardson_omega = s.omega;
        c.power_max_steps = s.power_steps;
        std::vector<double> hist;
        if (detail) {
            const long long want = max_steps > 0 ? (long long)max_steps + 1 : kMaxDetail;
            hist.resize((size_t)(want < kMaxDetail ? want : kMaxDetail));
            c.history = hist.data();
            c.history_capacity = (int32_t)hist.size();
            c.history_time = detail_type == DetailType::Time ? 1 : 0;
        }
        cf_perf perf;
        cf::solve(m.get(), s.solver, c, b.values, x->values, &perf);
        if (detail) detail->assign(hist.begin(), hist.begin() + perf.history_length);
        return perf.status;
    } catch (const cf::Error &e) {
        rethrow(e);
    }
}

} // namespace

CSR Transpose(const CSR &A)
{
    if (A.num_rows < 0 || A.num_cols < 0 || A.num_entries < 0)
        throw std::invalid_argument("libGIS (cufoam_gb300): bad matrix shape");
    CSR T;
    try {
        cf::Context *ctx = shim_context();
        CF_CUDA(cudaStreamSynchronize(cudaStreamLegacy));
        CF_CUDA(cudaMalloc(&T.row_offsets, sizeof(IndexType) * ((size_t)A.num_cols + 1)));
        CF_CUDA(cudaMalloc(&T.column_indices, sizeof(IndexType) * ((size_t)A.num_entries + 1)));
        CF_CUDA(cudaMalloc(&T.values, sizeof(ValueType) * ((size_t)A.num_entries + 1)));
        T.num_rows = A.num_cols;
        T.num_cols = A.num_rows;
        T.num_entries = A.num_entries;
        cf::csr_transpose(ctx, A.num_rows, A.num_cols, A.num_entries, A.row_offsets, A.column_indices,
                          A.values, T.row_offsets, T.column_indices, T.values);
        CF_CUDA(cudaStreamSynchronize(ctx->stream));
    } catch (const cf::Error &e) {
        rethrow(e);
    }
    return T;
}

void CG(Vec *x, const CSR &A, const Vec &b, ValueType error, int max_steps, std::vector<double> *detail,
        DetailType detail_type)
{
    SolveSpec s;
    s.solver = CF_CG;
    run(s, x, A, b, error, max_steps, detail, detail_type);
}

bool BiCG(Vec *x, const CSR &A, const Vec &b, ValueType error, IndexType max_steps, const ValueType int_bound,
          std::vector<double> *detail, DetailType detail_type)
{
    SolveSpec s;
    s.solver = CF_BICG;
    s.int_bound = int_bound;
    return run(s, x, A, b, error, max_steps, detail, detail_type) == CF_BREAKDOWN;
}

bool BiCG(Vec *x, const CSR &A, const CSR &At, const Vec &b, ValueType error, IndexType max_steps,
          const ValueType int_bound, std::vector<double> *detail, DetailType detail_type)
{
    SolveSpec s;
    s.solver = CF_BICG;
    s.At = &At;
    s.int_bound = int_bound;
    return run(s, x, A, b, error, max_steps, detail, detail_type) == CF_BREAKDOWN;
}

void Richardson(Vec *x, const CSR &A, const Vec &b, ValueType error, ValueType omega, IndexType power_max_steps,
                IndexType max_steps, std::vector<double> *detail, DetailType detail_type)
{
    SolveSpec s;
    s.solver = CF_RICHARDSON;
    s.omega = omega;
    s.power_steps = power_max_steps;
    run(s, x, A, b, error, max_steps, detail, detail_type);
}

void MR(Vec *x, const CSR &A, const Vec &b, ValueType error, IndexType max_steps, std::vector<double> *detail,
        DetailType detail_type)
{
    SolveSpec s;
    s.solver = CF_MR;
    run(s, x, A, b, error, max_steps, detail, detail_type);
}

void Jacobi(Vec *x, const CSR &A, const Vec &b, ValueType error, IndexType max_steps,
            std::vector<double> *detail, DetailType detail_type)
{
    SolveSpec s;
    s.solver = CF_JACOBI;
    run(s, x, A, b, error, max_steps, detail, detail_type);
}

void MRJacobi(Vec *x, const CSR &A, const Vec &b, ValueType error, IndexType max_steps,
              std::vector<double> *detail, DetailType detail_type)
{
    SolveSpec s;
    s.solver = CF_MRJACOBI;
    run(s, x, A, b, error, max_steps, detail, detail_type);
}

void JMR(Vec *x, const CSR &A, const Vec &b, ValueType error, IndexType max_steps, std::vector<double> *detail,
         DetailType detail_type)
{
    SolveSpec s;
    s.solver = CF_JMR;
    run(s, x, A, b, error, max_steps, detail, detail_type);
}

void MRS(Vec *x, const CSR &A, const Vec &b, const CSR &invM, ValueType error, IndexType max_steps,
         std::vector<double> *detail, DetailType detail_type)
{
    SolveSpec s;
    s.solver = CF_MRS;
    s.invM = &invM;
    run(s, x, A, b, error, max_steps, detail, detail_type);
}

ValueType NormFactor(const CSR &A, const Vec &b, const Vec &x)
{
    check_system(A, b, &x);
    try {
        cf::Context *ctx = shim_context();
        std::unique_ptr<cf::Matrix> m = device_matrix(ctx, A);
        const double nf = cf::norm_factor(m.get(), b.values, x.values, CF_NORM_REFERENCE_L2,
                                          reduction_order() == CF_REDUCE_REFERENCE);
        return nf;
    } catch (const cf::Error &e) {
        rethrow(e);
    }
}
