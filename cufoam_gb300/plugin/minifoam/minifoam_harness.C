/*
 * minifoam_harness.C -- drives the plugin sources the way OpenFOAM does,
 * without OpenFOAM: builds an lduAddressing/lduMatrix from plain arrays,
 * selects the solver by name from the run-time tables
 * (lduMatrix::solver::New) and calls solve(psi, source, cmpt).  Exposed as
 * a C function so the tests can exercise the plugin layer end to end.
 */
#include "lduMatrix.H"

#include <cstring>
#include <exception>

namespace Foam {
FatalErrorType FatalError;
}

extern "C" {

/* Solve with the plugin `solver_name` ("cuFoamCG", ...).  lower == NULL
 * means a symmetric matrix (OpenFOAM stores only upper then).  `keys` /
 * `values` are n_extra extra dictionary entries (e.g. "precision" "mixed").
 * out = {initialResidual, finalResidual, nIterations, converged}.
 * Returns 0, or -1 with the FatalError text in err. */
int mf_solve(const char *solver_name, int n, int n_faces, const double *diag, const double *lower,
             const double *upper, const int *lower_addr, const int *upper_addr, const double *source,
             double *psi, double tolerance, double rel_tol, int max_iter, int n_extra,
             const char *const *keys, const char *const *values, double *out, char *err, int err_len)
{
    try {
        using namespace Foam;
        labelList la(lower_addr, lower_addr + n_faces), ua(upper_addr, upper_addr + n_faces);
        lduAddressing addr(n, la, ua);
        scalarField d(diag, diag + n), up(upper, upper + n_faces);
        scalarField lo;
        if (lower) lo.assign(lower, lower + n_faces);
        lduMatrix matrix(addr, d, lower ? &lo : nullptr, &up);
        dictionary controls;
        controls.set("solver", solver_name);
        controls.set("tolerance", std::to_string(tolerance));
        {
            // exact text of the doubles
            char buf[64];
            std::snprintf(buf, sizeof(buf), "%.17g", tolerance);
            controls.set("tolerance", buf);
            std::snprintf(buf, sizeof(buf), "%.17g", rel_tol);
            controls.set("relTol", buf);
        }
        controls.set("maxIter", std::to_string(max_iter));
        for (int i = 0; i < n_extra; ++i) controls.set(keys[i], values[i]);
        FieldField<Field, scalar> bou, intc;
        lduInterfaceFieldPtrsList interfaces;
        std::unique_ptr<lduMatrix::solver> s =
            lduMatrix::solver::New("psi", matrix, bou, intc, interfaces, controls);
        scalarField x(psi, psi + n), b(source, source + n);
        solverPerformance perf = s->solve(x, b);
        std::memcpy(psi, x.cdata(), sizeof(double) * n);
        out[0] = perf.initialResidual();
        out[1] = perf.finalResidual();
        out[2] = perf.nIterations();
        out[3] = perf.converged() ? 1.0 : 0.0;
        if (err && err_len > 0) err[0] = 0;
        return 0;
    } catch (const std::exception &e) {
        if (err && err_len > 0) {
            std::strncpy(err, e.what(), err_len - 1);
            err[err_len - 1] = 0;
        }
        return -1;
    }
}

} // extern "C"
