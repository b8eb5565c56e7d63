/*
 * cuFoamGB300.C -- implementation of the eight plugins (see cuFoamGB300.H).
 *
 * What one solve() does, compared with the reference's plugin
 * (cuFoamCG/cuFoamCG.C:38-90):
 *   reference: host ldu2csr, cudaMalloc+copy of the CSR and vectors,
 *              NormFactor, the solver with tolerance*normFactor, copy back,
 *              free everything.
 *   here:      the lduAddressing is uploaded once and kept on the device
 *              (cached per addressing object); each call uploads the
 *              coefficients, converts them on the device, and runs
 *              normFactor + the solver inside one device-driven loop.
 * Fixed relative to the reference: the constructor forwards
 * interfaceBouCoeffs (the reference passes interfaceIntCoeffs twice,
 * cuFoamCG/cuFoamCG.C:30-31).
 */
#include "cuFoamGB300.H"

#include <cstdlib>
#include <cstring>
#include <string>

namespace Foam {

namespace {

cf_context *gb300Context()
{
    static cf_context *ctx = nullptr;
    if (!ctx) {
        const char *dev = std::getenv("CUFOAM_GB300_DEVICE");
        const int device = dev ? std::atoi(dev) : 0;
        const cf_status st = cf_context_create(device, &ctx);
        if (st != CF_OK) {
            FatalErrorInFunction << "cuFoamGB300: cannot open CUDA device " << device << ": "
                                 << cf_status_string(st) << exit(FatalError);
        }
    }
    return ctx;
}

// One device matrix per addressing object: reused by Ux/Uy/Uz and across
// time steps; coefficients are refreshed on every solve.
struct MatrixCache {
    const void *addr = nullptr;
    const void *lowerAddr = nullptr;
    const void *upperAddr = nullptr;
    label n = -1, nFaces = -1;
    cf_matrix *m = nullptr;
};

cf_matrix *deviceMatrix(const lduMatrix &M)
{
    static MatrixCache cache;
    const lduAddressing &A = M.lduAddr();
    const label n = M.diag().size();
    const label nFaces = A.lowerAddr().size();
    cf_context *ctx = gb300Context();
    const bool same = cache.m && cache.addr == &A && cache.n == n && cache.nFaces == nFaces &&
                      cache.lowerAddr == A.lowerAddr().cdata() &&
                      cache.upperAddr == A.upperAddr().cdata();
    cf_status st = CF_OK;
    if (same) {
        st = cf_matrix_update_values(cache.m, M.diag().cdata(), M.lower().cdata(), M.upper().cdata(),
                                     CF_MEM_HOST);
    } else {
        if (cache.m) cf_matrix_destroy(cache.m);
        cache = MatrixCache();
        cf_ldu_view v;
        std::memset(&v, 0, sizeof(v));
        v.n_cells = n;
        v.n_faces = nFaces;
        v.diag = M.diag().cdata();
        v.lower = M.lower().cdata();
        v.upper = M.upper().cdata();
        v.lower_addr = A.lowerAddr().cdata();
        v.upper_addr = A.upperAddr().cdata();
        v.losort = A.losortAddr().cdata();
        v.losort_start = A.losortStartAddr().cdata();
        v.owner_start = A.ownerStartAddr().cdata();
        v.memory = CF_MEM_HOST;
        st = cf_matrix_create_ldu(ctx, &v, &cache.m);
        if (st == CF_OK) {
            cache.addr = &A;
            cache.lowerAddr = A.lowerAddr().cdata();
            cache.upperAddr = A.upperAddr().cdata();
            cache.n = n;
            cache.nFaces = nFaces;
        }
    }
    if (st != CF_OK) {
        FatalErrorInFunction << "cuFoamGB300: cannot load the matrix: " << cf_status_string(st)
                             << ": " << cf_context_last_error(ctx) << exit(FatalError);
    }
    return cache.m;
}

} // namespace

static_assert(sizeof(label) == sizeof(int32_t), "cuFoamGB300 needs 32-bit labels");
static_assert(sizeof(scalar) == sizeof(double), "cuFoamGB300 needs double scalars");

cuFoamGB300Solver::cuFoamGB300Solver(int32_t kind, const word &fieldName, const lduMatrix &matrix,
                                     const FieldField<Field, scalar> &interfaceBouCoeffs,
                                     const FieldField<Field, scalar> &interfaceIntCoeffs,
                                     const lduInterfaceFieldPtrsList &interfaces,
                                     const dictionary &solverControls)
    : lduMatrix::solver(fieldName, matrix, interfaceBouCoeffs, interfaceIntCoeffs, interfaces,
                        solverControls),
      kind_(kind)
{
}

cf_controls cuFoamGB300Solver::gb300Controls() const
{
    cf_controls c;
    cf_controls_init(&c);
    c.tolerance = tolerance_;
    c.max_iter = maxIter_;
    const dictionary &d = controlDict();
    if (d.lookupOrDefault<bool>("useRelTol", false)) {
        c.rel_tol = relTol_;
        c.min_iter = minIter_;
    }
    const word precision = d.lookupOrDefault<word>("precision", word("FP64"));
    c.precision = (precision == "mixed") ? CF_PREC_MIXED : CF_PREC_FP64;
    const word reduction = d.lookupOrDefault<word>("reduction", word("fast"));
    c.reduction = (reduction == "reference") ? CF_REDUCE_REFERENCE : CF_REDUCE_FAST;
    const word normType = d.lookupOrDefault<word>("normType", word("reference"));
    c.norm_type = (normType == "openfoam") ? CF_NORM_OPENFOAM_L1 : CF_NORM_REFERENCE_L2;
    c.memory = CF_MEM_HOST;
    return c;
}

solverPerformance cuFoamGB300Solver::solve(scalarField &psi, const scalarField &source,
                                           const direction) const
{
    cf_matrix *m = deviceMatrix(matrix());
    const cf_controls c = gb300Controls();
    cf_perf perf;
    std::memset(&perf, 0, sizeof(perf));
    const cf_status st = cf_solve(m, kind_, &c, source.cdata(), psi.data(), &perf);
    if (st != CF_OK) {
        FatalErrorInFunction << type() << ": solve failed: " << cf_status_string(st) << ": "
                             << cf_context_last_error(gb300Context()) << exit(FatalError);
    }
    solverPerformance solverPerf(type(), fieldName());
    solverPerf.initialResidual() = perf.initial_residual;
    solverPerf.finalResidual() = perf.final_residual;
    solverPerf.nIterations() = perf.n_iterations;
    solverPerf.checkConvergence(tolerance_, relTol_);
    return solverPerf;
}

// ---------------------------------------------------------------------------
// the eight plugins and their run-time selection entries.  CG and
// Richardson register for symmetric matrices only, as the reference's do
// (cuFoamCG/cuFoamCG.C:14-15, cuFoamRichardson/cuFoamRichardson.C:11-12).
// ---------------------------------------------------------------------------
#define CUFOAM_GB300_DEFINE_SOLVER(Name, Kind)                                               \
    defineTypeNameAndDebug(Name, 0);                                                         \
    Name::Name(const word &fieldName, const lduMatrix &matrix,                               \
               const FieldField<Field, scalar> &interfaceBouCoeffs,                          \
               const FieldField<Field, scalar> &interfaceIntCoeffs,                          \
               const lduInterfaceFieldPtrsList &interfaces, const dictionary &solverControls) \
        : cuFoamGB300Solver(Kind, fieldName, matrix, interfaceBouCoeffs, interfaceIntCoeffs, \
                            interfaces, solverControls)                                      \
    {                                                                                        \
    }                                                                                        \
    lduMatrix::solver::addsymMatrixConstructorToTable<Name> add##Name##SymMatrixConstructorToTable_;

#define CUFOAM_GB300_ASYMMETRIC(Name)                                                        \
    lduMatrix::solver::addasymMatrixConstructorToTable<Name> add##Name##AsymMatrixConstructorToTable_;

CUFOAM_GB300_DEFINE_SOLVER(cuFoamCG, CF_CG)
CUFOAM_GB300_DEFINE_SOLVER(cuFoamBiCG, CF_BICG)
CUFOAM_GB300_ASYMMETRIC(cuFoamBiCG)
CUFOAM_GB300_DEFINE_SOLVER(cuFoamJacobi, CF_JACOBI)
CUFOAM_GB300_ASYMMETRIC(cuFoamJacobi)
CUFOAM_GB300_DEFINE_SOLVER(cuFoamMR, CF_MR)
CUFOAM_GB300_ASYMMETRIC(cuFoamMR)
CUFOAM_GB300_DEFINE_SOLVER(cuFoamMRJacobi, CF_MRJACOBI)
CUFOAM_GB300_ASYMMETRIC(cuFoamMRJacobi)
CUFOAM_GB300_DEFINE_SOLVER(cuFoamMRS, CF_MRS)
CUFOAM_GB300_ASYMMETRIC(cuFoamMRS)
CUFOAM_GB300_DEFINE_SOLVER(cuFoamJMR, CF_JMR)
CUFOAM_GB300_ASYMMETRIC(cuFoamJMR)
CUFOAM_GB300_DEFINE_SOLVER(cuFoamRichardson, CF_RICHARDSON)

} // namespace Foam
