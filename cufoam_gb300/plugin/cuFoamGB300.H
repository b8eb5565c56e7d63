/*
 * cuFoamGB300.H -- the eight cuFoam lduMatrix::solver plugins on top of the
 * GB300 C ABI (include/cufoam_gb300.h).
 *
 * Drop-in for the reference's plugin library: the same class names
 * (cuFoamCG, cuFoamBiCG, cuFoamJacobi, cuFoamMR, cuFoamMRJacobi, cuFoamMRS,
 * cuFoamJMR, cuFoamRichardson; e.g. cuFoamCG/cuFoamCG.H:8-31), the same
 * constructor and solve(psi, source, cmpt) signature, the same symmetric /
 * asymmetric registration tables, selected by name in fvSolution:
 *
 *     p { solver cuFoamCG; tolerance 1e-8; maxIter 5000; }
 *
 * Optional controls (all default to the reference's behaviour):
 *     precision   FP64 | mixed        (mixed: FP32 inner solve, FP64 refinement)
 *     reduction   auto | fast | reference
 *                 (auto: the reference's exact sums for BiCG, fast for the rest)
 *     normType    reference | openfoam
 *     useRelTol   false               (true: honour relTol_/minIter_ like OpenFOAM)
 *
 * Coupled interfaces: cyclic patches are folded into the device matrix
 * (OpenFOAM's interface update, result -= interfaceBouCoeffs * psi of the
 * neighbour patch's face cells, becomes the CSR entries (faceCell,
 * neighbour faceCell) = -coeff appended to each row).  In a parallel run
 * (Pstream::parRun()) the processor patches couple each rank's subdomain
 * to its neighbours: every solver runs on the decomposed system
 * (cf_solve_decomposed, FP64, transfers through OpenFOAM's Pstream,
 * cuFoamGB300Comm.H); `precision mixed` stops with a FatalError there.
 * The reference ignores all interfaces.
 *
 * Residuals in the returned solverPerformance are normalised by normFactor
 * (OpenFOAM's convention); the stopping test is the reference's
 * ||r||_2 <= tolerance * normFactor.
 *
 * Compiles against OpenFOAM (wmake, Make/files + Make/options) or against
 * the minimal stand-in in minifoam/ used by the tests.
 */
#ifndef CUFOAM_GB300_PLUGIN_H
#define CUFOAM_GB300_PLUGIN_H

#include "lduMatrix.H"
#include "cyclicLduInterface.H"
#include "processorLduInterface.H"
#include "cufoam_gb300.h"

namespace Foam {

class cuFoamGB300Solver : public lduMatrix::solver {
protected:
    const int32_t kind_;

    cf_controls gb300Controls() const;

    // The matrix with this solver's cyclic interfaces folded in (a new
    // device matrix, owned by the caller), or nullptr without coupling.
    cf_matrix *coupledMatrix() const;

public:
    cuFoamGB300Solver(int32_t kind, const word &fieldName, const lduMatrix &matrix,
                      const FieldField<Field, scalar> &interfaceBouCoeffs,
                      const FieldField<Field, scalar> &interfaceIntCoeffs,
                      const lduInterfaceFieldPtrsList &interfaces,
                      const dictionary &solverControls);

    virtual ~cuFoamGB300Solver() {}

    virtual solverPerformance solve(scalarField &psi, const scalarField &source,
                                    const direction cmpt = 0) const;
};

#define CUFOAM_GB300_DECLARE_SOLVER(Name)                                          \
    class Name : public cuFoamGB300Solver {                                        \
    public:                                                                        \
        TypeName(#Name);                                                           \
        Name(const word &fieldName, const lduMatrix &matrix,                       \
             const FieldField<Field, scalar> &interfaceBouCoeffs,                  \
             const FieldField<Field, scalar> &interfaceIntCoeffs,                  \
             const lduInterfaceFieldPtrsList &interfaces,                          \
             const dictionary &solverControls);                                    \
    };

CUFOAM_GB300_DECLARE_SOLVER(cuFoamCG)
CUFOAM_GB300_DECLARE_SOLVER(cuFoamBiCG)
CUFOAM_GB300_DECLARE_SOLVER(cuFoamJacobi)
CUFOAM_GB300_DECLARE_SOLVER(cuFoamMR)
CUFOAM_GB300_DECLARE_SOLVER(cuFoamMRJacobi)
CUFOAM_GB300_DECLARE_SOLVER(cuFoamMRS)
CUFOAM_GB300_DECLARE_SOLVER(cuFoamJMR)
CUFOAM_GB300_DECLARE_SOLVER(cuFoamRichardson)
CUFOAM_GB300_DECLARE_SOLVER(cuFoamPCG)

#undef CUFOAM_GB300_DECLARE_SOLVER

} // namespace Foam

#endif
