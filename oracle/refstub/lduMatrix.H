/*
 * Minimal stand-in for OpenFOAM's lduMatrix.H, just large enough to compile
 * the reference's gis/ldu2csr.h (getSparseCSRMat) from its own source file.
 * TEST INFRASTRUCTURE ONLY: used by oracle/refstub/ref_ldu2csr.cpp to build
 * the golden-CSR checker in oracle/_ref/.
 *
 * The reference reads only diag(), lower(), upper() and the lduAddressing
 * arrays lowerAddr(), upperAddr(), losortAddr(), losortStartAddr(),
 * ownerStartAddr() (gis/ldu2csr.h:9-35).  The arrays are filled by the
 * caller with OpenFOAM's semantics (computed by the oracle).
 */
#ifndef CUFOAM_REFSTUB_LDUMATRIX_H
#define CUFOAM_REFSTUB_LDUMATRIX_H

#include <vector>

namespace Foam {

typedef int label;
typedef double scalar;

struct labelList : std::vector<label> {
    using std::vector<label>::vector;
};

struct scalarField : std::vector<scalar> {
    using std::vector<scalar>::vector;
};

class lduAddressing {
public:
    labelList lower_, upper_, losort_, losortStart_, ownerStart_;
    const labelList &lowerAddr() const { return lower_; }
    const labelList &upperAddr() const { return upper_; }
    const labelList &losortAddr() const { return losort_; }
    const labelList &losortStartAddr() const { return losortStart_; }
    const labelList &ownerStartAddr() const { return ownerStart_; }
};

class lduMatrix {
public:
    scalarField diag_, lower_, upper_;
    lduAddressing addr_;
    const scalarField &diag() const { return diag_; }
    const scalarField &lower() const { return lower_; }
    const scalarField &upper() const { return upper_; }
    const lduAddressing &lduAddr() const { return addr_; }
};

} // namespace Foam

#endif
