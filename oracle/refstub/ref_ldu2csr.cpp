/*
 * Builds the reference's own getSparseCSRMat (gis/ldu2csr.h:7-40), compiled
 * unchanged from its source file against the lduMatrix.H stand-in in this
 * folder, and exposes it as a C function for the golden-fixture generator.
 * TEST INFRASTRUCTURE ONLY; the output library lives in oracle/_ref/.
 */
#include "ldu2csr.h"

#include <algorithm>

extern "C" int ref_ldu2csr(int n, int f, const double *diag, const double *lower,
                           const double *upper, const int *lower_addr,
                           const int *upper_addr, const int *losort,
                           const int *losort_start, const int *owner_start,
                           int *row_offsets, int *cols, double *vals)
{
    Foam::lduMatrix m;
    m.diag_.assign(diag, diag + n);
    m.lower_.assign(lower, lower + f);
    m.upper_.assign(upper, upper + f);
    m.addr_.lower_.assign(lower_addr, lower_addr + f);
    m.addr_.upper_.assign(upper_addr, upper_addr + f);
    m.addr_.losort_.assign(losort, losort + f);
    m.addr_.losortStart_.assign(losort_start, losort_start + n + 1);
    m.addr_.ownerStart_.assign(owner_start, owner_start + n + 1);
    CPU::SparseCSR<double, int> A = getSparseCSRMat<double, int>(m);
    if (A.num_rows != n || A.num_entries != n + 2 * f) return -1;
    std::copy(A.row_offsets.begin(), A.row_offsets.end(), row_offsets);
    std::copy(A.column_indices.begin(), A.column_indices.end(), cols);
    std::copy(A.values.begin(), A.values.end(), vals);
    return 0;
}
