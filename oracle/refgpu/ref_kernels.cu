// ref_kernels.cu -- test infrastructure, not product code.
//
// Instantiates the reference's own device kernels for <double, int>
// straight from its header (gis/SparseSystem/kernels.h, included from the
// reference tree at build time; nothing of it is copied here) so that they
// can be compiled into a cubin and launched on the GPU by ref_gpu.c.  The
// oracle's CPU emulation of the reference's arithmetic (FMA contraction,
// the 8-lane SpMV tree, the 256-wide block trees, the host sums) is pinned
// by running the same drivers once through these kernels.
#include "SparseSystem/kernels.h"

template __global__ void FillKernel<double, int>(double *, const int, const double);
template __global__ void ReductionKernel<double, int>(double *, const double *, const int);
template __global__ void DotKernel<double, int>(double *, const double *, const double *, const int);
template __global__ void SpMvKernel<double, int>(double *, const double *, const int *, const int *,
                                                 const int, const double *);
template __global__ void DistanceKernel<double, int>(double *, const double *, const double *, const int);
template __global__ void ScaleKernel<double, int>(double *, const double *, const int, const double);
template __global__ void AddKernel1<double, int>(double *, const double *, const double *, const int,
                                                 const double);
template __global__ void HadamardKernel<double, int>(double *, const double *, const double *, const int);
template __global__ void ResidualKernel<double, int>(double *, const double *, const int *, const int *,
                                                     const int, const double *, const double *);
template __global__ void FindDiag<double, int>(double *, const double *, const int *, const int *, const int);
template __global__ void MinAbsKernel<double, int>(double *, const double *, const int);
template __global__ void FindDiagInv<double, int>(double *, const double *, const int *, const int *, const int);
template __global__ void FindDiagInvSqrt<double, int>(double *, const double *, const int *, const int *,
                                                      const int);
