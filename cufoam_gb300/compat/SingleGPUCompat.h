/*
 * SingleGPUCompat.h -- the binary interface of the reference's solver
 * library (libGIS.so, gis/gis.h:10-93), declared anew so that a library
 * built from cufoam_gb300 can stand in for libGIS.so under the unmodified
 * reference plugins.
 *
 * The two container templates must have exactly the reference's data
 * members, in the reference's order (gis/SparseSystem/SparseSingleGPU.h:
 * 226-241 for SparseCSR, 403-409 for Vector): the plugins construct them
 * inline and pass them by reference / pointer.  Their special members are
 * user-provided (non-trivial), as in the reference, which fixes how a
 * SparseCSR returned by value (Transpose) is passed back: through a hidden
 * result pointer.  Device memory held by a container is cudaMalloc'd and
 * released by its owner with cudaFree.
 */
#ifndef CUFOAM_SINGLEGPU_COMPAT_H
#define CUFOAM_SINGLEGPU_COMPAT_H

#include <cuda_runtime.h>

#include <vector>

enum class DetailType { Error, Time };

namespace SingleGPU {

template <typename ValueType = double, typename IndexType = int>
class SparseCSR {
public:
    SparseCSR()
        : values(nullptr), row_offsets(nullptr), column_indices(nullptr), num_rows(0), num_cols(0),
          num_entries(0)
    {
    }
    SparseCSR(const SparseCSR &o) = delete;
    SparseCSR(SparseCSR &&o) noexcept
        : values(o.values), row_offsets(o.row_offsets), column_indices(o.column_indices),
          num_rows(o.num_rows), num_cols(o.num_cols), num_entries(o.num_entries)
    {
        o.values = nullptr;
        o.row_offsets = nullptr;
        o.column_indices = nullptr;
        o.num_rows = o.num_cols = o.num_entries = 0;
    }
    ~SparseCSR()
    {
        cudaFree(values);
        cudaFree(row_offsets);
        cudaFree(column_indices);
    }

    ValueType *values;
    IndexType *row_offsets;
    IndexType *column_indices;
    IndexType num_rows;
    IndexType num_cols;
    IndexType num_entries;
};

template <typename ValueType = double, typename IndexType = int>
class Vector {
public:
    Vector() : values(nullptr), size(0), capacity(0) {}
    Vector(const Vector &o) = delete;
    ~Vector() { cudaFree(values); }

    ValueType *values;
    IndexType size;
    IndexType capacity;
};

} // namespace SingleGPU

using ValueType = double;
using IndexType = int;

SingleGPU::SparseCSR<ValueType, IndexType> Transpose(const SingleGPU::SparseCSR<ValueType, IndexType> &A);

void CG(SingleGPU::Vector<ValueType, IndexType> *x, const SingleGPU::SparseCSR<ValueType, IndexType> &A,
        const SingleGPU::Vector<ValueType, IndexType> &b, ValueType error, int max_steps,
        std::vector<double> *detail, DetailType detail_type);

bool BiCG(SingleGPU::Vector<ValueType, IndexType> *x, const SingleGPU::SparseCSR<ValueType, IndexType> &A,
          const SingleGPU::Vector<ValueType, IndexType> &b, ValueType error, IndexType max_steps,
          const ValueType int_bound, std::vector<double> *detail, DetailType detail_type);

bool BiCG(SingleGPU::Vector<ValueType, IndexType> *x, const SingleGPU::SparseCSR<ValueType, IndexType> &A,
          const SingleGPU::SparseCSR<ValueType, IndexType> &At,
          const SingleGPU::Vector<ValueType, IndexType> &b, ValueType error, IndexType max_steps,
          const ValueType int_bound, std::vector<double> *detail, DetailType detail_type);

void Richardson(SingleGPU::Vector<ValueType, IndexType> *x,
                const SingleGPU::SparseCSR<ValueType, IndexType> &A,
                const SingleGPU::Vector<ValueType, IndexType> &b, ValueType error, ValueType omega,
                IndexType power_max_steps, IndexType max_steps, std::vector<double> *detail,
                DetailType detail_type);

void MR(SingleGPU::Vector<ValueType, IndexType> *x, const SingleGPU::SparseCSR<ValueType, IndexType> &A,
        const SingleGPU::Vector<ValueType, IndexType> &b, ValueType error, IndexType max_steps,
        std::vector<double> *detail, DetailType detail_type);

void Jacobi(SingleGPU::Vector<ValueType, IndexType> *x, const SingleGPU::SparseCSR<ValueType, IndexType> &A,
            const SingleGPU::Vector<ValueType, IndexType> &b, ValueType error, IndexType max_steps,
            std::vector<double> *detail, DetailType detail_type);

void MRJacobi(SingleGPU::Vector<ValueType, IndexType> *x,
              const SingleGPU::SparseCSR<ValueType, IndexType> &A,
              const SingleGPU::Vector<ValueType, IndexType> &b, ValueType error, IndexType max_steps,
              std::vector<double> *detail, DetailType detail_type);

void JMR(SingleGPU::Vector<ValueType, IndexType> *x, const SingleGPU::SparseCSR<ValueType, IndexType> &A,
         const SingleGPU::Vector<ValueType, IndexType> &b, ValueType error, IndexType max_steps,
         std::vector<double> *detail, DetailType detail_type);

void MRS(SingleGPU::Vector<ValueType, IndexType> *x, const SingleGPU::SparseCSR<ValueType, IndexType> &A,
         const SingleGPU::Vector<ValueType, IndexType> &b,
         const SingleGPU::SparseCSR<ValueType, IndexType> &invM, ValueType error, IndexType max_steps,
         std::vector<double> *detail, DetailType detail_type);

ValueType NormFactor(const SingleGPU::SparseCSR<ValueType, IndexType> &A,
                     const SingleGPU::Vector<ValueType, IndexType> &b,
                     const SingleGPU::Vector<ValueType, IndexType> &x);

#endif
