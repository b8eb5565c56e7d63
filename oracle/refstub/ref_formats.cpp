/*
 * Builds the reference's own file readers and writers (CPU::SparseCSR::read /
 * save and CPU::Vector::load / readMTX / save, gis/SparseSystem/SparseCPU.h),
 * compiled unchanged from their source file, behind C functions for the
 * golden-fixture generator of the file-format tests.
 * TEST INFRASTRUCTURE ONLY; the output library lives in oracle/_ref/.
 */
#include "SparseSystem/SparseCPU.h"

#include <algorithm>
#include <exception>

static CPU::SparseCSR<double, int> g_csr;
static CPU::Vector<double, int> g_vec;

// 0 = read, -1 = the reference threw
extern "C" int ref_csr_read(const char *path, int *rows, int *cols, int *nnz)
{
    try {
        g_csr = CPU::SparseCSR<double, int>();
        g_csr.read(path);
    } catch (const std::exception &) {
        return -1;
    }
    *rows = g_csr.num_rows;
    *cols = g_csr.num_cols;
    *nnz = g_csr.num_entries;
    return 0;
}

extern "C" void ref_csr_take(int *row_offsets, int *cols, double *vals)
{
    std::copy(g_csr.row_offsets.begin(), g_csr.row_offsets.begin() + g_csr.num_rows + 1, row_offsets);
    std::copy(g_csr.column_indices.begin(), g_csr.column_indices.begin() + g_csr.num_entries, cols);
    std::copy(g_csr.values.begin(), g_csr.values.begin() + g_csr.num_entries, vals);
}

extern "C" void ref_csr_save(const char *path, int rows, int cols, int nnz, const int *ro, const int *ci,
                             const double *v)
{
    CPU::SparseCSR<double, int> A(rows, cols, nnz);
    std::copy(ro, ro + rows + 1, A.row_offsets.begin());
    std::copy(ci, ci + nnz, A.column_indices.begin());
    std::copy(v, v + nnz, A.values.begin());
    A.save(path);
}

// mtx != 0: Matrix Market text, else the binary vector file
extern "C" int ref_vec_read(const char *path, int mtx, int *size)
{
    try {
        g_vec = CPU::Vector<double, int>();
        if (mtx) g_vec.readMTX(path);
        else g_vec.load(path);
    } catch (const std::exception &) {
        return -1;
    }
    *size = g_vec.size;
    return 0;
}

extern "C" void ref_vec_take(double *v) { std::copy(g_vec.values.begin(), g_vec.values.begin() + g_vec.size, v); }

extern "C" void ref_vec_save(const char *path, int size, const double *v)
{
    CPU::Vector<double, int> x(size);
    std::copy(v, v + size, x.values.begin());
    x.save(path);
}
