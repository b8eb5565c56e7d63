// formats.cpp -- the reference's on-disk formats for matrices and vectors
// (host code).
//
//   * binary CSR (gis/SparseSystem/SparseCPU.h:105-147): int32 rows, cols,
//     nnz; f64 values[nnz]; int32 row_offsets[rows] (the final offset is not
//     stored: it is nnz); int32 column_indices[nnz]; native byte order.
//   * Rutherford-Boeing (SparseCPU.h:149-297): real or integer, assembled
//     (column-compressed) matrices; types r/i x u/r/s/z.  Unsymmetric files
//     are transposed from CSC to CSR; symmetric and skew files store one
//     triangle, mirrored here with the reference's entry order (for rows
//     i = 0.. in order, a row's own entries go to the next free slot of row
//     i, each mirrored entry to the next free slot of its column's row).
//   * binary vector (SparseCPU.h:651-658, 680-684): int32 size, f64 values.
//   * Matrix Market vector (SparseCPU.h:661-678): a header line, the size as
//     the first number of the next line, then the values.  Comment lines
//     ('%') after the header are skipped (the reference reads them as data).
// A file name ending in ".rb" (matrices) or ".mtx" (vectors) selects the
// text format, anything else the binary one (SparseCPU.h:305-311).
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "internal.h"

namespace cf {

namespace {

bool ends_with(const std::string &s, const char *suf)
{
    const size_t n = std::strlen(suf);
    return s.size() >= n && s.compare(s.size() - n, n, suf) == 0;
}

[[noreturn]] void bad(const std::string &path, const std::string &what)
{
    throw Error{CF_BAD_INPUT, path + ": " + what};
}

// CSR of the transpose of an (nr x nc) CSR matrix; rows of the result list
// the entries of each column by ascending source row.
void csr_transpose_host(int nr, int nc, const std::vector<int32_t> &ro, const std::vector<int32_t> &col,
                        const std::vector<double> &val, std::vector<int32_t> &roT, std::vector<int32_t> &colT,
                        std::vector<double> &valT)
{
    const size_t nnz = col.size();
    roT.assign((size_t)nc + 1, 0);
    for (size_t j = 0; j < nnz; ++j) roT[(size_t)col[j] + 1] += 1;
    for (int c = 0; c < nc; ++c) roT[(size_t)c + 1] += roT[(size_t)c];
    colT.assign(nnz, 0);
    valT.assign(nnz, 0.0);
    std::vector<int32_t> next(roT.begin(), roT.end() - 1);
    for (int i = 0; i < nr; ++i)
        for (int32_t j = ro[(size_t)i]; j < ro[(size_t)i + 1]; ++j) {
            const int32_t pos = next[(size_t)col[(size_t)j]]++;
            colT[(size_t)pos] = i;
            valT[(size_t)pos] = val[(size_t)j];
        }
}

void read_rb(const std::string &path, HostCsr &out)
{
    std::ifstream in(path);
    if (!in) bad(path, "cannot open");
    std::string line;
    std::getline(in, line);
    std::getline(in, line);
    std::string type;
    long long rows = 0, cols = 0, entries = 0, unused = 0;
    if (!(in >> type >> rows >> cols >> entries >> unused) || type.size() < 3)
        bad(path, "malformed Rutherford-Boeing header");
    for (char &ch : type) ch = (char)std::tolower((unsigned char)ch);
    if (type[0] != 'r' && type[0] != 'i')
        throw Error{CF_UNSUPPORTED, path + ": only real and integer matrices are read"};
    if (type[2] != 'a') throw Error{CF_UNSUPPORTED, path + ": elemental matrices are not read"};
    if (type[1] != 'u' && type[1] != 'r' && type[1] != 's' && type[1] != 'z')
        throw Error{CF_UNSUPPORTED, path + ": matrix kind '" + std::string(1, type[1]) + "' is not read"};
    if (rows < 0 || cols < 0 || entries < 0 || rows > INT32_MAX - 1 || cols > INT32_MAX - 1 ||
        entries > INT32_MAX)
        bad(path, "matrix size out of range");
    std::getline(in, line);   // rest of the third line
    std::getline(in, line);   // Fortran formats
    // column-compressed data, read as the CSR of the transpose (cols x rows)
    const int nr = (int)cols, nc = (int)rows;
    const size_t nnz = (size_t)entries;
    std::vector<int32_t> ro((size_t)nr + 1), ci(nnz);
    std::vector<double> v(nnz);
    long long t = 0;
    for (int i = 0; i <= nr; ++i) {
        if (!(in >> t)) bad(path, "truncated column pointers");
        ro[(size_t)i] = (int32_t)(t - 1);
    }
    for (size_t j = 0; j < nnz; ++j) {
        if (!(in >> t)) bad(path, "truncated row indices");
        ci[j] = (int32_t)(t - 1);
    }
    for (size_t j = 0; j < nnz; ++j)
        if (!(in >> v[j])) bad(path, "truncated values");
    if (ro[0] != 0 || ro[(size_t)nr] != (int32_t)nnz) bad(path, "inconsistent column pointers");
    for (int i = 0; i < nr; ++i)
        if (ro[(size_t)i + 1] < ro[(size_t)i]) bad(path, "decreasing column pointers");
    for (size_t j = 0; j < nnz; ++j)
        if (ci[j] < 0 || ci[j] >= nc) bad(path, "row index out of range");
    if (type[1] == 'u' || type[1] == 'r') {
        out.rows = (int)rows;
        out.cols = (int)cols;
        csr_transpose_host(nr, nc, ro, ci, v, out.row_offsets, out.cols_idx, out.values);
        return;
    }
    // one stored triangle: mirror it (negated for skew-symmetric files)
    if (rows != cols) bad(path, "symmetric matrix that is not square");
    const double sign = type[1] == 'z' ? -1.0 : 1.0;
    const int n = nr;
    std::vector<int32_t> cnt((size_t)n + 1, 0);
    for (int i = 0; i < n; ++i)
        for (int32_t j = ro[(size_t)i]; j < ro[(size_t)i + 1]; ++j) {
            cnt[(size_t)i + 1] += 1;
            if (ci[(size_t)j] != i) cnt[(size_t)ci[(size_t)j] + 1] += 1;
        }
    for (int i = 0; i < n; ++i) cnt[(size_t)i + 1] += cnt[(size_t)i];
    out.rows = out.cols = n;
    out.row_offsets = cnt;
    const size_t total = (size_t)cnt[(size_t)n];
    out.cols_idx.assign(total, 0);
    out.values.assign(total, 0.0);
    std::vector<int32_t> next(cnt.begin(), cnt.end() - 1);
    for (int i = 0; i < n; ++i)
        for (int32_t j = ro[(size_t)i]; j < ro[(size_t)i + 1]; ++j) {
            const int32_t c = ci[(size_t)j];
            int32_t p = next[(size_t)i]++;
            out.cols_idx[(size_t)p] = c;
            out.values[(size_t)p] = v[(size_t)j];
            if (c != i) {
                p = next[(size_t)c]++;
                out.cols_idx[(size_t)p] = i;
                out.values[(size_t)p] = sign * v[(size_t)j];
            }
        }
}

void read_bin_csr(const std::string &path, HostCsr &out)
{
    std::ifstream in(path, std::ios::binary);
    if (!in) bad(path, "cannot open");
    int32_t hdr[3];
    if (!in.read(reinterpret_cast<char *>(hdr), sizeof(hdr))) bad(path, "truncated header");
    if (hdr[0] < 0 || hdr[1] < 0 || hdr[2] < 0) bad(path, "negative size in header");
    in.seekg(0, std::ios::end);
    const long long have = (long long)in.tellg();
    const long long need = 12 + 8LL * hdr[2] + 4LL * hdr[0] + 4LL * hdr[2];
    if (have < need) bad(path, "file shorter than its header says");
    in.seekg(12, std::ios::beg);
    out.rows = hdr[0];
    out.cols = hdr[1];
    out.values.resize((size_t)hdr[2]);
    out.row_offsets.resize((size_t)hdr[0] + 1);
    out.cols_idx.resize((size_t)hdr[2]);
    in.read(reinterpret_cast<char *>(out.values.data()), 8LL * hdr[2]);
    in.read(reinterpret_cast<char *>(out.row_offsets.data()), 4LL * hdr[0]);
    in.read(reinterpret_cast<char *>(out.cols_idx.data()), 4LL * hdr[2]);
    if (!in) bad(path, "read failed");
    out.row_offsets[(size_t)hdr[0]] = hdr[2];
}

} // namespace

void read_csr_file(const std::string &path, HostCsr &out)
{
    out = HostCsr{};
    if (ends_with(path, ".rb")) read_rb(path, out);
    else read_bin_csr(path, out);
}

void save_csr_file(const std::string &path, int rows, int cols, int64_t nnz, const int32_t *ro,
                   const int32_t *col, const double *val)
{
    require(rows >= 0 && cols >= 0 && nnz >= 0 && nnz <= INT32_MAX, CF_BAD_INPUT, "bad CSR size");
    std::ofstream out(path, std::ios::binary);
    if (!out) bad(path, "cannot create");
    const int32_t hdr[3] = {rows, cols, (int32_t)nnz};
    out.write(reinterpret_cast<const char *>(hdr), sizeof(hdr));
    out.write(reinterpret_cast<const char *>(val), 8 * nnz);
    out.write(reinterpret_cast<const char *>(ro), 4LL * rows);
    out.write(reinterpret_cast<const char *>(col), 4 * nnz);
    if (!out) bad(path, "write failed");
}

void read_vector_file(const std::string &path, std::vector<double> &out)
{
    out.clear();
    if (ends_with(path, ".mtx")) {
        std::ifstream in(path);
        if (!in) bad(path, "cannot open");
        std::string line;
        std::getline(in, line);   // %%MatrixMarket header
        while (in.peek() == '%') std::getline(in, line);
        long long size = 0;
        if (!(in >> size) || size < 0 || size > INT32_MAX) bad(path, "malformed size line");
        std::getline(in, line);
        out.resize((size_t)size);
        for (long long i = 0; i < size; ++i)
            if (!(in >> out[(size_t)i])) bad(path, "truncated values");
        return;
    }
    std::ifstream in(path, std::ios::binary);
    if (!in) bad(path, "cannot open");
    int32_t size = 0;
    if (!in.read(reinterpret_cast<char *>(&size), 4) || size < 0) bad(path, "bad header");
    out.resize((size_t)size);
    if (!in.read(reinterpret_cast<char *>(out.data()), 8LL * size)) bad(path, "truncated values");
}

void save_vector_file(const std::string &path, int size, const double *v)
{
    require(size >= 0, CF_BAD_INPUT, "bad vector size");
    std::ofstream out(path, std::ios::binary);
    if (!out) bad(path, "cannot create");
    const int32_t s = size;
    out.write(reinterpret_cast<const char *>(&s), 4);
    out.write(reinterpret_cast<const char *>(v), 8LL * size);
    if (!out) bad(path, "write failed");
}

} // namespace cf
