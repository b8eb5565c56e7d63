// matrix.cu -- device LDU -> CSR conversion and matrix objects.
//
// The CSR layout is exactly the reference's getSparseCSRMat
// (gis/ldu2csr.h:7-40): row c = [lower coefficients of the faces whose
// neighbour is c, in losort order] [diag c] [upper coefficients of the faces
// owned by c, in face order].  Row offsets follow from the addressing
// without a scan: row_offsets[c] = losortStart[c] + c + ownerStart[c]
// (relative to the first entries), which is the reference's running count.
#include "device.cuh"

#include <algorithm>
#include <cmath>

namespace cf {

// ---------------------------------------------------------------------------
// addressing validation / construction
// ---------------------------------------------------------------------------
enum AddrError { ADDR_RANGE = 1, ADDR_ORDER = 2, ADDR_START = 4, ADDR_COUNT = 8 };

__global__ void k_check_faces(int n, int nf, const int32_t *__restrict__ la,
                              const int32_t *__restrict__ ua, int *err)
{
    CF_FOR_ELEMS(f, nf) {
        const int o = la[f], u = ua[f];
        if (o < 0 || o >= n || u < 0 || u >= n) atomicOr(err, ADDR_RANGE);
        else if (u <= o) atomicOr(err, ADDR_ORDER);
        if (f > 0 && la[f - 1] > o) atomicOr(err, ADDR_ORDER);
    }
}

// Caller-provided losort/losortStart/ownerStart: ranges and monotonicity.
__global__ void k_check_given(int n, int nf, const int32_t *__restrict__ losort,
                              const int32_t *__restrict__ ls, const int32_t *__restrict__ os,
                              int *err)
{
    CF_FOR_ELEMS(i, nf) {
        if (losort[i] < 0 || losort[i] >= nf) atomicOr(err, ADDR_RANGE);
    }
    CF_FOR_ELEMS(c, n + 1) {
        if (ls[c] < 0 || ls[c] > nf || os[c] < 0 || os[c] > nf) atomicOr(err, ADDR_START);
        if (c < n && (ls[c + 1] < ls[c] || os[c + 1] < os[c])) atomicOr(err, ADDR_START);
    }
}

// ownerStart[c] = first face whose owner is >= c (faces sorted by owner).
__global__ void k_owner_start(int n, int nf, const int32_t *__restrict__ la, int32_t *os)
{
    CF_FOR_ELEMS(c, n + 1) {
        int lo = 0, hi = nf;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (__ldg(la + mid) < c) lo = mid + 1;
            else hi = mid;
        }
        os[c] = lo;
    }
}

__global__ void k_count_neighbours(int nf, const int32_t *__restrict__ ua, int32_t *cnt)
{
    CF_FOR_ELEMS(f, nf) atomicAdd(cnt + ua[f], 1);
}

// Exclusive scan of m int32 values, three kernels: per-block inclusive scan
// with block totals, a single-block scan of the totals, then the fix-up.
constexpr int kScanBlock = 1024;

__device__ __forceinline__ int block_inclusive_scan(int v, int *sm)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(kFull, v, o);
        if (lane >= o) v += t;
    }
    if (lane == 31) sm[warp] = v;
    __syncthreads();
    if (warp == 0) {
        int w = (lane < (int)(blockDim.x >> 5)) ? sm[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(kFull, w, o);
            if (lane >= o) w += t;
        }
        sm[lane] = w;
    }
    __syncthreads();
    if (warp > 0) v += sm[warp - 1];
    __syncthreads();
    return v;
}

__global__ void k_scan_blocks(int m, const int32_t *__restrict__ in, int32_t *out, int32_t *sums)
{
    __shared__ int sm[32];
    const int i = blockIdx.x * kScanBlock + threadIdx.x;
    const int v = (i < m) ? in[i] : 0;
    const int inc = block_inclusive_scan(v, sm);
    if (i < m) out[i] = inc - v; // exclusive within the block
    if (threadIdx.x == kScanBlock - 1) sums[blockIdx.x] = inc;
}

__global__ void k_scan_sums(int nb, int32_t *sums)
{
    __shared__ int sm[32];
    const int per = (nb + kScanBlock - 1) / kScanBlock;
    const int b0 = threadIdx.x * per;
    int local = 0;
    for (int j = 0; j < per && b0 + j < nb; ++j) local += sums[b0 + j];
    const int inc = block_inclusive_scan(local, sm);
    int run = inc - local;
    for (int j = 0; j < per && b0 + j < nb; ++j) {
        const int t = sums[b0 + j];
        sums[b0 + j] = run;
        run += t;
    }
}

__global__ void k_scan_add(int m, int32_t *out, const int32_t *__restrict__ sums)
{
    const int i = blockIdx.x * kScanBlock + threadIdx.x;
    if (i < m) out[i] += sums[blockIdx.x];
}

// Place every face in its neighbour's losort segment (arbitrary order inside
// the segment), then sort each segment by face index: the result is the
// stable order of OpenFOAM's losort.
__global__ void k_losort_place(int nf, const int32_t *__restrict__ ua,
                               const int32_t *__restrict__ ls, int32_t *cursor, int32_t *losort)
{
    CF_FOR_ELEMS(f, nf) {
        const int u = ua[f];
        const int pos = ls[u] + atomicAdd(cursor + u, 1);
        losort[pos] = f;
    }
}

__global__ void k_losort_sort(int n, const int32_t *__restrict__ ls, int32_t *losort)
{
    CF_FOR_ELEMS(c, n) {
        const int b = ls[c], e = ls[c + 1];
        for (int i = b + 1; i < e; ++i) {
            const int v = losort[i];
            int j = i - 1;
            while (j >= b && losort[j] > v) {
                losort[j + 1] = losort[j];
                --j;
            }
            losort[j + 1] = v;
        }
    }
}

__global__ void k_row_offsets(int n, const int32_t *__restrict__ ls, const int32_t *__restrict__ os,
                              int32_t *ro)
{
    const int l0 = ls[0], o0 = os[0];
    CF_FOR_ELEMS(c, n + 1) ro[c] = (ls[c] - l0) + c + (os[c] - o0);
}

// One thread per cell, in the reference's entry order.  `col` may be null
// (value-only refresh); `lower`/`upper` swapped gives A^T on the same
// pattern (faces are structurally symmetric).
__global__ void k_fill_csr(int n, const int32_t *__restrict__ ls, const int32_t *__restrict__ os,
                           const int32_t *__restrict__ losort, const int32_t *__restrict__ la,
                           const int32_t *__restrict__ ua, const double *__restrict__ diag,
                           const double *__restrict__ lower, const double *__restrict__ upper,
                           const int32_t *__restrict__ ro, int32_t *col, double *val)
{
    CF_FOR_ELEMS(c, n) {
        int e = ro[c];
        for (int idx = ls[c]; idx < ls[c + 1]; ++idx) {
            const int face = losort[idx];
            if (col) col[e] = la[face];
            val[e] = lower[face];
            ++e;
        }
        if (col) col[e] = c;
        val[e] = diag[c];
        ++e;
        for (int face = os[c]; face < os[c + 1]; ++face) {
            if (col) col[e] = ua[face];
            val[e] = upper[face];
            ++e;
        }
    }
}

// out[0]: max nnz over the 32-row chunks without a row longer than
// kLongRow (the staging capacity the fast CSR passes need); out[1]: 1 if
// some row is longer (those chunks are read unstaged, long rows by the
// whole warp)
__global__ void k_chunk_stats(int n, const int32_t *__restrict__ ro, int *out)
{
    int m = 0, lng = 0;
    for (int base = (blockIdx.x * blockDim.x + threadIdx.x) * 32; base < n;
         base += gridDim.x * blockDim.x * 32) {
        const int top = base + 32 < n ? base + 32 : n;
        bool has = false;
        for (int r = base; r < top; ++r) has = has || (ro[r + 1] - ro[r] > kLongRow);
        if (has) {
            lng = 1;
        } else {
            const int c = ro[top] - ro[base];
            m = c > m ? c : m;
        }
    }
    atomicMax(out, m);
    if (lng) atomicMax(out + 1, 1);
}

__global__ void k_diag_derived(int n, const double *__restrict__ diag, double *dinv,
                               double *dinv_sqrt)
{
    // FindDiagInv / FindDiagInvSqrt (gis/SparseSystem/kernels.h:563-603)
    CF_FOR_ELEMS(c, n) {
        const double inv = 1.0 / diag[c];
        dinv[c] = inv;
        dinv_sqrt[c] = sqrt(inv);
    }
}

__global__ void k_to_f32(int64_t m, const double *__restrict__ src, float *dst)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m;
         i += (int64_t)gridDim.x * blockDim.x)
        dst[i] = (float)src[i];
}

__global__ void k_min_abs(int n, const double *__restrict__ v, double *out_bits_as_u64)
{
    // min |v| (order independent); non-negative doubles order like their bits
    double m = INFINITY;
    CF_FOR_ELEMS(i, n) m = fmin(m, fabs(v[i]));
    for (int o = 16; o > 0; o >>= 1) m = fmin(m, __shfl_down_sync(kFull, m, o));
    if ((threadIdx.x & 31) == 0)
        atomicMin(reinterpret_cast<unsigned long long *>(out_bits_as_u64),
                  (unsigned long long)__double_as_longlong(m));
}

// y = A x (SpMv, SolverSingleGPU.h:173-184); each row one FMA chain.
__global__ void __launch_bounds__(kBlock) k_spmv_fast(int n, int cap, const int32_t *__restrict__ ro,
                                                      const int32_t *__restrict__ col,
                                                      const double *__restrict__ val,
                                                      const double *__restrict__ x, double *y)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const int warp = threadIdx.x >> 5;
    unsigned char *area = smem + warp * stage_bytes_per_warp<double>(cap);
    double *sv = reinterpret_cast<double *>(area);
    int32_t *sc = reinterpret_cast<int32_t *>(area + (size_t)(cap + 8) * sizeof(double));
    CF_FOR_CHUNKS(base, n) {
        const Chunk<double> ch = stage_chunk<double>(ro, col, val, n, base, cap, sv, sc);
        const int row = base + (threadIdx.x & 31);
        const double v = row_chain<double>(ch, col, val, [&](int c) { return __ldg(x + c); });
        if (row < n) y[row] = v;
        __syncwarp();
    }
}

// y = A x with the reference's row order (the 8-lane tree of SpMvKernel).
__global__ void __launch_bounds__(kBlock) k_spmv(int n, int cap, const int32_t *__restrict__ ro,
                                                 const int32_t *__restrict__ col,
                                                 const double *__restrict__ val,
                                                 const double *__restrict__ x, double *y)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const int warp = threadIdx.x >> 5;
    unsigned char *area = smem + warp * stage_bytes_per_warp<double>(cap);
    double *sv = reinterpret_cast<double *>(area);
    int32_t *sc = reinterpret_cast<int32_t *>(area + (size_t)(cap + 8) * sizeof(double));
    CF_FOR_CHUNKS(base, n) {
        const Chunk<double> ch = stage_chunk<double>(ro, col, val, n, base, cap, sv, sc);
        const int row = base + (threadIdx.x & 31);
        const double v = row_product<double>(ch, col, val, [&](int c) { return __ldg(x + c); });
        if (row < n) y[row] = v;
        __syncwarp();
    }
}

// y = A x with the reference's row order, read from the SELL-32 copy (one
// warp per slice; the same bits as k_spmv).
__global__ void __launch_bounds__(kBlock) k_spmv_sell_ref(int n, int n_slices, const int32_t *__restrict__ off,
                                                          const int32_t *__restrict__ col,
                                                          const double *__restrict__ val,
                                                          const int32_t *__restrict__ ro,
                                                          const double *__restrict__ x, double *y)
{
    const int lane = threadIdx.x & 31;
    const int nw = gridDim.x * kWarps;
    for (int s = blockIdx.x * kWarps + (threadIdx.x >> 5); s < n_slices; s += nw) {
        const int b = __ldg(off + s);
        const int len = (__ldg(off + s + 1) - b) >> 5;
        const int row = s * 32 + lane;
        const int rl = row < n ? __ldg(ro + row + 1) - __ldg(ro + row) : 0;
        const double v = sell_ref_row(col + b + lane, val + b + lane, len, rl, [&](int c) { return __ldg(x + c); });
        if (row < n) y[row] = v;
    }
}

// ---------------------------------------------------------------------------
// SELL-32 copy (layout described in device.cuh)
// ---------------------------------------------------------------------------
// slot s: 32 x the longest row of slice s (slot n_slices = 0); the stored
// total accumulates in 64 bits
__global__ void k_sell_len(int n, int n_slices, const int32_t *__restrict__ ro, int32_t *slen,
                           unsigned long long *total)
{
    CF_FOR_ELEMS(s, n_slices + 1) {
        int mx = 0;
        if (s < n_slices) {
            const int r1 = min(n, 32 * s + 32);
            for (int r = 32 * s; r < r1; ++r) mx = max(mx, __ldg(ro + r + 1) - __ldg(ro + r));
            atomicAdd(total, 32ull * (unsigned long long)mx);
        }
        slen[s] = 32 * mx;
    }
}

// one thread per slot of the last slice's 32 rows (rows >= n hold value 0,
// column 0); pattern (scol != nullptr) and / or values
template <class S, class V>
__global__ void k_sell_fill(int n, int n_slices, const int32_t *__restrict__ ro,
                            const int32_t *__restrict__ col, const S *__restrict__ val,
                            const int32_t *__restrict__ soff, int32_t *scol, V *sval)
{
    CF_FOR_ELEMS(i, 32 * n_slices) {
        const int s = i >> 5, lane = i & 31;
        const int b = soff[s], len = (soff[s + 1] - b) >> 5;
        const int rs = i < n ? ro[i] : 0, re = i < n ? ro[i + 1] : 0;
        for (int t = 0; t < len; ++t) {
            const int j = rs + t;
            const int o = b + 32 * t + lane;
            if (scol) scol[o] = j < re ? col[j] : (i < n ? i : 0);
            if (sval) sval[o] = j < re ? (V)val[j] : V(0);
        }
    }
}

// One-byte column codes of the SELL-32 slots (SellCodes8, device.cuh): the
// distinct offsets d = col - row of the CSR entries, and 0 (the padding
// slots' offset), go into an open-addressing set on the device while the
// SELL-32 layout is sized; when there are at most kMaxCodes of them the host
// numbers them in ascending order and a pass over the slots writes each
// slot's number.
constexpr int kCodeHash = 1024;              // slots of the set (power of two, > 2 kMaxCodes)
constexpr int kCodeTable = kMaxCodes;        // entries of the offset table (unused ones 0)
constexpr int32_t kNoOffset = INT32_MIN;     // empty slot (|d| < n < 2^31)

__device__ __forceinline__ uint32_t offset_hash(int32_t d) { return ((uint32_t)d * 2654435761u) >> 22; }

// d into the set.  With at most kMaxCodes keys no probe sequence meets more
// than kMaxCodes occupied slots, so one that meets more proves an overflow:
// it marks the count past the limit (every thread then stops) instead of
// walking a table that thousands of offsets filled.
__device__ void offset_insert(int32_t *keys, int32_t *count, int32_t d)
{
    uint32_t h = offset_hash(d);
    for (int probe = 0; probe <= kMaxCodes + 1; ++probe, h = (h + 1) & (kCodeHash - 1)) {
        const int32_t k = *(volatile int32_t *)(keys + h);
        if (k == d) return;
        if (k == kNoOffset) {
            const int32_t old = atomicCAS(keys + h, kNoOffset, d);
            if (old == kNoOffset) {
                atomicAdd(count, 1);
                return;
            }
            if (old == d) return;
        }
    }
    atomicMax(count, kMaxCodes + 1);
}

// keys = empty, count = 0, largest |offset| = 0
__global__ void k_offsets_clear(int32_t *keys, int32_t *count)
{
    CF_FOR_ELEMS(i, kCodeHash) keys[i] = kNoOffset;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        count[0] = 0;
        count[1] = 0;
    }
}

// the largest |col - row| over the CSR entries (the 16-bit deltas' range)
__global__ void k_csr_maxoff(int n, const int32_t *__restrict__ ro, const int32_t *__restrict__ col, int32_t *maxoff)
{
    int m = 0;
    CF_FOR_ELEMS(i, n) {
        const int re = ro[i + 1];
        for (int j = ro[i]; j < re; ++j) m = max(m, abs(col[j] - i));
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) m = max(m, __shfl_xor_sync(kFull, m, o));
    if ((threadIdx.x & 31) == 0 && m > 0) atomicMax(maxoff, m);
}

// the 16-bit delta of every slot, lane-major within the slice like the codes
__global__ void k_sell_encode16(int n, int n_slices, const int32_t *__restrict__ soff,
                                const int32_t *__restrict__ scol, int16_t *d16)
{
    CF_FOR_ELEMS(i, 32 * n_slices) {
        const int s = i >> 5, lane = i & 31;
        const int b = soff[s], len = (soff[s + 1] - b) >> 5;
        const int rb = sell_row_base(i, n);
        for (int t = 0; t < len; ++t) d16[b + len * lane + t] = (int16_t)(scol[b + 32 * t + lane] - rb);
    }
}

// every CSR entry's offset, and 0; stops early once more than kMaxCodes
// distinct offsets are in the set (the codes cannot be used then).  Each
// thread remembers the last eight offsets it inserted in registers, so a
// stencil's few offsets reach the set (and its hot cache lines) once per
// thread, not once per entry.
__global__ void k_csr_offsets(int n, const int32_t *__restrict__ ro, const int32_t *__restrict__ col,
                              int32_t *keys, int32_t *count)
{
    if (blockIdx.x == 0 && threadIdx.x == 0) offset_insert(keys, count, 0);
    int32_t s0 = kNoOffset, s1 = kNoOffset, s2 = kNoOffset, s3 = kNoOffset;
    int32_t s4 = kNoOffset, s5 = kNoOffset, s6 = kNoOffset, s7 = kNoOffset;
    CF_FOR_ELEMS(i, n) {
        const int re = ro[i + 1];
        for (int j = ro[i]; j < re; ++j) {
            const int32_t d = col[j] - i;
            if (d == s0 || d == s1 || d == s2 || d == s3 || d == s4 || d == s5 || d == s6 || d == s7) continue;
            if (*(volatile int32_t *)count > kMaxCodes) return;
            offset_insert(keys, count, d);
            s7 = s6;
            s6 = s5;
            s5 = s4;
            s4 = s3;
            s3 = s2;
            s2 = s1;
            s1 = s0;
            s0 = d;
        }
    }
}

// each slot's code: the number of its offset (slot_code, by set position);
// every offset is in the set, found within kCodeHash probes.  A slice's
// codes are stored lane-major: lane l's len codes at b + len l.
__global__ void k_sell_encode(int n, int n_slices, const int32_t *__restrict__ soff,
                              const int32_t *__restrict__ scol, const int32_t *__restrict__ keys,
                              const uint8_t *__restrict__ slot_code, uint8_t *code)
{
    CF_FOR_ELEMS(i, 32 * n_slices) {
        const int s = i >> 5, lane = i & 31;
        const int b = soff[s], len = (soff[s + 1] - b) >> 5;
        const int rb = sell_row_base(i, n);
        for (int t = 0; t < len; ++t) {
            const int32_t d = scol[b + 32 * t + lane] - rb;
            uint32_t h = offset_hash(d);
            for (int probe = 0; probe < kCodeHash && keys[h] != d; ++probe) h = (h + 1) & (kCodeHash - 1);
            code[b + len * lane + t] = slot_code[h];   // lane-major within the slice
        }
    }
}

// y = A x over the SELL-32 copy (the fast order of k_spmv_fast).  Entries
// per batch and resident blocks per SM (0: no register constraint) are
// tuning constants; measured on the 7-point 128^3 product (100 launches
// back to back): 4 entries at 5 blocks/SM 37.0 us, 2 at 6 37.1, 8 with no
// constraint 39.1, 4 at 4 39.6, 3 at 5 41.2, 16 70.7.
#ifndef CF_PLAIN_SPMV_BATCH
#define CF_PLAIN_SPMV_BATCH 4
#endif
#ifndef CF_PLAIN_SPMV_MINB
#define CF_PLAIN_SPMV_MINB 5
#endif
// The same over the one-byte column codes, with its own constants: a batch
// fetches its codes as one 16-byte window, so a 7-entry row is best one
// batch.
#ifndef CF_PLAIN_SPMV8_BATCH
#define CF_PLAIN_SPMV8_BATCH 8
#endif
#ifndef CF_PLAIN_SPMV8_MINB
#define CF_PLAIN_SPMV8_MINB 4
#endif
// (COLS: 0 the 32-bit columns, 1 the one-byte codes and their offset table,
// 2 the 16-bit deltas)
template <int COLS>
__global__ void
__launch_bounds__(kBlock, COLS ? CF_PLAIN_SPMV8_MINB : (CF_PLAIN_SPMV_MINB > 0 ? CF_PLAIN_SPMV_MINB : 1))
    k_spmv_sell(int n, int n_slices, const int32_t *__restrict__ off, const int32_t *__restrict__ col,
                const uint8_t *__restrict__ code, const int32_t *__restrict__ tab, const int16_t *__restrict__ d16,
                const double *__restrict__ val, const int32_t *__restrict__ ro, int has_long,
                const double *__restrict__ x, double *y)
{
    auto g = [&](int c) { return __ldg(x + c); };
    auto f = [&](int row, double v) { y[row] = v; };
    if constexpr (COLS == 1)
        sell_rows<double, CF_PLAIN_SPMV8_BATCH>(n, n_slices, off, SellCodes8(code, tab), val, ro, has_long != 0, g, f);
    else if constexpr (COLS == 2)
        sell_rows<double, CF_PLAIN_SPMV8_BATCH>(n, n_slices, off, SellDelta16{d16}, val, ro, has_long != 0, g, f);
    else
        sell_rows<double, CF_PLAIN_SPMV_BATCH>(n, n_slices, off, SellCols32{col}, val, ro, has_long != 0, g, f);
}

// ---------------------------------------------------------------------------
// matrices given as CSR (the libGIS-compatible entry points)
// ---------------------------------------------------------------------------
// FindDiag (gis/SparseSystem/kernels.h:447-464): the entry with col == row,
// scanning the row while col <= row; rows without one read as 0.
__global__ void k_csr_diag(int n, const int32_t *__restrict__ ro, const int32_t *__restrict__ col,
                           const double *__restrict__ val, double *diag)
{
    CF_FOR_ELEMS(i, n) {
        double d = 0.0;
        for (int j = ro[i]; j < ro[i + 1] && col[j] <= i; ++j)
            if (col[j] == i) d = val[j];
        diag[i] = d;
    }
}

__global__ void k_csr_check(int n, int n_cols, const int32_t *__restrict__ ro,
                            const int32_t *__restrict__ col, int64_t nnz, int *err)
{
    CF_FOR_ELEMS(i, n) {
        const int b = ro[i], e = ro[i + 1];
        if (b < 0 || e < b || (int64_t)e > nnz) atomicOr(err, 1);
        else
            for (int j = b; j < e; ++j)
                if (col[j] < 0 || col[j] >= n_cols) atomicOr(err, 2);
    }
}

__global__ void k_count_cols(int n, const int32_t *__restrict__ ro, const int32_t *__restrict__ col,
                             int32_t *cnt)
{
    CF_FOR_ELEMS(i, n)
        for (int j = ro[i]; j < ro[i + 1]; ++j) atomicAdd(cnt + col[j], 1);
}

__global__ void k_transpose_place(int n, const int32_t *__restrict__ ro, const int32_t *__restrict__ col,
                                  const double *__restrict__ val, const int32_t *__restrict__ roT,
                                  int32_t *cursor, int32_t *colT, double *valT)
{
    CF_FOR_ELEMS(i, n)
        for (int j = ro[i]; j < ro[i + 1]; ++j) {
            const int c = col[j];
            const int pos = roT[c] + atomicAdd(cursor + c, 1);
            colT[pos] = i;
            valT[pos] = val[j];
        }
}

// sort each row of the transpose by (original) row index: the result equals
// a stable sort of A's entries by column, as the reference's Transpose
// (Thrust stable_sort_by_key, SolverSingleGPU.h:33-71) produces
__global__ void k_sort_rows(int n, const int32_t *__restrict__ ro, int32_t *col, double *val)
{
    CF_FOR_ELEMS(i, n) {
        const int b = ro[i], e = ro[i + 1];
        for (int j = b + 1; j < e; ++j) {
            const int c = col[j];
            const double v = val[j];
            int t = j - 1;
            while (t >= b && col[t] > c) {
                col[t + 1] = col[t];
                val[t + 1] = val[t];
                --t;
            }
            col[t + 1] = c;
            val[t + 1] = v;
        }
    }
}

// one thread per row i: for the k-th occurrence of column j in row i, the
// value of the k-th occurrence of column i in row j (err = 1 if missing)
__global__ void k_transpose_on_pattern(int n, const int32_t *__restrict__ ro, const int32_t *__restrict__ col,
                                       const double *__restrict__ val, double *valT, int *err)
{
    CF_FOR_ELEMS(i, n) {
        for (int e = ro[i]; e < ro[i + 1]; ++e) {
            const int j = col[e];
            int k = 0;
            for (int t = ro[i]; t < e; ++t) k += col[t] == j;
            int found = -1;
            for (int t = ro[j]; t < ro[j + 1]; ++t)
                if (col[t] == i && k-- == 0) {
                    found = t;
                    break;
                }
            if (found < 0) {
                atomicOr(err, 1);
                valT[e] = 0.0;
            } else {
                valT[e] = val[found];
            }
        }
    }
}

__global__ void k_same_pattern(int64_t m, const int32_t *__restrict__ a, const int32_t *__restrict__ b,
                               int *diff)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m;
         i += (int64_t)gridDim.x * blockDim.x)
        if (a[i] != b[i]) atomicOr(diff, 1);
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static int grid_for(Context *ctx, int64_t work, int per_block = kBlock)
{
    int64_t g = (work + per_block - 1) / per_block;
    const int64_t cap = (int64_t)ctx->sm_count * 16;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (int)g;
}

// The offset set of m's pattern (one-byte column codes) and its largest
// |offset| (16-bit deltas) into the context's scratch: keys [kCodeHash],
// count, largest |offset|, then the slot -> code map [kCodeHash] bytes.
// Enqueued only; read back with the SELL-32 size.
static void queue_offsets(Matrix *m)
{
    Context *ctx = m->ctx;
    ctx->scratch_codes.ensure(sizeof(int32_t) * (kCodeHash + 4) + kCodeHash);
    int32_t *keys = ctx->scratch_codes.as<int32_t>();
    k_offsets_clear<<<grid_for(ctx, kCodeHash), kBlock, 0, ctx->stream>>>(keys, keys + kCodeHash);
    CF_CHECK_LAUNCH();
    k_csr_offsets<<<grid_for(ctx, m->n), kBlock, 0, ctx->stream>>>(m->n, m->ro.as<int32_t>(), m->col.as<int32_t>(),
                                                                  keys, keys + kCodeHash);
    CF_CHECK_LAUNCH();
    k_csr_maxoff<<<grid_for(ctx, m->n), kBlock, 0, ctx->stream>>>(m->n, m->ro.as<int32_t>(), m->col.as<int32_t>(),
                                                                 keys + kCodeHash + 1);
    CF_CHECK_LAUNCH();
}

// The 16-bit column deltas of m's SELL-32 copy (every |offset| <= 32767).
static void build_sell_d16(Matrix *m)
{
    Context *ctx = m->ctx;
    m->s_d16.ensure(sizeof(int16_t) * ((size_t)m->sell_nnz + 32));
    k_sell_encode16<<<grid_for(ctx, 32 * (int64_t)m->n_slices), kBlock, 0, ctx->stream>>>(
        m->n, m->n_slices, m->s_off.as<int32_t>(), m->s_col.as<int32_t>(), m->s_d16.as<int16_t>());
    CF_CHECK_LAUNCH();
    m->has_d16 = true;
}

// The codes of m's SELL-32 copy from the offset set read back into hk /
// count, when the pattern has at most kMaxCodes distinct offsets (m->n_codes
// > 0 then).  Asynchronous: the host tables are staged by the copies.
static void build_sell_codes(Matrix *m, const std::vector<int32_t> &hk, int32_t count)
{
    Context *ctx = m->ctx;
    m->n_codes = 0;
    if (count <= 0 || count > kMaxCodes) return;
    std::vector<int32_t> offs;
    for (int32_t k : hk)
        if (k != kNoOffset) offs.push_back(k);
    if ((int)offs.size() != count) return;
    std::sort(offs.begin(), offs.end());
    std::vector<int32_t> tab(kCodeTable, 0);
    std::copy(offs.begin(), offs.end(), tab.begin());
    std::vector<uint8_t> slot_code(kCodeHash, 0);
    for (int h = 0; h < kCodeHash; ++h)
        if (hk[h] != kNoOffset)
            slot_code[h] = (uint8_t)(std::lower_bound(offs.begin(), offs.end(), hk[h]) - offs.begin());
    int32_t *keys = ctx->scratch_codes.as<int32_t>();
    uint8_t *map = reinterpret_cast<uint8_t *>(keys + kCodeHash + 4);
    m->s_dtab.ensure(sizeof(int32_t) * kCodeTable);
    m->s_code.ensure((size_t)m->sell_nnz + 64);
    // pageable sources: each copy returns once its bytes are staged
    CF_CUDA(cudaMemcpyAsync(m->s_dtab.ptr, tab.data(), sizeof(int32_t) * kCodeTable, cudaMemcpyHostToDevice,
                            ctx->stream));
    CF_CUDA(cudaMemcpyAsync(map, slot_code.data(), kCodeHash, cudaMemcpyHostToDevice, ctx->stream));
    const int ns = m->n_slices;
    k_sell_encode<<<grid_for(ctx, 32 * (int64_t)ns), kBlock, 0, ctx->stream>>>(
        m->n, ns, m->s_off.as<int32_t>(), m->s_col.as<int32_t>(), keys, map, m->s_code.as<uint8_t>());
    CF_CHECK_LAUNCH();
    m->n_codes = count;
}

static void exclusive_scan(Context *ctx, int m, const int32_t *in, int32_t *out, DeviceBuffer &tmp)
{
    const int nb = (m + kScanBlock - 1) / kScanBlock;
    tmp.ensure(sizeof(int32_t) * (size_t)(nb + 1));
    k_scan_blocks<<<nb, kScanBlock, 0, ctx->stream>>>(m, in, out, tmp.as<int32_t>());
    CF_CHECK_LAUNCH();
    k_scan_sums<<<1, kScanBlock, 0, ctx->stream>>>(nb, tmp.as<int32_t>());
    CF_CHECK_LAUNCH();
    k_scan_add<<<nb, kScanBlock, 0, ctx->stream>>>(m, out, tmp.as<int32_t>());
    CF_CHECK_LAUNCH();
}

static int read_flag(Context *ctx, const int *d_flag)
{
    int h = 0;
    CF_CUDA(cudaMemcpyAsync(&h, d_flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    CF_CUDA(cudaStreamSynchronize(ctx->stream));
    return h;
}

// chunk statistics of m's CSR pattern into m->max_chunk / m->has_long
static void chunk_stats(Context *ctx, Matrix *m)
{
    DeviceBuffer &buf = ctx->scratch_stats;
    buf.ensure(2 * sizeof(int));
    CF_CUDA(cudaMemsetAsync(buf.ptr, 0, 2 * sizeof(int), ctx->stream));
    if (m->n > 0) {
        k_chunk_stats<<<grid_for(ctx, ((int64_t)m->n + 31) / 32), kBlock, 0, ctx->stream>>>(
            m->n, m->ro.as<int32_t>(), buf.as<int>());
        CF_CHECK_LAUNCH();
    }
    int h[2] = {0, 0};
    CF_CUDA(cudaMemcpyAsync(h, buf.ptr, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
    CF_CUDA(cudaStreamSynchronize(ctx->stream));
    m->max_chunk = h[0];
    m->has_long = h[1] != 0;
}

// Copies the LDU arrays to `m`, validates and completes the addressing,
// builds the CSR.  When `out_*` are given the CSR is written there instead.
// full = false: the CSR arrays only (a one-shot conversion), without the
// staging statistics and the diagonal-derived vectors the solvers use
static void build_from_ldu(Context *ctx, Matrix *m, const cf_ldu_view &v, bool full = true)
{
    const int n = v.n_cells, nf = v.n_faces;
    require(n >= 0 && nf >= 0, CF_BAD_INPUT, "negative matrix size");
    require((int64_t)n + 2 * (int64_t)nf < (int64_t)INT32_MAX - 16, CF_BAD_INPUT,
            "matrix too large for 32-bit CSR offsets");
    require(n == 0 || v.diag, CF_BAD_INPUT, "diag is null");
    require(nf == 0 || (v.lower && v.upper && v.lower_addr && v.upper_addr), CF_BAD_INPUT,
            "face arrays are null");
    const bool given = v.losort || v.losort_start || v.owner_start;
    require(!given || (v.losort && v.losort_start && v.owner_start), CF_BAD_INPUT,
            "losort, losort_start and owner_start must be given together");
    m->n = n;
    m->nf = nf;
    m->nnz = (int64_t)n + 2 * (int64_t)nf;
    const size_t pad = 4;
    m->diag.ensure(sizeof(double) * (n + pad));
    m->lower.ensure(sizeof(double) * (nf + pad));
    m->upper.ensure(sizeof(double) * (nf + pad));
    m->la.ensure(sizeof(int32_t) * (nf + pad));
    m->ua.ensure(sizeof(int32_t) * (nf + pad));
    m->losort.ensure(sizeof(int32_t) * (nf + pad));
    m->lstart.ensure(sizeof(int32_t) * (n + 1 + pad));
    m->ostart.ensure(sizeof(int32_t) * (n + 1 + pad));
    upload(ctx, m->diag.ptr, v.diag, sizeof(double) * n, v.memory);
    upload(ctx, m->lower.ptr, v.lower, sizeof(double) * nf, v.memory);
    upload(ctx, m->upper.ptr, v.upper, sizeof(double) * nf, v.memory);
    upload(ctx, m->la.ptr, v.lower_addr, sizeof(int32_t) * nf, v.memory);
    upload(ctx, m->ua.ptr, v.upper_addr, sizeof(int32_t) * nf, v.memory);

    DeviceBuffer &flag = ctx->scratch_flag, &tmp = ctx->scratch_tmp, &cnt = ctx->scratch_cnt;
    flag.ensure(sizeof(int) * 4);
    CF_CUDA(cudaMemsetAsync(flag.ptr, 0, sizeof(int) * 4, ctx->stream));
    int *d_err = flag.as<int>();
    const int gf = grid_for(ctx, nf > 0 ? nf : 1);
    const int gc = grid_for(ctx, (int64_t)n + 1);
    if (nf > 0) {
        k_check_faces<<<gf, kBlock, 0, ctx->stream>>>(n, nf, m->la.as<int32_t>(), m->ua.as<int32_t>(), d_err);
        CF_CHECK_LAUNCH();
    }
    if (given) {
        upload(ctx, m->losort.ptr, v.losort, sizeof(int32_t) * nf, v.memory);
        upload(ctx, m->lstart.ptr, v.losort_start, sizeof(int32_t) * (n + 1), v.memory);
        upload(ctx, m->ostart.ptr, v.owner_start, sizeof(int32_t) * (n + 1), v.memory);
        k_check_given<<<gc, kBlock, 0, ctx->stream>>>(n, nf, m->losort.as<int32_t>(),
                                                      m->lstart.as<int32_t>(), m->ostart.as<int32_t>(), d_err);
        CF_CHECK_LAUNCH();
    } else {
        k_owner_start<<<gc, kBlock, 0, ctx->stream>>>(n, nf, m->la.as<int32_t>(), m->ostart.as<int32_t>());
        CF_CHECK_LAUNCH();
    }
    int err = read_flag(ctx, d_err);
    require(err == 0, CF_BAD_INPUT,
            std::string("invalid LDU addressing:") + ((err & ADDR_RANGE) ? " index out of range" : "") +
                ((err & ADDR_ORDER) ? " faces not sorted by owner or not upper-triangular" : "") +
                ((err & ADDR_START) ? " bad losortStart/ownerStart" : ""));
    if (!given) {
        cnt.ensure(sizeof(int32_t) * (size_t)(n + 1));
        CF_CUDA(cudaMemsetAsync(cnt.ptr, 0, sizeof(int32_t) * (size_t)(n + 1), ctx->stream));
        if (nf > 0) {
            k_count_neighbours<<<gf, kBlock, 0, ctx->stream>>>(nf, m->ua.as<int32_t>(), cnt.as<int32_t>());
            CF_CHECK_LAUNCH();
        }
        exclusive_scan(ctx, n + 1, cnt.as<int32_t>(), m->lstart.as<int32_t>(), tmp);
        CF_CUDA(cudaMemsetAsync(cnt.ptr, 0, sizeof(int32_t) * (size_t)(n + 1), ctx->stream));
        if (nf > 0) {
            k_losort_place<<<gf, kBlock, 0, ctx->stream>>>(nf, m->ua.as<int32_t>(), m->lstart.as<int32_t>(),
                                                           cnt.as<int32_t>(), m->losort.as<int32_t>());
            CF_CHECK_LAUNCH();
            k_losort_sort<<<gc, kBlock, 0, ctx->stream>>>(n, m->lstart.as<int32_t>(), m->losort.as<int32_t>());
            CF_CHECK_LAUNCH();
        }
    }
    m->ro.ensure(sizeof(int32_t) * (n + 1 + pad));
    k_row_offsets<<<gc, kBlock, 0, ctx->stream>>>(n, m->lstart.as<int32_t>(), m->ostart.as<int32_t>(),
                                                   m->ro.as<int32_t>());
    CF_CHECK_LAUNCH();
    // the counts must describe exactly n + 2F entries
    int32_t last = 0;
    CF_CUDA(cudaMemcpyAsync(&last, m->ro.as<int32_t>() + n, sizeof(int32_t), cudaMemcpyDeviceToHost,
                            ctx->stream));
    CF_CUDA(cudaStreamSynchronize(ctx->stream));
    require((int64_t)last == m->nnz, CF_BAD_INPUT,
            "losortStart/ownerStart do not describe n + 2*nFaces entries");
    m->col.ensure(sizeof(int32_t) * (m->nnz + pad));
    m->val.ensure(sizeof(double) * (m->nnz + pad));
    // zero the padding read by 16-byte vector loads past nnz
    CF_CUDA(cudaMemsetAsync(m->col.as<int32_t>() + m->nnz, 0, sizeof(int32_t) * pad, ctx->stream));
    CF_CUDA(cudaMemsetAsync(m->val.as<double>() + m->nnz, 0, sizeof(double) * pad, ctx->stream));
    if (n > 0) {
        k_fill_csr<<<gc, kBlock, 0, ctx->stream>>>(n, m->lstart.as<int32_t>(), m->ostart.as<int32_t>(),
                                                   m->losort.as<int32_t>(), m->la.as<int32_t>(),
                                                   m->ua.as<int32_t>(), m->diag.as<double>(),
                                                   m->lower.as<double>(), m->upper.as<double>(),
                                                   m->ro.as<int32_t>(), m->col.as<int32_t>(),
                                                   m->val.as<double>());
        CF_CHECK_LAUNCH();
    }
    if (!full) return;
    // staging capacity and long rows
    chunk_stats(ctx, m);
    m->dinv.ensure(sizeof(double) * (n + pad));
    m->dinv_sqrt.ensure(sizeof(double) * (n + pad));
    if (n > 0) {
        k_diag_derived<<<gc, kBlock, 0, ctx->stream>>>(n, m->diag.as<double>(), m->dinv.as<double>(),
                                                       m->dinv_sqrt.as<double>());
        CF_CHECK_LAUNCH();
    }
    m->have_valT = m->have_32 = m->have_T32 = m->have_dmin = false;
    ++m->gen;
}

Matrix *matrix_create(Context *ctx, const cf_ldu_view &v)
{
    Matrix *m = new Matrix();
    m->ctx = ctx;
    try {
        build_from_ldu(ctx, m, v);
    } catch (...) {
        delete m;
        throw;
    }
    return m;
}

void matrix_update_values(Matrix *m, const double *diag, const double *lower, const double *upper,
                          int memory)
{
    Context *ctx = m->ctx;
    require(!m->from_csr, CF_UNSUPPORTED, "the matrix was created from CSR arrays (no LDU coefficients)");
    require(diag && (m->nf == 0 || (lower && upper)), CF_BAD_INPUT, "null coefficient array");
    upload(ctx, m->diag.ptr, diag, sizeof(double) * m->n, memory);
    upload(ctx, m->lower.ptr, lower, sizeof(double) * m->nf, memory);
    upload(ctx, m->upper.ptr, upper, sizeof(double) * m->nf, memory);
    const int gc = grid_for(ctx, (int64_t)m->n + 1);
    if (m->n > 0) {
        k_fill_csr<<<gc, kBlock, 0, ctx->stream>>>(m->n, m->lstart.as<int32_t>(), m->ostart.as<int32_t>(),
                                                   m->losort.as<int32_t>(), m->la.as<int32_t>(),
                                                   m->ua.as<int32_t>(), m->diag.as<double>(),
                                                   m->lower.as<double>(), m->upper.as<double>(),
                                                   m->ro.as<int32_t>(), nullptr, m->val.as<double>());
        CF_CHECK_LAUNCH();
        k_diag_derived<<<gc, kBlock, 0, ctx->stream>>>(m->n, m->diag.as<double>(), m->dinv.as<double>(),
                                                       m->dinv_sqrt.as<double>());
        CF_CHECK_LAUNCH();
    }
    m->have_valT = m->have_32 = m->have_T32 = m->have_dmin = false;
    m->have_sval = m->have_svalT = m->have_sval32 = m->have_svalT32 = false;
    ++m->gen;
}

// A^T values on A's pattern: the same fill with lower and upper swapped.
// Equals the reference's Transpose (Thrust stable sort by column,
// SolverSingleGPU.h:33-71) because row c of A^T lists A[i][c] by ascending i.
static void matrix_transpose_from_csr(Matrix *m);

void matrix_ensure_transpose(Matrix *m)
{
    if (m->have_valT) return;
    if (m->from_csr) {
        matrix_transpose_from_csr(m);
        return;
    }
    Context *ctx = m->ctx;
    m->valT.ensure(sizeof(double) * (m->nnz + 4));
    CF_CUDA(cudaMemsetAsync(m->valT.as<double>() + m->nnz, 0, sizeof(double) * 4, ctx->stream));
    if (m->n > 0) {
        k_fill_csr<<<grid_for(ctx, (int64_t)m->n + 1), kBlock, 0, ctx->stream>>>(
            m->n, m->lstart.as<int32_t>(), m->ostart.as<int32_t>(), m->losort.as<int32_t>(),
            m->la.as<int32_t>(), m->ua.as<int32_t>(), m->diag.as<double>(), m->upper.as<double>(),
            m->lower.as<double>(), m->ro.as<int32_t>(), nullptr, m->valT.as<double>());
        CF_CHECK_LAUNCH();
    }
    m->have_valT = true;
}

void matrix_ensure_fp32(Matrix *m, bool transpose)
{
    Context *ctx = m->ctx;
    if (!transpose && m->have_32) return;
    if (transpose && m->have_T32) return;
    if (transpose) matrix_ensure_transpose(m);
    DeviceBuffer &dst = transpose ? m->valT32 : m->val32;
    const double *src = transpose ? m->valT.as<double>() : m->val.as<double>();
    dst.ensure(sizeof(float) * (m->nnz + 4));
    CF_CUDA(cudaMemsetAsync(dst.as<float>() + m->nnz, 0, sizeof(float) * 4, ctx->stream));
    if (m->nnz > 0) {
        k_to_f32<<<grid_for(ctx, m->nnz), kBlock, 0, ctx->stream>>>(m->nnz, src, dst.as<float>());
        CF_CHECK_LAUNCH();
    }
    (transpose ? m->have_T32 : m->have_32) = true;
}

// FindDiagAbsMin (SolverSingleGPU.h:686-720): min |a_ii|.
void matrix_ensure_dmin(Matrix *m)
{
    if (m->have_dmin) return;
    Context *ctx = m->ctx;
    DeviceBuffer b;
    b.ensure(sizeof(double));
    const double inf = INFINITY;
    CF_CUDA(cudaMemcpyAsync(b.ptr, &inf, sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    if (m->n > 0) {
        k_min_abs<<<grid_for(ctx, m->n), kBlock, 0, ctx->stream>>>(m->n, m->diag.as<double>(), b.as<double>());
        CF_CHECK_LAUNCH();
    }
    double h = 0;
    CF_CUDA(cudaMemcpyAsync(&h, b.ptr, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    CF_CUDA(cudaStreamSynchronize(ctx->stream));
    m->diag_abs_min = h;
    m->have_dmin = true;
}

// The conversion runs in the context's scratch matrix, whose buffers only
// grow: after the first call of a size a conversion allocates nothing
// (device allocations and frees would dominate a small mesh's conversion).
void ldu2csr_into(Context *ctx, const cf_ldu_view &v, int32_t *ro, int32_t *col, double *val,
                  int memory)
{
    if (!ctx->ldu_scratch) {
        ctx->ldu_scratch = new Matrix();
        ctx->ldu_scratch->ctx = ctx;
    }
    Matrix &tmp = *ctx->ldu_scratch;
    build_from_ldu(ctx, &tmp, v, false);
    download(ctx, ro, tmp.ro.ptr, sizeof(int32_t) * (size_t)(tmp.n + 1), memory);
    download(ctx, col, tmp.col.ptr, sizeof(int32_t) * (size_t)tmp.nnz, memory);
    download(ctx, val, tmp.val.ptr, sizeof(double) * (size_t)tmp.nnz, memory);
    CF_CUDA(cudaStreamSynchronize(ctx->stream));
}

// General device transpose of an n_rows x n_cols CSR matrix into caller
// buffers (roT[n_cols+1], colT[nnz], valT[nnz]).
void csr_transpose(Context *ctx, int n_rows, int n_cols, int64_t nnz, const int32_t *ro,
                   const int32_t *col, const double *val, int32_t *roT, int32_t *colT, double *valT)
{
    DeviceBuffer cnt, tmp;
    cnt.ensure(sizeof(int32_t) * ((size_t)n_cols + 1));
    const int g = grid_for(ctx, (int64_t)n_rows + 1);
    // column counts in cnt[0..n_cols-1], cnt[n_cols] = 0: the exclusive scan
    // is the row offsets of A^T
    CF_CUDA(cudaMemsetAsync(cnt.ptr, 0, sizeof(int32_t) * ((size_t)n_cols + 1), ctx->stream));
    if (n_rows > 0) {
        k_count_cols<<<g, kBlock, 0, ctx->stream>>>(n_rows, ro, col, cnt.as<int32_t>());
        CF_CHECK_LAUNCH();
    }
    exclusive_scan(ctx, n_cols + 1, cnt.as<int32_t>(), roT, tmp);
    CF_CUDA(cudaMemsetAsync(cnt.ptr, 0, sizeof(int32_t) * ((size_t)n_cols + 1), ctx->stream));
    if (n_rows > 0) {
        k_transpose_place<<<g, kBlock, 0, ctx->stream>>>(n_rows, ro, col, val, roT, cnt.as<int32_t>(),
                                                         colT, valT);
        CF_CHECK_LAUNCH();
    }
    if (n_cols > 0) {
        k_sort_rows<<<grid_for(ctx, n_cols), kBlock, 0, ctx->stream>>>(n_cols, roT, colT, valT);
        CF_CHECK_LAUNCH();
    }
}

static bool same_pattern(Context *ctx, int64_t m, const int32_t *a, const int32_t *b)
{
    if (m == 0) return true;
    DeviceBuffer flag;
    flag.ensure(sizeof(int));
    CF_CUDA(cudaMemsetAsync(flag.ptr, 0, sizeof(int), ctx->stream));
    k_same_pattern<<<grid_for(ctx, m), kBlock, 0, ctx->stream>>>(m, a, b, flag.as<int>());
    CF_CHECK_LAUNCH();
    return read_flag(ctx, flag.as<int>()) == 0;
}

// A device matrix from a square CSR matrix in device memory (copied into
// padded buffers; the diagonal found as the reference's FindDiag does).
Matrix *matrix_from_csr(Context *ctx, int n, int64_t nnz, const int32_t *ro, const int32_t *col,
                        const double *val)
{
    require(n > 0 && nnz >= 0 && nnz < INT32_MAX, CF_BAD_INPUT, "bad CSR size");
    Matrix *m = new Matrix();
    try {
        m->ctx = ctx;
        m->n = n;
        m->nf = -1;
        m->nnz = nnz;
        m->from_csr = true;
        const size_t pad = 4;
        m->ro.ensure(sizeof(int32_t) * (n + 1 + pad));
        m->col.ensure(sizeof(int32_t) * (nnz + pad));
        m->val.ensure(sizeof(double) * (nnz + pad));
        CF_CUDA(cudaMemcpyAsync(m->ro.ptr, ro, sizeof(int32_t) * (n + 1), cudaMemcpyDeviceToDevice, ctx->stream));
        CF_CUDA(cudaMemcpyAsync(m->col.ptr, col, sizeof(int32_t) * nnz, cudaMemcpyDeviceToDevice, ctx->stream));
        CF_CUDA(cudaMemcpyAsync(m->val.ptr, val, sizeof(double) * nnz, cudaMemcpyDeviceToDevice, ctx->stream));
        CF_CUDA(cudaMemsetAsync(m->col.as<int32_t>() + nnz, 0, sizeof(int32_t) * pad, ctx->stream));
        CF_CUDA(cudaMemsetAsync(m->val.as<double>() + nnz, 0, sizeof(double) * pad, ctx->stream));
        DeviceBuffer flag;
        flag.ensure(sizeof(int) * 2);
        CF_CUDA(cudaMemsetAsync(flag.ptr, 0, sizeof(int) * 2, ctx->stream));
        const int gc = grid_for(ctx, (int64_t)n + 1);
        k_csr_check<<<gc, kBlock, 0, ctx->stream>>>(n, n, m->ro.as<int32_t>(), m->col.as<int32_t>(), nnz,
                                                    flag.as<int>());
        CF_CHECK_LAUNCH();
        int32_t last = 0;
        CF_CUDA(cudaMemcpyAsync(&last, m->ro.as<int32_t>() + n, sizeof(int32_t), cudaMemcpyDeviceToHost,
                                ctx->stream));
        const int err = read_flag(ctx, flag.as<int>());
        require(err == 0 && (int64_t)last == nnz, CF_BAD_INPUT, "invalid CSR matrix");
        m->diag.ensure(sizeof(double) * (n + pad));
        k_csr_diag<<<gc, kBlock, 0, ctx->stream>>>(n, m->ro.as<int32_t>(), m->col.as<int32_t>(),
                                                   m->val.as<double>(), m->diag.as<double>());
        CF_CHECK_LAUNCH();
        m->dinv.ensure(sizeof(double) * (n + pad));
        m->dinv_sqrt.ensure(sizeof(double) * (n + pad));
        k_diag_derived<<<gc, kBlock, 0, ctx->stream>>>(n, m->diag.as<double>(), m->dinv.as<double>(),
                                                       m->dinv_sqrt.as<double>());
        CF_CHECK_LAUNCH();
        chunk_stats(ctx, m);
    } catch (...) {
        delete m;
        throw;
    }
    return m;
}

// New values on a CSR-built matrix's pattern: the diagonal and its derived
// vectors are refreshed on the device, every other value copy is rebuilt
// when next needed.
void matrix_update_csr_values(Matrix *m, const double *vals, int memory)
{
    Context *ctx = m->ctx;
    require(m->from_csr, CF_UNSUPPORTED,
            "the matrix was created from LDU coefficients (its values change through cf_matrix_update_values)");
    require(vals || m->nnz == 0, CF_BAD_INPUT, "null value array");
    if (m->nnz > 0) upload(ctx, m->val.ptr, vals, sizeof(double) * (size_t)m->nnz, memory);
    const int gc = grid_for(ctx, (int64_t)m->n + 1);
    k_csr_diag<<<gc, kBlock, 0, ctx->stream>>>(m->n, m->ro.as<int32_t>(), m->col.as<int32_t>(), m->val.as<double>(),
                                               m->diag.as<double>());
    CF_CHECK_LAUNCH();
    k_diag_derived<<<gc, kBlock, 0, ctx->stream>>>(m->n, m->diag.as<double>(), m->dinv.as<double>(),
                                                   m->dinv_sqrt.as<double>());
    CF_CHECK_LAUNCH();
    m->have_valT = m->have_32 = m->have_T32 = m->have_dmin = false;
    m->have_sval = m->have_svalT = m->have_sval32 = m->have_svalT32 = false;
    ++m->gen;
}

// A^T values on A's pattern from a CSR A^T (given, or computed): the
// patterns must coincide (true for every LDU matrix).
void matrix_set_transpose_csr(Matrix *m, const int32_t *roT, const int32_t *colT, const double *valT)
{
    Context *ctx = m->ctx;
    require(same_pattern(ctx, (int64_t)m->n + 1, m->ro.as<int32_t>(), roT) &&
                same_pattern(ctx, m->nnz, m->col.as<int32_t>(), colT),
            CF_UNSUPPORTED, "A^T must have the sparsity pattern of A (structurally symmetric matrix)");
    m->valT.ensure(sizeof(double) * (m->nnz + 4));
    CF_CUDA(cudaMemcpyAsync(m->valT.ptr, valT, sizeof(double) * m->nnz, cudaMemcpyDeviceToDevice, ctx->stream));
    CF_CUDA(cudaMemsetAsync(m->valT.as<double>() + m->nnz, 0, sizeof(double) * 4, ctx->stream));
    m->have_valT = true;
    m->have_T32 = false;
    m->have_svalT = m->have_svalT32 = false;
    ++m->gen;
}

static void matrix_transpose_from_csr(Matrix *m)
{
    // A^T values on A's own pattern, whatever the order of A's rows: the
    // k-th entry (i, j) of row i takes the k-th entry (j, i) of row j
    Context *ctx = m->ctx;
    m->valT.ensure(sizeof(double) * ((size_t)m->nnz + 4));
    CF_CUDA(cudaMemsetAsync(m->valT.as<double>() + m->nnz, 0, sizeof(double) * 4, ctx->stream));
    DeviceBuffer flag;
    flag.ensure(sizeof(int));
    CF_CUDA(cudaMemsetAsync(flag.ptr, 0, sizeof(int), ctx->stream));
    if (m->n > 0) {
        k_transpose_on_pattern<<<grid_for(ctx, m->n), kBlock, 0, ctx->stream>>>(
            m->n, m->ro.as<int32_t>(), m->col.as<int32_t>(), m->val.as<double>(), m->valT.as<double>(),
            flag.as<int>());
        CF_CHECK_LAUNCH();
    }
    require(read_flag(ctx, flag.as<int>()) == 0, CF_UNSUPPORTED,
            "A^T needs a structurally symmetric matrix (every (i, j) entry matched by a (j, i) entry)");
    m->have_valT = true;
    m->have_T32 = false;
    m->have_svalT = m->have_svalT32 = false;
    ++m->gen;
}

// Decide the fast kernels' format (once per pattern) and bring the SELL-32
// value copies up to date: FP64 A, plus A^T (transpose) and FP32 (fp32)
// copies when asked.  Returns whether the fast kernels use SELL-32.
bool matrix_ensure_sell(Matrix *m, bool transpose, bool fp32)
{
    Context *ctx = m->ctx;
    if (m->sell < 0) {
        m->sell = 0;
        if (m->format_request != CF_FORMAT_CSR && m->n > 0) {
            const int ns = (m->n + 31) / 32;
            m->s_off.ensure(sizeof(int32_t) * ((size_t)ns + 1));
            DeviceBuffer slen, tmp, tot;
            slen.ensure(sizeof(int32_t) * ((size_t)ns + 1));
            tot.ensure(sizeof(unsigned long long));
            CF_CUDA(cudaMemsetAsync(tot.ptr, 0, sizeof(unsigned long long), ctx->stream));
            k_sell_len<<<grid_for(ctx, (int64_t)ns + 1), kBlock, 0, ctx->stream>>>(
                m->n, ns, m->ro.as<int32_t>(), slen.as<int32_t>(), tot.as<unsigned long long>());
            CF_CHECK_LAUNCH();
            const int req = m->format_request;
            const bool want_codes = req == CF_FORMAT_AUTO || req == CF_FORMAT_SELL_C8;
            const bool want_d16 = req == CF_FORMAT_AUTO || req == CF_FORMAT_SELL_D16;
            if (want_codes || want_d16) queue_offsets(m);
            unsigned long long total = 0;
            std::vector<int32_t> hk(want_codes || want_d16 ? kCodeHash + 2 : 0);
            CF_CUDA(cudaMemcpyAsync(&total, tot.ptr, sizeof(total), cudaMemcpyDeviceToHost, ctx->stream));
            if (want_codes || want_d16)
                CF_CUDA(cudaMemcpyAsync(hk.data(), ctx->scratch_codes.ptr, sizeof(int32_t) * (kCodeHash + 2),
                                        cudaMemcpyDeviceToHost, ctx->stream));
            CF_CUDA(cudaStreamSynchronize(ctx->stream));
            const bool fits = total < (unsigned long long)INT32_MAX - 64;
            const bool good = fits && (double)total <= 1.2 * (double)m->nnz + 32.0 * 8 &&
                              m->nnz <= 32 * (int64_t)m->n;
            const bool forced = req == CF_FORMAT_SELL || req == CF_FORMAT_SELL_C8 || req == CF_FORMAT_SELL_D16;
            require(!forced || fits, CF_UNSUPPORTED, "SELL-32 copy exceeds 2^31 entries");
            if (forced || good) {
                exclusive_scan(ctx, ns + 1, slen.as<int32_t>(), m->s_off.as<int32_t>(), tmp);
                m->n_slices = ns;
                m->sell_nnz = (int64_t)total;
                m->s_col.ensure(sizeof(int32_t) * ((size_t)total + 32));
                k_sell_fill<double, double><<<grid_for(ctx, 32 * (int64_t)ns), kBlock, 0, ctx->stream>>>(
                    m->n, ns, m->ro.as<int32_t>(), m->col.as<int32_t>(), nullptr, m->s_off.as<int32_t>(),
                    m->s_col.as<int32_t>(), (double *)nullptr);
                CF_CHECK_LAUNCH();
                m->sell = 1;
                m->n_codes = 0;
                m->has_d16 = false;
                const int32_t count = (want_codes || want_d16) ? hk[kCodeHash] : 0;
                const int32_t maxoff = (want_codes || want_d16) ? hk[kCodeHash + 1] : INT32_MAX;
                if (want_codes) {
                    hk.resize(kCodeHash);
                    build_sell_codes(m, hk, count);
                }
                if (want_d16 && m->n_codes == 0 && maxoff <= 32767) build_sell_d16(m);
                if (req == CF_FORMAT_SELL_C8 && m->n_codes == 0) {
                    m->sell = -1;   // decided again (and refused again) by the next call
                    throw Error{CF_UNSUPPORTED,
                                "one-byte column codes need at most " + std::to_string(kMaxCodes) +
                                    " distinct column offsets col - row"};
                }
                if (req == CF_FORMAT_SELL_D16 && !m->has_d16) {
                    m->sell = -1;
                    throw Error{CF_UNSUPPORTED, "16-bit column deltas need every |col - row| <= 32767"};
                }
            }
        }
        m->have_sval = m->have_svalT = m->have_sval32 = m->have_svalT32 = false;
        ++m->gen;
    }
    if (m->sell != 1) return false;
    if (transpose) matrix_ensure_transpose(m);
    auto fill = [&](const double *src, DeviceBuffer &dst, bool f32) {
        const int ns = m->n_slices;
        const dim3 g(grid_for(ctx, 32 * (int64_t)ns));
        if (f32) {
            dst.ensure(sizeof(float) * ((size_t)m->sell_nnz + 32));
            k_sell_fill<double, float><<<g, kBlock, 0, ctx->stream>>>(m->n, ns, m->ro.as<int32_t>(),
                                                                      m->col.as<int32_t>(), src,
                                                                      m->s_off.as<int32_t>(), nullptr,
                                                                      dst.as<float>());
        } else {
            dst.ensure(sizeof(double) * ((size_t)m->sell_nnz + 32));
            k_sell_fill<double, double><<<g, kBlock, 0, ctx->stream>>>(m->n, ns, m->ro.as<int32_t>(),
                                                                       m->col.as<int32_t>(), src,
                                                                       m->s_off.as<int32_t>(), nullptr,
                                                                       dst.as<double>());
        }
        CF_CHECK_LAUNCH();
    };
    if (!m->have_sval) {
        fill(m->val.as<double>(), m->s_val, false);
        m->have_sval = true;
    }
    if (transpose && !m->have_svalT) {
        fill(m->valT.as<double>(), m->s_valT, false);
        m->have_svalT = true;
    }
    if (fp32 && !m->have_sval32) {
        fill(m->val.as<double>(), m->s_val32, true);
        m->have_sval32 = true;
    }
    if (fp32 && transpose && !m->have_svalT32) {
        fill(m->valT.as<double>(), m->s_valT32, true);
        m->have_svalT32 = true;
    }
    return true;
}

// 1/a_ii taken from a diagonal preconditioner matrix (MRS's invM).
void matrix_set_inverse_diagonal(Matrix *m, const double *dinv)
{
    Context *ctx = m->ctx;
    CF_CUDA(cudaMemcpyAsync(m->dinv.ptr, dinv, sizeof(double) * m->n, cudaMemcpyDeviceToDevice, ctx->stream));
    ++m->gen;
}

int stage_cap_for(const Matrix *m)
{
    // stage a warp's rows when they fit a modest per-warp buffer
    if (m->max_chunk <= 256) return 256;
    if (m->max_chunk <= 1024) return 1024;
    return 0;
}

void spmv(Matrix *m, bool transpose, const double *x, double *y, bool ref_order)
{
    Context *ctx = m->ctx;
    const GridCap small(ctx, m->n);
    if (transpose) matrix_ensure_transpose(m);
    if (m->n == 0) return;
    if (matrix_ensure_sell(m, transpose, false)) {
        const double *sv = transpose ? m->s_valT.as<double>() : m->s_val.as<double>();
        if (ref_order) {
            const int g = ctx->fast_grid((const void *)k_spmv_sell_ref, 0);
            k_spmv_sell_ref<<<g, kBlock, 0, ctx->stream>>>(m->n, m->n_slices, m->s_off.as<int32_t>(),
                                                           m->s_col.as<int32_t>(), sv, m->ro.as<int32_t>(), x, y);
        } else {
            const int cols = m->n_codes > 0 ? 1 : m->has_d16 ? 2 : 0;
            auto kern = cols == 1 ? k_spmv_sell<1> : cols == 2 ? k_spmv_sell<2> : k_spmv_sell<0>;
            const int g = ctx->fast_grid((const void *)kern, 0);
            kern<<<g, kBlock, 0, ctx->stream>>>(m->n, m->n_slices, m->s_off.as<int32_t>(), m->s_col.as<int32_t>(),
                                                cols == 1 ? m->s_code.as<uint8_t>() : nullptr,
                                                cols == 1 ? m->s_dtab.as<int32_t>() : nullptr,
                                                cols == 2 ? m->s_d16.as<int16_t>() : nullptr, sv,
                                                m->ro.as<int32_t>(), m->has_long ? 1 : 0, x, y);
        }
        CF_CHECK_LAUNCH();
        return;
    }
    const int cap = stage_cap_for(m);
    const size_t smem = cap > 0 ? kWarps * stage_bytes_per_warp<double>(cap) : 0;
    auto kern = ref_order ? k_spmv : k_spmv_fast;
    if (smem > 48 * 1024)
        CF_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int g = ctx->fast_grid((const void *)kern, smem);
    kern<<<g, kBlock, smem, ctx->stream>>>(m->n, cap, m->ro.as<int32_t>(), m->col.as<int32_t>(),
                                           transpose ? m->valT.as<double>() : m->val.as<double>(), x, y);
    CF_CHECK_LAUNCH();
}

} // namespace cf
