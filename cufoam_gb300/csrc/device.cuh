// device.cuh -- device building blocks shared by the solver kernels:
//   * the reference's reduction tree (gis/SparseSystem/kernels.h:153-199)
//     and a single-pass "last block finishes" grid reduction,
//   * warp-staged CSR row products with the reference's 8-lane summation
//     order (gis/SparseSystem/kernels.h:206-237).
#pragma once

#include "internal.h"

namespace cf {

constexpr unsigned kFull = 0xffffffffu;

// Iterate this thread's rows in the reference's grid-stride order: thread
// s = block*256 + tid handles rows s, s + G*256, ...  All lanes of a warp
// iterate together (chunk base is warp-uniform), which the staging needs.
#define CF_FOR_CHUNKS(base, n)                                                   \
    for (int base = blockIdx.x * kBlock + (threadIdx.x & ~31); base < (n);      \
         base += gridDim.x * kBlock)

// Grid-stride over single elements with the same thread->index mapping.
#define CF_FOR_ELEMS(i, n)                                                        \
    for (int i = blockIdx.x * kBlock + threadIdx.x; i < (n); i += gridDim.x * kBlock)

template <class T> __device__ __forceinline__ T ld_cg(const T *p) { return __ldcg(p); }

// Programmatic dependent launch: a kernel launched with programmatic stream
// serialisation may start while its predecessor drains; pdl_wait() blocks
// until the predecessor grid has completed and its memory is visible (a
// no-op for ordinary launches).  pdl_trigger() lets the successor launch.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// Block tree over NV per-thread values in the reference's order: strides
// 128 and 64 through shared memory, then 32..1 inside warp 0 (the shuffle
// tree adds lane i+s into lane i exactly like the warp-synchronous steps).
// Result valid in thread 0.
template <int NV, class T>
__device__ __forceinline__ void block_tree(T (&v)[NV], T *sm)
{
    const int tid = threadIdx.x;
#pragma unroll
    for (int i = 0; i < NV; ++i) sm[i * kBlock + tid] = v[i];
    __syncthreads();
    if (tid < 128) {
#pragma unroll
        for (int i = 0; i < NV; ++i) sm[i * kBlock + tid] = sm[i * kBlock + tid] + sm[i * kBlock + tid + 128];
    }
    __syncthreads();
    if (tid < 64) {
#pragma unroll
        for (int i = 0; i < NV; ++i) sm[i * kBlock + tid] = sm[i * kBlock + tid] + sm[i * kBlock + tid + 64];
    }
    __syncthreads();
    if (tid < 32) {
#pragma unroll
        for (int i = 0; i < NV; ++i) {
            T x = sm[i * kBlock + tid] + sm[i * kBlock + tid + 32];
            x = x + __shfl_down_sync(kFull, x, 16);
            x = x + __shfl_down_sync(kFull, x, 8);
            x = x + __shfl_down_sync(kFull, x, 4);
            x = x + __shfl_down_sync(kFull, x, 2);
            x = x + __shfl_down_sync(kFull, x, 1);
            v[i] = x;
        }
    }
}

// The fast reduction order's block stage: the shuffle tree below
// (CF_FAST_BLOCK_SUM 1) or the reference's tree (0).
#ifndef CF_FAST_BLOCK_SUM
#define CF_FAST_BLOCK_SUM 1
#endif

// Fast-order block sum (result valid in thread 0): the 256 values through
// shared memory, lane l of warp 0 adds values l, l + 32, ..., l + 224 in a
// three-level tree, then a shuffle tree over the 32 lane sums.  A warp-wide
// FP64 instruction occupies a GB300 sub-partition's FP64 unit for the same
// time whatever its active lanes (measured: 19.6 G warp instructions/s with
// 32 or with 1 active lane), so the block spends 12 FP64 instructions per
// value here against 43 for a shuffle tree in every warp.
template <int NV, class T>
__device__ __forceinline__ void block_sum_fast(T (&v)[NV], T *sm)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < NV; ++i) sm[i * kBlock + threadIdx.x] = v[i];
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int i = 0; i < NV; ++i) {
            const T *s = sm + i * kBlock + lane;
            const T a = (s[0] + s[32]) + (s[64] + s[96]);
            const T b = (s[128] + s[160]) + (s[192] + s[224]);
            T x = a + b;
#pragma unroll
            for (int o = 16; o; o >>= 1) x = x + __shfl_xor_sync(kFull, x, o);
            v[i] = x;
        }
    }
}

// Single-pass grid reduction.  Every block publishes its NV partials; the
// block that arrives last sums them in a fixed order (sequentially in block
// order for the reference order, else a strided sum + block tree), so the
// result is deterministic.  Returns true in the last block, where `out`
// holds the totals (in thread 0).  The arrival counter is reset for the
// next launch.  No block ever waits for another.
template <int NV, class T>
__device__ __forceinline__ bool grid_reduce(T (&acc)[NV], T *partials, int stride,
                                            uint32_t *counter, bool ref_order, T (&out)[NV])
{
    __shared__ T sm[NV * kBlock];
    __shared__ bool s_last;
    pdl_trigger();
#if CF_FAST_BLOCK_SUM
    if (!ref_order) block_sum_fast<NV, T>(acc, sm);
    else
#endif
        block_tree<NV, T>(acc, sm);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int i = 0; i < NV; ++i) partials[i * stride + blockIdx.x] = acc[i];
        __threadfence();
        const uint32_t ticket = atomicAdd(counter, 1u);
        s_last = (ticket == gridDim.x - 1);
    }
    __syncthreads();
    if (!s_last) return false;
    __threadfence();
    const int G = gridDim.x;
    if (ref_order) {
        // the partials in block order, one sequential sum per value; the
        // whole block stages them through shared memory a chunk at a time
        // so that thread 0 adds from shared memory instead of waiting on
        // one L2 load per partial
        T run[NV];
#pragma unroll
        for (int i = 0; i < NV; ++i) run[i] = T(0);
        for (int b0 = 0; b0 < G; b0 += kBlock) {
            const int m = min(kBlock, G - b0);
            __syncthreads(); // the previous chunk (or the block sum) is consumed
            if (threadIdx.x < m)
#pragma unroll
                for (int i = 0; i < NV; ++i) sm[i * kBlock + threadIdx.x] = ld_cg(partials + i * stride + b0 + threadIdx.x);
            __syncthreads();
            if (threadIdx.x == 0) {
                if (m == kBlock) {
                    // a full chunk: a fixed trip count lets the shared
                    // loads run ahead of the dependent additions
#pragma unroll 32
                    for (int b = 0; b < kBlock; ++b)
#pragma unroll
                        for (int i = 0; i < NV; ++i) run[i] += sm[i * kBlock + b];
                } else {
                    for (int b = 0; b < m; ++b)
#pragma unroll
                        for (int i = 0; i < NV; ++i) run[i] += sm[i * kBlock + b];
                }
            }
        }
        if (threadIdx.x == 0)
#pragma unroll
            for (int i = 0; i < NV; ++i) out[i] = run[i];
    } else {
        // thread t adds partials t, t + 256, ... in that order; for grids of
        // up to 5 * 256 blocks (the fast grid is at most 8 blocks per SM,
        // 1,216 on 152 SMs) all its loads are issued before the first
        // addition: one L2 round trip instead of one per partial
        constexpr int kPer = 5;
        T v[NV];
#pragma unroll
        for (int i = 0; i < NV; ++i) {
            T s = T(0);
            if (G <= kPer * kBlock) {
                T t[kPer];
#pragma unroll
                for (int u = 0; u < kPer; ++u) {
                    const int b = threadIdx.x + u * kBlock;
                    t[u] = b < G ? ld_cg(partials + i * stride + b) : T(0);
                }
#pragma unroll
                for (int u = 0; u < kPer; ++u)
                    if (threadIdx.x + u * kBlock < G) s += t[u];
            } else {
                for (int b = threadIdx.x; b < G; b += kBlock) s += ld_cg(partials + i * stride + b);
            }
            v[i] = s;
        }
        __syncthreads();
#if CF_FAST_BLOCK_SUM
        block_sum_fast<NV, T>(v, sm);
#else
        block_tree<NV, T>(v, sm);
#endif
        if (threadIdx.x == 0) {
#pragma unroll
            for (int i = 0; i < NV; ++i) out[i] = v[i];
        }
    }
    if (threadIdx.x == 0) *counter = 0u;
    return true;
}

// ---------------------------------------------------------------------------
// CSR row products
// ---------------------------------------------------------------------------
// Per-warp staging area in dynamic shared memory: values, then columns.
template <class V>
__host__ __device__ __forceinline__ size_t stage_bytes_per_warp(int cap)
{
    return (size_t)(cap + 8) * sizeof(V) + (size_t)(cap + 8) * sizeof(int32_t);
}

// Rows longer than this are summed by the whole warp (fast order): lane j
// takes the row's entries j, j + 32, ... as one FMA chain, then a fixed
// xor-shuffle tree adds the 32 lane sums.  One lane per row stays the rule
// below it: every warp-wide FP64 instruction costs a GB300 sub-partition
// the same whatever its active lanes, so splitting short rows over lanes
// would multiply the FP64 instructions per row, while a long row summed by
// one lane serialises the warp (a 3,000-entry row: 3,000 dependent FMAs).
constexpr int kLongRow = 32;

template <class V>
struct Chunk {
    int rs, re;        // this lane's row [rs, re)
    int ov, oc;        // staging origins (element index of slot 0); -1 = not staged
    unsigned lng;      // lanes whose row is longer than kLongRow
    const V *sv;
    const int32_t *sc;
};

// Load the CSR entries of rows [base, base+32) into this warp's staging area
// with 16-byte vector loads (fully coalesced), or leave them in global
// memory when the chunk does not fit.  The arrays must be readable 16 bytes
// past nnz (the matrix allocations are padded).
template <class V>
__device__ __forceinline__ Chunk<V> stage_chunk(const int32_t *__restrict__ ro,
                                                const int32_t *__restrict__ col,
                                                const V *__restrict__ val, int n, int base,
                                                int cap, V *sv, int32_t *sc)
{
    const int lane = threadIdx.x & 31;
    const int row = base + lane;
    Chunk<V> c;
    c.rs = __ldg(ro + (row < n ? row : n));
    int nxt = __shfl_down_sync(kFull, c.rs, 1);
    const int last = __ldg(ro + (base + 32 < n ? base + 32 : n));
    c.re = (lane == 31) ? last : nxt;
    const int eb = __shfl_sync(kFull, c.rs, 0);
    const int ee = last;
    c.sv = sv;
    c.sc = sc;
    c.lng = __ballot_sync(kFull, c.re - c.rs > kLongRow);
    if (c.lng || cap <= 0 || ee - eb > cap) {
        c.ov = -1;
        c.oc = -1;
        return c;
    }
    constexpr int VPER = 16 / sizeof(V);
    const int av = eb & ~(VPER - 1);
    for (int i = av + lane * VPER; i < ee; i += 32 * VPER) {
        if (sizeof(V) == 8) {
            const double2 t = __ldg(reinterpret_cast<const double2 *>(val + i));
            double *d = reinterpret_cast<double *>(sv) + (i - av);
            d[0] = t.x;
            d[1] = t.y;
        } else {
            const float4 t = __ldg(reinterpret_cast<const float4 *>(val + i));
            float *d = reinterpret_cast<float *>(sv) + (i - av);
            d[0] = t.x;
            d[1] = t.y;
            d[2] = t.z;
            d[3] = t.w;
        }
    }
    const int ac = eb & ~3;
    for (int i = ac + lane * 4; i < ee; i += 128) {
        const int4 t = __ldg(reinterpret_cast<const int4 *>(col + i));
        int32_t *d = sc + (i - ac);
        d[0] = t.x;
        d[1] = t.y;
        d[2] = t.z;
        d[3] = t.w;
    }
    __syncwarp();
    c.ov = av;
    c.oc = ac;
    return c;
}

__device__ __forceinline__ double fma_t(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float fma_t(float a, float b, float c) { return __fmaf_rn(a, b, c); }

__device__ __forceinline__ double add_t(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float add_t(float a, float b) { return __fadd_rn(a, b); }

// ((t0+t4)+(t2+t6)) + ((t1+t5)+(t3+t7)): the reference's 8-lane tree
template <class V>
__device__ __forceinline__ V tree8(const V (&t)[8])
{
    return add_t(add_t(add_t(t[0], t[4]), add_t(t[2], t[6])), add_t(add_t(t[1], t[5]), add_t(t[3], t[7])));
}

// sum_j a_ij * g(j) for this lane's row in the reference's order: lane l of
// 8 accumulates entries rs+l, rs+l+8, ... with FMA, then
// ((t0+t4)+(t2+t6)) + ((t1+t5)+(t3+t7)).
template <class V, class G>
__device__ __forceinline__ V row_product(const Chunk<V> &c, const int32_t *__restrict__ col,
                                         const V *__restrict__ val, G g)
{
    V t[8];
    if (c.ov >= 0) {
#pragma unroll
        for (int l = 0; l < 8; ++l) {
            V acc = V(0);
            for (int j = c.rs + l; j < c.re; j += 8) acc = fma_t(c.sv[j - c.ov], g(c.sc[j - c.oc]), acc);
            t[l] = acc;
        }
    } else {
#pragma unroll
        for (int l = 0; l < 8; ++l) {
            V acc = V(0);
            for (int j = c.rs + l; j < c.re; j += 8) acc = fma_t(__ldg(val + j), g(__ldg(col + j)), acc);
            t[l] = acc;
        }
    }
    return tree8(t);
}

// The same sum for one row of a SELL-32 copy, where slot t of the row holds
// its t-th CSR entry: lane l of 8 takes slots l, l + 8, ... below the row's
// CSR length rl (len = the slice's slots per row; cp, vp point at this
// lane's column and value of slot 0, slots 32 elements apart).
template <class G>
__device__ __forceinline__ double sell_ref_row(const int32_t *__restrict__ cp, const double *__restrict__ vp,
                                               int len, int rl, G g)
{
    double t[8];
#pragma unroll
    for (int l = 0; l < 8; ++l) t[l] = 0.0;
    for (int t0 = 0; t0 < len; t0 += 8) {
#pragma unroll
        for (int l = 0; l < 8; ++l) {
            const int slot = t0 + l;
            if (slot < rl) t[l] = fma_t(__ldg(vp + 32 * slot), g(__ldg(cp + 32 * slot)), t[l]);
        }
    }
    return tree8(t);
}

// Two products over the same pattern (A and A^T values share row_offsets
// and column indices for LDU matrices): the column index is read once.
template <class V, class G1, class G2>
__device__ __forceinline__ void row_product2(const Chunk<V> &c, const int32_t *__restrict__ col,
                                             const V *__restrict__ val1, const V *__restrict__ val2,
                                             G1 g1, G2 g2, V &y1, V &y2)
{
    V t[8], u[8];
#pragma unroll
    for (int l = 0; l < 8; ++l) {
        V a1 = V(0), a2 = V(0);
        for (int j = c.rs + l; j < c.re; j += 8) {
            const int cc = (c.oc >= 0) ? c.sc[j - c.oc] : __ldg(col + j);
            const V v1 = (c.ov >= 0) ? c.sv[j - c.ov] : __ldg(val1 + j);
            a1 = fma_t(v1, g1(cc), a1);
            a2 = fma_t(__ldg(val2 + j), g2(cc), a2);
        }
        t[l] = a1;
        u[l] = a2;
    }
    y1 = tree8(t);
    y2 = tree8(u);
}

// The fixed xor-shuffle tree of a long row's 32 lane sums: every lane ends
// with the same bits (a + b == b + a in IEEE arithmetic).
template <class V>
__device__ __forceinline__ V warp_sum(V v)
{
#pragma unroll
    for (int o = 16; o; o >>= 1) v = add_t(v, __shfl_xor_sync(kFull, v, o));
    return v;
}

// One long row summed by the whole warp: entries at cp[stride * t],
// vp[stride * t] for t < len (CSR: stride 1; SELL slots: stride 32), lane j
// taking t = j, j + 32, ...
template <class V, class G>
__device__ __forceinline__ V warp_row(const int32_t *cp, const V *vp, int len, int stride, G g)
{
    V acc = V(0);
    for (int t = threadIdx.x & 31; t < len; t += 32)
        acc = fma_t(vp[(size_t)stride * t], g(cp[(size_t)stride * t]), acc);
    return warp_sum(acc);
}

// sum_j a_ij * g(j) as one FMA chain in entry order: one FP64 instruction
// per entry, the least work per row (the fast reduction order); rows longer
// than kLongRow summed by the whole warp (warp_row).
template <class V, class G>
__device__ __forceinline__ V row_chain(const Chunk<V> &c, const int32_t *__restrict__ col,
                                       const V *__restrict__ val, G g)
{
    V acc = V(0);
    if (c.ov >= 0) {
        for (int j = c.rs; j < c.re; ++j) acc = fma_t(c.sv[j - c.ov], g(c.sc[j - c.oc]), acc);
    } else {
        const int lane = threadIdx.x & 31;
        if (!((c.lng >> lane) & 1u))
            for (int j = c.rs; j < c.re; ++j) acc = fma_t(__ldg(val + j), g(__ldg(col + j)), acc);
        for (unsigned m = c.lng; m; m &= m - 1) {
            const int r = __ffs(m) - 1;
            const int rs = __shfl_sync(kFull, c.rs, r), re = __shfl_sync(kFull, c.re, r);
            const V s = warp_row(col + rs, val + rs, re - rs, 1, g);
            if (lane == r) acc = s;
        }
    }
    return acc;
}

// Two FMA chains over the same pattern (A and A^T values).
template <class V, class G1, class G2>
__device__ __forceinline__ void row_chain2(const Chunk<V> &c, const int32_t *__restrict__ col,
                                           const V *__restrict__ val1, const V *__restrict__ val2,
                                           G1 g1, G2 g2, V &y1, V &y2)
{
    V a1 = V(0), a2 = V(0);
    const int lane = threadIdx.x & 31;
    if (!((c.lng >> lane) & 1u)) {
        for (int j = c.rs; j < c.re; ++j) {
            const int cc = (c.oc >= 0) ? c.sc[j - c.oc] : __ldg(col + j);
            const V v1 = (c.ov >= 0) ? c.sv[j - c.ov] : __ldg(val1 + j);
            a1 = fma_t(v1, g1(cc), a1);
            a2 = fma_t(__ldg(val2 + j), g2(cc), a2);
        }
    }
    for (unsigned m = c.lng; m; m &= m - 1) {
        const int r = __ffs(m) - 1;
        const int rs = __shfl_sync(kFull, c.rs, r), re = __shfl_sync(kFull, c.re, r);
        const V s1 = warp_row(col + rs, val1 + rs, re - rs, 1, g1);
        const V s2 = warp_row(col + rs, val2 + rs, re - rs, 1, g2);
        if (lane == r) {
            a1 = s1;
            a2 = s2;
        }
    }
    y1 = a1;
    y2 = a2;
}

// Finish a device-driven loop iteration: set the graph's while condition.
__device__ __forceinline__ void set_loop_condition(const SolveArgs *a, bool cont)
{
    if (a->use_cond) cudaGraphSetConditional(a->cond, cont ? 1u : 0u);
}

// ---------------------------------------------------------------------------
// SELL-32: the matrix cut into slices of 32 consecutive rows; each slice is
// padded to its longest row and stored entry-major (entry t of the slice's
// 32 rows is 32 consecutive elements at off[s] + 32 t).  Lane l of a warp
// owns row 32 s + l and reads its entries with fully coalesced 128-byte
// (index) and 256-byte (value) loads, with no staging.  Padding entries hold
// value 0 and a valid column and add +-0 to the FMA chain, so rows sum in the
// same entry order, to the same value, as row_chain.
// ---------------------------------------------------------------------------

// L2 policy for arrays read once per pass: evict first, so that the Krylov
// vectors (re-read by the next kernels) stay resident in L2 while the matrix
// streams through.
__device__ __forceinline__ uint64_t l2_evict_first_policy()
{
    uint64_t p;
    asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
    return p;
}

__device__ __forceinline__ double ld_stream(const double *p, uint64_t pol)
{
    double v;
    asm("ld.global.nc.L1::no_allocate.L2::cache_hint.f64 %0, [%1], %2;" : "=d"(v) : "l"(p), "l"(pol));
    return v;
}
__device__ __forceinline__ float ld_stream(const float *p, uint64_t pol)
{
    float v;
    asm("ld.global.nc.L1::no_allocate.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(v) : "l"(p), "l"(pol));
    return v;
}
__device__ __forceinline__ int32_t ld_stream(const int32_t *p, uint64_t pol)
{
    int32_t v;
    asm("ld.global.nc.L1::no_allocate.L2::cache_hint.b32 %0, [%1], %2;" : "=r"(v) : "l"(p), "l"(pol));
    return v;
}
// 8 bytes (8-byte aligned) as two words
__device__ __forceinline__ uint2 ld_stream8(const uint8_t *p, uint64_t pol)
{
    uint2 v;
    asm("ld.global.nc.L1::no_allocate.L2::cache_hint.v2.u32 {%0, %1}, [%2], %3;"
        : "=r"(v.x), "=r"(v.y)
        : "l"(p), "l"(pol));
    return v;
}

// Column indices of a SELL-32 copy.  SellCols32 holds the 32-bit column of
// every slot, entry-major like the values (slot t of lane l's row at element
// b + 32 t + l of its slice).  SellCodes8 holds one byte per slot: an index
// into a table of the pattern's distinct offsets col - row (at most
// kMaxCodes; a 7-point stencil has 7, a 27-point one 27), so a slot costs 1
// byte instead of 4: 9 instead of 12 bytes per FP64 entry, 5 instead of 8
// per FP32 entry.  A padding slot holds offset 0 from its row base rb -- the
// row itself, or column 0 for the rows past n of the last slice -- which is
// the column the 32-bit copy stores there, so both give the same gathers
// and the same sums.
//
// The codes of a slice are stored lane-major (lane l's `len` codes at bytes
// b + len l ... of the slice), so a lane fetches up to eight of them with
// two aligned 8-byte loads: a load in flight holds a register until it
// returns, and four registers for eight codes leave room for more loads in
// flight than one register per one-byte load.  Lane l keeps table entry l
// in a register and decodes by a warp shuffle (col(), called by all 32
// lanes together).  Measured on GB300 against an L1-cached table load and a
// select tree over eight registers (7-point systems, byte loads): plain FP64
// SpMV at 128^3 33.2 us (table 37.2, select tree 36.4, 32-bit columns 35.7),
// FP32 MR step at 256^3 214 us (224, 228; 237).  A row longer than 32
// entries has more than 32 offsets, so matrices with long rows keep 32-bit
// columns; col_div() (any lanes) reads the table from memory.
constexpr int kMaxCodes = 32;

struct SellCols32 {
    const int32_t *p;
    // the columns of slots t0 .. t0 + M - 1 of this lane's row (slice at b)
    template <int M> struct Batch {
        int32_t c[M];
        __device__ __forceinline__ int32_t raw(int u) const { return c[u]; }
    };
    template <int M>
    __device__ __forceinline__ Batch<M> load_batch(int64_t b, int lane, int, int t0, uint64_t pol) const
    {
        Batch<M> r;
#pragma unroll
        for (int u = 0; u < M; ++u) r.c[u] = ld_stream(p + b + lane + 32 * (t0 + u), pol);
        return r;
    }
    // the same for the slots below len only (a batch may run past the row)
    template <int M>
    __device__ __forceinline__ Batch<M> load_guarded(int64_t b, int lane, int len, int t0, uint64_t pol) const
    {
        Batch<M> r;
#pragma unroll
        for (int u = 0; u < M; ++u)
            if (t0 + u < len) r.c[u] = ld_stream(p + b + lane + 32 * (t0 + u), pol);
        return r;
    }
    // slot t of row r of the slice (len slots)
    __device__ __forceinline__ int32_t plain_slot(int64_t b, int, int r, int t) const
    {
        return p[b + r + (int64_t)32 * t];
    }
    __device__ __forceinline__ int col(int32_t raw, int) const { return raw; }
    __device__ __forceinline__ int col_div(int32_t raw, int) const { return raw; }
    __device__ __forceinline__ const void *addr(int64_t o) const { return p + o; }
};
struct SellCodes8 {
    const uint8_t *p;
    const int32_t *tab;  // offsets col - row (kMaxCodes entries, unused ones 0)
    int treg;            // tab[lane]
    __device__ __forceinline__ SellCodes8(const uint8_t *p_, const int32_t *tab_)
        : p(p_), tab(tab_), treg(__ldg(tab_ + (threadIdx.x & 31)))
    {
    }
    // codes t0 .. t0 + M - 1 (M <= 8) of this lane, packed four to a word
    template <int M> struct Batch {
        uint32_t lo, hi;
        __device__ __forceinline__ uint32_t raw(int u) const { return ((u < 4 ? lo : hi) >> (8 * (u & 3))) & 0xffu; }
    };
    // bytes b + len lane + t0 ... inside the 16 bytes from the 8-byte
    // boundary below them (the array is padded, so the window may run past
    // the slice)
    template <int M>
    __device__ __forceinline__ Batch<M> load_batch(int64_t b, int lane, int len, int t0, uint64_t pol) const
    {
        static_assert(M <= 8, "at most eight codes per batch");
        const int64_t a = b + (int64_t)len * lane + t0;
        const int64_t a0 = a & ~(int64_t)7;
        const uint2 w01 = ld_stream8(p + a0, pol);
        const uint2 w23 = ld_stream8(p + a0 + 8, pol);
        const unsigned k = (unsigned)(a - a0);
        const bool up = k >= 4;
        const unsigned sh = 8u * (k & 3u);
        const uint32_t x0 = up ? w01.y : w01.x, x1 = up ? w23.x : w01.y, x2 = up ? w23.y : w23.x;
        Batch<M> r;
        r.lo = __funnelshift_r(x0, x1, sh);   // codes t0 .. t0 + 3
        r.hi = __funnelshift_r(x1, x2, sh);   // codes t0 + 4 .. t0 + 7
        return r;
    }
    // (the 16-byte window stays inside the padded array for any t0 < len)
    template <int M>
    __device__ __forceinline__ Batch<M> load_guarded(int64_t b, int lane, int len, int t0, uint64_t pol) const
    {
        return load_batch<M>(b, lane, len, t0, pol);
    }
    __device__ __forceinline__ uint32_t plain_slot(int64_t b, int len, int r, int t) const
    {
        return p[b + (int64_t)len * r + t];
    }
    __device__ __forceinline__ int col(uint32_t raw, int rb) const { return rb + __shfl_sync(kFull, treg, (int)raw); }
    __device__ __forceinline__ int col_div(uint32_t raw, int rb) const { return rb + __ldg(tab + raw); }
    __device__ __forceinline__ const void *addr(int64_t o) const { return p + o; }
};

// 16-bit column deltas: a slot's column is its row base plus a signed
// 16-bit delta (patterns whose offsets col - row all lie in [-32768, 32767]
// but number more than kMaxCodes: unstructured meshes in a bandwidth-reducing
// order).  Stored lane-major like the codes (lane l's len deltas at element
// b + len l of the slice); a batch of up to eight comes from three aligned
// 8-byte loads.  2 bytes per slot: 10 instead of 12 per FP64 entry, 6
// instead of 8 per FP32 entry.
struct SellDelta16 {
    const int16_t *p;
    template <int M> struct Batch {
        uint32_t z[4];   // deltas t0 .. t0 + 7, two to a word
        __device__ __forceinline__ int raw(int u) const { return (int)(int16_t)(z[u >> 1] >> (16 * (u & 1))); }
    };
    template <int M>
    __device__ __forceinline__ Batch<M> load_batch(int64_t b, int lane, int len, int t0, uint64_t pol) const
    {
        static_assert(M <= 8, "at most eight deltas per batch");
        const int64_t a = b + (int64_t)len * lane + t0;   // in deltas
        const int64_t a0 = a & ~(int64_t)3;               // 8-byte boundary
        const uint8_t *q = reinterpret_cast<const uint8_t *>(p + a0);
        const uint2 w01 = ld_stream8(q, pol);
        const uint2 w23 = ld_stream8(q + 8, pol);
        const uint2 w45 = ld_stream8(q + 16, pol);
        const unsigned k = (unsigned)(a - a0);            // 0..3 deltas into the window
        const bool skip = k >= 2, half = k & 1u;
        const uint32_t y0 = skip ? w01.y : w01.x, y1 = skip ? w23.x : w01.y, y2 = skip ? w23.y : w23.x;
        const uint32_t y3 = skip ? w45.x : w23.y, y4 = skip ? w45.y : w45.x;
        const unsigned sh = half ? 16u : 0u;
        Batch<M> r;
        r.z[0] = __funnelshift_r(y0, y1, sh);
        r.z[1] = __funnelshift_r(y1, y2, sh);
        r.z[2] = __funnelshift_r(y2, y3, sh);
        r.z[3] = __funnelshift_r(y3, y4, sh);
        return r;
    }
    // (the 24-byte window stays inside the padded array for any t0 < len)
    template <int M>
    __device__ __forceinline__ Batch<M> load_guarded(int64_t b, int lane, int len, int t0, uint64_t pol) const
    {
        return load_batch<M>(b, lane, len, t0, pol);
    }
    __device__ __forceinline__ int plain_slot(int64_t b, int len, int r, int t) const
    {
        return p[b + (int64_t)len * r + t];
    }
    __device__ __forceinline__ int col(int raw, int rb) const { return rb + raw; }
    __device__ __forceinline__ int col_div(int raw, int rb) const { return rb + raw; }
    __device__ __forceinline__ const void *addr(int64_t o) const { return p + o; }
};

// the row base a slot's code is relative to: the row, or 0 past n
__device__ __forceinline__ int sell_row_base(int row, int n) { return row < n ? row : 0; }

__device__ __forceinline__ void prefetch_l2(const void *p)
{
    asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

// L2 prefetch of the first (up to 8) entries of this warp's first slice:
// constant matrix data a loop-body kernel may request before it waits for
// its predecessor (programmatic launches start early), so that its first
// loads after the wait hit L2.  Only for matrices with more slices than
// the grid has warps: the slice offset it must load first would otherwise
// lengthen the short steps of a small system (64^2 Jacobi: 8.0 -> 8.4 us).
template <class C, class V>
__device__ __forceinline__ void sell_prefetch_first(int n_slices, const int32_t *__restrict__ off, const C &cs,
                                                    const V *__restrict__ val)
{
    const int s = blockIdx.x * kWarps + (threadIdx.x >> 5);
    if (n_slices <= (int)gridDim.x * kWarps) return;
    const int lane = threadIdx.x & 31;
    const int b = __ldg(off + s);
    const int len = (__ldg(off + s + 1) - b) >> 5;
    const int m = len < 8 ? len : 8;
    for (int u = 0; u < m; ++u) {
        prefetch_l2(cs.addr(b + lane + 32 * u));
        prefetch_l2(val + b + lane + 32 * u);
    }
}

// Slots t0 .. t0 + M - 1 of this lane's row (slice at element b, len slots;
// values 32 elements apart from vp = val + b + lane + 32 t0): all loads and
// gathers issued before the first FMA, then one FMA chain in slot order.
template <class V, int M, class C, class G>
__device__ __forceinline__ void sell_batch(const C &cs, int64_t b, int lane, int len, int t0, int rb, const V *vp,
                                           uint64_t pol, G g, V &acc)
{
    V v[M], x[M];
    const auto c = cs.template load_batch<M>(b, lane, len, t0, pol);
#pragma unroll
    for (int u = 0; u < M; ++u) v[u] = ld_stream(vp + 32 * u, pol);
#pragma unroll
    for (int u = 0; u < M; ++u) x[u] = g(cs.col(c.raw(u), rb));
#pragma unroll
    for (int u = 0; u < M; ++u) acc = fma_t(v[u], x[u], acc);
}

// the last r < B entries of a row as one exact batch
template <class V, int B, class C, class G>
__device__ __forceinline__ void sell_tail(int r, const C &cs, int64_t b, int lane, int len, int t0, int rb,
                                          const V *vp, uint64_t pol, G g, V &acc)
{
    if constexpr (B > 1) {
        if (r == B - 1) {
            sell_batch<V, B - 1>(cs, b, lane, len, t0, rb, vp, pol, g, acc);
            return;
        }
        sell_tail<V, B - 1>(r, cs, b, lane, len, t0, rb, vp, pol, g, acc);
    }
}

// A slice's rows longer than kLongRow (row lengths from the CSR offsets
// `ro`) summed by the whole warp over their own slots, the bits of the CSR
// passes (warp_row: lane j takes slots j, j + 32, ... as one FMA chain,
// then the xor-shuffle tree); `acc` is this lane's sum, replaced for those
// lanes.  b is the slice's first element, slen its slots per row, vp0 its
// first value.
template <class V, class C, class G>
__device__ __forceinline__ void sell_long_rows(int n, int s, const int32_t *__restrict__ ro, const C &cs,
                                               int64_t b, int slen, const V *vp0, G g, V &acc)
{
    const int lane = threadIdx.x & 31;
    const int row = s * 32 + lane;
    const int rl = row < n ? __ldg(ro + row + 1) - __ldg(ro + row) : 0;
    for (unsigned m = __ballot_sync(kFull, rl > kLongRow); m; m &= m - 1) {
        const int r = __ffs(m) - 1;
        const int len = __shfl_sync(kFull, rl, r);
        const int rb = s * 32 + r;
        V a = V(0);
        for (int t = lane; t < len; t += 32)
            a = fma_t(vp0[r + (int64_t)32 * t], g(cs.col_div(cs.plain_slot(b, slen, r, t), rb)), a);
        const V v = warp_sum(a);
        if (lane == r) acc = v;
    }
}

// f(row, sum_t val[t] g(col[t])) for every row, one warp per slice; the
// entries are taken B at a time (all B loads and gathers issued before the
// first FMA), the row's last r < B entries as an exact batch: a guarded slot
// of a full batch would still issue its FMA (measured: 9 DFMA per 7-entry
// row).  The slice length is warp-uniform, so the branches never diverge.
// Matrices with rows longer than kLongRow (has_long) sum those rows with
// the whole warp (sell_long_rows), as the CSR passes do.  cs: the columns
// (SellCols32 or SellCodes8).
template <class V, int B, class C, class G, class F>
__device__ __forceinline__ void sell_rows(int n, int n_slices, const int32_t *__restrict__ off, const C &cs,
                                          const V *__restrict__ val, const int32_t *__restrict__ ro,
                                          bool has_long, G g, F f)
{
    const uint64_t pol = l2_evict_first_policy();
    const int lane = threadIdx.x & 31;
    const int nw = gridDim.x * kWarps;
    for (int s = blockIdx.x * kWarps + (threadIdx.x >> 5); s < n_slices; s += nw) {
        const int b = __ldg(off + s);
        const int len = (__ldg(off + s + 1) - b) >> 5;
        const int row = s * 32 + lane;
        const int rb = sell_row_base(row, n);
        const V *vp = val + (int64_t)b + lane;
        V acc = V(0);
        int t0 = 0;
        for (; t0 + B <= len; t0 += B) sell_batch<V, B>(cs, b, lane, len, t0, rb, vp + 32 * t0, pol, g, acc);
        sell_tail<V, B>(len - t0, cs, b, lane, len, t0, rb, vp + 32 * t0, pol, g, acc);
        if (has_long) sell_long_rows(n, s, ro, cs, b, len, val + b, g, acc);
        if (row < n) f(row, acc);
    }
}

// Two products over one SELL pattern (A and A^T values): f(row, y1, y2).
template <class V, int B, class C, class G1, class G2, class F>
__device__ __forceinline__ void sell_rows2(int n, int n_slices, const int32_t *__restrict__ off, const C &cs,
                                           const V *__restrict__ val1, const V *__restrict__ val2,
                                           const int32_t *__restrict__ ro, bool has_long, G1 g1, G2 g2, F f)
{
    const uint64_t pol = l2_evict_first_policy();
    const int lane = threadIdx.x & 31;
    const int nw = gridDim.x * kWarps;
    for (int s = blockIdx.x * kWarps + (threadIdx.x >> 5); s < n_slices; s += nw) {
        const int b = __ldg(off + s);
        const int len = (__ldg(off + s + 1) - b) >> 5;
        const int row = s * 32 + lane;
        const int rb = sell_row_base(row, n);
        const int64_t o = (int64_t)b + lane;
        const V *vp1 = val1 + o;
        const V *vp2 = val2 + o;
        V a1 = V(0), a2 = V(0);
        for (int t0 = 0; t0 < len; t0 += B) {
            V v1[B], v2[B], x1[B], x2[B];
            const auto c = cs.template load_guarded<B>(b, lane, len, t0, pol);
#pragma unroll
            for (int u = 0; u < B; ++u)
                if (t0 + u < len) {
                    v1[u] = ld_stream(vp1 + 32 * (t0 + u), pol);
                    v2[u] = ld_stream(vp2 + 32 * (t0 + u), pol);
                }
#pragma unroll
            for (int u = 0; u < B; ++u)
                if (t0 + u < len) {
                    const int cc = cs.col(c.raw(u), rb);
                    x1[u] = g1(cc);
                    x2[u] = g2(cc);
                }
#pragma unroll
            for (int u = 0; u < B; ++u)
                if (t0 + u < len) {
                    a1 = fma_t(v1[u], x1[u], a1);
                    a2 = fma_t(v2[u], x2[u], a2);
                }
        }
        if (has_long) {
            sell_long_rows(n, s, ro, cs, b, len, val1 + b, g1, a1);
            sell_long_rows(n, s, ro, cs, b, len, val2 + b, g2, a2);
        }
        if (row < n) f(row, a1, a2);
    }
}

} // namespace cf
