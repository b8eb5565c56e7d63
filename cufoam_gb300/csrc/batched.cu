// batched.cu -- many independent LDU systems, each with R right-hand sides
// (the Ux/Uy/Uz components that share one matrix), solved by CG in ONE
// persistent kernel launch (captured in a CUDA graph).
//
// Schedule: the grid is one wave of thread-block clusters of CS CTAs.  A
// cluster takes the next system from a global work queue (systems ordered
// largest first), splits its 32-row slices over its CTAs, and runs the whole
// solve for all R right-hand sides at once: every matrix entry is read once
// per iteration for R vectors (R-wide SpMM, from the system's SELL-32 copy:
// one warp per slice, coalesced entry loads streamed with an L2 evict-first
// hint), vectors are stored row-major with the R components adjacent.  A
// thread owns the same rows in every phase.  One CG step is three passes:
//   P  x += alpha_{k-1} p (the previous step, deferred), p = r + beta p
//   A  q = A p, (p, q)          (gathers p only)
//   B  r -= alpha q, (r, r)
// with a cluster barrier after P and a cluster reduction after A and B.
// Dot products are reduced inside each CTA and then across the cluster
// through distributed shared memory, after a hardware cluster barrier;
// every CTA sums the per-CTA partials in rank order, so all CTAs reach
// bit-identical scalars and take identical control flow.  Each right-hand
// side keeps its own CG scalars and stopping test (the reference's loop,
// SolverSingleGPU.h:366-445, with its normFactor, gis/gis.cu:106-123); a
// converged component is frozen after its last step reaches x.
//
// Mixed precision (k_batch_cg<R, BT, true>): after the FP64 normFactor and
// residual, each refinement sweep solves A e = r / ||r|| by CG with FP32
// values, FP32 vectors and FP32 per-thread sums (combined across threads
// and CTAs in FP64) to a relative inner tolerance, then adds ||r|| e to x
// and forms the FP64 residual b - A x again; the FP64 tolerance decides
// convergence.
//
// The same kernel with one system and one component is the single-launch
// CG of small systems (solve_cg_single_cluster, at the end of this file).
#include <cooperative_groups.h>

#include "device.cuh"

#include <algorithm>
#include <climits>
#include <cmath>
#include <numeric>

namespace cgp = cooperative_groups;

namespace cf {

constexpr int kBatchMaxR = 4;
// SELL entries loaded (and their R gathers issued) before the first FMA
#ifndef CF_BATCH_ENTRY_BATCH
#define CF_BATCH_ENTRY_BATCH 1
#endif
constexpr int kBatchEntryBatch = CF_BATCH_ENTRY_BATCH;
// the same for the FP32 inner sweeps (single-width values and gathers leave
// the registers for a deeper batch)
#ifndef CF_BATCH_ENTRY_BATCH32
#define CF_BATCH_ENTRY_BATCH32 4
#endif
constexpr int kBatchEntryBatch32 = CF_BATCH_ENTRY_BATCH32;
// 1: matrix entries loaded with an L2 evict-first hint (they are re-read
// only in the next step), 0: plain read-only loads
#ifndef CF_BATCH_STREAM_HINT
#define CF_BATCH_STREAM_HINT 1
#endif
// resident threads per SM the register budget is sized for
#ifndef CF_BATCH_THREADS_PER_SM
#define CF_BATCH_THREADS_PER_SM 1024
#endif

struct BatchSystem {
    int32_t n;
    int32_t sell;            // 1: the SELL-32 copy below, 0: CSR rows
    int64_t vec_offset;      // first row of this system in the batch vectors
    const int32_t *ro;       // CSR
    const int32_t *col;
    const double *val;
    const float *val32;      // FP32 CSR values (mixed precision)
    const int32_t *s_off;    // SELL-32: slice offsets, entry-major columns / values
    const int32_t *s_col;
    const double *s_val;
    const float *s_val32;
};

struct BatchResult {
    double nf, norm0, norm;
    int32_t iters, status;
};

struct BatchArgs {
    const BatchSystem *sys;
    const int32_t *order;    // processing order (largest first)
    int32_t n_systems;
    int32_t max_iter;
    double tolerance;
    const double *b;         // [rows][R]
    double *x;               // [rows][R]
    double *r, *p, *q;       // [rows][R] work
    int32_t *queue;          // next position in `order`
    BatchResult *out;        // [n_systems][R]
    // mixed precision: FP32 inner CG on A32 e = r / ||r||, FP64 refinement
    float *r32, *p32, *q32, *e32;   // [rows][R]
    double inner_rtol;
    int32_t max_outer;
};

struct NoPost {
    __device__ void operator()(int, double) const {}
};

// Sum over the block, then over the cluster: warp sums by shuffle trees,
// the block's warp sums by a shuffle tree in warp 0, then -- after a
// hardware cluster barrier -- the CTAs' sums by a shuffle tree in warp 0
// (lane k reads CTA k's slot through distributed shared memory).  Every CTA
// runs the same trees on the same values, so all reach bit-identical
// totals.  Trees rather than sequential sums: on GB300 every dependent FP64
// addition of a single thread costs its sub-partition's FP64 pipe 64
// cycles, so a tree's log2 levels replace W - 1 and CS - 1 chained adds.
// post(i, total) runs in lane 0 of warp 0 for each value before the final
// block barrier (the scalar step logic that every thread then reads).
template <int NV, int BT, class Post = NoPost>
__device__ __forceinline__ void cluster_sum(cgp::cluster_group &cl, double (&v)[NV],
                                            double *wsm /*[NV][BT/32]*/, double *slot /*[NV]*/,
                                            double *out /*[NV]*/, Post post = Post())
{
    constexpr int W = BT / 32;
    static_assert((W & (W - 1)) == 0 && W <= 32, "warps per block: a power of two");
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < NV; ++i) {
        double s = v[i];
        s += __shfl_down_sync(kFull, s, 16);
        s += __shfl_down_sync(kFull, s, 8);
        s += __shfl_down_sync(kFull, s, 4);
        s += __shfl_down_sync(kFull, s, 2);
        s += __shfl_down_sync(kFull, s, 1);
        if (lane == 0) wsm[i * W + warp] = s;
    }
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int i = 0; i < NV; ++i) {
            double s = lane < W ? wsm[i * W + lane] : 0.0;
#pragma unroll
            for (int o = W / 2; o; o >>= 1) s += __shfl_xor_sync(kFull, s, o);
            if (lane == 0) slot[i] = s;
        }
    }
    cl.sync(); // every CTA's slot is written and visible cluster-wide
    if (warp == 0) {
        const int cs = (int)cl.num_blocks();
#pragma unroll 1
        for (int i = 0; i < NV; ++i) {
            double s = lane < cs ? cl.map_shared_rank(slot, lane)[i] : 0.0;
#pragma unroll
            for (int o = 8; o; o >>= 1) s += __shfl_xor_sync(kFull, s, o);
            if (lane == 0) {
                out[i] = s;
                post(i, s);
            }
        }
    }
    __syncthreads();
}

// Row stride of the gathered search direction p: the R components of a
// cell padded to 4 when R = 3, so that one gather is one 32-byte (FP64) or
// 16-byte (FP32) load.  A random gather costs the L1 one wavefront per
// lane and instruction whatever its width, so fewer, wider gathers are
// what speeds up the SpMM pass.
template <int R> constexpr int pad_r() { return R == 3 ? 4 : R; }

// the R components of padded row c of p (L2 only: other CTAs write p)
template <int R>
__device__ __forceinline__ void ld_row(const double *p, int64_t c, double (&o)[R])
{
    if constexpr (R == 1) {
        o[0] = __ldcg(p + c);
    } else if constexpr (R == 2) {
        const double2 t = __ldcg(reinterpret_cast<const double2 *>(p) + c);
        o[0] = t.x;
        o[1] = t.y;
    } else {
        double t[4];
        asm volatile("ld.global.cg.v4.f64 {%0, %1, %2, %3}, [%4];"
                     : "=d"(t[0]), "=d"(t[1]), "=d"(t[2]), "=d"(t[3])
                     : "l"(p + 4 * c));
#pragma unroll
        for (int j = 0; j < R; ++j) o[j] = t[j];
    }
}
template <int R>
__device__ __forceinline__ void ld_row(const float *p, int64_t c, float (&o)[R])
{
    if constexpr (R == 1) {
        o[0] = __ldcg(p + c);
    } else if constexpr (R == 2) {
        const float2 t = __ldcg(reinterpret_cast<const float2 *>(p) + c);
        o[0] = t.x;
        o[1] = t.y;
    } else {
        const float4 t = __ldcg(reinterpret_cast<const float4 *>(p) + c);
        o[0] = t.x;
        o[1] = t.y;
        o[2] = t.z;
        if constexpr (R == 4) o[3] = t.w;
    }
}
template <int R>
__device__ __forceinline__ void st_row(double *p, int64_t c, const double (&v)[R])
{
    if constexpr (R == 1) {
        p[c] = v[0];
    } else if constexpr (R == 2) {
        reinterpret_cast<double2 *>(p)[c] = make_double2(v[0], v[1]);
    } else {
        asm volatile("st.global.v4.f64 [%0], {%1, %2, %3, %4};" ::"l"(p + 4 * c), "d"(v[0]), "d"(v[1]),
                     "d"(v[2]), "d"(R == 4 ? v[R - 1] : 0.0)
                     : "memory");
    }
}
template <int R>
__device__ __forceinline__ void st_row(float *p, int64_t c, const float (&v)[R])
{
    if constexpr (R == 1) {
        p[c] = v[0];
    } else if constexpr (R == 2) {
        reinterpret_cast<float2 *>(p)[c] = make_float2(v[0], v[1]);
    } else {
        reinterpret_cast<float4 *>(p)[c] = make_float4(v[0], v[1], v[2], R == 4 ? v[R - 1] : 0.f);
    }
}

// The R-wide product of row `row` (this lane's row of 32-row slice s):
// y[j] = sum_e a_e g(col_e)[j] over the components j with on[j], where
// g(c, out) gathers the R components of row c; ys = sum_e a_e.
// SELL-32: the slice's entries, kBatchEntryBatch loaded (streamed, L2
// evict-first) before their gathers; CSR: the row's own range.
template <int R, class V, class T, class G>
__device__ __forceinline__ void row_product(const BatchSystem &S, const V *__restrict__ sval,
                                            const V *__restrict__ cval, int s, int row, const bool (&on)[R],
                                            G g, T (&y)[R], T &ys)
{
#pragma unroll
    for (int j = 0; j < R; ++j) y[j] = T(0);
    ys = T(0);
    if (S.sell) {
        constexpr int B = sizeof(V) == 4 ? kBatchEntryBatch32 : kBatchEntryBatch;
#if CF_BATCH_STREAM_HINT
        const uint64_t pol = l2_evict_first_policy();
#define CF_BATCH_LD(ptr) ld_stream(ptr, pol)
#else
#define CF_BATCH_LD(ptr) __ldg(ptr)
#endif
        const int lane = threadIdx.x & 31;
        const int b = __ldg(S.s_off + s);
        const int len = (__ldg(S.s_off + s + 1) - b) >> 5;
        const int32_t *cp = S.s_col + b + lane;
        const V *vp = sval + b + lane;
        for (int t0 = 0; t0 < len; t0 += B) {
            int c[B];
            V v[B];
            T xv[B][R];
#pragma unroll
            for (int u = 0; u < B; ++u)
                if (t0 + u < len) {
                    c[u] = CF_BATCH_LD(cp + 32 * (t0 + u));
                    v[u] = CF_BATCH_LD(vp + 32 * (t0 + u));
                }
#pragma unroll
            for (int u = 0; u < B; ++u)
                if (t0 + u < len) g(c[u], xv[u]);
#pragma unroll
            for (int u = 0; u < B; ++u)
                if (t0 + u < len) {
#pragma unroll
                    for (int j = 0; j < R; ++j) y[j] = fma_t((T)v[u], on[j] ? xv[u][j] : T(0), y[j]);
                    ys += (T)v[u];
                }
        }
#undef CF_BATCH_LD
    } else if (row < S.n) {
        const int e1 = __ldg(S.ro + row + 1);
        for (int e = __ldg(S.ro + row); e < e1; ++e) {
            const T v = (T)__ldg(cval + e);
            T xv[R];
            g(__ldg(S.col + e), xv);
#pragma unroll
            for (int j = 0; j < R; ++j) y[j] = fma_t(v, on[j] ? xv[j] : T(0), y[j]);
            ys += v;
        }
    }
}

// Per-component CG state, identical in every CTA of the cluster (each CTA
// derives it from the same cluster sums).
template <int R>
struct CompState {
    double rho[R], rho_old[R], nrm[R], tol[R], nf[R];
    double alpha[R];          // step length not yet applied to x (or e)
    double beta[R];           // direction update factor of the next step
    float rho32[R], rho32_old[R], eta[R];
    int act[R], act_in[R], iters[R];
};

// FP64 residual r = b - A x and ||r||^2 per component over this CTA's slices,
// summed over the cluster into tot[0..R)
template <int R, int BT>
__device__ __forceinline__ void batch_residual(cgp::cluster_group &cl, const BatchSystem &S, int s_lo, int s_hi,
                                               const double *b, const double *x, double *r, double *wsm,
                                               double *slot, double *tot)
{
    constexpr int W = BT / 32;
    const int lane = threadIdx.x & 31;
    bool on[R];
#pragma unroll
    for (int j = 0; j < R; ++j) on[j] = true;
    double acc[R];
#pragma unroll
    for (int j = 0; j < R; ++j) acc[j] = 0.0;
    for (int s = s_lo + (threadIdx.x >> 5); s < s_hi; s += W) {
        const int row = s * 32 + lane;
        double y[R], ys;
        row_product<R, double, double>(S, S.s_val, S.val, s, row, on,
                                       [&](int c, double(&o)[R]) {
#pragma unroll
                                                   for (int j = 0; j < R; ++j) o[j] = __ldcg(x + (int64_t)c * R + j);
                                               }, y, ys);
        if (row < S.n)
#pragma unroll
            for (int j = 0; j < R; ++j) {
                const int64_t o = (int64_t)row * R + j;
                const double ri = b[o] - y[j];
                r[o] = ri;
                acc[j] = fma_t(ri, ri, acc[j]);
            }
    }
    cluster_sum<R, BT>(cl, acc, wsm, slot, tot);
}

// Minimum CTAs per SM for the register budget (1,024 threads: 64
// registers).  Measured on the 512-system Poisson batch: occupancy beats
// deeper entry batching (1 entry at 1,024 threads per SM: 2.20 s; 2 at 768:
// 2.66 s; 4 at 512: 2.93 s).
template <int BT> constexpr int batch_min_blocks()
{
    return CF_BATCH_THREADS_PER_SM / BT > 0 ? CF_BATCH_THREADS_PER_SM / BT : 1;
}

template <int R, int BT, bool MIXED>
__global__ void __launch_bounds__(BT, batch_min_blocks<BT>()) k_batch_cg(const BatchArgs a)
{
    cgp::cluster_group cl = cgp::this_cluster();
    const int cs = (int)cl.num_blocks();
    const int rank = (int)cl.block_rank();
    constexpr int W = BT / 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __shared__ double wsm[3 * R * W];
    __shared__ double slot[2][3 * R]; // double-buffered cluster slots
    __shared__ double tot[3 * R];
    __shared__ CompState<R> st;
    // the system being solved; its fields are read where they are used, so
    // that they do not hold registers through the row loops
    __shared__ BatchSystem S;
    __shared__ int32_t s_next;
    int parity = 0;

    for (;;) {
        if (rank == 0 && threadIdx.x == 0) s_next = atomicAdd(a.queue, 1);
        cl.sync();
        const int pos = *cl.map_shared_rank(&s_next, 0);
        cl.sync();
        if (pos >= a.n_systems) break;
        const int sid = a.order[pos];
        if (threadIdx.x == 0) S = a.sys[sid];
        __syncthreads();
        const int n = S.n;
        const int ns = (n + 31) >> 5;
        // this CTA's slices; a thread owns rows s * 32 + lane of the slices
        // s = s_lo + warp + k W in every phase
        const int s_lo = (int)((int64_t)ns * rank / cs), s_hi = (int)((int64_t)ns * (rank + 1) / cs);

        // ---- normFactor part 1: mean of psi per component ----------------
        {
            const double *x = a.x + S.vec_offset * R;
            double acc1[R];
#pragma unroll
            for (int j = 0; j < R; ++j) acc1[j] = 0.0;
            for (int s = s_lo + warp; s < s_hi; s += W) {
                const int row = s * 32 + lane;
                if (row < n)
#pragma unroll
                    for (int j = 0; j < R; ++j) acc1[j] += x[(int64_t)row * R + j];
            }
            cluster_sum<R, BT>(cl, acc1, wsm, slot[parity], tot);
            parity ^= 1;
        }
        // ---- normFactor part 2 + initial residual r = b - A x ------------
        {
            const double *x = a.x + S.vec_offset * R, *b = a.b + S.vec_offset * R;
            double *r = a.r + S.vec_offset * R;
            double xbar[R];
#pragma unroll
            for (int j = 0; j < R; ++j) xbar[j] = tot[j] / n;
            bool on[R];
#pragma unroll
            for (int j = 0; j < R; ++j) on[j] = true;
            double acc3[3 * R];
#pragma unroll
            for (int j = 0; j < 3 * R; ++j) acc3[j] = 0.0;
            for (int s = s_lo + warp; s < s_hi; s += W) {
                const int row = s * 32 + lane;
                double y[R], ys;
                row_product<R, double, double>(S, S.s_val, S.val, s, row, on,
                                               [&](int c, double(&o)[R]) {
#pragma unroll
                                                   for (int j = 0; j < R; ++j) o[j] = __ldcg(x + (int64_t)c * R + j);
                                               },
                                               y, ys);
                if (row < n)
#pragma unroll
                    for (int j = 0; j < R; ++j) {
                        const int64_t o = (int64_t)row * R + j;
                        const double yb = ys * xbar[j];
                        const double bi = b[o];
                        const double d1 = y[j] - yb, d2 = bi - yb, ri = bi - y[j];
                        r[o] = ri;
                        acc3[j] = fma_t(d1, d1, acc3[j]);
                        acc3[R + j] = fma_t(d2, d2, acc3[R + j]);
                        acc3[2 * R + j] = fma_t(ri, ri, acc3[2 * R + j]);
                    }
            }
            cluster_sum<3 * R, BT>(cl, acc3, wsm, slot[parity], tot);
            parity ^= 1;
        }
        if (threadIdx.x < R) {
            const int j = threadIdx.x;
            st.nf[j] = sqrt(tot[j]) + sqrt(tot[R + j]) + 1e-20;
            st.tol[j] = a.tolerance * st.nf[j];
            st.rho[j] = tot[2 * R + j];
            st.rho_old[j] = 0.0;
            st.nrm[j] = sqrt(st.rho[j]);
            st.alpha[j] = 0.0;
            st.act[j] = isfinite(st.nrm[j]) && st.nrm[j] > st.tol[j] && a.max_iter >= 1;
            st.iters[j] = 0;
            if (rank == 0) {
                a.out[(int64_t)sid * R + j].nf = st.nf[j];
                a.out[(int64_t)sid * R + j].norm0 = st.nrm[j];
            }
        }
        __syncthreads();

        if constexpr (MIXED) {
            // ---- FP32 CG sweeps on A e = r / ||r|| inside FP64 refinement ----
            for (int sweep = 0; sweep < a.max_outer; ++sweep) {
                bool act[R], any = false;
#pragma unroll
                for (int j = 0; j < R; ++j) {
                    act[j] = st.act[j];
                    any = any || act[j];
                }
                if (!any) break;
                // inner right-hand side r / ||r||, e = 0, and its squared norm
                {
                    const double *r = a.r + S.vec_offset * R;
                    float *r32 = a.r32 + S.vec_offset * R, *e32 = a.e32 + S.vec_offset * R;
                    float inv[R];
#pragma unroll
                    for (int j = 0; j < R; ++j) inv[j] = act[j] ? (float)(1.0 / st.nrm[j]) : 0.f;
                    double acc0[R];
#pragma unroll
                    for (int j = 0; j < R; ++j) acc0[j] = 0.0;
                    for (int s = s_lo + warp; s < s_hi; s += W) {
                        const int row = s * 32 + lane;
                        if (row < n)
#pragma unroll
                            for (int j = 0; j < R; ++j) {
                                const int64_t o = (int64_t)row * R + j;
                                const float v = (float)(r[o] * (double)inv[j]);
                                r32[o] = v;
                                e32[o] = 0.f;
                                acc0[j] += (double)(v * v);
                            }
                    }
                    cluster_sum<R, BT>(cl, acc0, wsm, slot[parity], tot);
                    parity ^= 1;
                }
                if (threadIdx.x < R) {
                    const int j = threadIdx.x;
                    st.rho32[j] = (float)tot[j];
                    st.rho32_old[j] = 0.f;
                    st.alpha[j] = 0.0;
                    st.act_in[j] = st.act[j];
                    // the last sweep only has to reach the FP64 target
                    st.eta[j] = (float)fmax(a.inner_rtol, fmin(0.5, 0.8 * st.tol[j] / st.nrm[j]));
                }
                __syncthreads();
                for (int k = 1;; ++k) {
                    bool ain[R], any_in = false;
#pragma unroll
                    for (int j = 0; j < R; ++j) {
                        ain[j] = st.act_in[j];
                        any_in = any_in || ain[j];
                    }
                    // P: e += alpha_{k-1} p (deferred), p = r + beta p
                    {
                        float beta[R], pend[R];
#pragma unroll
                        for (int j = 0; j < R; ++j) {
                            beta[j] = (k > 1 && ain[j]) ? st.rho32[j] / st.rho32_old[j] : 0.f;
                            pend[j] = (float)st.alpha[j];
                        }
                        const float *__restrict__ r32 = a.r32 + S.vec_offset * R;
                        float *__restrict__ p32 = a.p32 + S.vec_offset * pad_r<R>();
                        float *__restrict__ e32 = a.e32 + S.vec_offset * R;
                        // two rows (slices s and s + W) per step, all loads first
                        for (int s = s_lo + warp; s < s_hi; s += 2 * W) {
                            const int rows[2] = {s * 32 + lane, (s + W) * 32 + lane};
                            const bool ok[2] = {rows[0] < n, s + W < s_hi && rows[1] < n};
                            float pv[2][R], rv[2][R], ev[2][R];
#pragma unroll
                            for (int h = 0; h < 2; ++h)
                                if (ok[h]) {
                                    if (k > 1) ld_row<R>(p32, rows[h], pv[h]);
#pragma unroll
                                    for (int j = 0; j < R; ++j) {
                                        const int64_t o = (int64_t)rows[h] * R + j;
                                        rv[h][j] = r32[o];
                                        ev[h][j] = (k > 1 && pend[j] != 0.f) ? e32[o] : 0.f;
                                    }
                                }
#pragma unroll
                            for (int h = 0; h < 2; ++h)
                                if (ok[h]) {
#pragma unroll
                                    for (int j = 0; j < R; ++j) {
                                        const int64_t o = (int64_t)rows[h] * R + j;
                                        if (k == 1) {
                                            pv[h][j] = ain[j] ? rv[h][j] : 0.f;
                                        } else {
                                            if (pend[j] != 0.f) e32[o] = fma_t(pend[j], pv[h][j], ev[h][j]);
                                            if (ain[j]) pv[h][j] = fma_t(beta[j], pv[h][j], rv[h][j]);
                                        }
                                    }
                                    st_row<R>(p32, rows[h], pv[h]);
                                }
                        }
                    }
                    if (!any_in) break;
                    cl.sync(); // p complete before any CTA gathers it
                    // A: q = A p, (p, q)
                    {
                        const float *p32 = a.p32 + S.vec_offset * pad_r<R>();
                        float *q32 = a.q32 + S.vec_offset * R;
                        float accf[R];
#pragma unroll
                        for (int j = 0; j < R; ++j) accf[j] = 0.f;
                        for (int s = s_lo + warp; s < s_hi; s += W) {
                            const int row = s * 32 + lane;
                            float y[R], ys;
                            row_product<R, float, float>(
                                S, S.s_val32, S.val32, s, row, ain,
                                [&](int c, float(&o)[R]) { ld_row<R>(p32, c, o); }, y, ys);
                            if (row < n) {
                                float pv[R];
                                ld_row<R>(p32, row, pv);
#pragma unroll
                                for (int j = 0; j < R; ++j)
                                    if (ain[j]) {
                                        q32[(int64_t)row * R + j] = y[j];
                                        accf[j] = fma_t(pv[j], y[j], accf[j]);
                                    }
                            }
                        }
                        double acc[R];
#pragma unroll
                        for (int j = 0; j < R; ++j) acc[j] = accf[j];
                        cluster_sum<R, BT>(cl, acc, wsm, slot[parity], tot);
                        parity ^= 1;
                    }
                    // B: r -= alpha q, (r, r)
                    {
                        float alpha[R];
#pragma unroll
                        for (int j = 0; j < R; ++j) alpha[j] = ain[j] ? st.rho32[j] / (float)tot[j] : 0.f;
                        const float *__restrict__ q32 = a.q32 + S.vec_offset * R;
                        float *__restrict__ r32 = a.r32 + S.vec_offset * R;
                        float accf[R];
#pragma unroll
                        for (int j = 0; j < R; ++j) accf[j] = 0.f;
                        // two rows per step, all loads first
                        for (int s = s_lo + warp; s < s_hi; s += 2 * W) {
                            const int rows[2] = {s * 32 + lane, (s + W) * 32 + lane};
                            const bool ok[2] = {rows[0] < n, s + W < s_hi && rows[1] < n};
                            float qv[2][R], rv[2][R];
#pragma unroll
                            for (int h = 0; h < 2; ++h)
#pragma unroll
                                for (int j = 0; j < R; ++j) {
                                    const int64_t o = (int64_t)rows[h] * R + j;
                                    const bool use = ok[h] && ain[j];
                                    qv[h][j] = use ? q32[o] : 0.f;
                                    rv[h][j] = use ? r32[o] : 0.f;
                                }
#pragma unroll
                            for (int h = 0; h < 2; ++h)
#pragma unroll
                                for (int j = 0; j < R; ++j)
                                    if (ok[h] && ain[j]) {
                                        const float ri = fma_t(-alpha[j], qv[h][j], rv[h][j]);
                                        r32[(int64_t)rows[h] * R + j] = ri;
                                        accf[j] = fma_t(ri, ri, accf[j]);
                                    }
                        }
                        double acc2[R];
#pragma unroll
                        for (int j = 0; j < R; ++j) acc2[j] = accf[j];
                        if (threadIdx.x < R) st.alpha[threadIdx.x] = alpha[threadIdx.x];
                        cluster_sum<R, BT>(cl, acc2, wsm, slot[parity], tot);
                        parity ^= 1;
                    }
                    if (threadIdx.x < R) {
                        const int j = threadIdx.x;
                        if (st.act_in[j]) {
                            st.rho32_old[j] = st.rho32[j];
                            st.rho32[j] = (float)tot[j];
                            st.iters[j] += 1;
                            const float nin = sqrtf(st.rho32[j]);
                            st.act_in[j] = isfinite(nin) && nin > st.eta[j] && st.iters[j] < a.max_iter;
                        } else {
                            st.alpha[j] = 0.0;
                        }
                    }
                    __syncthreads();
                }
                // the inner loop ended with a P pass that applied every
                // pending step to e: x += ||r|| e in FP64
                {
                    const float *e32 = a.e32 + S.vec_offset * R;
                    double *x = a.x + S.vec_offset * R;
                    for (int s = s_lo + warp; s < s_hi; s += W) {
                        const int row = s * 32 + lane;
                        if (row < n)
#pragma unroll
                            for (int j = 0; j < R; ++j)
                                if (act[j]) {
                                    const int64_t o = (int64_t)row * R + j;
                                    x[o] = fma_t(st.nrm[j], (double)e32[o], x[o]);
                                }
                    }
                }
                cl.sync(); // every CTA's x rows are written before anyone gathers them
                batch_residual<R, BT>(cl, S, s_lo, s_hi, a.b + S.vec_offset * R, a.x + S.vec_offset * R,
                                      a.r + S.vec_offset * R, wsm, slot[parity], tot);
                parity ^= 1;
                if (threadIdx.x < R) {
                    const int j = threadIdx.x;
                    if (st.act[j]) {
                        const double nn = sqrt(tot[j]);
                        // a sweep that does not reduce the FP64 residual ends the solve
                        const bool progress = nn < st.nrm[j];
                        st.nrm[j] = nn;
                        st.act[j] = isfinite(nn) && nn > st.tol[j] && progress && st.iters[j] < a.max_iter;
                    }
                }
                __syncthreads();
            }
        } else {
            // ---- CG iterations, all components together ----------------------
            for (int k = 1;; ++k) {
                bool act[R], any = false;
#pragma unroll
                for (int j = 0; j < R; ++j) {
                    act[j] = st.act[j];
                    any = any || act[j];
                }
                // P: x += alpha_{k-1} p (deferred), p = r + beta p
                {
                    double beta[R], pend[R];
#pragma unroll
                    for (int j = 0; j < R; ++j) {
                        beta[j] = (k > 1 && act[j]) ? st.beta[j] : 0.0;
                        pend[j] = st.alpha[j];
                    }
                    const double *r = a.r + S.vec_offset * R;
                    double *p = a.p + S.vec_offset * pad_r<R>(), *x = a.x + S.vec_offset * R;
                    for (int s = s_lo + warp; s < s_hi; s += W) {
                        const int row = s * 32 + lane;
                        if (row < n) {
                            double pv[R];
                            if (k > 1) ld_row<R>(p, row, pv);
#pragma unroll
                            for (int j = 0; j < R; ++j) {
                                const int64_t o = (int64_t)row * R + j;
                                if (k == 1) {
                                    pv[j] = act[j] ? r[o] : 0.0;
                                } else {
                                    if (pend[j] != 0.0) x[o] = fma_t(pend[j], pv[j], x[o]);
                                    if (act[j]) pv[j] = fma_t(beta[j], pv[j], r[o]);
                                }
                            }
                            st_row<R>(p, row, pv);
                        }
                    }
                }
                if (!any) break;
                cl.sync(); // p complete before any CTA gathers it
                // A: q = A p, (p, q)
                {
                    const double *p = a.p + S.vec_offset * pad_r<R>();
                    double *q = a.q + S.vec_offset * R;
                    double acc[R];
#pragma unroll
                    for (int j = 0; j < R; ++j) acc[j] = 0.0;
                    for (int s = s_lo + warp; s < s_hi; s += W) {
                        const int row = s * 32 + lane;
                        double y[R], ys;
                        row_product<R, double, double>(
                            S, S.s_val, S.val, s, row, act,
                            [&](int c, double(&o)[R]) { ld_row<R>(p, c, o); }, y, ys);
                        if (row < n) {
                            double pv[R];
                            ld_row<R>(p, row, pv);
#pragma unroll
                            for (int j = 0; j < R; ++j)
                                if (act[j]) {
                                    q[(int64_t)row * R + j] = y[j];
                                    acc[j] = fma_t(pv[j], y[j], acc[j]);
                                }
                        }
                    }
                    // the step lengths, once per CTA (a division is a chain of
                    // dependent FP64 instructions)
                    cluster_sum<R, BT>(cl, acc, wsm, slot[parity], tot, [&](int j, double pq) {
                        st.alpha[j] = st.act[j] ? st.rho[j] / pq : 0.0;
                    });
                    parity ^= 1;
                }
                // B: r -= alpha q, (r, r)
                {
                    double alpha[R];
#pragma unroll
                    for (int j = 0; j < R; ++j) alpha[j] = st.alpha[j];
                    const double *q = a.q + S.vec_offset * R;
                    double *r = a.r + S.vec_offset * R;
                    double acc2[R];
#pragma unroll
                    for (int j = 0; j < R; ++j) acc2[j] = 0.0;
                    for (int s = s_lo + warp; s < s_hi; s += W) {
                        const int row = s * 32 + lane;
                        if (row < n)
#pragma unroll
                            for (int j = 0; j < R; ++j)
                                if (act[j]) {
                                    const int64_t o = (int64_t)row * R + j;
                                    const double ri = fma_t(-alpha[j], q[o], r[o]);
                                    r[o] = ri;
                                    acc2[j] = fma_t(ri, ri, acc2[j]);
                                }
                    }
                    cluster_sum<R, BT>(cl, acc2, wsm, slot[parity], tot);
                    parity ^= 1;
                }
                if (threadIdx.x < R) {
                    const int j = threadIdx.x;
                    if (st.act[j]) {
                        st.rho_old[j] = st.rho[j];
                        st.rho[j] = tot[j];
                        st.beta[j] = st.rho[j] / st.rho_old[j];
                        st.nrm[j] = sqrt(st.rho[j]);
                        st.iters[j] = k;
                        st.act[j] = isfinite(st.nrm[j]) && k < a.max_iter && st.nrm[j] > st.tol[j];
                    } else {
                        st.alpha[j] = 0.0;
                    }
                }
                __syncthreads();
            }
        }
        if (rank == 0 && threadIdx.x < R) {
            const int j = threadIdx.x;
            BatchResult &o = a.out[(int64_t)sid * R + j];
            o.norm = st.nrm[j];
            o.iters = st.iters[j];
            o.status = !isfinite(st.nrm[j]) ? CF_NONFINITE : (st.nrm[j] > st.tol[j] ? CF_NOT_CONVERGED : CF_OK);
        }
        __syncthreads();
    }
    cl.sync(); // no CTA leaves while a peer may still read its shared memory
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct Batch {
    Context *ctx = nullptr;
    std::vector<Matrix *> mats;
    std::vector<int64_t> offsets;   // first row of each system
    int64_t rows = 0;
    DeviceBuffer d_sys, d_order, d_queue, d_out, d_b, d_x, d_r, d_p, d_q;
    DeviceBuffer d_r32, d_p32, d_q32, d_e32;
    bool have_32 = false;
    std::vector<int32_t> order;
    ~Batch()
    {
        for (Matrix *m : mats) delete m;
    }
};

Batch *batch_create(Context *ctx, int n_systems, const cf_ldu_view *views)
{
    require(n_systems > 0 && views, CF_BAD_INPUT, "empty batch");
    Batch *B = new Batch();
    B->ctx = ctx;
    try {
        std::vector<BatchSystem> hs(n_systems);
        for (int s = 0; s < n_systems; ++s) {
            Matrix *m = matrix_create(ctx, views[s]);
            B->mats.push_back(m);
            require(m->n > 0, CF_BAD_INPUT, "empty system in batch");
            hs[s].n = m->n;
            hs[s].vec_offset = B->rows;
            hs[s].ro = m->ro.as<int32_t>();
            hs[s].col = m->col.as<int32_t>();
            hs[s].val = m->val.as<double>();
            hs[s].val32 = nullptr;
            // the SELL-32 copy, unless the rows are too uneven for it
            hs[s].sell = matrix_ensure_sell(m, false, false) ? 1 : 0;
            hs[s].s_off = hs[s].sell ? m->s_off.as<int32_t>() : nullptr;
            hs[s].s_col = hs[s].sell ? m->s_col.as<int32_t>() : nullptr;
            hs[s].s_val = hs[s].sell ? m->s_val.as<double>() : nullptr;
            hs[s].s_val32 = nullptr;
            B->offsets.push_back(B->rows);
            B->rows += m->n;
        }
        // largest systems first (longest-processing-time order)
        B->order.resize(n_systems);
        std::iota(B->order.begin(), B->order.end(), 0);
        std::stable_sort(B->order.begin(), B->order.end(), [&](int a, int b) {
            return B->mats[a]->nnz > B->mats[b]->nnz;
        });
        B->d_sys.ensure(sizeof(BatchSystem) * n_systems);
        B->d_order.ensure(sizeof(int32_t) * n_systems);
        B->d_queue.ensure(sizeof(int32_t) * 4);
        CF_CUDA(cudaMemcpyAsync(B->d_sys.ptr, hs.data(), sizeof(BatchSystem) * n_systems,
                                cudaMemcpyHostToDevice, ctx->stream));
        CF_CUDA(cudaStreamSynchronize(ctx->stream));
    } catch (...) {
        delete B;
        throw;
    }
    return B;
}

void batch_destroy(Batch *B) { delete B; }

template <int R, int BT, bool MIXED>
static void launch_batch(Context *ctx, const BatchArgs &args, int cs, int max_clusters, cudaStream_t s)
{
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.blockDim = dim3(BT);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const auto kernel = k_batch_cg<R, BT, MIXED>;
    // cs == 0: 16-CTA clusters where they fit on the device, else 8
    const bool pick = cs == 0;
    int nclusters = 0;
    for (int c = pick ? 16 : cs; c >= (pick ? 8 : cs); c /= 2) {
        if (c > 8) // 16-CTA clusters are beyond the portable limit of 8
            CF_CUDA(cudaFuncSetAttribute((const void *)kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
        attr[0].val.clusterDim.x = c;
        cfg.gridDim = dim3(c);
        nclusters = 0;
        if (cudaOccupancyMaxActiveClusters(&nclusters, (void *)kernel, &cfg) != cudaSuccess) {
            cudaGetLastError();
            nclusters = 0;
        }
        cs = c;
        if (nclusters >= 1) break;
    }
    require(nclusters >= 1, CF_UNSUPPORTED, "no cluster of this size and block size fits on the device");
    if (max_clusters > 0 && nclusters > max_clusters) nclusters = max_clusters;
    cfg.gridDim = dim3(nclusters * cs);
    CF_CUDA(cudaLaunchKernelEx(&cfg, kernel, args));
}

template <int R, bool MIXED>
static void launch_batch_m(Context *ctx, const BatchArgs &args, int cs, int bt, int max_clusters,
                           cudaStream_t s)
{
    if (bt == 128) launch_batch<R, 128, MIXED>(ctx, args, cs, max_clusters, s);
    else if (bt == 512) launch_batch<R, 512, MIXED>(ctx, args, cs, max_clusters, s);
    else launch_batch<R, 256, MIXED>(ctx, args, cs, max_clusters, s);
}

template <int R>
static void launch_batch_r(Context *ctx, const BatchArgs &args, bool mixed, int cs, int bt, int max_clusters,
                           cudaStream_t s)
{
    if (mixed) launch_batch_m<R, true>(ctx, args, cs, bt, max_clusters, s);
    else launch_batch_m<R, false>(ctx, args, cs, bt, max_clusters, s);
}

// Solve all systems for `nrhs` right-hand sides (b, x: [rows][nrhs]).
void batch_solve(Batch *B, const cf_controls &c, int nrhs, const double *b_in, double *x_io,
                 int memory, const cf_batch_config *cfg, cf_batch_result *results, float *ms_out)
{
    Context *ctx = B->ctx;
    require(nrhs >= 1 && nrhs <= kBatchMaxR, CF_BAD_INPUT, "1..4 right-hand sides per system");
    require(c.precision == CF_PREC_FP64 || c.precision == CF_PREC_MIXED, CF_BAD_INPUT, "bad precision");
    const bool mixed = c.precision == CF_PREC_MIXED;
    const int S = (int)B->mats.size();
    if (mixed && !B->have_32) {
        // FP32 value copies, then the system table with their pointers
        std::vector<BatchSystem> hs(S);
        CF_CUDA(cudaMemcpy(hs.data(), B->d_sys.ptr, sizeof(BatchSystem) * S, cudaMemcpyDeviceToHost));
        for (int s2 = 0; s2 < S; ++s2) {
            Matrix *m = B->mats[s2];
            matrix_ensure_fp32(m, false);
            hs[s2].val32 = m->val32.as<float>();
            if (hs[s2].sell) {
                matrix_ensure_sell(m, false, true);
                hs[s2].s_val32 = m->s_val32.as<float>();
            }
        }
        CF_CUDA(cudaMemcpyAsync(B->d_sys.ptr, hs.data(), sizeof(BatchSystem) * S, cudaMemcpyHostToDevice,
                                ctx->stream));
        CF_CUDA(cudaStreamSynchronize(ctx->stream));
        B->have_32 = true;
    }
    if (mixed) {
        const size_t fb = sizeof(float) * (size_t)(B->rows * nrhs + 8);
        B->d_r32.ensure(fb);
        B->d_p32.ensure(sizeof(float) * (size_t)(B->rows * 4 + 8));   // rows padded to 4 components
        B->d_q32.ensure(fb);
        B->d_e32.ensure(fb);
    }
    const size_t vb = sizeof(double) * (size_t)(B->rows * nrhs + 8);
    B->d_r.ensure(vb);
    B->d_p.ensure(sizeof(double) * (size_t)(B->rows * 4 + 8));   // rows padded to 4 components
    B->d_q.ensure(vb);
    double *x, *b;
    if (memory == CF_MEM_HOST) {
        B->d_b.ensure(vb);
        B->d_x.ensure(vb);
        b = B->d_b.as<double>();
        x = B->d_x.as<double>();
        upload(ctx, b, b_in, sizeof(double) * (size_t)B->rows * nrhs, CF_MEM_HOST);
        upload(ctx, x, x_io, sizeof(double) * (size_t)B->rows * nrhs, CF_MEM_HOST);
    } else {
        b = const_cast<double *>(b_in);
        x = x_io;
    }
    B->d_out.ensure(sizeof(BatchResult) * (size_t)S * nrhs);
    // processing order: largest first unless the configuration asks otherwise
    std::vector<int32_t> order = B->order;
    if (cfg && cfg->order == 1) std::iota(order.begin(), order.end(), 0);
    CF_CUDA(cudaMemcpyAsync(B->d_order.ptr, order.data(), sizeof(int32_t) * S, cudaMemcpyHostToDevice,
                            ctx->stream));
    CF_CUDA(cudaMemsetAsync(B->d_queue.ptr, 0, sizeof(int32_t), ctx->stream));
    BatchArgs a;
    a.sys = B->d_sys.as<BatchSystem>();
    a.order = B->d_order.as<int32_t>();
    a.n_systems = S;
    a.max_iter = c.max_iter <= 0 ? INT_MAX : c.max_iter;
    a.tolerance = c.tolerance;
    a.b = b;
    a.x = x;
    a.r = B->d_r.as<double>();
    a.p = B->d_p.as<double>();
    a.q = B->d_q.as<double>();
    a.queue = B->d_queue.as<int32_t>();
    a.out = B->d_out.as<BatchResult>();
    a.r32 = mixed ? B->d_r32.as<float>() : nullptr;
    a.p32 = mixed ? B->d_p32.as<float>() : nullptr;
    a.q32 = mixed ? B->d_q32.as<float>() : nullptr;
    a.e32 = mixed ? B->d_e32.as<float>() : nullptr;
    a.inner_rtol = (c.mixed_inner_rtol > 0 && c.mixed_inner_rtol < 1) ? c.mixed_inner_rtol : 1e-6;
    a.max_outer = c.mixed_max_outer > 0 ? c.mixed_max_outer : 50;
    const int cs = cfg && cfg->cluster_size > 0 ? cfg->cluster_size : 0;   // 0: 16, else 8
    const int bt = cfg && cfg->threads > 0 ? cfg->threads : 256;
    const int maxc = cfg ? cfg->max_clusters : 0;
    require(cs == 0 || cs == 1 || cs == 2 || cs == 4 || cs == 8 || cs == 16, CF_BAD_INPUT,
            "cluster size must be 1, 2, 4, 8 or 16");
    require(bt == 128 || bt == 256 || bt == 512, CF_BAD_INPUT, "threads must be 128, 256 or 512");

    // one persistent launch, captured in a CUDA graph together with the
    // queue reset so the whole batch is a single graph launch
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ge = nullptr;
    cudaStream_t cs_stream = nullptr;
    const bool use_graph = c.use_graph != 0;
    CF_CUDA(cudaEventRecord(ctx->ev_start, ctx->stream));
    if (use_graph) {
        CF_CUDA(cudaStreamCreateWithFlags(&cs_stream, cudaStreamNonBlocking));
        try {
            CF_CUDA(cudaStreamBeginCapture(cs_stream, cudaStreamCaptureModeThreadLocal));
            CF_CUDA(cudaMemsetAsync(B->d_queue.ptr, 0, sizeof(int32_t), cs_stream));
            switch (nrhs) {
            case 1: launch_batch_r<1>(ctx, a, mixed, cs, bt, maxc, cs_stream); break;
            case 2: launch_batch_r<2>(ctx, a, mixed, cs, bt, maxc, cs_stream); break;
            case 3: launch_batch_r<3>(ctx, a, mixed, cs, bt, maxc, cs_stream); break;
            default: launch_batch_r<4>(ctx, a, mixed, cs, bt, maxc, cs_stream); break;
            }
            CF_CUDA(cudaStreamEndCapture(cs_stream, &g));
            CF_CUDA(cudaGraphInstantiate(&ge, g, 0));
            CF_CUDA(cudaGraphLaunch(ge, ctx->stream));
        } catch (...) {
            cudaGraph_t junk = nullptr;
            cudaStreamEndCapture(cs_stream, &junk);
            if (junk) cudaGraphDestroy(junk);
            if (ge) cudaGraphExecDestroy(ge);
            if (g) cudaGraphDestroy(g);
            cudaStreamDestroy(cs_stream);
            cudaGetLastError();
            throw;
        }
    } else {
        switch (nrhs) {
        case 1: launch_batch_r<1>(ctx, a, mixed, cs, bt, maxc, ctx->stream); break;
        case 2: launch_batch_r<2>(ctx, a, mixed, cs, bt, maxc, ctx->stream); break;
        case 3: launch_batch_r<3>(ctx, a, mixed, cs, bt, maxc, ctx->stream); break;
        default: launch_batch_r<4>(ctx, a, mixed, cs, bt, maxc, ctx->stream); break;
        }
    }
    CF_CUDA(cudaEventRecord(ctx->ev_stop, ctx->stream));
    CF_CUDA(cudaStreamSynchronize(ctx->stream));
    if (ge) cudaGraphExecDestroy(ge);
    if (g) cudaGraphDestroy(g);
    if (cs_stream) cudaStreamDestroy(cs_stream);
    float ms = 0.f;
    CF_CUDA(cudaEventElapsedTime(&ms, ctx->ev_start, ctx->ev_stop));
    if (ms_out) *ms_out = ms;
    if (memory == CF_MEM_HOST)
        download(ctx, x_io, x, sizeof(double) * (size_t)B->rows * nrhs, CF_MEM_HOST);
    if (results) {
        std::vector<BatchResult> h((size_t)S * nrhs);
        CF_CUDA(cudaMemcpyAsync(h.data(), B->d_out.ptr, sizeof(BatchResult) * h.size(),
                                cudaMemcpyDeviceToHost, ctx->stream));
        CF_CUDA(cudaStreamSynchronize(ctx->stream));
        for (size_t i = 0; i < h.size(); ++i) {
            results[i].norm_factor = h[i].nf;
            results[i].initial_residual = h[i].norm0 / h[i].nf;
            results[i].final_residual = h[i].norm / h[i].nf;
            results[i].n_iterations = h[i].iters;
            results[i].status = h[i].status;
        }
    }
    CF_CUDA(cudaStreamSynchronize(ctx->stream));
}

// ---------------------------------------------------------------------------
// One small system: the whole CG solve in one cluster-persistent launch
// ---------------------------------------------------------------------------
// Rows per CTA the single-system path aims for when it sizes its cluster
// (one row per thread: its passes are latency chains, so the most threads
// win; measured at 64^2: 256 rows 8.7 us per step, 512 10.2, 2048 22.6).
#ifndef CF_SMALL_CG_ROWS_PER_CTA
#define CF_SMALL_CG_ROWS_PER_CTA 256
#endif

// Whether a 16-CTA cluster of the single-system kernel fits on this device
// (asked once per context; the solve takes the multi-kernel loop otherwise).
bool small_cg_ok(Context *ctx)
{
    if (ctx->small_cg_ok < 0) {
        const auto kernel = k_batch_cg<1, 256, false>;
        cudaLaunchConfig_t cfg = {};
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = 16;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.blockDim = dim3(256);
        cfg.gridDim = dim3(16);
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        int nclusters = 0;
        const bool ok = cudaFuncSetAttribute((const void *)kernel, cudaFuncAttributeNonPortableClusterSizeAllowed,
                                             1) == cudaSuccess &&
                        cudaOccupancyMaxActiveClusters(&nclusters, (void *)kernel, &cfg) == cudaSuccess &&
                        nclusters >= 1;
        cudaGetLastError();
        ctx->small_cg_ok = ok ? 1 : 0;
    }
    return ctx->small_cg_ok == 1;
}

// CG (FP64, the fast summation order) on one system with the batched
// kernel: one cluster of up to 16 CTAs runs normFactor, the initial residual
// and every step, with hardware cluster barriers where the multi-kernel
// loop has kernel boundaries.  x, b, r, p, q are device vectors of n rows.
SmallSolveResult solve_cg_single_cluster(Matrix *m, const cf_controls &c, const double *b, double *x,
                                         double *r, double *p, double *q)
{
    Context *ctx = m->ctx;
    const int n = m->n;
    const bool sell = matrix_ensure_sell(m, false, false);
    struct Block {
        BatchSystem sys;
        int32_t order[4];
        int32_t queue[4];
        BatchResult out;
    };
    DeviceBuffer &blk = ctx->vec[23];
    blk.ensure(sizeof(Block));
    Block h{};
    h.sys.n = n;
    h.sys.sell = sell ? 1 : 0;
    h.sys.vec_offset = 0;
    h.sys.ro = m->ro.as<int32_t>();
    h.sys.col = m->col.as<int32_t>();
    h.sys.val = m->val.as<double>();
    h.sys.val32 = nullptr;
    h.sys.s_off = sell ? m->s_off.as<int32_t>() : nullptr;
    h.sys.s_col = sell ? m->s_col.as<int32_t>() : nullptr;
    h.sys.s_val = sell ? m->s_val.as<double>() : nullptr;
    h.sys.s_val32 = nullptr;
    Block *d = blk.as<Block>();
    CF_CUDA(cudaMemcpyAsync(d, &h, sizeof(Block), cudaMemcpyHostToDevice, ctx->stream));
    BatchArgs a{};
    a.sys = &d->sys;
    a.order = d->order;
    a.n_systems = 1;
    a.max_iter = c.max_iter <= 0 ? INT_MAX : c.max_iter;
    a.tolerance = c.tolerance;
    a.b = b;
    a.x = x;
    a.r = r;
    a.p = p;
    a.q = q;
    a.queue = d->queue;
    a.out = &d->out;
    int cs = 1;
    while (cs < 16 && (int64_t)cs * CF_SMALL_CG_ROWS_PER_CTA < n) cs <<= 1;
    CF_CUDA(cudaEventRecord(ctx->ev_start, ctx->stream));
    launch_batch<1, 256, false>(ctx, a, cs, 1, ctx->stream);
    CF_CUDA(cudaEventRecord(ctx->ev_stop, ctx->stream));
    BatchResult res;
    CF_CUDA(cudaMemcpyAsync(&res, &d->out, sizeof(res), cudaMemcpyDeviceToHost, ctx->stream));
    CF_CUDA(cudaStreamSynchronize(ctx->stream));
    float ms = 0.f;
    CF_CUDA(cudaEventElapsedTime(&ms, ctx->ev_start, ctx->ev_stop));
    SmallSolveResult o;
    o.nf = res.nf;
    o.norm0 = res.norm0;
    o.norm = res.norm;
    o.iters = res.iters;
    o.status = res.status;
    o.ms = ms;
    return o;
}

int64_t batch_rows(const Batch *B) { return B->rows; }
int batch_systems(const Batch *B) { return (int)B->mats.size(); }
int64_t batch_offset(const Batch *B, int s) { return B->offsets[s]; }

} // namespace cf

namespace cf {

// ---------------------------------------------------------------------------
// Jacobi, Richardson and the MR family on one small system in one
// cluster-persistent launch (the CG kernel's schedule: one cluster of up to
// 16 CTAs, rows split by 32-row slices, hardware cluster barriers where the
// multi-kernel loop has kernel boundaries), fast summation order.  The
// drivers are the reference's (SolverSingleGPU.h: Richardson 762-819 with
// OptimizePower 723-752, MR 825-890, Jacobi 924-994, MRJacobi 1000-1073,
// JMR 1079-1155, MRS 1236-1303); the stopping rule the library's.
// ---------------------------------------------------------------------------
struct SmallArgs {
    const BatchSystem *sys;
    int32_t solver;
    int32_t max_iter;
    double tolerance;
    double omega;            // Richardson: 0 = the power method
    int32_t power_steps;
    const double *b;
    double *x, *r, *d, *y;
    const double *dinv, *dsq, *diag;
    SmallSolveOut *out;
};

// all CTAs' values of one row owned by this thread, or 0
template <class F>
__device__ __forceinline__ void small_rows(int n, int s_lo, int s_hi, F f)
{
    constexpr int W = 256 / 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int s = s_lo + warp; s < s_hi; s += W) {
        const int row = s * 32 + lane;
        f(s, row, row < n);
    }
}

__global__ void __launch_bounds__(256, 1) k_small_solve(const SmallArgs a)
{
    cgp::cluster_group cl = cgp::this_cluster();
    const int cs = (int)cl.num_blocks();
    const int rank = (int)cl.block_rank();
    __shared__ double wsm[3 * 8];
    __shared__ double slot[2][3];
    __shared__ double tot[3];
    __shared__ BatchSystem S;
    __shared__ double s_alpha, s_nrm, s_tol, s_omega;
    __shared__ int s_act;
    int parity = 0;
    if (threadIdx.x == 0) S = *a.sys;
    __syncthreads();
    const int n = S.n;
    const int ns = (n + 31) >> 5;
    const int s_lo = (int)((int64_t)ns * rank / cs), s_hi = (int)((int64_t)ns * (rank + 1) / cs);
    const int solver = a.solver;
    const bool on[1] = {true};
    double *x = a.x, *r = a.r, *d = a.d, *y = a.y;
    const double *b = a.b;
    auto gather = [](const double *v) {
        return [v](int c, double(&o)[1]) { o[0] = __ldcg(v + c); };
    };
    auto reduce = [&](double (&acc)[1]) {
        cluster_sum<1, 256>(cl, acc, wsm, slot[parity], tot);
        parity ^= 1;
        return tot[0];
    };

    // ---- normFactor and the initial residual -----------------------------
    double acc1[1] = {0.0};
    small_rows(n, s_lo, s_hi, [&](int, int row, bool ok) {
        if (ok) acc1[0] += x[row];
    });
    const double xbar = reduce(acc1) / n;
    {
        double acc3[3] = {0.0, 0.0, 0.0};
        small_rows(n, s_lo, s_hi, [&](int s, int row, bool ok) {
            double yv[1], ys;
            row_product<1, double, double>(S, S.s_val, S.val, s, row, on, gather(x), yv, ys);
            if (ok) {
                const double yb = ys * xbar, bi = b[row];
                const double d1 = yv[0] - yb, d2 = bi - yb;
                double ri = bi - yv[0];
                if (solver == CF_JMR) ri = __dmul_rn(a.dsq[row], ri);
                r[row] = ri;
                acc3[0] = fma_t(d1, d1, acc3[0]);
                acc3[1] = fma_t(d2, d2, acc3[1]);
                acc3[2] = fma_t(ri, ri, acc3[2]);
            }
        });
        cluster_sum<3, 256>(cl, acc3, wsm, slot[parity], tot);
        parity ^= 1;
    }
    if (threadIdx.x == 0) {
        const double nf = sqrt(tot[0]) + sqrt(tot[1]) + 1e-20;
        s_tol = a.tolerance * nf;
        s_nrm = sqrt(tot[2]);
        s_omega = a.omega;
        if (rank == 0) {
            a.out->nf = nf;
            a.out->norm0 = s_nrm;
        }
    }
    __syncthreads();

    // ---- Richardson's relaxation factor: OptimizePower on the system ------
    if (solver == CF_RICHARDSON && s_omega > -1e-15 && s_omega < 1e-15) {
        // x2 (in y) = 1/N; steps of x1 (in d) = x2, x2 = A x1 / ||A x1||
        small_rows(n, s_lo, s_hi, [&](int, int row, bool ok) {
            if (ok) y[row] = 1.0 / n;
        });
        for (int st = 0; st < a.power_steps; ++st) {
            small_rows(n, s_lo, s_hi, [&](int, int row, bool ok) {
                if (ok) d[row] = y[row];
            });
            cl.sync(); // every CTA's x1 rows are written before anyone gathers them
            double acc[1] = {0.0};
            small_rows(n, s_lo, s_hi, [&](int s, int row, bool ok) {
                double yv[1], ys;
                row_product<1, double, double>(S, S.s_val, S.val, s, row, on, gather(d), yv, ys);
                if (ok) {
                    y[row] = yv[0];
                    acc[0] = fma_t(yv[0], yv[0], acc[0]);
                }
            });
            const double inv = 1 / sqrt(reduce(acc));
            small_rows(n, s_lo, s_hi, [&](int, int row, bool ok) {
                if (ok) y[row] = __dmul_rn(y[row], inv);
            });
        }
        cl.sync(); // x2 complete before anyone gathers it
        double acc[1] = {0.0}, amin = HUGE_VAL;
        small_rows(n, s_lo, s_hi, [&](int s, int row, bool ok) {
            double yv[1], ys;
            row_product<1, double, double>(S, S.s_val, S.val, s, row, on, gather(y), yv, ys);
            if (ok) {
                acc[0] = fma_t(y[row], yv[0], acc[0]);
                amin = fmin(amin, fabs(a.diag[row]));
            }
        });
        const double lmax = reduce(acc);
        // the smallest |a_ii|: -max(-|a_ii|) through the same reduction slots
        double m = -amin;
#pragma unroll
        for (int o = 16; o; o >>= 1) m = fmax(m, __shfl_xor_sync(kFull, m, o));
        if ((threadIdx.x & 31) == 0) wsm[threadIdx.x >> 5] = m;
        __syncthreads();
        if (threadIdx.x == 0) {
            double mm = wsm[0];
            for (int w = 1; w < 8; ++w) mm = fmax(mm, wsm[w]);
            slot[parity][0] = mm;
        }
        cl.sync();
        if (threadIdx.x == 0) {
            double mm = -HUGE_VAL;
            for (int k = 0; k < cs; ++k) mm = fmax(mm, cl.map_shared_rank(slot[parity], k)[0]);
            s_omega = 2.0 / (lmax + (-mm));
            if (rank == 0) a.out->omega = s_omega;
        }
        parity ^= 1;
        __syncthreads();
    } else if (threadIdx.x == 0 && rank == 0) {
        a.out->omega = s_omega;
    }

    // ---- the iterations ---------------------------------------------------
    const double *w = solver == CF_MR ? nullptr : (solver == CF_JMR ? a.dsq : a.dinv);
    int k = 0;
    if (threadIdx.x == 0) s_act = isfinite(s_nrm) && a.max_iter >= 1 && s_nrm > s_tol;
    __syncthreads();
    while (s_act) {
        ++k;
        double acc[1] = {0.0};
        if (solver == CF_RICHARDSON) {
            const double om = s_omega;
            small_rows(n, s_lo, s_hi, [&](int, int row, bool ok) {
                if (ok) x[row] = fma_t(om, r[row], x[row]);
            });
            cl.sync(); // x complete before anyone gathers it
            small_rows(n, s_lo, s_hi, [&](int s, int row, bool ok) {
                double yv[1], ys;
                row_product<1, double, double>(S, S.s_val, S.val, s, row, on, gather(x), yv, ys);
                if (ok) {
                    const double ri = b[row] - yv[0];
                    r[row] = ri;
                    acc[0] = fma_t(ri, ri, acc[0]);
                }
            });
        } else {
            // d = R r (MR: r itself), y = A d (JMR: D^-1/2 A d)
            const double *dv = r;
            if (w) {
                small_rows(n, s_lo, s_hi, [&](int, int row, bool ok) {
                    if (ok) d[row] = __dmul_rn(w[row], r[row]);
                });
                cl.sync(); // d complete before anyone gathers it
                dv = d;
            }
            double t2[2] = {0.0, 0.0};
            small_rows(n, s_lo, s_hi, [&](int s, int row, bool ok) {
                double yv[1], ys;
                row_product<1, double, double>(S, S.s_val, S.val, s, row, on, gather(dv), yv, ys);
                if (ok) {
                    double yi = yv[0];
                    if (solver == CF_JMR) yi = __dmul_rn(a.dsq[row], yi);
                    y[row] = yi;
                    if (solver != CF_JACOBI) {
                        t2[0] = fma_t(r[row], yi, t2[0]);
                        t2[1] = fma_t(yi, yi, t2[1]);
                    }
                }
            });
            if (solver != CF_JACOBI) {
                // every CTA has gathered r (MR) before anyone updates it
                cluster_sum<2, 256>(cl, t2, wsm, slot[parity], tot, [&](int i, double v) {
                    if (i == 1) s_alpha = tot[0] / v;
                });
                parity ^= 1;
            } else if (threadIdx.x == 0) {
                s_alpha = 1.0;
            }
            if (solver == CF_JACOBI) __syncthreads();
            const double al = s_alpha;
            small_rows(n, s_lo, s_hi, [&](int, int row, bool ok) {
                if (ok) {
                    x[row] = fma_t(al, dv[row], x[row]);
                    const double ri = fma_t(-al, y[row], r[row]);
                    r[row] = ri;
                    acc[0] = fma_t(ri, ri, acc[0]);
                }
            });
        }
        const double nrm = sqrt(reduce(acc));
        if (threadIdx.x == 0) {
            s_nrm = nrm;
            s_act = isfinite(nrm) && k < a.max_iter && nrm > s_tol;
        }
        __syncthreads();
    }
    if (rank == 0 && threadIdx.x == 0) {
        a.out->norm = s_nrm;
        a.out->iters = k;
        a.out->status = !isfinite(s_nrm) ? CF_NONFINITE : (s_nrm > s_tol ? CF_NOT_CONVERGED : CF_OK);
    }
    cl.sync(); // no CTA leaves while a peer may still read its shared memory
}

SmallSolveResult solve_small_single_cluster(Matrix *m, int solver, const cf_controls &c, const double *b,
                                            double *x, double *r, double *d, double *y)
{
    Context *ctx = m->ctx;
    const int n = m->n;
    const bool sell = matrix_ensure_sell(m, false, false);
    struct Block {
        BatchSystem sys;
        SmallSolveOut out;
    };
    DeviceBuffer &blk = ctx->vec[23];
    blk.ensure(sizeof(Block));
    Block h{};
    h.sys.n = n;
    h.sys.sell = sell ? 1 : 0;
    h.sys.ro = m->ro.as<int32_t>();
    h.sys.col = m->col.as<int32_t>();
    h.sys.val = m->val.as<double>();
    h.sys.s_off = sell ? m->s_off.as<int32_t>() : nullptr;
    h.sys.s_col = sell ? m->s_col.as<int32_t>() : nullptr;
    h.sys.s_val = sell ? m->s_val.as<double>() : nullptr;
    Block *dblk = blk.as<Block>();
    CF_CUDA(cudaMemcpyAsync(dblk, &h, sizeof(Block), cudaMemcpyHostToDevice, ctx->stream));
    SmallArgs a{};
    a.sys = &dblk->sys;
    a.solver = solver;
    a.max_iter = c.max_iter <= 0 ? INT_MAX : c.max_iter;
    a.tolerance = c.tolerance;
    a.omega = c.richardson_omega;
    a.power_steps = c.power_max_steps > 0 ? c.power_max_steps : 30;
    a.b = b;
    a.x = x;
    a.r = r;
    a.d = d;
    a.y = y;
    a.dinv = m->dinv.as<double>();
    a.dsq = m->dinv_sqrt.as<double>();
    a.diag = m->diag.as<double>();
    a.out = &dblk->out;
    int cs = 1;
    while (cs < 16 && (int64_t)cs * CF_SMALL_CG_ROWS_PER_CTA < n) cs <<= 1;
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = cs;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.blockDim = dim3(256);
    cfg.gridDim = dim3(cs);
    cfg.stream = ctx->stream;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (cs > 8)
        CF_CUDA(cudaFuncSetAttribute((const void *)k_small_solve, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    CF_CUDA(cudaEventRecord(ctx->ev_start, ctx->stream));
    CF_CUDA(cudaLaunchKernelEx(&cfg, k_small_solve, a));
    CF_CUDA(cudaEventRecord(ctx->ev_stop, ctx->stream));
    SmallSolveOut res;
    CF_CUDA(cudaMemcpyAsync(&res, &dblk->out, sizeof(res), cudaMemcpyDeviceToHost, ctx->stream));
    CF_CUDA(cudaStreamSynchronize(ctx->stream));
    float ms = 0.f;
    CF_CUDA(cudaEventElapsedTime(&ms, ctx->ev_start, ctx->ev_stop));
    SmallSolveResult o;
    o.nf = res.nf;
    o.norm0 = res.norm0;
    o.norm = res.norm;
    o.iters = res.iters;
    o.status = res.status;
    o.ms = ms;
    o.omega = res.omega;
    return o;
}

} // namespace cf
