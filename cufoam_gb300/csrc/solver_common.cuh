// solver_common.cuh -- pieces shared by the FP64 and mixed-precision solver
// translation units: per-warp staging declaration, loop bookkeeping run by
// the last block of a reduction, and the host-side launch / CUDA-graph
// helpers of the device-driven iteration loop.
#pragma once

#include "device.cuh"

namespace cf {

// shared-memory staging area of this warp (declared in every SpMV kernel)
#define CF_STAGE(V, cap)                                                              \
    extern __shared__ __align__(16) unsigned char smem_raw_[];                        \
    unsigned char *area_ = smem_raw_ + (threadIdx.x >> 5) * stage_bytes_per_warp<V>(cap); \
    V *sv_ = reinterpret_cast<V *>(area_);                                            \
    int32_t *sc_ = reinterpret_cast<int32_t *>(area_ + (size_t)((cap) + 8) * sizeof(V))

// ---------------------------------------------------------------------------
// SpMV row passes.  The fast kernels read the matrix either as CSR with
// warp-chunk staging (kCsr) or from its SELL-32 copy (kSell); both sum each
// row as one FMA chain in entry order.  for_rows calls f(row, sum_j a_ij g(j))
// for every row; val is the CSR value array, sval its SELL-32 copy.
// ---------------------------------------------------------------------------
// kSellC: the SELL-32 copy with one-byte column codes (SellCodes8); kSellD:
// with 16-bit column deltas (SellDelta16)
enum { kCsr = 0, kSell = 1, kSellC = 2, kSellD = 3 };

// SELL passes take CF_SELL_BATCH entries per thread per batch: all their
// loads and gathers are issued before the first FMA, and a row's last
// entries form one exact batch.  With eight a 7-entry row is a single batch;
// with four resident blocks per SM (64 registers) that measured best on
// GB300 for the 7-point 128^3 system: CG step 71.4 us against 72.8 us with
// batches of four at five blocks per SM (SpMV 41.8 against 43.3 us), Jacobi
// 53.5 against 55.6 us, MR 62.8 against 64.7 us per step.
#ifndef CF_SELL_BATCH
#define CF_SELL_BATCH 8
#endif
// Resident blocks per SM the SpMV passes ask nvcc for (it sizes their
// register budget from it).  With batches of eight, 4, 5 and 6 measured
// within 0.6 us of one another per 128^3 CG step (71.2, 70.6, 71.0 us); at 5
// and 6 the MR passes spill.
#ifndef CF_SPMV_MIN_BLOCKS
#define CF_SPMV_MIN_BLOCKS 4
#endif
// the two-value BiCG passes
#ifndef CF_BICG_SPMV_MIN_BLOCKS
#define CF_BICG_SPMV_MIN_BLOCKS 4
#endif
constexpr int kSellBatch = CF_SELL_BATCH;
// the same for the FP32 passes of the mixed-precision inner solves: with
// eight a 7-entry row is one exact batch (all seven loads in flight), which
// measured best on GB300 for the 256^3 upwind MR inner solve (245 us per
// step against 280 us with four and 320 us with two) and the 128^3 CG one
#ifndef CF_SELL_BATCH32
#define CF_SELL_BATCH32 8
#endif
constexpr int kSellBatch32 = CF_SELL_BATCH32;


// (BATCH > 0 overrides the SELL batch of the value type for one kernel; the
// sums do not depend on it: every row is one FMA chain in entry order)
template <int FMT, class V, int BATCH = 0, class G, class F>
__device__ __forceinline__ void for_rows(const SolveArgs *a, const V *val, const V *sval, G g, F f)
{
    if constexpr (FMT == kSell) {
        constexpr int B = BATCH > 0 ? BATCH : (sizeof(V) == 4 ? kSellBatch32 : kSellBatch);
        sell_rows<V, B>(a->n, a->n_slices, a->s_off, SellCols32{a->s_col}, sval, a->ro, a->has_long != 0, g, f);
    } else if constexpr (FMT == kSellC) {
        constexpr int B = BATCH > 0 ? BATCH : (sizeof(V) == 4 ? kSellBatch32 : kSellBatch);
        sell_rows<V, B>(a->n, a->n_slices, a->s_off, SellCodes8(a->s_code, a->s_dtab), sval, a->ro,
                        a->has_long != 0, g, f);
    } else if constexpr (FMT == kSellD) {
        constexpr int B = BATCH > 0 ? BATCH : (sizeof(V) == 4 ? kSellBatch32 : kSellBatch);
        sell_rows<V, B>(a->n, a->n_slices, a->s_off, SellDelta16{a->s_d16}, sval, a->ro, a->has_long != 0, g, f);
    } else {
        const int n = a->n, cap = a->stage_cap;
        CF_STAGE(V, cap);
        CF_FOR_CHUNKS(base, n) {
            const Chunk<V> ch = stage_chunk<V>(a->ro, a->col, val, n, base, cap, sv_, sc_);
            const int row = base + (threadIdx.x & 31);
            const V y = row_chain<V>(ch, a->col, val, g);
            if (row < n) f(row, y);
            __syncwarp();
        }
    }
}

// The same for two value arrays on one pattern: f(row, y1, y2).
template <int FMT, class V, class G1, class G2, class F>
__device__ __forceinline__ void for_rows2(const SolveArgs *a, const V *val1, const V *val2, const V *sval1,
                                          const V *sval2, G1 g1, G2 g2, F f)
{
    if constexpr (FMT == kSell) {
        sell_rows2<V, 1>(a->n, a->n_slices, a->s_off, SellCols32{a->s_col}, sval1, sval2, a->ro, a->has_long != 0,
                         g1, g2, f);
    } else if constexpr (FMT == kSellC) {
        sell_rows2<V, 1>(a->n, a->n_slices, a->s_off, SellCodes8(a->s_code, a->s_dtab), sval1, sval2, a->ro,
                         a->has_long != 0, g1, g2, f);
    } else if constexpr (FMT == kSellD) {
        sell_rows2<V, 1>(a->n, a->n_slices, a->s_off, SellDelta16{a->s_d16}, sval1, sval2, a->ro,
                         a->has_long != 0, g1, g2, f);
    } else {
        const int n = a->n, cap = a->stage_cap;
        CF_STAGE(V, cap);
        CF_FOR_CHUNKS(base, n) {
            const Chunk<V> ch = stage_chunk<V>(a->ro, a->col, val1, n, base, cap, sv_, sc_);
            const int row = base + (threadIdx.x & 31);
            V y1, y2;
            row_chain2<V>(ch, a->col, val1, val2, g1, g2, y1, y2);
            if (row < n) f(row, y1, y2);
            __syncwarp();
        }
    }
}

// L2 prefetch of this warp's first slice in the format in use (nothing for
// CSR): sval is the value array the kernel streams.
template <int FMT, class V>
__device__ __forceinline__ void sell_prefetch(const SolveArgs *a, const V *sval)
{
    if constexpr (FMT == kSell) sell_prefetch_first(a->n_slices, a->s_off, SellCols32{a->s_col}, sval);
    if constexpr (FMT == kSellC) sell_prefetch_first(a->n_slices, a->s_off, SellCodes8(a->s_code, a->s_dtab), sval);
    if constexpr (FMT == kSellD) sell_prefetch_first(a->n_slices, a->s_off, SellDelta16{a->s_d16}, sval);
}

// ---------------------------------------------------------------------------
// Reference-order row products.  The reference's SpMV (kernels.h:206-237)
// lets lane l of 8 accumulate a row's entries l, l + 8, ... with FMA and
// adds the 8 lane sums in a fixed tree.  A SELL-32 copy keeps a row's t-th
// CSR entry in slot t, so the same sums read from SELL slots l, l + 8, ...
// of the row: the bits are the reference's, the loads coalesced and the
// loop free of per-row trip counts.  RefRow serves one chunk of 32 rows
// (base + lane) from the SELL copy when the solve has one (a->s_off set),
// else from the staged CSR chunk.
// ---------------------------------------------------------------------------
struct RefRow {
    const SolveArgs *a;
    bool sell;
    int off, len, rl;  // SELL: slice start, slots per row, this row's CSR length
    Chunk<double> ch;

    __device__ __forceinline__ RefRow(const SolveArgs *a_, int base, int cap, double *sv, int32_t *sc)
        : a(a_), sell(a_->s_off != nullptr)
    {
        const int n = a->n, row = base + (threadIdx.x & 31);
        if (sell) {
            const int s = base >> 5;
            off = __ldg(a->s_off + s);
            len = (__ldg(a->s_off + s + 1) - off) >> 5;
            rl = row < n ? __ldg(a->ro + row + 1) - __ldg(a->ro + row) : 0;
        } else {
            ch = stage_chunk<double>(a->ro, a->col, a->val, n, base, cap, sv, sc);
        }
    }

    template <class G>
    __device__ __forceinline__ double product(G g) const
    {
        if (!sell) return row_product<double>(ch, a->col, a->val, g);
        const int lane = threadIdx.x & 31;
        return sell_ref_row(a->s_col + off + lane, a->s_val + off + lane, len, rl, g);
    }

    // A and A^T values on the same pattern (row_product2)
    template <class G1, class G2>
    __device__ __forceinline__ void product2(G1 g1, G2 g2, double &y1, double &y2) const
    {
        if (!sell) {
            row_product2<double>(ch, a->col, a->val, a->valT, g1, g2, y1, y2);
            return;
        }
        const int lane = threadIdx.x & 31;
        const int32_t *cp = a->s_col + off + lane;
        const double *vp1 = a->s_val + off + lane;
        const double *vp2 = a->s_valT + off + lane;
        double t[8], u[8];
#pragma unroll
        for (int l = 0; l < 8; ++l) t[l] = u[l] = 0.0;
        for (int t0 = 0; t0 < len; t0 += 8) {
#pragma unroll
            for (int l = 0; l < 8; ++l) {
                const int slot = t0 + l;
                if (slot < rl) {
                    const int c = __ldg(cp + 32 * slot);
                    t[l] = fma_t(__ldg(vp1 + 32 * slot), g1(c), t[l]);
                    u[l] = fma_t(__ldg(vp2 + 32 * slot), g2(c), u[l]);
                }
            }
        }
        y1 = tree8(t);
        y2 = tree8(u);
    }
};

// ---------------------------------------------------------------------------
// loop bookkeeping (thread 0 of the last block)
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// history entry k: ||r|| and / or the device clock
static __device__ __forceinline__ void record_hist(const SolveArgs *a, const DevState *st, int k, double norm)
{
    if (k < st->hist_cap) {
        if (a->hist) a->hist[k] = norm;
        if (a->hist_t) a->hist_t[k] = global_ns();
    }
}

static __device__ __noinline__ void finish_init(const SolveArgs *a, DevState *st, double rr, bool bicg)
{
    const double norm0 = sqrt(rr);
    st->rho0 = rr;
    st->rho1 = 0.0;
    st->norm0 = norm0;
    st->norm = norm0;
    record_hist(a, st, 0, norm0);
    double tol = st->tol;
    if (st->rel_tol > 0.0) tol = fmax(tol, st->rel_tol * norm0);
    st->tol = tol;
    st->k = 0;
    st->x_pending = 0;
    st->body_count = 0;
    const bool finite = isfinite(norm0);
    bool cont = st->max_steps >= 1;
    if (!bicg) cont = cont && (norm0 > tol || st->min_steps > 0);
    if (!finite) cont = false;
    st->done = cont ? 0 : 1;
    st->status = !finite ? CF_NONFINITE : (norm0 > tol ? CF_NOT_CONVERGED : CF_OK);
}

// One step of a `while (k++ <= max_steps && norm_r > error)` / CG `for`
// loop: record ||r|| and decide whether another step runs.
static __device__ __noinline__ void finish_step(const SolveArgs *a, DevState *st, double norm)
{
    const int k = st->k + 1;
    st->k = k;
    st->norm = norm;
    record_hist(a, st, k, norm);
    const bool finite = isfinite(norm);
    bool cont = finite && k < st->max_steps && (norm > st->tol || k < st->min_steps);
    int status = !finite ? CF_NONFINITE : (norm > st->tol ? CF_NOT_CONVERGED : CF_OK);
    st->body_count += 1;
    if (st->body_count > k + 2 || (a->abort_flag && *a->abort_flag)) {
        cont = false;
        status = CF_TIMEOUT;
    }
    if (!cont) {
        st->done = 1;
        st->status = status;
    }
    set_loop_condition(a, cont);
}

// Prologue of every loop-body kernel: wait for the predecessor kernel
// (programmatic launches start early), then end the graph loop if the solve
// has already finished.
#define CF_EXIT_IF_DONE(a, st, is_last_kernel)                                  \
    pdl_wait();                                                                 \
    if (ld_cg(&(st)->done)) {                                                   \
        if ((is_last_kernel) && blockIdx.x == 0 && threadIdx.x == 0)            \
            set_loop_condition(a, false);                                       \
        return;                                                                 \
    }


// ---------------------------------------------------------------------------
// host-side launch helpers
// ---------------------------------------------------------------------------
struct Kernels {
    const void *k0 = nullptr;    // element-wise prep kernel (may be null)
    const void *k1 = nullptr;    // SpMV body kernel
    const void *k2 = nullptr;    // update body kernel (may be null)
    const void *k3 = nullptr;    // a fourth element-wise kernel (may be null)
    bool k1_spmv = false, k2_spmv = false;
    size_t value_bytes = sizeof(double);
};

struct Launch {
    int grid;
    size_t smem;
};

static Launch launch_cfg(Context *ctx, const void *kern, bool is_spmv, int cap, bool ref_order,
                         size_t value_bytes = sizeof(double))
{
    Launch l;
    l.smem = (is_spmv && cap > 0) ? kWarps * ((size_t)(cap + 8) * (value_bytes + sizeof(int32_t))) : 0;
    if (l.smem > 48 * 1024)
        CF_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)l.smem));
    l.grid = ref_order ? ctx->ref_grid : ctx->fast_grid(kern, l.smem);
    return l;
}

// pdl: launch with programmatic stream serialisation (the kernel must begin
// with pdl_wait(), as every loop-body kernel does through CF_EXIT_IF_DONE).
static void launch(Context *ctx, cudaStream_t s, const void *kern, const Launch &l, void **args,
                   bool pdl = false)
{
    (void)ctx;
    if (!pdl) {
        CF_CUDA(cudaLaunchKernel(kern, dim3(l.grid), dim3(kBlock), args, l.smem, s));
        return;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(l.grid);
    cfg.blockDim = dim3(kBlock);
    cfg.dynamicSmemBytes = l.smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    CF_CUDA(cudaLaunchKernelExC(&cfg, kern, args));
}

static void launch_body(Context *ctx, cudaStream_t s, const Kernels &kk, int cap, bool ref,
                        SolveArgs *d_args, bool pdl = false)
{
    void *args[] = {&d_args};
    if (kk.k0) launch(ctx, s, kk.k0, launch_cfg(ctx, kk.k0, false, cap, ref, kk.value_bytes), args, pdl);
    launch(ctx, s, kk.k1, launch_cfg(ctx, kk.k1, kk.k1_spmv, cap, ref, kk.value_bytes), args, pdl);
    if (kk.k2) launch(ctx, s, kk.k2, launch_cfg(ctx, kk.k2, kk.k2_spmv, cap, ref, kk.value_bytes), args, pdl);
    if (kk.k3) launch(ctx, s, kk.k3, launch_cfg(ctx, kk.k3, false, cap, ref, kk.value_bytes), args, pdl);
}

// Solver steps captured per pass of the device-driven loop (fewer
// evaluations of the conditional node; measured on GB300, 8 against 1: CG
// 19.2 -> 16.7 us per step at 64^2, 84.5 -> 81.6 at 128^3; Jacobi 65.4 ->
// 62.2 at 128^3).  A solve that converges mid-pass launches at most 7 steps
// of kernels that return at once.
#ifndef CF_LOOP_UNROLL
#define CF_LOOP_UNROLL 8
#endif

static bool build_loop_graph(Context *ctx, const Kernels &kk, int cap, bool ref, SolveArgs *d_args,
                             bool pdl, GraphEntry &ge)
{
    cudaStream_t cs = nullptr;
    try {
        CF_CUDA(cudaGraphCreate(&ge.graph, 0));
        cudaGraphConditionalHandle h = 0;
        CF_CUDA(cudaGraphConditionalHandleCreate(&h, ge.graph, 1, cudaGraphCondAssignDefault));
        ge.cond = (unsigned long long)h;
        cudaGraphNodeParams cp = {};
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = h;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        cudaGraphNode_t node;
        CF_CUDA(cudaGraphAddNode(&node, ge.graph, nullptr, nullptr, 0, &cp));
        cudaGraph_t body = cp.conditional.phGraph_out[0];
        CF_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
        CF_CUDA(cudaStreamBeginCaptureToGraph(cs, body, nullptr, nullptr, 0,
                                              cudaStreamCaptureModeThreadLocal));
        // CF_LOOP_UNROLL steps per evaluation of the loop condition: the
        // kernels of steps past convergence return at once (CF_EXIT_IF_DONE)
        for (int u = 0; u < CF_LOOP_UNROLL; ++u) launch_body(ctx, cs, kk, cap, ref, d_args, pdl);
        cudaGraph_t out = nullptr;
        CF_CUDA(cudaStreamEndCapture(cs, &out));
        CF_CUDA(cudaStreamDestroy(cs));
        cs = nullptr;
        CF_CUDA(cudaGraphInstantiate(&ge.exec, ge.graph, 0));
        ge.pdl = pdl;
        return true;
    } catch (const Error &) {
        if (cs) {
            cudaGraph_t junk = nullptr;
            cudaStreamEndCapture(cs, &junk);
            cudaStreamDestroy(cs);
        }
        if (ge.exec) cudaGraphExecDestroy(ge.exec);
        if (ge.graph) cudaGraphDestroy(ge.graph);
        ge = GraphEntry();
        cudaGetLastError();
        return false;
    }
}

// The device-driven loop of one solver configuration, built once per
// context: with programmatic launches between the body kernels where the
// driver accepts them in a conditional body, else without.
// Loop-body kernels launched with programmatic dependent launch inside the
// loop graphs (1), or as plain serialised launches (0).
#ifndef CF_LOOP_PDL
#define CF_LOOP_PDL 1
#endif

static GraphEntry *loop_graph(Context *ctx, const Kernels &kk, int solver, int precision, int cap,
                              bool ref, SolveArgs *d_args, int format = 0)
{
    GraphKey key{solver, precision, ref ? 1 : 0, cap, 0, format, ref ? 0 : ctx->grid_cap};
    auto it = ctx->graphs.find(key);
    if (it != ctx->graphs.end()) return &it->second;
    GraphEntry ge;
    if (!(CF_LOOP_PDL && ctx->pdl_ok && build_loop_graph(ctx, kk, cap, ref, d_args, true, ge))) {
        if (CF_LOOP_PDL) ctx->pdl_ok = false; // a programmatic launch failed to capture
        if (!build_loop_graph(ctx, kk, cap, ref, d_args, false, ge))
            throw Error{CF_CUDA_ERROR, "cannot build the solver loop graph"};
    }
    return &(ctx->graphs[key] = ge);
}

// format: kCsr, kSell, kSellC or kSellD (solve_format)
Kernels fast_body_kernels(int solver, int format);

// The format of a solve's fast kernels from its arguments: CSR (no SELL-32
// copy), SELL-32 with 32-bit columns, with one-byte column codes, or with
// 16-bit column deltas.
inline int solve_format(const SolveArgs &A)
{
    return A.n_slices == 0 ? kCsr : A.s_code ? kSellC : A.s_d16 ? kSellD : kSell;
}
const void *fast_flush_kernel();

// ---------------------------------------------------------------------------
// The diagonally preconditioned MR solvers as MR on a scaled matrix.
// MRJacobi's and MRS's step (y = A D^-1 r, alpha = (r, y)/(y, y),
// x += alpha D^-1 r, r -= alpha y) is MR on A D^-1; JMR's (y = D^-1/2 A
// D^-1/2 r on the scaled residual r = D^-1/2 (b - A x), x += alpha D^-1/2
// r) is MR on D^-1/2 A D^-1/2.  The scaled values take the place of the
// preconditioned vector: a step is MR's two passes, with R r formed in the
// x update.
// ---------------------------------------------------------------------------
// values of L A R (L, R diagonal, L = null: the identity) on A's pattern,
// over the SELL-32 slots (padding stays 0) ...
template <class T>
__global__ void __launch_bounds__(kBlock) k_scaled_sell(int n, int n_slices, const int32_t *__restrict__ soff,
                                                        const int32_t *__restrict__ scol,
                                                        const double *__restrict__ sval,
                                                        const double *__restrict__ L,
                                                        const double *__restrict__ R, T *__restrict__ out)
{
    CF_FOR_ELEMS(i, 32 * n_slices) {
        const int sl = i >> 5, lane = i & 31;
        const int b = soff[sl], len = (soff[sl + 1] - b) >> 5;
        const double li = (L && i < n) ? L[i] : 1.0;
        for (int t = 0; t < len; ++t) {
            const int o = b + 32 * t + lane;
            const double v = sval[o];
            out[o] = v == 0.0 ? T(0) : (T)(li * v * R[scol[o]]);
        }
    }
}

// ... or over the CSR entries
template <class T>
__global__ void __launch_bounds__(kBlock) k_scaled_csr(int n, const int32_t *__restrict__ ro,
                                                       const int32_t *__restrict__ col,
                                                       const double *__restrict__ val,
                                                       const double *__restrict__ L,
                                                       const double *__restrict__ R, T *__restrict__ out)
{
    CF_FOR_ELEMS(i, n) {
        const double li = L ? L[i] : 1.0;
        for (int j = ro[i]; j < ro[i + 1]; ++j) out[j] = (T)(li * val[j] * R[col[j]]);
    }
}

inline bool mr_scaled_solver(int solver) { return solver == CF_MRJACOBI || solver == CF_MRS || solver == CF_JMR; }

// L A R of the solved matrix in the layout in use (A.val / A.s_val point at
// A^T's values for a transposed solve): D^-1/2 A D^-1/2 for JMR, A D^-1 for
// the others (MRJacobi, MRS; the FP64 fast-order Jacobi step too); R is
// returned in *R_out.  Kept on the matrix until its values change.
template <class T>
static const T *scaled_values(Context *ctx, Matrix *m, const SolveArgs &A, int solver, bool transpose,
                              ScaledCopy &sc, const double **R_out)
{
    const double *L = solver == CF_JMR ? A.dinv_sqrt : nullptr;
    const double *R = solver == CF_JMR ? A.dinv_sqrt : A.dinv;
    *R_out = R;
    const int scale = solver == CF_JMR ? 2 : 1;
    const int sell = A.n_slices > 0 ? 1 : 0;
    const int tr = transpose ? 1 : 0;
    if (sc.gen == m->gen && sc.scale == scale && sc.transpose == tr && sc.sell == sell) return sc.buf.as<T>();
    sc.gen = 0;
    const Launch l = launch_cfg(ctx, sell ? (const void *)k_scaled_sell<T> : (const void *)k_scaled_csr<T>,
                                false, 0, false);
    if (sell) {
        sc.buf.ensure(sizeof(T) * ((size_t)m->sell_nnz + 32));
        k_scaled_sell<T><<<l.grid, kBlock, 0, ctx->stream>>>(m->n, A.n_slices, A.s_off, A.s_col, A.s_val, L, R,
                                                             sc.buf.as<T>());
    } else {
        sc.buf.ensure(sizeof(T) * ((size_t)m->nnz + 4));
        CF_CUDA(cudaMemsetAsync(sc.buf.as<T>() + m->nnz, 0, sizeof(T) * 4, ctx->stream));
        k_scaled_csr<T><<<l.grid, kBlock, 0, ctx->stream>>>(m->n, A.ro, A.col, A.val, L, R, sc.buf.as<T>());
    }
    CF_CUDA(cudaGetLastError());
    sc.gen = m->gen;
    sc.scale = scale;
    sc.transpose = tr;
    sc.sell = sell;
    return sc.buf.as<T>();
}

} // namespace cf
