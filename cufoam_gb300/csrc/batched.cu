// batched.cu -- many independent LDU systems, each with R right-hand sides
// (the Ux/Uy/Uz components that share one matrix), solved by CG in ONE
// persistent kernel launch (captured in a CUDA graph).
//
// Schedule: the grid is one wave of thread-block clusters of CS CTAs.  A
// cluster takes the next system from a global work queue (systems ordered
// largest first), splits its rows over its CTAs, and runs the whole solve
// for all R right-hand sides at once: every matrix entry is read once per
// iteration for R vectors (R-wide SpMM), vectors are stored row-major with
// the R components adjacent.  The two dot products per CG step are reduced
// inside each CTA and then across the cluster through distributed shared
// memory, after a hardware cluster barrier; every CTA sums the per-CTA
// partials in rank order, so all CTAs reach bit-identical scalars and take
// identical control flow.  Each right-hand side keeps its own CG scalars and
// stopping test (the reference's loop, SolverSingleGPU.h:366-445, with its
// normFactor, gis/gis.cu:106-123); a converged component is frozen.
//
// Mixed precision (k_batch_cg<R, BT, true>): after the FP64 normFactor and
// residual, each refinement sweep solves A e = r / ||r|| by CG with FP32
// values, FP32 vectors and FP32 per-thread sums (combined across CTAs in
// FP64) to a relative inner tolerance, then adds ||r|| e to x and forms the
// FP64 residual b - A x again; the FP64 tolerance decides convergence.
#include <cooperative_groups.h>

#include "device.cuh"

#include <algorithm>
#include <climits>
#include <cmath>
#include <numeric>

namespace cgp = cooperative_groups;

namespace cf {

constexpr int kBatchMaxR = 4;

struct BatchSystem {
    int32_t n;
    int32_t pad;
    int64_t vec_offset;      // first row of this system in the batch vectors
    const int32_t *ro;
    const int32_t *col;
    const double *val;
    const float *val32;      // FP32 copy (mixed precision)
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
    double *r, *p0, *p1, *q; // [rows][R] work
    int32_t *queue;          // next position in `order`
    BatchResult *out;        // [n_systems][R]
    // mixed precision: FP32 inner CG on A32 e = r / ||r||, FP64 refinement
    float *r32, *p32a, *p32b, *q32, *e32;   // [rows][R]
    double inner_rtol;
    int32_t max_outer;
};

// sum over the block (fixed order), then over the cluster in rank order
template <int NV, int BT>
__device__ __forceinline__ void cluster_sum(cgp::cluster_group &cl, double (&v)[NV],
                                            double *wsm /*[NV][BT/32]*/, double *slot /*[NV]*/,
                                            double *out /*[NV]*/)
{
    constexpr int W = BT / 32;
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
    if (threadIdx.x < NV) {
        double s = 0.0;
        for (int w = 0; w < W; ++w) s += wsm[threadIdx.x * W + w];
        slot[threadIdx.x] = s;
    }
    cl.sync(); // every CTA's slot is written and visible cluster-wide
    if (threadIdx.x < NV) {
        double s = 0.0;
        const int cs = (int)cl.num_blocks();
        for (int rk = 0; rk < cs; ++rk) s += cl.map_shared_rank(slot, rk)[threadIdx.x];
        out[threadIdx.x] = s;
    }
    __syncthreads();
}

// FP64 residual r = b - A x and ||r||^2 per component over this CTA's rows,
// summed over the cluster into tot[0..R)
template <int R, int BT>
__device__ __forceinline__ void batch_residual(cgp::cluster_group &cl, int lo, int hi, const int32_t *ro,
                                               const int32_t *col, const double *val, const double *b,
                                               const double *x, double *r, double *wsm, double *slot,
                                               double *tot)
{
    double acc[R];
#pragma unroll
    for (int j = 0; j < R; ++j) acc[j] = 0.0;
    for (int i = lo + threadIdx.x; i < hi; i += BT) {
        double y[R];
#pragma unroll
        for (int j = 0; j < R; ++j) y[j] = 0.0;
        for (int e = ro[i]; e < ro[i + 1]; ++e) {
            const double v = val[e];
            const int64_t c = (int64_t)col[e] * R;
#pragma unroll
            for (int j = 0; j < R; ++j) y[j] = fma_t(v, __ldcg(x + c + j), y[j]);
        }
#pragma unroll
        for (int j = 0; j < R; ++j) {
            const double ri = b[(int64_t)i * R + j] - y[j];
            r[(int64_t)i * R + j] = ri;
            acc[j] = fma_t(ri, ri, acc[j]);
        }
    }
    cluster_sum<R, BT>(cl, acc, wsm, slot, tot);
}

template <int R, int BT, bool MIXED>
__global__ void __launch_bounds__(BT) k_batch_cg(const BatchArgs a)
{
    cgp::cluster_group cl = cgp::this_cluster();
    const int cs = (int)cl.num_blocks();
    const int rank = (int)cl.block_rank();
    constexpr int W = BT / 32;
    __shared__ double wsm[3 * R * W];
    __shared__ double slot[2][3 * R]; // double-buffered cluster slots
    __shared__ double tot[3 * R];
    __shared__ int32_t s_next;
    int parity = 0;

    for (;;) {
        if (rank == 0 && threadIdx.x == 0) s_next = atomicAdd(a.queue, 1);
        cl.sync();
        const int pos = *cl.map_shared_rank(&s_next, 0);
        cl.sync();
        if (pos >= a.n_systems) break;
        const int sid = a.order[pos];
        const BatchSystem S = a.sys[sid];
        const int n = S.n;
        const int lo = (int)((int64_t)n * rank / cs), hi = (int)((int64_t)n * (rank + 1) / cs);
        const double *b = a.b + S.vec_offset * R;
        double *x = a.x + S.vec_offset * R;
        double *r = a.r + S.vec_offset * R;
        double *q = a.q + S.vec_offset * R;
        double *pb[2] = {a.p0 + S.vec_offset * R, a.p1 + S.vec_offset * R};
        const int32_t *ro = S.ro, *col = S.col;
        const double *val = S.val;

        // ---- normFactor part 1: mean of psi per component ----------------
        double acc1[R];
#pragma unroll
        for (int j = 0; j < R; ++j) acc1[j] = 0.0;
        for (int i = lo + threadIdx.x; i < hi; i += BT)
#pragma unroll
            for (int j = 0; j < R; ++j) acc1[j] += x[(int64_t)i * R + j];
        cluster_sum<R, BT>(cl, acc1, wsm, slot[parity], tot);
        parity ^= 1;
        double xbar[R];
#pragma unroll
        for (int j = 0; j < R; ++j) xbar[j] = tot[j] / n;
        __syncthreads();

        // ---- normFactor part 2 + initial residual r = b - A x ------------
        double acc3[3 * R];
#pragma unroll
        for (int j = 0; j < 3 * R; ++j) acc3[j] = 0.0;
        for (int i = lo + threadIdx.x; i < hi; i += BT) {
            double y[R], ys = 0.0;
#pragma unroll
            for (int j = 0; j < R; ++j) y[j] = 0.0;
            for (int e = ro[i]; e < ro[i + 1]; ++e) {
                const double v = val[e];
                const int64_t c = (int64_t)col[e] * R;
#pragma unroll
                for (int j = 0; j < R; ++j) y[j] = fma_t(v, __ldcg(x + c + j), y[j]);
                ys += v;
            }
#pragma unroll
            for (int j = 0; j < R; ++j) {
                const double yb = ys * xbar[j];
                const double bi = b[(int64_t)i * R + j];
                const double d1 = y[j] - yb, d2 = bi - yb, ri = bi - y[j];
                r[(int64_t)i * R + j] = ri;
                acc3[j] = fma_t(d1, d1, acc3[j]);
                acc3[R + j] = fma_t(d2, d2, acc3[R + j]);
                acc3[2 * R + j] = fma_t(ri, ri, acc3[2 * R + j]);
            }
        }
        cluster_sum<3 * R, BT>(cl, acc3, wsm, slot[parity], tot);
        parity ^= 1;
        double tolj[R], rho0[R], rho1[R], nrm[R], nf[R];
        bool active[R];
        int iters[R];
        bool any = false;
#pragma unroll
        for (int j = 0; j < R; ++j) {
            nf[j] = sqrt(tot[j]) + sqrt(tot[R + j]) + 1e-20;
            tolj[j] = a.tolerance * nf[j];
            rho0[j] = tot[2 * R + j];
            rho1[j] = 0.0;
            nrm[j] = sqrt(rho0[j]);
            active[j] = isfinite(nrm[j]) && nrm[j] > tolj[j] && a.max_iter >= 1;
            iters[j] = 0;
            any = any || active[j];
        }
        __syncthreads();
        if (rank == 0 && threadIdx.x < R) {
            const int j = threadIdx.x;
            a.out[(int64_t)sid * R + j].nf = nf[j];
            a.out[(int64_t)sid * R + j].norm0 = nrm[j];
        }

        // ---- mixed precision: FP32 CG sweeps inside FP64 refinement -----
        if constexpr (MIXED) {
            float *r32 = a.r32 + S.vec_offset * R;
            float *e32 = a.e32 + S.vec_offset * R;
            float *q32 = a.q32 + S.vec_offset * R;
            float *pb32[2] = {a.p32a + S.vec_offset * R, a.p32b + S.vec_offset * R};
            const float *val32 = S.val32;
            for (int sweep = 0; any && sweep < a.max_outer; ++sweep) {
                // inner right-hand side r / ||r||, e = 0
                float inv[R], eta[R];
                bool act[R];
                bool any_in = false;
#pragma unroll
                for (int j = 0; j < R; ++j) {
                    act[j] = active[j];
                    inv[j] = active[j] ? (float)(1.0 / nrm[j]) : 0.f;
                    // the last sweep only has to reach the FP64 target
                    eta[j] = (float)fmax(a.inner_rtol, fmin(0.5, 0.8 * tolj[j] / nrm[j]));
                    any_in = any_in || act[j];
                }
                double acc0[R];
#pragma unroll
                for (int j = 0; j < R; ++j) acc0[j] = 0.0;
                for (int i = lo + threadIdx.x; i < hi; i += BT)
#pragma unroll
                    for (int j = 0; j < R; ++j) {
                        const int64_t o = (int64_t)i * R + j;
                        const float v = (float)(r[o] * (double)inv[j]);
                        r32[o] = v;
                        e32[o] = 0.f;
                        acc0[j] += (double)(v * v);
                    }
                cluster_sum<R, BT>(cl, acc0, wsm, slot[parity], tot);
                parity ^= 1;
                float rho0f[R], rho1f[R];
#pragma unroll
                for (int j = 0; j < R; ++j) {
                    rho0f[j] = (float)tot[j];
                    rho1f[j] = 0.f;
                }
                __syncthreads();
                int kin = 0;
                for (int k = 1; any_in; ++k) {
                    const float *pin = pb32[(k + 1) & 1];
                    float *pout = pb32[k & 1];
                    float beta[R];
#pragma unroll
                    for (int j = 0; j < R; ++j) beta[j] = (k > 1) ? rho0f[j] / rho1f[j] : 0.f;
                    double acc[R];
#pragma unroll
                    for (int j = 0; j < R; ++j) acc[j] = 0.0;
                    for (int i = lo + threadIdx.x; i < hi; i += BT) {
                        float y[R], part[R];
#pragma unroll
                        for (int j = 0; j < R; ++j) y[j] = 0.f;
                        for (int e = ro[i]; e < ro[i + 1]; ++e) {
                            const float v = val32[e];
                            const int64_t c = (int64_t)col[e] * R;
#pragma unroll
                            for (int j = 0; j < R; ++j) {
                                const float pc = (k > 1) ? fma_t(beta[j], __ldcg(pin + c + j), __ldcg(r32 + c + j))
                                                         : __ldcg(r32 + c + j);
                                y[j] = fma_t(v, act[j] ? pc : 0.f, y[j]);
                            }
                        }
#pragma unroll
                        for (int j = 0; j < R; ++j) {
                            const int64_t o = (int64_t)i * R + j;
                            const float pi = (k > 1) ? fma_t(beta[j], __ldcg(pin + o), __ldcg(r32 + o))
                                                     : __ldcg(r32 + o);
                            pout[o] = act[j] ? pi : __ldcg(pin + o);
                            q32[o] = y[j];
                            part[j] = pi * y[j];
                            acc[j] += (double)part[j];
                        }
                    }
                    cluster_sum<R, BT>(cl, acc, wsm, slot[parity], tot);
                    parity ^= 1;
                    float xi[R];
#pragma unroll
                    for (int j = 0; j < R; ++j) xi[j] = act[j] ? rho0f[j] / (float)tot[j] : 0.f;
                    __syncthreads();
                    double acc2[R];
#pragma unroll
                    for (int j = 0; j < R; ++j) acc2[j] = 0.0;
                    for (int i = lo + threadIdx.x; i < hi; i += BT) {
#pragma unroll
                        for (int j = 0; j < R; ++j) {
                            const int64_t o = (int64_t)i * R + j;
                            if (act[j]) {
                                e32[o] = fma_t(xi[j], pout[o], e32[o]);
                                const float ri = fma_t(-xi[j], q32[o], r32[o]);
                                r32[o] = ri;
                                acc2[j] += (double)(ri * ri);
                            }
                        }
                    }
                    cluster_sum<R, BT>(cl, acc2, wsm, slot[parity], tot);
                    parity ^= 1;
                    any_in = false;
#pragma unroll
                    for (int j = 0; j < R; ++j) {
                        if (act[j]) {
                            rho1f[j] = rho0f[j];
                            rho0f[j] = (float)tot[j];
                            iters[j] += 1;
                            const float nin = sqrtf(rho0f[j]);
                            act[j] = isfinite(nin) && nin > eta[j] && iters[j] < a.max_iter;
                        }
                        any_in = any_in || act[j];
                    }
                    kin = k;
                    __syncthreads();
                }
                (void)kin;
                // x += ||r|| e in FP64, then the FP64 residual
                for (int i = lo + threadIdx.x; i < hi; i += BT)
#pragma unroll
                    for (int j = 0; j < R; ++j) {
                        const int64_t o = (int64_t)i * R + j;
                        if (active[j]) x[o] = fma_t(nrm[j], (double)e32[o], x[o]);
                    }
                cl.sync(); // every CTA's x rows are written before anyone gathers them
                batch_residual<R, BT>(cl, lo, hi, ro, col, val, b, x, r, wsm, slot[parity], tot);
                parity ^= 1;
                any = false;
#pragma unroll
                for (int j = 0; j < R; ++j) {
                    if (active[j]) {
                        const double nn = sqrt(tot[j]);
                        // a sweep that does not reduce the FP64 residual ends the solve
                        const bool progress = nn < nrm[j];
                        nrm[j] = nn;
                        active[j] = isfinite(nn) && nn > tolj[j] && progress && iters[j] < a.max_iter;
                    }
                    any = any || active[j];
                }
                __syncthreads();
            }
        } else {
            // ---- CG iterations, all components together ----------------------
            for (int k = 1; any && k <= a.max_iter; ++k) {
                const double *pin = pb[(k + 1) & 1];
                double *pout = pb[k & 1];
                double beta[R];
    #pragma unroll
                for (int j = 0; j < R; ++j) beta[j] = (k > 1) ? rho0[j] / rho1[j] : 0.0;
                // phase A: p = r + beta p_old (on the fly), q = A p, (p, q)
                double acc[R];
    #pragma unroll
                for (int j = 0; j < R; ++j) acc[j] = 0.0;
                for (int i = lo + threadIdx.x; i < hi; i += BT) {
                    double y[R];
    #pragma unroll
                    for (int j = 0; j < R; ++j) y[j] = 0.0;
                    for (int e = ro[i]; e < ro[i + 1]; ++e) {
                        const double v = val[e];
                        const int64_t c = (int64_t)col[e] * R;
    #pragma unroll
                        for (int j = 0; j < R; ++j) {
                            const double pc = (k > 1) ? fma_t(beta[j], __ldcg(pin + c + j), __ldcg(r + c + j))
                                                      : __ldcg(r + c + j);
                            y[j] = fma_t(v, active[j] ? pc : 0.0, y[j]);
                        }
                    }
    #pragma unroll
                    for (int j = 0; j < R; ++j) {
                        const int64_t o = (int64_t)i * R + j;
                        const double pi = (k > 1) ? fma_t(beta[j], __ldcg(pin + o), __ldcg(r + o)) : __ldcg(r + o);
                        pout[o] = active[j] ? pi : __ldcg(pin + o);
                        q[o] = y[j];
                        acc[j] = fma_t(pi, y[j], acc[j]);
                    }
                }
                cluster_sum<R, BT>(cl, acc, wsm, slot[parity], tot);
                parity ^= 1;
                double xi[R];
    #pragma unroll
                for (int j = 0; j < R; ++j) xi[j] = active[j] ? rho0[j] / tot[j] : 0.0;
                __syncthreads();
                // phase B: x += xi p, r -= xi q, (r, r)
                double acc2[R];
    #pragma unroll
                for (int j = 0; j < R; ++j) acc2[j] = 0.0;
                for (int i = lo + threadIdx.x; i < hi; i += BT) {
    #pragma unroll
                    for (int j = 0; j < R; ++j) {
                        const int64_t o = (int64_t)i * R + j;
                        if (active[j]) {
                            x[o] = fma_t(xi[j], pout[o], x[o]);
                            const double ri = fma_t(-xi[j], q[o], r[o]);
                            r[o] = ri;
                            acc2[j] = fma_t(ri, ri, acc2[j]);
                        }
                    }
                }
                cluster_sum<R, BT>(cl, acc2, wsm, slot[parity], tot);
                parity ^= 1;
                any = false;
    #pragma unroll
                for (int j = 0; j < R; ++j) {
                    if (active[j]) {
                        rho1[j] = rho0[j];
                        rho0[j] = tot[j];
                        nrm[j] = sqrt(rho0[j]);
                        iters[j] = k;
                        active[j] = isfinite(nrm[j]) && k < a.max_iter && nrm[j] > tolj[j];
                    }
                    any = any || active[j];
                }
                __syncthreads();
            }
        }
        if (rank == 0 && threadIdx.x < R) {
            const int j = threadIdx.x;
            BatchResult &o = a.out[(int64_t)sid * R + j];
            o.norm = nrm[j];
            o.iters = iters[j];
            o.status = !isfinite(nrm[j]) ? CF_NONFINITE : (nrm[j] > tolj[j] ? CF_NOT_CONVERGED : CF_OK);
        }
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
    DeviceBuffer d_sys, d_order, d_queue, d_out, d_b, d_x, d_r, d_p0, d_p1, d_q;
    DeviceBuffer d_r32, d_p32a, d_p32b, d_q32, d_e32;
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
    attr[0].val.clusterDim.x = cs;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.blockDim = dim3(BT);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int nclusters = 0;
    cfg.gridDim = dim3(cs);
    CF_CUDA(cudaOccupancyMaxActiveClusters(&nclusters, (void *)k_batch_cg<R, BT, MIXED>, &cfg));
    if (nclusters < 1) nclusters = 1;
    if (max_clusters > 0 && nclusters > max_clusters) nclusters = max_clusters;
    cfg.gridDim = dim3(nclusters * cs);
    CF_CUDA(cudaLaunchKernelEx(&cfg, k_batch_cg<R, BT, MIXED>, args));
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
            matrix_ensure_fp32(B->mats[s2], false);
            hs[s2].val32 = B->mats[s2]->val32.as<float>();
        }
        CF_CUDA(cudaMemcpyAsync(B->d_sys.ptr, hs.data(), sizeof(BatchSystem) * S, cudaMemcpyHostToDevice,
                                ctx->stream));
        CF_CUDA(cudaStreamSynchronize(ctx->stream));
        B->have_32 = true;
    }
    if (mixed) {
        const size_t fb = sizeof(float) * (size_t)(B->rows * nrhs + 8);
        B->d_r32.ensure(fb);
        B->d_p32a.ensure(fb);
        B->d_p32b.ensure(fb);
        B->d_q32.ensure(fb);
        B->d_e32.ensure(fb);
    }
    const size_t vb = sizeof(double) * (size_t)(B->rows * nrhs + 8);
    B->d_r.ensure(vb);
    B->d_p0.ensure(vb);
    B->d_p1.ensure(vb);
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
    a.p0 = B->d_p0.as<double>();
    a.p1 = B->d_p1.as<double>();
    a.q = B->d_q.as<double>();
    a.queue = B->d_queue.as<int32_t>();
    a.out = B->d_out.as<BatchResult>();
    a.r32 = mixed ? B->d_r32.as<float>() : nullptr;
    a.p32a = mixed ? B->d_p32a.as<float>() : nullptr;
    a.p32b = mixed ? B->d_p32b.as<float>() : nullptr;
    a.q32 = mixed ? B->d_q32.as<float>() : nullptr;
    a.e32 = mixed ? B->d_e32.as<float>() : nullptr;
    a.inner_rtol = (c.mixed_inner_rtol > 0 && c.mixed_inner_rtol < 1) ? c.mixed_inner_rtol : 1e-4;
    a.max_outer = c.mixed_max_outer > 0 ? c.mixed_max_outer : 50;
    const int cs = cfg && cfg->cluster_size > 0 ? cfg->cluster_size : 4;
    const int bt = cfg && cfg->threads > 0 ? cfg->threads : 256;
    const int maxc = cfg ? cfg->max_clusters : 0;
    require(cs == 1 || cs == 2 || cs == 4 || cs == 8, CF_BAD_INPUT, "cluster size must be 1, 2, 4 or 8");
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

int64_t batch_rows(const Batch *B) { return B->rows; }
int batch_systems(const Batch *B) { return (int)B->mats.size(); }
int64_t batch_offset(const Batch *B, int s) { return B->offsets[s]; }

} // namespace cf
