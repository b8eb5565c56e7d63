// capi.cu -- the extern "C" boundary (include/cufoam_gb300.h): argument
// checks, exception-to-status translation, context and buffer management.
#include "internal.h"

#include <cstdio>
#include <cstring>
#include <new>
#include <set>

struct cf_matrix;
struct cf_batch;

// A context owns the device memory of the matrices and batches made on it:
// cf_context_destroy releases it and leaves their handles orphaned (owner
// null), so that a later cf_matrix_destroy / cf_batch_destroy -- in any
// order, e.g. from a garbage collector -- only frees the handle.
struct cf_context {
    cf::Context *impl;
    std::set<cf_matrix *> matrices;
    std::set<cf_batch *> batches;
};

struct cf_matrix {
    cf::Matrix *impl;
    cf_context *owner;
};

struct cf_batch {
    cf::Batch *impl;
    cf_context *owner;
};

namespace cf {

[[noreturn]] void throw_cuda(cudaError_t e, const char *what, const char *file, int line)
{
    char buf[512];
    std::snprintf(buf, sizeof(buf), "%s failed: %s (%s:%d)", what, cudaGetErrorString(e), file, line);
    cudaGetLastError(); // clear a sticky launch error where possible
    throw Error{e == cudaErrorMemoryAllocation ? CF_OUT_OF_MEMORY
                : (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) ? CF_NO_DEVICE
                                                                               : CF_CUDA_ERROR,
                buf};
}

void DeviceBuffer::ensure(size_t nbytes)
{
    if (nbytes <= bytes && ptr) return;
    release();
    if (nbytes == 0) nbytes = 16;
    CF_CUDA(cudaMalloc(&ptr, nbytes));
    bytes = nbytes;
}

void DeviceBuffer::release()
{
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
}

int Context::fast_grid(const void *kernel, size_t dyn_smem) const
{
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kBlock, dyn_smem) != cudaSuccess ||
        per_sm < 1) {
        cudaGetLastError();
        per_sm = 1;
    }
    int g = per_sm * sm_count;
    const int cap = sm_count * 8;
    if (g > cap) g = cap;
    return (grid_cap > 0 && g > grid_cap) ? grid_cap : g;
}

Context::~Context()
{
    cudaSetDevice(device);
    delete ldu_scratch;
    for (auto &kv : graphs) {
        if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
        if (kv.second.graph) cudaGraphDestroy(kv.second.graph);
    }
    if (h_args) cudaFreeHost(h_args);
    if (h_state) cudaFreeHost(h_state);
    if (h_state_in) cudaFreeHost(h_state_in);
    if (h_abort) cudaFreeHost(h_abort);
    if (ev_start) cudaEventDestroy(ev_start);
    if (ev_stop) cudaEventDestroy(ev_stop);
    if (ev_mid) cudaEventDestroy(ev_mid);
    for (cudaEvent_t e : prof_events) cudaEventDestroy(e);
    if (stream && own_stream) cudaStreamDestroy(stream);
}

Context *context_create(int device)
{
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        cudaGetLastError();
        throw Error{CF_NO_DEVICE, "no CUDA device available"};
    }
    require(device >= 0 && device < count, CF_BAD_INPUT, "device index out of range");
    CF_CUDA(cudaSetDevice(device));
    Context *ctx = new Context();
    try {
        ctx->device = device;
        CF_CUDA(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
        ctx->own_stream = true;
        CF_CUDA(cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device));
        CF_CUDA(cudaDeviceGetAttribute(&ctx->max_threads_sm, cudaDevAttrMaxThreadsPerMultiProcessor, device));
        int l2 = 0;
        CF_CUDA(cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, device));
        ctx->l2_bytes = (size_t)l2;
        // the reference's LaunchConfig (gis/SparseSystem/launch.h:116-139)
        ctx->ref_grid = ctx->max_threads_sm / kBlock * ctx->sm_count;
        ctx->state.ensure(sizeof(DevState));
        ctx->args.ensure(sizeof(SolveArgs));
        CF_CUDA(cudaMemset(ctx->state.ptr, 0, sizeof(DevState)));
        CF_CUDA(cudaHostAlloc((void **)&ctx->h_args, sizeof(SolveArgs), cudaHostAllocDefault));
        CF_CUDA(cudaHostAlloc((void **)&ctx->h_state, sizeof(DevState), cudaHostAllocDefault));
        CF_CUDA(cudaHostAlloc((void **)&ctx->h_state_in, sizeof(DevState), cudaHostAllocDefault));
        CF_CUDA(cudaHostAlloc((void **)&ctx->h_abort, sizeof(int32_t), cudaHostAllocMapped));
        *ctx->h_abort = 0;
        CF_CUDA(cudaHostGetDevicePointer((void **)&ctx->d_abort, ctx->h_abort, 0));
        CF_CUDA(cudaEventCreate(&ctx->ev_start));
        CF_CUDA(cudaEventCreate(&ctx->ev_stop));
        CF_CUDA(cudaEventCreate(&ctx->ev_mid));
    } catch (...) {
        delete ctx;
        throw;
    }
    return ctx;
}

void context_bind(Context *ctx) { CF_CUDA(cudaSetDevice(ctx->device)); }

void upload(Context *ctx, void *dst, const void *src, size_t bytes, int memory)
{
    if (bytes == 0) return;
    CF_CUDA(cudaMemcpyAsync(dst, src, bytes,
                            memory == CF_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice,
                            ctx->stream));
}

void download(Context *ctx, void *dst, const void *src, size_t bytes, int memory)
{
    if (bytes == 0) return;
    CF_CUDA(cudaMemcpyAsync(dst, src, bytes,
                            memory == CF_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice,
                            ctx->stream));
}

double norm_factor(Matrix *m, const double *b, const double *x, int norm_type, bool ref_order);

} // namespace cf

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
using cf::Error;

template <class F>
static cf_status guarded(cf_context *ctx, F f)
{
    try {
        if (ctx) {
            ctx->impl->last_error.clear();
            cf::context_bind(ctx->impl);
        }
        f();
        return CF_OK;
    } catch (const Error &e) {
        if (ctx) ctx->impl->last_error = e.msg;
        return e.status;
    } catch (const std::bad_alloc &) {
        if (ctx) ctx->impl->last_error = "host allocation failed";
        return CF_OUT_OF_MEMORY;
    } catch (...) {
        if (ctx) ctx->impl->last_error = "unexpected internal error";
        return CF_CUDA_ERROR;
    }
}

// file calls have no context: their errors go to a per-thread message
static thread_local std::string g_file_error;

template <class F>
static cf_status file_guarded(F f)
{
    try {
        g_file_error.clear();
        f();
        return CF_OK;
    } catch (const Error &e) {
        g_file_error = e.msg;
        return e.status;
    } catch (const std::bad_alloc &) {
        g_file_error = "host allocation failed";
        return CF_OUT_OF_MEMORY;
    } catch (...) {
        g_file_error = "unexpected internal error";
        return CF_CUDA_ERROR;
    }
}

extern "C" {

int32_t cf_abi_version(void) { return CF_ABI_VERSION; }

const char *cf_file_last_error(void) { return g_file_error.c_str(); }

cf_status cf_csr_file_info(const char *path, int32_t *rows, int32_t *cols, int64_t *nnz)
{
    if (!path) return CF_BAD_INPUT;
    return file_guarded([&] {
        cf::HostCsr A;
        cf::read_csr_file(path, A);
        if (rows) *rows = A.rows;
        if (cols) *cols = A.cols;
        if (nnz) *nnz = (int64_t)A.values.size();
    });
}

cf_status cf_csr_file_read(const char *path, int32_t *row_offsets, int32_t *cols, double *vals)
{
    if (!path || !row_offsets) return CF_BAD_INPUT;
    return file_guarded([&] {
        cf::HostCsr A;
        cf::read_csr_file(path, A);
        cf::require(A.values.empty() || (cols && vals), CF_BAD_INPUT, "null output array");
        std::memcpy(row_offsets, A.row_offsets.data(), sizeof(int32_t) * A.row_offsets.size());
        if (!A.values.empty()) {
            std::memcpy(cols, A.cols_idx.data(), sizeof(int32_t) * A.cols_idx.size());
            std::memcpy(vals, A.values.data(), sizeof(double) * A.values.size());
        }
    });
}

cf_status cf_csr_file_save(const char *path, int32_t rows, int32_t cols, int64_t nnz,
                           const int32_t *row_offsets, const int32_t *cols_idx, const double *vals)
{
    if (!path || (rows > 0 && !row_offsets) || (nnz > 0 && (!cols_idx || !vals))) return CF_BAD_INPUT;
    return file_guarded([&] { cf::save_csr_file(path, rows, cols, nnz, row_offsets, cols_idx, vals); });
}

cf_status cf_vector_file_info(const char *path, int32_t *size)
{
    if (!path) return CF_BAD_INPUT;
    return file_guarded([&] {
        std::vector<double> v;
        cf::read_vector_file(path, v);
        if (size) *size = (int32_t)v.size();
    });
}

cf_status cf_vector_file_read(const char *path, double *values)
{
    if (!path) return CF_BAD_INPUT;
    return file_guarded([&] {
        std::vector<double> v;
        cf::read_vector_file(path, v);
        cf::require(v.empty() || values, CF_BAD_INPUT, "null output array");
        if (!v.empty()) std::memcpy(values, v.data(), sizeof(double) * v.size());
    });
}

cf_status cf_vector_file_save(const char *path, int32_t size, const double *values)
{
    if (!path || (size > 0 && !values)) return CF_BAD_INPUT;
    return file_guarded([&] { cf::save_vector_file(path, size, values); });
}

const char *cf_status_string(int32_t s)
{
    switch (s) {
    case CF_OK: return "ok";
    case CF_NOT_CONVERGED: return "not converged";
    case CF_BREAKDOWN: return "breakdown";
    case CF_NONFINITE: return "non-finite residual";
    case CF_BAD_INPUT: return "bad input";
    case CF_CUDA_ERROR: return "CUDA error";
    case CF_TIMEOUT: return "timeout";
    case CF_NO_DEVICE: return "no device";
    case CF_UNSUPPORTED: return "unsupported";
    case CF_OUT_OF_MEMORY: return "out of memory";
    default: return "unknown status";
    }
}

cf_status cf_solver_from_name(const char *name, int32_t *solver)
{
    if (!name || !solver) return CF_BAD_INPUT;
    static const struct { const char *name; int32_t kind; } table[] = {
        {"CG", CF_CG}, {"BiCG", CF_BICG}, {"Jacobi", CF_JACOBI}, {"MR", CF_MR},
        {"MRJacobi", CF_MRJACOBI}, {"MRS", CF_MRS}, {"JMR", CF_JMR}, {"Richardson", CF_RICHARDSON},
        {"PCG", CF_PCG}};
    const char *s = name;
    if (std::strncmp(s, "cuFoam", 6) == 0) s += 6;
    for (const auto &t : table)
        if (std::strcmp(s, t.name) == 0) {
            *solver = t.kind;
            return CF_OK;
        }
    return CF_BAD_INPUT;
}

void cf_controls_init(cf_controls *c)
{
    if (!c) return;
    std::memset(c, 0, sizeof(*c));
    c->tolerance = 1e-6;      // OpenFOAM lduMatrix::solver default tolerance
    c->rel_tol = 0.0;
    c->max_iter = 1000;       // OpenFOAM default maxIter
    c->min_iter = 0;
    c->precision = CF_PREC_FP64;
    c->reduction = CF_REDUCE_AUTO;
    c->memory = CF_MEM_HOST;
    c->norm_type = CF_NORM_REFERENCE_L2;
    c->bicg_int_bound = 1e-10;   // cuFoamBiCG/cuFoamBiCG.C:68
    c->richardson_omega = 0.0;   // cuFoamRichardson/cuFoamRichardson.C:66
    c->power_max_steps = 30;
    c->mixed_max_outer = 50;
    c->mixed_inner_rtol = 0.0; // the solver's default
    c->history = nullptr;
    c->history_capacity = 0;
    c->use_graph = 1;
    c->time_limit_s = 0.0;
}

cf_status cf_context_create(int32_t device, cf_context **out)
{
    if (!out) return CF_BAD_INPUT;
    *out = nullptr;
    cf::Context *impl = nullptr;
    cf_status st = guarded(nullptr, [&] { impl = cf::context_create(device); });
    if (st != CF_OK) return st;
    *out = new (std::nothrow) cf_context{impl};
    if (!*out) {
        delete impl;
        return CF_OUT_OF_MEMORY;
    }
    return CF_OK;
}

void cf_context_destroy(cf_context *ctx)
{
    if (!ctx) return;
    cudaSetDevice(ctx->impl->device);
    cudaStreamSynchronize(ctx->impl->stream);
    for (cf_matrix *m : ctx->matrices) {
        delete m->impl;
        m->impl = nullptr;
        m->owner = nullptr;
    }
    for (cf_batch *b : ctx->batches) {
        cf::batch_destroy(b->impl);
        b->impl = nullptr;
        b->owner = nullptr;
    }
    delete ctx->impl;
    delete ctx;
}

cf_status cf_context_set_stream(cf_context *ctx, void *stream)
{
    if (!ctx) return CF_BAD_INPUT;
    return guarded(ctx, [&] {
        cf::Context *c = ctx->impl;
        CF_CUDA(cudaStreamSynchronize(c->stream));
        cudaStream_t next = static_cast<cudaStream_t>(stream);
        if (!stream) {
            if (c->own_stream) return;   // already on a private stream
            CF_CUDA(cudaStreamCreateWithFlags(&next, cudaStreamNonBlocking));
        }
        if (c->own_stream) cudaStreamDestroy(c->stream);
        c->stream = next;
        c->own_stream = stream == nullptr;
    });
}

const char *cf_context_last_error(const cf_context *ctx)
{
    return ctx ? ctx->impl->last_error.c_str() : "null context";
}

cf_status cf_device_query(cf_context *ctx, cf_device_info *out)
{
    if (!ctx || !out) return CF_BAD_INPUT;
    return guarded(ctx, [&] {
        cf::Context *c = ctx->impl;
        cudaDeviceProp p;
        CF_CUDA(cudaGetDeviceProperties(&p, c->device));
        std::memset(out, 0, sizeof(*out));
        out->device = c->device;
        out->sm_count = c->sm_count;
        out->cc_major = p.major;
        out->cc_minor = p.minor;
        out->max_threads_per_sm = c->max_threads_sm;
        out->reference_grid = c->ref_grid;
        out->l2_bytes = (int64_t)c->l2_bytes;
        out->global_mem_bytes = (int64_t)p.totalGlobalMem;
        std::strncpy(out->name, p.name, sizeof(out->name) - 1);
    });
}

// a new matrix handle, registered with its context (or the matrix freed)
static cf_status register_matrix(cf_context *ctx, cf::Matrix *m, cf_matrix **out)
{
    cf_matrix *h = new (std::nothrow) cf_matrix{m, ctx};
    try {
        if (h) ctx->matrices.insert(h);
    } catch (...) {
        delete h;
        h = nullptr;
    }
    if (!h) {
        delete m;
        return CF_OUT_OF_MEMORY;
    }
    *out = h;
    return CF_OK;
}

cf_status cf_matrix_create_ldu(cf_context *ctx, const cf_ldu_view *ldu, cf_matrix **out)
{
    if (!ctx || !ldu || !out) return CF_BAD_INPUT;
    *out = nullptr;
    cf::Matrix *m = nullptr;
    cf_status st = guarded(ctx, [&] {
        cf::require(ldu->memory == CF_MEM_HOST || ldu->memory == CF_MEM_DEVICE, CF_BAD_INPUT,
                    "bad memory kind");
        m = cf::matrix_create(ctx->impl, *ldu);
        CF_CUDA(cudaStreamSynchronize(ctx->impl->stream));
    });
    if (st != CF_OK) return st;
    return register_matrix(ctx, m, out);
}

cf_status cf_matrix_create_csr(cf_context *ctx, int32_t n, int64_t nnz, const int32_t *row_offsets,
                               const int32_t *cols, const double *vals, int32_t memory, cf_matrix **out)
{
    if (!ctx || !out || !row_offsets || (nnz > 0 && (!cols || !vals))) return CF_BAD_INPUT;
    *out = nullptr;
    cf::Matrix *m = nullptr;
    cf_status st = guarded(ctx, [&] {
        cf::require(memory == CF_MEM_HOST || memory == CF_MEM_DEVICE, CF_BAD_INPUT, "bad memory kind");
        cf::require(n > 0 && nnz >= 0 && nnz < INT32_MAX, CF_BAD_INPUT, "bad CSR size");
        cf::Context *c = ctx->impl;
        if (memory == CF_MEM_HOST) {
            cf::DeviceBuffer dro, dcol, dval;
            dro.ensure(sizeof(int32_t) * ((size_t)n + 1));
            dcol.ensure(sizeof(int32_t) * ((size_t)nnz + 1));
            dval.ensure(sizeof(double) * ((size_t)nnz + 1));
            cf::upload(c, dro.ptr, row_offsets, sizeof(int32_t) * ((size_t)n + 1), CF_MEM_HOST);
            if (nnz > 0) {
                cf::upload(c, dcol.ptr, cols, sizeof(int32_t) * (size_t)nnz, CF_MEM_HOST);
                cf::upload(c, dval.ptr, vals, sizeof(double) * (size_t)nnz, CF_MEM_HOST);
            }
            m = cf::matrix_from_csr(c, n, nnz, dro.as<int32_t>(), dcol.as<int32_t>(), dval.as<double>());
            CF_CUDA(cudaStreamSynchronize(c->stream));
        } else {
            m = cf::matrix_from_csr(c, n, nnz, row_offsets, cols, vals);
            CF_CUDA(cudaStreamSynchronize(c->stream));
        }
    });
    if (st != CF_OK) return st;
    return register_matrix(ctx, m, out);
}

cf_status cf_matrix_update_values(cf_matrix *m, const double *diag, const double *lower,
                                  const double *upper, int32_t memory)
{
    if (!m || !m->owner) return CF_BAD_INPUT;
    return guarded(m->owner, [&] {
        cf::require(memory == CF_MEM_HOST || memory == CF_MEM_DEVICE, CF_BAD_INPUT, "bad memory kind");
        cf::matrix_update_values(m->impl, diag, lower, upper, memory);
    });
}

cf_status cf_matrix_update_csr_values(cf_matrix *m, const double *vals, int32_t memory)
{
    if (!m || !m->owner) return CF_BAD_INPUT;
    return guarded(m->owner, [&] {
        cf::require(memory == CF_MEM_HOST || memory == CF_MEM_DEVICE, CF_BAD_INPUT, "bad memory kind");
        cf::matrix_update_csr_values(m->impl, vals, memory);
    });
}

cf_status cf_matrix_set_format(cf_matrix *m, int32_t format)
{
    if (!m || !m->owner) return CF_BAD_INPUT;
    return guarded(m->owner, [&] {
        cf::require(format == CF_FORMAT_AUTO || format == CF_FORMAT_CSR || format == CF_FORMAT_SELL ||
                        format == CF_FORMAT_SELL_C8 || format == CF_FORMAT_SELL_D16,
                    CF_BAD_INPUT, "bad format");
        cf::Matrix *mi = m->impl;
        if (mi->format_request != format) {
            mi->format_request = format;
            mi->sell = -1;
            mi->have_sval = mi->have_svalT = mi->have_sval32 = mi->have_svalT32 = false;
            ++mi->gen;
        }
    });
}

cf_status cf_matrix_format(cf_matrix *m, int32_t *format, int64_t *stored_entries)
{
    if (!m || !m->owner) return CF_BAD_INPUT;
    return guarded(m->owner, [&] {
        const bool sell = cf::matrix_ensure_sell(m->impl, false, false);
        CF_CUDA(cudaStreamSynchronize(m->owner->impl->stream));
        if (format)
            *format = !sell                    ? CF_FORMAT_CSR
                      : m->impl->n_codes > 0 ? CF_FORMAT_SELL_C8
                      : m->impl->has_d16     ? CF_FORMAT_SELL_D16
                                             : CF_FORMAT_SELL;
        if (stored_entries) *stored_entries = sell ? m->impl->sell_nnz : m->impl->nnz;
    });
}

void cf_matrix_destroy(cf_matrix *m)
{
    if (!m) return;
    if (m->owner) {   // else orphaned: its context already released the memory
        cudaSetDevice(m->owner->impl->device);
        cudaStreamSynchronize(m->owner->impl->stream);
        delete m->impl;
        m->owner->matrices.erase(m);
    }
    delete m;
}

cf_status cf_matrix_shape(const cf_matrix *m, int32_t *n_rows, int32_t *n_faces, int64_t *nnz)
{
    if (!m || !m->owner) return CF_BAD_INPUT;
    if (n_rows) *n_rows = m->impl->n;
    if (n_faces) *n_faces = m->impl->nf;
    if (nnz) *nnz = m->impl->nnz;
    return CF_OK;
}

cf_status cf_matrix_export_csr(cf_matrix *m, int32_t transpose, int32_t *row_offsets, int32_t *cols,
                               double *vals, int32_t memory)
{
    if (!m || !m->owner || !row_offsets || !cols || !vals) return CF_BAD_INPUT;
    return guarded(m->owner, [&] {
        cf::Matrix *mm = m->impl;
        cf::Context *c = mm->ctx;
        if (transpose) cf::matrix_ensure_transpose(mm);
        cf::download(c, row_offsets, mm->ro.ptr, sizeof(int32_t) * ((size_t)mm->n + 1), memory);
        cf::download(c, cols, mm->col.ptr, sizeof(int32_t) * (size_t)mm->nnz, memory);
        cf::download(c, vals, transpose ? mm->valT.ptr : mm->val.ptr, sizeof(double) * (size_t)mm->nnz,
                     memory);
        CF_CUDA(cudaStreamSynchronize(c->stream));
    });
}

cf_status cf_ldu2csr(cf_context *ctx, const cf_ldu_view *ldu, int32_t *row_offsets, int32_t *cols,
                     double *vals, int32_t memory)
{
    if (!ctx || !ldu || !row_offsets || !cols || !vals) return CF_BAD_INPUT;
    return guarded(ctx, [&] { cf::ldu2csr_into(ctx->impl, *ldu, row_offsets, cols, vals, memory); });
}

cf_status cf_spmv_async(cf_matrix *m, int32_t transpose, const double *x, double *y, int32_t row_order)
{
    if (!m || !m->owner || !x || !y) return CF_BAD_INPUT;
    return guarded(m->owner, [&] {
        cf::spmv(m->impl, transpose != 0, x, y, row_order == CF_REDUCE_REFERENCE);
    });
}

cf_status cf_spmv(cf_matrix *m, int32_t transpose, const double *x, double *y, int32_t memory,
                  int32_t row_order)
{
    if (!m || !m->owner || !x || !y) return CF_BAD_INPUT;
    return guarded(m->owner, [&] {
        cf::Matrix *mm = m->impl;
        cf::Context *c = mm->ctx;
        const size_t nb = sizeof(double) * ((size_t)mm->n + 8);
        const double *dx = x;
        double *dy = y;
        if (memory == CF_MEM_HOST) {
            c->vec[0].ensure(nb);
            c->vec[1].ensure(nb);
            cf::upload(c, c->vec[0].ptr, x, sizeof(double) * mm->n, CF_MEM_HOST);
            dx = c->vec[0].as<double>();
            dy = c->vec[1].as<double>();
        }
        cf::spmv(mm, transpose != 0, dx, dy, row_order == CF_REDUCE_REFERENCE);
        if (memory == CF_MEM_HOST) cf::download(c, y, dy, sizeof(double) * mm->n, CF_MEM_HOST);
        CF_CUDA(cudaStreamSynchronize(c->stream));
    });
}

cf_status cf_norm_factor(cf_matrix *m, const double *source, const double *psi, int32_t memory,
                         int32_t norm_type, int32_t reduction, double *out)
{
    if (!m || !m->owner || !source || !psi || !out) return CF_BAD_INPUT;
    return guarded(m->owner, [&] {
        cf::Matrix *mm = m->impl;
        cf::Context *c = mm->ctx;
        const double *b = source, *x = psi;
        if (memory == CF_MEM_HOST) {
            const size_t nb = sizeof(double) * ((size_t)mm->n + 8);
            c->vec[0].ensure(nb);
            c->vec[1].ensure(nb);
            cf::upload(c, c->vec[0].ptr, psi, sizeof(double) * mm->n, CF_MEM_HOST);
            cf::upload(c, c->vec[1].ptr, source, sizeof(double) * mm->n, CF_MEM_HOST);
            x = c->vec[0].as<double>();
            b = c->vec[1].as<double>();
        }
        *out = cf::norm_factor(mm, b, x, norm_type, reduction == CF_REDUCE_REFERENCE);
    });
}

cf_status cf_solve(cf_matrix *m, int32_t solver, const cf_controls *controls, const double *source,
                   double *psi, cf_perf *perf)
{
    if (!m || !m->owner || !source || !psi) return CF_BAD_INPUT;
    cf_controls c;
    if (controls) c = *controls;
    else cf_controls_init(&c);
    cf_status st = guarded(m->owner, [&] { cf::solve(m->impl, solver, c, source, psi, perf); });
    if (st != CF_OK && perf) perf->status = st;
    return st;
}

cf_status cf_solve_decomposed(cf_matrix *m, int32_t solver, const cf_controls *controls,
                              const cf_interfaces *interfaces, const cf_comm *comm, const double *source,
                              double *psi, cf_perf *perf)
{
    if (!m || !m->owner || !source || !psi || !interfaces || !comm) return CF_BAD_INPUT;
    cf_controls c;
    if (controls) c = *controls;
    else cf_controls_init(&c);
    cf_status st = guarded(m->owner, [&] {
        cf::solve_distributed(m->impl, solver, c, *interfaces, *comm, source, psi, perf);
    });
    if (st != CF_OK && perf) perf->status = st;
    return st;
}

cf_status cf_adjoint_gradients(cf_matrix *m, const double *lambda, const double *x,
                               double *d_diag, double *d_lower, double *d_upper, int32_t memory)
{
    if (!m || !m->owner || !lambda || !x) return CF_BAD_INPUT;
    return guarded(m->owner, [&] {
        cf::Matrix *mm = m->impl;
        cf::Context *c = mm->ctx;
        cf::require(memory == CF_MEM_HOST || memory == CF_MEM_DEVICE, CF_BAD_INPUT, "bad memory kind");
        if (memory == CF_MEM_DEVICE) {
            cf::adjoint_gradients(mm, lambda, x, d_diag, d_lower, d_upper);
        } else {
            const size_t nb = sizeof(double) * ((size_t)mm->n + 8);
            const size_t fb = sizeof(double) * ((size_t)mm->nf + 8);
            c->vec[0].ensure(nb);
            c->vec[1].ensure(nb);
            c->vec[2].ensure(nb);
            c->vec[3].ensure(fb);
            c->vec[4].ensure(fb);
            cf::upload(c, c->vec[0].ptr, lambda, sizeof(double) * mm->n, CF_MEM_HOST);
            cf::upload(c, c->vec[1].ptr, x, sizeof(double) * mm->n, CF_MEM_HOST);
            cf::adjoint_gradients(mm, c->vec[0].as<double>(), c->vec[1].as<double>(),
                                  d_diag ? c->vec[2].as<double>() : nullptr,
                                  d_lower ? c->vec[3].as<double>() : nullptr,
                                  d_upper ? c->vec[4].as<double>() : nullptr);
            if (d_diag) cf::download(c, d_diag, c->vec[2].ptr, sizeof(double) * mm->n, CF_MEM_HOST);
            if (d_lower) cf::download(c, d_lower, c->vec[3].ptr, sizeof(double) * mm->nf, CF_MEM_HOST);
            if (d_upper) cf::download(c, d_upper, c->vec[4].ptr, sizeof(double) * mm->nf, CF_MEM_HOST);
        }
        CF_CUDA(cudaStreamSynchronize(c->stream));
    });
}

cf_status cf_batch_create(cf_context *ctx, int32_t n_systems, const cf_ldu_view *systems,
                          cf_batch **out)
{
    if (!ctx || !systems || !out || n_systems <= 0) return CF_BAD_INPUT;
    *out = nullptr;
    cf::Batch *b = nullptr;
    cf_status st = guarded(ctx, [&] { b = cf::batch_create(ctx->impl, n_systems, systems); });
    if (st != CF_OK) return st;
    cf_batch *h = new (std::nothrow) cf_batch{b, ctx};
    try {
        if (h) ctx->batches.insert(h);
    } catch (...) {
        delete h;
        h = nullptr;
    }
    if (!h) {
        cf::batch_destroy(b);
        return CF_OUT_OF_MEMORY;
    }
    *out = h;
    return CF_OK;
}

void cf_batch_destroy(cf_batch *b)
{
    if (!b) return;
    if (b->owner) {   // else orphaned: its context already released the memory
        cudaSetDevice(b->owner->impl->device);
        cudaStreamSynchronize(b->owner->impl->stream);
        cf::batch_destroy(b->impl);
        b->owner->batches.erase(b);
    }
    delete b;
}

cf_status cf_batch_shape(const cf_batch *b, int32_t *n_systems, int64_t *total_rows,
                         int64_t *row_offsets)
{
    if (!b || !b->owner) return CF_BAD_INPUT;
    const int s = cf::batch_systems(b->impl);
    if (n_systems) *n_systems = s;
    if (total_rows) *total_rows = cf::batch_rows(b->impl);
    if (row_offsets)
        for (int i = 0; i < s; ++i) row_offsets[i] = cf::batch_offset(b->impl, i);
    return CF_OK;
}

cf_status cf_batch_solve(cf_batch *b, int32_t solver, const cf_controls *controls,
                         const cf_batch_config *config, int32_t n_rhs, const double *sources,
                         double *psi, cf_batch_result *results, double *device_ms)
{
    if (!b || !b->owner || !sources || !psi) return CF_BAD_INPUT;
    if (solver != CF_CG) return CF_UNSUPPORTED;
    cf_controls c;
    if (controls) c = *controls;
    else cf_controls_init(&c);
    return guarded(b->owner, [&] {
        float ms = 0.f;
        cf::batch_solve(b->impl, c, n_rhs, sources, psi, c.memory, config, results, &ms);
        if (device_ms) *device_ms = ms;
    });
}

} // extern "C"
