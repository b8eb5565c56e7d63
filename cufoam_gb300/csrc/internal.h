// internal.h -- host/device structures shared by the library's translation
// units.  Nothing here is part of the C ABI (include/cufoam_gb300.h).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <string>
#include <tuple>
#include <vector>

#include "cufoam_gb300.h"

namespace cf {

// ---------------------------------------------------------------------------
// errors: thrown inside the library, turned into cf_status at the C ABI
// ---------------------------------------------------------------------------
struct Error {
    cf_status status;
    std::string msg;
};

[[noreturn]] void throw_cuda(cudaError_t e, const char *what, const char *file, int line);

#define CF_CUDA(call)                                                   \
    do {                                                                \
        cudaError_t e_ = (call);                                        \
        if (e_ != cudaSuccess) ::cf::throw_cuda(e_, #call, __FILE__, __LINE__); \
    } while (0)

#define CF_CHECK_LAUNCH() CF_CUDA(cudaGetLastError())

inline void require(bool ok, cf_status st, const std::string &msg)
{
    if (!ok) throw Error{st, msg};
}

// ---------------------------------------------------------------------------
// device-side solver state (one per context, reused by every solve)
// ---------------------------------------------------------------------------
struct DevState {
    double rho0, rho1;   // CG / BiCG inner products
    double xi;           // CG / BiCG step length
    double theta;        // BiCG direction update factor
    double beta;         // CG direction update factor rho0 / rho1 of the next step
    double omega;        // MR / MRJacobi / JMR / MRS step, Richardson relaxation
    double norm;         // latest ||r||_2 as recorded by the reference
    double norm0;        // initial ||r||_2
    double tol;          // absolute stopping threshold (tolerance * normFactor)
    double tolerance;    // relative tolerance as given (tolerance_)
    double rel_tol;      // relTol_ (0 = off)
    double nf;           // normFactor
    double int_bound;    // BiCG breakdown bound
    double pow_inv;      // power method: 1 / ||x2||
    double lambda_max;   // power method eigenvalue estimate
    double diag_abs_min; // min |a_ii|
    double xbar;         // normFactor: mean of psi
    double scale;        // mixed: residual scaling
    int32_t k;           // completed iterations
    int32_t done;        // loop finished
    int32_t status;      // cf_status of the loop
    int32_t max_steps;   // iteration limit (INT_MAX when unlimited)
    int32_t min_steps;   // minIter_
    int32_t x_pending;   // CG/BiCG: x += xi * p not yet applied
    int32_t hist_cap;    // capacity of the device history
    int32_t body_count;  // loop-guard counter (device-driven loops)
    int32_t pow_step;    // power method step counter
    int32_t flags;
    uint32_t counters[16];
};

constexpr int32_t kFlagAbsTol = 1;   // DevState::flags: tolerance is absolute

enum CounterSlot {
    SLOT_A = 0, SLOT_B, SLOT_C, SLOT_D, SLOT_NF1, SLOT_NF2, SLOT_INIT, SLOT_POW, SLOT_MISC
};

constexpr int kMaxNV = 3;       // reductions per kernel
constexpr int kBlock = 256;     // threads per block (the reference's BLOCK_SIZE)
constexpr int kWarps = kBlock / 32;

// Everything a solver kernel needs, resident in device memory so that one
// instantiated CUDA graph serves any matrix and any vectors.
struct SolveArgs {
    // matrix (CSR produced by ldu2csr; valT = A^T values on the same pattern)
    int32_t n;
    int32_t stage_cap;         // staged nnz per warp (0 = no staging)
    const int32_t *ro;
    const int32_t *col;
    const double *val;
    const double *valT;
    const float *val32;
    const float *valT32;
    // SELL-32 copy of the matrix for the fast kernels (n_slices = 0: none)
    int32_t n_slices;
    int32_t has_long;          // some row has more than kLongRow entries (device.cuh)
    const int32_t *s_off;      // [n_slices + 1] element offset of each slice
    const int32_t *s_col;
    const uint8_t *s_code;     // one-byte column codes of the same slots (null: none)
    const int32_t *s_dtab;     // offsets col - row the codes stand for
    const int16_t *s_d16;      // 16-bit column deltas col - row (null: none)
    const double *s_val;
    const double *s_valT;
    const float *s_val32;
    const float *s_valT32;
    const double *diag;        // a_ii
    const double *dinv;        // 1 / a_ii
    const double *dinv_sqrt;   // sqrt(1 / a_ii)
    // vectors (FP64)
    double *x;                 // psi (in/out)
    const double *b;           // source
    double *r[2];
    double *p[2];
    double *q;
    double *rs;
    double *ps[2];
    double *qs;
    double *w[2];
    // vectors (FP32, mixed precision inner solve)
    float *fx, *fr, *fp[2], *fq, *frs, *fps[2], *fqs;
    const double *corr_scale;  // MR family on L A R: x += s * corr_scale * d (1 / a_ii or sqrt(1 / a_ii))
    const double *sc_val;      // FP64 fast order (MR family, Jacobi): values of L A R (the format in use)
    // reductions / state
    double *partials;          // [kMaxNV][partial_stride]
    float *partials32;
    int32_t partial_stride;
    int32_t ref_order;         // reduce in the reference's order
    DevState *st;
    DevState *st_in;           // inner (FP32) solve of the mixed-precision loop
    double *hist;
    unsigned long long *hist_t; // device clock (ns) at the end of each step
    unsigned long long cond;   // cudaGraphConditionalHandle of the running loop
    int32_t use_cond;
    int32_t power_steps;       // Richardson: power-method steps
    const volatile int32_t *abort_flag; // host-mapped flag: stop the loop (time limit)
};

// ---------------------------------------------------------------------------
// host objects
// ---------------------------------------------------------------------------
struct DeviceBuffer {
    void *ptr = nullptr;
    size_t bytes = 0;
    void ensure(size_t nbytes);   // grow-only
    void release();
    ~DeviceBuffer() { release(); }
    template <class T> T *as() const { return static_cast<T *>(ptr); }
};

struct GraphKey {
    int solver, precision, reduction, stage_cap, phase, format, grid_cap;
    bool operator<(const GraphKey &o) const
    {
        return std::tie(solver, precision, reduction, stage_cap, phase, format, grid_cap) <
               std::tie(o.solver, o.precision, o.reduction, o.stage_cap, o.phase, o.format, o.grid_cap);
    }
};

struct GraphEntry {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    unsigned long long cond = 0;
    bool pdl = false;
};

struct Context {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;   // created (and destroyed) by the library
    int sm_count = 0;
    int max_threads_sm = 0;
    int ref_grid = 0;          // the reference's LaunchConfig grid on this GPU
    size_t l2_bytes = 0;
    std::string last_error;
    bool graphs_ok = true;
    bool pdl_ok = true;        // programmatic launches accepted in loop graphs

    // workspace (grow-only, reused by every solve)
    DeviceBuffer vec[24];
    DeviceBuffer partials, partials32, hist, hist_t, state, state_in, args;
    SolveArgs *h_args = nullptr;   // pinned
    DevState *h_state = nullptr;   // pinned
    DevState *h_state_in = nullptr; // pinned
    int32_t *h_abort = nullptr;    // pinned, mapped
    int32_t *d_abort = nullptr;
    cudaEvent_t ev_start = nullptr, ev_stop = nullptr, ev_mid = nullptr;
    std::vector<cudaEvent_t> prof_events;
    std::map<GraphKey, GraphEntry> graphs;

    // > 0: fast-order launches use at most this many blocks (a small
    // system, see GridCap); the reference order keeps the reference's grid
    int grid_cap = 0;
    int small_cg_ok = -1;      // 16-CTA clusters schedulable (-1: not asked yet)

    // scratch of the matrix builds (grow-only: a conversion after the first
    // allocates nothing) and the matrix of one-shot ldu2csr conversions
    DeviceBuffer scratch_flag, scratch_tmp, scratch_cnt, scratch_stats;
    DeviceBuffer scratch_codes;   // offset set of the one-byte column codes, largest |offset| (matrix.cu)
    struct Matrix *ldu_scratch = nullptr;

    int fast_grid(const void *kernel, size_t dyn_smem) const;
    ~Context();
};

// A small system's fast-order launches take one row per thread at most,
// rounded up to a power of two of blocks (so that few loop graphs exist):
// idle blocks would only add grid-reduction arrivals and last-block work.
// Set for the duration of one library call.
struct GridCap {
    Context *ctx;
    int old;
    GridCap(Context *c, int64_t rows) : ctx(c), old(c->grid_cap)
    {
        const int64_t need = (rows + kBlock - 1) / kBlock;
        int cap = 0;
        if (need < (int64_t)c->sm_count * 4) {
            cap = 1;
            while (cap < need) cap <<= 1;
        }
        c->grid_cap = cap;
    }
    ~GridCap() { ctx->grid_cap = old; }
    GridCap(const GridCap &) = delete;
    GridCap &operator=(const GridCap &) = delete;
};

struct ScaledCopy {
    DeviceBuffer buf;
    uint64_t gen = 0;          // Matrix::gen it was made at (0: none)
    int scale = 0, transpose = 0, sell = 0;
};

struct Matrix {
    Context *ctx = nullptr;
    int32_t n = 0, nf = 0;
    int64_t nnz = 0;
    int32_t max_chunk = 0;     // max nnz over 32-row chunks without a long row
    bool has_long = false;     // some row has more than kLongRow entries (device.cuh)
    // CSR (reference layout) + transpose values on the same pattern
    DeviceBuffer ro, col, val, valT, val32, valT32;
    // LDU copy (for value updates, the transpose and adjoint scatter)
    DeviceBuffer diag, lower, upper, la, ua, losort, lstart, ostart;
    DeviceBuffer dinv, dinv_sqrt;
    bool have_valT = false, have_32 = false, have_T32 = false;
    double diag_abs_min = 0.0;
    bool have_dmin = false;
    bool from_csr = false;     // built from a CSR matrix (no LDU arrays)
    // SELL-32 copy for the fast kernels; the layout depends on the pattern
    // only, the value copies are refreshed after every value change
    int format_request = CF_FORMAT_AUTO;
    int sell = -1;             // -1 not decided, 0 CSR kernels, 1 SELL-32
    int32_t n_slices = 0;
    int64_t sell_nnz = 0;      // stored entries including padding
    DeviceBuffer s_off, s_col, s_val, s_valT, s_val32, s_valT32;
    // one-byte column codes of the SELL-32 slots and the table of offsets
    // col - row they index (n_codes distinct offsets; 0: 32-bit columns only)
    DeviceBuffer s_code, s_dtab;
    int32_t n_codes = 0;
    // 16-bit column deltas col - row of the slots, when the codes cannot be
    // used and every offset fits
    DeviceBuffer s_d16;
    bool has_d16 = false;
    bool have_sval = false, have_svalT = false, have_sval32 = false, have_svalT32 = false;
    // bumped by every change of the values, of 1/a_ii or of the format
    uint64_t gen = 1;
    // diagonally scaled values L A R of the MR family's loop (FP64 fast
    // order, FP32 mixed sweeps), kept until `gen` or the request changes
    ScaledCopy sc64, sc32;
};

// ---------------------------------------------------------------------------
// entry points between translation units
// ---------------------------------------------------------------------------
Context *context_create(int device);
void context_bind(Context *ctx);
void upload(Context *ctx, void *dst, const void *src, size_t bytes, int memory);
void download(Context *ctx, void *dst, const void *src, size_t bytes, int memory);

Matrix *matrix_create(Context *ctx, const cf_ldu_view &v);
void matrix_update_values(Matrix *m, const double *diag, const double *lower,
                          const double *upper, int memory);
void matrix_ensure_transpose(Matrix *m);
void matrix_ensure_fp32(Matrix *m, bool transpose);
void matrix_ensure_dmin(Matrix *m);
void ldu2csr_into(Context *ctx, const cf_ldu_view &v, int32_t *ro, int32_t *col,
                  double *val, int memory);

int stage_cap_for(const Matrix *m);
bool matrix_ensure_sell(Matrix *m, bool transpose, bool fp32);
Matrix *matrix_from_csr(Context *ctx, int n, int64_t nnz, const int32_t *ro, const int32_t *col,
                        const double *val);
void matrix_set_transpose_csr(Matrix *m, const int32_t *roT, const int32_t *colT, const double *valT);
void matrix_update_csr_values(Matrix *m, const double *vals, int memory);
void matrix_set_inverse_diagonal(Matrix *m, const double *dinv);
void csr_transpose(Context *ctx, int n_rows, int n_cols, int64_t nnz, const int32_t *ro,
                   const int32_t *col, const double *val, int32_t *roT, int32_t *colT, double *valT);
void spmv(Matrix *m, bool transpose, const double *x, double *y, bool ref_order);
double norm_factor(Matrix *m, const double *b, const double *x, int norm_type, bool ref_order);
void solve(Matrix *m, int solver, const cf_controls &c, const double *b, double *x,
           cf_perf *perf);
// CG on one subdomain of a decomposed case (distributed.cu)
void solve_distributed(Matrix *m, int solver, const cf_controls &c, const cf_interfaces &ifc,
                       const cf_comm &comm, const double *b, double *x, cf_perf *perf);

// CG, and Jacobi, Richardson and the MR family, on one small system in a
// single cluster-persistent launch (batched.cu)
struct SmallSolveResult {
    double nf, norm0, norm;
    int32_t iters, status;
    float ms;
    double omega = 0.0;
};
struct SmallSolveOut {
    double nf, norm0, norm, omega;
    int32_t iters, status;
};
SmallSolveResult solve_cg_single_cluster(Matrix *m, const cf_controls &c, const double *b, double *x,
                                         double *r, double *p, double *q);
SmallSolveResult solve_small_single_cluster(Matrix *m, int solver, const cf_controls &c, const double *b,
                                            double *x, double *r, double *d, double *y);
bool small_cg_ok(Context *ctx);

struct Batch;
Batch *batch_create(Context *ctx, int n_systems, const cf_ldu_view *views);
void batch_destroy(Batch *B);
void batch_solve(Batch *B, const cf_controls &c, int nrhs, const double *b_in, double *x_io,
                 int memory, const cf_batch_config *cfg, cf_batch_result *results, float *ms_out);
int64_t batch_rows(const Batch *B);
int batch_systems(const Batch *B);
int64_t batch_offset(const Batch *B, int s);

// host CSR / vector files (formats.cpp)
struct HostCsr {
    int rows = 0, cols = 0;
    std::vector<int32_t> row_offsets, cols_idx;
    std::vector<double> values;
};
void read_csr_file(const std::string &path, HostCsr &out);
void save_csr_file(const std::string &path, int rows, int cols, int64_t nnz, const int32_t *ro,
                   const int32_t *col, const double *val);
void read_vector_file(const std::string &path, std::vector<double> &out);
void save_vector_file(const std::string &path, int size, const double *v);

void adjoint_gradients(Matrix *m, const double *lam, const double *x, double *d_diag,
                       double *d_lower, double *d_upper);

struct MixedResult {
    int inner_iterations = 0;
    int outer = 0;
    int status = CF_OK;
};
bool mixed_supported(int solver);
void mixed_prepare(Context *ctx, Matrix *m, int solver, SolveArgs &A);
MixedResult run_mixed(Context *ctx, Matrix *m, int solver, const cf_controls &c, SolveArgs *d_args,
                      int cap, bool use_graph);

} // namespace cf
