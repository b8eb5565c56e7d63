/*
 * ref_gpu.c -- TEST INFRASTRUCTURE ONLY (the oracle's checker, never the
 * product path).
 *
 * An orc_backend whose primitives launch the reference's own kernels
 * (gis/SparseSystem/kernels.h, instantiated by ref_kernels.cu and compiled
 * into a cubin from the reference sources by oracle/build.py) on the GPU,
 * the way the reference's host functions do (gis/SparseSystem/
 * SolverSingleGPU.h): grid = maxThreadsPerSM / 256 x SMs blocks of 256
 * threads (LaunchConfig, launch.h:116-139), block partials copied to the
 * host and summed there in block order (Sum / Dot, SolverSingleGPU.h:
 * 74-126), the diagonal minimum taken on the host (FindDiagAbsMin,
 * :686-720).  Every primitive copies its inputs to the device, launches,
 * and copies its outputs back, so the oracle's drivers (oracle.c) run
 * unchanged on top of it; speed is irrelevant, bits are the point.
 *
 * The CUDA driver is opened with dlopen, so this library builds and loads
 * on a machine without one; rg_open then reports the failure.
 */
#define _POSIX_C_SOURCE 200809L
#include "../oracle.h"

#include <cuda.h>
#include <dlfcn.h>
#include <float.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

enum {
    K_FILL, K_REDUCTION, K_DOT, K_SPMV, K_DISTANCE, K_SCALE, K_ADD1, K_HADAMARD, K_RESIDUAL,
    K_FINDDIAG, K_MINABS, K_FINDDIAGINV, K_FINDDIAGINVSQRT, K_COUNT
};
static const char *const kKernelNames[K_COUNT] = {
    "FillKernel", "ReductionKernel", "DotKernel", "SpMvKernel", "DistanceKernel", "ScaleKernel",
    "AddKernel1", "HadamardKernel", "ResidualKernel", "FindDiag", "MinAbsKernel", "FindDiagInv",
    "FindDiagInvSqrt"};

/* ---- the driver entry points used ------------------------------------- */
typedef CUresult (*PFN_Init)(unsigned int);
typedef CUresult (*PFN_DeviceGet)(CUdevice *, int);
typedef CUresult (*PFN_DeviceGetAttribute)(int *, CUdevice_attribute, CUdevice);
typedef CUresult (*PFN_PrimaryCtxRetain)(CUcontext *, CUdevice);
typedef CUresult (*PFN_PrimaryCtxRelease)(CUdevice);
typedef CUresult (*PFN_CtxPushCurrent)(CUcontext);
typedef CUresult (*PFN_CtxPopCurrent)(CUcontext *);
typedef CUresult (*PFN_ModuleLoad)(CUmodule *, const char *);
typedef CUresult (*PFN_ModuleUnload)(CUmodule);
typedef CUresult (*PFN_ModuleGetFunction)(CUfunction *, CUmodule, const char *);
typedef CUresult (*PFN_MemAlloc)(CUdeviceptr *, size_t);
typedef CUresult (*PFN_MemFree)(CUdeviceptr);
typedef CUresult (*PFN_MemcpyHtoD)(CUdeviceptr, const void *, size_t);
typedef CUresult (*PFN_MemcpyDtoH)(void *, CUdeviceptr, size_t);
typedef CUresult (*PFN_MemsetD8)(CUdeviceptr, unsigned char, size_t);
typedef CUresult (*PFN_MemcpyDtoD)(CUdeviceptr, CUdeviceptr, size_t);
typedef CUresult (*PFN_LaunchKernel)(CUfunction, unsigned, unsigned, unsigned, unsigned, unsigned,
                                     unsigned, unsigned, CUstream, void **, void **);
typedef CUresult (*PFN_CtxSynchronize)(void);

static struct {
    void *lib;
    PFN_Init Init;
    PFN_DeviceGet DeviceGet;
    PFN_DeviceGetAttribute DeviceGetAttribute;
    PFN_PrimaryCtxRetain PrimaryCtxRetain;
    PFN_PrimaryCtxRelease PrimaryCtxRelease;
    PFN_CtxPushCurrent CtxPushCurrent;
    PFN_CtxPopCurrent CtxPopCurrent;
    PFN_ModuleLoad ModuleLoad;
    PFN_ModuleUnload ModuleUnload;
    PFN_ModuleGetFunction ModuleGetFunction;
    PFN_MemAlloc MemAlloc;
    PFN_MemFree MemFree;
    PFN_MemcpyHtoD MemcpyHtoD;
    PFN_MemcpyDtoH MemcpyDtoH;
    PFN_MemsetD8 MemsetD8;
    PFN_MemcpyDtoD MemcpyDtoD;
    PFN_LaunchKernel LaunchKernel;
    PFN_CtxSynchronize CtxSynchronize;
} cu;

static struct {
    int open;
    CUdevice dev;
    CUcontext ctx;
    CUmodule mod;
    CUfunction fn[K_COUNT];
    int grid;           /* LaunchConfig: maxThreadsPerSM / 256 x SMs */
    int error;          /* first failing CUresult (0: none) */
    long launches;      /* kernels launched since rg_open */
    char where[128];
} g;

static int fail(CUresult r, const char *where)
{
    if (r != CUDA_SUCCESS && !g.error) {
        g.error = (int)r;
        snprintf(g.where, sizeof(g.where), "%s", where);
    }
    return r != CUDA_SUCCESS;
}

/* ---- scratch device buffers ------------------------------------------- */
#define NBUF 8
static CUdeviceptr buf[NBUF];
static size_t cap[NBUF];

static CUdeviceptr scratch(int i, size_t bytes)
{
    if (bytes == 0) bytes = 8;
    if (cap[i] < bytes) {
        if (buf[i]) cu.MemFree(buf[i]);
        buf[i] = 0;
        cap[i] = 0;
        if (fail(cu.MemAlloc(&buf[i], bytes), "cuMemAlloc")) return 0;
        cap[i] = bytes;
    }
    return buf[i];
}

static CUdeviceptr put(int i, const void *src, size_t bytes)
{
    CUdeviceptr d = scratch(i, bytes);
    if (d && bytes) fail(cu.MemcpyHtoD(d, src, bytes), "cuMemcpyHtoD");
    return d;
}

static void get(void *dst, CUdeviceptr src, size_t bytes)
{
    if (bytes) fail(cu.MemcpyDtoH(dst, src, bytes), "cuMemcpyDtoH");
}

static void launch(int k, int grid, void **args)
{
    if (g.error) return;
    if (fail(cu.LaunchKernel(g.fn[k], (unsigned)grid, 1, 1, 256, 1, 1, 0, NULL, args, NULL), kKernelNames[k]))
        return;
    ++g.launches;
    fail(cu.CtxSynchronize(), kKernelNames[k]);
}

/* buffers 0..2 vectors, 3 partials, 4..6 the matrix, 7 the result */
static void put_matrix(const orc_csr *A, CUdeviceptr *ro, CUdeviceptr *col, CUdeviceptr *val)
{
    *ro = put(4, A->row_offsets, sizeof(int32_t) * ((size_t)A->n + 1));
    *col = put(5, A->cols, sizeof(int32_t) * (size_t)A->nnz);
    *val = put(6, A->vals, sizeof(double) * (size_t)A->nnz);
}

/* ---- primitives -------------------------------------------------------- */
static double be_reduce(int kind, const double *a, const double *b, int32_t n, int32_t grid)
{
    if (grid <= 0) grid = 1;
    CUdeviceptr part = scratch(3, sizeof(double) * (size_t)grid);
    CUdeviceptr da = put(0, a, sizeof(double) * (size_t)n);
    CUdeviceptr db = kind == 1 ? 0 : put(1, b, sizeof(double) * (size_t)n);
    int nn = n;
    if (kind == 1) {
        void *args[] = {&part, &da, &nn};
        launch(K_REDUCTION, grid, args);
    } else {
        void *args[] = {&part, &da, &db, &nn};
        launch(kind == 0 ? K_DOT : K_DISTANCE, grid, args);
    }
    double *h = (double *)malloc(sizeof(double) * (size_t)grid);
    double sum = 0.0;
    if (h) {
        get(h, part, sizeof(double) * (size_t)grid);
        for (int i = 0; i < grid; ++i) sum += h[i];
        free(h);
    }
    return sum;
}

static void be_spmv(const orc_csr *A, const double *x, double *y)
{
    CUdeviceptr ro, col, val;
    put_matrix(A, &ro, &col, &val);
    CUdeviceptr dx = put(0, x, sizeof(double) * (size_t)A->n);
    CUdeviceptr dy = scratch(7, sizeof(double) * (size_t)A->n);
    int n = A->n;
    void *args[] = {&dy, &val, &ro, &col, &n, &dx};
    launch(K_SPMV, g.grid, args);
    get(y, dy, sizeof(double) * (size_t)A->n);
}

static void be_residual(const orc_csr *A, const double *b, const double *x, double *r)
{
    CUdeviceptr ro, col, val;
    put_matrix(A, &ro, &col, &val);
    CUdeviceptr db = put(0, b, sizeof(double) * (size_t)A->n);
    CUdeviceptr dx = put(1, x, sizeof(double) * (size_t)A->n);
    CUdeviceptr dr = scratch(7, sizeof(double) * (size_t)A->n);
    int n = A->n;
    void *args[] = {&dr, &val, &ro, &col, &n, &db, &dx};
    launch(K_RESIDUAL, g.grid, args);
    get(r, dr, sizeof(double) * (size_t)A->n);
}

static void be_add(double *res, const double *v1, const double *v2, double alpha, int32_t n)
{
    CUdeviceptr d1 = put(0, v1, sizeof(double) * (size_t)n);
    CUdeviceptr d2 = put(1, v2, sizeof(double) * (size_t)n);
    CUdeviceptr dr = scratch(7, sizeof(double) * (size_t)n);
    int nn = n;
    void *args[] = {&dr, &d1, &d2, &nn, &alpha};
    launch(K_ADD1, g.grid, args);
    get(res, dr, sizeof(double) * (size_t)n);
}

static void be_hadamard(double *res, const double *v1, const double *v2, int32_t n)
{
    CUdeviceptr d1 = put(0, v1, sizeof(double) * (size_t)n);
    CUdeviceptr d2 = put(1, v2, sizeof(double) * (size_t)n);
    CUdeviceptr dr = scratch(7, sizeof(double) * (size_t)n);
    int nn = n;
    void *args[] = {&dr, &d1, &d2, &nn};
    launch(K_HADAMARD, g.grid, args);
    get(res, dr, sizeof(double) * (size_t)n);
}

static void be_scale(double *res, const double *v, double alpha, int32_t n)
{
    CUdeviceptr dv = put(0, v, sizeof(double) * (size_t)n);
    CUdeviceptr dr = scratch(7, sizeof(double) * (size_t)n);
    int nn = n;
    void *args[] = {&dr, &dv, &nn, &alpha};
    launch(K_SCALE, g.grid, args);
    get(res, dr, sizeof(double) * (size_t)n);
}

static void be_fill(double *res, double val, int32_t n)
{
    CUdeviceptr dr = scratch(7, sizeof(double) * (size_t)n);
    int nn = n;
    void *args[] = {&dr, &nn, &val};
    launch(K_FILL, g.grid, args);
    get(res, dr, sizeof(double) * (size_t)n);
}

static void be_diag(const orc_csr *A, double *d, int mode)
{
    CUdeviceptr ro, col, val;
    put_matrix(A, &ro, &col, &val);
    CUdeviceptr dd = scratch(7, sizeof(double) * (size_t)A->n);
    if (dd) fail(cu.MemsetD8(dd, 0, sizeof(double) * (size_t)A->n), "cuMemsetD8");
    int n = A->n;
    void *args[] = {&dd, &val, &ro, &col, &n};
    launch(mode == 0 ? K_FINDDIAG : mode == 1 ? K_FINDDIAGINV : K_FINDDIAGINVSQRT, g.grid, args);
    get(d, dd, sizeof(double) * (size_t)A->n);
}

static double be_diag_abs_min(const orc_csr *A)
{
    CUdeviceptr ro, col, val;
    put_matrix(A, &ro, &col, &val);
    CUdeviceptr dd = scratch(7, sizeof(double) * (size_t)A->n);
    if (dd) fail(cu.MemsetD8(dd, 0, sizeof(double) * (size_t)A->n), "cuMemsetD8");
    int n = A->n;
    void *a1[] = {&dd, &val, &ro, &col, &n};
    launch(K_FINDDIAG, g.grid, a1);
    CUdeviceptr part = scratch(3, sizeof(double) * (size_t)g.grid);
    void *a2[] = {&part, &dd, &n};
    launch(K_MINABS, g.grid, a2);
    double *h = (double *)malloc(sizeof(double) * (size_t)g.grid);
    double result = DBL_MAX;
    if (h) {
        get(h, part, sizeof(double) * (size_t)g.grid);
        for (int i = 0; i < g.grid; ++i)
            if (result > h[i]) result = h[i];
        free(h);
    }
    return result;
}

/* ---- the reference's CG on device-resident data, timed ------------------ */
/* Kernels go to the legacy default stream without a synchronisation after
 * each one, as the reference's LaunchKernel does; Dot synchronises through
 * its copy of the block partials. */
static void launch_async(int k, void **args)
{
    if (g.error) return;
    if (fail(cu.LaunchKernel(g.fn[k], (unsigned)g.grid, 1, 1, 256, 1, 1, 0, NULL, args, NULL), kKernelNames[k]))
        return;
    ++g.launches;
}

/* Dot (SolverSingleGPU.h:101-126): a fresh device partial buffer, the
 * DotKernel, a synchronous copy of the partials, a host sum in block order,
 * and the buffers freed again. */
static double dev_dot(CUdeviceptr a, CUdeviceptr b, int n)
{
    CUdeviceptr part = 0;
    if (fail(cu.MemAlloc(&part, sizeof(double) * (size_t)g.grid), "cuMemAlloc")) return NAN;
    void *args[] = {&part, &a, &b, &n};
    launch_async(K_DOT, args);
    double *h = (double *)malloc(sizeof(double) * (size_t)g.grid);
    double sum = 0.0;
    if (h) {
        get(h, part, sizeof(double) * (size_t)g.grid);
        for (int i = 0; i < g.grid; ++i) sum += h[i];
        free(h);
    }
    cu.MemFree(part);
    return sum;
}

static void dev_add(CUdeviceptr res, CUdeviceptr v1, CUdeviceptr v2, int n, double alpha)
{
    void *args[] = {&res, &v1, &v2, &n, &alpha};
    launch_async(K_ADD1, args);
}

static double now_ms(void)
{
    struct timespec t;
    clock_gettime(CLOCK_MONOTONIC, &t);
    return 1e3 * (double)t.tv_sec + 1e-6 * (double)t.tv_nsec;
}

/* The reference's CG (SolverSingleGPU.h:366-445) with the matrix, b and x
 * already on the device: r = b - Ax, p = r, rho = (r, r), then per step
 * p = r + (rho0/rho1) p, q = A p, xi = rho0 / (p, q), x += xi p,
 * r -= xi q, rho = (r, r), stopping at ||r|| <= error.  x is updated in
 * place; history gets ||r|| per step (initial first).  *solve_ms is the wall
 * time of the solver call, its work vectors' allocation and release
 * included (the reference allocates them per call).  Returns the number of
 * steps, or -1 on a driver error. */
int rg_cg_device(int n, int nnz, const int32_t *ro, const int32_t *col, const double *val,
                 const double *b, double *x, double error, int max_steps, double *history,
                 int hist_cap, int *n_hist, double *solve_ms)
{
    if (!g.open) return -1;
    orc_csr A = {n, nnz, ro, col, val};
    CUdeviceptr dro, dcol, dval;
    put_matrix(&A, &dro, &dcol, &dval);
    CUdeviceptr db = put(0, b, sizeof(double) * (size_t)n);
    CUdeviceptr dx = put(1, x, sizeof(double) * (size_t)n);
    fail(cu.CtxSynchronize(), "upload");
    if (g.error) return -1;
    int len = 0;
    const double t0 = now_ms();
    CUdeviceptr r = 0, p = 0, q = 0;
    const size_t vb = sizeof(double) * (size_t)(n > 0 ? n : 1);
    fail(cu.MemAlloc(&r, vb), "cuMemAlloc");
    {
        void *args[] = {&r, &dval, &dro, &dcol, &n, &db, &dx};
        launch_async(K_RESIDUAL, args);
    }
    fail(cu.MemAlloc(&p, vb), "cuMemAlloc");
    fail(cu.MemcpyDtoD(p, r, vb), "cuMemcpyDtoD");
    double rho0 = dev_dot(r, r, n), rho1 = 0.0;
    double norm_r = sqrt(rho0);
    fail(cu.MemAlloc(&q, vb), "cuMemAlloc");
    if (max_steps <= 0) max_steps = 0x7fffffff;
    if (len < hist_cap) history[len++] = norm_r;
    int k = 1;
    for (; k <= max_steps && norm_r > error && !g.error; ++k) {
        if (k > 1) dev_add(p, r, p, n, rho0 / rho1);
        {
            void *args[] = {&q, &dval, &dro, &dcol, &n, &p};
            launch_async(K_SPMV, args);
        }
        const double xi = rho0 / dev_dot(p, q, n);
        dev_add(dx, dx, p, n, xi);
        dev_add(r, r, q, n, -xi);
        rho1 = rho0;
        rho0 = dev_dot(r, r, n);
        norm_r = sqrt(rho0);
        if (len < hist_cap) history[len++] = norm_r;
    }
    fail(cu.CtxSynchronize(), "CG");
    cu.MemFree(r);
    cu.MemFree(p);
    cu.MemFree(q);
    *solve_ms = now_ms() - t0;
    get(x, dx, sizeof(double) * (size_t)n);
    *n_hist = len;
    return g.error ? -1 : k - 1;
}

static const orc_backend kBackend = {be_reduce, be_spmv,  be_residual, be_add,         be_hadamard,
                                     be_scale,  be_fill,  be_diag,     be_diag_abs_min};

/* ---- set-up ------------------------------------------------------------ */
static int load_driver(void)
{
    if (cu.lib) return 0;
    cu.lib = dlopen("libcuda.so.1", RTLD_NOW | RTLD_LOCAL);
    if (!cu.lib) return -1;
#define SYM(field, name)                                   \
    do {                                                   \
        *(void **)&cu.field = dlsym(cu.lib, name);         \
        if (!cu.field) return -1;                          \
    } while (0)
    SYM(Init, "cuInit");
    SYM(DeviceGet, "cuDeviceGet");
    SYM(DeviceGetAttribute, "cuDeviceGetAttribute");
    SYM(PrimaryCtxRetain, "cuDevicePrimaryCtxRetain");
    SYM(PrimaryCtxRelease, "cuDevicePrimaryCtxRelease_v2");
    SYM(CtxPushCurrent, "cuCtxPushCurrent_v2");
    SYM(CtxPopCurrent, "cuCtxPopCurrent_v2");
    SYM(ModuleLoad, "cuModuleLoad");
    SYM(ModuleUnload, "cuModuleUnload");
    SYM(ModuleGetFunction, "cuModuleGetFunction");
    SYM(MemAlloc, "cuMemAlloc_v2");
    SYM(MemFree, "cuMemFree_v2");
    SYM(MemcpyHtoD, "cuMemcpyHtoD_v2");
    SYM(MemcpyDtoH, "cuMemcpyDtoH_v2");
    SYM(MemsetD8, "cuMemsetD8_v2");
    SYM(MemcpyDtoD, "cuMemcpyDtoD_v2");
    SYM(LaunchKernel, "cuLaunchKernel");
    SYM(CtxSynchronize, "cuCtxSynchronize");
#undef SYM
    return 0;
}

/* Load the cubin and look up its kernels; `names` lists "Key mangled-name"
 * lines (written by the build recipe from ptxas's entry list).  Returns 0,
 * or -1 with a message in err. */
int rg_open(const char *cubin, const char *names, int device, char *err, int err_len)
{
    memset(&g, 0, sizeof(g));
    if (load_driver()) {
        snprintf(err, (size_t)err_len, "cannot open the CUDA driver (libcuda.so.1)");
        return -1;
    }
    int sms = 0, threads = 0;
    if (fail(cu.Init(0), "cuInit") || fail(cu.DeviceGet(&g.dev, device), "cuDeviceGet") ||
        fail(cu.DeviceGetAttribute(&sms, CU_DEVICE_ATTRIBUTE_MULTIPROCESSOR_COUNT, g.dev), "attr") ||
        fail(cu.DeviceGetAttribute(&threads, CU_DEVICE_ATTRIBUTE_MAX_THREADS_PER_MULTIPROCESSOR, g.dev),
             "attr") ||
        fail(cu.PrimaryCtxRetain(&g.ctx, g.dev), "cuDevicePrimaryCtxRetain") ||
        fail(cu.CtxPushCurrent(g.ctx), "cuCtxPushCurrent") || fail(cu.ModuleLoad(&g.mod, cubin), "cuModuleLoad")) {
        snprintf(err, (size_t)err_len, "%s failed (CUresult %d)", g.where, g.error);
        return -1;
    }
    g.grid = threads / 256 * sms;
    FILE *f = fopen(names, "r");
    if (!f) {
        snprintf(err, (size_t)err_len, "cannot read %s", names);
        return -1;
    }
    char key[128], mangled[512];
    int found = 0;
    while (fscanf(f, "%127s %511s", key, mangled) == 2) {
        for (int k = 0; k < K_COUNT; ++k)
            if (strcmp(key, kKernelNames[k]) == 0 && !g.fn[k]) {
                if (fail(cu.ModuleGetFunction(&g.fn[k], g.mod, mangled), "cuModuleGetFunction")) break;
                ++found;
            }
    }
    fclose(f);
    if (found != K_COUNT || g.error) {
        snprintf(err, (size_t)err_len, "found %d of %d reference kernels (%s)", found, K_COUNT, g.where);
        return -1;
    }
    g.open = 1;
    return 0;
}

const orc_backend *rg_backend(void) { return g.open ? &kBackend : NULL; }

int rg_grid(void) { return g.grid; }

long rg_launches(void) { return g.launches; }

/* 0, or the first CUresult that failed since rg_open, with where it failed */
int rg_error(char *where, int len)
{
    if (where && len > 0) snprintf(where, (size_t)len, "%s", g.where);
    return g.error;
}

void rg_close(void)
{
    if (!g.open) return;
    for (int i = 0; i < NBUF; ++i) {
        if (buf[i]) cu.MemFree(buf[i]);
        buf[i] = 0;
        cap[i] = 0;
    }
    cu.ModuleUnload(g.mod);
    CUcontext c;
    cu.CtxPopCurrent(&c);
    cu.PrimaryCtxRelease(g.dev);
    g.open = 0;
}
