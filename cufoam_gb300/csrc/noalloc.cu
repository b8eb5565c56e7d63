// noalloc.cu -- normFactor without any device allocation.
//
// cf_norm_factor_noalloc computes the reference's normFactor
// (gis/gis.cu:106-123) of a CSR matrix the caller already holds on the
// device, for callers that must not allocate device memory: an application
// that hands the GPU to its own memory pool and forbids further driver
// allocations, or code on a latency-critical path where a cudaMalloc /
// cudaFree (which can synchronise the whole device) is not acceptable.
//
// Its only scratch -- the block partial sums, the mean of psi and the
// arrival counters of the grid reductions -- lives in one file-scope
// __device__ array of fixed size (kScratchBytes below, about 33 KB), which
// every GPU that loads the library keeps until the process exits.  Host code
// never uses the array's name as an address: the device address is looked
// up once per device with cudaGetSymbolAddress (on the first call on that
// device, with that device current) and passed to the kernels.
#include "device.cuh"

#include <mutex>

namespace cf {

namespace {

constexpr int kNoAllocMaxBlocks = 2048; // grid-reduction partials the scratch holds

struct NoAllocScratch {
    double partials[2 * kNoAllocMaxBlocks];
    double xbar;
    double pad;
    uint32_t counters[4];
};

constexpr size_t kScratchBytes = sizeof(NoAllocScratch);

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
void *g_scratch_addr[kMaxDevices] = {nullptr};

__global__ void __launch_bounds__(kBlock) k_na_sum(int n, const double *__restrict__ x,
                                                  NoAllocScratch *s, bool ref)
{
    double acc[1] = {0.0};
    CF_FOR_ELEMS(i, n) acc[0] = acc[0] + x[i];
    double tot[1];
    if (grid_reduce<1, double>(acc, s->partials, kNoAllocMaxBlocks, &s->counters[0], ref, tot) &&
        threadIdx.x == 0)
        s->xbar = tot[0] / n;
}

// Y = A x, Ybar = A (xbar 1), distances; rows read straight from the
// caller's arrays (no staging, so nothing is read past nnz).
__global__ void __launch_bounds__(kBlock) k_na_dist(int n, const int32_t *__restrict__ ro,
                                                   const int32_t *__restrict__ col,
                                                   const double *__restrict__ val,
                                                   const double *__restrict__ x,
                                                   const double *__restrict__ b, NoAllocScratch *s,
                                                   bool ref, double *out)
{
    const double xbar = __ldcg(&s->xbar);
    double acc[2] = {0.0, 0.0};
    CF_FOR_CHUNKS(base, n) {
        const int row = base + (threadIdx.x & 31);
        Chunk<double> ch;
        ch.rs = __ldg(ro + (row < n ? row : n));
        ch.re = __ldg(ro + (row < n ? row + 1 : n));
        ch.ov = ch.oc = -1;
        ch.sv = nullptr;
        ch.sc = nullptr;
        const double Y = row_product<double>(ch, col, val, [&](int c) { return x[c]; });
        const double Yb = row_product<double>(ch, col, val, [&](int) { return xbar; });
        if (row < n) {
            const double d1 = Y - Yb, d2 = b[row] - Yb;
            acc[0] = fma_t(d1, d1, acc[0]);
            acc[1] = fma_t(d2, d2, acc[1]);
        }
    }
    double tot[2];
    if (grid_reduce<2, double>(acc, s->partials, kNoAllocMaxBlocks, &s->counters[1], ref, tot) &&
        threadIdx.x == 0)
        *out = sqrt(tot[0]) + sqrt(tot[1]) + 1e-20;
}

} // namespace

// Device address of the scratch array on the current device (looked up once
// per device).
static cf_status noalloc_scratch(int device, void **ptr)
{
    if (device < 0 || device >= kMaxDevices) return CF_UNSUPPORTED;
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_scratch_addr[device]) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) {
            cudaGetLastError();
            return CF_CUDA_ERROR;
        }
        g_scratch_addr[device] = p;
    }
    *ptr = g_scratch_addr[device];
    return CF_OK;
}

static cf_status norm_factor_noalloc(int32_t n, const int32_t *ro, const int32_t *col, const double *val,
                                     const double *b, const double *x, int32_t reduction, double *out,
                                     void *stream)
{
    if (n <= 0 || !ro || !col || !val || !b || !x || !out) return CF_BAD_INPUT;
    if (reduction != CF_REDUCE_FAST && reduction != CF_REDUCE_REFERENCE) return CF_BAD_INPUT;
    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess) {
        cudaGetLastError();
        return CF_NO_DEVICE;
    }
    int sms = 0, tpsm = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
        cudaDeviceGetAttribute(&tpsm, cudaDevAttrMaxThreadsPerMultiProcessor, device) != cudaSuccess) {
        cudaGetLastError();
        return CF_CUDA_ERROR;
    }
    const bool ref = reduction == CF_REDUCE_REFERENCE;
    // the reference order needs its own grid; reject it when the scratch
    // cannot hold that many block partials
    int grid = ref ? tpsm / kBlock * sms : std::min(sms * 4, kNoAllocMaxBlocks);
    if (grid < 1 || grid > kNoAllocMaxBlocks) return CF_UNSUPPORTED;
    cudaStream_t cs = static_cast<cudaStream_t>(stream);
    // the scratch address is the current device's: a stream of another
    // device would run the kernels there against this device's address
    int stream_device = -1;
    if (cudaStreamGetDevice(cs, &stream_device) != cudaSuccess) {
        cudaGetLastError();
        return CF_BAD_INPUT;
    }
    if (stream_device != device) return CF_BAD_INPUT;
    void *p = nullptr;
    cf_status st = noalloc_scratch(device, &p);
    if (st != CF_OK) return st;
    NoAllocScratch *s = static_cast<NoAllocScratch *>(p);
    // the array keeps the last call's contents: restart the arrival counters
    if (cudaMemsetAsync(s->counters, 0, sizeof(s->counters), cs) != cudaSuccess) {
        cudaGetLastError();
        return CF_CUDA_ERROR;
    }
    k_na_sum<<<grid, kBlock, 0, cs>>>(n, x, s, ref);
    k_na_dist<<<grid, kBlock, 0, cs>>>(n, ro, col, val, x, b, s, ref, out);
    if (cudaGetLastError() != cudaSuccess) return CF_CUDA_ERROR;
    return CF_OK;
}

} // namespace cf

extern "C" cf_status cf_norm_factor_noalloc(int32_t n_rows, const int32_t *row_offsets,
                                            const int32_t *cols, const double *vals,
                                            const double *source, const double *psi,
                                            int32_t reduction, double *norm_factor,
                                            void *cuda_stream)
{
    return cf::norm_factor_noalloc(n_rows, row_offsets, cols, vals, source, psi, reduction,
                                   norm_factor, cuda_stream);
}
