// noalloc.cu -- residual norm of a caller-owned device field with no device
// allocation.
//
// The norm is the deterministic two-level reduction used by the solver's
// convergence test (per-block partials, then the last block to finish sums them
// in block order).  Here its scratch -- the per-block partials and the
// completion counter -- is a file-scope __device__ array rather than memory
// from cudaMalloc, so a caller that cannot allocate device memory can still use
// it: for example a process whose device memory is all held by another
// allocator (a framework's caching allocator), or code that must not trigger
// the device-wide synchronisation cudaMalloc/cudaFree can cause.
//
// Limits and sharing:
//   * the array holds 32768 partials: at most 32768 * 8192 = 268435456 values
//     per call (each block reduces a fixed chunk of 8192 values, so the result
//     depends only on the values and n, not on the GPU);
//   * every GPU that loads the library holds the array (256 KiB + 256 B)
//     until the process exits;
//   * all calls on one GPU share the array: calls that overlap on the GPU (on
//     different streams, or from different threads) race on it and must be
//     serialised by the caller.
#include "../../include/fans_gb300.h"
#include "fans_common.cuh"

#include <cuda_runtime.h>
#include <mutex>

namespace fansgpu {
int fail(fansgpu_ctx *ctx, int code, const char *fmt, ...);
}

namespace {

constexpr int       kThreads      = 256;
constexpr long long kChunk        = 8192;
constexpr int       kMaxBlocks    = 32768;
constexpr size_t    kPartialBytes = sizeof(double) * kMaxBlocks;
constexpr size_t    kScratchBytes = kPartialBytes + 256; // + one line for the completion counter
static_assert(FANSGPU_NOALLOC_MAX_VALUES == (long long)kMaxBlocks * kChunk, "limit in the header");

// The scratch.  Host code must not pass this name to a kernel: on the host it
// is a stand-in symbol, not a device address (see scratch_address()).
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

__global__ void __launch_bounds__(kThreads) k_norm_noalloc(const double *__restrict__ r, long long n, int measure,
                                                           unsigned char *scratch, double *out)
{
    __shared__ double red[32];
    __shared__ bool   s_last;
    double           *partials = reinterpret_cast<double *>(scratch);
    unsigned int     *counter  = reinterpret_cast<unsigned int *>(scratch + kPartialBytes);
    const bool        mx       = measure == FANSGPU_LINF;
    const long long   lo       = (long long)blockIdx.x * kChunk;
    const long long   hi       = min(n, lo + kChunk);
    double            acc      = 0.0;
    for (long long i = lo + threadIdx.x; i < hi; i += blockDim.x) {
        const double a = fabs(r[i]);
        const double t = measure == FANSGPU_L2 ? a * a : a;
        acc            = mx ? fansgpu::nan_max(acc, t) : acc + t;
    }
    double    v[1]   = {acc};
    const int ops[1] = {mx ? fansgpu::RED_MAX : fansgpu::RED_SUM};
    fansgpu::block_reduce<1>(v, ops, red);
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = v[0];
        __threadfence();
        const unsigned int done = atomicAdd(counter, 1u);
        s_last                  = (done == gridDim.x - 1);
    }
    __syncthreads();
    if (!s_last)
        return;
    __threadfence();
    // last block: fold the partials in block order (fixed for a given n)
    const int per = (gridDim.x + blockDim.x - 1) / blockDim.x;
    const int b0 = threadIdx.x * per, b1 = min((int)gridDim.x, b0 + per);
    double    s  = 0.0;
    for (int b = b0; b < b1; ++b) {
        const double t = __ldcg(&partials[b]);
        s              = mx ? fansgpu::nan_max(s, t) : s + t;
    }
    v[0] = s;
    fansgpu::block_reduce<1>(v, ops, red);
    if (threadIdx.x == 0) {
        *out     = measure == FANSGPU_L2 ? sqrt(v[0]) : v[0];
        *counter = 0;
    }
}

// Device address of the scratch array.  It is looked up on every call made
// outside stream capture (cudaGetSymbolAddress is cheap), so a context that was
// destroyed and made again (cudaDeviceReset, a new primary context) never sees
// a stale address.  A call made while its stream is being captured cannot make
// that lookup safely and uses the address the last uncaptured call on the same
// device found: the first call on a device must therefore come before any
// stream capture.
std::mutex     g_mu;
unsigned char *g_addr[256] = {nullptr};

int scratch_address(cudaStream_t st, unsigned char **addr)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return fansgpu::fail(nullptr, FANSGPU_ECUDA, "fansgpu_residual_norm_noalloc: no current device: %s",
                             cudaGetErrorString(e));
    if (dev < 0 || dev >= 256)
        return fansgpu::fail(nullptr, FANSGPU_EUNSUPPORTED, "fansgpu_residual_norm_noalloc: device id %d", dev);
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    e = cudaStreamIsCapturing(st, &cap);
    if (e != cudaSuccess)
        return fansgpu::fail(nullptr, FANSGPU_ECUDA, "fansgpu_residual_norm_noalloc: stream query: %s",
                             cudaGetErrorString(e));
    std::lock_guard<std::mutex> lock(g_mu);
    if (cap != cudaStreamCaptureStatusNone) {
        if (!g_addr[dev])
            return fansgpu::fail(nullptr, FANSGPU_ESTATE,
                                 "fansgpu_residual_norm_noalloc: first call on device %d made during stream capture; "
                                 "call it once before capturing",
                                 dev);
        *addr = g_addr[dev];
        return 0;
    }
    void *p = nullptr;
    e       = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
        return fansgpu::fail(nullptr, FANSGPU_ECUDA,
                             "fansgpu_residual_norm_noalloc: cudaGetSymbolAddress failed on device %d: %s", dev,
                             cudaGetErrorString(e));
    g_addr[dev] = static_cast<unsigned char *>(p);
    *addr       = g_addr[dev];
    return 0;
}

} // namespace

extern "C" int fansgpu_residual_norm_noalloc(const double *r_dev, int64_t n, int32_t measure, double *out_dev,
                                             void *stream)
{
    if (!out_dev || (n > 0 && !r_dev))
        return fansgpu::fail(nullptr, FANSGPU_EINVAL, "fansgpu_residual_norm_noalloc: null pointer");
    if (measure < FANSGPU_L1 || measure > FANSGPU_LINF)
        return fansgpu::fail(nullptr, FANSGPU_EINVAL, "fansgpu_residual_norm_noalloc: unknown measure %d", measure);
    if (n < 0 || n > FANSGPU_NOALLOC_MAX_VALUES)
        return fansgpu::fail(nullptr, FANSGPU_EINVAL,
                             "fansgpu_residual_norm_noalloc: n = %lld outside [0, %lld] (the static scratch holds "
                             "%d block partials of %lld values each)",
                             (long long)n, (long long)FANSGPU_NOALLOC_MAX_VALUES, kMaxBlocks, kChunk);
    cudaStream_t   st      = static_cast<cudaStream_t>(stream);
    unsigned char *scratch = nullptr;
    int            rc      = scratch_address(st, &scratch);
    if (rc)
        return rc;
    cudaError_t  e;
    if (n == 0) {
        e = cudaMemsetAsync(out_dev, 0, sizeof(double), st);
    } else {
        // the completion counter must start at zero (a previous call leaves it zero
        // unless it was interrupted, so clear it on every call)
        e = cudaMemsetAsync(scratch + kPartialBytes, 0, sizeof(unsigned int), st);
        if (e == cudaSuccess) {
            const int blocks = (int)((n + kChunk - 1) / kChunk);
            k_norm_noalloc<<<blocks, kThreads, 0, st>>>(r_dev, (long long)n, measure, scratch, out_dev);
            e = cudaGetLastError();
        }
    }
    if (e != cudaSuccess)
        return fansgpu::fail(nullptr, FANSGPU_ECUDA, "fansgpu_residual_norm_noalloc: %s", cudaGetErrorString(e));
    return 0;
}
