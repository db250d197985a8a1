// k_diag.cu -- device-rate measurement for the roofline of the FP64 path.
//
// The FP64 CG operator (k_stencil<double, C>: 576 dependent-free DFMA per node
// for mechanics) is bound by the FP64 pipe, not by HBM.  Its roofline needs the
// device's FP64 FMA rate, which no vendor table states for this part: this file
// measures it with a kernel of independent FMA chains on every SM.
#include "../../include/fans_gb300.h"
#include "fans_common.cuh"

#include <cuda_runtime.h>

namespace fansgpu {
int fail(fansgpu_ctx *ctx, int code, const char *fmt, ...);
}

namespace {

constexpr int kChains = 8, kIters = 4096, kThreads = 256;

// kChains independent FMA chains per thread, kIters steps each; `out` is only
// written for an impossible result so that the chains are not optimised away.
__global__ void __launch_bounds__(kThreads) k_fp64_fma(double a, double b, double *out)
{
    double acc[kChains];
#pragma unroll
    for (int c = 0; c < kChains; ++c)
        acc[c] = (double)(threadIdx.x + c);
    for (int i = 0; i < kIters; ++i)
#pragma unroll
        for (int c = 0; c < kChains; ++c)
            acc[c] = fma(acc[c], a, b);
    double s = 0.0;
#pragma unroll
    for (int c = 0; c < kChains; ++c)
        s += acc[c];
    if (s == -1.2345e300 && out)
        *out = s;
}

} // namespace

extern "C" int fansgpu_fp64_fma_rate(double *dfma_per_s)
{
    if (!dfma_per_s)
        return fansgpu::fail(nullptr, FANSGPU_EINVAL, "fansgpu_fp64_fma_rate: null output");
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess)
        e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (e == cudaSuccess)
        e = cudaEventCreate(&e0);
    if (e == cudaSuccess)
        e = cudaEventCreate(&e1);
    float ms = 0.f;
    const int blocks = sms * 8;
    if (e == cudaSuccess) {
        k_fp64_fma<<<blocks, kThreads>>>(1.0000001, 1e-9, nullptr); // warm-up (clocks up)
        e = cudaEventRecord(e0);
    }
    if (e == cudaSuccess) {
        for (int r = 0; r < 4; ++r)
            k_fp64_fma<<<blocks, kThreads>>>(1.0000001, 1e-9, nullptr);
        e = cudaEventRecord(e1);
    }
    if (e == cudaSuccess)
        e = cudaEventSynchronize(e1);
    if (e == cudaSuccess)
        e = cudaGetLastError();
    if (e == cudaSuccess)
        e = cudaEventElapsedTime(&ms, e0, e1);
    if (e0)
        cudaEventDestroy(e0);
    if (e1)
        cudaEventDestroy(e1);
    if (e != cudaSuccess || !(ms > 0.f))
        return fansgpu::fail(nullptr, FANSGPU_ECUDA, "fansgpu_fp64_fma_rate: %s", cudaGetErrorString(e));
    *dfma_per_s = 4.0 * blocks * kThreads * (double)kChains * kIters / (ms * 1e-3);
    return 0;
}
