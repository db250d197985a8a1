// fans_common.cuh -- shared device types and helpers of the GB300 FANS solve path.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace fansgpu {

template <typename T>
struct __align__(sizeof(T) * 2) cplx {
    T x, y;
};

template <typename T>
__device__ __forceinline__ cplx<T> cmul(cplx<T> a, cplx<T> b)
{
    return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
template <typename T>
__device__ __forceinline__ cplx<T> cmulc(cplx<T> a, cplx<T> b) // a * conj(b)
{
    return {a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y};
}
template <typename T>
__device__ __forceinline__ cplx<T> cadd(cplx<T> a, cplx<T> b)
{
    return {a.x + b.x, a.y + b.y};
}
template <typename T>
__device__ __forceinline__ cplx<T> csub(cplx<T> a, cplx<T> b)
{
    return {a.x - b.x, a.y - b.y};
}

// Periodic wrap of an index that is at most one period out of range.
__device__ __forceinline__ int wrap(int i, int n)
{
    return i < 0 ? i + n : (i >= n ? i - n : i);
}

// Reduction kinds used by the fused CG kernels.
enum RedOp { RED_SUM = 0, RED_MAX = 1 };

// Scalars of one CG state, resident in device memory so that consecutive
// kernels read the values the previous kernel's last block produced.
struct CgScalars {
    double delta, delta0, deltamid, beta, dAd, alpha, err, err0;
    double aux[8];
    int    converged;
    int    pad[3];
};

// Scratch for grid reductions: per-block partials plus a completion counter.
// The last block to finish sums the partials in block order (deterministic).
struct GridRed {
    double      *partials; // [max_blocks][kMaxRed]
    unsigned int *counter;  // one counter per reduction site
};
constexpr int kMaxRed = 20; // large-strain averages reduce 2*9+1 values
constexpr int kMaxRhs = 6;  // right-hand sides of one multi-RHS solve (the 6 Mandel load cases)

// The device's opt-in maximum of shared memory per block (static + dynamic).
inline int smem_optin_max()
{
    static const int v = [] {
        int dev = 0, b = 48 * 1024;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&b, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        return b;
    }();
    return v;
}

// Lets `fn` take as much dynamic shared memory as the device allows next to
// its static shared memory.  MaxDynamicSharedMemorySize is a per-kernel,
// process-wide attribute: one fixed value per kernel means contexts driven
// from several host threads never race one another to different limits.
// Occupancy follows each launch's actual size.
template <typename F>
inline cudaError_t allow_max_dyn_smem(F *fn)
{
    cudaFuncAttributes fa;
    cudaError_t        e = cudaFuncGetAttributes(&fa, (const void *)fn);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute((const void *)fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                smem_optin_max() - (int)fa.sharedSizeBytes);
}

// The same, and the largest shared-memory carveout, for kernels that need more than half
// of an SM's shared memory per CTA to keep two CTAs resident.
template <typename F>
inline cudaError_t allow_max_dyn_smem_carveout(F *fn)
{
    cudaError_t e = allow_max_dyn_smem(fn);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute((const void *)fn, cudaFuncAttributePreferredSharedMemoryCarveout,
                                (int)cudaSharedmemCarveoutMaxShared);
}

// Maxima that keep NaN (fmax returns the other operand), so that a non-finite
// residual reaches the host through the Linfinity norm as well.
__device__ __forceinline__ double nan_max(double a, double b) { return (a > b || a != a) ? a : b; }
__device__ __forceinline__ float  nan_maxf(float a, float b) { return (a > b || a != a) ? a : b; }

// Block-wide reduction of NV values (sum or max per value), result valid in
// thread 0.  Uses warp shuffles then one pass through shared memory.
template <int NV>
__device__ __forceinline__ void block_reduce(double (&v)[NV], const int (&ops)[NV], double *smem /* 32*NV */)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            double t = __shfl_down_sync(0xffffffffu, v[k], o);
            v[k]     = ops[k] == RED_MAX ? nan_max(v[k], t) : v[k] + t;
        }
    }
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < NV; ++k)
            smem[warp * NV + k] = v[k];
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            double t = (lane < nw) ? smem[lane * NV + k] : (ops[k] == RED_MAX ? 0.0 : 0.0);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                double t2 = __shfl_down_sync(0xffffffffu, t, o);
                t         = ops[k] == RED_MAX ? nan_max(t, t2) : t + t2;
            }
            v[k] = t;
        }
    }
}

// Write this block's partials; returns true in the block that finished last
// (after which the caller sums `partials` over all blocks in order).
template <int NV>
__device__ __forceinline__ bool grid_partial_commit(const double (&v)[NV], double *partials, unsigned int *counter,
                                                    int nblocks)
{
    static_assert(NV <= kMaxRed, "a block's partials must fit its kMaxRed slots");
    __shared__ bool s_last;
    const int       bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k)
            partials[(size_t)bid * kMaxRed + k] = v[k];
        __threadfence();
        unsigned int done = atomicAdd(counter, 1u);
        s_last            = (done == (unsigned int)nblocks - 1);
        if (s_last)
            *counter = 0; // reset for the next launch (stream-ordered)
    }
    __syncthreads();
    if (s_last)
        __threadfence();
    return s_last;
}

// Deterministic final sum over block partials (called by every thread of the
// last block); result valid in thread 0.
template <int NV>
__device__ __forceinline__ void grid_final(double (&v)[NV], const int (&ops)[NV], const double *partials,
                                           int nblocks, double *smem)
{
#pragma unroll
    for (int k = 0; k < NV; ++k)
        v[k] = 0.0;
    // each thread folds a contiguous stripe of blocks in order, then the block
    // reduction combines stripes in thread order: fixed order for a given grid.
    const int per = (nblocks + blockDim.x - 1) / blockDim.x;
    const int b0 = threadIdx.x * per, b1 = min(nblocks, b0 + per);
    for (int b = b0; b < b1; ++b)
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            double t = __ldcg(&partials[(size_t)b * kMaxRed + k]);
            v[k]     = ops[k] == RED_MAX ? nan_max(v[k], t) : v[k] + t;
        }
    block_reduce<NV>(v, ops, smem);
}

// Deterministic final sum over the partials of blocks [b0, b0 + count) (called
// by every thread of the last block; result valid in thread 0): the per-RHS
// sums of a grid whose blockIdx.y is the right-hand side.  With b0 = 0 and
// count = all blocks it is grid_final.
template <int NV>
__device__ __forceinline__ void grid_final_range(double (&v)[NV], const int (&ops)[NV], const double *partials,
                                                 int b0, int count, double *smem)
{
#pragma unroll
    for (int k = 0; k < NV; ++k)
        v[k] = 0.0;
    const int per = (count + blockDim.x - 1) / blockDim.x;
    const int s0 = threadIdx.x * per, s1 = min(count, s0 + per);
    for (int b = s0; b < s1; ++b)
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            double t = __ldcg(&partials[(size_t)(b0 + b) * kMaxRed + k]);
            v[k]     = ops[k] == RED_MAX ? nan_max(v[k], t) : v[k] + t;
        }
    block_reduce<NV>(v, ops, smem);
}

} // namespace fansgpu

#define FANS_CUDA_CHECK(...)                                                                                     \
    do {                                                                                                         \
        cudaError_t _e = (__VA_ARGS__);                                                                          \
        if (_e != cudaSuccess)                                                                                   \
            return fansgpu::fail(ctx, FANSGPU_ECUDA, "%s failed: %s (%s:%d)", #__VA_ARGS__,                      \
                                 cudaGetErrorString(_e), __FILE__, __LINE__);                                    \
    } while (0)
