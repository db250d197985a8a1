// k_vec.cu -- streaming CG vector kernels with fused FP64 reductions.
#include "kernels.cuh"

#include <type_traits>

namespace fansgpu {

namespace {
constexpr int kVecThreads = 256;

__device__ __forceinline__ double norm_term(double v, int measure)
{
    double a = fabs(v);
    return measure == 1 ? a * a : a; // L2: squares; L1 / Linf: |v|
}

// r -= alpha*Kd; u -= alpha*d; partial ||r|| and <r, s>  (solverCG.h:105-113, solver.h:415-430).
// Element arithmetic in T (FP32 in the mixed inner loop, where u is the FP32
// correction since the last reliable update, or FP64); partial sums of four
// strided elements are formed in T and accumulated in FP64.
template <typename T, typename TU>
__global__ void __launch_bounds__(kVecThreads) k_cg_update(UpdateArgs a)
{
    __shared__ double red_smem[32 * 2];
    const T      alpha = (T)a.scal->alpha;
    T           *r  = reinterpret_cast<T *>(a.r);
    const T     *Kd = reinterpret_cast<const T *>(a.Kd);
    TU          *u  = reinterpret_cast<TU *>(a.u);
    const T     *d  = reinterpret_cast<const T *>(a.d);
    const T     *s  = reinterpret_cast<const T *>(a.s);
    double       nrm = 0.0, rs = 0.0;
    const int    measure = a.measure;
    const bool   mx  = measure == 2;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long base = blockIdx.x * (long long)blockDim.x + threadIdx.x; base < a.n; base += 4 * stride) {
        T cn = (T)0, crs = (T)0;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const long long i = base + j * stride;
            if (i < a.n) {
                const T rv = r[i] - alpha * Kd[i];
                r[i]       = rv;
                if (a.do_u)
                    u[i] = u[i] - (TU)alpha * (TU)d[i];
                const T av = rv < (T)0 ? -rv : rv;
                const T t  = measure == 1 ? av * av : av;
                cn         = mx ? ((t > cn || t != t) ? t : cn) : cn + t; // NaN-keeping max
                crs += rv * s[i];
            }
        }
        nrm = mx ? nan_max(nrm, (double)cn) : nrm + (double)cn;
        rs += (double)crs;
    }
    double v[2]   = {nrm, rs};
    int    ops[2] = {mx ? RED_MAX : RED_SUM, RED_SUM};
    block_reduce<2>(v, ops, red_smem);
    if (grid_partial_commit<2>(v, a.red.partials, a.red.counter + a.red_site, gridDim.x)) {
        grid_final<2>(v, ops, a.red.partials, gridDim.x, red_smem);
        if (threadIdx.x == 0) {
            a.scal->err      = a.measure == 1 ? sqrt(v[0]) : v[0];
            a.scal->deltamid = v[1];
            if (!isfinite(a.scal->err))
                a.scal->converged = -1;
        }
    }
}

// FP32 inner-loop update with 16-byte accesses (n is a multiple of 8: even grid
// dimensions); same arithmetic and FP64 partials as k_cg_update<float, float>.
// Several right-hand sides: blockIdx.y = k works on RHS k's fields (offset k n)
// with alpha_k, and the last block finishes ||r_k|| and <r_k, s_k> of every
// active RHS from its blocks' partials in block order.
__global__ void __launch_bounds__(kVecThreads) k_cg_update_f4(UpdateArgs a)
{
    __shared__ double red_smem[32 * 2];
    const int       k     = blockIdx.y;
    const bool      on    = !a.active || a.active[k];
    const long long off   = (long long)k * a.n / 4;
    const float     alpha = on ? (float)a.scal[k].alpha : 0.f;
    float4       *r  = reinterpret_cast<float4 *>(a.r) + off;
    const float4 *Kd = reinterpret_cast<const float4 *>(a.Kd) + off;
    float4       *u  = reinterpret_cast<float4 *>(a.u) + off;
    const float4 *d  = reinterpret_cast<const float4 *>(a.d) + off;
    const float4 *s  = reinterpret_cast<const float4 *>(a.s) + off;
    const int     measure = a.measure;
    const bool    mx = measure == 2;
    const long long nv = on ? a.n / 4 : 0;
    double        nrm = 0.0, rs = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nv; i += (long long)gridDim.x * blockDim.x) {
        float4       rv = r[i];
        const float4 kv = Kd[i], sv = s[i];
        rv.x -= alpha * kv.x;
        rv.y -= alpha * kv.y;
        rv.z -= alpha * kv.z;
        rv.w -= alpha * kv.w;
        r[i] = rv;
        if (a.do_u) {
            float4       uv = u[i];
            const float4 dv = d[i];
            uv.x -= alpha * dv.x;
            uv.y -= alpha * dv.y;
            uv.z -= alpha * dv.z;
            uv.w -= alpha * dv.w;
            u[i] = uv;
        }
        float cn;
        if (measure == 1)
            cn = rv.x * rv.x + rv.y * rv.y + rv.z * rv.z + rv.w * rv.w;
        else if (mx)
            cn = nan_maxf(nan_maxf(fabsf(rv.x), fabsf(rv.y)), nan_maxf(fabsf(rv.z), fabsf(rv.w)));
        else
            cn = fabsf(rv.x) + fabsf(rv.y) + fabsf(rv.z) + fabsf(rv.w);
        nrm = mx ? nan_max(nrm, (double)cn) : nrm + (double)cn;
        rs += (double)(rv.x * sv.x + rv.y * sv.y + rv.z * sv.z + rv.w * sv.w);
    }
    double v[2]   = {nrm, rs};
    int    ops[2] = {mx ? RED_MAX : RED_SUM, RED_SUM};
    block_reduce<2>(v, ops, red_smem);
    const int gx = gridDim.x;
    if (grid_partial_commit<2>(v, a.red.partials, a.red.counter + a.red_site, gx * gridDim.y)) {
        for (int q = 0; q < (int)gridDim.y; ++q) {
            if (a.active && !a.active[q])
                continue;
            grid_final_range<2>(v, ops, a.red.partials, q * gx, gx, red_smem);
            if (threadIdx.x == 0) {
                CgScalars *sc = a.scal + q;
                sc->err       = a.measure == 1 ? sqrt(v[0]) : v[0];
                sc->deltamid  = v[1];
                if (!isfinite(sc->err))
                    sc->converged = -1;
            }
            __syncthreads(); // red_smem is reused by the next right-hand side
        }
    }
}

// ||r|| of an FP64 field with the re-seed copy to FP32; `fast`: squares and
// short partial sums in FP32 (relative accuracy ~1e-7 of the norm, enough for
// the mixed path's refresh test), FP64 otherwise.
template <typename T, typename TO>
__global__ void __launch_bounds__(kVecThreads) k_norm_fast(const T *__restrict__ r, long long n, int measure,
                                                           CgScalars *scal, int set_err0, TO *r_out, GridRed red,
                                                           int site)
{
    __shared__ double red_smem[32];
    const bool mx = measure == 2;
    double     nrm = 0.0;
    const long long nv = n / 2;
    const double2 *r2 = reinterpret_cast<const double2 *>(r);
    float2        *o2 = reinterpret_cast<float2 *>(r_out);
    auto           one = [&](const double2 v, long long i) {
        const float2 f = make_float2((float)v.x, (float)v.y);
        if (o2)
            o2[i] = f;
        float cn;
        if (measure == 1)
            cn = f.x * f.x + f.y * f.y;
        else if (mx)
            cn = nan_maxf(fabsf(f.x), fabsf(f.y));
        else
            cn = fabsf(f.x) + fabsf(f.y);
        nrm = mx ? nan_max(nrm, (double)cn) : nrm + (double)cn;
    };
    // four independent 16-byte loads in flight per thread and step, then the remainder
    const long long stride = (long long)gridDim.x * blockDim.x;
    long long       i      = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    for (; i + 3 * stride < nv; i += 4 * stride) {
        const double2 v0 = r2[i], v1 = r2[i + stride], v2 = r2[i + 2 * stride], v3 = r2[i + 3 * stride];
        one(v0, i);
        one(v1, i + stride);
        one(v2, i + 2 * stride);
        one(v3, i + 3 * stride);
    }
    for (; i < nv; i += stride)
        one(r2[i], i);
    double v[1]   = {nrm};
    int    ops[1] = {mx ? RED_MAX : RED_SUM};
    block_reduce<1>(v, ops, red_smem);
    if (grid_partial_commit<1>(v, red.partials, red.counter + site, gridDim.x)) {
        grid_final<1>(v, ops, red.partials, gridDim.x, red_smem);
        if (threadIdx.x == 0) {
            double e  = measure == 1 ? sqrt(v[0]) : v[0];
            scal->err = e;
            if (set_err0)
                scal->err0 = e;
            if (!isfinite(e))
                scal->converged = -1;
        }
    }
}

template <typename T, typename TO>
__global__ void __launch_bounds__(kVecThreads) k_norm(const T *__restrict__ r, long long n, int measure,
                                                      CgScalars *scal, int set_err0, TO *r_out, GridRed red,
                                                      int site)
{
    __shared__ double red_smem[32];
    double     nrm = 0.0;
    const bool mx  = measure == 2;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        T      v = r[i];
        double t = norm_term((double)v, measure);
        nrm      = mx ? nan_max(nrm, t) : nrm + t;
        if (r_out)
            r_out[i] = (TO)v;
    }
    double v[1]   = {nrm};
    int    ops[1] = {mx ? RED_MAX : RED_SUM};
    block_reduce<1>(v, ops, red_smem);
    if (grid_partial_commit<1>(v, red.partials, red.counter + site, gridDim.x)) {
        grid_final<1>(v, ops, red.partials, gridDim.x, red_smem);
        if (threadIdx.x == 0) {
            double e  = measure == 1 ? sqrt(v[0]) : v[0];
            scal->err = e;
            if (set_err0)
                scal->err0 = e;
            if (!isfinite(e))
                scal->converged = -1;
        }
    }
}

template <typename T>
__global__ void k_axpy(T *__restrict__ y, const T *__restrict__ x, double a, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        y[i] = (T)((double)y[i] + a * (double)x[i]);
}

__global__ void k_extrapolate(double *__restrict__ u, double *__restrict__ up, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double delta = u[i] - up[i];
        up[i]              = u[i];
        u[i] += delta;
    }
}

__global__ void k_fold(double *__restrict__ u, float *__restrict__ e, long long n)
{
    // four values per step with 16-byte accesses where u and e are 16-byte aligned (every
    // field of the context is), else one at a time; the same additions either way
    const long long stride = (long long)gridDim.x * blockDim.x, t0 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    long long       done   = 0;
    if (((reinterpret_cast<uintptr_t>(u) | reinterpret_cast<uintptr_t>(e)) & 15) == 0) {
        const long long nq = n / 4;
        double2        *u2 = reinterpret_cast<double2 *>(u);
        float4         *e4 = reinterpret_cast<float4 *>(e);
        for (long long i = t0; i < nq; i += stride) {
            const float4 ev = e4[i];
            double2      a  = u2[2 * i], b = u2[2 * i + 1];
            a.x += (double)ev.x;
            a.y += (double)ev.y;
            b.x += (double)ev.z;
            b.y += (double)ev.w;
            u2[2 * i]     = a;
            u2[2 * i + 1] = b;
            e4[i]         = make_float4(0.f, 0.f, 0.f, 0.f);
        }
        done = 4 * nq;
    }
    for (long long i = done + t0; i < n; i += stride) {
        u[i] += (double)e[i];
        e[i] = 0.0f;
    }
}
__global__ void k_ms_convert(const uint16_t *__restrict__ in, uint8_t *__restrict__ out, long long n,
                             unsigned int *max_id)
{
    unsigned int mx = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const unsigned int v = in[i];
        out[i]               = (uint8_t)(v & 0xffu);
        mx                   = v > mx ? v : mx;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        mx = max(mx, __shfl_down_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0)
        atomicMax(max_id, mx);
}
} // namespace

cudaError_t launch_ms_convert(const uint16_t *in, uint8_t *out, long long n, unsigned int *max_id, cudaStream_t st)
{
    k_ms_convert<<<grid_blocks_for(n), kVecThreads, 0, st>>>(in, out, n, max_id);
    return cudaGetLastError();
}

template <typename T, typename TU>
cudaError_t launch_cg_update(const UpdateArgs &a, cudaStream_t st)
{
    const int nrhs = a.nrhs > 1 ? a.nrhs : 1;
    if (std::is_same<T, float>::value && std::is_same<TU, float>::value && a.n % 4 == 0)
        k_cg_update_f4<<<dim3(grid_blocks_for(a.n / 4), nrhs), kVecThreads, 0, st>>>(a);
    else if (nrhs == 1)
        k_cg_update<T, TU><<<grid_blocks_for(a.n), kVecThreads, 0, st>>>(a);
    else
        return cudaErrorInvalidValue; // several right-hand sides: the 16-byte FP32 update only
    return cudaGetLastError();
}

cudaError_t launch_norm_fast(const double *r, long long n, int measure, CgScalars *scal, int set_err0, float *r_out,
                             GridRed red, int site, cudaStream_t st)
{
    k_norm_fast<double, float><<<grid_blocks_for(n / 2), kVecThreads, 0, st>>>(r, n, measure, scal, set_err0, r_out,
                                                                              red, site);
    return cudaGetLastError();
}
template cudaError_t launch_cg_update<double, double>(const UpdateArgs &, cudaStream_t);
template cudaError_t launch_cg_update<float, float>(const UpdateArgs &, cudaStream_t);

template <typename T, typename TO>
cudaError_t launch_norm(const T *r, long long n, int measure, CgScalars *scal, int set_err0, TO *r_out, GridRed red,
                        int site, cudaStream_t st)
{
    k_norm<T, TO><<<grid_blocks_for(n), kVecThreads, 0, st>>>(r, n, measure, scal, set_err0, r_out, red, site);
    return cudaGetLastError();
}
template cudaError_t launch_norm<double, float>(const double *, long long, int, CgScalars *, int, float *, GridRed, int,
                                                cudaStream_t);
template cudaError_t launch_norm<float, float>(const float *, long long, int, CgScalars *, int, float *, GridRed, int,
                                               cudaStream_t);

template <typename T>
cudaError_t launch_axpy(T *y, const T *x, double a, long long n, cudaStream_t st)
{
    k_axpy<T><<<grid_blocks_for(n), kVecThreads, 0, st>>>(y, x, a, n);
    return cudaGetLastError();
}
template cudaError_t launch_axpy<double>(double *, const double *, double, long long, cudaStream_t);

cudaError_t launch_extrapolate(double *u, double *u_prev, long long n, cudaStream_t st)
{
    k_extrapolate<<<grid_blocks_for(n), kVecThreads, 0, st>>>(u, u_prev, n);
    return cudaGetLastError();
}

cudaError_t launch_fold(double *u, float *e, long long n, cudaStream_t st)
{
    k_fold<<<grid_blocks_for(n), kVecThreads, 0, st>>>(u, e, n);
    return cudaGetLastError();
}

} // namespace fansgpu
