// k_stencil.cu -- voxel-element kernels of the FANS solve path on sm_103a.
//
// The CG operator and the linear residual are node-centric gathers: node n sums
// the rows of its 8 surrounding elements' stiffness (solver.h:315-385 visits
// elements and scatters; gathering per node gives the same sum with no write
// conflicts, no atomics and a fixed summation order).  A CTA stages a
// (TX+2)x(TY+2)x(TZ+2) halo tile of the input field and the (TX+1)(TY+1)(TZ+1)
// element phases in shared memory with periodic wrap, then each thread computes
// TX nodes of one (y,z) column.
#include "kernels.cuh"

#include <cstring>

namespace fansgpu {

namespace {
constexpr int TX = 4, TY = 8, TZ = 32;
constexpr int HX = TX + 2, HY = TY + 2, HZ = TZ + 2;
constexpr int EX = TX + 1, EY = TY + 1, EZ = TZ + 1;
constexpr int kStencilThreads = TY * TZ; // 256

__device__ __forceinline__ int pmod(int i, int n)
{
    int r = i % n;
    return r < 0 ? r + n : r;
}

template <typename T, int C>
__global__ void __launch_bounds__(kStencilThreads) k_stencil(StencilArgs a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int nx = a.g.nx, ny = a.g.ny, nz = a.g.nz;
    const long long N = (long long)nx * ny * nz;
    constexpr int NC  = 8 * C;
    T       *xs  = reinterpret_cast<T *>(smem_raw);                 // C * HX*HY*HZ
    T       *Ks  = xs + C * HX * HY * HZ;                           // nph * NC*NC
    T       *fs  = Ks + (size_t)a.nph * NC * NC;                    // nph * NC (if fph)
    uint8_t *mss = reinterpret_cast<uint8_t *>(fs + (a.fph ? a.nph * NC : 0)); // EX*EY*EZ
    __shared__ double red_smem[32 * 2];

    const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY, z0 = blockIdx.z * TZ;
    const int tid = threadIdx.x;

    // stage per-phase tables
    const T *Kg = reinterpret_cast<const T *>(a.Kph);
    for (int i = tid; i < a.nph * NC * NC; i += blockDim.x)
        Ks[i] = Kg[i];
    if (a.fph) {
        const T *fg = reinterpret_cast<const T *>(a.fph);
        for (int i = tid; i < a.nph * NC; i += blockDim.x)
            fs[i] = fg[i];
    }
    // stage element phases of elements (x0-1 .. x0+TX-1, ...)
    for (int i = tid; i < EX * EY * EZ; i += blockDim.x) {
        int ez = i % EZ, ey = (i / EZ) % EY, ex = i / (EZ * EY);
        int gx = pmod(x0 - 1 + ex, nx), gy = pmod(y0 - 1 + ey, ny), gz = pmod(z0 - 1 + ez, nz);
        mss[i] = a.ms[((long long)gx * ny + gy) * nz + gz];
    }
    // stage the input field on nodes (x0-1 .. x0+TX, ...), computing d = s + beta d_old when fused
    const T     *xin  = reinterpret_cast<const T *>(a.x);
    const T     *dold = reinterpret_cast<const T *>(a.d_old);
    const double beta = a.fuse_d ? a.scal->beta : 0.0;
    for (int i = tid; i < (a.force_only ? 0 : HX * HY * HZ); i += blockDim.x) {
        int hz = i % HZ, hy = (i / HZ) % HY, hx = i / (HZ * HY);
        int gx = pmod(x0 - 1 + hx, nx), gy = pmod(y0 - 1 + hy, ny), gz = pmod(z0 - 1 + hz, nz);
        long long gi = ((long long)gx * ny + gy) * nz + gz;
#pragma unroll
        for (int c = 0; c < C; ++c) {
            T v = xin[c * N + gi];
            if (a.fuse_d)
                v = (T)((double)v + beta * (double)dold[c * N + gi]);
            xs[c * HX * HY * HZ + i] = v;
        }
    }
    __syncthreads();

    const int tz = tid % TZ, ty = tid / TZ;
    const int gy = y0 + ty, gz = z0 + tz;
    double    dot = 0.0;
    const bool col_ok = (gy < ny) && (gz < nz);
    for (int tx = 0; tx < TX; ++tx) {
        const int gx = x0 + tx;
        if (!col_ok || gx >= nx)
            break;
        // halo-tile coordinates of this node: (tx+1, ty+1, tz+1)
        const int hc = ((tx + 1) * HY + (ty + 1)) * HZ + (tz + 1);
        T         ctr[C];
#pragma unroll
        for (int c = 0; c < C; ++c)
            ctr[c] = a.force_only ? (T)0 : xs[c * HX * HY * HZ + hc];
        T acc[C];
#pragma unroll
        for (int c = 0; c < C; ++c)
            acc[c] = (T)0;
#pragma unroll
        for (int p = 0; p < 8; ++p) {
            const int a0 = p & 1, b0 = (p >> 1) & 1, c0 = (p >> 2) & 1;
            // element whose local node p is this node: origin (tx-a0, ty-b0, tz-c0)
            const int ex = tx - a0 + 1, ey = ty - b0 + 1, ez = tz - c0 + 1; // element-tile coords
            const int ph = mss[(ex * EY + ey) * EZ + ez];
            const T  *Kr = Ks + (size_t)ph * NC * NC + (size_t)(p * C) * NC;
            if (!a.force_only) {
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    const int qa = q & 1, qb = (q >> 1) & 1, qc = (q >> 2) & 1;
                    // node e + q in halo coordinates: (tx - a0 + qa + 1, ...)
                    const int hq = ((tx - a0 + qa + 1) * HY + (ty - b0 + qb + 1)) * HZ + (tz - c0 + qc + 1);
#pragma unroll
                    for (int cb = 0; cb < C; ++cb) {
                        const T v = xs[cb * HX * HY * HZ + hq] - ctr[cb];
#pragma unroll
                        for (int cr = 0; cr < C; ++cr)
                            acc[cr] += Kr[cr * NC + q * C + cb] * v;
                    }
                }
            }
            if (a.fph) {
                const T *fr = fs + (size_t)ph * NC + p * C;
#pragma unroll
                for (int cr = 0; cr < C; ++cr)
                    acc[cr] += fr[cr];
            }
        }
        const long long gi = ((long long)gx * ny + gy) * nz + gz;
        T *yout = reinterpret_cast<T *>(a.y);
#pragma unroll
        for (int c = 0; c < C; ++c) {
            yout[c * N + gi] = acc[c];
            if (a.reduce)
                dot += (double)ctr[c] * (double)acc[c];
        }
        if (a.fuse_d) {
            T *dn = reinterpret_cast<T *>(a.d_new);
#pragma unroll
            for (int c = 0; c < C; ++c)
                dn[c * N + gi] = ctr[c];
        }
    }
    if (a.reduce) {
        double    v[1]   = {dot};
        const int ops[1] = {RED_SUM};
        block_reduce<1>(v, ops, red_smem);
        const int nb = gridDim.x * gridDim.y * gridDim.z;
        double   *partials = a.red.partials;
        if (grid_partial_commit<1>(v, partials, a.red.counter + a.red_site, nb)) {
            grid_final<1>(v, ops, partials, nb, red_smem);
            if (threadIdx.x == 0) {
                a.scal->dAd   = v[0];
                a.scal->alpha = a.scal->delta / v[0];
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Same operator with the per-phase stiffness passed by value as a kernel
// parameter (constant bank): every coefficient is an immediate-offset operand
// of its FMA, so the inner product issues no shared-memory loads for K.  The
// 27-node neighbourhood (minus the centre value) sits in registers.  Phases are
// handled as warp-uniform branches: a warp pays for each phase present among
// its lanes' elements at a given element position.
template <typename T, int C, int NPH>
struct StencilCoef {
    T K[NPH][8 * C][8 * C];
    T f[NPH][8 * C];
};

template <typename T, int C, int NPH>
__global__ void __launch_bounds__(kStencilThreads)
    k_stencil_pk(StencilArgs a, const __grid_constant__ StencilCoef<T, C, NPH> P)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int nx = a.g.nx, ny = a.g.ny, nz = a.g.nz;
    const long long N = (long long)nx * ny * nz;
    constexpr int HXYZ = HX * HY * HZ;
    T       *xs  = reinterpret_cast<T *>(smem_raw);
    uint8_t *mss = reinterpret_cast<uint8_t *>(xs + C * HXYZ);
    __shared__ double red_smem[32 * 2];

    const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY, z0 = blockIdx.z * TZ;
    const int tid = threadIdx.x;
    for (int i = tid; i < EX * EY * EZ; i += blockDim.x) {
        int ez = i % EZ, ey = (i / EZ) % EY, ex = i / (EZ * EY);
        int gx = pmod(x0 - 1 + ex, nx), gy = pmod(y0 - 1 + ey, ny), gz = pmod(z0 - 1 + ez, nz);
        mss[i] = a.ms[((long long)gx * ny + gy) * nz + gz];
    }
    const T     *xin  = reinterpret_cast<const T *>(a.x);
    const T     *dold = reinterpret_cast<const T *>(a.d_old);
    const T      beta = a.fuse_d ? (T)a.scal->beta : (T)0;
    for (int i = tid; i < (a.force_only ? 0 : HXYZ); i += blockDim.x) {
        int hz = i % HZ, hy = (i / HZ) % HY, hx = i / (HZ * HY);
        int gx = pmod(x0 - 1 + hx, nx), gy = pmod(y0 - 1 + hy, ny), gz = pmod(z0 - 1 + hz, nz);
        long long gi = ((long long)gx * ny + gy) * nz + gz;
#pragma unroll
        for (int c = 0; c < C; ++c) {
            T v = xin[c * N + gi];
            if (a.fuse_d)
                v += beta * dold[c * N + gi];
            xs[c * HXYZ + i] = v;
        }
    }
    __syncthreads();

    const int  tz = tid % TZ, ty = tid / TZ;
    const int  gy = y0 + ty, gz = z0 + tz;
    const bool col_ok = (gy < ny) && (gz < nz);
    const bool with_f = a.fph != nullptr;
    double     dot    = 0.0;
    for (int tx = 0; tx < TX; ++tx) {
        const int  gx    = x0 + tx;
        const bool valid = col_ok && gx < nx;
        const int  hc    = ((tx + 1) * HY + (ty + 1)) * HZ + (tz + 1);
        T          ctr[C], xv[27][C], acc[C];
#pragma unroll
        for (int c = 0; c < C; ++c) {
            ctr[c] = a.force_only ? (T)0 : xs[c * HXYZ + hc];
            acc[c] = (T)0;
        }
#pragma unroll
        for (int dx = 0; dx < 3; ++dx)
#pragma unroll
            for (int dy = 0; dy < 3; ++dy)
#pragma unroll
                for (int dz = 0; dz < 3; ++dz) {
                    const int hq = ((tx + dx) * HY + (ty + dy)) * HZ + (tz + dz);
#pragma unroll
                    for (int c = 0; c < C; ++c)
                        xv[(dx * 3 + dy) * 3 + dz][c] = a.force_only ? (T)0 : xs[c * HXYZ + hq] - ctr[c];
                }
#pragma unroll
        for (int p = 0; p < 8; ++p) {
            const int a0 = p & 1, b0 = (p >> 1) & 1, c0 = (p >> 2) & 1;
            const int ph = mss[((tx - a0 + 1) * EY + (ty - b0 + 1)) * EZ + (tz - c0 + 1)];
#pragma unroll
            for (int k = 0; k < NPH; ++k) {
                const bool mine = (ph == k);
                if (NPH == 1 || __any_sync(0xffffffffu, mine)) {
                    if ((NPH == 1 || mine) && !a.force_only) {
#pragma unroll
                        for (int q = 0; q < 8; ++q) {
                            const int qa = q & 1, qb = (q >> 1) & 1, qc = (q >> 2) & 1;
                            const int nb = ((qa - a0 + 1) * 3 + (qb - b0 + 1)) * 3 + (qc - c0 + 1);
#pragma unroll
                            for (int cb = 0; cb < C; ++cb)
#pragma unroll
                                for (int cr = 0; cr < C; ++cr)
                                    acc[cr] += P.K[k][p * C + cr][q * C + cb] * xv[nb][cb];
                        }
                    }
                    if ((NPH == 1 || mine) && with_f) {
#pragma unroll
                        for (int cr = 0; cr < C; ++cr)
                            acc[cr] += P.f[k][p * C + cr];
                    }
                }
            }
        }
        if (valid) {
            const long long gi   = ((long long)gx * ny + gy) * nz + gz;
            T              *yout = reinterpret_cast<T *>(a.y);
            T dl = (T)0;
#pragma unroll
            for (int c = 0; c < C; ++c) {
                yout[c * N + gi] = acc[c];
                dl += ctr[c] * acc[c];
            }
            dot += (double)dl;
            if (a.fuse_d) {
                T *dn = reinterpret_cast<T *>(a.d_new);
#pragma unroll
                for (int c = 0; c < C; ++c)
                    dn[c * N + gi] = ctr[c];
            }
        }
    }
    if (a.reduce) {
        double    v[1]   = {dot};
        const int ops[1] = {RED_SUM};
        block_reduce<1>(v, ops, red_smem);
        const int nb = gridDim.x * gridDim.y * gridDim.z;
        if (grid_partial_commit<1>(v, a.red.partials, a.red.counter + a.red_site, nb)) {
            grid_final<1>(v, ops, a.red.partials, nb, red_smem);
            if (threadIdx.x == 0) {
                a.scal->dAd   = v[0];
                a.scal->alpha = a.scal->delta / v[0];
            }
        }
    }
}

template <typename T, int C, int NPH>
cudaError_t launch_stencil_pk(const StencilArgs &a, cudaStream_t st)
{
    constexpr int NC = 8 * C;
    StencilCoef<T, C, NPH> P;
    std::memset(&P, 0, sizeof P);
    const T *Kh = reinterpret_cast<const T *>(a.Kph_host);
    const T *fh = reinterpret_cast<const T *>(a.fph_host);
    for (int k = 0; k < a.nph; ++k)
        for (int i = 0; i < NC; ++i) {
            for (int j = 0; j < NC; ++j)
                P.K[k][i][j] = Kh[((size_t)k * NC + i) * NC + j];
            P.f[k][i] = fh ? fh[(size_t)k * NC + i] : (T)0;
        }
    dim3         grid((a.g.nx + TX - 1) / TX, (a.g.ny + TY - 1) / TY, (a.g.nz + TZ - 1) / TZ);
    const size_t sm = sizeof(T) * (size_t)C * HX * HY * HZ + EX * EY * EZ;
    cudaError_t  e  = allow_max_dyn_smem(k_stencil_pk<T, C, NPH>);
    if (e != cudaSuccess)
        return e;
    k_stencil_pk<T, C, NPH><<<grid, kStencilThreads, sm, st>>>(a, P);
    return cudaGetLastError();
}

template <typename T, int C>
size_t stencil_smem(const StencilArgs &a)
{
    constexpr int NC = 8 * C;
    size_t        b  = sizeof(T) * ((size_t)C * HX * HY * HZ + (size_t)a.nph * NC * NC + (a.fph ? a.nph * NC : 0));
    return b + EX * EY * EZ;
}

template <typename T, int C>
cudaError_t launch_stencil_c(const StencilArgs &a, cudaStream_t st)
{
    // FP32: stiffness as kernel-parameter operands; FP64 stays on the shared-
    // memory variant, which keeps more warps resident for the FP64 pipe.
    if (sizeof(T) == 4 && a.Kph_host && (!a.fph || a.fph_host)) {
        if (a.nph <= 1)
            return launch_stencil_pk<T, C, 1>(a, st);
        if (a.nph <= 2)
            return launch_stencil_pk<T, C, 2>(a, st);
        if (a.nph <= 4)
            return launch_stencil_pk<T, C, 4>(a, st);
    }
    dim3   grid((a.g.nx + TX - 1) / TX, (a.g.ny + TY - 1) / TY, (a.g.nz + TZ - 1) / TZ);
    size_t sm = stencil_smem<T, C>(a);
    cudaError_t e = allow_max_dyn_smem(k_stencil<T, C>);
    if (e != cudaSuccess)
        return e;
    k_stencil<T, C><<<grid, kStencilThreads, sm, st>>>(a);
    return cudaGetLastError();
}

// ------------------------------------------------------------ strain/stress --
template <int C, int NSTR>
__global__ void __launch_bounds__(256) k_strain_stress(StrainStressArgs a)
{
    const double     *Cs = a.Cph; // per-phase constitutive matrices (read through L1)
    __shared__ double red_smem[32 * (2 * NSTR + 1)];
    const int         nx = a.g.nx, ny = a.g.ny, nz = a.g.nz;
    const long long   N  = (long long)nx * ny * nz;
    double se[NSTR], ss[NSTR], cnt = 0.0;
#pragma unroll
    for (int i = 0; i < NSTR; ++i)
        se[i] = ss[i] = 0.0;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < N; e += (long long)gridDim.x * blockDim.x) {
        const int z = (int)(e % nz), y = (int)((e / nz) % ny), x = (int)(e / ((long long)nz * ny));
        const int ph = a.ms[e];
        const bool take = (a.phase_filter < 0) || (a.phase_filter == ph);
        if (!take && !a.strain && !a.stress)
            continue;
        const int x1 = x + 1 == nx ? 0 : x + 1, y1 = y + 1 == ny ? 0 : y + 1, z1 = z + 1 == nz ? 0 : z + 1;
        long long idx[8];
        idx[0] = ((long long)x * ny + y) * nz + z;
        idx[1] = ((long long)x1 * ny + y) * nz + z;
        idx[2] = ((long long)x * ny + y1) * nz + z;
        idx[3] = ((long long)x1 * ny + y1) * nz + z;
        idx[4] = ((long long)x * ny + y) * nz + z1;
        idx[5] = ((long long)x1 * ny + y) * nz + z1;
        idx[6] = ((long long)x * ny + y1) * nz + z1;
        idx[7] = ((long long)x1 * ny + y1) * nz + z1;
        // GP-averaged gradient = gradient at the element centre (true for HEX8,
        // HEX8R and BBAR): mean of the four edge differences per direction.
        double g[C][3];
#pragma unroll
        for (int c = 0; c < C; ++c) {
            double u[8];
#pragma unroll
            for (int q = 0; q < 8; ++q)
                u[q] = a.u[c * N + idx[q]];
            g[c][0] = ((u[1] - u[0]) + (u[3] - u[2]) + (u[5] - u[4]) + (u[7] - u[6])) * a.inv4l[0];
            g[c][1] = ((u[2] - u[0]) + (u[3] - u[1]) + (u[6] - u[4]) + (u[7] - u[5])) * a.inv4l[1];
            g[c][2] = ((u[4] - u[0]) + (u[5] - u[1]) + (u[6] - u[2]) + (u[7] - u[3])) * a.inv4l[2];
        }
        double eps[NSTR];
        if (C == 1) {
#pragma unroll
            for (int i = 0; i < 3; ++i)
                eps[i] = g[0][i];
        } else {
            const double sh = 7.071067811865476e-01; // sqrt(1/2), matmodel.h:288
            eps[0] = g[0][0];
            eps[1] = g[C > 1 ? 1 : 0][1];
            eps[2] = g[C > 2 ? 2 : 0][2];
            eps[3] = sh * (g[0][1] + g[C > 1 ? 1 : 0][0]);
            eps[4] = sh * (g[0][2] + g[C > 2 ? 2 : 0][0]);
            eps[5] = sh * (g[C > 1 ? 1 : 0][2] + g[C > 2 ? 2 : 0][1]);
        }
        double sig[NSTR];
#pragma unroll
        for (int i = 0; i < NSTR; ++i)
            eps[i] += a.g0[i];
#pragma unroll
        for (int i = 0; i < NSTR; ++i) {
            double acc = 0.0;
#pragma unroll
            for (int k = 0; k < NSTR; ++k)
                acc += Cs[(ph * NSTR + i) * NSTR + k] * eps[k];
            sig[i] = acc;
        }
        if (a.strain)
#pragma unroll
            for (int i = 0; i < NSTR; ++i)
                a.strain[e * NSTR + i] = eps[i];
        if (a.stress)
#pragma unroll
            for (int i = 0; i < NSTR; ++i)
                a.stress[e * NSTR + i] = sig[i];
        if (take) {
#pragma unroll
            for (int i = 0; i < NSTR; ++i) {
                se[i] += eps[i];
                ss[i] += sig[i];
            }
            cnt += 1.0;
        }
    }
    double v[2 * NSTR + 1];
    int    ops[2 * NSTR + 1];
#pragma unroll
    for (int i = 0; i < NSTR; ++i) {
        v[i]        = se[i];
        v[NSTR + i] = ss[i];
    }
    v[2 * NSTR] = cnt;
#pragma unroll
    for (int i = 0; i < 2 * NSTR + 1; ++i)
        ops[i] = RED_SUM;
    block_reduce<2 * NSTR + 1>(v, ops, red_smem);
    if (grid_partial_commit<2 * NSTR + 1>(v, a.red.partials, a.red.counter + a.red_site, gridDim.x)) {
        grid_final<2 * NSTR + 1>(v, ops, a.red.partials, gridDim.x, red_smem);
        if (threadIdx.x == 0)
            for (int i = 0; i < 2 * NSTR + 1; ++i)
                a.out_red[i] = v[i];
    }
}

// ----------------------------------------------------------------- layout ---
template <typename TI, typename TO>
__global__ void k_aos_to_soa(const TI *__restrict__ aos, TO *__restrict__ soa, long long N, int C)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N * C; i += (long long)gridDim.x * blockDim.x) {
        long long node = i / C;
        int       c    = (int)(i % C);
        soa[c * N + node] = (TO)aos[i];
    }
}
template <typename TI, typename TO>
__global__ void k_soa_to_aos(const TI *__restrict__ soa, TO *__restrict__ aos, long long N, int C)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N * C; i += (long long)gridDim.x * blockDim.x) {
        long long node = i / C;
        int       c    = (int)(i % C);
        aos[i] = (TO)soa[c * N + node];
    }
}
template <typename TI, typename TO>
__global__ void k_convert(const TI *__restrict__ in, TO *__restrict__ out, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = (TO)in[i];
}

// ---------------------------------------------------------------------------
// R(u) = K u + F with FP64 accuracy from FP32 arithmetic (double-float).  GB300
// issues FP64 at a small fraction of its FP32 rate, so the mixed path's true
// residual is evaluated with error-free transformations instead of DFMA:
//   * each FP64 input value is split into hi + lo FP32 parts in the tile;
//   * neighbour differences u_q - u_c are formed with TwoSum (exact hi part);
//   * K (hi + lo) times the difference uses the exact FMA product error;
//   * the row sums accumulate in (S_hi, S_lo) with TwoSum.
// The result is written as FP64 (S_hi + S_lo); its error is ~2^-47 of the
// summed magnitudes, far below what a 1e-8 relative tolerance needs.
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e)
{
    s       = a + b;
    float z = s - a;
    e       = (a - (s - z)) + (b - z);
}

template <int C>
__global__ void __launch_bounds__(kStencilThreads) k_residual_df(StencilArgs a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int nx = a.g.nx, ny = a.g.ny, nz = a.g.nz;
    const long long N = (long long)nx * ny * nz;
    constexpr int NC = 8 * C, HXYZ = HX * HY * HZ;
    float   *xh  = reinterpret_cast<float *>(smem_raw);  // C * HXYZ
    float   *xl  = xh + C * HXYZ;                        // C * HXYZ
    float   *Kh  = xl + C * HXYZ;                        // nph * NC * NC
    float   *Kl  = Kh + (size_t)a.nph * NC * NC;         // nph * NC * NC
    uint8_t *mss = reinterpret_cast<uint8_t *>(Kl + (size_t)a.nph * NC * NC);

    const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY, z0 = blockIdx.z * TZ;
    const int tid = threadIdx.x;
    const float *Kg = reinterpret_cast<const float *>(a.Kph); // [hi | lo]
    for (int i = tid; i < a.nph * NC * NC; i += blockDim.x) {
        Kh[i] = Kg[i];
        Kl[i] = Kg[(size_t)a.nph * NC * NC + i];
    }
    for (int i = tid; i < EX * EY * EZ; i += blockDim.x) {
        int ez = i % EZ, ey = (i / EZ) % EY, ex = i / (EZ * EY);
        int gx = pmod(x0 - 1 + ex, nx), gy = pmod(y0 - 1 + ey, ny), gz = pmod(z0 - 1 + ez, nz);
        mss[i] = a.ms[((long long)gx * ny + gy) * nz + gz];
    }
    // x = u, or with fuse_d the CG direction d = s + beta d_old in FP64 (written to d_new
    // for the nodes this CTA owns)
    const double *u    = reinterpret_cast<const double *>(a.x);
    const double *dold = reinterpret_cast<const double *>(a.d_old);
    double       *dnew = reinterpret_cast<double *>(a.d_new);
    const double  beta = a.fuse_d ? a.scal->beta : 0.0;
    for (int i = tid; i < HXYZ; i += blockDim.x) {
        int hz = i % HZ, hy = (i / HZ) % HY, hx = i / (HZ * HY);
        int gx = pmod(x0 - 1 + hx, nx), gy = pmod(y0 - 1 + hy, ny), gz = pmod(z0 - 1 + hz, nz);
        long long gi = ((long long)gx * ny + gy) * nz + gz;
        const bool own = a.fuse_d && hx >= 1 && hx <= TX && hy >= 1 && hy <= TY && hz >= 1 && hz <= TZ &&
                         x0 - 1 + hx < nx && y0 - 1 + hy < ny && z0 - 1 + hz < nz;
#pragma unroll
        for (int c = 0; c < C; ++c) {
            double v = u[c * N + gi];
            if (a.fuse_d)
                v = v + beta * dold[c * N + gi];
            if (own)
                dnew[c * N + gi] = v;
            const float hi = (float)v;
            xh[c * HXYZ + i] = hi;
            xl[c * HXYZ + i] = (float)(v - (double)hi);
        }
    }
    __syncthreads();
    double dot = 0.0; // <x, y> of this thread's nodes (reduce)

    const float *fg = reinterpret_cast<const float *>(a.fph); // [hi | lo], nph * NC each
    const int  tz = tid % TZ, ty = tid / TZ;
    const int  gy = y0 + ty, gz = z0 + tz;
    const bool col_ok = (gy < ny) && (gz < nz);
    for (int tx = 0; tx < TX; ++tx) {
        const int gx = x0 + tx;
        if (!col_ok || gx >= nx)
            break;
        const int hc = ((tx + 1) * HY + (ty + 1)) * HZ + (tz + 1);
        float     ch[C], cl[C], Sh[C], Sl[C];
#pragma unroll
        for (int c = 0; c < C; ++c) {
            ch[c] = xh[c * HXYZ + hc];
            cl[c] = xl[c * HXYZ + hc];
            Sh[c] = 0.f;
            Sl[c] = 0.f;
        }
#pragma unroll
        for (int p = 0; p < 8; ++p) {
            const int    a0 = p & 1, b0 = (p >> 1) & 1, c0 = (p >> 2) & 1;
            const int    ph = mss[((tx - a0 + 1) * EY + (ty - b0 + 1)) * EZ + (tz - c0 + 1)];
            const float *kh = Kh + (size_t)ph * NC * NC + (size_t)(p * C) * NC;
            const float *kl = Kl + (size_t)ph * NC * NC + (size_t)(p * C) * NC;
            // element-local double-float accumulators: independent chains per element
            float Eh[C], El[C];
#pragma unroll
            for (int cr = 0; cr < C; ++cr) {
                Eh[cr] = 0.f;
                El[cr] = 0.f;
            }
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const int qa = q & 1, qb = (q >> 1) & 1, qc = (q >> 2) & 1;
                const int hq = ((tx - a0 + qa + 1) * HY + (ty - b0 + qb + 1)) * HZ + (tz - c0 + qc + 1);
#pragma unroll
                for (int cb = 0; cb < C; ++cb) {
                    float dh, de;
                    two_sum(xh[cb * HXYZ + hq], -ch[cb], dh, de);
                    const float dl = de + (xl[cb * HXYZ + hq] - cl[cb]);
#pragma unroll
                    for (int cr = 0; cr < C; ++cr) {
                        const float k1 = kh[cr * NC + q * C + cb], k2 = kl[cr * NC + q * C + cb];
                        const float pr = k1 * dh;
                        const float pe = fmaf(k1, dh, -pr);
                        const float lo = fmaf(k1, dl, fmaf(k2, dh, pe));
                        float       t, e;
                        two_sum(Eh[cr], pr, t, e);
                        Eh[cr] = t;
                        El[cr] += e + lo;
                    }
                }
            }
#pragma unroll
            for (int cr = 0; cr < C; ++cr) {
                float t, e;
                two_sum(Sh[cr], Eh[cr], t, e);
                Sh[cr] = t;
                Sl[cr] += e + El[cr];
            }
            if (fg)
#pragma unroll
                for (int cr = 0; cr < C; ++cr) {
                    float t, e;
                    two_sum(Sh[cr], fg[(size_t)ph * NC + p * C + cr], t, e);
                    Sh[cr] = t;
                    Sl[cr] += e + fg[(size_t)a.nph * NC + (size_t)ph * NC + p * C + cr];
                }
        }
        const long long gi   = ((long long)gx * ny + gy) * nz + gz;
        double         *yout = reinterpret_cast<double *>(a.y);
#pragma unroll
        for (int c = 0; c < C; ++c) {
            const double yv = (double)Sh[c] + (double)Sl[c];
            yout[c * N + gi] = yv;
            if (a.reduce)
                dot += ((double)ch[c] + (double)cl[c]) * yv;
        }
    }
    if (a.reduce) { // <d, K d> and alpha = delta / <d, K d> (solverCG.h:101)
        __shared__ double red_smem[32];
        double    v[1]   = {dot};
        const int ops[1] = {RED_SUM};
        block_reduce<1>(v, ops, red_smem);
        const int nb = gridDim.x * gridDim.y * gridDim.z;
        if (grid_partial_commit<1>(v, a.red.partials, a.red.counter + a.red_site, nb)) {
            grid_final<1>(v, ops, a.red.partials, nb, red_smem);
            if (threadIdx.x == 0) {
                a.scal->dAd   = v[0];
                a.scal->alpha = a.scal->delta / v[0];
            }
        }
    }
}

} // namespace

int grid_blocks_for(long long n)
{
    long long b = (n + 255) / 256;
    const long long cap = 152LL * 16;
    return (int)(b < cap ? (b < 1 ? 1 : b) : cap);
}

long long stencil_blocks(const Grid3 &g)
{
    return (long long)((g.nx + TX - 1) / TX) * ((g.ny + TY - 1) / TY) * ((g.nz + TZ - 1) / TZ);
}

template <typename T>
cudaError_t launch_stencil(const StencilArgs &a, cudaStream_t st)
{
    if (a.C == 1)
        return launch_stencil_c<T, 1>(a, st);
    return launch_stencil_c<T, 3>(a, st);
}
template cudaError_t launch_stencil<double>(const StencilArgs &, cudaStream_t);
template cudaError_t launch_stencil<float>(const StencilArgs &, cudaStream_t);

cudaError_t launch_residual_df(const StencilArgs &a, cudaStream_t st)
{
    dim3         grid((a.g.nx + TX - 1) / TX, (a.g.ny + TY - 1) / TY, (a.g.nz + TZ - 1) / TZ);
    const int    NC = 8 * a.C;
    const size_t sm = sizeof(float) * (2 * (size_t)a.C * HX * HY * HZ + 2 * (size_t)a.nph * NC * NC) + EX * EY * EZ;
    cudaError_t  e;
    if (a.C == 1) {
        if ((e = allow_max_dyn_smem(k_residual_df<1>)))
            return e;
        k_residual_df<1><<<grid, kStencilThreads, sm, st>>>(a);
    } else {
        if ((e = allow_max_dyn_smem(k_residual_df<3>)))
            return e;
        k_residual_df<3><<<grid, kStencilThreads, sm, st>>>(a);
    }
    return cudaGetLastError();
}

// Per-phase sums of the element strain (centre gradient + g0) and element
// counts for at most two phases: out[ph*NSTR + i], out[2*NSTR + ph].  With
// linear laws the stress sums follow on the host as C_ph times the strain sums
// (matmodel.h:203-225 by linearity), so the averages need no per-element stress.
//
// The element strain average is the centre gradient of u (the Gauss-point mean
// of B for HEX8, HEX8R and BBAR): du_c/dx_d = (sum of u_c over the element's
// four far-d corners - the four near-d corners) / (4 l_d).  Summed over the
// phase-0 elements this is sum_n u_c(n) w_d(n) / (4 l_d), where w_d(n) =
// (# phase-0 elements having n as a far-d corner) - (# having it as a near-d
// corner) is an integer in [-4, 4] read from the 8 elements around node n.  Over
// all elements the sum vanishes (periodicity), so phase 1 carries minus phase 0.
// One thread per node: 3C FP64 FMAs instead of ~30C FP64 operations per
// element -- FP64 is the scarce pipe on this part.
template <int C, int NSTR>
__global__ void __launch_bounds__(256) k_strain_sums(StrainStressArgs a)
{
    constexpr int NV = 3 * C + 1; // sum_n u_c w_d at c*3 + d, then the phase-0 element count
    static_assert(NV <= kMaxRed, "reduction partial slots");
    __shared__ double red_smem[32 * NV];
    const int nx = a.g.nx, ny = a.g.ny, nz = a.g.nz;
    const long long N = (long long)nx * ny * nz;
    double acc[NV];
#pragma unroll
    for (int i = 0; i < NV; ++i)
        acc[i] = 0.0;
    for (int row = blockIdx.x; row < nx * ny; row += gridDim.x) {
        const int x = row / ny, y = row % ny;
        const int xm = x == 0 ? nx - 1 : x - 1, ym = y == 0 ? ny - 1 : y - 1;
        const long long r00 = ((long long)x * ny + y) * nz, r10 = ((long long)xm * ny + y) * nz;
        const long long r01 = ((long long)x * ny + ym) * nz, r11 = ((long long)xm * ny + ym) * nz;
        for (int z = threadIdx.x; z < nz; z += blockDim.x) {
            const int zm = z == 0 ? nz - 1 : z - 1;
            // element with origin node - (a, b, c): node n is its corner (a, b, c)
            const int p000 = a.ms[r00 + z] == 0, p001 = a.ms[r00 + zm] == 0;
            const int p010 = a.ms[r01 + z] == 0, p011 = a.ms[r01 + zm] == 0;
            const int p100 = a.ms[r10 + z] == 0, p101 = a.ms[r10 + zm] == 0;
            const int p110 = a.ms[r11 + z] == 0, p111 = a.ms[r11 + zm] == 0;
            const int far_x = p100 + p101 + p110 + p111, near_x = p000 + p001 + p010 + p011;
            const int far_y = p010 + p011 + p110 + p111, near_y = p000 + p001 + p100 + p101;
            const int far_z = p001 + p011 + p101 + p111, near_z = p000 + p010 + p100 + p110;
            const double w[3] = {(double)(far_x - near_x), (double)(far_y - near_y), (double)(far_z - near_z)};
#pragma unroll
            for (int c = 0; c < C; ++c) {
                const double u = a.u[c * N + r00 + z];
#pragma unroll
                for (int d = 0; d < 3; ++d)
                    acc[c * 3 + d] = fma(w[d], u, acc[c * 3 + d]);
            }
            acc[3 * C] += (double)p000;
        }
    }
    int ops[NV];
#pragma unroll
    for (int i = 0; i < NV; ++i)
        ops[i] = RED_SUM;
    block_reduce<NV>(acc, ops, red_smem);
    if (grid_partial_commit<NV>(acc, a.red.partials, a.red.counter + a.red_site, gridDim.x)) {
        grid_final<NV>(acc, ops, a.red.partials, gridDim.x, red_smem);
        if (threadIdx.x == 0) {
            double G[C][3]; // sum over phase-0 elements of du_c/dx_d
            for (int c = 0; c < C; ++c)
                for (int d = 0; d < 3; ++d)
                    G[c][d] = acc[c * 3 + d] * a.inv4l[d];
            double sgrad[NSTR];
            if (C == 1) {
                for (int i = 0; i < 3; ++i)
                    sgrad[i] = G[0][i];
            } else {
                const double sh = 7.071067811865476e-01;
                sgrad[0] = G[0][0];
                sgrad[1] = G[C > 1 ? 1 : 0][1];
                sgrad[2] = G[C > 2 ? 2 : 0][2];
                sgrad[3] = sh * (G[0][1] + G[C > 1 ? 1 : 0][0]);
                sgrad[4] = sh * (G[0][2] + G[C > 2 ? 2 : 0][0]);
                sgrad[5] = sh * (G[C > 1 ? 1 : 0][2] + G[C > 2 ? 2 : 0][1]);
            }
            const double n0 = acc[3 * C], n1 = (double)N - n0;
            for (int i = 0; i < NSTR; ++i) {
                a.out_red[i]        = sgrad[i] + n0 * a.g0[i];
                a.out_red[NSTR + i] = -sgrad[i] + n1 * a.g0[i];
            }
            a.out_red[2 * NSTR]     = n0;
            a.out_red[2 * NSTR + 1] = n1;
        }
    }
}

cudaError_t launch_strain_sums(const StrainStressArgs &a, cudaStream_t st)
{
    const long long rows = (long long)a.g.nx * a.g.ny;
    const int       nb   = (int)(rows < 152 * 8 ? rows : 152 * 8);
    if (a.nph > 2)
        return cudaErrorInvalidValue;
    if (a.C == 1)
        k_strain_sums<1, 3><<<nb, 256, 0, st>>>(a);
    else
        k_strain_sums<3, 6><<<nb, 256, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_strain_stress(const StrainStressArgs &a, cudaStream_t st)
{
    const int nb = grid_blocks_for(a.g.N());
    if (a.C == 1)
        k_strain_stress<1, 3><<<nb, 256, 0, st>>>(a);
    else
        k_strain_stress<3, 6><<<nb, 256, 0, st>>>(a);
    return cudaGetLastError();
}

// r = F(g0) alone (u = 0, the initial residual of a load case, solver.h:231-270 with zero u):
// node (x, y, z) sums row p of the g0 force of the element whose local node p it is, p = 0..7,
// in that order.  With at most two phases the 8 element phases form an 8-bit key and `table`
// holds the 256 sums per component, made on the host in the same order (bitwise the sums the
// full stencil forms), so a node costs 8 phase loads and C stores.
template <int C>
__global__ void __launch_bounds__(256) k_force_nodes(const uint8_t *__restrict__ ms, const double *__restrict__ table,
                                                     double *__restrict__ y, Grid3 g)
{
    __shared__ double T[256 * C];
    for (int i = threadIdx.x; i < 256 * C; i += blockDim.x)
        T[i] = table[i];
    __syncthreads();
    const int       nx = g.nx, ny = g.ny, nz = g.nz;
    const long long N  = (long long)nx * ny * nz;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (long long)gridDim.x * blockDim.x) {
        const int z = (int)(i % nz), yy = (int)((i / nz) % ny), x = (int)(i / ((long long)ny * nz));
        unsigned  key = 0;
#pragma unroll
        for (int p = 0; p < 8; ++p) {
            const int ex = pmod(x - (p & 1), nx), ey = pmod(yy - ((p >> 1) & 1), ny), ez = pmod(z - ((p >> 2) & 1), nz);
            key |= (unsigned)(ms[((long long)ex * ny + ey) * nz + ez] & 1) << p;
        }
#pragma unroll
        for (int c = 0; c < C; ++c)
            y[c * N + i] = T[key * C + c];
    }
}

cudaError_t launch_force_nodes(const Grid3 &g, int C, const uint8_t *ms, const double *table, double *y, cudaStream_t st)
{
    const long long N  = (long long)g.nx * g.ny * g.nz;
    const int       nb = grid_blocks_for(N);
    if (C == 3)
        k_force_nodes<3><<<nb, 256, 0, st>>>(ms, table, y, g);
    else if (C == 1)
        k_force_nodes<1><<<nb, 256, 0, st>>>(ms, table, y, g);
    else
        return cudaErrorInvalidValue;
    return cudaGetLastError();
}

template <typename TI, typename TO>
cudaError_t launch_aos_to_soa(const TI *aos, TO *soa, long long N, int C, cudaStream_t st)
{
    k_aos_to_soa<TI, TO><<<grid_blocks_for(N * C), 256, 0, st>>>(aos, soa, N, C);
    return cudaGetLastError();
}
template <typename TI, typename TO>
cudaError_t launch_soa_to_aos(const TI *soa, TO *aos, long long N, int C, cudaStream_t st)
{
    k_soa_to_aos<TI, TO><<<grid_blocks_for(N * C), 256, 0, st>>>(soa, aos, N, C);
    return cudaGetLastError();
}
template <typename TI, typename TO>
cudaError_t launch_convert(const TI *in, TO *out, long long n, cudaStream_t st)
{
    k_convert<TI, TO><<<grid_blocks_for(n), 256, 0, st>>>(in, out, n);
    return cudaGetLastError();
}
template cudaError_t launch_aos_to_soa<double, double>(const double *, double *, long long, int, cudaStream_t);
template cudaError_t launch_soa_to_aos<double, double>(const double *, double *, long long, int, cudaStream_t);
template cudaError_t launch_convert<double, float>(const double *, float *, long long, cudaStream_t);
template cudaError_t launch_convert<float, double>(const float *, double *, long long, cudaStream_t);

} // namespace fansgpu
