// k_fft.cu -- the Green's-operator convolution s = IFFT(G . FFT(r)) as five
// shared-memory passes over HBM, plus the Green's table builder.
//
//   z-fwd : r2c along z of each real row (half-length complex FFT + unpack)
//   y-fwd : complex FFT along y of (x, kz-chunk) tiles
//   x     : complex FFT along x of (ky, kz-chunk) tiles for all C components,
//           Green multiply (C x C real symmetric per frequency), inverse FFT
//           along x -- the forward and inverse x transforms never leave smem
//   y-inv : inverse along y
//   z-inv : Hermitian pack + half-length inverse FFT to real rows, scaled by
//           `sign` (the CG negation s *= -1 of solverCG.h:90), fused <r, s>
// Transforms are unnormalised (FFTW convention); the 1/N lives in G
// (solver.h:198).  Spectrum layout: [c][kx][ky][kz], row stride nzp >= nz/2+1.
#include "kernels.cuh"

namespace fansgpu {

namespace {
constexpr int kFftThreads = 256;

template <typename T>
__device__ __forceinline__ void load_tw(cplx<T> *dst, const cplx<T> *src, int n)
{
    for (int i = threadIdx.x; i < n; i += blockDim.x)
        dst[i] = src[i];
}

// ------------------------------------------------------------------ z fwd ---
template <typename T>
__global__ void __launch_bounds__(kFftThreads) k_z_fwd(ConvPlan<T> p, const T *__restrict__ r, int rows_per_cta)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int M = p.M, nzh = p.nzh;
    cplx<T>  *A  = reinterpret_cast<cplx<T> *>(smem_raw);
    cplx<T>  *B  = A + rows_per_cta * M;
    cplx<T>  *tw = B + rows_per_cta * M;
    cplx<T>  *tr = tw + M;
    load_tw(tw, p.tw_z, M);
    load_tw(tr, p.tw_r2c, M + 1);
    const long long nrows = (long long)p.C * p.g.nx * p.g.ny;
    const long long row0  = (long long)blockIdx.x * rows_per_cta;
    const int       nl    = (int)min((long long)rows_per_cta, nrows - row0);
    const cplx<T>  *rin   = reinterpret_cast<const cplx<T> *>(r);
    for (int i = threadIdx.x; i < nl * M; i += blockDim.x)
        A[i] = rin[(row0 + i / M) * M + (i % M)];
    __syncthreads();
    cplx<T> *Z = fft_lines<T, false, false>(A, B, p.dz, nl, 1, M, 1, tw, threadIdx.x, blockDim.x);
    for (int i = threadIdx.x; i < nl * nzh; i += blockDim.x) {
        const int L = i / nzh, k = i % nzh;
        cplx<T>   zk = Z[L * M + (k == M ? 0 : k)];
        cplx<T>   zm = Z[L * M + (k == 0 ? 0 : M - k)];
        zm.y         = -zm.y;
        cplx<T> E    = {(T)0.5 * (zk.x + zm.x), (T)0.5 * (zk.y + zm.y)};
        cplx<T> O    = {(T)0.5 * (zk.x - zm.x), (T)0.5 * (zk.y - zm.y)};
        cplx<T> P    = cmul(tr[k], O); // W^k O
        // X_k = E - i W^k O
        p.spec[(row0 + L) * p.nzp + k] = cplx<T>{E.x + P.y, E.y - P.x};
    }
}

// ------------------------------------------------------------------ y pass ---
template <typename T, bool INV>
__global__ void __launch_bounds__(kFftThreads) k_y(ConvPlan<T> p)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int KC = p.kc_y, ny = p.g.ny;
    cplx<T>  *A  = reinterpret_cast<cplx<T> *>(smem_raw);
    cplx<T>  *B  = A + ny * KC;
    cplx<T>  *tw = B + ny * KC;
    load_tw(tw, p.tw_y, ny);
    const int kz0 = blockIdx.x * KC, x = blockIdx.y, comp = blockIdx.z;
    const int nk  = min(KC, p.nzh - kz0);
    cplx<T>  *base = p.spec + ((long long)comp * p.g.nx + x) * ny * p.nzp + kz0;
    for (int i = threadIdx.x; i < ny * KC; i += blockDim.x) {
        const int y = i / KC, l = i % KC;
        A[i]        = (l < nk) ? base[(long long)y * p.nzp + l] : cplx<T>{0, 0};
    }
    __syncthreads();
    cplx<T> *R = fft_lines<T, INV, true>(A, B, p.dy, KC, KC, 0, KC, tw, threadIdx.x, blockDim.x);
    for (int i = threadIdx.x; i < ny * KC; i += blockDim.x) {
        const int y = i / KC, l = i % KC;
        if (l < nk)
            base[(long long)y * p.nzp + l] = R[i];
    }
}

// ----------------------------------------------------- x pass + Green's op ---
template <typename T, int C>
__global__ void __launch_bounds__(kFftThreads) k_x_green(ConvPlan<T> p)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int KC = p.kc_x, nx = p.g.nx, ny = p.g.ny;
    cplx<T>  *A  = reinterpret_cast<cplx<T> *>(smem_raw);
    cplx<T>  *B  = A + C * nx * KC;
    cplx<T>  *tw = B + C * nx * KC;
    load_tw(tw, p.tw_x, nx);
    const int kz0 = blockIdx.x * KC, ky = blockIdx.y;
    const int nk  = min(KC, p.nzh - kz0);
    for (int i = threadIdx.x; i < C * nx * KC; i += blockDim.x) {
        const int comp = i / (nx * KC), rem = i % (nx * KC), x = rem / KC, l = rem % KC;
        A[i] = (l < nk) ? p.spec[(((long long)comp * nx + x) * ny + ky) * p.nzp + kz0 + l] : cplx<T>{0, 0};
    }
    __syncthreads();
    cplx<T> *F = fft_lines<T, false, true>(A, B, p.dx, C * KC, KC, nx * KC, KC, tw, threadIdx.x, blockDim.x);
    constexpr int NT = C * (C + 1) / 2;
    for (int i = threadIdx.x; i < nx * KC; i += blockDim.x) {
        const int x = i / KC, l = i % KC;
        if (l >= nk)
            continue;
        const T *g = p.G + (((long long)x * ny + ky) * p.gzs + kz0 + l) * NT;
        T        gm[NT];
#pragma unroll
        for (int t = 0; t < NT; ++t)
            gm[t] = g[t];
        cplx<T> v[C], o[C];
#pragma unroll
        for (int c = 0; c < C; ++c)
            v[c] = F[c * nx * KC + i];
#pragma unroll
        for (int a = 0; a < C; ++a) {
            cplx<T> acc = {0, 0};
#pragma unroll
            for (int b = 0; b < C; ++b) {
                const int ia = a > b ? a : b, ib = a > b ? b : a;
                const T   gab = gm[ia * (ia + 1) / 2 + ib];
                acc.x += gab * v[b].x;
                acc.y += gab * v[b].y;
            }
            o[a] = acc;
        }
#pragma unroll
        for (int c = 0; c < C; ++c)
            F[c * nx * KC + i] = o[c];
    }
    __syncthreads();
    cplx<T> *O = (F == A) ? B : A;
    cplx<T> *R = fft_lines<T, true, true>(F, O, p.dx, C * KC, KC, nx * KC, KC, tw, threadIdx.x, blockDim.x);
    for (int i = threadIdx.x; i < C * nx * KC; i += blockDim.x) {
        const int comp = i / (nx * KC), rem = i % (nx * KC), x = rem / KC, l = rem % KC;
        if (l < nk)
            p.spec[(((long long)comp * nx + x) * ny + ky) * p.nzp + kz0 + l] = R[i];
    }
}

// ------------------------------------------------------------------ z inv ---
template <typename T>
__global__ void __launch_bounds__(kFftThreads) k_z_inv(ConvPlan<T> p, ConvArgs a, int rows_per_cta)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ double red_smem[32];
    const int M = p.M;
    cplx<T>  *A  = reinterpret_cast<cplx<T> *>(smem_raw);
    cplx<T>  *B  = A + rows_per_cta * (M + 1);
    cplx<T>  *tw = B + rows_per_cta * (M + 1);
    cplx<T>  *tr = tw + M;
    load_tw(tw, p.tw_z, M);
    load_tw(tr, p.tw_r2c, M + 1);
    const long long nrows = (long long)p.C * p.g.nx * p.g.ny;
    const long long row0  = (long long)blockIdx.x * rows_per_cta;
    const int       nl    = (int)min((long long)rows_per_cta, nrows - row0);
    // stage the half spectrum rows (M+1 entries each) in B
    for (int i = threadIdx.x; i < nl * (M + 1); i += blockDim.x)
        B[i] = p.spec[(row0 + i / (M + 1)) * p.nzp + (i % (M + 1))];
    __syncthreads();
    // Hermitian pack: Z'_k = E'_k + i O'_k, E' = X_k + conj(X_{M-k}),
    // O' = (X_k - conj(X_{M-k})) exp(+2 pi i k/nz); DC/Nyquist imaginary parts dropped.
    for (int i = threadIdx.x; i < nl * M; i += blockDim.x) {
        const int L = i / M, k = i % M;
        cplx<T>   xk = B[L * (M + 1) + k];
        cplx<T>   xm = B[L * (M + 1) + (M - k)];
        if (k == 0) {
            xk.y = 0;
            xm.y = 0;
        }
        xm.y      = -xm.y;
        cplx<T> E = cadd(xk, xm);
        cplx<T> O = cmulc(csub(xk, xm), tr[k]);
        A[L * M + k] = cplx<T>{E.x - O.y, E.y + O.x};
    }
    __syncthreads();
    cplx<T> *Z = fft_lines<T, true, false>(A, B, p.dz, nl, 1, M, 1, tw, threadIdx.x, blockDim.x);
    cplx<T> *sout = reinterpret_cast<cplx<T> *>(a.s);
    const cplx<T> *rin = reinterpret_cast<const cplx<T> *>(a.r);
    const T  sg  = (T)a.sign;
    T        dot = (T)0; // per-thread partial (a few elements), folded into FP64 below
    for (int i = threadIdx.x; i < nl * M; i += blockDim.x) {
        const long long gi = (row0 + i / M) * M + (i % M);
        cplx<T>         z  = Z[(i / M) * M + (i % M)];
        z.x *= sg;
        z.y *= sg;
        sout[gi] = z;
        if (a.reduce) {
            cplx<T> rv = rin[gi];
            dot += rv.x * z.x + rv.y * z.y;
        }
    }
    if (a.reduce) {
        double    v[1]   = {(double)dot};
        const int ops[1] = {RED_SUM};
        block_reduce<1>(v, ops, red_smem);
        if (grid_partial_commit<1>(v, a.red.partials, a.red.counter + a.red_site, gridDim.x)) {
            grid_final<1>(v, ops, a.red.partials, gridDim.x, red_smem);
            if (threadIdx.x == 0) {
                CgScalars *s = a.scal;
                s->delta0    = s->delta;
                s->delta     = v[0];
                double beta  = (s->delta - s->deltamid) / s->delta0;
                s->beta      = beta > 0.0 ? beta : 0.0; // fmax(0, .) of solverCG.h:94
            }
        }
    }
}

template <typename T>
int z_rows_per_cta(const ConvPlan<T> &p)
{
    // ~32 KB of ping-pong buffers per CTA
    int r = (int)(16384 / (sizeof(cplx<T>) * (p.M + 1)));
    return r < 1 ? 1 : (r > 64 ? 64 : r);
}

template <typename T>
cudaError_t set_smem(const void *fn, size_t bytes)
{
    return allow_max_dyn_smem(fn);
}

// ------------------------------------------------------------ Green's table --
__device__ void sym_pinv3(int n, const double *Ain, double tol, double *P)
{
    double a[3][3], v[3][3];
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
            a[i][j] = Ain[i * n + j];
            v[i][j] = (i == j) ? 1.0 : 0.0;
        }
    for (int sweep = 0; sweep < 50; ++sweep) {
        double off = 0.0, diag = 0.0;
        for (int i = 0; i < n; ++i) {
            diag += a[i][i] * a[i][i];
            for (int j = i + 1; j < n; ++j)
                off += a[i][j] * a[i][j];
        }
        if (off <= 1e-36 * diag || off == 0.0)
            break;
        for (int pp = 0; pp < n; ++pp)
            for (int q = pp + 1; q < n; ++q) {
                if (a[pp][q] == 0.0)
                    continue;
                double theta = (a[q][q] - a[pp][pp]) / (2.0 * a[pp][q]);
                double t     = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                double cs = 1.0 / sqrt(t * t + 1.0), sn = t * cs;
                for (int k = 0; k < n; ++k) {
                    double akp = a[k][pp], akq = a[k][q];
                    a[k][pp] = cs * akp - sn * akq;
                    a[k][q]  = sn * akp + cs * akq;
                }
                for (int k = 0; k < n; ++k) {
                    double apk = a[pp][k], aqk = a[q][k];
                    a[pp][k] = cs * apk - sn * aqk;
                    a[q][k]  = sn * apk + cs * aqk;
                }
                for (int k = 0; k < n; ++k) {
                    double vkp = v[k][pp], vkq = v[k][q];
                    v[k][pp] = cs * vkp - sn * vkq;
                    v[k][q]  = sn * vkp + cs * vkq;
                }
            }
    }
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
            double acc = 0.0;
            for (int k = 0; k < n; ++k) {
                double lam = a[k][k];
                if (fabs(lam) > tol)
                    acc += v[i][k] * v[j][k] / lam;
            }
            P[i * n + j] = acc;
        }
}

// Inverse of a symmetric positive-definite n x n block (n <= 3) by LDL^T when
// every pivot exceeds 1e-4 of the largest diagonal entry and 1e-8 in absolute
// value: the block is then well conditioned and its eigenvalues lie far above
// the pseudo-inverse's absolute cut of 1e-14, so its inverse equals that
// pseudo-inverse to round-off.  Returns false (caller takes the Jacobi path)
// otherwise -- singular blocks (hourglass frequencies of HEX8R, round-off-sized
// blocks) always do.
__device__ bool spd_inv3(int n, const double *A, double *P)
{
    double dmax = 0.0;
    for (int i = 0; i < n; ++i)
        dmax = fmax(dmax, fabs(A[i * n + i]));
    double L[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}}, D[3];
    for (int j = 0; j < n; ++j) {
        double d = A[j * n + j];
        for (int k = 0; k < j; ++k)
            d -= L[j][k] * L[j][k] * D[k];
        if (!(d > 1e-4 * dmax) || !(d > 1e-8)) // well conditioned and far above the 1e-14 cut
            return false;
        D[j] = d;
        for (int i = j + 1; i < n; ++i) {
            double s = A[i * n + j];
            for (int k = 0; k < j; ++k)
                s -= L[i][k] * L[j][k] * D[k];
            L[i][j] = s / d;
        }
    }
    // inverse of the unit lower-triangular L, then P = L^-T D^-1 L^-1
    double Li[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    for (int i = 1; i < n; ++i)
        for (int j = 0; j < i; ++j) {
            double s = 0.0;
            for (int k = j; k < i; ++k)
                s -= L[i][k] * Li[k][j];
            Li[i][j] = s;
        }
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
            double s = 0.0;
            for (int k = (i > j ? i : j); k < n; ++k)
                s += Li[k][i] * Li[k][j] / D[k];
            P[i * n + j] = s;
        }
    return true;
}

// Node offset class of d = x_p - x_q in {-1, 0, 1}^3 (x_p: the bits of node p, x first): 0 for
// d = 0, else 1..13 for the representative of {d, -d} whose first non-zero coordinate (x, y, z
// order) is positive, in the order of cos(theta . d) in k_green.
__device__ __forceinline__ int offset_class(int dx, int dy, int dz)
{
    if (dx < 0 || (dx == 0 && (dy < 0 || (dy == 0 && dz < 0)))) {
        dx = -dx;
        dy = -dy;
        dz = -dz;
    }
    if (dx == 0 && dy == 0)
        return dz == 0 ? 0 : 3;
    if (dx == 0)
        return dz == 0 ? 2 : (dz > 0 ? 8 : 9);
    if (dy == 0)
        return dz == 0 ? 1 : (dz > 0 ? 6 : 7);
    if (dy > 0)
        return dz == 0 ? 4 : (dz > 0 ? 10 : 11);
    return dz == 0 ? 5 : (dz > 0 ? 12 : 13);
}

// The weighted contraction of solver.h:177-186, block_ij = sum_pq K0_ij[p][q] Re(A_p conj A_q),
// depends on the node pair only through d = x_p - x_q, since Re(A_p conj A_q) = cos(theta . d):
// block_ij = sum_d S_ij(d) cos(theta . d) with S_ij(d) the sum of K0_ij over the pairs of
// offset d.  cos is even, so d and -d share one term: 14 coefficients per block entry (summed
// by every CTA from K0 in shared memory) replace the 64 products per entry and frequency.
template <int C>
__global__ void __launch_bounds__(256) k_green(GreenArgs a)
{
    constexpr int NC = 8 * C, NT = C * (C + 1) / 2;
    __shared__ double K0[NC * NC];
    __shared__ double Tc[NT * 14]; // [entry (i <= j, row-major)][offset class]
    for (int i = threadIdx.x; i < NC * NC; i += blockDim.x)
        K0[i] = a.K0c[i];
    __syncthreads();
    for (int idx = threadIdx.x; idx < NT * 14; idx += blockDim.x) {
        const int e = idx / 14, m = idx % 14;
        int       i = 0, j = 0;
        for (int r = 0, n = 0; r < C; ++r)
            for (int c = r; c < C; ++c, ++n)
                if (n == e) {
                    i = r;
                    j = c;
                }
        double acc = 0.0;
        for (int pp = 0; pp < 8; ++pp)
            for (int q = 0; q < 8; ++q)
                if (offset_class((pp & 1) - (q & 1), ((pp >> 1) & 1) - ((q >> 1) & 1), (pp >> 2) - (q >> 2)) == m)
                    acc += K0[(8 * i + pp) * NC + 8 * j + q];
        Tc[idx] = acc;
    }
    __syncthreads();
    const int       nx = a.g.nx, ny = a.g.ny, nz = a.g.nz, nzh = nz / 2 + 1;
    const long long F  = (long long)nx * ny * nzh;
    const double    Ninv = 1.0 / ((double)nx * (double)ny * (double)nz);
    for (long long f = blockIdx.x * (long long)blockDim.x + threadIdx.x; f < F; f += (long long)gridDim.x * blockDim.x) {
        const int iz = (int)(f % nzh), iy = (int)((f / nzh) % ny), ix = (int)(f / ((long long)nzh * ny));
        double    out[NT];
        if (ix == 0 && iy == 0 && iz == 0) {
#pragma unroll
            for (int t = 0; t < NT; ++t)
                out[t] = 0.0;
        } else {
            const double cx = a.cx[ix], sx = a.sx[ix], cy = a.cy[iy], sy = a.sy[iy], cz = a.cz[iz], sz = a.sz[iz];
            const double pr = cx * cy - sx * sy, pi = sx * cy + cx * sy; // e^{i(tx + ty)}
            const double mr = cx * cy + sx * sy, mi = sx * cy - cx * sy; // e^{i(tx - ty)}
            const double cv[14] = {1.0,
                                   cx,
                                   cy,
                                   cz,
                                   pr,
                                   mr,
                                   cx * cz - sx * sz,
                                   cx * cz + sx * sz,
                                   cy * cz - sy * sz,
                                   cy * cz + sy * sz,
                                   pr * cz - pi * sz,
                                   pr * cz + pi * sz,
                                   mr * cz - mi * sz,
                                   mr * cz + mi * sz};
            double blk[9], pinv[9];
            int    e = 0;
#pragma unroll
            for (int i = 0; i < C; ++i)
#pragma unroll
                for (int j = i; j < C; ++j, ++e) {
                    double acc = 0.0;
#pragma unroll
                    for (int m = 0; m < 14; ++m)
                        acc += Tc[e * 14 + m] * cv[m];
                    blk[i * C + j] = acc;
                    blk[j * C + i] = acc;
                }
            if (!spd_inv3(C, blk, pinv))
                sym_pinv3(C, blk, 1e-14, pinv);
            int t = 0;
#pragma unroll
            for (int i = 0; i < C; ++i)
#pragma unroll
                for (int j = 0; j <= i; ++j)
                    out[t++] = pinv[i * C + j] * Ninv;
        }
#pragma unroll
        for (int t = 0; t < NT; ++t) {
            a.G64[f * NT + t] = out[t];
            if (a.G32)
                a.G32[((f / nzh) * a.g32s + iz) * NT + t] = (float)out[t]; // row (ix, iy) at stride g32s
        }
    }
}

} // namespace

template <typename T>
size_t conv_smem_bytes(const ConvPlan<T> &p, int pass)
{
    const size_t cs = sizeof(cplx<T>);
    switch (pass) {
    case 0: return cs * (2 * (size_t)z_rows_per_cta(p) * p.M + p.M + p.M + 1);
    case 1: return cs * (2 * (size_t)p.g.ny * p.kc_y + p.g.ny);
    case 2: return cs * (2 * (size_t)p.C * p.g.nx * p.kc_x + p.g.nx);
    default: return cs * (2 * (size_t)z_rows_per_cta(p) * (p.M + 1) + p.M + p.M + 1);
    }
}

template <typename T>
cudaError_t launch_convolution(const ConvPlan<T> &p, const ConvArgs &a, cudaStream_t st)
{
    if (p.use_reg)
        return launch_convolution_reg<T>(p, a, st);
    cudaError_t     e;
    const long long nrows = (long long)p.C * p.g.nx * p.g.ny;
    const int       rz    = z_rows_per_cta(p);
    const int       nbz   = (int)((nrows + rz - 1) / rz);
    auto mark = [&](int i) {
        if (a.ev)
            cudaEventRecord(a.ev[i], st);
    };
    mark(0);
    // z forward
    size_t s0 = conv_smem_bytes(p, 0);
    if ((e = set_smem<T>((const void *)k_z_fwd<T>, s0)) != cudaSuccess)
        return e;
    k_z_fwd<T><<<nbz, kFftThreads, s0, st>>>(p, reinterpret_cast<const T *>(a.r), rz);
    mark(1);
    // y forward
    size_t s1 = conv_smem_bytes(p, 1);
    dim3   gy((p.nzh + p.kc_y - 1) / p.kc_y, p.g.nx, p.C);
    if ((e = set_smem<T>((const void *)k_y<T, false>, s1)) != cudaSuccess)
        return e;
    k_y<T, false><<<gy, kFftThreads, s1, st>>>(p);
    mark(2);
    // x + Green + x inverse
    size_t s2 = conv_smem_bytes(p, 2);
    dim3   gx((p.nzh + p.kc_x - 1) / p.kc_x, p.g.ny);
    if (p.C == 1) {
        if ((e = set_smem<T>((const void *)k_x_green<T, 1>, s2)) != cudaSuccess)
            return e;
        k_x_green<T, 1><<<gx, kFftThreads, s2, st>>>(p);
    } else {
        if ((e = set_smem<T>((const void *)k_x_green<T, 3>, s2)) != cudaSuccess)
            return e;
        k_x_green<T, 3><<<gx, kFftThreads, s2, st>>>(p);
    }
    mark(3);
    // y inverse
    if ((e = set_smem<T>((const void *)k_y<T, true>, s1)) != cudaSuccess)
        return e;
    k_y<T, true><<<gy, kFftThreads, s1, st>>>(p);
    mark(4);
    // z inverse
    size_t s3 = conv_smem_bytes(p, 3);
    if ((e = set_smem<T>((const void *)k_z_inv<T>, s3)) != cudaSuccess)
        return e;
    k_z_inv<T><<<nbz, kFftThreads, s3, st>>>(p, a, rz);
    mark(5);
    return cudaGetLastError();
}

template cudaError_t launch_convolution<double>(const ConvPlan<double> &, const ConvArgs &, cudaStream_t);
template cudaError_t launch_convolution<float>(const ConvPlan<float> &, const ConvArgs &, cudaStream_t);
template size_t      conv_smem_bytes<double>(const ConvPlan<double> &, int);
template size_t      conv_smem_bytes<float>(const ConvPlan<float> &, int);

cudaError_t launch_green(const GreenArgs &a, cudaStream_t st)
{
    const long long F  = (long long)a.g.nx * a.g.ny * (a.g.nz / 2 + 1);
    const int       nb = grid_blocks_for(F);
    if (a.C == 1)
        k_green<1><<<nb, 256, 0, st>>>(a);
    else
        k_green<3><<<nb, 256, 0, st>>>(a);
    return cudaGetLastError();
}

} // namespace fansgpu
