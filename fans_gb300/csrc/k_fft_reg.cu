// k_fft_reg.cu -- register-resident convolution passes (two-phase line FFTs).
//
// Same five passes and spectrum layout as k_fft.cu, but each line lives in
// registers: threads load their strided values straight from global memory
// (128-byte rows), transform in registers, and meet once in shared memory per
// line transform.  Shared memory holds one copy of the tile (no ping-pong), so
// more CTAs are resident.  Used for line lengths with a register plan
// (reg_n1(n) != 0); other sizes use the shared-memory Stockham passes.
#include <cuda.h> // CUtensorMap (the encoder is reached through the runtime)
#include <cudaTypedefs.h>

#include <cstring>
#include <type_traits>

#include "fft_reg.cuh"
#include "kernels.cuh"

namespace fansgpu {

namespace {

// Tile shapes with two variants each, picked per grid by tune_convolution_reg
// (variant 0 is the default): kz columns per CTA of the y and x passes (row
// segments of 128 / 64 bytes for y, 64 / 32 bytes for x) and threads per CTA of
// the z passes.
template <typename T>
struct Tiles {
    static constexpr int cs   = (int)sizeof(cplx<T>);
    static constexpr int y[2] = {128 / cs, 64 / cs};
    static constexpr int x[2] = {64 / cs, 32 / cs > 1 ? 32 / cs : 2};
    static constexpr int z[2] = {sizeof(T) == 4 ? 256 : 128, sizeof(T) == 4 ? 128 : 64};
};

// <r, s> of a reducing convolution from the spectra, by Parseval: with r^ the forward spectrum
// and y^ = G r^ (G holding 1/N), s = sign * c2r(y^) unnormalised gives <r, s> = sign * sum over
// the full spectrum of Re(r^ conj y^); on the half spectrum kz = 1..M-1 count twice (the
// conjugate half has equal terms), kz = 0 and M once.
__device__ __forceinline__ int dot_weight(int kz, int M) { return (kz == 0 || kz == M) ? 1 : 2; }

// this thread's per-RHS partial sums -> block -> grid partials; the last block sets delta0 <-
// delta, delta <- <r, s>, beta = max(0, (delta - deltamid) / delta0) per active RHS
// (solverCG.h:86-94), as the z-inverse pass does for the spatial dot
template <typename T>
__device__ void conv_dot_finish(const double (&dk)[kMaxRhs], const ConvPlan<T> &p, const ConvArgs &a,
                                double *red_smem)
{
    double vv[kMaxRhs];
    int    ops[kMaxRhs];
#pragma unroll
    for (int q = 0; q < kMaxRhs; ++q) {
        vv[q]  = a.sign * dk[q];
        ops[q] = RED_SUM;
    }
    block_reduce<kMaxRhs>(vv, ops, red_smem);
    const int nb = gridDim.x * gridDim.y * gridDim.z;
    if (grid_partial_commit<kMaxRhs>(vv, a.red.partials, a.red.counter + a.red_site, nb)) {
        grid_final<kMaxRhs>(vv, ops, a.red.partials, nb, red_smem);
        if (threadIdx.x == 0)
            for (int q = 0; q < p.nrhs; ++q) {
                if (p.active && !p.active[q])
                    continue;
                CgScalars *sc = a.scal + q;
                sc->delta0    = sc->delta;
                sc->delta     = vv[q];
                double beta   = (sc->delta - sc->deltamid) / sc->delta0;
                sc->beta      = beta > 0.0 ? beta : 0.0;
            }
    }
}

// ------------------------------------------------------------------ y pass ---
// FP32 tiles of 256 threads: registers for five CTAs per SM (the inverse pass would take four)
template <typename T, int N1, int N2, bool INV, int KC>
__global__ void __launch_bounds__(KC * N1, (sizeof(T) == 4 && KC * N1 == 256) ? 5 : 1) k_y_reg(ConvPlan<T> p)
{
    constexpr int n = N1 * N2;
    __shared__ cplx<T> S[n * KC];
    const int t = threadIdx.x, l = t % KC, w = t / KC;
    const int kz0 = blockIdx.x * KC, x = blockIdx.y, comp = blockIdx.z; // comp = rhs * C + c
    if (p.active && !p.active[comp / p.C])
        return;
    const bool valid = l < p.nzh - kz0;
    cplx<T> *base = p.spec + ((long long)comp * p.g.nx + x) * (long long)p.g.ny * p.nzp + kz0 + l;
    cplx<T>  v[N2];
#pragma unroll
    for (int j2 = 0; j2 < N2; ++j2)
        v[j2] = valid ? base[(long long)(w + N1 * j2) * p.nzp] : cplx<T>{0, 0};
    line_phase1<T, N1, N2, INV>(v, w, p.tw_y);
#pragma unroll
    for (int k2 = 0; k2 < N2; ++k2)
        S[(k2 * N1 + w) * KC + l] = v[k2];
    __syncthreads();
    if (w < N2) {
        cplx<T> u[N1];
#pragma unroll
        for (int j1 = 0; j1 < N1; ++j1)
            u[j1] = S[(w * N1 + j1) * KC + l];
        Dft<T, N1, INV>::run(u);
        if (valid)
#pragma unroll
            for (int k1 = 0; k1 < N1; ++k1)
                base[(long long)(w + N2 * k1) * p.nzp] = u[k1];
    }
}

// ----------------------------------------------------- x pass + Green's op ---
// One CTA per ky and KX kz columns (64-byte row segments), all kx and all C
// components: forward FFT along x, the C x C Green multiply, inverse FFT along
// x.  The CTA's slice of the Green's table is copied into shared memory with
// cp.async at the start, so its reads overlap the forward transform; the
// smaller tile lets two CTAs share an SM and overlap their load, compute and
// store phases.
template <typename T, int KC>
struct KXCtas { // resident CTAs per SM the register budget is set for
    static constexpr int value = (sizeof(T) == 4 && KC * (int)sizeof(cplx<T>) <= 32) ? 4 : 2;
};

template <typename T, int N1, int N2, int C, int KC>
__global__ void __launch_bounds__(C * KC * N1, KXCtas<T, KC>::value) k_x_green_reg(ConvPlan<T> p, ConvArgs a)
{
    __shared__ double red_smem[32 * kMaxRhs];
    const bool        sdot = p.spectral_dot && a.reduce;
    double            dk[kMaxRhs];
#pragma unroll
    for (int q = 0; q < kMaxRhs; ++q)
        dk[q] = 0.0;
    constexpr int n = N1 * N2, NT = C * (C + 1) / 2;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cplx<T>  *F  = reinterpret_cast<cplx<T> *>(smem_raw);        // [C][n][KC]
    T        *Gs = reinterpret_cast<T *>(F + (size_t)C * n * KC); // [n][KC][NT]
    const int nx = n, ny = p.g.ny;
    const int t = threadIdx.x, comp = t / (KC * N1), rem = t % (KC * N1), w = rem / KC, l = rem % KC;
    const int kz0 = blockIdx.x * KC, ky = blockIdx.y;
    const int nk  = min(KC, p.nzh - kz0);
    const bool valid = l < nk;
    cplx<T> *gbase = p.spec + ((long long)comp * nx * ny + ky) * p.nzp + kz0 + l; // + x * ny * nzp
    const long long xstride = (long long)ny * p.nzp;
    cplx<T> *Fc = F + (size_t)comp * n * KC;

    // Green's table slice [kx][kz0 .. kz0+nk)[NT] -> Gs, asynchronously
    for (int i = t; i < n * nk * NT; i += blockDim.x) {
        const int kx = i / (nk * NT), r2 = i % (nk * NT);
        const T  *src = p.G + (((long long)kx * ny + ky) * p.gzs + kz0) * NT + r2;
        T        *dst = Gs + (size_t)kx * KC * NT + r2;
        if constexpr (sizeof(T) == 4)
            asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)),
                         "l"(src)
                         : "memory");
        else
            asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)),
                         "l"(src)
                         : "memory");
    }
    asm volatile("cp.async.commit_group;" ::: "memory");

    // the same Green's slice serves every right-hand side: RHS k's spectrum follows RHS k-1's
    const long long rhs_spec = (long long)p.C * nx * ny * p.nzp;
    for (int k = 0; k < p.nrhs; ++k) {
        if (p.active && !p.active[k])
            continue;
        cplx<T> *gb = gbase + k * rhs_spec;
        // forward FFT along x
        cplx<T> v[N2];
#pragma unroll
        for (int j2 = 0; j2 < N2; ++j2)
            v[j2] = valid ? gb[(w + N1 * j2) * xstride] : cplx<T>{0, 0};
        {   // the next active RHS's column into L2 while this one is transformed
            int kn = k + 1;
            while (kn < p.nrhs && p.active && !p.active[kn])
                ++kn;
            if (kn < p.nrhs && valid) {
                const cplx<T> *gn = gbase + kn * rhs_spec;
#pragma unroll
                for (int j2 = 0; j2 < N2; ++j2)
                    asm volatile("prefetch.global.L2 [%0];" ::"l"(gn + (w + N1 * j2) * xstride));
            }
        }
        line_phase1<T, N1, N2, false>(v, w, p.tw_x);
#pragma unroll
        for (int k2 = 0; k2 < N2; ++k2)
            Fc[(k2 * N1 + w) * KC + l] = v[k2];
        __syncthreads();
        cplx<T> u[N1];
        if (w < N2)
#pragma unroll
            for (int j1 = 0; j1 < N1; ++j1)
                u[j1] = Fc[(w * N1 + j1) * KC + l];
        __syncthreads();
        if (w < N2) {
            Dft<T, N1, false>::run(u);
#pragma unroll
            for (int k1 = 0; k1 < N1; ++k1)
                Fc[(w + N2 * k1) * KC + l] = u[k1];
        }
        asm volatile("cp.async.wait_all;" ::: "memory");
        __syncthreads();

        // Green's operator: C x C real symmetric per frequency (solver.h:400-406)
        T dsum = (T)0;
        for (int i = t; i < n * KC; i += blockDim.x) {
            const int kx = i / KC, ll = i % KC;
            if (ll >= nk)
                continue;
            const T *g = Gs + ((size_t)kx * KC + ll) * NT;
            T        gm[NT];
#pragma unroll
            for (int q = 0; q < NT; ++q)
                gm[q] = g[q];
            cplx<T> fr[C], o[C];
#pragma unroll
            for (int c = 0; c < C; ++c)
                fr[c] = F[((size_t)c * n + kx) * KC + ll];
#pragma unroll
            for (int r = 0; r < C; ++r) {
                cplx<T> acc = {0, 0};
#pragma unroll
                for (int c = 0; c < C; ++c) {
                    const int ia = r > c ? r : c, ib = r > c ? c : r;
                    const T   gv = gm[ia * (ia + 1) / 2 + ib];
                    acc.x += gv * fr[c].x;
                    acc.y += gv * fr[c].y;
                }
                o[r] = acc;
            }
#pragma unroll
            for (int c = 0; c < C; ++c)
                F[((size_t)c * n + kx) * KC + ll] = o[c];
            if (sdot) {
                T dd = (T)0;
#pragma unroll
                for (int c = 0; c < C; ++c)
                    dd += fr[c].x * o[c].x + fr[c].y * o[c].y;
                dsum += (T)dot_weight(kz0 + ll, p.M) * dd;
            }
        }
        if (sdot)
#pragma unroll
            for (int q = 0; q < kMaxRhs; ++q)
                if (q == k)
                    dk[q] += (double)dsum;
        __syncthreads();

        // inverse FFT along x
#pragma unroll
        for (int j2 = 0; j2 < N2; ++j2)
            v[j2] = Fc[(w + N1 * j2) * KC + l];
        __syncthreads();
        line_phase1<T, N1, N2, true>(v, w, p.tw_x);
#pragma unroll
        for (int k2 = 0; k2 < N2; ++k2)
            Fc[(k2 * N1 + w) * KC + l] = v[k2];
        __syncthreads();
        if (w < N2) {
#pragma unroll
            for (int j1 = 0; j1 < N1; ++j1)
                u[j1] = Fc[(w * N1 + j1) * KC + l];
            Dft<T, N1, true>::run(u);
            if (valid)
#pragma unroll
                for (int k1 = 0; k1 < N1; ++k1)
                    gb[(w + N2 * k1) * xstride] = u[k1];
        }
        __syncthreads(); // F is reused by the next right-hand side
    }
    if (sdot)
        conv_dot_finish<T>(dk, p, a, red_smem);
}

// ------------------------------------------- x pass + Green's op, TMA-fed ---
// FP32 form of the x pass with its inputs brought in by the tensor memory
// accelerator.  Persistent: CTA b takes a contiguous share of the jobs
// (tile, RHS), tile = (ky, KX kz columns), and keeps two job buffers.  A job's
// [C][nx][KX] spectrum tile arrives by one tensor-map copy per component and
// completes on its buffer's mbarrier; the buffer then serves as the job's
// inverse exchange, and the copy of job q + 1 into the other buffer is issued at
// job q's first barrier, so the reads run one job ahead of the transforms.  The
// tile's Green's slice [nx][KX][NT] arrives the same way, issued when the
// previous tile's last job has applied its slice.  The Green multiply is fused
// into the load of the inverse transform (each thread forms its component's row
// of G . F for its own kx, and with the spectral dot also its share of <r, s>),
// the twiddles of a worker live in registers, and the exchanges of one component
// meet only its own warps (named barriers).  The operations per value are those
// of k_x_green_reg; the compiler may contract them differently, so the two agree
// to FP32 rounding.  Every wait is bounded: one that runs out sets an abort flag
// that releases the others, no further copies are issued, the CTA waits
// (bounded) for the copies it has in flight, and the status -3 goes to every
// active RHS's converged field.
constexpr int      kTmaKC        = 8;       // kz columns per tile: 64-byte rows of complex FP32
constexpr unsigned kTmaWaitLimit = 1u << 22; // polls of one mbarrier wait

__device__ __forceinline__ bool tma_bar_try(uint32_t bar, uint32_t parity)
{
    uint32_t done;
    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                 " selp.u32 %0, 1, 0, p;\n}\n"
                 : "=r"(done)
                 : "r"(bar), "r"(parity)
                 : "memory");
    return done != 0;
}

__device__ __forceinline__ void tma_bar_wait(uint32_t bar, uint32_t parity, volatile int *abort_flag)
{
    for (unsigned it = 0; it < kTmaWaitLimit; ++it)
        if (tma_bar_try(bar, parity) || *abort_flag)
            return;
    *abort_flag = 1;
}

// box {2 KX floats, 1, n} of a 3-d float tensor map at (x, y, z) into shared memory,
// completing `bytes` on `bar` (the caller has posted them with expect_tx)
__device__ __forceinline__ void tma_load3(uint32_t dst, const CUtensorMap *tm, int x, int y, int z, uint32_t bar)
{
    asm volatile("cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
                 " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(dst),
                 "l"(reinterpret_cast<uint64_t>(tm)), "r"(x), "r"(y), "r"(z), "r"(bar)
                 : "memory");
}

__device__ __forceinline__ void tma_expect(uint32_t bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

template <int N1, int N2, int C>
struct XTma {
    static constexpr int n = N1 * N2, KX = kTmaKC, NT = C * (C + 1) / 2;
    static constexpr int JOB_BYTES = C * n * KX * 8; // one job's spectrum tile
    static constexpr int G_BYTES   = n * KX * NT * 4;
    static constexpr int OFF_F     = 2 * JOB_BYTES;  // exchange buffer [C][n][KX]
    static constexpr int OFF_G     = 3 * JOB_BYTES;  // Green's slice [n][KX][NT]
    static constexpr int OFF_BAR   = (OFF_G + G_BYTES + 15) / 16 * 16; // full[2], green, flags
    static constexpr int SMEM      = OFF_BAR + 64;
};

template <int N1, int N2, int C>
__global__ void __launch_bounds__(C * kTmaKC * N1, 1)
    k_x_green_tma(ConvPlan<float> p, ConvArgs a, const __grid_constant__ CUtensorMap tm_spec,
                  const __grid_constant__ CUtensorMap tm_green)
{
    using L          = XTma<N1, N2, C>;
    constexpr int n  = L::n, KX = L::KX, NT = L::NT;
    extern __shared__ __align__(1024) unsigned char xsm[];
    cplx<float>  *Bf  = reinterpret_cast<cplx<float> *>(xsm);            // [2][C][n][KX]
    cplx<float>  *F   = reinterpret_cast<cplx<float> *>(xsm + L::OFF_F); // [C][n][KX]
    const float  *Gs  = reinterpret_cast<const float *>(xsm + L::OFF_G); // [n][KX][NT]
    const uint32_t sb = (uint32_t)__cvta_generic_to_shared(xsm);
    const uint32_t bar_full = sb + L::OFF_BAR, bar_green = bar_full + 16;
    volatile int  *abort_flag = reinterpret_cast<volatile int *>(xsm + L::OFF_BAR + 24);
    int           *s_act      = reinterpret_cast<int *>(xsm + L::OFF_BAR + 28); // nact, then kMaxRhs ids

    const int t = threadIdx.x, comp = t / (KX * N1), rem = t % (KX * N1), w = rem / KX, l = rem % KX;
    const int ny = p.g.ny, ntz = (p.nzh + KX - 1) / KX;
    const bool sdot = p.spectral_dot && a.reduce;
    double     dk[kMaxRhs];
#pragma unroll
    for (int q = 0; q < kMaxRhs; ++q)
        dk[q] = 0.0;
    if (t == 0) {
        int nact = 0;
        for (int k = 0; k < p.nrhs; ++k)
            if (!p.active || p.active[k])
                s_act[1 + nact++] = k;
        s_act[0]    = nact;
        *abort_flag = (sb & 127) ? 1 : 0; // copies land on 128-byte boundaries of the window
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar_full) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar_full + 8) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar_green) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    const int       nact = s_act[0];
    const long long J    = (long long)ntz * ny * nact;
    const long long jb   = J * blockIdx.x / gridDim.x, je = J * (blockIdx.x + 1) / gridDim.x;
    if (nact == 0 || *abort_flag) { // uniform over the grid: no CTA commits reduction partials
        if (*abort_flag && t == 0 && a.scal)
            for (int kk = 0; kk < nact; ++kk)
                a.scal[s_act[1 + kk]].converged = -3;
        return; // no copy was issued
    }
    // a CTA may have no jobs when converged RHS left fewer jobs than CTAs: it still commits its
    // (zero) partials of the spectral <r, s> below
    const int nq = (int)(je - jb);

    // thread 0 only: issue the copies of job q (into buffer q & 1) or of job q's Green's slice
    int iss[3] = {0, 0, 0}; // phases issued per barrier (full 0, full 1, green)
    auto issue_job = [&](int q) {
        const long long jg = jb + q;
        const int       tile = (int)(jg / nact), k = s_act[1 + (int)(jg % nact)], b = q & 1;
        const int       kz0 = (tile % ntz) * KX, ky = tile / ntz;
        const uint32_t  bar = bar_full + 8 * b;
        tma_expect(bar, L::JOB_BYTES);
#pragma unroll
        for (int c = 0; c < C; ++c)
            tma_load3(sb + b * L::JOB_BYTES + c * n * KX * 8, &tm_spec, 2 * kz0, ky, (k * C + c) * n, bar);
        ++iss[b];
    };
    auto issue_green = [&](int q) {
        const int tile = (int)((jb + q) / nact), kz0 = (tile % ntz) * KX, ky = tile / ntz;
        tma_expect(bar_green, L::G_BYTES);
        tma_load3(sb + L::OFF_G, &tm_green, kz0 * NT, ky, 0, bar_green);
        ++iss[2];
    };
    if (t == 0 && nq > 0) {
        asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tm_spec)) : "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tm_green)) : "memory");
        issue_green(0);
        issue_job(0);
        if (nq > 1)
            issue_job(1);
    }

    // this worker's twiddles W_n^(w k2), k2 = 1..N2-1 (line_phase1's table values)
    cplx<float> twr[N2];
#pragma unroll
    for (int k2 = 1; k2 < N2; ++k2)
        twr[k2] = p.tw_x[w * k2];
    const long long xstride  = (long long)ny * p.nzp;
    const long long rhs_spec = (long long)p.C * n * ny * p.nzp;
    cplx<float>    *Fc       = F + (size_t)comp * n * KX;
    int             gph      = 0; // Green's slices waited for
    // barrier of this component's KX * N1 threads (named barriers 1..C; 0 is __syncthreads)
    auto comp_bar = [&]() { asm volatile("bar.sync %0, %1;" ::"r"(1 + comp), "n"(KX * N1) : "memory"); };

    for (int q = 0; q < nq; ++q) {
        const long long jg = jb + q;
        const int tile = (int)(jg / nact), kk = (int)(jg % nact), k = s_act[1 + kk], b = q & 1;
        const int kz0 = (tile % ntz) * KX, ky = tile / ntz;
        const bool valid = l < p.nzh - kz0;
        const bool first_of_tile = q == 0 || kk == 0, last_of_tile = kk == nact - 1;

        // forward FFT along x: phase 1 from the job's buffer
        tma_bar_wait(bar_full + 8 * b, (uint32_t)((q >> 1) & 1), abort_flag);
        const cplx<float> *Bc = Bf + ((size_t)b * C + comp) * n * KX;
        cplx<float>        v[N2];
#pragma unroll
        for (int j2 = 0; j2 < N2; ++j2)
            v[j2] = Bc[(w + N1 * j2) * KX + l];
        __syncthreads(); // the buffer is read, F is free, and job q - 1 is done with its buffer
        if (t == 0 && q >= 1 && q + 1 < nq && !*abort_flag) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            issue_job(q + 1); // into the buffer job q - 1 used for its inverse exchange
        }
        Dft<float, N2, false>::run(v);
#pragma unroll
        for (int k2 = 1; k2 < N2; ++k2)
            v[k2] = cmul(v[k2], twr[k2]);
#pragma unroll
        for (int k2 = 0; k2 < N2; ++k2)
            Fc[(k2 * N1 + w) * KX + l] = v[k2];
        comp_bar(); // the transforms of one component meet only its own warps
        cplx<float> u[N1];
        if (w < N2) {
#pragma unroll
            for (int j1 = 0; j1 < N1; ++j1)
                u[j1] = Fc[(w * N1 + j1) * KX + l];
            Dft<float, N1, false>::run(u);
        }
        comp_bar();
        if (w < N2)
#pragma unroll
            for (int k1 = 0; k1 < N1; ++k1)
                Fc[(w + N2 * k1) * KX + l] = u[k1];
        if (first_of_tile)
            tma_bar_wait(bar_green, (uint32_t)(gph++ & 1), abort_flag);
        __syncthreads();

        // Green's operator (solver.h:400-406), row `comp` of the C x C real symmetric block per
        // frequency, fused into the inverse transform's load
        float dsum = 0.f;
#pragma unroll
        for (int j2 = 0; j2 < N2; ++j2) {
            const int    kx = w + N1 * j2;
            const float *g  = Gs + ((size_t)kx * KX + l) * NT;
            cplx<float>  acc = {0, 0}, xc = {0, 0};
#pragma unroll
            for (int c = 0; c < C; ++c) {
                const int         ia = comp > c ? comp : c, ib = comp > c ? c : comp;
                const float       gv = g[ia * (ia + 1) / 2 + ib];
                const cplx<float> x  = F[((size_t)c * n + kx) * KX + l];
                acc.x += gv * x.x;
                acc.y += gv * x.y;
                if (c == comp)
                    xc = x;
            }
            v[j2] = acc;
            dsum += xc.x * acc.x + xc.y * acc.y;
        }
        if (sdot)
#pragma unroll
            for (int q = 0; q < kMaxRhs; ++q)
                if (q == k)
                    dk[q] += (double)((float)dot_weight(kz0 + l, p.M) * dsum);
        // the inverse exchange goes to this job's input buffer (read by every component before
        // the first barrier), so the Green's reads of F need no barrier after them; only the
        // refill of the Green's slice waits for them, on a tile's last job
        if (last_of_tile) {
            __syncthreads();
            if (t == 0 && q + 1 < nq && !*abort_flag) {
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                issue_green(q + 1);
            }
        }
        cplx<float> *Xc = Bf + ((size_t)b * C + comp) * n * KX;
        // inverse FFT along x
        Dft<float, N2, true>::run(v);
#pragma unroll
        for (int k2 = 1; k2 < N2; ++k2) {
            cplx<float> tc = twr[k2];
            tc.y           = -tc.y;
            v[k2]          = cmul(v[k2], tc);
        }
#pragma unroll
        for (int k2 = 0; k2 < N2; ++k2)
            Xc[(k2 * N1 + w) * KX + l] = v[k2];
        comp_bar();
        if (w < N2) {
#pragma unroll
            for (int j1 = 0; j1 < N1; ++j1)
                u[j1] = Xc[(w * N1 + j1) * KX + l];
            Dft<float, N1, true>::run(u);
            if (valid) {
                cplx<float> *gb = p.spec + k * rhs_spec + ((long long)comp * n * ny + ky) * p.nzp + kz0 + l;
#pragma unroll
                for (int k1 = 0; k1 < N1; ++k1)
                    gb[(w + N2 * k1) * xstride] = u[k1];
            }
        }
    }
    __syncthreads();
    if (*abort_flag && t == 0) {
        // wait (bounded) for the copies still in flight: the last issued phase of each barrier
        for (int i = 0; i < 3; ++i)
            if (iss[i] > 0) {
                const uint32_t bar = i < 2 ? bar_full + 8 * i : bar_green;
                for (unsigned it = 0; it < kTmaWaitLimit && !tma_bar_try(bar, (uint32_t)((iss[i] - 1) & 1)); ++it)
                    ;
            }
        if (a.scal)
            for (int kk = 0; kk < nact; ++kk)
                a.scal[s_act[1 + kk]].converged = -3; // a copy of the TMA-fed x pass did not arrive
    }
    if (sdot) // every CTA of the grid commits
        conv_dot_finish<float>(dk, p, a, reinterpret_cast<double *>(xsm + L::OFF_F));
}

// ------------------------------------------------------------------ z fwd ---
// r2c of R rows per CTA: complex half-length line (z_m = x_2m + i x_2m+1), then
// X_k = (Z_k + conj Z_{M-k})/2 - i W^k (Z_k - conj Z_{M-k})/2, k = 0..M.
template <typename T, int N1, int N2, int R>
__global__ void __launch_bounds__(R * N1) k_z_fwd_reg(ConvPlan<T> p, const T *__restrict__ r)
{
    constexpr int M = N1 * N2, EP = N1 + 1; // exchange row padded against bank conflicts
    static_assert(32 % N1 == 0, "a row's workers share one warp");
    __shared__ cplx<T> E[R * N2 * EP];
    __shared__ cplx<T> Z[R * M];
    const int       t = threadIdx.x, L = t / N1, w = t % N1;
    const long long rpr   = (long long)p.C * p.g.nx * p.g.ny; // rows per right-hand side
    const long long nrows = rpr * p.nrhs;
    const long long row0b = (long long)blockIdx.x * R;
    // A block's rows belong to at most two right-hand sides (R <= 64 rows per block, and
    // the register plans need n_x, n_y >= 16, so every RHS has >= 256 rows): RHS k0 below
    // row bnd, k0 + 1 from there.
    const int       k0  = p.active ? (int)(row0b / rpr) : 0;
    const long long bnd = p.active ? (k0 + 1) * rpr : nrows;
    auto            on  = [&](long long rw) { return !p.active || p.active[k0 + (rw >= bnd ? 1 : 0)]; };
    if (p.active && !on(row0b) && !on(min(row0b + R, nrows) - 1))
        return; // every row of this block belongs to an inactive right-hand side
    const long long row   = row0b + L;
    const bool      valid = row < nrows && on(row);
    const cplx<T>  *rin   = reinterpret_cast<const cplx<T> *>(r) + row * M;
    cplx<T>         v[N2];
#pragma unroll
    for (int j2 = 0; j2 < N2; ++j2)
        v[j2] = valid ? rin[w + N1 * j2] : cplx<T>{0, 0};
    line_phase1<T, N1, N2, false>(v, w, p.tw_z);
    // a row's N1 <= 16 workers are lanes of one warp: its exchanges need only that warp
#pragma unroll
    for (int k2 = 0; k2 < N2; ++k2)
        E[(L * N2 + k2) * EP + w] = v[k2];
    __syncwarp();
    if (w < N2) {
        cplx<T> u[N1];
#pragma unroll
        for (int j1 = 0; j1 < N1; ++j1)
            u[j1] = E[(L * N2 + w) * EP + j1];
        Dft<T, N1, false>::run(u);
#pragma unroll
        for (int k1 = 0; k1 < N1; ++k1)
            Z[L * M + w + N2 * k1] = u[k1];
    }
    __syncwarp();
    // unpack the row to the half spectrum, k = 0..M, by its own workers (coalesced over k)
    if (valid)
        for (int k = w; k <= M; k += N1) {
            cplx<T> zk = Z[L * M + (k == M ? 0 : k)];
            cplx<T> zm = Z[L * M + (k == 0 ? 0 : M - k)];
            zm.y       = -zm.y;
            cplx<T> Ev = {(T)0.5 * (zk.x + zm.x), (T)0.5 * (zk.y + zm.y)};
            cplx<T> Od = {(T)0.5 * (zk.x - zm.x), (T)0.5 * (zk.y - zm.y)};
            cplx<T> P  = cmul(p.tw_r2c[k], Od);
            p.spec[row * p.nzp + k] = cplx<T>{Ev.x + P.y, Ev.y - P.x};
        }
}

// ------------------------------------------- fused z + y forward, cluster ---
// r2c along z and the complex FFT along y of one (RHS, component, x) plane in one
// pass, so the half spectrum after z is never written to and read back from HBM.
// A plane of ny rows does not fit one CTA's shared memory at 256^2, so a cluster
// of CL CTAs holds it: CTA h loads rows [h RY, (h+1) RY), RY = ny / CL, with
// 16-byte cp.async and transforms them along z in place (rows of ZS = M + 2
// complex; the half-length FFT as in k_z_fwd_reg, then the unpack to kz = 0..M
// by (k, M - k) pairs, each pair by one thread).  After a cluster barrier, CTA h
// runs the y FFTs of the kz tiles h, h + CL, ... (KC columns, 256 / N1y threads
// per line), reading the rows of every CTA of the cluster through distributed
// shared memory, and writes the spectrum plane [ky][kz] (stride nzp) once.  A
// last cluster barrier keeps every CTA's rows alive until its peers have read
// them.  The arithmetic per value is that of k_z_fwd_reg and k_y_reg.
template <int N1z, int N2z, int N1y, int N2y, int CL>
struct ZyFwd {
    static constexpr int NT = 256, M = N1z * N2z, NY = N1y * N2y, RY = NY / CL, ZS = M + 2;
    static constexpr int RZ = NT / N1z, EPz = N1z + 1, KC = NT / N1y;
    static constexpr int EX_Z = RZ * N2z * EPz, EX_Y = NY * KC;
    static constexpr int SMEM = (RY * ZS + (EX_Z > EX_Y ? EX_Z : EX_Y)) * 8;
};

__device__ __forceinline__ void cluster_sync_all()
{
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

__device__ __forceinline__ cplx<float> ld_dsmem(uint32_t local_addr, uint32_t rank)
{
    uint32_t    ra;
    cplx<float> v;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(ra) : "r"(local_addr), "r"(rank));
    asm volatile("ld.shared::cluster.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(ra) : "memory");
    return v;
}

template <int N1z, int N2z, int N1y, int N2y, int CL>
__global__ void __launch_bounds__(256, 2) k_zy_fwd(ConvPlan<float> p, const float *__restrict__ r)
{
    using L = ZyFwd<N1z, N2z, N1y, N2y, CL>;
    constexpr int M = L::M, NY = L::NY, RY = L::RY, ZS = L::ZS, RZ = L::RZ, EPz = L::EPz, KC = L::KC;
    extern __shared__ __align__(16) unsigned char zysm[];
    cplx<float> *Zs = reinterpret_cast<cplx<float> *>(zysm); // [RY][ZS]
    cplx<float> *Ex = Zs + RY * ZS;                          // exchange (z) / line staging (y)
    uint32_t     rank;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(rank));
    const long long plane = blockIdx.x / CL;                  // (rhs * C + c) * nx + x
    const int       t     = threadIdx.x;
    const long long ppr   = (long long)p.C * p.g.nx;          // planes per right-hand side
    if (p.active && !p.active[plane / ppr])
        return; // the whole cluster leaves: its RHS is inactive

    // rows [rank * RY, rank * RY + RY) of the plane, 16-byte copies into rows of ZS complex
    {
        const float *src = r + plane * (long long)NY * (2 * M) + (long long)rank * RY * (2 * M);
        for (int i = t; i < RY * (M / 2); i += L::NT) {
            const int row = i / (M / 2), q = i % (M / 2); // q: 16-byte chunk (2 complex) of the row
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(
                             (uint32_t)__cvta_generic_to_shared(Zs + row * ZS + 2 * q)),
                         "l"(src + (long long)row * (2 * M) + 4 * q)
                         : "memory");
        }
        asm volatile("cp.async.commit_group;\n\tcp.async.wait_all;" ::: "memory");
        __syncthreads();
    }

    // r2c along z, RZ rows at a time
    {
        const int Lr = t / N1z, w = t % N1z;
        for (int r0 = 0; r0 < RY; r0 += RZ) {
            const int    row = r0 + Lr;
            const bool   ok  = row < RY;
            cplx<float> *Zr  = Zs + (ok ? row : 0) * ZS;
            cplx<float>  v[N2z];
#pragma unroll
            for (int j2 = 0; j2 < N2z; ++j2)
                v[j2] = ok ? Zr[w + N1z * j2] : cplx<float>{0, 0};
            line_phase1<float, N1z, N2z, false>(v, w, p.tw_z);
#pragma unroll
            for (int k2 = 0; k2 < N2z; ++k2)
                Ex[(Lr * N2z + k2) * EPz + w] = v[k2];
            __syncthreads();
            if (w < N2z && ok) {
                cplx<float> u[N1z];
#pragma unroll
                for (int j1 = 0; j1 < N1z; ++j1)
                    u[j1] = Ex[(Lr * N2z + w) * EPz + j1];
                Dft<float, N1z, false>::run(u);
#pragma unroll
                for (int k1 = 0; k1 < N1z; ++k1)
                    Zr[w + N2z * k1] = u[k1]; // the row's inputs were all read before the barrier
            }
            __syncthreads();
            // unpack to the half spectrum in place: the pair (k, M - k) by one thread
            for (int i = t; i < RZ * (M / 2 + 1); i += L::NT) {
                const int rr = r0 + i / (M / 2 + 1), k = i % (M / 2 + 1);
                if (rr >= RY)
                    continue;
                cplx<float> *Z  = Zs + rr * ZS;
                const int    km = k == 0 ? 0 : M - k;
                const cplx<float> a = Z[k], b = Z[km];
                auto out = [&](cplx<float> zk, cplx<float> zm, int kk) {
                    zm.y = -zm.y;
                    cplx<float> Ev = {0.5f * (zk.x + zm.x), 0.5f * (zk.y + zm.y)};
                    cplx<float> Od = {0.5f * (zk.x - zm.x), 0.5f * (zk.y - zm.y)};
                    cplx<float> P  = cmul(p.tw_r2c[kk], Od);
                    return cplx<float>{Ev.x + P.y, Ev.y - P.x};
                };
                if (k == 0) {
                    Z[0] = out(a, a, 0);
                    Z[M] = out(a, a, M);
                } else if (k == M / 2) {
                    Z[k] = out(a, a, k);
                } else {
                    Z[k]  = out(a, b, k);
                    Z[km] = out(b, a, km);
                }
            }
            __syncthreads();
        }
    }
    cluster_sync_all(); // every CTA's rows hold their half spectra

    // FFT along y of this CTA's kz tiles, the rows of the whole cluster through DSMEM
    {
        const int       w = t / KC, l = t % KC;
        const uint32_t  zbase = (uint32_t)__cvta_generic_to_shared(Zs);
        cplx<float>    *out   = p.spec + plane * (long long)NY * p.nzp;
        const int       ntz   = (M + 1 + KC - 1) / KC;
        for (int tz = (int)rank; tz < ntz; tz += CL) {
            const int  kz    = tz * KC + l;
            const bool valid = kz <= M;
            cplx<float> v[N2y];
#pragma unroll
            for (int j2 = 0; j2 < N2y; ++j2) {
                const int y = w + N1y * j2;
                v[j2]       = valid ? ld_dsmem(zbase + (uint32_t)(((y % RY) * ZS + kz) * 8), (uint32_t)(y / RY))
                                    : cplx<float>{0, 0};
            }
            line_phase1<float, N1y, N2y, false>(v, w, p.tw_y);
#pragma unroll
            for (int k2 = 0; k2 < N2y; ++k2)
                Ex[(k2 * N1y + w) * KC + l] = v[k2];
            __syncthreads();
            if (w < N2y) {
                cplx<float> u[N1y];
#pragma unroll
                for (int j1 = 0; j1 < N1y; ++j1)
                    u[j1] = Ex[(w * N1y + j1) * KC + l];
                Dft<float, N1y, false>::run(u);
                if (valid)
#pragma unroll
                    for (int k1 = 0; k1 < N1y; ++k1)
                        out[(long long)(w + N2y * k1) * p.nzp + kz] = u[k1];
            }
            __syncthreads();
        }
    }
    cluster_sync_all(); // peers may still read this CTA's rows until here
}

// ------------------------------------------------------------------ z inv ---
// Hermitian pack of the half spectrum, half-length inverse, real rows scaled by
// `sign`; fused partial <r, s> (solverCG.h:90-92) with delta/beta in the last block.
// Persistent: each CTA loops over blocks of R rows, and while one block is
// transformed cp.async brings the next block's spectrum rows (and, for the
// fused dot, its r rows) into the other buffer, so the DRAM reads overlap the
// transforms instead of alternating with them.
// RED: the pass takes the fused <r, s> (FP64 path, FANSGPU_SPECTRAL_DOT=0); without it the
// reduction and the r rows are compiled out, and more CTAs fit an SM
template <typename T, int N1, int N2, int R, bool RED>
__global__ void __launch_bounds__(R * N1, RED ? 2 : 4) k_z_inv_reg(ConvPlan<T> p, ConvArgs a)
{
    constexpr int M = N1 * N2, EP = N1 + 1;
    const int     XS = R * p.nzp; // spectrum rows at their global stride nzp
    extern __shared__ __align__(16) unsigned char zsm[];
    static_assert(32 % N1 == 0, "a row's workers share one warp");
    cplx<T>          *Xb = reinterpret_cast<cplx<T> *>(zsm); // [2][XS]
    cplx<T>          *E  = Xb + 2 * XS;                      // [R*N2*EP] exchange, per row
    cplx<T>          *Rb = E + R * N2 * EP;                  // [2][R*M] r rows (fused dot only)
    __shared__ double red_smem[32 * kMaxRhs];
    __shared__ __align__(8) uint64_t zbar[2];                // block copies of buffer 0 / 1
    __shared__ int    s_abort;
    volatile int     *abort_flag = &s_abort;
    const int       t = threadIdx.x, L = t / N1, w = t % N1;
    const long long rpr   = (long long)p.C * p.g.nx * p.g.ny; // rows per right-hand side
    const long long nrows = rpr * p.nrhs;
    const long long nblk  = (nrows + R - 1) / R;
    const uint32_t  bar0  = (uint32_t)__cvta_generic_to_shared(&zbar[0]);
    if (t == 0) {
        s_abort = 0;
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar0) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar0 + 8) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    // a block's rows belong to at most two right-hand sides (as in k_z_fwd_reg); a block is
    // skipped when all its rows belong to inactive ones
    auto live = [&](long long blk) {
        if (!p.active)
            return true;
        const int       k0   = (int)(blk * R / rpr);
        const long long last = min(blk * R + R, nrows) - 1;
        return p.active[k0] || (last >= (k0 + 1) * rpr && p.active[k0 + 1]);
    };
    // the block's spectrum rows (and r rows) are contiguous in global memory: one bulk copy each
    // by thread 0, completing on the buffer's mbarrier
    int waited[2] = {0, 0}; // block copies per buffer waited for (every thread keeps the count)
    int sent[2]   = {0, 0}; // block copies per buffer issued (thread 0; none after an abort)
    auto fetch = [&](long long blk, int b) {
        if (t != 0 || blk >= nblk || !live(blk) || *abort_flag)
            return;
        ++sent[b];
        const long long row0  = blk * R;
        const int       nval  = (int)(nrows - row0 < R ? nrows - row0 : R);
        const uint32_t  bytes = (uint32_t)(nval * p.nzp * sizeof(cplx<T>));
        const uint32_t  rbyt  = RED ? (uint32_t)(nval * M * sizeof(cplx<T>)) : 0u;
        const uint32_t  bar   = bar0 + 8 * b;
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        tma_expect(bar, bytes + rbyt);
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                         (uint32_t)__cvta_generic_to_shared(Xb + b * XS)),
                     "l"(p.spec + row0 * p.nzp), "r"(bytes), "r"(bar)
                     : "memory");
        if (RED)
            asm volatile(
                "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                    (uint32_t)__cvta_generic_to_shared(Rb + b * R * M)),
                "l"(reinterpret_cast<const cplx<T> *>(a.r) + row0 * M), "r"(rbyt), "r"(bar)
                : "memory");
    };
    T dotk[kMaxRhs]; // <r, s> per right-hand side, this thread's rows
#pragma unroll
    for (int q = 0; q < kMaxRhs; ++q)
        dotk[q] = (T)0;
    fetch(blockIdx.x, 0);
    int it = 0;
    for (long long blk = blockIdx.x; blk < nblk; blk += gridDim.x, ++it) {
        const int b = it & 1;
        fetch(blk + gridDim.x, b ^ 1); // the next block, into the other buffer (read two blocks ago)
        if (!live(blk))
            continue; // uniform across the CTA: nothing was fetched for it
        tma_bar_wait(bar0 + 8 * b, (uint32_t)(waited[b]++ & 1), abort_flag);
        const long long row0 = blk * R;
        // Hermitian pack of row L by its own N1 workers (lanes of one warp), straight into the
        // registers of phase 1: only that warp meets at the exchange
        const cplx<T> *Xr = Xb + b * XS + L * p.nzp;
        cplx<T>        v[N2];
#pragma unroll
        for (int j2 = 0; j2 < N2; ++j2) {
            const int k  = w + N1 * j2;
            cplx<T>   xk = Xr[k];
            cplx<T>   xm = Xr[M - k];
            if (k == 0) {
                xk.y = 0;
                xm.y = 0;
            }
            xm.y       = -xm.y;
            cplx<T> Ev = cadd(xk, xm);
            cplx<T> Od = cmulc(csub(xk, xm), p.tw_r2c[k]);
            v[j2]      = cplx<T>{Ev.x - Od.y, Ev.y + Od.x};
        }
        line_phase1<T, N1, N2, true>(v, w, p.tw_z);
#pragma unroll
        for (int k2 = 0; k2 < N2; ++k2)
            E[(L * N2 + k2) * EP + w] = v[k2];
        __syncwarp();
        const long long row = row0 + L;
        const int       rk0 = p.active || p.nrhs > 1 ? (int)(row0 / rpr) : 0;
        const int       rk  = rk0 + (row >= (rk0 + 1) * rpr ? 1 : 0);
        if (row < nrows && w < N2 && (!p.active || p.active[rk])) {
            cplx<T> u[N1];
#pragma unroll
            for (int j1 = 0; j1 < N1; ++j1)
                u[j1] = E[(L * N2 + w) * EP + j1];
            Dft<T, N1, true>::run(u);
            cplx<T>       *sout = reinterpret_cast<cplx<T> *>(a.s) + row * M;
            const cplx<T> *rr   = Rb + b * R * M + L * M;
            const T        sg   = (T)a.sign;
            T              dot  = (T)0;
#pragma unroll
            for (int k1 = 0; k1 < N1; ++k1) {
                const int m = w + N2 * k1;
                cplx<T>   z = {sg * u[k1].x, sg * u[k1].y};
                sout[m]     = z;
                if (RED) {
                    const cplx<T> rv = rr[m];
                    dot += rv.x * z.x + rv.y * z.y;
                }
            }
#pragma unroll
            for (int q = 0; q < kMaxRhs; ++q)
                if (q == rk)
                    dotk[q] += dot;
        }
        __syncthreads(); // buffer b is free for the fetch two blocks on
    }
    __syncthreads();
    if (t == 0 && *abort_flag) {
        // wait (bounded) for the copies still in flight, then report the expired wait
        for (int b = 0; b < 2; ++b)
            if (sent[b] > 0)
                for (unsigned n = 0;
                     n < kTmaWaitLimit && !tma_bar_try(bar0 + 8 * b, (uint32_t)((sent[b] - 1) & 1)); ++n)
                    ;
        if (a.scal)
            for (int q = 0; q < p.nrhs; ++q)
                if (!p.active || p.active[q])
                    a.scal[q].converged = -3;
    }
    if (RED) {
        double vv[kMaxRhs];
        int    ops[kMaxRhs];
#pragma unroll
        for (int q = 0; q < kMaxRhs; ++q) {
            vv[q]  = (double)dotk[q];
            ops[q] = RED_SUM;
        }
        block_reduce<kMaxRhs>(vv, ops, red_smem);
        if (grid_partial_commit<kMaxRhs>(vv, a.red.partials, a.red.counter + a.red_site, gridDim.x)) {
            grid_final<kMaxRhs>(vv, ops, a.red.partials, gridDim.x, red_smem);
            if (threadIdx.x == 0)
                for (int q = 0; q < p.nrhs; ++q) {
                    if (p.active && !p.active[q])
                        continue;
                    CgScalars *s = a.scal + q;
                    s->delta0    = s->delta;
                    s->delta     = vv[q];
                    double beta  = (s->delta - s->deltamid) / s->delta0;
                    s->beta      = beta > 0.0 ? beta : 0.0;
                }
        }
    }
}

// --------------------------------------------------------------- dispatch ---
template <typename T, int N1, int N2, bool INV, int KC>
void go_y(const ConvPlan<T> &p, cudaStream_t st)
{
    dim3 g((p.nzh + KC - 1) / KC, p.g.nx, p.C * p.nrhs);
    k_y_reg<T, N1, N2, INV, KC><<<g, KC * N1, 0, st>>>(p);
}

template <typename T, int N1, int N2, int KC>
cudaError_t go_x(const ConvPlan<T> &p, const ConvArgs &a, cudaStream_t st)
{
    dim3         g((p.nzh + KC - 1) / KC, p.g.ny);
    const size_t n = (size_t)N1 * N2;
    if (p.C == 1) {
        const size_t sm = sizeof(cplx<T>) * n * KC + sizeof(T) * n * KC * 1;
        cudaError_t  e  = allow_max_dyn_smem(k_x_green_reg<T, N1, N2, 1, KC>);
        if (e != cudaSuccess)
            return e;
        k_x_green_reg<T, N1, N2, 1, KC><<<g, KC * N1, sm, st>>>(p, a);
    } else {
        const size_t sm = sizeof(cplx<T>) * 3 * n * KC + sizeof(T) * n * KC * 6;
        cudaError_t  e  = allow_max_dyn_smem(k_x_green_reg<T, N1, N2, 3, KC>);
        if (e != cudaSuccess)
            return e;
        k_x_green_reg<T, N1, N2, 3, KC><<<g, 3 * KC * N1, sm, st>>>(p, a);
    }
    return cudaSuccess;
}

// the TMA-fed x pass (FP32 plans with tensor maps): persistent, as many CTAs per SM as fit
template <int N1, int N2>
cudaError_t go_x_tma(const ConvPlan<float> &p, const ConvArgs &a, cudaStream_t st)
{
    const TmaMaps *m   = static_cast<const TmaMaps *>(p.tma);
    const int      ntz = (p.nzh + kTmaKC - 1) / kTmaKC;
    auto           run = [&]<int C>() -> cudaError_t {
        constexpr int  NTH = C * kTmaKC * N1;
        constexpr int  SM  = XTma<N1, N2, C>::SMEM;
        auto           fn  = k_x_green_tma<N1, N2, C>;
        static int     grid_per_sm = 0, nsm = 0;
        cudaError_t    e   = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, SM);
        if (e != cudaSuccess)
            return e;
        if (!grid_per_sm) {
            int dev = 0;
            cudaGetDevice(&dev);
            cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&grid_per_sm, fn, NTH, SM) != cudaSuccess ||
                grid_per_sm < 1)
                grid_per_sm = 1;
        }
        long long jobs = (long long)ntz * p.g.ny * p.nrhs;
        const int grid = (int)(jobs < (long long)grid_per_sm * nsm ? jobs : (long long)grid_per_sm * nsm);
        CUtensorMap ts, tg;
        std::memcpy(&ts, m->spec, sizeof ts);
        std::memcpy(&tg, m->green, sizeof tg);
        fn<<<grid, NTH, SM, st>>>(p, a, ts, tg);
        return cudaGetLastError();
    };
    return p.C == 1 ? run.template operator()<1>() : run.template operator()<3>();
}

template <typename T, int N1, int N2, int R>
void go_zf(const ConvPlan<T> &p, const T *r, cudaStream_t st)
{
    const long long nrows = (long long)p.C * p.g.nx * p.g.ny * p.nrhs;
    k_z_fwd_reg<T, N1, N2, R><<<(int)((nrows + R - 1) / R), R * N1, 0, st>>>(p, r);
}

template <typename T, int N1, int N2, int R>
cudaError_t go_zi(const ConvPlan<T> &p, const ConvArgs &a, cudaStream_t st)
{
    constexpr int   M     = N1 * N2;
    const long long nrows = (long long)p.C * p.g.nx * p.g.ny * p.nrhs;
    const long long nblk  = (nrows + R - 1) / R;
    static int      nsm   = 0;
    if (!nsm) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    }
    // spectrum rows [2][R][nzp], the rows' exchange [R][N2][N1 + 1], and r rows [2][R][M] for
    // the fused dot
    const size_t sm = sizeof(cplx<T>) * (size_t)(2 * R * p.nzp + R * N2 * (N1 + 1) + (a.reduce ? 2 * R * M : 0));
    auto        fn = a.reduce ? k_z_inv_reg<T, N1, N2, R, true> : k_z_inv_reg<T, N1, N2, R, false>;
    cudaError_t e  = allow_max_dyn_smem(fn);
    if (e != cudaSuccess)
        return e;
    // persistent: as many CTAs per SM as fit (at least two), at most one per block of rows
    static int occ[2] = {0, 0};
    int       &oc     = occ[a.reduce ? 1 : 0];
    if (!oc) {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&oc, fn, R * N1, sm) != cudaSuccess)
            oc = 2;
        oc = oc < 2 ? 2 : oc;
    }
    const int grid = (int)(nblk < (long long)oc * nsm ? nblk : (long long)oc * nsm);
    fn<<<grid, R * N1, sm, st>>>(p, a);
    return cudaSuccess;
}

// call F<N1, N2>() for the register plan of length n; false if none
template <typename Fn>
bool with_plan(int n, Fn &&f)
{
    switch (n) {
    case 16: f.template operator()<4, 4>(); return true;
    case 24: f.template operator()<8, 3>(); return true;
    case 32: f.template operator()<8, 4>(); return true;
    case 40: f.template operator()<8, 5>(); return true;
    case 48: f.template operator()<8, 6>(); return true;
    case 64: f.template operator()<8, 8>(); return true;
    case 80: f.template operator()<16, 5>(); return true;
    case 96: f.template operator()<16, 6>(); return true;
    case 128: f.template operator()<16, 8>(); return true;
    case 256: f.template operator()<16, 16>(); return true;
    default: return false;
    }
}

// z-pass plans (M <= 128)
template <typename Fn>
bool with_plan_z(int n, Fn &&f)
{
    return n <= 128 && with_plan(n, f);
}

// the fused z + y forward pass for cubic-in-(y, z) grids (nz == ny) whose half length has a
// register plan; CL = the smallest cluster whose CTAs fit two per SM
template <int N1y, int N2y>
struct ZyPick {
    static constexpr int  NY = N1y * N2y, M = NY / 2, N1z = reg_n1(M) ? reg_n1(M) : 1, N2z = M / N1z;
    template <int CL>
    static constexpr bool fits = NY % CL == 0 && ZyFwd<N1z, N2z, N1y, N2y, CL>::SMEM <= 113 * 1024;
    static constexpr int  CL = !reg_n1(M) ? 0 : fits<1> ? 1 : fits<2> ? 2 : fits<4> ? 4 : fits<8> ? 8 : 0;
};

bool zy_supported_impl(const Grid3 &g)
{
    bool ok = false;
    if (g.nz == g.ny && g.nz / 2 <= 128)
        with_plan(g.ny, [&]<int N1, int N2>() { ok = ZyPick<N1, N2>::CL != 0; });
    return ok;
}

cudaError_t go_zy(const ConvPlan<float> &p, const float *r, cudaStream_t st)
{
    cudaError_t e = cudaErrorNotSupported;
    if (p.g.nz != p.g.ny)
        return e;
    with_plan(p.g.ny, [&]<int N1y, int N2y>() {
        using P = ZyPick<N1y, N2y>;
        if constexpr (P::CL != 0) {
            constexpr int CL = P::CL;
            using L          = ZyFwd<P::N1z, P::N2z, N1y, N2y, CL>;
            auto fn          = k_zy_fwd<P::N1z, P::N2z, N1y, N2y, CL>;
            if ((e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, L::SMEM)) != cudaSuccess)
                return;
            cudaLaunchConfig_t  cfg{};
            cudaLaunchAttribute at[1];
            at[0].id               = cudaLaunchAttributeClusterDimension;
            at[0].val.clusterDim.x = CL;
            at[0].val.clusterDim.y = 1;
            at[0].val.clusterDim.z = 1;
            cfg.gridDim            = dim3((unsigned)(CL * (long long)p.nrhs * p.C * p.g.nx));
            cfg.blockDim           = dim3(L::NT);
            cfg.dynamicSmemBytes   = L::SMEM;
            cfg.stream             = st;
            cfg.attrs              = at;
            cfg.numAttrs           = 1;
            e                      = cudaLaunchKernelEx(&cfg, fn, p, r);
        }
    });
    return e;
}


} // namespace

bool zy_supported(const Grid3 &g) { return zy_supported_impl(g); }

bool conv_reg_supported(const Grid3 &g)
{
    // z passes keep R rows of M complex twice in static shared memory: M <= 128
    return reg_n1(g.nx) && reg_n1(g.ny) && reg_n1(g.nz / 2) && g.nz / 2 <= 128;
}

template <typename T>
cudaError_t launch_convolution_reg(const ConvPlan<T> &p, const ConvArgs &a, cudaStream_t st)
{
    if (!conv_reg_supported(p.g))
        return cudaErrorNotSupported;
    auto mark = [&](int i) {
        if (a.ev)
            cudaEventRecord(a.ev[i], st);
    };
    cudaError_t e = cudaSuccess;
    using TL      = Tiles<T>;
    const T *r    = reinterpret_cast<const T *>(a.r);
    mark(0);
    bool fused = false;
    if constexpr (std::is_same_v<T, float>)
        if (p.fuse_zy) {
            if ((e = go_zy(p, r, st)) != cudaSuccess)
                return e;
            fused = true;
        }
    if (!fused)
        with_plan_z(p.M, [&]<int N1, int N2>() {
            p.var_z ? go_zf<T, N1, N2, TL::z[1] / N1>(p, r, st) : go_zf<T, N1, N2, TL::z[0] / N1>(p, r, st);
        });
    mark(1);
    if (!fused)
        with_plan(p.g.ny, [&]<int N1, int N2>() {
            p.var_y ? go_y<T, N1, N2, false, TL::y[1]>(p, st) : go_y<T, N1, N2, false, TL::y[0]>(p, st);
        });
    mark(2);
    with_plan(p.g.nx, [&]<int N1, int N2>() {
        if constexpr (std::is_same_v<T, float>)
            if (p.var_x == 2 && p.tma) {
                e = go_x_tma<N1, N2>(p, a, st);
                return;
            }
        e = p.var_x == 1 ? go_x<T, N1, N2, TL::x[1]>(p, a, st) : go_x<T, N1, N2, TL::x[0]>(p, a, st);
    });
    if (e != cudaSuccess)
        return e;
    mark(3);
    with_plan(p.g.ny, [&]<int N1, int N2>() {
        p.var_y ? go_y<T, N1, N2, true, TL::y[1]>(p, st) : go_y<T, N1, N2, true, TL::y[0]>(p, st);
    });
    mark(4);
    ConvArgs az = a; // with the spectral <r, s>, the z-inverse pass only transforms
    if (p.spectral_dot)
        az.reduce = 0;
    with_plan_z(p.M, [&]<int N1, int N2>() {
        e = p.var_z ? go_zi<T, N1, N2, TL::z[1] / N1>(p, az, st) : go_zi<T, N1, N2, TL::z[0] / N1>(p, az, st);
    });
    if (e != cudaSuccess)
        return e;
    mark(5);
    return cudaGetLastError();
}

// The autotuner of the register passes: for each of the z, y and x passes,
// time its two tile variants on this plan's buffers (r in, s out, no fused
// dot; one warm-up and three timed launches each, CUDA events on `st`) and
// keep the faster in p.var_*.  The variants compute the same values per line,
// so the choice changes the speed only (the fused dot of the z inverse pass
// sums in another block order).
template <typename T>
cudaError_t tune_convolution_reg(ConvPlan<T> &p, const T *r, T *s, CgScalars *scal, GridRed red, int red_site,
                                 cudaStream_t st)
{
    if (!conv_reg_supported(p.g))
        return cudaSuccess;
    using TL = Tiles<T>;
    ConvArgs    a{r, s, 1.0, 1, scal, red, red_site, nullptr}; // with the fused <r, s>, as in the iteration
    ConvArgs    az = a;                                        // in the x pass when spectral
    if (p.spectral_dot)
        az.reduce = 0;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t e  = cudaEventCreate(&e0);
    if (e == cudaSuccess)
        e = cudaEventCreate(&e1);
    auto timed = [&](auto &&launch) -> float {
        float ms = 1e30f;
        if (e != cudaSuccess)
            return ms;
        launch();
        if ((e = cudaEventRecord(e0, st)) != cudaSuccess)
            return ms;
        for (int k = 0; k < 5; ++k)
            launch();
        if ((e = cudaEventRecord(e1, st)) == cudaSuccess && (e = cudaEventSynchronize(e1)) == cudaSuccess &&
            (e = cudaGetLastError()) == cudaSuccess)
            cudaEventElapsedTime(&ms, e0, e1);
        return ms;
    };
    float t[2];
    for (int v = 0; v < 2; ++v)
        t[v] = timed([&] {
            with_plan_z(p.M, [&]<int N1, int N2>() {
                if (v) {
                    go_zf<T, N1, N2, TL::z[1] / N1>(p, r, st);
                    e = go_zi<T, N1, N2, TL::z[1] / N1>(p, az, st);
                } else {
                    go_zf<T, N1, N2, TL::z[0] / N1>(p, r, st);
                    e = go_zi<T, N1, N2, TL::z[0] / N1>(p, az, st);
                }
            });
        });
    p.var_z = t[1] < t[0] ? 1 : 0;
    for (int v = 0; v < 2; ++v)
        t[v] = timed([&] {
            with_plan(p.g.ny, [&]<int N1, int N2>() {
                v ? go_y<T, N1, N2, false, TL::y[1]>(p, st) : go_y<T, N1, N2, false, TL::y[0]>(p, st);
            });
        });
    p.var_y = t[1] < t[0] ? 1 : 0;
    // x: 64- and 32-byte rows, the TMA-fed pass (FP32 with tensor maps)
    float tx[3] = {1e30f, 1e30f, 1e30f};
    for (int v = 0; v < 3; ++v) {
        if (v == 2 && !(std::is_same_v<T, float> && p.tma))
            continue;
        tx[v] = timed([&] {
            with_plan(p.g.nx, [&]<int N1, int N2>() {
                if constexpr (std::is_same_v<T, float>)
                    if (v == 2) {
                        e = go_x_tma<N1, N2>(p, a, st);
                        return;
                    }
                e = v ? go_x<T, N1, N2, TL::x[1]>(p, a, st) : go_x<T, N1, N2, TL::x[0]>(p, a, st);
            });
        });
    }
    p.var_x = 0;
    for (int v = 1; v < 3; ++v)
        if (tx[v] < tx[p.var_x])
            p.var_x = v;
    // the forward z and y passes (the chosen variants) against the fused cluster pass
    p.fuse_zy = 0;
    if constexpr (std::is_same_v<T, float>)
        if (zy_supported_impl(p.g)) {
            const float t_sep = timed([&] {
                with_plan_z(p.M, [&]<int N1, int N2>() {
                    p.var_z ? go_zf<T, N1, N2, TL::z[1] / N1>(p, r, st) : go_zf<T, N1, N2, TL::z[0] / N1>(p, r, st);
                });
                with_plan(p.g.ny, [&]<int N1, int N2>() {
                    p.var_y ? go_y<T, N1, N2, false, TL::y[1]>(p, st) : go_y<T, N1, N2, false, TL::y[0]>(p, st);
                });
            });
            const float t_fused = timed([&] { e = go_zy(p, r, st); });
            p.fuse_zy = t_fused < t_sep ? 1 : 0;
        }
    if (e0)
        cudaEventDestroy(e0);
    if (e1)
        cudaEventDestroy(e1);
    return e;
}

bool make_x_tma_maps(const ConvPlan<float> &p, TmaMaps *out)
{
    static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    static bool                              looked = false;
    if (!looked) {
        looked                               = true;
        cudaDriverEntryPointQueryResult qres = cudaDriverEntryPointSymbolNotFound;
        void                           *fn   = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &qres) ==
                cudaSuccess &&
            qres == cudaDriverEntryPointSuccess)
            encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
        else
            cudaGetLastError();
    }
    const int nx = p.g.nx, ny = p.g.ny, NT = p.C * (p.C + 1) / 2;
    if (!encode || !reg_n1(nx) || nx > 256 || (p.C != 1 && p.C != 3) || p.gzs != p.nzp)
        return false;
    const cuuint32_t one[3] = {1, 1, 1};
    // spectrum: floats [nrhs_alloc * C * nx][ny][2 * nzh], rows 2 * nzp floats apart
    const cuuint64_t sd[3]  = {(cuuint64_t)2 * p.nzh, (cuuint64_t)ny, (cuuint64_t)p.nrhs_alloc * p.C * nx};
    const cuuint64_t ss[2]  = {(cuuint64_t)2 * p.nzp * 4, (cuuint64_t)ny * 2 * p.nzp * 4};
    const cuuint32_t sbx[3] = {2 * kTmaKC, 1, (cuuint32_t)nx};
    // Green's table: floats [nx][ny][nzh * NT], rows nzp * NT floats apart
    const cuuint64_t gd[3]  = {(cuuint64_t)p.nzh * NT, (cuuint64_t)ny, (cuuint64_t)nx};
    const cuuint64_t gs[2]  = {(cuuint64_t)p.nzp * NT * 4, (cuuint64_t)ny * p.nzp * NT * 4};
    const cuuint32_t gbx[3] = {(cuuint32_t)(kTmaKC * NT), 1, (cuuint32_t)nx};
    CUresult r1 = encode(reinterpret_cast<CUtensorMap *>(out->spec), CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, p.spec, sd,
                         ss, sbx, one, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                         CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    CUresult r2 = encode(reinterpret_cast<CUtensorMap *>(out->green), CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3,
                         const_cast<float *>(p.G), gd, gs, gbx, one, CU_TENSOR_MAP_INTERLEAVE_NONE,
                         CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r1 == CUDA_SUCCESS && r2 == CUDA_SUCCESS;
}

template cudaError_t launch_convolution_reg<double>(const ConvPlan<double> &, const ConvArgs &, cudaStream_t);
template cudaError_t launch_convolution_reg<float>(const ConvPlan<float> &, const ConvArgs &, cudaStream_t);
template cudaError_t tune_convolution_reg<double>(ConvPlan<double> &, const double *, double *, CgScalars *, GridRed,
                                                   int, cudaStream_t);
template cudaError_t tune_convolution_reg<float>(ConvPlan<float> &, const float *, float *, CgScalars *, GridRed, int,
                                                  cudaStream_t);

} // namespace fansgpu
