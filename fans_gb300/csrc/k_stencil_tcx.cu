// k_stencil_tcx.cu -- the FP64-accurate linear operator y = K x (+ F), with the
// fused CG direction d = s + beta d_old and <d, K d>, on the tensor cores of
// sm_103a: the true residual of the mixed path's reliable updates
// (solver.h:231-270 with phase_stiffness, solverCG.h:97-103) and the operator
// of the FP64 CG path.
//
// Arithmetic.  K_ph = sum_b c_ph,b q_b W_b with exact integer basis blocks W_b
// (as in k_stencil_tcb.cu).  Per element the 8C displacements relative to its
// first node (solver.h:252) are formed from the FP64 input as double-float
// values d = dh + dl, then written in fixed point against the element's largest
// |dh|: with scale = 2^(10 - e), d scale = s0 + s1 2^-11 + s2 2^-22 + s3 2^-33
// + O(2^-34), each slice an integer of at most 11 bits (exact in tf32).  A slice
// times an integer W_b entry (at most 7 bits) and the sum over the 8C columns
// stay integers below 2^24, so the tensor core computes each D_j = s_j W_b^T
// exactly in its FP32 accumulator.  The consumers recombine
// D_0 + 2^-11 D_1 + 2^-22 D_2 + 2^-33 D_3 as a double-float, undo the scale,
// multiply by the phase coefficient (a double-float) and sum element rows into
// nodes in double-float: relative error about 2^-44 of the element's largest
// displacement difference, as the double-float kernel on the CUDA cores.
//
// Pipeline as in the FP32 operators: a CTA owns a 3 (y) x 31 (z) node column
// and marches over 64 x planes; producers stage node planes (FP64 copied by
// cp.async three planes ahead, split into FP32 hi/lo) and write the four slices
// of each element row into shared memory (the MMAs' A operand); one thread
// issues the 4 x 8C/8 MMAs into four tensor-memory accumulators; consumers
// recombine, add the element force and sum into nodes (register carry in x, warp
// shuffle in z, exchange buffer in y).  Bounded mbarrier waits with an abort
// flag, as in the other operators.
#include "kernels.cuh"

#include <cmath>
#include <cstring>

namespace fansgpu {

namespace {

constexpr int BY = 3, BZ = 31;
constexpr int PY = BY + 2, PZ = BZ + 2;
constexpr int EYN = BY + 1, EZN = BZ + 1;
constexpr int NEL  = EYN * EZN; // 128 elements = one M-tile
constexpr int NGRP = 128;
constexpr int TPB  = 2 * NGRP + 32;
constexpr int NPL  = PY * PZ;
constexpr int XL   = 64;
constexpr int R    = 4; // node-plane slots
constexpr int RAWD = 3; // raw FP64 planes in flight
constexpr int NSL  = 4; // fixed-point slices
constexpr int TCOLS = 256;           // accumulator j at columns j NW
constexpr int SMEM_REQ = 110 * 1024; // two CTAs per SM (256 tensor-memory columns each)
constexpr unsigned kWaitLimit  = 1u << 22;
constexpr unsigned kDrainLimit = 1u << 22;
constexpr int kMaxPhX = 16;
enum {
    BAR_AFULL  = 0,
    BAR_DFULL  = 1,
    BAR_DFREE  = 2,
    BAR_STAGED = 3,
    BAR_SFREE  = 3 + R,
    BAR_DRAIN  = 3 + 2 * R,
    BAR_INV    = 4 + 2 * R, // + (plane & 1): the element scales of a plane written (producers -> consumers)
    NBAR       = 6 + 2 * R
};

template <int C, int NB>
struct TxCfg {
    static constexpr int NCOL    = 8 * C;
    static constexpr int KC      = NCOL / 4;
    static constexpr int SBO     = KC * 128;
    static constexpr int LBO     = 128;
    static constexpr int NROW    = NB * NCOL;
    static constexpr int NW      = (NROW + 15) / 16 * 16;
    static constexpr int KSTEPS  = NCOL / 8;
    static constexpr int W_BYTES = NW * NCOL * 4;
    static constexpr int NPF     = (C * NPL + NGRP - 1) / NGRP;
    static constexpr int al(int b) { return (b + 127) / 128 * 128; }
    static constexpr int A_BYTES  = NEL * NCOL * 4;                        // one slice of A, K-major core matrices
    static constexpr int OFF_W    = 0;
    static constexpr int OFF_A    = al(OFF_W + W_BYTES);                   // [NSL][A_BYTES]
    static constexpr int OFF_COEF = al(OFF_A + NSL * A_BYTES);             // [kMaxPhX][NB][hi, lo]
    static constexpr int OFF_F    = al(OFF_COEF + kMaxPhX * NB * 2 * 4);   // [hi, lo][kMaxPhX][NCOL]
    static constexpr int OFF_SH   = al(OFF_F + 2 * kMaxPhX * NCOL * 4);    // staged hi [R][C][NPL]
    static constexpr int OFF_SL   = al(OFF_SH + R * C * NPL * 4);          // staged lo
    static constexpr int OFF_RAW  = al(OFF_SL + R * C * NPL * 4);          // [RAWD][x, d_old][C][NPL] double
    static constexpr int OFF_X    = al(OFF_RAW + RAWD * 2 * C * NPL * 8);  // [2][EYN][hi, lo][C][32]
    static constexpr int OFF_INV  = al(OFF_X + 2 * EYN * 2 * C * 32 * 4);  // [2][NEL] 1 / scale
    static constexpr int OFF_BAR  = al(OFF_INV + 2 * NEL * 4);
    static constexpr int OFF_RED  = al(OFF_BAR + NBAR * 8 + 8);
    static constexpr int SMEM     = OFF_RED + 32 * 8;
    static_assert(NSL * NW <= TCOLS, "tensor-memory map");
    static_assert(SMEM <= SMEM_REQ, "shared memory");
};

__device__ __forceinline__ int pmod(int i, int n)
{
    int r = i % n;
    return r < 0 ? r + n : r;
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

template <int SBO_, int LBO_>
__device__ __forceinline__ uint64_t umma_desc(uint32_t addr)
{
    uint64_t d = (uint64_t)((addr & 0x3FFFF) >> 4);
    d |= (uint64_t)(LBO_ >> 4) << 16;
    d |= (uint64_t)(SBO_ >> 4) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

__device__ __forceinline__ int wrapi(int x, int n) { return x < 0 ? x + n : (x >= n ? x - n : x); }

// s + e = a + b exactly
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e)
{
    s       = a + b;
    float z = s - a;
    e       = (a - (s - z)) + (b - z);
}

// (h, l) += (bh, bl)
__device__ __forceinline__ void df_add(float &h, float &l, float bh, float bl)
{
    float s, e;
    two_sum(h, bh, s, e);
    h = s;
    l = l + bl + e;
}

// the same on two lanes at once (packed FP32x2; each lane is an IEEE single operation)
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }

__device__ __forceinline__ void two_sum2(float2 a, float2 b, float2 &s, float2 &e)
{
    s              = __fadd2_rn(a, b);
    const float2 z = __fadd2_rn(s, neg2(a));
    e              = __fadd2_rn(__fadd2_rn(a, neg2(__fadd2_rn(s, neg2(z)))), __fadd2_rn(b, neg2(z)));
}

__device__ __forceinline__ void df_add2(float2 &h, float2 &l, float2 bh, float2 bl)
{
    float2 s, e;
    two_sum2(h, bh, s, e);
    h = s;
    l = __fadd2_rn(__fadd2_rn(l, bl), e);
}

__device__ __forceinline__ void tmem_ld4(uint32_t taddr, float *v)
{
    uint32_t r[4];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(taddr));
#pragma unroll
    for (int j = 0; j < 4; ++j)
        v[j] = __uint_as_float(r[j]);
}

// D (tmem) += A (smem descriptor) * B^T (smem descriptor); acc = 0 overwrites
__device__ __forceinline__ void umma_tf32_ss(uint32_t dtmem, uint64_t ad, uint64_t bd, uint32_t idesc, uint32_t acc)
{
    asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                 " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
                 "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity)
{
    uint32_t done;
    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                 " selp.u32 %0, 1, 0, p;\n}\n"
                 : "=r"(done)
                 : "r"(bar), "r"(parity)
                 : "memory");
    return done != 0;
}

__device__ __forceinline__ void mbar_wait(uint32_t bar, uint32_t parity, volatile int *abort_flag, unsigned limit)
{
    for (unsigned it = 0; it < limit; ++it)
        if (mbar_try(bar, parity) || *abort_flag)
            return;
    *abort_flag = 1;
}

__device__ __forceinline__ void named_bar(int id, int nthreads)
{
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

// 96 registers: two CTAs of nine warps per SM need five warps' registers on one scheduler
// (5 x 32 x 96 <= 16384); at 104-112 only one CTA was resident and the kernel ran 1.6x slower.
template <int C, int NB>
__global__ void __maxnreg__(96)
    k_stencil_tcx(StencilArgs a, const float *__restrict__ Wg, const float *__restrict__ coefg,
                  const float *__restrict__ fg)
{
    using Cfg = TxCfg<C, NB>;
    constexpr int NCOL = Cfg::NCOL, NPF = Cfg::NPF, NW = Cfg::NW;
    extern __shared__ __align__(16) unsigned char smem[];
    float        *SH         = reinterpret_cast<float *>(smem + Cfg::OFF_SH);
    float        *SL         = reinterpret_cast<float *>(smem + Cfg::OFF_SL);
    double       *Raw        = reinterpret_cast<double *>(smem + Cfg::OFF_RAW);
    float        *Xch        = reinterpret_cast<float *>(smem + Cfg::OFF_X);
    float        *Inv        = reinterpret_cast<float *>(smem + Cfg::OFF_INV);
    const float  *coef       = reinterpret_cast<const float *>(smem + Cfg::OFF_COEF);
    const float  *fsm        = reinterpret_cast<const float *>(smem + Cfg::OFF_F);
    const uint32_t bar0      = smem_u32(smem + Cfg::OFF_BAR);
    uint32_t     *tmem_slot  = reinterpret_cast<uint32_t *>(smem + Cfg::OFF_BAR + NBAR * 8);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(smem + Cfg::OFF_BAR + NBAR * 8 + 4);
    double       *red_smem   = reinterpret_cast<double *>(smem + Cfg::OFF_RED);
    auto bar = [&](int i) { return bar0 + 8u * (uint32_t)i; };
    const unsigned wlim = a.wait_limit > 0 ? (unsigned)a.wait_limit : kWaitLimit;

    const int nx = a.g.nx, ny = a.g.ny, nz = a.g.nz;
    const long long N = (long long)nx * ny * nz;
    const int tid = threadIdx.x, warp = tid / 32, lane = tid % 32;
    const int y0 = blockIdx.y * BY, z0 = blockIdx.z * BZ;
    const int xs = blockIdx.x * XL, xe = min(xs + XL, nx);
    const int J  = xe - xs + 1;
    const long long plane = (long long)ny * nz;
    const bool fuse = a.fuse_d != 0, force = fg != nullptr;

    // ---- setup: W, phase coefficients (hi, lo), element force (hi, lo), barriers, tensor memory
    for (int i = tid; i < Cfg::W_BYTES / 16; i += TPB)
        reinterpret_cast<float4 *>(smem + Cfg::OFF_W)[i] = reinterpret_cast<const float4 *>(Wg)[i];
    for (int i = tid; i < a.nph * NB * 2; i += TPB)
        reinterpret_cast<float *>(smem + Cfg::OFF_COEF)[i] = coefg[i];
    if (force)
        for (int i = tid; i < a.nph * NCOL; i += TPB) {
            reinterpret_cast<float *>(smem + Cfg::OFF_F)[i]                   = fg[i];
            reinterpret_cast<float *>(smem + Cfg::OFF_F)[kMaxPhX * NCOL + i] = fg[(size_t)a.nph * NCOL + i];
        }
    if (tid == 0) {
        mbar_init(bar(BAR_AFULL), NGRP);
        mbar_init(bar(BAR_DFULL), 1);
        mbar_init(bar(BAR_DFREE), NGRP);
        for (int s = 0; s < R; ++s) {
            mbar_init(bar(BAR_STAGED + s), NGRP);
            mbar_init(bar(BAR_SFREE + s), NGRP);
        }
        mbar_init(bar(BAR_DRAIN), 1);
        mbar_init(bar(BAR_INV), NGRP);
        mbar_init(bar(BAR_INV + 1), NGRP);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "n"(TCOLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;
    double         dot  = 0.0;

    if (warp < 4) {
        // ================================================================ producers
        const int     ey = warp, ez = lane;
        const double *xin  = reinterpret_cast<const double *>(a.x);
        const double *dold = reinterpret_cast<const double *>(a.d_old);
        double       *dnew = reinterpret_cast<double *>(a.d_new);
        const double  beta = fuse ? a.scal->beta : 0.0;
        // this element's row of A: row e = 32 ey + ez in K-major core matrices (8 rows x 16 bytes)
        const int e_row = ey * 32 + ez;
        float    *arow  = reinterpret_cast<float *>(smem + Cfg::OFF_A) + ((e_row / 8) * Cfg::SBO + (e_row % 8) * 16) / 4;
        long long goff[NPF];
        int       loff[NPF];
        unsigned  owned_mask = 0, valid_mask = 0;
#pragma unroll
        for (int k = 0; k < NPF; ++k) {
            const int idx = tid + k * NGRP;
            goff[k] = 0;
            loff[k] = 0;
            if (idx < C * NPL) {
                const int c = idx / NPL, rem = idx % NPL, hy = rem / PZ, hz = rem % PZ;
                const int y = y0 - 1 + hy, z = z0 - 1 + hz;
                goff[k] = c * N + (long long)pmod(y, ny) * nz + pmod(z, nz);
                loff[k] = c * NPL + rem;
                valid_mask |= 1u << k;
                if (hy >= 1 && hy <= BY && hz >= 1 && hz <= BZ && y < ny && z < nz)
                    owned_mask |= 1u << k;
            }
        }
        // node plane m (xs-1+m): x (and d_old) in FP64 into raw slot m % RAWD, RAWD-1 planes ahead
        auto fetch = [&](int m) {
            if (m <= J) {
                const long long gx  = (long long)wrapi(xs - 1 + m, nx) * plane;
                double         *raw = Raw + (m % RAWD) * 2 * C * NPL;
#pragma unroll
                for (int k = 0; k < NPF; ++k)
                    if (valid_mask & (1u << k)) {
                        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_u32(raw + loff[k])),
                                     "l"(xin + goff[k] + gx)
                                     : "memory");
                        if (fuse)
                            asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(
                                             smem_u32(raw + C * NPL + loff[k])),
                                         "l"(dold + goff[k] + gx)
                                         : "memory");
                    }
            }
            asm volatile("cp.async.commit_group;" ::: "memory");
        };
        // node plane m into slot m % R as FP32 hi + lo (d = s + beta d_old first when fused,
        // d_new written for owned nodes)
        auto stage = [&](int m) {
            asm volatile("cp.async.wait_group %0;" ::"n"(RAWD - 2) : "memory");
            const int       X       = xs - 1 + m;
            const bool      owned_x = X >= xs && X < xe;
            const long long gx      = (long long)wrapi(X, nx) * plane;
            const double   *raw     = Raw + (m % RAWD) * 2 * C * NPL;
            float          *sh      = SH + (m % R) * C * NPL;
            float          *sl      = SL + (m % R) * C * NPL;
#pragma unroll
            for (int k = 0; k < NPF; ++k)
                if (valid_mask & (1u << k)) {
                    double v = raw[loff[k]];
                    if (fuse) {
                        v = fma(beta, raw[C * NPL + loff[k]], v);
                        if (owned_x && (owned_mask & (1u << k)))
                            dnew[goff[k] + gx] = v;
                    }
                    const float hi = (float)v;
                    sh[loff[k]]    = hi;
                    sl[loff[k]]    = (float)(v - (double)hi);
                }
            mbar_arrive(bar(BAR_STAGED + m % R));
        };
        for (int m = 0; m < RAWD - 1; ++m)
            fetch(m);
        stage(0);
        fetch(RAWD - 1);
        for (int j = 0; j < J; ++j) {
            const int m = j + 1;
            if (m >= R)
                mbar_wait(bar(BAR_SFREE + m % R), (uint32_t)(((m - R) / R) & 1), abort_flag, wlim);
            stage(m);
            fetch(m + RAWD - 1);
            named_bar(1, NGRP);
            // element row: differences to the first node as double-float, then the slices
            const float *H0 = SH + (j % R) * C * NPL, *H1 = SH + ((j + 1) % R) * C * NPL;
            const float *L0 = SL + (j % R) * C * NPL, *L1 = SL + ((j + 1) % R) * C * NPL;
            float u0h[C], u0l[C], dh[NCOL], dl[NCOL];
#pragma unroll
            for (int c = 0; c < C; ++c) {
                u0h[c] = H0[c * NPL + ey * PZ + ez];
                u0l[c] = L0[c * NPL + ey * PZ + ez];
            }
            uint32_t emax = 0;
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const int qa = q & 1, qb = (q >> 1) & 1, qc = (q >> 2) & 1;
                const float *Hq = qa ? H1 : H0, *Lq = qa ? L1 : L0;
#pragma unroll
                for (int c = 0; c < C; ++c) {
                    const int o = c * NPL + (ey + qb) * PZ + ez + qc;
                    float     t, e;
                    two_sum(Hq[o], -u0h[c], t, e);
                    const float lo = e + (Lq[o] - u0l[c]);
                    two_sum(t, lo, dh[q * C + c], dl[q * C + c]); // |dl| <= ulp(dh) / 2
                    emax = max(emax, __float_as_uint(dh[q * C + c]) & 0x7F800000u);
                }
            }
            // scale = 2^(10 - e): |dh scale| < 2^10; inverse 2^(e - 10) (biased exponents)
            const uint32_t eb    = emax >> 23;
            const bool     tiny  = eb < 10;
            const float    scale = tiny ? 1.f : __uint_as_float((263u - eb) << 23);
            const float    inv   = tiny ? 1.f : __uint_as_float((eb - 9u) << 23);
            if (j >= 1) // the MMAs of plane j-1 have read A (and the consumers its 1/scale)
                mbar_wait(bar(BAR_DFULL), (uint32_t)((j - 1) & 1), abort_flag, wlim);
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            Inv[(j & 1) * NEL + ey * 32 + ez] = inv;
#pragma unroll
            for (int k0 = 0; k0 < NCOL; k0 += 4) { // one 16-byte core-matrix row per slice
                float4 q0, q1, q2, q3;
                float *f0 = &q0.x, *f1 = &q1.x, *f2 = &q2.x, *f3 = &q3.x;
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const float t  = dh[k0 + i] * scale;
                    const float a0 = rintf(t);
                    const float t1 = (t - a0) * 2048.f;
                    const float a1 = rintf(t1);
                    const float t2 = fmaf(dl[k0 + i] * scale, 4194304.f, (t1 - a1) * 2048.f);
                    const float a2 = rintf(t2);
                    f0[i]          = a0;
                    f1[i]          = a1;
                    f2[i]          = a2;
                    f3[i]          = rintf((t2 - a2) * 2048.f);
                }
                float *dst = arow + (k0 / 4) * 32; // + 128 bytes per K-adjacent core matrix
                *reinterpret_cast<float4 *>(dst)                              = q0;
                *reinterpret_cast<float4 *>(dst + Cfg::A_BYTES / 4)           = q1;
                *reinterpret_cast<float4 *>(dst + 2 * (Cfg::A_BYTES / 4))     = q2;
                *reinterpret_cast<float4 *>(dst + 3 * (Cfg::A_BYTES / 4))     = q3;
            }
            // the MMAs read A through the async proxy
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            mbar_arrive(bar(BAR_INV + (j & 1)));
            mbar_arrive(bar(BAR_AFULL));
        }
    } else if (warp < 8) {
        // ================================================================ consumers
        const int       ey = warp - 4, ez = lane;
        const long long el_yz = (long long)pmod(y0 - 1 + ey, ny) * nz + pmod(z0 - 1 + ez, nz);
        double         *yout  = reinterpret_cast<double *>(a.y);
        const uint32_t  lane_base = tmem + ((uint32_t)(ey * 32) << 16);
        const bool      out_ok = ey >= 1 && ez >= 1 && y0 - 1 + ey < ny && z0 - 1 + ez < nz;
        const int       onode  = ey * PZ + ez;
        const long long oyz    = out_ok ? (long long)(y0 - 1 + ey) * nz + (z0 - 1 + ez) : 0;
        float ch_[4 * C], cl_[4 * C]; // far-x rows of the previous plane (hi, lo)
#pragma unroll
        for (int i = 0; i < 4 * C; ++i) {
            ch_[i] = 0.f;
            cl_[i] = 0.f;
        }
        float doth = 0.f, dotl = 0.f; // <d, K d> of this thread's nodes (double-float)
        int   ph_next = a.ms[(long long)wrapi(xs - 1, nx) * plane + el_yz];
        for (int j = 0; j < J; ++j) {
            const int X = xs - 1 + j, b = j & 1;
            const int ph = ph_next;
            if (j + 1 < J)
                ph_next = a.ms[(long long)wrapi(X + 1, nx) * plane + el_yz];
            float cfh[NB], cfl[NB];
#pragma unroll
            for (int bb = 0; bb < NB; ++bb) {
                cfh[bb] = coef[(ph * NB + bb) * 2];
                cfl[bb] = coef[(ph * NB + bb) * 2 + 1];
            }
            mbar_wait(bar(BAR_DFULL), (uint32_t)(j & 1), abort_flag, wlim);
            __syncwarp();
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            // one barrier per scale buffer: the producers can complete plane j+1's
            // arrival before this wait, but not plane j+2's (that needs this
            // plane's DFREE), so the parity of a buffer's barrier never aliases
            mbar_wait(bar(BAR_INV + b), (uint32_t)((j >> 1) & 1), abort_flag, wlim);
            const float inv = Inv[b * NEL + ey * 32 + ez];
            float       oh[NCOL], ol[NCOL]; // K_ph u_e (+ f_ph) in double-float
#pragma unroll
            for (int c0 = 0; c0 < NW; c0 += 4) {
                float v0[4], v1[4], v2[4], v3[4];
                tmem_ld4(lane_base + (uint32_t)(c0), v0);
                tmem_ld4(lane_base + (uint32_t)(NW + c0), v1);
                tmem_ld4(lane_base + (uint32_t)(2 * NW + c0), v2);
                tmem_ld4(lane_base + (uint32_t)(3 * NW + c0), v3);
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                for (int jj = 0; jj < 4; jj += 2) { // two columns per packed FP32x2 instruction
                    const int col = c0 + jj, bb = col / NCOL, r = col % NCOL; // NCOL % 4 == 0
                    if (col < Cfg::NROW) {
                        // the exact integer sums back to one double-float value, unscaled
                        float2 h, l;
                        two_sum2(make_float2(v0[jj], v0[jj + 1]),
                                 __fmul2_rn(make_float2(v1[jj], v1[jj + 1]), make_float2(4.8828125e-4f, 4.8828125e-4f)),
                                 h, l); // 2^-11 (exact)
                        l = __ffma2_rn(make_float2(v2[jj], v2[jj + 1]), make_float2(2.384185791015625e-7f, 2.384185791015625e-7f),
                                       __ffma2_rn(make_float2(v3[jj], v3[jj + 1]),
                                                  make_float2(1.1641532182693481e-10f, 1.1641532182693481e-10f), l)); // 2^-22, 2^-33
                        const float2 inv2 = make_float2(inv, inv);
                        h                 = __fmul2_rn(h, inv2);
                        l                 = __fmul2_rn(l, inv2);
                        // times the phase coefficient (double-float product)
                        const int    b2  = bb < NB ? bb : 0;
                        const float2 ch2 = make_float2(cfh[b2], cfh[b2]), cl2 = make_float2(cfl[b2], cfl[b2]);
                        const float2 p   = __fmul2_rn(ch2, h);
                        const float2 pe  = __ffma2_rn(ch2, h, make_float2(-p.x, -p.y));
                        const float2 pl  = __ffma2_rn(ch2, l, __ffma2_rn(cl2, h, pe));
                        if (bb == 0) {
                            oh[r]     = p.x;
                            oh[r + 1] = p.y;
                            ol[r]     = pl.x;
                            ol[r + 1] = pl.y;
                        } else {
                            float2 sh = make_float2(oh[r], oh[r + 1]), sl = make_float2(ol[r], ol[r + 1]);
                            df_add2(sh, sl, p, pl);
                            oh[r]     = sh.x;
                            oh[r + 1] = sh.y;
                            ol[r]     = sl.x;
                            ol[r + 1] = sl.y;
                        }
                    }
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            mbar_arrive(bar(BAR_DFREE));
            if (force)
#pragma unroll
                for (int r = 0; r < NCOL; r += 2) {
                    float2 sh = make_float2(oh[r], oh[r + 1]), sl = make_float2(ol[r], ol[r + 1]);
                    df_add2(sh, sl, make_float2(fsm[ph * NCOL + r], fsm[ph * NCOL + r + 1]),
                            make_float2(fsm[kMaxPhX * NCOL + ph * NCOL + r], fsm[kMaxPhX * NCOL + ph * NCOL + r + 1]));
                    oh[r]     = sh.x;
                    oh[r + 1] = sh.y;
                    ol[r]     = sl.x;
                    ol[r + 1] = sl.y;
                }
            // x: near-x rows plus the carried far-x rows
            float Ph[4 * C], Pl[4 * C];
#pragma unroll
            for (int g = 0; g < 4; ++g)
#pragma unroll
                for (int c = 0; c < C; ++c) {
                    float h = oh[2 * g * C + c], l = ol[2 * g * C + c];
                    df_add(h, l, ch_[g * C + c], cl_[g * C + c]);
                    Ph[g * C + c]  = h;
                    Pl[g * C + c]  = l;
                    ch_[g * C + c] = oh[(2 * g + 1) * C + c];
                    cl_[g * C + c] = ol[(2 * g + 1) * C + c];
                }
            // z: lane ez-1's far-z rows
            float Zh[2 * C], Zl[2 * C];
#pragma unroll
            for (int qb = 0; qb < 2; ++qb)
#pragma unroll
                for (int c = 0; c < C; ++c) {
                    float h = Ph[qb * C + c], l = Pl[qb * C + c];
                    df_add(h, l, __shfl_up_sync(0xffffffffu, Ph[(qb + 2) * C + c], 1),
                           __shfl_up_sync(0xffffffffu, Pl[(qb + 2) * C + c], 1));
                    Zh[qb * C + c] = h;
                    Zl[qb * C + c] = l;
                }
            // y: far-y partial through the exchange to warp ey+1
            float *xw = Xch + (b * EYN + ey) * 2 * C * 32 + ez;
#pragma unroll
            for (int c = 0; c < C; ++c) {
                xw[c * 32]           = Zh[C + c];
                xw[(C + c) * 32]     = Zl[C + c];
            }
            named_bar(2, NGRP);
            if (X >= xs) {
                mbar_wait(bar(BAR_STAGED + j % R), (uint32_t)((j / R) & 1), abort_flag, wlim);
                if (out_ok) {
                    const long long gi = (long long)wrapi(X, nx) * plane + oyz;
                    const float    *xr = Xch + (b * EYN + ey - 1) * 2 * C * 32 + ez;
                    const float    *dh = SH + (j % R) * C * NPL + onode;
                    const float    *dl = SL + (j % R) * C * NPL + onode;
#pragma unroll
                    for (int c = 0; c < C; ++c) {
                        float h = Zh[c], l = Zl[c];
                        df_add(h, l, xr[c * 32], xr[(C + c) * 32]);
                        yout[c * N + gi] = (double)h + (double)l;
                        if (a.reduce) { // <d, y> in double-float
                            const float xh = dh[c * NPL], xl = dl[c * NPL];
                            const float p  = xh * h;
                            const float pe = fmaf(xh, h, -p);
                            df_add(doth, dotl, p, fmaf(xh, l, fmaf(xl, h, pe)));
                        }
                    }
                }
            }
            mbar_arrive(bar(BAR_SFREE + j % R));
        }
        dot = (double)doth + (double)dotl;
    } else if (lane == 0) {
        // ================================================================ MMA issuer
        const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(NW >> 3) << 17) | (8u << 24);
        const uint32_t wbase = smem_u32(smem + Cfg::OFF_W);
        const uint32_t abase = smem_u32(smem + Cfg::OFF_A);
        for (int j = 0; j < J; ++j) {
            mbar_wait(bar(BAR_AFULL), (uint32_t)(j & 1), abort_flag, wlim);
            if (j >= 1)
                mbar_wait(bar(BAR_DFREE), (uint32_t)((j - 1) & 1), abort_flag, wlim);
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            if (!*abort_flag) {
#pragma unroll
                for (int sl = 0; sl < NSL; ++sl)
#pragma unroll
                    for (int s = 0; s < Cfg::KSTEPS; ++s)
                        umma_tf32_ss(tmem + sl * NW, umma_desc<Cfg::SBO, Cfg::LBO>(abase + sl * Cfg::A_BYTES + s * 256),
                                     umma_desc<Cfg::SBO, Cfg::LBO>(wbase + s * 256), idesc, s > 0 ? 1u : 0u);
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                 bar(BAR_DFULL))
                             : "memory");
            } else {
                mbar_arrive(bar(BAR_DFULL));
            }
        }
        if (*abort_flag) {
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             bar(BAR_DRAIN))
                         : "memory");
            for (unsigned it = 0; it < kDrainLimit && !mbar_try(bar(BAR_DRAIN), 0u); ++it) {
            }
        }
    }

    __syncthreads();
    if (*abort_flag && tid == 0)
        a.scal->converged = -3;

    if (a.reduce) {
        double    vv[1]  = {dot};
        const int ops[1] = {RED_SUM};
        block_reduce<1>(vv, ops, red_smem);
        const int nb = gridDim.x * gridDim.y * gridDim.z;
        if (grid_partial_commit<1>(vv, a.red.partials, a.red.counter + a.red_site, nb)) {
            grid_final<1>(vv, ops, a.red.partials, nb, red_smem);
            if (threadIdx.x == 0) {
                a.scal->dAd   = vv[0];
                a.scal->alpha = a.scal->delta / vv[0];
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "n"(TCOLS) : "memory");
}

} // namespace

bool stencil_tcx_supported(const Grid3 &g, int C, int nb, int nph)
{
    return (C == 3 || C == 1) && nb >= 1 && nb <= 2 && nph >= 1 && nph <= kMaxPhX && g.nx >= 2 && g.ny >= 2 &&
           g.nz >= 2;
}

cudaError_t launch_stencil_tcx(const StencilArgs &a, const float *W, const float *coef_df, const float *f_df, int nb,
                               cudaStream_t st)
{
    dim3 grid((a.g.nx + XL - 1) / XL, (a.g.ny + BY - 1) / BY, (a.g.nz + BZ - 1) / BZ);
#define FANSGPU_TCX(C_, B_)                                                                                      \
    do {                                                                                                       \
        cudaError_t e = allow_max_dyn_smem_carveout(k_stencil_tcx<C_, B_>);                                             \
        if (e != cudaSuccess)                                                                                  \
            return e;                                                                                          \
        k_stencil_tcx<C_, B_><<<grid, TPB, SMEM_REQ, st>>>(a, W, coef_df, f_df);                                \
    } while (0)
    if (a.C == 3 && nb == 2)
        FANSGPU_TCX(3, 2);
    else if (a.C == 1 && nb == 1)
        FANSGPU_TCX(1, 1);
    else
        return cudaErrorInvalidValue;
#undef FANSGPU_TCX
    return cudaGetLastError();
}

} // namespace fansgpu
