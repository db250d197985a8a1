// k_stencil_tcb.cu -- the FP32 CG operator (d = s + beta d_old, K d, <d, K d>)
// for several right-hand sides on the 5th-generation tensor cores of sm_103a,
// with the element stiffness written in an exact basis.
//
// Every isotropic law of the linear solve has an element stiffness that is a
// combination of fixed basis matrices (solverCG.h:97-103 with
// LinearElastic.h:32-40 / LinearThermal.h:21-31): K_ph = lambda_ph K_lambda +
// mu_ph K_mu for isotropic elasticity, K_ph = kappa_ph K_kappa for isotropic
// conduction.  For the trilinear hexahedron on voxels of simple aspect ratios
// each basis matrix is a small integer multiple of one quantum q_b, so
// W_b = K_b / q_b is exact in tf32 and needs no hi/lo split; only the element
// rows U (8C displacements relative to the element's first node, solver.h:252)
// are split, U = hi + lo (hi: tf32 truncation, lo: the exact FP32 remainder,
// read by the MMA at tf32).  The GEMM is then
//     D[e][b*8C + i] = sum_k (hi + lo)[e][k] W_b[i][k]      (2 products)
// as tcgen05.mma kind::tf32 with M = 128 elements, N = 8C x NB, K = 8C, and
// the consumers form K_ph u_e = sum_b (c_ph,b q_b) D_b with the phase's
// coefficients -- any number of phases, no per-phase columns.
//
// Right-hand sides: the fields of RHS k sit at offset k * rhs_stride; a CTA
// marches its node column through the x planes of each active RHS in turn, so
// one launch covers all of them with one pipeline fill, one W load and one
// tensor-memory allocation per CTA.  <d_k, K d_k> is reduced per RHS and
// alpha_k = delta_k / <d_k, K d_k> is written to scal[k].
//
// Tiling, roles and hand-over follow the single-RHS tensor-core operator
// (k_stencil_tc.cu): a CTA owns a 3 (y) x 31 (z) node column, one element plane
// of which is one M-tile; producers stage node planes (16-byte cp.async chunks of
// z-aligned node rows, three planes ahead; d = s + beta d_old four nodes at a
// time with packed FP32x2 arithmetic) and build A in tensor memory, one thread
// issues the MMAs, consumers
// read D and sum element rows into nodes without atomics (register carry in x,
// a warp shuffle in z, an exchange buffer in y).  Every mbarrier wait is bounded;
// an expired wait sets an abort flag that releases the others, the issuer waits
// (bounded) for its MMAs in flight, tensor memory is freed and the status -3 is
// reported in scal[k].converged.
#include "kernels.cuh"

#include <cmath>
#include <cstdint>
#include <cstring>

namespace fansgpu {

namespace {

constexpr int BY = 3, BZ = 31;
constexpr int PY = BY + 2; // node rows of a column plane (halo included)
constexpr int EYN = BY + 1, EZN = BZ + 1;
constexpr int NEL = EYN * EZN; // 128 elements = one M-tile
constexpr int NGRP = 128;
constexpr int TPB  = 2 * NGRP + 32;
constexpr int XL   = 64;
constexpr int R    = 4; // node-plane slots
constexpr int RAWD = 4; // raw (s, d_old) planes in flight
// A node plane of the column is held as PY rows of ZR floats: the nodes from the 16-byte
// aligned z = za on (at most ZMAIN of them), then the periodic neighbours z = nz-4..nz-1
// (columns ZMAIN..ZMAIN+3) and z = 0..3 (ZMAIN+4..ZMAIN+7); rows move as 16-byte chunks.
constexpr int ZMAIN = 40, ZR = 48, CPRMAX = ZMAIN / 4 + 2;
constexpr int TCOLS = 128, COL_LO = 32, COL_A = 0, COL_D = 64;
constexpr int SMEM_REQ = 64 * 1024; // three CTAs per SM
constexpr unsigned kWaitLimit  = 1u << 22;
constexpr unsigned kDrainLimit = 1u << 22;
constexpr int kMaxPh = 256;
enum {
    BAR_AFULL  = 0,
    BAR_DFULL  = 1,
    BAR_DFREE  = 2,
    BAR_STAGED = 3,
    BAR_SFREE  = 3 + R,
    BAR_DRAIN  = 3 + 2 * R,
    NBAR       = 4 + 2 * R
};
static_assert(NEL == 128 && EYN == 4 && EZN == 32, "one M-tile per element plane, one warp per element row");

template <int C, int NB>
struct TbCfg {
    static constexpr int NCOL    = 8 * C;
    static constexpr int KC      = NCOL / 4;
    static constexpr int SBO     = KC * 128;
    static constexpr int LBO     = 128;
    static constexpr int NROW    = NB * NCOL;
    static constexpr int NW      = (NROW + 15) / 16 * 16;
    static constexpr int KSTEPS  = NCOL / 8;
    static constexpr int W_BYTES = NW * NCOL * 4;
    static constexpr int ROWF    = C * PY * ZR;                        // floats of one node plane
    static constexpr int NCH     = (C * PY * CPRMAX + NGRP - 1) / NGRP; // 16-byte chunks per producer
    static constexpr int al(int b) { return (b + 127) / 128 * 128; }
    static constexpr int OFF_W    = 0;
    static constexpr int OFF_COEF = al(OFF_W + W_BYTES);                 // [kMaxPh][NB] float
    static constexpr int OFF_D    = al(OFF_COEF + kMaxPh * NB * 4);      // [R][C][PY][ZR]
    static constexpr int OFF_RAW  = al(OFF_D + R * ROWF * 4);            // [RAWD][s, d_old][C][PY][ZR]
    static constexpr int OFF_X    = al(OFF_RAW + RAWD * 2 * ROWF * 4);   // [2][EYN][C][32]
    static constexpr int OFF_BAR  = al(OFF_X + 2 * EYN * C * 32 * 4);     // NBAR mbarriers, tmem slot, abort flag
    static constexpr int OFF_ACT  = OFF_BAR + NBAR * 8 + 8;              // active RHS list + count
    static constexpr int OFF_BETA = OFF_ACT + (kMaxRhs + 1) * 4;         // beta of each active RHS (float)
    static constexpr int OFF_SEG  = al(OFF_BETA + kMaxRhs * 4);           // [4 warps][kMaxRhs] double
    static constexpr int OFF_RED  = al(OFF_SEG + 4 * kMaxRhs * 8);        // [32][kMaxRhs] double
    static constexpr int SMEM     = OFF_RED + 32 * kMaxRhs * 8;
    static_assert(NW <= TCOLS - COL_D && NCOL <= COL_LO && COL_LO + NCOL <= COL_D, "tensor-memory map");
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
    // shared-memory matrix descriptor: K-major, no swizzle (core matrices of 8 rows x 16 bytes)
    uint64_t d = (uint64_t)((addr & 0x3FFFF) >> 4);
    d |= (uint64_t)(LBO_ >> 4) << 16;
    d |= (uint64_t)(SBO_ >> 4) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

__device__ __forceinline__ float to_tf32(float x) { return __uint_as_float(__float_as_uint(x) & 0xFFFFE000u); }

__device__ __forceinline__ int wrapi(int x, int n) { return x < 0 ? x + n : (x >= n ? x - n : x); }

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v)
{
    uint32_t r[16];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                 : "r"(taddr));
#pragma unroll
    for (int j = 0; j < 16; ++j)
        v[j] = __uint_as_float(r[j]);
}

__device__ __forceinline__ void tmem_st8(uint32_t taddr, const float *v)
{
    asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"r"(taddr),
                 "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])),
                 "r"(__float_as_uint(v[3])), "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])),
                 "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7]))
                 : "memory");
}

__device__ __forceinline__ void umma_tf32_ts(uint32_t dtmem, uint32_t atmem, uint64_t bd, uint32_t idesc, uint32_t acc)
{
    asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                 " tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n}\n" ::"r"(dtmem),
                 "r"(atmem), "l"(bd), "r"(idesc), "r"(acc));
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

// Bounded wait (`limit` polls) for the phase with the given parity, released by the abort flag.
__device__ __forceinline__ void mbar_wait(uint32_t bar, uint32_t parity, volatile int *abort_flag, unsigned limit)
{
    for (unsigned it = 0; it < limit; ++it)
        if (mbar_try(bar, parity) || *abort_flag)
            return;
    *abort_flag = 1;
}

// The same with a pause of `ns` nanoseconds between polls: for waits off the critical path,
// so that the waiting warps leave their issue slots to the warps doing the work.
__device__ __forceinline__ void mbar_wait_sleep(uint32_t bar, uint32_t parity, volatile int *abort_flag, unsigned limit,
                                                unsigned ns)
{
    for (unsigned it = 0; it < limit; ++it) {
        if (mbar_try(bar, parity) || *abort_flag)
            return;
        __nanosleep(ns);
    }
    *abort_flag = 1;
}

__device__ __forceinline__ void named_bar(int id, int nthreads)
{
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

template <int C, int NB>
__global__ void __launch_bounds__(TPB, 3)
    k_stencil_tcb(StencilArgs a, const float *__restrict__ Wg, const float *__restrict__ coefg)
{
    using Cfg = TbCfg<C, NB>;
    constexpr int NCOL = Cfg::NCOL, NCH = Cfg::NCH, ROWF = Cfg::ROWF;
    extern __shared__ __align__(16) unsigned char smem[];
    float        *Dp         = reinterpret_cast<float *>(smem + Cfg::OFF_D);
    float        *Xch        = reinterpret_cast<float *>(smem + Cfg::OFF_X);
    float        *Raw        = reinterpret_cast<float *>(smem + Cfg::OFF_RAW);
    const float  *coef       = reinterpret_cast<const float *>(smem + Cfg::OFF_COEF);
    const uint32_t bar0      = smem_u32(smem + Cfg::OFF_BAR);
    uint32_t     *tmem_slot  = reinterpret_cast<uint32_t *>(smem + Cfg::OFF_BAR + NBAR * 8);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(smem + Cfg::OFF_BAR + NBAR * 8 + 4);
    int          *s_act      = reinterpret_cast<int *>(smem + Cfg::OFF_ACT); // [kMaxRhs] RHS ids, then the count
    float        *s_beta     = reinterpret_cast<float *>(smem + Cfg::OFF_BETA); // beta of segment kk
    double       *seg_red    = reinterpret_cast<double *>(smem + Cfg::OFF_SEG);
    double       *red_smem   = reinterpret_cast<double *>(smem + Cfg::OFF_RED);
    auto bar = [&](int i) { return bar0 + 8u * (uint32_t)i; };
    const unsigned wlim = a.wait_limit > 0 ? (unsigned)a.wait_limit : kWaitLimit;

    const int nx = a.g.nx, ny = a.g.ny, nz = a.g.nz;
    const long long N = (long long)nx * ny * nz;
    const int tid = threadIdx.x, warp = tid / 32, lane = tid % 32;
    const int y0 = blockIdx.y * BY, z0 = blockIdx.z * BZ;
    const int xs = blockIdx.x * XL, xe = min(xs + XL, nx);
    const int J  = xe - xs + 1; // element planes xs-1 .. xe-1 per RHS
    const long long plane = (long long)ny * nz;
    const long long rstr  = a.rhs_stride;

    // ---- setup: W, phase coefficients, active RHS, barriers, tensor memory
    for (int i = tid; i < Cfg::W_BYTES / 16; i += TPB)
        reinterpret_cast<float4 *>(smem + Cfg::OFF_W)[i] = reinterpret_cast<const float4 *>(Wg)[i];
    for (int i = tid; i < a.nph * NB; i += TPB)
        reinterpret_cast<float *>(smem + Cfg::OFF_COEF)[i] = coefg[i];
    for (int i = tid; i < 4 * kMaxRhs; i += TPB)
        seg_red[i] = 0.0;
    if (tid == 0) {
        int n = 0;
        for (int k = 0; k < a.nrhs; ++k)
            if (!a.active || a.active[k]) {
                s_beta[n]  = (float)a.scal[k].beta;
                s_act[n++] = k;
            }
        s_act[kMaxRhs] = n;
        mbar_init(bar(BAR_AFULL), NGRP);
        mbar_init(bar(BAR_DFULL), 1);
        mbar_init(bar(BAR_DFREE), NGRP);
        for (int s = 0; s < R; ++s) {
            mbar_init(bar(BAR_STAGED + s), NGRP);
            mbar_init(bar(BAR_SFREE + s), NGRP);
        }
        mbar_init(bar(BAR_DRAIN), 1);
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
    const int      nact = s_act[kMaxRhs];
    const int      nU   = nact * J;       // element units (RHS, element plane)
    const int      nG   = nact * (J + 1); // node planes (RHS, node plane)

    if (warp < 4) {
        // ================================================================ producers
        const int    ey = warp, ez = lane;
        const float *sin  = reinterpret_cast<const float *>(a.x);
        const float *dold = reinterpret_cast<const float *>(a.d_old);
        float       *dnew = reinterpret_cast<float *>(a.d_new);
        const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
        // the column's node rows in z: from za (16-byte aligned) on, zlen nodes, plus the wrap chunks
        const int  za   = z0 == 0 ? 0 : ((z0 - 1) & ~3);
        const int  zlen = min(ZMAIN, nz - za);
        const bool wlo = z0 == 0, whi = z0 + BZ >= nz;
        const int  cpr  = zlen / 4 + (wlo ? 1 : 0) + (whi ? 1 : 0); // chunks per row
        // node z of the column -> its row column (rows past nz only feed elements outside the grid)
        auto zcol = [&](int z) { return z < 0 ? ZMAIN + 3 : (z >= nz ? ZMAIN + 4 + min(z - nz, 3) : z - za); };
        // this thread's 16-byte chunks of a node plane (row (c, hy), 4 nodes): global offset of
        // the row chunk, offset in a plane's rows, and which of its 4 nodes this CTA owns
        long long goff[NCH];
        int       soff[NCH];
        unsigned  omask[NCH];
        unsigned  valid_mask = 0;
#pragma unroll
        for (int k = 0; k < NCH; ++k) {
            const int q = tid + k * NGRP;
            goff[k]  = 0;
            soff[k]  = 0;
            omask[k] = 0;
            if (q < C * PY * cpr) {
                const int row = q / cpr, h = q % cpr, c = row / PY, hy = row % PY;
                const int y   = y0 - 1 + hy;
                int zsrc, col;
                if (h < zlen / 4) {
                    zsrc = za + 4 * h;
                    col  = 4 * h;
                } else if (wlo && h == zlen / 4) {
                    zsrc = nz - 4;
                    col  = ZMAIN;
                } else {
                    zsrc = 0;
                    col  = ZMAIN + 4;
                }
                goff[k] = c * N + (long long)pmod(y, ny) * nz + zsrc;
                soff[k] = (c * PY + hy) * ZR + col;
                valid_mask |= 1u << k;
                if (col < ZMAIN && hy >= 1 && hy <= BY && y < ny)
                    for (int i = 0; i < 4; ++i) {
                        const int z = zsrc + i;
                        if (z >= z0 && z < z0 + BZ && z < nz)
                            omask[k] |= 1u << i;
                    }
            }
        }
        // node plane g = (segment kk, plane m) with g = kk (J+1) + m: s and d_old of its RHS
        // copied into raw slot g % RAWD, RAWD-1 planes ahead of their use.  fetch and stage
        // walk the node planes in order, each with its own (kk, m) counter.  A thread stages
        // exactly the chunks it fetched, so its own cp.async wait orders them.
        int fk = 0, fm = 0, fg = 0; // next node plane to fetch
        auto fetch_next = [&]() {
            if (fg < nG) {
                const long long off = (long long)s_act[fk] * rstr + (long long)wrapi(xs - 1 + fm, nx) * plane;
                const uint32_t  raw = smem_u32(Raw + (fg % RAWD) * 2 * ROWF);
#pragma unroll
                for (int k = 0; k < NCH; ++k)
                    if (valid_mask & (1u << k)) {
                        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(raw + 4u * (uint32_t)soff[k]),
                                     "l"(sin + off + goff[k])
                                     : "memory");
                        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(
                                         raw + 4u * (uint32_t)(ROWF + soff[k])),
                                     "l"(dold + off + goff[k])
                                     : "memory");
                    }
            }
            asm volatile("cp.async.commit_group;" ::: "memory");
            ++fg;
            if (++fm == J + 1) {
                fm = 0;
                ++fk;
            }
        };
        // d = s + beta_k d_old of the next node plane into slot g % R (+ d_new for owned nodes)
        int sk = 0, sm = 0, sg = 0; // next node plane to stage
        auto stage_next = [&]() {
            asm volatile("cp.async.wait_group %0;" ::"n"(RAWD - 2) : "memory");
            const int       rk      = s_act[sk];
            const int       X       = xs - 1 + sm;
            const bool      owned_x = X >= xs && X < xe;
            const long long off     = (long long)rk * rstr + (long long)wrapi(X, nx) * plane;
            const float     beta    = s_beta[sk];
            const float2    b2      = make_float2(beta, beta);
            const float    *raw     = Raw + (sg % RAWD) * 2 * ROWF;
            float          *slot    = Dp + (sg % R) * ROWF;
#pragma unroll
            for (int k = 0; k < NCH; ++k)
                if (valid_mask & (1u << k)) {
                    const float4 sv = *reinterpret_cast<const float4 *>(raw + soff[k]);
                    const float4 dv = *reinterpret_cast<const float4 *>(raw + ROWF + soff[k]);
                    const float2 v0 = __ffma2_rn(b2, make_float2(dv.x, dv.y), make_float2(sv.x, sv.y));
                    const float2 v1 = __ffma2_rn(b2, make_float2(dv.z, dv.w), make_float2(sv.z, sv.w));
                    const float4 v  = make_float4(v0.x, v0.y, v1.x, v1.y);
                    *reinterpret_cast<float4 *>(slot + soff[k]) = v;
                    if (owned_x && omask[k]) {
                        float *dst = dnew + off + goff[k];
                        if (omask[k] == 0xFu) {
                            *reinterpret_cast<float4 *>(dst) = v;
                        } else {
                            if (omask[k] & 1u) dst[0] = v.x;
                            if (omask[k] & 2u) dst[1] = v.y;
                            if (omask[k] & 4u) dst[2] = v.z;
                            if (omask[k] & 8u) dst[3] = v.w;
                        }
                    }
                }
            mbar_arrive(bar(BAR_STAGED + sg % R));
            ++sg;
            if (++sm == J + 1) {
                sm = 0;
                ++sk;
            }
        };
        for (int g = 0; g < RAWD - 1; ++g)
            fetch_next();
        if (nU > 0) {
            stage_next(); // node plane 0
            fetch_next();
        }
        // this element's nodes (ey + qb, ez + qc) in a plane's rows
        int noff[4];
#pragma unroll
        for (int qq = 0; qq < 4; ++qq)
            noff[qq] = (ey + (qq >> 1)) * ZR + zcol(z0 - 1 + ez + (qq & 1));
        int kk = 0, j = 0; // segment and element plane of unit U
        for (int U = 0; U < nU; ++U, j = (j + 1 == J) ? 0 : j + 1, kk += (j == 0)) {
            const int g0 = kk * (J + 1) + j; // near-x node plane of element plane j
            while (sg < g0 + 2) {             // at a segment start: its first two node planes
                if (sg >= R)                  // consumers are done with node plane sg - R
                    mbar_wait(bar(BAR_SFREE + sg % R), (uint32_t)(((sg - R) / R) & 1), abort_flag, wlim);
                stage_next();
                fetch_next();
            }
            named_bar(1, NGRP); // node planes g0 and g0+1 staged by all producers
            if (U >= 1)         // the MMAs of unit U-1 have read A
                mbar_wait(bar(BAR_DFULL), (uint32_t)((U - 1) & 1), abort_flag, wlim);
            __syncwarp();
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const float *P0 = Dp + (g0 % R) * ROWF, *P1 = Dp + ((g0 + 1) % R) * ROWF;
            float u0[C], w[NCOL];
#pragma unroll
            for (int c = 0; c < C; ++c)
                u0[c] = P0[c * PY * ZR + noff[0]];
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const int qa = q & 1, qb = (q >> 1) & 1, qc = (q >> 2) & 1;
                const float *P = qa ? P1 : P0;
#pragma unroll
                for (int c = 0; c < C; ++c)
                    w[q * C + c] = P[c * PY * ZR + noff[qb * 2 + qc]];
            }
            // differences to the first node, then hi (tf32 truncation) and lo = v - hi, two
            // values per packed FP32x2 instruction
            float h[NCOL], l[NCOL];
            const float2 m1 = make_float2(-1.f, -1.f);
#pragma unroll
            for (int k = 0; k < NCOL; k += 2) {
                const float2 v2 = __ffma2_rn(make_float2(u0[k % C], u0[(k + 1) % C]), m1, make_float2(w[k], w[k + 1]));
                h[k]            = to_tf32(v2.x);
                h[k + 1]        = to_tf32(v2.y);
                const float2 l2 = __ffma2_rn(make_float2(h[k], h[k + 1]), m1, v2);
                l[k]            = l2.x;
                l[k + 1]        = l2.y;
            }
#pragma unroll
            for (int k0 = 0; k0 < NCOL; k0 += 8) {
                tmem_st8(lane_base + (uint32_t)(COL_A + k0), h + k0);
                tmem_st8(lane_base + (uint32_t)(COL_A + COL_LO + k0), l + k0);
            }
            asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            mbar_arrive(bar(BAR_AFULL));
        }
    } else if (warp < 8) {
        // ================================================================ consumers
        const int       ey = warp - 4, ez = lane;
        const long long el_yz = (long long)pmod(y0 - 1 + ey, ny) * nz + pmod(z0 - 1 + ez, nz);
        float          *yout  = reinterpret_cast<float *>(a.y);
        const uint32_t  lane_base = tmem + ((uint32_t)(ey * 32) << 16);
        const bool      out_ok = ey >= 1 && ez >= 1 && y0 - 1 + ey < ny && z0 - 1 + ez < nz;
        // this thread's node (ey, ez) in a plane's rows (16-byte aligned z from za on)
        const int       za     = z0 == 0 ? 0 : ((z0 - 1) & ~3);
        const int       onode  = ey * ZR + (z0 - 1 + ez - za);
        const long long oyz    = out_ok ? (long long)(y0 - 1 + ey) * nz + (z0 - 1 + ez) : 0;
        float carry[4 * C];
#pragma unroll
        for (int i = 0; i < 4 * C; ++i)
            carry[i] = 0.f;
        float dot = 0.f; // <d_k, K d_k> of this thread's nodes in the current segment (FP64 from the warp sum on)
        int ph_next = nU > 0 ? a.ms[(long long)wrapi(xs - 1, nx) * plane + el_yz] : 0;
        int kk = 0, j = 0; // segment and element plane of unit U
        for (int U = 0; U < nU; ++U, j = (j + 1 == J) ? 0 : j + 1, kk += (j == 0)) {
            const int X = xs - 1 + j, b = U & 1;
            const int g0 = kk * (J + 1) + j;
            const int ph = ph_next;
            if (U + 1 < nU)
                ph_next = a.ms[(long long)wrapi(j + 1 == J ? xs - 1 : X + 1, nx) * plane + el_yz];
            float cf[NB];
#pragma unroll
            for (int bb = 0; bb < NB; ++bb)
                cf[bb] = coef[ph * NB + bb];
            if (a.wait_sleep_ns > 0)
                mbar_wait_sleep(bar(BAR_DFULL), (uint32_t)(U & 1), abort_flag, wlim, (unsigned)a.wait_sleep_ns);
            else
                mbar_wait(bar(BAR_DFULL), (uint32_t)(U & 1), abort_flag, wlim);
            __syncwarp();
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            float out[NCOL]; // K_ph u_e = sum_b cf_b D_b, two rows per packed FP32x2 instruction
            // the first two 16-column loads share one wait, the rest wait one at a time
            constexpr int NLD0 = Cfg::NW >= 32 ? 2 : 1;
            float         vv[16 * NLD0];
#pragma unroll
            for (int h = 0; h < NLD0; ++h)
                tmem_ld16(lane_base + (uint32_t)(COL_D + 16 * h), vv + 16 * h);
#pragma unroll
            for (int c0 = 0; c0 < Cfg::NW; c0 += 16) {
                float *vc = c0 < 16 * NLD0 ? vv + c0 : vv;
                if (c0 >= 16 * NLD0)
                    tmem_ld16(lane_base + (uint32_t)(COL_D + c0), vc);
                if (c0 == 0 || c0 >= 16 * NLD0)
                    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                for (int jj = 0; jj < 16; jj += 2) { // NCOL is even: a pair never straddles two blocks
                    const int col = c0 + jj, bb = col / NCOL, r = col % NCOL;
                    if (col < Cfg::NROW) {
                        const float  c1 = cf[bb < NB ? bb : 0];
                        const float2 v2 = make_float2(vc[jj], vc[jj + 1]);
                        const float2 o2 = bb == 0 ? __fmul2_rn(make_float2(c1, c1), v2)
                                                  : __ffma2_rn(make_float2(c1, c1), v2, make_float2(out[r], out[r + 1]));
                        out[r]     = o2.x;
                        out[r + 1] = o2.y;
                    }
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            mbar_arrive(bar(BAR_DFREE));
            float P[4 * C];
#pragma unroll
            for (int g = 0; g < 4; ++g) {
#pragma unroll
                for (int c = 0; c < C; ++c) {
                    P[g * C + c]     = out[2 * g * C + c] + carry[g * C + c];
                    carry[g * C + c] = out[(2 * g + 1) * C + c];
                }
            }
            float Z[2 * C];
#pragma unroll
            for (int qb = 0; qb < 2; ++qb)
#pragma unroll
                for (int c = 0; c < C; ++c)
                    Z[qb * C + c] = P[qb * C + c] + __shfl_up_sync(0xffffffffu, P[(qb + 2) * C + c], 1);
            float *xw = Xch + (b * EYN + ey) * C * 32 + ez;
#pragma unroll
            for (int c = 0; c < C; ++c)
                xw[c * 32] = Z[C + c];
            named_bar(2, NGRP);
            if (X >= xs) {
                mbar_wait(bar(BAR_STAGED + g0 % R), (uint32_t)((g0 / R) & 1), abort_flag, wlim); // node plane X
                if (out_ok) {
                    const long long gi = (long long)s_act[kk] * rstr + (long long)wrapi(X, nx) * plane + oyz;
                    const float    *xr = Xch + (b * EYN + ey - 1) * C * 32 + ez;
                    const float    *dp = Dp + (g0 % R) * ROWF + onode;
                    float           dl = 0.f;
#pragma unroll
                    for (int c = 0; c < C; ++c) {
                        const float vo = Z[c] + xr[c * 32];
                        yout[c * N + gi] = vo;
                        dl += dp[c * PY * ZR] * vo;
                    }
                    dot += dl;
                }
            }
            mbar_arrive(bar(BAR_SFREE + g0 % R));
            if (j == J - 1) {
                // end of the segment: release its last node plane (read only by the producers,
                // whose A build of this unit the MMAs have consumed) and fold <d, K d>
                mbar_arrive(bar(BAR_SFREE + (g0 + 1) % R));
                double dd = (double)dot;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1)
                    dd += __shfl_down_sync(0xffffffffu, dd, o);
                if (lane == 0)
                    seg_red[ey * kMaxRhs + s_act[kk]] = dd;
                dot = 0.f;
            }
        }
    } else if (lane == 0) {
        // ================================================================ MMA issuer
        const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(Cfg::NW >> 3) << 17) | (8u << 24);
        const uint32_t wbase = smem_u32(smem + Cfg::OFF_W);
        for (int U = 0; U < nU; ++U) {
            mbar_wait(bar(BAR_AFULL), (uint32_t)(U & 1), abort_flag, wlim);
            if (U >= 1)
                mbar_wait(bar(BAR_DFREE), (uint32_t)((U - 1) & 1), abort_flag, wlim);
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            if (!*abort_flag) {
                const uint32_t d = tmem + COL_D, ah = tmem + COL_A, al = tmem + COL_A + COL_LO;
#pragma unroll
                for (int s = 0; s < Cfg::KSTEPS; ++s) // lo * W first (the small terms)
                    umma_tf32_ts(d, al + 8 * s, umma_desc<Cfg::SBO, Cfg::LBO>(wbase + s * 256), idesc, s > 0 ? 1u : 0u);
#pragma unroll
                for (int s = 0; s < Cfg::KSTEPS; ++s)
                    umma_tf32_ts(d, ah + 8 * s, umma_desc<Cfg::SBO, Cfg::LBO>(wbase + s * 256), idesc, 1u);
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
        for (int kk = 0; kk < nact; ++kk)
            a.scal[s_act[kk]].converged = -3; // a tensor-core pipeline wait expired

    // <d_k, K d_k> over the grid, per RHS (solverCG.h:101), and alpha_k
    if (a.reduce) {
        double vv[kMaxRhs];
        int    ops[kMaxRhs];
#pragma unroll
        for (int k = 0; k < kMaxRhs; ++k) {
            vv[k]  = seg_red[k] + seg_red[kMaxRhs + k] + seg_red[2 * kMaxRhs + k] + seg_red[3 * kMaxRhs + k];
            ops[k] = RED_SUM;
        }
        const int nb = gridDim.x * gridDim.y * gridDim.z;
        if (grid_partial_commit<kMaxRhs>(vv, a.red.partials, a.red.counter + a.red_site, nb)) {
            grid_final<kMaxRhs>(vv, ops, a.red.partials, nb, red_smem);
            if (threadIdx.x == 0)
                for (int kk = 0; kk < nact; ++kk) {
                    const int k     = s_act[kk];
                    a.scal[k].dAd   = vv[k];
                    a.scal[k].alpha = a.scal[k].delta / vv[k];
                }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "n"(TCOLS) : "memory");
}

// Quantum q (> 0) with K = q * n, n integers of magnitude < 2048 (exact in tf32), or 0.
double exact_quantum(const double *K, int n)
{
    double mx = 0.0;
    for (int i = 0; i < n; ++i)
        mx = std::fmax(mx, std::fabs(K[i]));
    if (!(mx > 0.0))
        return 0.0;
    double mn = mx;
    for (int i = 0; i < n; ++i) {
        const double a = std::fabs(K[i]);
        if (a > 1e-12 * mx && a < mn)
            mn = a;
    }
    for (int den = 1; den <= 2048; ++den) {
        const double q  = mn / den;
        bool         ok = mx / q < 2047.5;
        for (int i = 0; i < n && ok; ++i) {
            const double t = K[i] / q;
            if (std::fabs(K[i]) <= 1e-12 * mx)
                continue;
            ok = std::fabs(t - std::nearbyint(t)) <= 1e-9 * (mx / q);
        }
        if (ok)
            return q;
    }
    return 0.0;
}

} // namespace

bool stencil_tcb_quanta(int C, const double *Kb, int nb, double *q_out)
{
    const int ncol = 8 * C;
    for (int b = 0; b < nb; ++b) {
        const double q = exact_quantum(Kb + (size_t)b * ncol * ncol, ncol * ncol);
        if (!(q > 0.0))
            return false;
        q_out[b] = q;
    }
    return true;
}

size_t stencil_tcb_weights(int C, int nb)
{
    const int ncol = 8 * C, nw = (nb * ncol + 15) / 16 * 16;
    return (size_t)nw * ncol;
}

// W[b*8C + i][k] = K_b[i][k] / q_b (integers, exact in tf32), rows padded to the MMA N, in the
// K-major no-swizzle core-matrix layout.
void stencil_tcb_pack_weights(int C, int nb, const double *Kb, const double *q, float *out)
{
    const int    ncol = 8 * C, kc = ncol / 4, nrow = nb * ncol, nw = (nrow + 15) / 16 * 16;
    const int    sbo  = kc * 128;
    const size_t tot  = (size_t)nw * ncol;
    for (size_t i = 0; i < tot; ++i)
        out[i] = 0.f;
    for (int n = 0; n < nrow; ++n)
        for (int k = 0; k < ncol; ++k) {
            const int    b   = n / ncol, i = n % ncol;
            const double t   = std::nearbyint(Kb[((size_t)b * ncol + i) * ncol + k] / q[b]);
            const size_t off = ((size_t)(n / 8) * sbo + (size_t)(k / 4) * 128 + (n % 8) * 16 + (k % 4) * 4) / 4;
            out[off]         = (float)t;
        }
}

bool stencil_tcb_supported(const Grid3 &g, int C, int nb, int nph)
{
    // node rows move as 16-byte chunks: nz a multiple of 4 (every grid of the register FFT passes)
    return (C == 3 || C == 1) && nb >= 1 && nb <= 2 && nph >= 1 && nph <= kMaxPh && g.nx >= 2 && g.ny >= 2 &&
           g.nz >= 4 && g.nz % 4 == 0;
}

cudaError_t launch_stencil_tcb(const StencilArgs &a, const float *W, const float *coef, int nb, cudaStream_t st)
{
    if (a.nrhs < 1 || a.nrhs > kMaxRhs || a.g.nz % 4 != 0 || a.rhs_stride % 4 != 0 || (uintptr_t)a.x % 16 != 0 ||
        (uintptr_t)a.d_old % 16 != 0 || (uintptr_t)a.d_new % 16 != 0)
        return cudaErrorInvalidValue; // 16-byte node-row chunks
    dim3 grid((a.g.nx + XL - 1) / XL, (a.g.ny + BY - 1) / BY, (a.g.nz + BZ - 1) / BZ);
#define FANSGPU_TCB(C_, B_)                                                                                      \
    do {                                                                                                       \
        cudaError_t e = allow_max_dyn_smem(k_stencil_tcb<C_, B_>);                                             \
        if (e != cudaSuccess)                                                                                  \
            return e;                                                                                          \
        k_stencil_tcb<C_, B_><<<grid, TPB, SMEM_REQ, st>>>(a, W, coef);                                         \
    } while (0)
    if (a.C == 3 && nb == 2)
        FANSGPU_TCB(3, 2);
    else if (a.C == 3 && nb == 1)
        FANSGPU_TCB(3, 1);
    else if (a.C == 1 && nb == 1)
        FANSGPU_TCB(1, 1);
    else
        return cudaErrorInvalidValue;
#undef FANSGPU_TCB
    return cudaGetLastError();
}

} // namespace fansgpu
