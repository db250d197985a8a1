// k_stencil_tc.cu -- the FP32 CG operator (d = s + beta d_old, K d, <d, K d>)
// on the 5th-generation tensor cores of sm_103a.
//
// The element matvec r_e = K_ph u_e of every voxel element (solverCG.h:97-103)
// is a GEMM over elements: D[e][ph*8C + i] = sum_k U[e][k] W[ph*8C + i][k] with
// U[e] = u_e - u_e,node0 (the 8C element displacements relative to the element's
// first node, solver.h:252) and W the per-phase element stiffnesses.  The GEMM
// runs as tcgen05.mma kind::tf32 (M = 128 elements, N = 8C x phases, K = 8C)
// with both operands split hi + lo (hi = the top 11 significant bits, lo = the
// exact FP32 remainder; 3xTF32: lo*hi + hi*lo + hi*hi), which keeps the product
// at FP32 accuracy.  A (the element rows) is written straight into tensor memory
// with tcgen05.st; W sits in shared memory; D accumulates in tensor memory.
//
// A CTA owns a 3 (y) x 31 (z) column of nodes, whose element plane is exactly
// one M-tile (4 x 32 = 128 elements), and marches along x over XL planes.  Its
// warps specialise, so that the work around consecutive MMAs overlaps:
//   producers (warps 0-3, element row ey = warp, column ez = lane): stage node
//     plane X+1 (d = s + beta d_old from s and d_old that cp.async brought into
//     shared memory three planes ahead; d_new for owned nodes) into a ring of R
//     shared slots, then -- once the MMAs of plane X-1 have read A -- build the
//     element rows of plane X, split hi/lo, into A in tensor memory;
//   issuer (warp 8, one thread): the 9 MMAs of plane X into D once A is full and
//     the consumers have read the previous D;
//   consumers (warps 4-7, same element mapping): read their element's phase
//     columns of D and sum them into nodes without atomics or colour copies --
//     x: the far-x rows are carried in registers to the next plane; z: one warp
//     shuffle adds lane ez-1's far-z rows; y: the far-y partial goes through a
//     small exchange buffer to warp ey+1 -- then write K d of node plane X and
//     accumulate <d, K d>.  Every node is a fixed-order sum (deterministic).
// The groups hand over through mbarriers (A full, D full, D free, node slot
// staged, node slot free); every wait is bounded and an expired wait sets an
// abort flag that releases all other waits, so the kernel always ends and
// reports the error status.  A and D are single-buffered (128 tensor-memory
// columns per CTA), so three CTAs share an SM and keep its tensor pipe fed: the
// SM's tensor pipe is shared, and more CTAs fill the gaps between one CTA's MMA
// bursts better than deeper buffering within a CTA.
#include "kernels.cuh"

#include <cstring>

namespace fansgpu {

namespace {

constexpr int BY = 3, BZ = 31;
constexpr int PY = BY + 2, PZ = BZ + 2;   // node plane incl. halo: y0-1..y0+3, z0-1..z0+31
constexpr int EYN = BY + 1, EZN = BZ + 1; // element plane: origins y0-1..y0+2, z0-1..z0+30
constexpr int NEL = EYN * EZN;            // 128 elements = one M-tile
constexpr int NGRP = 128;                 // threads per role group (one per element)
constexpr int TPB = 2 * NGRP + 32;        // producers, consumers, issuer warp
constexpr int NPL = PY * PZ;              // 165 nodes per plane incl. halo
constexpr int XL  = 64;                   // planes per CTA
constexpr int R   = 4;                    // node-plane slots
constexpr int RAWD = 4;                   // raw (s, d_old) planes in flight: fetched RAWD-1 planes ahead
constexpr int TCOLS = 128;                // tensor memory: A (hi at 0, lo at 32), D at 64
constexpr int COL_LO = 32, COL_A = 0, COL_D = 64;
// dynamic shared memory requested: with the 1 KB reserved per block, 3 CTAs fit in an SM's 228 KB
// and 4 do not (4 x 128 tensor-memory columns would fit, 4 x 288 threads' registers would not)
constexpr int SMEM_REQ = 64 * 1024;
// Bounded mbarrier waits: try_wait polls (each suspends the thread for a while) before a wait
// gives up; StencilArgs::wait_limit overrides it (a diagnostics control that lets a test make the
// waits expire).  Draining the tensor pipe after an abort has its own, fixed bound.
constexpr unsigned kWaitLimit  = 1u << 22;
constexpr unsigned kDrainLimit = 1u << 22;
enum {
    BAR_AFULL  = 0,
    BAR_DFULL  = 1,
    BAR_DFREE  = 2,
    BAR_STAGED = 3,
    BAR_SFREE  = 3 + R,
    BAR_DRAIN  = 3 + 2 * R, // the issuer's MMAs in flight after an abort
    NBAR       = 4 + 2 * R
};
static_assert(NEL == 128 && EYN == 4 && EZN == 32, "one M-tile per element plane, one warp per element row");

template <int C, int NPH>
struct TcCfg {
    static constexpr int NCOL    = 8 * C;                 // GEMM K
    static constexpr int KC      = NCOL / 4;              // 16-byte core-matrix columns along K
    static constexpr int SBO     = KC * 128;              // bytes between 8-row groups
    static constexpr int LBO     = 128;                   // bytes between K-adjacent core matrices
    static constexpr int NROW    = NPH * NCOL;            // stacked phase rows
    static constexpr int NW      = (NROW + 15) / 16 * 16; // MMA N
    static constexpr int KSTEPS  = NCOL / 8;              // K = 8 per tf32 MMA
    static constexpr int W_BYTES = NW * NCOL * 4;
    static constexpr int NPF     = (C * NPL + NGRP - 1) / NGRP; // prefetched node values per producer and field
    static constexpr int al(int b) { return (b + 127) / 128 * 128; }
    static constexpr int OFF_W   = 0;                                  // [hi, lo][W_BYTES]
    static constexpr int OFF_D   = al(OFF_W + 2 * W_BYTES);            // [R slots][C][NPL] float
    static constexpr int OFF_RAW = al(OFF_D + R * C * NPL * 4);        // [RAWD][s, d_old][C][NPL] float
    static constexpr int OFF_X   = al(OFF_RAW + RAWD * 2 * C * NPL * 4); // [2][EYN][C][32] float
    static constexpr int OFF_BAR = al(OFF_X + 2 * EYN * C * 32 * 4);   // NBAR mbarriers, tmem slot, abort flag
    static constexpr int OFF_RED = al(OFF_BAR + NBAR * 8 + 8);          // 32 doubles
    static constexpr int SMEM    = OFF_RED + 32 * 8;
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
    // tcgen05 shared-memory matrix descriptor: K-major, no swizzle (core matrices of 8 rows x 16 bytes)
    uint64_t d = (uint64_t)((addr & 0x3FFFF) >> 4);
    d |= (uint64_t)(LBO_ >> 4) << 16;
    d |= (uint64_t)(SBO_ >> 4) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// tf32 part of x by truncation to the 10 explicit mantissa bits the MMA reads;
// x - hi is exact in FP32 and carries the rest (one LOP3 instead of a rounding
// conversion).
__device__ __forceinline__ float to_tf32(float x) { return __uint_as_float(__float_as_uint(x) & 0xFFFFE000u); }

// x in [-n, 2n): periodic index without a division
__device__ __forceinline__ int wrap(int x, int n) { return x < 0 ? x + n : (x >= n ? x - n : x); }

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

// this thread's lane, 8 consecutive 32-bit columns from taddr
__device__ __forceinline__ void tmem_st8(uint32_t taddr, const float *v)
{
    asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"r"(taddr),
                 "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])),
                 "r"(__float_as_uint(v[3])), "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])),
                 "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7]))
                 : "memory");
}

// D (tmem) += A (tmem, 128 lanes x 8 columns) * B^T (smem descriptor); acc = 0 overwrites
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

// One poll of the phase with the given parity.
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

// Wait for the phase with the given parity; bounded (`limit` polls), and released by the abort flag.
__device__ __forceinline__ void mbar_wait(uint32_t bar, uint32_t parity, volatile int *abort_flag, unsigned limit)
{
    for (unsigned it = 0; it < limit; ++it) {
        uint32_t done;
        asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                     " selp.u32 %0, 1, 0, p;\n}\n"
                     : "=r"(done)
                     : "r"(bar), "r"(parity)
                     : "memory");
        if (done || *abort_flag)
            return;
    }
    *abort_flag = 1;
}

__device__ __forceinline__ void named_bar(int id, int nthreads)
{
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

template <int C, int NPH>
__global__ void __launch_bounds__(TPB, 3) k_stencil_tc(StencilArgs a, const float *__restrict__ Wg)
{
    // one RHS of a multi-RHS solve: a.active points at its flag, and a converged RHS is skipped
    // by every CTA (before any barrier, tensor memory or reduction partial)
    if (a.active && !*a.active)
        return;
    using Cfg = TcCfg<C, NPH>;
    constexpr int NCOL = Cfg::NCOL, NPF = Cfg::NPF;
    extern __shared__ __align__(16) unsigned char smem[];
    float        *Dp        = reinterpret_cast<float *>(smem + Cfg::OFF_D);
    float        *Xch       = reinterpret_cast<float *>(smem + Cfg::OFF_X);
    float        *Raw       = reinterpret_cast<float *>(smem + Cfg::OFF_RAW);
    const uint32_t bar0     = smem_u32(smem + Cfg::OFF_BAR);
    uint32_t     *tmem_slot = reinterpret_cast<uint32_t *>(smem + Cfg::OFF_BAR + NBAR * 8);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(smem + Cfg::OFF_BAR + NBAR * 8 + 4);
    double       *red_smem  = reinterpret_cast<double *>(smem + Cfg::OFF_RED);
    auto bar = [&](int i) { return bar0 + 8u * (uint32_t)i; };
    const unsigned wlim = a.wait_limit > 0 ? (unsigned)a.wait_limit : kWaitLimit;

    const int nx = a.g.nx, ny = a.g.ny, nz = a.g.nz;
    const long long N = (long long)nx * ny * nz;
    const int tid = threadIdx.x, warp = tid / 32, lane = tid % 32;
    const int y0 = blockIdx.y * BY, z0 = blockIdx.z * BZ;
    const int xs = blockIdx.x * XL, xe = min(xs + XL, nx);
    const int J  = xe - xs + 1; // element planes xs-1 .. xe-1
    const long long plane = (long long)ny * nz;

    // ---- setup: W (hi, lo), barriers, tensor memory
    for (int i = tid; i < 2 * Cfg::W_BYTES / 16; i += TPB)
        reinterpret_cast<float4 *>(smem + Cfg::OFF_W)[i] = reinterpret_cast<const float4 *>(Wg)[i];
    if (tid == 0) {
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
    double         dot  = 0.0;

    if (warp < 4) {
        // ================================================================ producers
        const int   ey = warp, ez = lane;
        const float *sin  = reinterpret_cast<const float *>(a.x);
        const float *dold = reinterpret_cast<const float *>(a.d_old);
        float       *dnew = reinterpret_cast<float *>(a.d_new);
        const float  beta = (float)a.scal->beta;
        const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
        // prefetch slots: value tid + k*NGRP of the plane ([c][hy][hz]): global offset without x,
        // plane-local offset, owned node (d_new written)
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
        // node plane index m (node plane xs-1+m): s and d_old copied asynchronously into raw
        // ring slot m % RAWD, RAWD-1 planes ahead of their use; each thread copies and later
        // reads only its own entries, so cp.async.wait_group orders everything it needs
        auto fetch = [&](int m) {
            if (m <= J) {
                const long long gx  = (long long)wrap(xs - 1 + m, nx) * plane;
                float          *raw = Raw + (m % RAWD) * 2 * C * NPL;
#pragma unroll
                for (int k = 0; k < NPF; ++k)
                    if (valid_mask & (1u << k)) {
                        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_u32(raw + loff[k])),
                                     "l"(sin + goff[k] + gx)
                                     : "memory");
                        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(
                                         smem_u32(raw + C * NPL + loff[k])),
                                     "l"(dold + goff[k] + gx)
                                     : "memory");
                    }
            }
            asm volatile("cp.async.commit_group;" ::: "memory");
        };
        // d = s + beta d_old of node plane m into slot m % R (+ d_new for owned nodes)
        auto stage = [&](int m) {
            asm volatile("cp.async.wait_group %0;" ::"n"(RAWD - 2) : "memory"); // plane m has landed
            const int       X       = xs - 1 + m;
            const bool      owned_x = X >= xs && X < xe;
            const long long gx      = (long long)wrap(X, nx) * plane;
            const float    *raw     = Raw + (m % RAWD) * 2 * C * NPL;
            float          *slot    = Dp + (m % R) * C * NPL;
#pragma unroll
            for (int k = 0; k < NPF; ++k)
                if (valid_mask & (1u << k)) {
                    const float v = raw[loff[k]] + beta * raw[C * NPL + loff[k]];
                    slot[loff[k]] = v;
                    if (owned_x && (owned_mask & (1u << k)))
                        dnew[goff[k] + gx] = v;
                }
            mbar_arrive(bar(BAR_STAGED + m % R));
        };
        for (int m = 0; m < RAWD - 1; ++m)
            fetch(m);
        stage(0);
        fetch(RAWD - 1);
        for (int j = 0; j < J; ++j) {
            const int m = j + 1; // node plane to stage
            if (m >= R)                     // consumers are done with node plane m - R
                mbar_wait(bar(BAR_SFREE + m % R), (uint32_t)(((m - R) / R) & 1), abort_flag, wlim);
            stage(m);
            fetch(m + RAWD - 1);            // into the raw slot node plane m-1 used
            named_bar(1, NGRP);     // node planes j and j+1 staged by all producers
            if (j >= 1)             // the MMAs of plane j-1 have read A
                mbar_wait(bar(BAR_DFULL), (uint32_t)((j - 1) & 1), abort_flag, wlim);
            __syncwarp(); // tcgen05.st is warp-aligned
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            // element row of plane j, split hi/lo, into this thread's lane of A
            const float *P0 = Dp + (j % R) * C * NPL, *P1 = Dp + ((j + 1) % R) * C * NPL;
            float u0[C], v[NCOL];
#pragma unroll
            for (int c = 0; c < C; ++c)
                u0[c] = P0[c * NPL + ey * PZ + ez];
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const int qa = q & 1, qb = (q >> 1) & 1, qc = (q >> 2) & 1;
                const float *P = qa ? P1 : P0;
#pragma unroll
                for (int c = 0; c < C; ++c)
                    v[q * C + c] = P[c * NPL + (ey + qb) * PZ + ez + qc] - u0[c];
            }
            float h[NCOL], l[NCOL];
#pragma unroll
            for (int k = 0; k < NCOL; ++k) {
                h[k] = to_tf32(v[k]);
                l[k] = v[k] - h[k];
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
        const int       onode  = ey * PZ + ez;
        const long long oyz    = out_ok ? (long long)(y0 - 1 + ey) * nz + (z0 - 1 + ez) : 0;
        float carry[4 * C]; // far-x rows of this element in the previous plane, [qb + 2 qc][c]
#pragma unroll
        for (int i = 0; i < 4 * C; ++i)
            carry[i] = 0.f;
        int ph_cur = NPH > 1 ? a.ms[(long long)wrap(xs - 1, nx) * plane + el_yz] : 0;
        for (int j = 0; j < J; ++j) {
            const int X = xs - 1 + j, b = j & 1; // b: exchange parity
            const int ph_next = (NPH > 1 && j + 1 < J) ? (int)a.ms[(long long)wrap(X + 1, nx) * plane + el_yz] : 0;
            mbar_wait(bar(BAR_DFULL), (uint32_t)(j & 1), abort_flag, wlim);
            __syncwarp(); // tcgen05.ld is warp-aligned
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            float out[NCOL]; // this element's phase columns, 16 at a time
#pragma unroll
            for (int c0 = 0; c0 < Cfg::NW; c0 += 16) {
                float v[16];
                tmem_ld16(lane_base + (uint32_t)(COL_D + c0), v);
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                for (int jj = 0; jj < 16; ++jj) {
                    const int col = c0 + jj, k = col / NCOL, r = col % NCOL;
                    if (col < Cfg::NROW) {
                        if (k == 0)
                            out[r] = v[jj];
                        else if (ph_cur == k)
                            out[r] = v[jj];
                    }
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            mbar_arrive(bar(BAR_DFREE));
            // x: near-x rows plus the far-x rows carried from the previous plane
            float P[4 * C];
#pragma unroll
            for (int g = 0; g < 4; ++g) { // g = qb + 2 qc, near-x node q = 2g, far-x node 2g + 1
#pragma unroll
                for (int c = 0; c < C; ++c) {
                    P[g * C + c]     = out[2 * g * C + c] + carry[g * C + c];
                    carry[g * C + c] = out[(2 * g + 1) * C + c];
                }
            }
            // z: node (ey + qb, ez) gets lane ez-1's far-z rows
            float Z[2 * C];
#pragma unroll
            for (int qb = 0; qb < 2; ++qb)
#pragma unroll
                for (int c = 0; c < C; ++c)
                    Z[qb * C + c] = P[qb * C + c] + __shfl_up_sync(0xffffffffu, P[(qb + 2) * C + c], 1);
            // y: far-y partial to the exchange, read back by warp ey+1
            float *xw = Xch + (b * EYN + ey) * C * 32 + ez;
#pragma unroll
            for (int c = 0; c < C; ++c)
                xw[c * 32] = Z[C + c];
            named_bar(2, NGRP);
            if (X >= xs) {
                mbar_wait(bar(BAR_STAGED + j % R), (uint32_t)((j / R) & 1), abort_flag, wlim); // node plane X
                if (out_ok) {
                    const long long gi = (long long)wrap(X, nx) * plane + oyz;
                    const float    *xr = Xch + (b * EYN + ey - 1) * C * 32 + ez;
                    const float    *dp = Dp + (j % R) * C * NPL + onode;
                    float           dl = 0.f;
#pragma unroll
                    for (int c = 0; c < C; ++c) {
                        const float v = Z[c] + xr[c * 32];
                        yout[c * N + gi] = v;
                        dl += dp[c * NPL] * v;
                    }
                    dot += (double)dl;
                }
            }
            mbar_arrive(bar(BAR_SFREE + j % R));
            ph_cur = ph_next;
        }
    } else if (lane == 0) {
        // ================================================================ MMA issuer
        const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(Cfg::NW >> 3) << 17) | (8u << 24);
        const uint32_t wbase = smem_u32(smem + Cfg::OFF_W);
        for (int j = 0; j < J; ++j) {
            mbar_wait(bar(BAR_AFULL), (uint32_t)(j & 1), abort_flag, wlim);
            if (j >= 1) // consumers have read D of plane j-1
                mbar_wait(bar(BAR_DFREE), (uint32_t)((j - 1) & 1), abort_flag, wlim);
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            if (!*abort_flag) {
                const uint32_t d = tmem + COL_D, ah = tmem + COL_A, al = tmem + COL_A + COL_LO;
                // 3xTF32: lo*hi + hi*lo + hi*hi (small terms first)
#pragma unroll
                for (int s = 0; s < Cfg::KSTEPS; ++s)
                    umma_tf32_ts(d, al + 8 * s, umma_desc<Cfg::SBO, Cfg::LBO>(wbase + s * 256), idesc, s > 0 ? 1u : 0u);
#pragma unroll
                for (int s = 0; s < Cfg::KSTEPS; ++s)
                    umma_tf32_ts(d, ah + 8 * s, umma_desc<Cfg::SBO, Cfg::LBO>(wbase + Cfg::W_BYTES + s * 256), idesc,
                                 1u);
#pragma unroll
                for (int s = 0; s < Cfg::KSTEPS; ++s)
                    umma_tf32_ts(d, ah + 8 * s, umma_desc<Cfg::SBO, Cfg::LBO>(wbase + s * 256), idesc, 1u);
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                 bar(BAR_DFULL))
                             : "memory");
            } else {
                mbar_arrive(bar(BAR_DFULL)); // keep the consumers' phases moving
            }
        }
        if (*abort_flag) {
            // the consumers may have stopped waiting for MMAs still in flight: wait (bounded) for
            // every MMA this thread issued before tensor memory is released
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             bar(BAR_DRAIN))
                         : "memory");
            for (unsigned it = 0; it < kDrainLimit && !mbar_try(bar(BAR_DRAIN), 0u); ++it) {
            }
        }
    }

    __syncthreads();
    if (*abort_flag && tid == 0)
        a.scal->converged = -3; // a tensor-core pipeline wait expired

    // <d, K d> over the grid (solverCG.h:101)
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

bool stencil_tc_supported(const Grid3 &g, int C, int nph)
{
    return (C == 3 || C == 1) && nph >= 1 && nph <= 2 && g.nx >= 2 && g.ny >= 2 && g.nz >= 2;
}

size_t stencil_tc_weights(int C, int nph)
{
    const int ncol = 8 * C, nrow = nph * ncol, nw = (nrow + 15) / 16 * 16;
    return (size_t)2 * nw * ncol; // floats: hi then lo
}

// W[n][k] = K_{n / 8C}[n % 8C][k] (rows padded to the MMA N) in the K-major
// no-swizzle core-matrix layout, split into tf32 hi and FP32 remainder lo.
void stencil_tc_pack_weights(int C, int nph, const float *K32, float *out)
{
    const int ncol = 8 * C, kc = ncol / 4, nrow = nph * ncol, nw = (nrow + 15) / 16 * 16;
    const int sbo = kc * 128;
    const size_t half = (size_t)nw * ncol;
    for (size_t i = 0; i < 2 * half; ++i)
        out[i] = 0.f;
    for (int n = 0; n < nrow; ++n)
        for (int k = 0; k < ncol; ++k) {
            const float x = K32[((size_t)(n / ncol) * ncol + n % ncol) * ncol + k];
            uint32_t    u;
            std::memcpy(&u, &x, 4);
            // top 11 significant bits (10 explicit mantissa bits), as the kernel splits its operand
            const uint32_t h = u & 0xFFFFE000u;
            float          hi;
            std::memcpy(&hi, &h, 4);
            const float  lo  = x - hi;
            const size_t off = ((size_t)(n / 8) * sbo + (size_t)(k / 4) * 128 + (n % 8) * 16 + (k % 4) * 4) / 4;
            out[off]        = hi;
            out[half + off] = lo;
        }
}

cudaError_t launch_stencil_tc(const StencilArgs &a, const float *W, int nph, cudaStream_t st)
{
    dim3 grid((a.g.nx + XL - 1) / XL, (a.g.ny + BY - 1) / BY, (a.g.nz + BZ - 1) / BZ);
#define FANSGPU_TC(C_, P_)                                                                                       \
    do {                                                                                                       \
        constexpr int sm = SMEM_REQ;                                                                           \
        cudaError_t   e  = allow_max_dyn_smem(k_stencil_tc<C_, P_>); \
        if (e != cudaSuccess)                                                                                  \
            return e;                                                                                          \
        k_stencil_tc<C_, P_><<<grid, TPB, sm, st>>>(a, W);                                                     \
    } while (0)
    if (a.C == 3 && nph == 1)
        FANSGPU_TC(3, 1);
    else if (a.C == 3)
        FANSGPU_TC(3, 2);
    else if (nph == 1)
        FANSGPU_TC(1, 1);
    else
        FANSGPU_TC(1, 2);
#undef FANSGPU_TC
    return cudaGetLastError();
}

long long stencil_tc_blocks(const Grid3 &g)
{
    return (long long)((g.nx + XL - 1) / XL) * ((g.ny + BY - 1) / BY) * ((g.nz + BZ - 1) / BZ);
}

} // namespace fansgpu
