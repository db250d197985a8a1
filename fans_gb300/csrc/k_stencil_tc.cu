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
// at FP32 accuracy.  A (the element rows) is written by each thread straight
// into its tensor-memory lane with tcgen05.st; W sits in shared memory; D
// accumulates in tensor memory.
//
// A CTA owns a 3 (y) x 31 (z) column of nodes, whose element plane is exactly
// one M-tile (4 x 32 = 128 elements; warp w holds element row ey = w, lane l
// element ez = l) and marches along x over XL planes.  Per step it stages node
// plane X+1 (d = s + beta d_old from registers prefetched one step earlier;
// written to d_new for owned nodes), builds the element rows of plane X into
// tensor memory, issues the 9 MMAs, writes node plane X-1 (K d and <d, K d>)
// while the tensor cores run, then reads its element's phase columns of D and
// sums them into nodes without shared-memory atomics or colour copies:
//   x: the rows of the element's far-x nodes are carried in registers to the
//      next plane, where the same thread adds its near-x rows;
//   z: one warp shuffle adds lane ez-1's far-z rows;
//   y: the far-y partial goes through a small shared exchange buffer and warp
//      ey+1 adds it when it writes the node.
// Every node is therefore a fixed-order sum (deterministic).  About 12 KB of
// shared memory is used; 48 KB is requested so that exactly four CTAs share an
// SM, which is what their 4 x 128 tensor-memory columns allow.
#include "kernels.cuh"

#include <cstring>

namespace fansgpu {

namespace {

constexpr int BY = 3, BZ = 31;
constexpr int PY = BY + 2, PZ = BZ + 2;   // node plane incl. halo: y0-1..y0+3, z0-1..z0+31
constexpr int EYN = BY + 1, EZN = BZ + 1; // element plane: origins y0-1..y0+2, z0-1..z0+30
constexpr int NEL = EYN * EZN;            // 128 elements = one M-tile
constexpr int TPB = 128;
constexpr int NPL = PY * PZ;              // 165 nodes per plane incl. halo
constexpr int XL  = 32;                   // planes per CTA
constexpr int TCOLS  = 128;               // tensor memory: D [0, 64), A hi [64, 96), A lo [96, 128)
constexpr int COL_AH = 64, COL_AL = 96;
// dynamic shared memory requested: with the 1 KB the driver reserves per block, 4 CTAs fit in an
// SM's 228 KB and 5 do not -- residency is capped at the 4 x 128 tensor-memory columns an SM has
constexpr int SMEM_REQ = 48 * 1024;
constexpr unsigned kWaitLimit = 1u << 24; // bounded mbarrier wait
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
    static constexpr int NPF     = (C * NPL + TPB - 1) / TPB; // prefetched node values per thread and field
    static constexpr int al(int b) { return (b + 127) / 128 * 128; }
    static constexpr int OFF_W   = 0;                                  // [hi, lo][W_BYTES]
    static constexpr int OFF_D   = al(OFF_W + 2 * W_BYTES);            // [3 slots][C][NPL] float
    static constexpr int OFF_X   = al(OFF_D + 3 * C * NPL * 4);        // [2 parity][4 warps][C][32] float
    static constexpr int OFF_BAR = al(OFF_X + 2 * EYN * C * 32 * 4);
    static constexpr int SMEM    = OFF_BAR + 16 + 32 * 8;
    static_assert(NW <= COL_AH && NCOL <= COL_AL - COL_AH && NCOL <= TCOLS - COL_AL, "tensor-memory map");
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

template <int C, int NPH>
__global__ void __launch_bounds__(TPB, 4) k_stencil_tc(StencilArgs a, const float *__restrict__ Wg)
{
    using Cfg = TcCfg<C, NPH>;
    constexpr int NCOL = Cfg::NCOL, NPF = Cfg::NPF;
    extern __shared__ __align__(16) unsigned char smem[];
    float    *Dp        = reinterpret_cast<float *>(smem + Cfg::OFF_D);
    float    *Xch       = reinterpret_cast<float *>(smem + Cfg::OFF_X);
    uint64_t *mbar      = reinterpret_cast<uint64_t *>(smem + Cfg::OFF_BAR);
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(smem + Cfg::OFF_BAR + 8);
    double   *red_smem  = reinterpret_cast<double *>(smem + Cfg::OFF_BAR + 16);

    const int nx = a.g.nx, ny = a.g.ny, nz = a.g.nz;
    const long long N = (long long)nx * ny * nz;
    const int tid = threadIdx.x, warp = tid / 32, lane = tid % 32;
    const int y0 = blockIdx.y * BY, z0 = blockIdx.z * BZ;
    const int xs = blockIdx.x * XL, xe = min(xs + XL, nx);
    const float *sin  = reinterpret_cast<const float *>(a.x);
    const float *dold = reinterpret_cast<const float *>(a.d_old);
    float       *dnew = reinterpret_cast<float *>(a.d_new);
    float       *yout = reinterpret_cast<float *>(a.y);
    const float  beta = (float)a.scal->beta;

    // this thread's element (row ey = warp, column ez = lane) and global (y, z)
    const int       ey = warp, ez = lane;
    const long long el_yz = (long long)pmod(y0 - 1 + ey, ny) * nz + pmod(z0 - 1 + ez, nz);
    const long long plane = (long long)ny * nz;

    // ---- one-off setup: W (hi, lo), barrier, TMEM
    for (int i = tid; i < 2 * Cfg::W_BYTES / 16; i += TPB)
        reinterpret_cast<float4 *>(smem + Cfg::OFF_W)[i] = reinterpret_cast<const float4 *>(Wg)[i];
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(mbar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "n"(TCOLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }

    // prefetch slots: value tid + k*TPB of the plane ([c][hy][hz]); global offset without x,
    // plane-local offset, and whether it is an owned node (d_new written)
    long long goff[NPF];
    int       loff[NPF];
    unsigned  owned_mask = 0, valid_mask = 0;
#pragma unroll
    for (int k = 0; k < NPF; ++k) {
        const int idx = tid + k * TPB;
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
    // output node of this thread: node (ey, ez) of the halo plane, owned for ey >= 1, ez >= 1
    const bool      out_ok = ey >= 1 && ez >= 1 && y0 - 1 + ey < ny && z0 - 1 + ez < nz;
    const int       onode  = ey * PZ + ez;
    const long long oyz    = out_ok ? (long long)(y0 - 1 + ey) * nz + (z0 - 1 + ez) : 0;

    // node plane X: thread's share of (s, d_old) into registers
    float sv[NPF], dv[NPF];
    auto load_plane = [&](int X) {
        const long long gx = (long long)wrap(X, nx) * plane;
#pragma unroll
        for (int k = 0; k < NPF; ++k)
            if (valid_mask & (1u << k)) {
                sv[k] = __ldg(sin + goff[k] + gx);
                dv[k] = __ldg(dold + goff[k] + gx);
            }
    };
    // d = s + beta d_old of the registered plane X into node slot ds (+ d_new for owned nodes)
    auto store_plane = [&](int X, int ds) {
        const bool      owned_x = X >= xs && X < xe;
        const long long gx      = (long long)wrap(X, nx) * plane;
#pragma unroll
        for (int k = 0; k < NPF; ++k)
            if (valid_mask & (1u << k)) {
                const float v = sv[k] + beta * dv[k];
                Dp[ds * C * NPL + loff[k]] = v;
                if (owned_x && (owned_mask & (1u << k)))
                    dnew[goff[k] + gx] = v;
            }
    };
    // node plane Xo: this thread's near-y partial plus warp ey-1's far-y partial (exchange
    // parity xp); d from node slot ds
    float  pend[C];
    double dot = 0.0;
    auto output_plane = [&](int Xo, int xp, int ds) {
        if (!out_ok)
            return;
        const long long gi = (long long)wrap(Xo, nx) * plane + oyz;
        const float    *xc = Xch + ((xp * EYN + ey - 1) * C) * 32 + ez;
        float           dl = 0.f;
#pragma unroll
        for (int c = 0; c < C; ++c) {
            const float v = pend[c] + xc[c * 32];
            yout[c * N + gi] = v;
            dl += Dp[(ds * C + c) * NPL + onode] * v;
        }
        dot += (double)dl;
    };

    // ---- prologue: node plane xs-1 stored, node plane xs and the phases of element plane xs-1 in registers
    load_plane(xs - 1);
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;
    const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
    store_plane(xs - 1, 0);
    load_plane(xs);
    int ph_cur = a.ms[(long long)wrap(xs - 1, nx) * plane + el_yz];

    const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(Cfg::NW >> 3) << 17) | (8u << 24);
    bool  ok = true;
    float carry[4 * C]; // far-x rows (qa = 1) of this thread's element in plane X-1, [qb + 2 qc][c]
#pragma unroll
    for (int i = 0; i < 4 * C; ++i)
        carry[i] = 0.f;

    for (int X = xs - 1; X < xe; ++X) {
        const int j = X - xs + 1; // 0 .. xe-xs
        // node plane X+1 into slot (j+1)%3: its last readers (element plane X-2, output of
        // node plane X-2) finished before the previous step's completion barrier
        store_plane(X + 1, (j + 1) % 3);
        if (X + 2 <= xe)
            load_plane(X + 2);
        const int ph_next = X + 1 < xe ? (int)a.ms[(long long)wrap(X + 1, nx) * plane + el_yz] : 0;
        __syncthreads(); // S2: node planes X, X+1 staged; exchange of node plane X-1 visible

        // element row of plane X, split hi/lo, into this thread's tensor-memory lane
        {
            const float *P0 = Dp + (j % 3) * C * NPL, *P1 = Dp + ((j + 1) % 3) * C * NPL;
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
                tmem_st8(lane_base + (uint32_t)(COL_AH + k0), h + k0);
                tmem_st8(lane_base + (uint32_t)(COL_AL + k0), l + k0);
            }
            asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads(); // S3: A of plane X in tensor memory

        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t wbase = smem_u32(smem + Cfg::OFF_W);
            // 3xTF32: lo*hi + hi*lo + hi*hi (small terms first)
#pragma unroll
            for (int s = 0; s < Cfg::KSTEPS; ++s)
                umma_tf32_ts(tmem, tmem + COL_AL + 8 * s, umma_desc<Cfg::SBO, Cfg::LBO>(wbase + s * 256), idesc,
                             s > 0 ? 1u : 0u);
#pragma unroll
            for (int s = 0; s < Cfg::KSTEPS; ++s)
                umma_tf32_ts(tmem, tmem + COL_AH + 8 * s,
                             umma_desc<Cfg::SBO, Cfg::LBO>(wbase + Cfg::W_BYTES + s * 256), idesc, 1u);
#pragma unroll
            for (int s = 0; s < Cfg::KSTEPS; ++s)
                umma_tf32_ts(tmem, tmem + COL_AH + 8 * s, umma_desc<Cfg::SBO, Cfg::LBO>(wbase + s * 256), idesc, 1u);
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             smem_u32(mbar))
                         : "memory");
        }

        // node plane X-1 (its exchange was written before S2) while the MMAs run
        if (X - 1 >= xs)
            output_plane(X - 1, (X - 1) & 1, (j + 2) % 3);

        uint32_t done = 1;
        if (tid == 0) { // one poller; the other threads wait at the barrier below
            done = 0;
            for (unsigned it = 0; it < kWaitLimit && !done; ++it)
                asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                             " selp.u32 %0, 1, 0, p;\n}\n"
                             : "=r"(done)
                             : "r"(smem_u32(mbar)), "r"((uint32_t)(j & 1))
                             : "memory");
        }
        if (!__syncthreads_and(done ? 1 : 0)) { // S4: D ready; output of node plane X-1 done
            ok = false;
            break;
        }

        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        {
            // this element's phase rows: out[q*C + c], local node q = qa + 2 qb + 4 qc
            float out[NCOL];
            {
                float v[Cfg::NW];
#pragma unroll
                for (int c0 = 0; c0 < Cfg::NW; c0 += 16)
                    tmem_ld16(lane_base + (uint32_t)c0, v + c0);
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                for (int r = 0; r < NCOL; ++r)
                    out[r] = (NPH > 1 && ph_cur == 1) ? v[NCOL + r] : v[r];
            }
            // x: near-x rows plus the far-x rows carried from element plane X-1
            float P[4 * C];
#pragma unroll
            for (int b = 0; b < 4; ++b) { // b = qb + 2 qc
                const int q0 = 2 * b;     // qa = 0
#pragma unroll
                for (int c = 0; c < C; ++c) {
                    P[b * C + c]     = out[q0 * C + c] + carry[b * C + c];
                    carry[b * C + c] = out[(q0 + 1) * C + c];
                }
            }
            // z: node (ey + qb, ez) gets lane ez-1's far-z rows (qc = 1)
            float Z[2 * C];
#pragma unroll
            for (int qb = 0; qb < 2; ++qb)
#pragma unroll
                for (int c = 0; c < C; ++c)
                    Z[qb * C + c] = P[qb * C + c] + __shfl_up_sync(0xffffffffu, P[(qb + 2) * C + c], 1);
            // y: far-y partial (node ey+1) to the exchange; near-y partial kept for the output
            float *xc = Xch + ((X & 1) * EYN + ey) * C * 32 + ez;
#pragma unroll
            for (int c = 0; c < C; ++c) {
                xc[c * 32] = Z[C + c];
                pend[c]    = Z[c];
            }
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        ph_cur = ph_next;
    }
    __syncthreads();
    if (ok)
        output_plane(xe - 1, (xe - 1) & 1, (xe - xs) % 3);
    else if (tid == 0)
        a.scal->converged = -3; // tensor-core completion wait timed out

    // <d, K d> over the grid (solverCG.h:101)
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
