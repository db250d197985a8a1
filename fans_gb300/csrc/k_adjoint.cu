// k_adjoint.cu -- per-Gauss-point kernels of the yield-stress adjoint of a
// strain-controlled J2PlasticityNew load path.
//
// Load step n solves R_n(u_n; alpha_{n-1}, sigma_y) = 0 and commits
// alpha_n = A(eps_n, alpha_{n-1}; sigma_y), alpha = (eps_p, q) per Gauss point
// (J2PlasticityNew.h:43-108, solver.h:283-311).  For L = w . <sigma_N> the
// reverse sweep runs n = N..1 with mu_N = 0:
//   K_n^T lambda_n = -f_n,  f_n = sum_gp B^T VJP_e(cw [n = N], mu_n)
//   tau_n          = (v_e/n_gp) B lambda_n + cw [n = N]
//   mu_{n-1}       = VJP_alpha(tau_n, mu_n)
//   dL/dsigma_y(e) += sum_gp VJP_sy(tau_n, mu_n)
// with cw = w/(N n_gp), the weight of one Gauss point in <sigma>.  The solve of
// lambda_n is a linear CG whose residual K_n^T lambda + f_n is the affine map
// ADJ_RESIDUAL below; ADJ_OPERATOR is its linear part.  Both have the form
// sum_gp B^T sigma_adj of a residual, so the Green's operator preconditions
// them as it does the forward solve.
//
// One thread per (element, Gauss point); the n_gp threads of an element are
// adjacent lanes of a warp, the element row B^T g is summed over them by the
// same butterfly reduce-scatter as the element kernel.  The trip count is a
// whole number of warps so that every shuffle sees all lanes.
#include "../../include/fans_gb300.h"
#include "j2_law.cuh"
#include "kernels.cuh"

namespace fansgpu {

namespace {

constexpr int kAdjThreads = 128;
constexpr int kAdjPrm     = 8; // law parameters per phase

// eps = B_gp x_e + off, x_e relative to the element's node 0 (as the residual
// forms it, solver.h:252), SoA x [3][N]; with the basic B (Bb) by the same
// 72-term kinematics as the element kernel, so that replayed states match the
// forward ones bit for bit.
__device__ __forceinline__ void gp_strain(const double *Bg, const double *Bb, const double *__restrict__ x,
                                          const long long (&idx)[8], long long N, bool valid, const double *off,
                                          double (&e)[6])
{
    double ue[24];
    if (valid) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const double u0 = x[c * N + idx[0]];
#pragma unroll
            for (int q = 0; q < 8; ++q)
                ue[q * 3 + c] = x[c * N + idx[q]] - u0;
        }
    } else {
#pragma unroll
        for (int k = 0; k < 24; ++k)
            ue[k] = 0.0;
    }
    if (Bb) {
        strain_basic_b(Bb, ue, off, e);
        return;
    }
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        double acc = 0.0;
#pragma unroll
        for (int k = 0; k < 24; ++k)
            acc += Bg[i * 24 + k] * ue[k];
        e[i] = acc + (off ? off[i] : 0.0);
    }
}

template <int NGP, int MODE>
__global__ void __launch_bounds__(kAdjThreads) k_adjoint(AdjArgs a)
{
    static_assert(32 % NGP == 0 && 24 % NGP == 0, "group layout");
    __shared__ double Bs[NGP * 6 * 24];
    __shared__ double Bbs[NGP * 24];
    for (int i = threadIdx.x; i < NGP * 6 * 24; i += blockDim.x)
        Bs[i] = a.B[i];
    if (a.Bb)
        for (int i = threadIdx.x; i < NGP * 24; i += blockDim.x)
            Bbs[i] = a.Bb[i];
    __syncthreads();
    const int       nx = a.g.nx, ny = a.g.ny, nz = a.g.nz;
    const long long N  = (long long)nx * ny * nz;
    const long long T  = (N * NGP + 31) / 32 * 32;
    const int       gp = (int)(threadIdx.x % NGP);
    const double   *Bg = Bs + gp * 6 * 24;
    const double   *Bb = a.Bb ? Bbs + gp * 24 : nullptr;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < T; t += (long long)gridDim.x * blockDim.x) {
        const long long el    = t / NGP;
        const bool      valid = el < N;
        const int       ph    = valid ? a.ms[el] : 0;
        const bool      j2    = valid && a.law[ph] == FANSGPU_LAW_J2_LINEAR;
        long long       idx[8];
        if (valid)
            elem_nodes(nx, ny, nz, el, idx);
        else
#pragma unroll
            for (int q = 0; q < 8; ++q)
                idx[q] = 0;
        const long long base = (long long)gp * N + el;
        double          e[6], ep_in[6], q_in = 0.0;
        gp_strain(Bg, Bb, a.u, idx, N, valid, a.g0, e);
#pragma unroll
        for (int i = 0; i < 6; ++i)
            ep_in[i] = valid ? a.ep_in[(long long)i * NGP * N + base] : 0.0;
        if (valid)
            q_in = a.q_in[base];
        const double *pj  = a.prm + ph * kAdjPrm;
        const double  sy0 = j2 ? (a.sy ? a.sy[el] : pj[2]) : 0.0;

        if constexpr (MODE == ADJ_REPLAY) {
            if (valid) {
                double sig[6], ep_out[6], q_out = q_in;
                if (j2)
                    j2_sigma(pj, sy0, e, ep_in, q_in, sig, ep_out, q_out);
                else
#pragma unroll
                    for (int i = 0; i < 6; ++i)
                        ep_out[i] = ep_in[i];
#pragma unroll
                for (int i = 0; i < 6; ++i)
                    a.ep_out[(long long)i * NGP * N + base] = ep_out[i];
                a.q_out[base] = q_out;
            }
        } else {
            double tau[6];
            gp_strain(Bg, Bb, a.x, idx, N, valid, nullptr, tau);
            const double w    = a.ve / NGP;
            const bool   seed = MODE != ADJ_OPERATOR && a.cw; // the operator is the linear part alone
#pragma unroll
            for (int i = 0; i < 6; ++i)
                tau[i] = w * tau[i] + (seed ? a.cw[i] : 0.0);
            double mep[6], mq = 0.0;
            const bool with_mu = MODE != ADJ_OPERATOR && j2 && a.mu_ep;
#pragma unroll
            for (int i = 0; i < 6; ++i)
                mep[i] = with_mu ? a.mu_ep[(long long)i * NGP * N + base] : 0.0;
            if (with_mu)
                mq = a.mu_q[base];
            double ge[6], gep[6], gq = 0.0, gsy = 0.0;
            if (j2) {
                j2_vjp(pj, sy0, e, ep_in, q_in, tau, mep, mq, ge, gep, gq, gsy);
            } else {
                const double *Cm = a.Cph + ph * 36;
#pragma unroll
                for (int i = 0; i < 6; ++i) {
                    double acc = 0.0;
#pragma unroll
                    for (int k = 0; k < 6; ++k)
                        acc += Cm[k * 6 + i] * tau[k];
                    ge[i]  = acc;
                    gep[i] = 0.0;
                }
            }
            if constexpr (MODE == ADJ_STEP) {
                if (j2) {
#pragma unroll
                    for (int i = 0; i < 6; ++i)
                        a.mu_ep[(long long)i * NGP * N + base] = gep[i];
                    a.mu_q[base] = gq;
                }
                double g = j2 ? gsy : 0.0;
#pragma unroll
                for (int m = NGP / 2; m >= 1; m /= 2)
                    g += __shfl_xor_sync(0xffffffffu, g, m);
                if (valid && gp == 0)
                    a.grad[el] += g;
            } else {
                double v[24];
                if (Bb)
                    bt_sigma_basic_b(Bb, ge, v);
                else
#pragma unroll
                    for (int k = 0; k < 24; ++k) {
                        double acc = 0.0;
#pragma unroll
                        for (int i = 0; i < 6; ++i)
                            acc += Bg[i * 24 + k] * ge[i];
                        v[k] = acc;
                    }
                // reduce-scatter over the NGP lanes of the element
                int kb = 0;
#pragma unroll
                for (int m = NGP / 2, cntv = 24; m >= 1; m /= 2, cntv /= 2) {
                    const bool hi = (gp & m) != 0;
#pragma unroll
                    for (int j = 0; j < cntv / 2; ++j) {
                        const double keep = hi ? v[cntv / 2 + j] : v[j];
                        const double send = hi ? v[j] : v[cntv / 2 + j];
                        v[j]              = keep + __shfl_xor_sync(0xffffffffu, send, m);
                    }
                    if (hi)
                        kb += cntv / 2;
                }
                if (valid)
#pragma unroll
                    for (int j = 0; j < 24 / NGP; ++j)
                        a.rows[(long long)(kb + j) * N + el] = v[j];
            }
        }
    }
}

} // namespace

cudaError_t launch_adjoint(const AdjArgs &a, cudaStream_t st)
{
    const long long want = (a.g.N() * a.ngp + kAdjThreads - 1) / kAdjThreads;
    const int       nb   = (int)(want < 152 * 16 ? (want < 1 ? 1 : want) : 152 * 16);
#define FANSGPU_ADJ(G_)                                                                                      \
    switch (a.mode) {                                                                                        \
    case ADJ_OPERATOR: k_adjoint<G_, ADJ_OPERATOR><<<nb, kAdjThreads, 0, st>>>(a); break;                    \
    case ADJ_RESIDUAL: k_adjoint<G_, ADJ_RESIDUAL><<<nb, kAdjThreads, 0, st>>>(a); break;                    \
    case ADJ_STEP: k_adjoint<G_, ADJ_STEP><<<nb, kAdjThreads, 0, st>>>(a); break;                            \
    case ADJ_REPLAY: k_adjoint<G_, ADJ_REPLAY><<<nb, kAdjThreads, 0, st>>>(a); break;                        \
    default: return cudaErrorInvalidValue;                                                                   \
    }
    if (a.ngp == 8) {
        FANSGPU_ADJ(8)
    } else if (a.ngp == 1) {
        FANSGPU_ADJ(1)
    } else {
        return cudaErrorInvalidValue;
    }
#undef FANSGPU_ADJ
    return cudaGetLastError();
}

} // namespace fansgpu
