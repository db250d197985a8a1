// k_element.cu -- element-centric kernels for constitutive laws with internal
// variables (J2PlasticityNew) and the general residual R(u) of any law.
//
// k_element: one thread per (element, Gauss point).  u_e relative to the
// element's node 0 (solver.h:252), eps_gp = B_gp u_e + g0 (matmodel.h:194),
// sigma_gp from the phase's law (linear C, or the J2 radial return of
// J2PlasticityNew.h:43-108 writing trial internal variables), then either
//   mode RESIDUAL: r_e = sum_gp B_gp^T sigma_gp v_e/n_gp (matmodel.h:199) into a
//                  row-plane scratch [8C][N] for the node gather, or
//   mode AVERAGES: element means of eps and sigma (matmodel.h:203-225) summed
//                  into FP64 block partials (phase-filtered), optional fields.
// k_gather: r_node = sum over the 8 elements around the node of their rows for
// that node -- the scatter of solver.h:257-261 as a deterministic gather.
// Internal variables are SoA: eps_p[6][n_gp][N], q[n_gp][N] (trial and
// committed copies), in FP64.
#include "../../include/fans_gb300.h"
#include "j2_law.cuh"
#include "kernels.cuh"

namespace fansgpu {

namespace {

constexpr int kElThreads = 128;
constexpr int kPrm       = 8; // law parameters per phase

// LargeStrainMechModel::get_sigma (LargeStrainMechModel.h:190-196) for
// SaintVenantKirchhoff (S = lambda tr(E) I + 2 mu E, E = (F^T F - I)/2,
// SaintVenantKirchhoff.h:36-41) and CompressibleNeoHookean (S = lambda log(J)
// C^-1 + mu (I - C^-1), CompressibleNeoHookean.h:36-49): P = F S, F and P stored
// row-major (F_iJ at 3i + J).  prm: {K, G}, lambda = K - 2G/3, mu = G.  A
// non-positive det F (where the reference throws) yields NaN, which the solver
// reports as a non-finite residual.
__device__ __forceinline__ void large_strain_sigma(int law, const double *prm, const double (&F)[9], double (&P)[9])
{
    const double mu = prm[1], lam = prm[0] - (2.0 / 3.0) * mu;
    double       Cg[9]; // right Cauchy-Green C = F^T F
#pragma unroll
    for (int I = 0; I < 3; ++I)
#pragma unroll
        for (int J = 0; J < 3; ++J)
            Cg[3 * I + J] = F[I] * F[J] + F[3 + I] * F[3 + J] + F[6 + I] * F[6 + J];
    double S[9];
    if (law == FANSGPU_LAW_SVK) {
        const double trE = 0.5 * (Cg[0] + Cg[4] + Cg[8] - 3.0);
#pragma unroll
        for (int k = 0; k < 9; ++k)
            S[k] = mu * (Cg[k] - ((k % 4) == 0 ? 1.0 : 0.0)) + ((k % 4) == 0 ? lam * trE : 0.0);
    } else {
        const double J = F[0] * (F[4] * F[8] - F[5] * F[7]) - F[1] * (F[3] * F[8] - F[5] * F[6]) +
                         F[2] * (F[3] * F[7] - F[4] * F[6]);
        // C^-1 = adj(C) / det(C), det(C) = J^2
        double Ci[9];
        Ci[0] = Cg[4] * Cg[8] - Cg[5] * Cg[7];
        Ci[1] = Cg[2] * Cg[7] - Cg[1] * Cg[8];
        Ci[2] = Cg[1] * Cg[5] - Cg[2] * Cg[4];
        Ci[3] = Cg[5] * Cg[6] - Cg[3] * Cg[8];
        Ci[4] = Cg[0] * Cg[8] - Cg[2] * Cg[6];
        Ci[5] = Cg[2] * Cg[3] - Cg[0] * Cg[5];
        Ci[6] = Cg[3] * Cg[7] - Cg[4] * Cg[6];
        Ci[7] = Cg[1] * Cg[6] - Cg[0] * Cg[7];
        Ci[8] = Cg[0] * Cg[4] - Cg[1] * Cg[3];
        const double inv_det = 1.0 / (J * J);
        const double c1      = J > 0.0 ? lam * log(J) - mu : __longlong_as_double(0x7ff8000000000000LL);
#pragma unroll
        for (int k = 0; k < 9; ++k)
            S[k] = c1 * Ci[k] * inv_det + ((k % 4) == 0 ? mu : 0.0);
    }
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int J = 0; J < 3; ++J)
            P[3 * i + J] = F[3 * i] * S[J] + F[3 * i + 1] * S[3 + J] + F[3 * i + 2] * S[6 + J];
}

// One thread per (element, Gauss point): the NGP threads of an element are
// adjacent lanes of one warp.  Each computes eps, sigma (and the J2 update) of
// its Gauss point; the element row B^T sigma is summed over the group by a
// butterfly reduce-scatter, after which lane gp holds NCOL/NGP of the sums.
// The loop runs whole warps (the trip count is rounded up to 32) so that every
// shuffle sees all lanes; lanes past the end compute on zeros and store nothing.
// PseudoPlasticLinearHardening / NonLinearHardening::get_sigma (PseudoPlastic.h:
// 92-115, 138-160), history-free.  prm (8 per phase): linear {K, G, sigma_y, h,
// eps_crit, E_s, flag_elastic, flag_plastic}; nonlinear {K, G, sigma_y, n, eps_0,
// eps_crit, flag_elastic, flag_plastic}.  Returns the Gauss point's plastic flag.
__device__ __forceinline__ double pseudo_sigma(int law, const double *prm, const double (&e)[6], double (&sig)[6])
{
    const double K = prm[0], G = prm[1], sy = prm[2];
    const double treps = e[0] + e[1] + e[2];
    double       dev[6];
#pragma unroll
    for (int i = 0; i < 3; ++i)
        dev[i] = e[i] - (1.0 / 3.0) * treps;
#pragma unroll
    for (int i = 3; i < 6; ++i)
        dev[i] = e[i];
    double n2 = 0.0;
#pragma unroll
    for (int i = 0; i < 6; ++i)
        n2 += dev[i] * dev[i];
    const double nrm  = sqrt(n2);
    const double buf1 = K * treps;
    double       buf2, flag;
    if (law == FANSGPU_LAW_PSEUDO_LINEAR) {
        const double h = prm[3], eps_crit = prm[4], E_s = prm[5];
        if (nrm <= eps_crit) {
            buf2 = 2.0 * G;
            flag = prm[6];
        } else {
            buf2 = (sqrt(2.0 / 3.0) * sy + (2.0 / 3.0) * E_s * h * (nrm - eps_crit)) / nrm;
            flag = prm[7];
        }
    } else {
        const double n = prm[3], eps0 = prm[4], eps_crit = prm[5];
        const double eq = sqrt(2.0 / 3.0) * nrm;
        if (eq <= eps_crit) {
            buf2 = 2.0 * G;
            flag = prm[6];
        } else {
            buf2 = sqrt(2.0 / 3.0) * sy * pow(eq / eps0, n) / nrm;
            flag = prm[7];
        }
    }
#pragma unroll
    for (int i = 0; i < 3; ++i)
        sig[i] = buf1 + buf2 * dev[i];
#pragma unroll
    for (int i = 3; i < 6; ++i)
        sig[i] = buf2 * dev[i];
    return flag;
}

// J2Plasticity::get_sigma with J2ViscoPlastic hardening (J2Plasticity.h:62-108,
// :158-225), one Gauss point.  prm: {K, G, sigma_y, K_iso, H_kin, eta/dt,
// sigma_inf, delta}.  The trial psi and psi_bar accumulate over evaluations
// (psi += c23 gamma, psi_bar -= gamma n), as in the reference; eps_p is rebuilt
// from its committed value.  Returns gamma; writes sigma and the direction n.
__device__ __forceinline__ double j2visco_sigma(bool nonlin, const double *prm, const double (&e)[6],
                                                const double (&ep_in)[6], double psit, const double (&pbt)[6],
                                                double (&sig)[6], double (&nv)[6])
{
    const double K = prm[0], G = prm[1], sy = prm[2], Ki = prm[3], H = prm[4], eta_dt = prm[5];
    const double c23 = sqrt(2.0 / 3.0);
    double       ee[6], st[6];
#pragma unroll
    for (int i = 0; i < 6; ++i)
        ee[i] = e[i] - ep_in[i];
    const double treps = ee[0] + ee[1] + ee[2];
#pragma unroll
    for (int i = 0; i < 3; ++i)
        st[i] = (K - 2.0 * G / 3.0) * treps + 2 * G * ee[i];
#pragma unroll
    for (int i = 3; i < 6; ++i)
        st[i] = 2 * G * ee[i];
    const double mean = (st[0] + st[1] + st[2]) / 3.0;
    double       qtr  = -Ki * psit;
    if (nonlin)
        qtr -= (prm[6] - sy) * (1 - exp(-prm[7] * psit));
    double dmq[6], n2 = 0.0;
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        dmq[i] = (i < 3 ? st[i] - mean : st[i]) + (2.0 / 3.0) * H * pbt[i];
        n2 += dmq[i] * dmq[i];
    }
    const double nrm = sqrt(n2);
#pragma unroll
    for (int i = 0; i < 6; ++i)
        nv[i] = nrm < 1e-12 ? 0.0 : dmq[i] / nrm;
    const double f   = nrm - c23 * (sy - qtr);
    const double den = 2 * G + (2.0 / 3.0) * (Ki + H) + eta_dt;
    double       gam = 0.0;
    if (f >= 0) {
        if (!nonlin) {
            gam = f / den;
        } else { // Newton iteration of J2Plasticity.h:203-214 (its (2 / 3) factor is integer zero)
            const double sdiff = c23 * (prm[6] - sy), del = prm[7];
            double       inc   = 1.0;
            for (int it = 0; inc > 1e-10 && it < 10; ++it) {
                const double g = f - gam * den - sdiff * (-exp(-del * (psit + c23 * gam)) + exp(-del * psit));
                inc            = g / den; // -g / dg with dg = -den
                gam += inc;
            }
        }
    }
#pragma unroll
    for (int i = 0; i < 6; ++i)
        sig[i] = st[i] - gam * 2 * G * nv[i];
    return gam;
}

template <int C, int NGP, int MODE, bool LARGE = false>
__global__ void __launch_bounds__(kElThreads) k_element(ElementArgs a)
{
    constexpr int NSTR = LARGE ? 9 : (C == 1 ? 3 : 6), NCOL = 8 * C, NE = NSTR > 6 ? NSTR : 6;
    static_assert(32 % NGP == 0 && NCOL % NGP == 0, "group layout");
    __shared__ double Bs[NGP * NSTR * NCOL];
    __shared__ double Bbs[NGP * 24];
    for (int i = threadIdx.x; i < NGP * NSTR * NCOL; i += blockDim.x)
        Bs[i] = a.B[i];
    constexpr bool STRUCT = C == 3; // mechanics: the 72-term kinematics when a.Bb is set
    const bool     bb     = STRUCT && a.Bb;
    if (bb)
        for (int i = threadIdx.x; i < NGP * 24; i += blockDim.x)
            Bbs[i] = a.Bb[i];
    __syncthreads();
    const int       nx = a.g.nx, ny = a.g.ny, nz = a.g.nz;
    const long long N  = (long long)nx * ny * nz;
    const long long T  = (N * NGP + 31) / 32 * 32;
    const int       gp = (int)(threadIdx.x % NGP);
    const double   *Bg = Bs + gp * NSTR * NCOL;
    const double   *Bb = Bbs + gp * 24;
    double          se[MODE == ELEM_AVERAGES ? NSTR : 1], ss[MODE == ELEM_AVERAGES ? NSTR : 1], cnt = 0.0;
    if constexpr (MODE == ELEM_AVERAGES) {
#pragma unroll
        for (int i = 0; i < NSTR; ++i)
            se[i] = ss[i] = 0.0;
    }
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < T; t += (long long)gridDim.x * blockDim.x) {
        const long long el    = t / NGP;
        const bool      valid = el < N;
        const int       ph    = valid ? a.ms[el] : 0;
        double          e[NE], sig[NE];
        {
            double ue[NCOL];
            if (valid) {
                long long idx[8];
                elem_nodes(nx, ny, nz, el, idx);
#pragma unroll
                for (int c = 0; c < C; ++c) {
                    const double u0 = MODE == ELEM_RESIDUAL ? a.u[c * N + idx[0]] : 0.0;
#pragma unroll
                    for (int q = 0; q < 8; ++q)
                        ue[q * C + c] = a.u[c * N + idx[q]] - u0;
                }
            } else {
#pragma unroll
                for (int k = 0; k < NCOL; ++k)
                    ue[k] = 0.0;
            }
            if constexpr (STRUCT) {
                if (bb) {
                    if constexpr (LARGE)
                        defgrad_basic_b(Bb, ue, a.g0, e);
                    else
                        strain_basic_b(Bb, ue, a.g0, e);
                } else {
#pragma unroll
                    for (int i = 0; i < NSTR; ++i) {
                        double acc = 0.0;
#pragma unroll
                        for (int k = 0; k < NCOL; ++k)
                            acc += Bg[i * NCOL + k] * ue[k];
                        e[i] = acc + a.g0[i];
                    }
                }
            } else {
#pragma unroll
                for (int i = 0; i < NSTR; ++i) {
                    double acc = 0.0;
#pragma unroll
                    for (int k = 0; k < NCOL; ++k)
                        acc += Bg[i * NCOL + k] * ue[k];
                    e[i] = acc + a.g0[i];
                }
            }
        }
        const int law = valid ? a.law[ph] : -1;
        double    flag = 0.0; // elements outside a PseudoPlastic model keep flag 0 (PseudoPlastic.h:37-40)
        if constexpr (LARGE) {
            large_strain_sigma(law, a.prm + ph * kPrm, e, sig);
        } else if (C == 3 && (law == FANSGPU_LAW_PSEUDO_LINEAR || law == FANSGPU_LAW_PSEUDO_NONLINEAR)) {
            flag = pseudo_sigma(law, a.prm + ph * kPrm, e, sig);
        } else if (C == 3 && (law == FANSGPU_LAW_J2VISCO_LINEAR || law == FANSGPU_LAW_J2VISCO_NONLINEAR)) {
            double          ep_in[6], pbt[6], nv[6];
            const long long base = (long long)gp * N + el;
#pragma unroll
            for (int i = 0; i < 6; ++i) {
                ep_in[i] = a.ep_t[(long long)i * NGP * N + base];
                pbt[i]   = a.pb_t[(long long)i * NGP * N + base];
            }
            const double gam = j2visco_sigma(law == FANSGPU_LAW_J2VISCO_NONLINEAR, a.prm + ph * kPrm, e, ep_in,
                                             a.q_t[base], pbt, sig, nv);
            if (a.ep) {
#pragma unroll
                for (int i = 0; i < 6; ++i) {
                    a.ep[(long long)i * NGP * N + base] = ep_in[i] + gam * nv[i];
                    a.pb[(long long)i * NGP * N + base] -= gam * nv[i];
                }
                a.q[base] += gam * sqrt(2.0 / 3.0);
            }
        } else if (C == 3 && law == FANSGPU_LAW_J2_LINEAR) {
            double          ep_in[6], ep_out[6], q_out;
            const long long base = (long long)gp * N + el;
#pragma unroll
            for (int i = 0; i < 6; ++i)
                ep_in[i] = a.ep_t[(long long)i * NGP * N + base];
            const double *pj = a.prm + ph * kPrm;
            j2_sigma(pj, a.sy ? a.sy[el] : pj[2], e, ep_in, a.q_t[base], sig, ep_out, q_out);
            if (a.ep) {
#pragma unroll
                for (int i = 0; i < 6; ++i)
                    a.ep[(long long)i * NGP * N + base] = ep_out[i];
                a.q[base] = q_out;
            }
        } else {
            const double *Cm = a.Cph + ph * NSTR * NSTR;
#pragma unroll
            for (int i = 0; i < NSTR; ++i) {
                double acc = 0.0;
#pragma unroll
                for (int k = 0; k < NSTR; ++k)
                    acc += Cm[i * NSTR + k] * e[k];
                sig[i] = acc;
            }
        }
        if (valid && a.scale) {
            const double sc = a.scale[el];
#pragma unroll
            for (int i = 0; i < NSTR; ++i)
                sig[i] *= sc;
        }
        if constexpr (MODE == ELEM_RESIDUAL) {
            double v[NCOL];
            bool   done = false;
            if constexpr (STRUCT) {
                if (bb) {
                    if constexpr (LARGE)
                        bt_piola_basic_b(Bb, sig, v);
                    else
                        bt_sigma_basic_b(Bb, sig, v);
                    done = true;
                }
            }
            if (!done)
#pragma unroll
                for (int k = 0; k < NCOL; ++k) {
                    double acc = 0.0;
#pragma unroll
                    for (int i = 0; i < NSTR; ++i)
                        acc += Bg[i * NCOL + k] * sig[i];
                    v[k] = acc;
                }
            // reduce-scatter over the NGP lanes of the element
            int kb = 0;
#pragma unroll
            for (int m = NGP / 2, cntv = NCOL; m >= 1; m /= 2, cntv /= 2) {
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
            if (valid) {
                const double sc = a.ve / NGP;
#pragma unroll
                for (int j = 0; j < NCOL / NGP; ++j)
                    a.rows[(long long)(kb + j) * N + el] = v[j] * sc;
            }
        } else {
            if (valid && a.strain_gp)
#pragma unroll
                for (int i = 0; i < NSTR; ++i)
                    a.strain_gp[(el * NGP + gp) * NSTR + i] = e[i];
            if (valid && a.stress_gp)
#pragma unroll
                for (int i = 0; i < NSTR; ++i)
                    a.stress_gp[(el * NGP + gp) * NSTR + i] = sig[i];
#pragma unroll
            for (int m = NGP / 2; m >= 1; m /= 2) {
#pragma unroll
                for (int i = 0; i < NSTR; ++i) {
                    e[i] += __shfl_xor_sync(0xffffffffu, e[i], m);
                    sig[i] += __shfl_xor_sync(0xffffffffu, sig[i], m);
                }
                flag += __shfl_xor_sync(0xffffffffu, flag, m);
            }
            if (valid && gp == 0 && a.flag)
                a.flag[el] = flag / NGP;
            if (valid && gp == 0) {
#pragma unroll
                for (int i = 0; i < NSTR; ++i) {
                    e[i] /= NGP;
                    sig[i] /= NGP;
                }
                if (a.strain)
#pragma unroll
                    for (int i = 0; i < NSTR; ++i)
                        a.strain[el * NSTR + i] = e[i];
                if (a.stress)
#pragma unroll
                    for (int i = 0; i < NSTR; ++i)
                        a.stress[el * NSTR + i] = sig[i];
                if (a.phase_filter < 0 || a.phase_filter == ph) {
#pragma unroll
                    for (int i = 0; i < NSTR; ++i) {
                        se[i] += e[i];
                        ss[i] += sig[i];
                    }
                    cnt += 1.0;
                }
            }
        }
    }
    if constexpr (MODE == ELEM_AVERAGES) {
        __shared__ double red_smem[32 * (2 * NSTR + 1)];
        double            v[2 * NSTR + 1];
        int               ops[2 * NSTR + 1];
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
}

// r[c][node] = sum_p rows[p*C + c][element whose local node p is this node]
template <int C>
__global__ void __launch_bounds__(256) k_gather(const double *__restrict__ rows, double *__restrict__ r, Grid3 g)
{
    const long long N = g.N();
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < N; n += (long long)gridDim.x * blockDim.x) {
        const int z = (int)(n % g.nz), y = (int)((n / g.nz) % g.ny), x = (int)(n / ((long long)g.nz * g.ny));
        double    acc[C];
#pragma unroll
        for (int c = 0; c < C; ++c)
            acc[c] = 0.0;
#pragma unroll
        for (int p = 0; p < 8; ++p) {
            const int ex = (p & 1) ? (x == 0 ? g.nx - 1 : x - 1) : x;
            const int ey = (p & 2) ? (y == 0 ? g.ny - 1 : y - 1) : y;
            const int ez = (p & 4) ? (z == 0 ? g.nz - 1 : z - 1) : z;
            const long long e = ((long long)ex * g.ny + ey) * g.nz + ez;
#pragma unroll
            for (int c = 0; c < C; ++c)
                acc[c] += rows[(long long)(p * C + c) * N + e];
        }
#pragma unroll
        for (int c = 0; c < C; ++c)
            r[c * N + n] = acc[c];
    }
}

// <a, b> in FP64 -> *out (deterministic grid reduction)
__global__ void __launch_bounds__(256) k_dot(const double *__restrict__ a, const double *__restrict__ b, long long n,
                                             double *out, GridRed red, int site)
{
    __shared__ double red_smem[32];
    double            s = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        s += a[i] * b[i];
    double    v[1]   = {s};
    const int ops[1] = {RED_SUM};
    block_reduce<1>(v, ops, red_smem);
    if (grid_partial_commit<1>(v, red.partials, red.counter + site, gridDim.x)) {
        grid_final<1>(v, ops, red.partials, gridDim.x, red_smem);
        if (threadIdx.x == 0)
            *out = v[0];
    }
}

// d = s + beta*d (beta from scal), the direction update of solverCG.h:94
__global__ void k_direction(double *__restrict__ d, const double *__restrict__ s, long long n, const CgScalars *scal)
{
    const double beta = scal->beta;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        d[i] = s[i] + beta * d[i];
}

__global__ void k_ivar_mean(const double *__restrict__ ep_t, const double *__restrict__ q_t, int ngp, long long N,
                            double *__restrict__ ep_out, double *__restrict__ q_out)
{
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < N; e += (long long)gridDim.x * blockDim.x) {
        if (ep_out)
            for (int i = 0; i < 6; ++i) {
                double s = 0.0;
                for (int gp = 0; gp < ngp; ++gp)
                    s += ep_t[((long long)i * ngp + gp) * N + e];
                ep_out[e * 6 + i] = s / ngp;
            }
        if (q_out) {
            double s = 0.0;
            for (int gp = 0; gp < ngp; ++gp)
                s += q_t[(long long)gp * N + e];
            q_out[e] = s / ngp;
        }
    }
}

// Gauss-point values of the committed variables in element-major order:
// ep_out[(e*ngp + gp)*6 + i], q_out[e*ngp + gp] (J2PlasticityNew.h:179-188).
__global__ void k_ivar_gp(const double *__restrict__ ep_t, const double *__restrict__ q_t, int ngp, long long N,
                          double *__restrict__ ep_out, double *__restrict__ q_out)
{
    const long long total = N * ngp;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
        const long long e  = t / ngp;
        const int       gp = (int)(t % ngp);
        if (ep_out)
            for (int i = 0; i < 6; ++i)
                ep_out[t * 6 + i] = ep_t[((long long)i * ngp + gp) * N + e];
        if (q_out)
            q_out[t] = q_t[(long long)gp * N + e];
    }
}

// one thread per element; the Gauss-point strains of the n solutions in registers
template <int C, int NGP, int NMAX>
__global__ void __launch_bounds__(128) k_sensitivity(SensArgs a)
{
    constexpr int NSTR = C == 1 ? 3 : 6, NCOL = 8 * C;
    __shared__ double Bs[NGP * NSTR * NCOL];
    for (int i = threadIdx.x; i < NGP * NSTR * NCOL; i += blockDim.x)
        Bs[i] = a.B[i];
    __syncthreads();
    const int       nx = a.g.nx, ny = a.g.ny, nz = a.g.nz;
    const long long N  = (long long)nx * ny * nz;
    for (long long el = blockIdx.x * (long long)blockDim.x + threadIdx.x; el < N; el += (long long)gridDim.x * blockDim.x) {
        long long idx[8];
        elem_nodes(nx, ny, nz, el, idx);
        const double *Cm  = a.Cph + a.ms[el] * NSTR * NSTR;
        double        acc = 0.0;
        for (int gp = 0; gp < NGP; ++gp) {
            const double *Bg = Bs + gp * NSTR * NCOL;
            double        eps[NMAX][NSTR];
            for (int k = 0; k < a.n; ++k) {
                const double *u = a.u + (long long)k * C * N;
                double        ue[NCOL];
#pragma unroll
                for (int c = 0; c < C; ++c) {
                    const double u0 = u[c * N + idx[0]];
#pragma unroll
                    for (int q = 0; q < 8; ++q)
                        ue[q * C + c] = u[c * N + idx[q]] - u0;
                }
#pragma unroll
                for (int i = 0; i < NSTR; ++i) {
                    double s = a.g0[k * NSTR + i];
#pragma unroll
                    for (int q = 0; q < NCOL; ++q)
                        s += Bg[i * NCOL + q] * ue[q];
                    eps[k][i] = s;
                }
            }
            for (int j = 0; j < a.n; ++j) {
                double ce[NSTR];
#pragma unroll
                for (int i = 0; i < NSTR; ++i) {
                    double s = 0.0;
#pragma unroll
                    for (int k = 0; k < NSTR; ++k)
                        s += Cm[i * NSTR + k] * eps[j][k];
                    ce[i] = s;
                }
                for (int i = 0; i < a.n; ++i) {
                    double s = 0.0;
#pragma unroll
                    for (int k = 0; k < NSTR; ++k)
                        s += eps[i][k] * ce[k];
                    acc += a.W[i * a.n + j] * s;
                }
            }
        }
        a.grad[el] = acc / (NGP * (double)N);
    }
}

__global__ void k_set_alpha(CgScalars *scal)
{
    scal->alpha = scal->delta / scal->dAd;
}

} // namespace

cudaError_t launch_sensitivity(const SensArgs &a, cudaStream_t st)
{
    const int nb = grid_blocks_for(a.g.N());
    if (a.n < 1 || a.n > 6)
        return cudaErrorInvalidValue;
    if (a.C == 1)
        a.ngp == 8 ? k_sensitivity<1, 8, 6><<<nb, 128, 0, st>>>(a) : k_sensitivity<1, 1, 6><<<nb, 128, 0, st>>>(a);
    else
        a.ngp == 8 ? k_sensitivity<3, 8, 6><<<nb, 128, 0, st>>>(a) : k_sensitivity<3, 1, 6><<<nb, 128, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_set_alpha(CgScalars *scal, cudaStream_t st)
{
    k_set_alpha<<<1, 1, 0, st>>>(scal);
    return cudaGetLastError();
}

cudaError_t launch_ivar_gp(const double *ep_t, const double *q_t, int ngp, long long N, double *ep_out, double *q_out,
                           cudaStream_t st)
{
    k_ivar_gp<<<grid_blocks_for(N * ngp), 256, 0, st>>>(ep_t, q_t, ngp, N, ep_out, q_out);
    return cudaGetLastError();
}

cudaError_t launch_ivar_mean(const double *ep_t, const double *q_t, int ngp, long long N, double *ep_out,
                             double *q_out, cudaStream_t st)
{
    k_ivar_mean<<<grid_blocks_for(N), 256, 0, st>>>(ep_t, q_t, ngp, N, ep_out, q_out);
    return cudaGetLastError();
}

cudaError_t launch_element(const ElementArgs &a, cudaStream_t st)
{
    // one (element, Gauss point) per thread, at most 152*16 blocks (the reduction partials are sized for that)
    const long long want = (a.g.N() * a.ngp + kElThreads - 1) / kElThreads;
    const int       nb   = (int)(want < 152 * 16 ? (want < 1 ? 1 : want) : 152 * 16);
    const bool      res  = a.mode == ELEM_RESIDUAL;
#define FANSGPU_EL(C_, G_)                                                                                   \
    (res ? (k_element<C_, G_, ELEM_RESIDUAL><<<nb, kElThreads, 0, st>>>(a), 0)                                 \
         : (k_element<C_, G_, ELEM_AVERAGES><<<nb, kElThreads, 0, st>>>(a), 0))
#define FANSGPU_EL_LARGE(G_)                                                                                 \
    (res ? (k_element<3, G_, ELEM_RESIDUAL, true><<<nb, kElThreads, 0, st>>>(a), 0)                            \
         : (k_element<3, G_, ELEM_AVERAGES, true><<<nb, kElThreads, 0, st>>>(a), 0))
    if (a.nstr == 9)
        a.ngp == 8 ? FANSGPU_EL_LARGE(8) : FANSGPU_EL_LARGE(1);
    else if (a.C == 1)
        a.ngp == 8 ? FANSGPU_EL(1, 8) : FANSGPU_EL(1, 1);
    else
        a.ngp == 8 ? FANSGPU_EL(3, 8) : FANSGPU_EL(3, 1);
#undef FANSGPU_EL
#undef FANSGPU_EL_LARGE
    return cudaGetLastError();
}

cudaError_t launch_gather(const double *rows, double *r, const Grid3 &g, int C, cudaStream_t st)
{
    if (C == 1)
        k_gather<1><<<grid_blocks_for(g.N()), 256, 0, st>>>(rows, r, g);
    else
        k_gather<3><<<grid_blocks_for(g.N()), 256, 0, st>>>(rows, r, g);
    return cudaGetLastError();
}

cudaError_t launch_dot(const double *a, const double *b, long long n, double *out, GridRed red, int site,
                       cudaStream_t st)
{
    k_dot<<<grid_blocks_for(n), 256, 0, st>>>(a, b, n, out, red, site);
    return cudaGetLastError();
}

cudaError_t launch_direction(double *d, const double *s, long long n, const CgScalars *scal, cudaStream_t st)
{
    k_direction<<<grid_blocks_for(n), 256, 0, st>>>(d, s, n, scal);
    return cudaGetLastError();
}

} // namespace fansgpu
