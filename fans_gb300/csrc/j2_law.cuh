// j2_law.cuh -- the J2PlasticityNew return map (J2PlasticityNew.h:43-108) at one
// Gauss point and its vector-Jacobian product, shared by the element kernel and
// the yield-stress adjoint.
#pragma once
#include "fans_common.cuh"

namespace fansgpu {

// Node indices of element e (x-major, z fastest) in the element's local node
// order p = bx + 2 by + 4 bz (solver.h:318-385), periodic in every direction.
__device__ __forceinline__ void elem_nodes(int nx, int ny, int nz, long long e, long long idx[8])
{
    const int z = (int)(e % nz), y = (int)((e / nz) % ny), x = (int)(e / ((long long)nz * ny));
    const int x1 = x + 1 == nx ? 0 : x + 1, y1 = y + 1 == ny ? 0 : y + 1, z1 = z + 1 == nz ? 0 : z + 1;
    idx[0] = ((long long)x * ny + y) * nz + z;
    idx[1] = ((long long)x1 * ny + y) * nz + z;
    idx[2] = ((long long)x * ny + y1) * nz + z;
    idx[3] = ((long long)x1 * ny + y1) * nz + z;
    idx[4] = ((long long)x * ny + y) * nz + z1;
    idx[5] = ((long long)x1 * ny + y) * nz + z1;
    idx[6] = ((long long)x * ny + y1) * nz + z1;
    idx[7] = ((long long)x1 * ny + y1) * nz + z1;
}

// Small-strain element kinematics from the basic B at a Gauss point,
// b[j * 8 + q] = dN_q/dx_j (Compute_basic_B, matmodel.h:158-188).  The Mandel
// B (matmodel.h:284-304) has 72 nonzeros of its 6 x 24: the displacement
// gradient G_ij = sum_q b_j[q] u_i[q] (72 FMAs) gives
//   eps = (G00, G11, G22, s(G01 + G10), s(G02 + G20), s(G12 + G21)) + off,
// s = sqrt(1/2), and B^T sig = sum_j b_j[q] T_ij with T the stress tensor
// (T01 = s sig3, T02 = s sig4, T12 = s sig5).  u_e is in the element's node
// order, ue[3 q + c].
__device__ __forceinline__ void strain_basic_b(const double *b, const double (&ue)[24], const double *off,
                                               double (&e)[6])
{
    double G[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            double acc = 0.0;
#pragma unroll
            for (int q = 0; q < 8; ++q)
                acc += b[j * 8 + q] * ue[3 * q + i];
            G[i][j] = acc;
        }
    const double s = 7.071067811865476e-01;
    e[0]           = G[0][0];
    e[1]           = G[1][1];
    e[2]           = G[2][2];
    e[3]           = s * (G[0][1] + G[1][0]);
    e[4]           = s * (G[0][2] + G[2][0]);
    e[5]           = s * (G[1][2] + G[2][1]);
    if (off)
#pragma unroll
        for (int i = 0; i < 6; ++i)
            e[i] += off[i];
}

__device__ __forceinline__ void bt_sigma_basic_b(const double *b, const double (&sig)[6], double (&v)[24])
{
    const double s    = 7.071067811865476e-01;
    const double T[3][3] = {{sig[0], s * sig[3], s * sig[4]}, {s * sig[3], sig[1], s * sig[5]},
                            {s * sig[4], s * sig[5], sig[2]}};
#pragma unroll
    for (int q = 0; q < 8; ++q)
#pragma unroll
        for (int i = 0; i < 3; ++i)
            v[3 * q + i] = b[q] * T[i][0] + b[8 + q] * T[i][1] + b[16 + q] * T[i][2];
}

// Large strain: the deformation-gradient B_F (LargeStrainMechModel.h:209-225,
// row 3i + J, column 3q + i = dN_q/dX_J) has 72 nonzeros of its 9 x 24:
// F_iJ = sum_q b_J[q] u_i[q] + off_iJ and (B_F^T P)_{3q+i} = sum_J b_J[q] P_iJ.
__device__ __forceinline__ void defgrad_basic_b(const double *b, const double (&ue)[24], const double *off,
                                                double (&F)[9])
{
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int J = 0; J < 3; ++J) {
            double acc = 0.0;
#pragma unroll
            for (int q = 0; q < 8; ++q)
                acc += b[J * 8 + q] * ue[3 * q + i];
            F[3 * i + J] = acc + off[3 * i + J];
        }
}

__device__ __forceinline__ void bt_piola_basic_b(const double *b, const double (&P)[9], double (&v)[24])
{
#pragma unroll
    for (int q = 0; q < 8; ++q)
#pragma unroll
        for (int i = 0; i < 3; ++i)
            v[3 * q + i] = b[q] * P[3 * i] + b[8 + q] * P[3 * i + 1] + b[16 + q] * P[3 * i + 2];
}

// J2PlasticityNew::get_sigma (J2PlasticityNew.h:43-108), one Gauss point, Mandel
// vectors.  prm = {K, G, sigma_y, h}; sy0 is the initial yield stress in use
// (prm[2], or the voxel's own value when a per-voxel field is set).
__device__ __forceinline__ void j2_sigma(const double *prm, double sy0, const double (&e)[6], const double (&ep_in)[6],
                                         double q_in, double (&sig)[6], double (&ep_out)[6], double &q_out)
{
    const double K = prm[0], G = prm[1], h = prm[3];
    const double c23 = sqrt(2.0 / 3.0);
    double       s[6], st[6];
#pragma unroll
    for (int i = 0; i < 6; ++i)
        s[i] = 2.0 * G * (e[i] - ep_in[i]);
    const double lam = K - 2.0 / 3.0 * G;
    const double tr  = e[0] + e[1] + e[2];
#pragma unroll
    for (int i = 0; i < 3; ++i)
        s[i] += lam * tr;
#pragma unroll
    for (int i = 0; i < 6; ++i)
        st[i] = s[i];
    const double mean = (s[0] + s[1] + s[2]) / 3.0;
#pragma unroll
    for (int i = 0; i < 3; ++i)
        st[i] -= mean;
    double n2 = 0.0;
#pragma unroll
    for (int i = 0; i < 6; ++i)
        n2 += st[i] * st[i];
    const double s_t    = sqrt(n2);
    const double sy     = sy0 + q_in * h;
    const double phi    = s_t - c23 * sy;
    double       dgamma = phi / (2.0 * G + 2.0 / 3.0 * h);
    if (dgamma < 0.0)
        dgamma = 0.0;
    const bool on = s_t > 1e-12;
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        ep_out[i] = on ? ep_in[i] + dgamma * st[i] / s_t : ep_in[i];
        sig[i]    = on ? s[i] - dgamma * 2.0 * G * st[i] / s_t : s[i];
    }
    q_out = q_in + c23 * dgamma;
}

// Vector-Jacobian product of j2_sigma: for the scalar
//   J = tau . sig + m_ep . ep_out + m_q q_out
// returns ge = dJ/de, gep = dJ/dep_in, gq = dJ/dq_in and gsy = dJ/dsy0.
// With the trial deviator s_tr = 2G dev(e - ep_in), n = s_tr/|s_tr|,
// a = 2G + 2h/3 and dgamma = (|s_tr| - sqrt(2/3)(sy0 + h q_in))/a > 0 (plastic):
//   kappa = -2G tau.n + m_ep.n + sqrt(2/3) m_q        (coefficient of d dgamma)
//   v     = dgamma (m_ep - 2G tau)                     (coefficient of d n)
//   w     = (kappa/a) n + (v - (v.n) n)/|s_tr|         (coefficient of d s_tr)
//   ge  = 2G tau + lambda tr(tau) m + 2G dev(w),  gep = m_ep - 2G tau - 2G dev(w),
//   gq  = m_q - sqrt(2/3) h kappa/a,              gsy = -sqrt(2/3) kappa/a;
// in the elastic branch (dgamma = 0, as j2_sigma clamps it) the w, kappa terms
// vanish.  With m_ep = m_q = 0, ge is the consistent tangent applied to tau
// (symmetric, so this is also K_alg tau).
__device__ __forceinline__ void j2_vjp(const double *prm, double sy0, const double (&e)[6], const double (&ep_in)[6],
                                       double q_in, const double (&tau)[6], const double (&mep)[6], double mq,
                                       double (&ge)[6], double (&gep)[6], double &gq, double &gsy)
{
    const double K = prm[0], G = prm[1], h = prm[3];
    const double c23 = sqrt(2.0 / 3.0);
    const double lam = K - 2.0 / 3.0 * G;
    double       st[6]; // the trial deviator, formed as j2_sigma forms it (same branch decision)
#pragma unroll
    for (int i = 0; i < 6; ++i)
        st[i] = 2.0 * G * (e[i] - ep_in[i]);
    const double tre = e[0] + e[1] + e[2];
#pragma unroll
    for (int i = 0; i < 3; ++i)
        st[i] += lam * tre;
    const double mean = (st[0] + st[1] + st[2]) / 3.0;
#pragma unroll
    for (int i = 0; i < 3; ++i)
        st[i] -= mean;
    double n2 = 0.0;
#pragma unroll
    for (int i = 0; i < 6; ++i)
        n2 += st[i] * st[i];
    const double s_t = sqrt(n2);
    const double a   = 2.0 * G + 2.0 / 3.0 * h;
    const double phi = s_t - c23 * (sy0 + q_in * h);
    const double trt = tau[0] + tau[1] + tau[2];
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        ge[i]  = 2.0 * G * tau[i] + (i < 3 ? lam * trt : 0.0);
        gep[i] = mep[i] - 2.0 * G * tau[i];
    }
    gq  = mq;
    gsy = 0.0;
    if (phi > 0.0 && s_t > 1e-12) {
        const double dgamma = phi / a, inv = 1.0 / s_t;
        double       n[6], v[6], tn = 0.0, mn = 0.0, vn = 0.0;
#pragma unroll
        for (int i = 0; i < 6; ++i) {
            n[i] = st[i] * inv;
            v[i] = dgamma * (mep[i] - 2.0 * G * tau[i]);
            tn += tau[i] * n[i];
            mn += mep[i] * n[i];
            vn += v[i] * n[i];
        }
        const double ka = (-2.0 * G * tn + mn + c23 * mq) / a;
        double       w[6];
#pragma unroll
        for (int i = 0; i < 6; ++i)
            w[i] = ka * n[i] + (v[i] - vn * n[i]) * inv;
        const double wm = (w[0] + w[1] + w[2]) / 3.0;
#pragma unroll
        for (int i = 0; i < 6; ++i) {
            const double pw = 2.0 * G * (w[i] - (i < 3 ? wm : 0.0));
            ge[i] += pw;
            gep[i] -= pw;
        }
        gq -= c23 * h * ka;
        gsy = -c23 * ka;
    }
}

} // namespace fansgpu
