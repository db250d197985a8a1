// fe_host.hpp -- host-side finite-element setup of the FANS solve path:
// Gauss-point B matrices, per-phase constitutive matrices, element stiffness
// and the reference element stiffness.  One-off per context, in FP64.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace fansgpu {
namespace fe {

// Trilinear shape-function gradients at reference point (x,y,z), 3 x 8
// (Matmodel::Compute_basic_B, matmodel.h:158-188).  Node p = bx + 2 by + 4 bz.
inline void basic_B(double x, double y, double z, const double le[3], double out[3][8])
{
    for (int p = 0; p < 8; ++p) {
        const int    bx = p & 1, by = (p >> 1) & 1, bz = (p >> 2) & 1;
        const double wx = bx ? x : 1.0 - x, wy = by ? y : 1.0 - y, wz = bz ? z : 1.0 - z;
        const double sx = bx ? 1.0 : -1.0, sy = by ? 1.0 : -1.0, sz = bz ? 1.0 : -1.0;
        out[0][p] = sx * wy * wz / le[0];
        out[1][p] = wx * sy * wz / le[1];
        out[2][p] = wx * wy * sz / le[2];
    }
}

// Model B: thermal 3 x 8 (matmodel.h:267-270), small-strain Mandel 6 x 24
// with shear rows scaled by sqrt(1/2) (matmodel.h:284-304), or (nstr = 9) the
// large-strain deformation-gradient B_F: row 3i + J, column 3q + i holds
// dN_q/dX_J (LargeStrainMechModel.h:209-225).
inline void model_B(int C, double x, double y, double z, const double le[3], double *out, int nstr = 0)
{
    double b[3][8];
    basic_B(x, y, z, le, b);
    if (nstr == 9) {
        std::memset(out, 0, sizeof(double) * 9 * 24);
        for (int i = 0; i < 3; ++i)
            for (int J = 0; J < 3; ++J)
                for (int q = 0; q < 8; ++q)
                    out[(3 * i + J) * 24 + 3 * q + i] = b[J][q];
        return;
    }
    if (C == 1) {
        for (int i = 0; i < 3; ++i)
            for (int q = 0; q < 8; ++q)
                out[i * 8 + q] = b[i][q];
        return;
    }
    const double s = 7.071067811865476e-01;
    std::memset(out, 0, sizeof(double) * 6 * 24);
    for (int q = 0; q < 8; ++q) {
        out[0 * 24 + 3 * q + 0] = b[0][q];
        out[1 * 24 + 3 * q + 1] = b[1][q];
        out[2 * 24 + 3 * q + 2] = b[2][q];
        out[3 * 24 + 3 * q + 0] = s * b[1][q];
        out[3 * 24 + 3 * q + 1] = s * b[0][q];
        out[4 * 24 + 3 * q + 0] = s * b[2][q];
        out[4 * 24 + 3 * q + 2] = s * b[0][q];
        out[5 * 24 + 3 * q + 1] = s * b[2][q];
        out[5 * 24 + 3 * q + 2] = s * b[1][q];
    }
}

// Gauss-point B matrices (Construct_B, matmodel.h:104-155): HEX8 and BBAR use
// the 2x2x2 rule at 0.5 +- sqrt(3)/6, HEX8R the centre; BBAR replaces the
// volumetric part of the normal rows with its centre value (small strain only).
inline int gauss_B(int fe_type, int C, const double le[3], std::vector<double> &B, int nstr_in = 0)
{
    const int nstr = nstr_in ? nstr_in : (C == 1 ? 3 : 6), ncol = 8 * C;
    if (fe_type == 1) {
        B.assign(nstr * ncol, 0.0);
        model_B(C, 0.5, 0.5, 0.5, le, B.data(), nstr);
        return 1;
    }
    const double p = 0.5 + std::sqrt(3.) / 6., m = 0.5 - std::sqrt(3.) / 6.;
    const double xi[8][3] = {{m, m, m}, {p, m, m}, {m, p, m}, {p, p, m}, {m, m, p}, {p, m, p}, {m, p, p}, {p, p, p}};
    B.assign(8 * nstr * ncol, 0.0);
    for (int g = 0; g < 8; ++g)
        model_B(C, xi[g][0], xi[g][1], xi[g][2], le, B.data() + g * nstr * ncol, nstr);
    if (fe_type == 2 && nstr > 3) {
        std::vector<double> Bv(nstr * ncol);
        model_B(C, 0.5, 0.5, 0.5, le, Bv.data(), nstr);
        for (int g = 0; g < 8; ++g) {
            double *Bg = B.data() + g * nstr * ncol;
            for (int col = 0; col < ncol; ++col) {
                const double vf = (Bg[0 * ncol + col] + Bg[1 * ncol + col] + Bg[2 * ncol + col]) / 3.0;
                const double vb = (Bv[0 * ncol + col] + Bv[1 * ncol + col] + Bv[2 * ncol + col]) / 3.0;
                for (int row = 0; row < 3; ++row)
                    Bg[row * ncol + col] += vb - vf;
            }
        }
    }
    return 8;
}

// Basic B (dN_q/dx_j, matmodel.h:158-188) at the Gauss points of HEX8 (8, in
// gauss_B's order) or HEX8R (1, the centre): ngp x 3 x 8.
inline std::vector<double> gauss_basic_B(int fe_type, const double le[3])
{
    const double p = 0.5 + std::sqrt(3.) / 6., m = 0.5 - std::sqrt(3.) / 6.;
    const double xi[8][3] = {{m, m, m}, {p, m, m}, {m, p, m}, {p, p, m}, {m, m, p}, {p, m, p}, {m, p, p}, {p, p, p}};
    const int    ngp      = fe_type == 1 ? 1 : 8;
    std::vector<double> out(ngp * 24);
    for (int g = 0; g < ngp; ++g) {
        double b[3][8];
        if (fe_type == 1)
            basic_B(0.5, 0.5, 0.5, le, b);
        else
            basic_B(xi[g][0], xi[g][1], xi[g][2], le, b);
        for (int j = 0; j < 3; ++j)
            for (int q = 0; q < 8; ++q)
                out[g * 24 + j * 8 + q] = b[j][q];
    }
    return out;
}

// Constitutive matrix of a linear law (nstr x nstr, row-major).
// law 0 thermal iso: kappa I (LinearThermal.h:186);
// law 1 elastic iso: lambda on the normal 3x3 block + 2 mu I (LinearElastic.h:28-35);
// laws 2, 5-8 (J2, PseudoPlastic, J2ViscoPlastic; their elastic part, for the reference/tangent): as law 1;
// law 3/4 triclinic: the given matrix (LinearThermal.h:250-254, LinearElastic.h:114-129).
inline bool law_C(int law, const std::vector<double> &prm, int nstr, double *C)
{
    std::memset(C, 0, sizeof(double) * nstr * nstr);
    if (law == 0 && nstr == 3) {
        for (int i = 0; i < 3; ++i)
            C[i * 3 + i] = prm[0];
        return true;
    }
    if ((law == 1 || law == 2 || law == 5 || law == 6 || law == 7 || law == 8) && nstr == 6) {
        const double lam = prm[0] - (2.0 / 3.0) * prm[1];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j)
                C[i * 6 + j] = lam;
        for (int i = 0; i < 6; ++i)
            C[i * 6 + i] += 2.0 * prm[1];
        return true;
    }
    if ((law == 9 || law == 10) && nstr == 9) {
        // dP/dF at F = I of SaintVenantKirchhoff / CompressibleNeoHookean as
        // LargeStrainMechModel::compute_spatial_tangent builds it (LargeStrainMechModel.h:96-170,
        // S = 0): lambda d_iJ d_kL + mu (d_ik d_JL + d_iL d_Jk), halved where k != L
        // because that loop takes each symmetric pair (P, Q) once.  Row 3i + J, column 3k + L.
        const double mu = prm[1], lam = prm[0] - (2.0 / 3.0) * mu;
        for (int i = 0; i < 3; ++i)
            for (int J = 0; J < 3; ++J)
                for (int k = 0; k < 3; ++k)
                    for (int L = 0; L < 3; ++L)
                        C[(3 * i + J) * 9 + 3 * k + L] =
                            (k == L ? 1.0 : 0.5) *
                            (lam * (i == J) * (k == L) + mu * ((i == k) * (J == L) + (i == L) * (J == k)));
        return true;
    }
    if ((law == 3 && nstr == 3) || (law == 4 && nstr == 6)) {
        if ((int)prm.size() < nstr * nstr)
            return false;
        for (int i = 0; i < nstr * nstr; ++i)
            C[i] = prm[i];
        return true;
    }
    return false;
}

// K = sum_gp B^T C B v_e / n_gp, node-major 8C x 8C (LinearElastic.h:37-39).
inline void element_stiffness(int C, int ngp, const std::vector<double> &B, const double *Cm, double ve,
                              std::vector<double> &K)
{
    const int ncol = 8 * C, nstr = (int)(B.size() / ((size_t)ngp * ncol));
    K.assign(ncol * ncol, 0.0);
    std::vector<double> CB(nstr * ncol);
    for (int g = 0; g < ngp; ++g) {
        const double *Bg = B.data() + g * nstr * ncol;
        for (int i = 0; i < nstr; ++i)
            for (int j = 0; j < ncol; ++j) {
                double acc = 0.0;
                for (int k = 0; k < nstr; ++k)
                    acc += Cm[i * nstr + k] * Bg[k * ncol + j];
                CB[i * ncol + j] = acc;
            }
        for (int i = 0; i < ncol; ++i)
            for (int j = 0; j < ncol; ++j) {
                double acc = 0.0;
                for (int k = 0; k < nstr; ++k)
                    acc += Bg[k * ncol + i] * CB[k * ncol + j];
                K[i * ncol + j] += acc * ve / ngp;
            }
    }
}

// f = sum_gp B^T C g0 v_e / n_gp (8C): the g0 part of element_residual (matmodel.h:194-199).
inline void element_force(int C, int ngp, const std::vector<double> &B, const double *Cm, const double *g0, double ve,
                          double *f)
{
    const int ncol = 8 * C, nstr = (int)(B.size() / ((size_t)ngp * ncol));
    double    sig[9];
    for (int i = 0; i < nstr; ++i) {
        double acc = 0.0;
        for (int k = 0; k < nstr; ++k)
            acc += Cm[i * nstr + k] * g0[k];
        sig[i] = acc;
    }
    for (int j = 0; j < ncol; ++j) {
        double acc = 0.0;
        for (int g = 0; g < ngp; ++g) {
            const double *Bg = B.data() + g * nstr * ncol;
            for (int i = 0; i < nstr; ++i)
                acc += Bg[i * ncol + j] * sig[i];
        }
        f[j] = acc * ve / ngp;
    }
}

// Node-major -> component-major ("C groups of 8", matmodel.h:246-251).
inline void to_component_major(int C, const std::vector<double> &Kn, std::vector<double> &Kc)
{
    const int ncol = 8 * C;
    Kc.assign(ncol * ncol, 0.0);
    for (int i = 0; i < ncol; ++i)
        for (int j = 0; j < ncol; ++j)
            Kc[((i % C) * 8 + i / C) * ncol + (j % C) * 8 + j / C] = Kn[i * ncol + j];
}

// Radix plan for a transform of length n: radix-8 stages first, then one 4 or
// 2, then odd primes.  Returns false for lengths with a prime factor > 13.
inline bool radix_plan(int n, int *rad, int *nrad, int maxr)
{
    int m = n, k = 0;
    while (m % 8 == 0 && k < maxr) {
        rad[k++] = 8;
        m /= 8;
    }
    if (m % 4 == 0 && k < maxr) {
        rad[k++] = 4;
        m /= 4;
    }
    if (m % 2 == 0 && k < maxr) {
        rad[k++] = 2;
        m /= 2;
    }
    for (int f = 3; m > 1 && k < maxr; f += 2)
        while (m % f == 0 && k < maxr) {
            if (f > 13)
                return false;
            rad[k++] = f;
            m /= f;
        }
    *nrad = k;
    return m == 1;
}

// Pseudo-inverse of a symmetric n x n matrix (cyclic Jacobi eigen-decomposition;
// eigenvalues below n * eps * max|lambda| are dropped) -- the
// completeOrthogonalDecomposition().pseudoInverse() of mixedBCs.h:45 for the
// symmetric Q_F^T C0 Q_F.
inline std::vector<double> sym_pinv(std::vector<double> A, int n)
{
    std::vector<double> V(n * n, 0.0);
    for (int i = 0; i < n; ++i)
        V[i * n + i] = 1.0;
    for (int sweep = 0; sweep < 64; ++sweep) {
        double off = 0.0;
        for (int p = 0; p < n; ++p)
            for (int q = p + 1; q < n; ++q)
                off += A[p * n + q] * A[p * n + q];
        if (off < 1e-300)
            break;
        for (int p = 0; p < n; ++p)
            for (int q = p + 1; q < n; ++q) {
                const double apq = A[p * n + q];
                if (std::fabs(apq) < 1e-300)
                    continue;
                const double theta = (A[q * n + q] - A[p * n + p]) / (2.0 * apq);
                const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
                const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < n; ++k) { // A <- A J
                    const double akp = A[k * n + p], akq = A[k * n + q];
                    A[k * n + p] = c * akp - s * akq;
                    A[k * n + q] = s * akp + c * akq;
                }
                for (int k = 0; k < n; ++k) { // A <- J^T A
                    const double apk = A[p * n + k], aqk = A[q * n + k];
                    A[p * n + k] = c * apk - s * aqk;
                    A[q * n + k] = s * apk + c * aqk;
                }
                for (int k = 0; k < n; ++k) {
                    const double vkp = V[k * n + p], vkq = V[k * n + q];
                    V[k * n + p] = c * vkp - s * vkq;
                    V[k * n + q] = s * vkp + c * vkq;
                }
            }
    }
    double lmax = 0.0;
    for (int i = 0; i < n; ++i)
        lmax = std::max(lmax, std::fabs(A[i * n + i]));
    const double thr = n * 2.220446049250313e-16 * lmax;
    std::vector<double> P(n * n, 0.0);
    for (int k = 0; k < n; ++k) {
        const double l = A[k * n + k];
        if (std::fabs(l) <= thr)
            continue;
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j)
                P[i * n + j] += V[i * n + k] * V[j * n + k] / l;
    }
    return P;
}

} // namespace fe
} // namespace fansgpu
