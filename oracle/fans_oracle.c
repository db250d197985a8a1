/*
 * fans_oracle.c -- FP64 CPU restatement of the FANS per-iteration solve path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the CUDA product in
 * fans_gb300/csrc: only tests/, __graft_entry__.smoke() and the cpu_baseline /
 * reference arm of bench.py may load it.  Nothing in the product links it.
 *
 * It restates, in plain C with FP64 arithmetic, what the reference (FANS v0.6.2)
 * computes on the solve path.  Each function cites the reference file:line it
 * follows.  The reference itself cannot be built in this image (it needs MPI,
 * FFTW3-MPI, parallel HDF5, Eigen and nlohmann_json, none of which exist), so
 * FFTW's transform and Eigen's JacobiSVD pseudo-inverse are restated here from
 * their published definitions:
 *   - FFTW 3.3.10 r2c/c2r: the unnormalised DFT X_k = sum_j x_j exp(-2 pi i jk/n),
 *     half spectrum along the last dimension, backward transform unnormalised.
 *     Implemented as a mixed-radix Stockham FFT (radices 2..8 + naive DFT for
 *     any other prime factor).
 *   - Eigen 3.4 JacobiSVD pseudo-inverse with an absolute singular-value
 *     threshold: for the real symmetric c x c blocks used here the singular
 *     values are |eigenvalues|, computed by cyclic Jacobi rotations.
 *
 * Parity pinning: the reference itself cannot be built or run here.  Its test
 * inputs test/input_files/test_MixedBCs.json and test_MixedBCs_LargeStrain.json
 * carry macroscopic states the reference computed on test/microstructures/
 * sphere32.h5 (the loading of their later load cases); this oracle reproduces
 * them (small-strain mixed BCs with PseudoPlasticLinearHardening + linear
 * elasticity to 2.4e-9 relative, CompressibleNeoHookean at F33 = 2 to 3e-10
 * absolute on P33 = 74.757449712464).  Laws those two files do not exercise
 * (J2 plasticity, J2ViscoPlastic, SaintVenantKirchhoff, thermal, triclinic,
 * HEX8R/BBAR) are anchored by an independent numpy restatement
 * (oracle/numpy_ref.py), known answers (homogeneous media, laminates, strain
 * energy derivatives) and the invariants the reference's own tests check; for
 * those, parity is unpinned.
 *
 * Layouts follow the reference: nodal fields are [x][y][z][c] (c fastest,
 * solver.h:123-127 without the FFTW z padding), the microstructure is
 * uint16 [x][y][z] (reader.cpp:380-398), element index = index of its node 0
 * (solver.h:333, :255).
 *
 * Loops are parallelised with OpenMP in a way that keeps every floating-point
 * summation order independent of the thread count (per-plane partial sums
 * added in plane order; element planes split by x parity for the scatter).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define FO_API __attribute__((visibility("default")))

enum { FO_HEX8 = 0, FO_HEX8R = 1, FO_BBAR = 2 };
enum { FO_LAW_THERMAL_ISO = 0, FO_LAW_ELASTIC_ISO = 1, FO_LAW_J2 = 2, FO_LAW_THERMAL_TRI = 3, FO_LAW_ELASTIC_TRI = 4,
       FO_LAW_PSEUDO_LIN = 5, FO_LAW_PSEUDO_NL = 6, FO_LAW_J2VISCO_LIN = 7, FO_LAW_J2VISCO_NL = 8,
       FO_LAW_SVK = 9, FO_LAW_NEOHOOKEAN = 10 };

/* Strain measure of mechanical problems: 0 small strain <3,6> (Mandel), 1 large
 * strain <3,9> (deformation gradient, row-major F_iJ at 3i + J; main.cpp:64-77).
 * Set before building B and before calls that evaluate the laws. */
static int g_large = 0;
FO_API void fo_set_large_strain(int on) { g_large = on ? 1 : 0; }
static int nstr_of(int c) { return c == 1 ? 3 : (g_large ? 9 : 6); }

/* Kinematic-hardening internal variable psi_bar of J2ViscoPlastic [N][ngp][6]
 * (committed and trial), bound before calls that evaluate the laws. */
static const double *g_pb_t = 0;
static double       *g_pb   = 0;
FO_API void fo_bind_kinematic(const double *pb_t, double *pb)
{
    g_pb_t = pb_t;
    g_pb   = pb;
}
enum { FO_L1 = 0, FO_L2 = 1, FO_LINF = 2 };
enum { FO_ABS = 0, FO_REL = 1 };

/* -------------------------------------------------------------------------- */
/* Kinematics: shape-function gradients and B matrices (matmodel.h:104-188,    */
/* matmodel.h:267-304).                                                        */
/* -------------------------------------------------------------------------- */

/* Trilinear shape-function gradient at reference point (x,y,z), 3 x 8, row-major.
 * Follows Matmodel::Compute_basic_B (matmodel.h:158-188). */
static void basic_B(double x, double y, double z, const double le[3], double out[3][8])
{
    const double lx = le[0], ly = le[1], lz = le[2];
    out[0][0] = -(1. - y) * (1. - z) / lx;
    out[0][1] = (1. - y) * (1. - z) / lx;
    out[0][2] = -y * (1. - z) / lx;
    out[0][3] = y * (1. - z) / lx;
    out[0][4] = -(1. - y) * z / lx;
    out[0][5] = (1. - y) * z / lx;
    out[0][6] = -y * z / lx;
    out[0][7] = y * z / lx;

    out[1][0] = -(1. - x) * (1. - z) / ly;
    out[1][1] = -x * (1. - z) / ly;
    out[1][2] = (1. - x) * (1. - z) / ly;
    out[1][3] = x * (1. - z) / ly;
    out[1][4] = -(1. - x) * z / ly;
    out[1][5] = -x * z / ly;
    out[1][6] = (1. - x) * z / ly;
    out[1][7] = x * z / ly;

    out[2][0] = -(1. - x) * (1. - y) / lz;
    out[2][1] = -x * (1. - y) / lz;
    out[2][2] = -(1. - x) * y / lz;
    out[2][3] = -x * y / lz;
    out[2][4] = (1. - x) * (1. - y) / lz;
    out[2][5] = x * (1. - y) / lz;
    out[2][6] = (1. - x) * y / lz;
    out[2][7] = x * y / lz;
}

/* Compute_B for the thermal (c=1, 3x8) or small-strain Mandel (c=3, 6x24) model.
 * Thermal: matmodel.h:267-270.  Mechanical: matmodel.h:284-304. */
static void model_B(int c, double x, double y, double z, const double le[3], double *out /* nstr x 8c */)
{
    double b[3][8];
    basic_B(x, y, z, le, b);
    if (c == 3 && g_large) { /* LargeStrainMechModel::Compute_B (LargeStrainMechModel.h:209-225) */
        memset(out, 0, sizeof(double) * 9 * 24);
        for (int i = 0; i < 3; ++i)
            for (int J = 0; J < 3; ++J)
                for (int q = 0; q < 8; ++q)
                    out[(3 * i + J) * 24 + 3 * q + i] = b[J][q];
        return;
    }
    if (c == 1) {
        for (int i = 0; i < 3; ++i)
            for (int q = 0; q < 8; ++q)
                out[i * 8 + q] = b[i][q];
        return;
    }
    const double sqrt_half = 7.071067811865476e-01;
    memset(out, 0, sizeof(double) * 6 * 24);
    for (int q = 0; q < 8; ++q) {
        out[0 * 24 + 3 * q + 0] = b[0][q];
        out[1 * 24 + 3 * q + 1] = b[1][q];
        out[2 * 24 + 3 * q + 2] = b[2][q];
        out[3 * 24 + 3 * q + 0] = sqrt_half * b[1][q];
        out[4 * 24 + 3 * q + 0] = sqrt_half * b[2][q];
        out[5 * 24 + 3 * q + 1] = sqrt_half * b[2][q];
        out[3 * 24 + 3 * q + 1] = sqrt_half * b[0][q];
        out[4 * 24 + 3 * q + 2] = sqrt_half * b[0][q];
        out[5 * 24 + 3 * q + 2] = sqrt_half * b[1][q];
    }
}

/* B_int at every Gauss point (Construct_B, matmodel.h:104-155).
 * Returns n_gp; B is n_gp blocks of nstr x 8c (row-major). */
FO_API int fo_build_B(int fe_type, int c, const double le[3], double *B)
{
    const int nstr = nstr_of(c);
    const int ncol = 8 * c;
    if (fe_type == FO_HEX8R) {
        model_B(c, 0.5, 0.5, 0.5, le, B);
        return 1;
    }
    const double xi_p = 0.5 + sqrt(3.) / 6.;
    const double xi_m = 0.5 - sqrt(3.) / 6.;
    const double xi[8][3] = {{xi_m, xi_m, xi_m}, {xi_p, xi_m, xi_m}, {xi_m, xi_p, xi_m}, {xi_p, xi_p, xi_m},
                             {xi_m, xi_m, xi_p}, {xi_p, xi_m, xi_p}, {xi_m, xi_p, xi_p}, {xi_p, xi_p, xi_p}};
    if (fe_type == FO_BBAR && nstr > 3) {
        double Bvol[9 * 24], Bfull[9 * 24];
        model_B(c, 0.5, 0.5, 0.5, le, Bvol);
        for (int p = 0; p < 8; ++p) {
            model_B(c, xi[p][0], xi[p][1], xi[p][2], le, Bfull);
            double *Bp = B + (size_t)p * nstr * ncol;
            for (int col = 0; col < ncol; ++col) {
                double vol_full = (Bfull[0 * ncol + col] + Bfull[1 * ncol + col] + Bfull[2 * ncol + col]) / 3.0;
                double vol_bar  = (Bvol[0 * ncol + col] + Bvol[1 * ncol + col] + Bvol[2 * ncol + col]) / 3.0;
                for (int row = 0; row < 3; ++row)
                    Bp[row * ncol + col] = Bfull[row * ncol + col] - vol_full + vol_bar;
                for (int row = 3; row < nstr; ++row)
                    Bp[row * ncol + col] = Bfull[row * ncol + col];
            }
        }
        return 8;
    }
    for (int p = 0; p < 8; ++p)
        model_B(c, xi[p][0], xi[p][1], xi[p][2], le, B + (size_t)p * nstr * ncol);
    return 8;
}

/* K = sum_gp B^T C B * v_e / n_gp  (8c x 8c, node-major [node][comp] ordering).
 * LinearElastic.h:37-39, LinearThermal.h:189-191, matmodel.h:243-245. */
FO_API void fo_element_stiffness(int c, int ngp, const double *B, const double *C, double ve, double *K)
{
    const int nstr = nstr_of(c), ncol = 8 * c;
    memset(K, 0, sizeof(double) * ncol * ncol);
    double CB[9 * 24];
    for (int p = 0; p < ngp; ++p) {
        const double *Bp = B + (size_t)p * nstr * ncol;
        for (int i = 0; i < nstr; ++i)
            for (int j = 0; j < ncol; ++j) {
                double acc = 0.0;
                for (int k = 0; k < nstr; ++k)
                    acc += C[i * nstr + k] * Bp[k * ncol + j];
                CB[i * ncol + j] = acc;
            }
        for (int i = 0; i < ncol; ++i)
            for (int j = 0; j < ncol; ++j) {
                double acc = 0.0;
                for (int k = 0; k < nstr; ++k)
                    acc += Bp[k * ncol + i] * CB[k * ncol + j];
                K[i * ncol + j] += acc * ve / ngp;
            }
    }
}

/* -------------------------------------------------------------------------- */
/* Symmetric pseudo-inverse (Eigen JacobiSVD restated for symmetric blocks,    */
/* solver.h:89-96).                                                            */
/* -------------------------------------------------------------------------- */
static void sym_pinv(int n, const double *A, double tol, double *P)
{
    double a[3][3], v[3][3];
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
            a[i][j] = A[i * n + j];
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
        for (int p = 0; p < n; ++p)
            for (int q = p + 1; q < n; ++q) {
                if (a[p][q] == 0.0)
                    continue;
                double theta = (a[q][q] - a[p][p]) / (2.0 * a[p][q]);
                double t     = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                double cs = 1.0 / sqrt(t * t + 1.0), sn = t * cs;
                for (int k = 0; k < n; ++k) {
                    double akp = a[k][p], akq = a[k][q];
                    a[k][p] = cs * akp - sn * akq;
                    a[k][q] = sn * akp + cs * akq;
                }
                for (int k = 0; k < n; ++k) {
                    double apk = a[p][k], aqk = a[q][k];
                    a[p][k] = cs * apk - sn * aqk;
                    a[q][k] = sn * apk + cs * aqk;
                }
                for (int k = 0; k < n; ++k) {
                    double vkp = v[k][p], vkq = v[k][q];
                    v[k][p] = cs * vkp - sn * vkq;
                    v[k][q] = sn * vkp + cs * vkq;
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

/* -------------------------------------------------------------------------- */
/* Green's operator (Solver::computeFundamentalSolution, solver.h:145-204).    */
/* K0n: element stiffness of the reference material in node-major ordering    */
/* (8c x 8c).  G out: [kx][ky][kz] (kz < nz/2+1), c(c+1)/2 lower-triangle      */
/* entries per frequency (row-major lower: 00,10,11,20,21,22), scaled by 1/N.  */
/* -------------------------------------------------------------------------- */
FO_API void fo_green(int nx, int ny, int nz, int c, const double *K0n, double *G)
{
    const int nzh = nz / 2 + 1, ncol = 8 * c, nt = c * (c + 1) / 2;
    /* reorder to "c groups of 8" as in matmodel.h:246-251 */
    double *K0 = (double *)malloc(sizeof(double) * ncol * ncol);
    for (int i = 0; i < ncol; ++i)
        for (int j = 0; j < ncol; ++j)
            K0[((i % c) * 8 + i / c) * ncol + (j % c) * 8 + j / c] = K0n[i * ncol + j];
    const double tpi = 2.0 * acos(-1.0);
    const double Ninv = 1.0 / ((double)nx * (double)ny * (double)nz);
#pragma omp parallel for schedule(static)
    for (int ix = 0; ix < nx; ++ix) {
        double ex_r = cos(tpi * ix / (double)nx), ex_i = sin(tpi * ix / (double)nx);
        for (int iy = 0; iy < ny; ++iy) {
            double ey_r = cos(tpi * iy / (double)ny), ey_i = sin(tpi * iy / (double)ny);
            for (int iz = 0; iz < nzh; ++iz) {
                double *g = G + (((size_t)ix * ny + iy) * nzh + iz) * nt;
                if (ix == 0 && iy == 0 && iz == 0) {
                    for (int t = 0; t < nt; ++t)
                        g[t] = 0.0;
                    continue;
                }
                double ez_r = cos(tpi * iz / (double)nz), ez_i = sin(tpi * iz / (double)nz);
                double Ar[8], Ai[8];
                /* A = [1, ex, ey, ex*ey, ez, ex*ez, ez*ey, ex*ey*ez] (solver.h:171-178) */
                Ar[0] = 1.0; Ai[0] = 0.0;
                Ar[1] = ex_r; Ai[1] = ex_i;
                Ar[2] = ey_r; Ai[2] = ey_i;
                Ar[3] = ex_r * ey_r - ex_i * ey_i; Ai[3] = ex_r * ey_i + ex_i * ey_r;
                Ar[4] = ez_r; Ai[4] = ez_i;
                Ar[5] = ex_r * ez_r - ex_i * ez_i; Ai[5] = ex_r * ez_i + ex_i * ez_r;
                Ar[6] = ez_r * ey_r - ez_i * ey_i; Ai[6] = ez_r * ey_i + ez_i * ey_r;
                Ar[7] = Ar[3] * ez_r - Ai[3] * ez_i; Ai[7] = Ar[3] * ez_i + Ai[3] * ez_r;
                double AA[8][8];
                for (int p = 0; p < 8; ++p)
                    for (int q = 0; q < 8; ++q)
                        AA[p][q] = Ar[p] * Ar[q] + Ai[p] * Ai[q];
                double block[9], pinv[9];
                for (int i = 0; i < c; ++i)
                    for (int j = i; j < c; ++j) {
                        double acc = 0.0;
                        for (int p = 0; p < 8; ++p)
                            for (int q = 0; q < 8; ++q)
                                acc += K0[(8 * i + p) * ncol + 8 * j + q] * AA[p][q];
                        block[i * c + j] = acc;
                        block[j * c + i] = acc;
                    }
                sym_pinv(c, block, 1e-14, pinv);
                int t = 0;
                for (int i = 0; i < c; ++i)
                    for (int j = 0; j <= i; ++j)
                        g[t++] = pinv[i * c + j] * Ninv;
            }
        }
    }
    free(K0);
}

/* -------------------------------------------------------------------------- */
/* FFT (restating FFTW's unnormalised DFT).  Mixed-radix Stockham, complex.    */
/* -------------------------------------------------------------------------- */
typedef struct {
    int     n, nrad, rad[40];
    double *twr, *twi; /* exp(sign * 2 pi i q / n), q < n */
} fo_plan;

static void plan_init(fo_plan *p, int n, int sign)
{
    p->n    = n;
    p->nrad = 0;
    int m   = n;
    while (m % 8 == 0 && m > 8) { p->rad[p->nrad++] = 8; m /= 8; }
    while (m % 4 == 0 && m > 4) { p->rad[p->nrad++] = 4; m /= 4; }
    while (m % 2 == 0 && m > 1) { p->rad[p->nrad++] = 2; m /= 2; }
    for (int f = 3; m > 1; f += 2)
        while (m % f == 0) { p->rad[p->nrad++] = f; m /= f; }
    p->twr = (double *)malloc(sizeof(double) * n);
    p->twi = (double *)malloc(sizeof(double) * n);
    const double tpi = 2.0 * acos(-1.0);
    for (int q = 0; q < n; ++q) {
        p->twr[q] = cos(tpi * q / (double)n);
        p->twi[q] = sign * sin(tpi * q / (double)n);
    }
}
static void plan_free(fo_plan *p)
{
    free(p->twr);
    free(p->twi);
}

/* in-place FFT of one complex line (re, im arrays, contiguous) using scratch */
static void fft_line(const fo_plan *p, double *re, double *im, double *sr, double *si)
{
    const int n = p->n;
    double *ar = re, *ai = im, *br = sr, *bi = si;
    int Ns = 1;
    for (int s = 0; s < p->nrad; ++s) {
        const int R = p->rad[s], m = n / R;
        for (int j = 0; j < m; ++j) {
            const int k = j % Ns;
            double vr[64], vi[64];
            for (int r = 0; r < R; ++r) {
                double xr = ar[j + r * m], xi = ai[j + r * m];
                int    q  = (r * k * (n / (Ns * R))) % n;
                double wr = p->twr[q], wi = p->twi[q];
                vr[r] = xr * wr - xi * wi;
                vi[r] = xr * wi + xi * wr;
            }
            const int idxD = (j / Ns) * Ns * R + k;
            const int step = n / R;
            for (int o = 0; o < R; ++o) {
                double accr = 0.0, acci = 0.0;
                for (int r = 0; r < R; ++r) {
                    int    q  = ((r * o) % R) * step;
                    double wr = p->twr[q], wi = p->twi[q];
                    accr += vr[r] * wr - vi[r] * wi;
                    acci += vr[r] * wi + vi[r] * wr;
                }
                br[idxD + o * Ns] = accr;
                bi[idxD + o * Ns] = acci;
            }
        }
        double *t;
        t = ar; ar = br; br = t;
        t = ai; ai = bi; bi = t;
        Ns *= R;
    }
    if (ar != re) {
        memcpy(re, ar, sizeof(double) * n);
        memcpy(im, ai, sizeof(double) * n);
    }
}

/* r2c of one real component field f[x][y][z] (stride between values = fstride)
 * into spectrum (sre, sim) [x][y][kz], kz < nz/2+1.  FFTW sign convention. */
FO_API void fo_rfft3(int nx, int ny, int nz, const double *f, int fstride, double *sre, double *sim)
{
    const int nzh = nz / 2 + 1;
    fo_plan pz, py, px;
    plan_init(&pz, nz, -1);
    plan_init(&py, ny, -1);
    plan_init(&px, nx, -1);
    const int nmax = nx > ny ? (nx > nz ? nx : nz) : (ny > nz ? ny : nz);
#pragma omp parallel
    {
        double *br = (double *)malloc(sizeof(double) * nmax), *bi = (double *)malloc(sizeof(double) * nmax);
        double *sr = (double *)malloc(sizeof(double) * nmax), *si = (double *)malloc(sizeof(double) * nmax);
#pragma omp for schedule(static)
        for (int xy = 0; xy < nx * ny; ++xy) {
            for (int z = 0; z < nz; ++z) {
                br[z] = f[((size_t)xy * nz + z) * fstride];
                bi[z] = 0.0;
            }
            fft_line(&pz, br, bi, sr, si);
            for (int k = 0; k < nzh; ++k) {
                sre[(size_t)xy * nzh + k] = br[k];
                sim[(size_t)xy * nzh + k] = bi[k];
            }
        }
#pragma omp for schedule(static)
        for (int xk = 0; xk < nx * nzh; ++xk) {
            int x = xk / nzh, k = xk % nzh;
            for (int y = 0; y < ny; ++y) {
                size_t o = ((size_t)x * ny + y) * nzh + k;
                br[y] = sre[o];
                bi[y] = sim[o];
            }
            fft_line(&py, br, bi, sr, si);
            for (int y = 0; y < ny; ++y) {
                size_t o = ((size_t)x * ny + y) * nzh + k;
                sre[o] = br[y];
                sim[o] = bi[y];
            }
        }
#pragma omp for schedule(static)
        for (int yk = 0; yk < ny * nzh; ++yk) {
            int y = yk / nzh, k = yk % nzh;
            for (int x = 0; x < nx; ++x) {
                size_t o = ((size_t)x * ny + y) * nzh + k;
                br[x] = sre[o];
                bi[x] = sim[o];
            }
            fft_line(&px, br, bi, sr, si);
            for (int x = 0; x < nx; ++x) {
                size_t o = ((size_t)x * ny + y) * nzh + k;
                sre[o] = br[x];
                sim[o] = bi[x];
            }
        }
        free(br); free(bi); free(sr); free(si);
    }
    plan_free(&pz);
    plan_free(&py);
    plan_free(&px);
}

/* c2r (unnormalised, FFTW_BACKWARD).  Destroys the spectrum.  The imaginary
 * parts of the kz=0 and kz=nz/2 planes are treated as FFTW's c2r treats them:
 * the z-line is rebuilt from Hermitian symmetry using the first nz/2+1 entries. */
FO_API void fo_irfft3(int nx, int ny, int nz, double *sre, double *sim, double *f, int fstride)
{
    const int nzh = nz / 2 + 1;
    fo_plan pz, py, px;
    plan_init(&pz, nz, +1);
    plan_init(&py, ny, +1);
    plan_init(&px, nx, +1);
    const int nmax = nx > ny ? (nx > nz ? nx : nz) : (ny > nz ? ny : nz);
#pragma omp parallel
    {
        double *br = (double *)malloc(sizeof(double) * nmax), *bi = (double *)malloc(sizeof(double) * nmax);
        double *sr = (double *)malloc(sizeof(double) * nmax), *si = (double *)malloc(sizeof(double) * nmax);
#pragma omp for schedule(static)
        for (int yk = 0; yk < ny * nzh; ++yk) {
            int y = yk / nzh, k = yk % nzh;
            for (int x = 0; x < nx; ++x) {
                size_t o = ((size_t)x * ny + y) * nzh + k;
                br[x] = sre[o];
                bi[x] = sim[o];
            }
            fft_line(&px, br, bi, sr, si);
            for (int x = 0; x < nx; ++x) {
                size_t o = ((size_t)x * ny + y) * nzh + k;
                sre[o] = br[x];
                sim[o] = bi[x];
            }
        }
#pragma omp for schedule(static)
        for (int xk = 0; xk < nx * nzh; ++xk) {
            int x = xk / nzh, k = xk % nzh;
            for (int y = 0; y < ny; ++y) {
                size_t o = ((size_t)x * ny + y) * nzh + k;
                br[y] = sre[o];
                bi[y] = sim[o];
            }
            fft_line(&py, br, bi, sr, si);
            for (int y = 0; y < ny; ++y) {
                size_t o = ((size_t)x * ny + y) * nzh + k;
                sre[o] = br[y];
                sim[o] = bi[y];
            }
        }
#pragma omp for schedule(static)
        for (int xy = 0; xy < nx * ny; ++xy) {
            for (int k = 0; k < nzh; ++k) {
                br[k] = sre[(size_t)xy * nzh + k];
                bi[k] = sim[(size_t)xy * nzh + k];
            }
            /* Hermitian completion; DC and (even nz) Nyquist imaginary parts dropped */
            bi[0] = 0.0;
            if (nz % 2 == 0)
                bi[nz / 2] = 0.0;
            for (int k = nzh; k < nz; ++k) {
                br[k] = br[nz - k];
                bi[k] = -bi[nz - k];
            }
            fft_line(&pz, br, bi, sr, si);
            for (int z = 0; z < nz; ++z)
                f[((size_t)xy * nz + z) * fstride] = br[z];
        }
        free(br); free(bi); free(sr); free(si);
    }
    plan_free(&pz);
    plan_free(&py);
    plan_free(&px);
}

/* s = IFFT( G . FFT(r) ), r and s [x][y][z][c] (Solver::convolution,
 * solver.h:388-412; G from fo_green already carries the 1/N factor). */
FO_API void fo_convolve(int nx, int ny, int nz, int c, const double *G, const double *r, double *s)
{
    const int    nzh = nz / 2 + 1, nt = c * (c + 1) / 2;
    const size_t F   = (size_t)nx * ny * nzh;
    double      *re  = (double *)malloc(sizeof(double) * F * c);
    double      *im  = (double *)malloc(sizeof(double) * F * c);
    for (int a = 0; a < c; ++a)
        fo_rfft3(nx, ny, nz, r + a, c, re + a * F, im + a * F);
#pragma omp parallel for schedule(static)
    for (size_t f = 0; f < F; ++f) {
        const double *g = G + f * nt;
        double        Gm[3][3];
        int           t = 0;
        for (int i = 0; i < c; ++i)
            for (int j = 0; j <= i; ++j) {
                Gm[i][j] = g[t];
                Gm[j][i] = g[t];
                ++t;
            }
        double xr[3], xi[3];
        for (int a = 0; a < c; ++a) {
            xr[a] = re[a * F + f];
            xi[a] = im[a * F + f];
        }
        for (int a = 0; a < c; ++a) {
            double ar = 0.0, ai = 0.0;
            for (int b = 0; b < c; ++b) {
                ar += Gm[a][b] * xr[b];
                ai += Gm[a][b] * xi[b];
            }
            re[a * F + f] = ar;
            im[a * F + f] = ai;
        }
    }
    for (int a = 0; a < c; ++a)
        fo_irfft3(nx, ny, nz, re + a * F, im + a * F, s + a, c);
    free(re);
    free(im);
}

/* -------------------------------------------------------------------------- */
/* Material laws (per Gauss point).                                            */
/* -------------------------------------------------------------------------- */
typedef struct {
    int           nx, ny, nz, c, nstr, ngp;
    double        ve;
    const double *B;       /* ngp x nstr x 8c */
    const uint16_t *ms;
    int           nphase;
    const int    *law;     /* per phase */
    const double *param;   /* per phase, 24 doubles */
    const double *g0;      /* nstr */
    /* J2 internal variables, element-major: eps_p [N][ngp][6], q [N][ngp] */
    const double *ep_t, *q_t;
    double       *ep, *q;
} fo_problem;

/* LinearThermalIsotropic::get_sigma (LinearThermal.h:35-40); param[0] = conductivity.
 * LinearElasticIsotropic::get_sigma (LinearElastic.h:43-53); param = {K, G}, lambda = K - 2G/3.
 * Triclinic laws: sigma = C eps with C row-major nstr x nstr in param (LinearElastic.h:141-144).
 * J2PlasticityNew::get_sigma (J2PlasticityNew.h:43-108); param = {K, G, sigma_y, h}. */
static void law_sigma(const fo_problem *P, int phase, size_t elem, int gp, const double *eps, double *sig)
{
    const double *pr = P->param + (size_t)phase * 36;
    switch (P->law[phase]) {
    case FO_LAW_THERMAL_ISO:
        for (int i = 0; i < 3; ++i)
            sig[i] = pr[0] * eps[i];
        break;
    case FO_LAW_ELASTIC_ISO: {
        double lambda = pr[0] - (2.0 / 3.0) * pr[1];
        double buf1 = lambda * (eps[0] + eps[1] + eps[2]);
        double buf2 = 2 * pr[1];
        sig[0] = buf1 + buf2 * eps[0];
        sig[1] = buf1 + buf2 * eps[1];
        sig[2] = buf1 + buf2 * eps[2];
        sig[3] = buf2 * eps[3];
        sig[4] = buf2 * eps[4];
        sig[5] = buf2 * eps[5];
        break;
    }
    case FO_LAW_THERMAL_TRI:
    case FO_LAW_ELASTIC_TRI: {
        const int n = P->nstr;
        for (int i = 0; i < n; ++i) {
            double acc = 0.0;
            for (int k = 0; k < n; ++k)
                acc += pr[i * n + k] * eps[k];
            sig[i] = acc;
        }
        break;
    }
    case FO_LAW_PSEUDO_LIN:
    case FO_LAW_PSEUDO_NL: {
        /* PseudoPlasticLinearHardening::get_sigma (PseudoPlastic.h:92-115), param = {K, G, sigma_y, h};
         * PseudoPlasticNonLinearHardening::get_sigma (PseudoPlastic.h:138-160), param = {K, G, sigma_y, n, eps_0} */
        const double Kb = pr[0], G = pr[1], sy = pr[2];
        double treps = eps[0] + eps[1] + eps[2], dev[6], nrm = 0.0, buf2;
        for (int i = 0; i < 3; ++i)
            dev[i] = eps[i] - (1.0 / 3.0) * treps;
        for (int i = 3; i < 6; ++i)
            dev[i] = eps[i];
        for (int i = 0; i < 6; ++i)
            nrm += dev[i] * dev[i];
        nrm = sqrt(nrm);
        const double buf1 = Kb * treps;
        if (P->law[phase] == FO_LAW_PSEUDO_LIN) {
            const double h = pr[3], ec = sqrt(2. / 3.) * sy / (2. * G), Es = (3. * G) / (3. * G + h);
            buf2 = nrm <= ec ? 2.0 * G : (sqrt(2. / 3.) * sy + (2. / 3.) * Es * h * (nrm - ec)) / nrm;
        } else {
            const double n = pr[3], e0 = pr[4], ec = e0 * pow(sy / (3.0 * G * e0), 1.0 / (1.0 - n));
            const double eq = sqrt(2.0 / 3.0) * nrm;
            buf2 = eq <= ec ? 2.0 * G : sqrt(2.0 / 3.0) * sy * pow(eq / e0, n) / nrm;
        }
        for (int i = 0; i < 3; ++i)
            sig[i] = buf1 + buf2 * dev[i];
        for (int i = 3; i < 6; ++i)
            sig[i] = buf2 * dev[i];
        break;
    }
    case FO_LAW_J2VISCO_LIN:
    case FO_LAW_J2VISCO_NL: {
        /* J2Plasticity::get_sigma (J2Plasticity.h:62-108) with compute_q_trial / compute_gamma of
         * J2ViscoPlastic_{Linear,NonLinear}IsotropicHardening (:158-225); param = {K, G, sigma_y,
         * K_iso, H_kin, eta, dt, sigma_inf, delta}.  As the reference does, the trial psi and psi_bar
         * accumulate over every evaluation (psi += ..., psi_bar -= ...); the plastic strain is
         * recomputed from its committed value. */
        const double Kb = pr[0], G = pr[1], sy = pr[2], Ki = pr[3], H = pr[4], eta = pr[5], dt = pr[6];
        const double c23 = sqrt(2.0 / 3.0);
        const size_t gi  = elem * P->ngp + gp;
        const double *ep_in = P->ep_t + gi * 6, *pbt = g_pb_t + gi * 6;
        double ee[6], st[6], dev[6], dmq[6], nv[6], nrm = 0.0;
        for (int i = 0; i < 6; ++i)
            ee[i] = eps[i] - ep_in[i];
        const double treps = ee[0] + ee[1] + ee[2];
        for (int i = 0; i < 3; ++i)
            st[i] = (Kb - 2.0 * G / 3.0) * treps + 2 * G * ee[i];
        for (int i = 3; i < 6; ++i)
            st[i] = 2 * G * ee[i];
        const double mean = (st[0] + st[1] + st[2]) / 3.0;
        for (int i = 0; i < 6; ++i)
            dev[i] = i < 3 ? st[i] - mean : st[i];
        const double psit = P->q_t[gi];
        double qtr = -Ki * psit;
        if (P->law[phase] == FO_LAW_J2VISCO_NL)
            qtr -= (pr[7] - sy) * (1 - exp(-pr[8] * psit));
        for (int i = 0; i < 6; ++i) {
            dmq[i] = dev[i] + (2.0 / 3.0) * H * pbt[i]; /* dev - qbar, qbar = -(2/3) H psi_bar_t */
            nrm += dmq[i] * dmq[i];
        }
        nrm = sqrt(nrm);
        for (int i = 0; i < 6; ++i)
            nv[i] = nrm < 1e-12 ? 0.0 : dmq[i] / nrm;
        const double f = nrm - c23 * (sy - qtr);
        const double den = 2 * G + (2.0 / 3.0) * (Ki + H) + eta / dt;
        double gam = 0.0;
        if (f >= 0) {
            if (P->law[phase] == FO_LAW_J2VISCO_LIN) {
                gam = f / den;
            } else { /* Newton iteration of J2Plasticity.h:203-214; its (2 / 3) is integer 0 */
                const double sdiff = c23 * (pr[7] - sy), del = pr[8];
                double inc = 1.0;
                int it = 0;
                while (inc > 1e-10 && it < 10) {
                    const double g  = f - gam * den - sdiff * (-exp(-del * (psit + c23 * gam)) + exp(-del * psit));
                    const double dg = -den - 0.0 * (pr[7] - sy) * del * exp(-del * (psit + c23 * gam));
                    inc = -g / dg;
                    gam += inc;
                    it++;
                }
            }
        }
        for (int i = 0; i < 6; ++i)
            sig[i] = st[i] - gam * 2 * G * nv[i];
        double *ep_out = P->ep + gi * 6, *pb = g_pb + gi * 6;
        for (int i = 0; i < 6; ++i) {
            ep_out[i] = ep_in[i] + gam * nv[i];
            pb[i] -= gam * nv[i];
        }
        P->q[gi] += gam * c23;
        break;
    }
    case FO_LAW_SVK:
    case FO_LAW_NEOHOOKEAN: {
        /* LargeStrainMechModel::get_sigma (LargeStrainMechModel.h:190-196): P = F S with
         * SaintVenantKirchhoff S = lambda tr(E) I + 2 mu E, E = (F^T F - I)/2 (SaintVenantKirchhoff.h:36-41)
         * or CompressibleNeoHookean S = lambda log(J) C^-1 + mu (I - C^-1) (CompressibleNeoHookean.h:36-49);
         * param = {K, G}, lambda = K - 2G/3, mu = G.  det F <= 0 (the reference throws) gives NaN. */
        const double mu = pr[1], lam = pr[0] - (2.0 / 3.0) * mu;
        const double *F = eps;
        double Cm[3][3], S[3][3];
        for (int I = 0; I < 3; ++I)
            for (int J = 0; J < 3; ++J) {
                double a = 0.0;
                for (int k = 0; k < 3; ++k)
                    a += F[3 * k + I] * F[3 * k + J];
                Cm[I][J] = a;
            }
        if (P->law[phase] == FO_LAW_SVK) {
            double E[3][3], trE = 0.0;
            for (int I = 0; I < 3; ++I)
                for (int J = 0; J < 3; ++J)
                    E[I][J] = 0.5 * (Cm[I][J] - (I == J ? 1.0 : 0.0));
            trE = E[0][0] + E[1][1] + E[2][2];
            for (int I = 0; I < 3; ++I)
                for (int J = 0; J < 3; ++J)
                    S[I][J] = (I == J ? lam * trE : 0.0) + 2.0 * mu * E[I][J];
        } else {
            const double J = F[0] * (F[4] * F[8] - F[5] * F[7]) - F[1] * (F[3] * F[8] - F[5] * F[6]) +
                             F[2] * (F[3] * F[7] - F[4] * F[6]);
            /* C^-1 by Gauss-Jordan elimination with partial pivoting */
            double A[3][6];
            for (int I = 0; I < 3; ++I)
                for (int K = 0; K < 6; ++K)
                    A[I][K] = K < 3 ? Cm[I][K] : (K - 3 == I ? 1.0 : 0.0);
            for (int col = 0; col < 3; ++col) {
                int piv = col;
                for (int r2 = col + 1; r2 < 3; ++r2)
                    if (fabs(A[r2][col]) > fabs(A[piv][col]))
                        piv = r2;
                for (int K = 0; K < 6; ++K) {
                    const double t = A[col][K];
                    A[col][K] = A[piv][K];
                    A[piv][K] = t;
                }
                const double d = A[col][col];
                for (int K = 0; K < 6; ++K)
                    A[col][K] /= d;
                for (int r2 = 0; r2 < 3; ++r2)
                    if (r2 != col) {
                        const double f = A[r2][col];
                        for (int K = 0; K < 6; ++K)
                            A[r2][K] -= f * A[col][K];
                    }
            }
            const double logJ = J > 0.0 ? log(J) : NAN;
            for (int I = 0; I < 3; ++I)
                for (int K = 0; K < 3; ++K)
                    S[I][K] = lam * logJ * A[I][3 + K] + mu * ((I == K ? 1.0 : 0.0) - A[I][3 + K]);
        }
        for (int i = 0; i < 3; ++i)
            for (int J = 0; J < 3; ++J)
                sig[3 * i + J] = F[3 * i] * S[0][J] + F[3 * i + 1] * S[1][J] + F[3 * i + 2] * S[2][J];
        break;
    }
    case FO_LAW_J2: {
        const double Kb = pr[0], G = pr[1], sy0 = pr[2], h = pr[3];
        const double c23 = sqrt(2.0 / 3.0);
        const double *ep_in = P->ep_t + (elem * P->ngp + gp) * 6;
        double s[6], sig_t[6];
        for (int i = 0; i < 6; ++i)
            s[i] = 2.0 * G * (eps[i] - ep_in[i]);
        double lam = Kb - 2.0 / 3.0 * G;
        double tr  = eps[0] + eps[1] + eps[2];
        for (int i = 0; i < 3; ++i)
            s[i] += lam * tr;
        for (int i = 0; i < 6; ++i)
            sig_t[i] = s[i];
        double mean = (s[0] + s[1] + s[2]) / 3.0;
        for (int i = 0; i < 3; ++i)
            sig_t[i] -= mean;
        double nrm2 = 0.0;
        for (int i = 0; i < 6; ++i)
            nrm2 += sig_t[i] * sig_t[i];
        double s_t    = sqrt(nrm2);
        double q_in   = P->q_t[elem * P->ngp + gp];
        double sy     = sy0 + q_in * h;
        double phi    = s_t - c23 * sy;
        double dgamma = phi / (2.0 * G + 2.0 / 3.0 * h);
        if (dgamma < 0.0)
            dgamma = 0.0;
        double *ep_out = P->ep + (elem * P->ngp + gp) * 6;
        for (int i = 0; i < 6; ++i)
            ep_out[i] = (s_t > 1e-12) ? ep_in[i] + dgamma * sig_t[i] / s_t : ep_in[i];
        P->q[elem * P->ngp + gp] = q_in + c23 * dgamma;
        for (int i = 0; i < 6; ++i)
            sig[i] = (s_t > 1e-12) ? s[i] - dgamma * 2.0 * G * sig_t[i] / s_t : s[i];
        break;
    }
    }
}

/* Node indices of element (x,y,z) in iterateCubes order (solver.h:318-385). */
static inline void elem_nodes(int nx, int ny, int nz, int x, int y, int z, size_t idx[8])
{
    int x1 = (x + 1 == nx) ? 0 : x + 1, y1 = (y + 1 == ny) ? 0 : y + 1, z1 = (z + 1 == nz) ? 0 : z + 1;
    idx[0] = ((size_t)x * ny + y) * nz + z;
    idx[1] = ((size_t)x1 * ny + y) * nz + z;
    idx[2] = ((size_t)x * ny + y1) * nz + z;
    idx[3] = ((size_t)x1 * ny + y1) * nz + z;
    idx[4] = ((size_t)x * ny + y) * nz + z1;
    idx[5] = ((size_t)x1 * ny + y) * nz + z1;
    idx[6] = ((size_t)x * ny + y1) * nz + z1;
    idx[7] = ((size_t)x1 * ny + y1) * nz + z1;
}

/* Scatter-add element results into r, processing element x-planes in two
 * parity groups so that planes handled concurrently never share nodes. */
typedef void (*elem_fn)(const void *ctx, int x, int y, int z, const size_t idx[8], double *res_e);

static void assemble(int nx, int ny, int nz, int c, elem_fn fn, const void *ctx, double *r)
{
    memset(r, 0, sizeof(double) * (size_t)nx * ny * nz * c);
    const int ngroups = (nx % 2 == 0) ? 2 : 3;
    for (int grp = 0; grp < ngroups; ++grp) {
        int x0, x1, step = 2;
        if (ngroups == 2) { x0 = grp; x1 = nx; }
        else if (grp < 2) { x0 = grp; x1 = nx - 1; }
        else { x0 = nx - 1; x1 = nx; step = 1; }
#pragma omp parallel for schedule(dynamic, 1)
        for (int x = x0; x < x1; x += step) {
            double res_e[24];
            size_t idx[8];
            for (int y = 0; y < ny; ++y)
                for (int z = 0; z < nz; ++z) {
                    elem_nodes(nx, ny, nz, x, y, z, idx);
                    fn(ctx, x, y, z, idx, res_e);
                    for (int i = 0; i < 8; ++i)
                        for (int j = 0; j < c; ++j)
                            r[c * idx[i] + j] += res_e[c * i + j];
                }
        }
    }
}

/* element_residual (matmodel.h:191-201) with ue relative to node 0 (solver.h:252). */
typedef struct {
    const fo_problem *P;
    const double     *u;
} res_ctx;

static void elem_residual(const void *vctx, int x, int y, int z, const size_t idx[8], double *res_e)
{
    const res_ctx    *rc = (const res_ctx *)vctx;
    const fo_problem *P  = rc->P;
    const int         c = P->c, nstr = P->nstr, ncol = 8 * c;
    double            ue[24], eps[9], sig[8 * 9];
    for (int i = 0; i < 8; ++i)
        for (int j = 0; j < c; ++j)
            ue[c * i + j] = rc->u[c * idx[i] + j] - rc->u[c * idx[0] + j];
    const int phase = P->ms[idx[0]];
    for (int gp = 0; gp < P->ngp; ++gp) {
        const double *Bp = P->B + (size_t)gp * nstr * ncol;
        for (int i = 0; i < nstr; ++i) {
            double acc = 0.0;
            for (int k = 0; k < ncol; ++k)
                acc += Bp[i * ncol + k] * ue[k];
            eps[i] = acc + P->g0[i];
        }
        law_sigma(P, phase, idx[0], gp, eps, sig + gp * nstr);
    }
    for (int k = 0; k < ncol; ++k) {
        double acc = 0.0;
        for (int gp = 0; gp < P->ngp; ++gp) {
            const double *Bp = P->B + (size_t)gp * nstr * ncol;
            for (int i = 0; i < nstr; ++i)
                acc += Bp[i * ncol + k] * sig[gp * nstr + i];
        }
        res_e[k] = acc * P->ve / P->ngp;
    }
    (void)x; (void)y; (void)z;
}

/* Linear operator rnew = sum_e A_e^T (K_phase ue) (solverCG.h:97-103). */
typedef struct {
    int             c;
    const uint16_t *ms;
    const double   *Kph; /* nphase x (8c x 8c) */
    const double   *d;
} lin_ctx;

static void elem_linear(const void *vctx, int x, int y, int z, const size_t idx[8], double *res_e)
{
    const lin_ctx *lc = (const lin_ctx *)vctx;
    const int      c = lc->c, ncol = 8 * c;
    double         ue[24];
    for (int i = 0; i < 8; ++i)
        for (int j = 0; j < c; ++j)
            ue[c * i + j] = lc->d[c * idx[i] + j] - lc->d[c * idx[0] + j];
    const double *K = lc->Kph + (size_t)lc->ms[idx[0]] * ncol * ncol;
    for (int i = 0; i < ncol; ++i) {
        double acc = 0.0;
        for (int k = 0; k < ncol; ++k)
            acc += K[i * ncol + k] * ue[k];
        res_e[i] = acc;
    }
    (void)x; (void)y; (void)z;
}

static void fill_problem(fo_problem *P, int nx, int ny, int nz, int c, int ngp, double ve, const double *B,
                         const uint16_t *ms, int nphase, const int *law, const double *param, const double *g0,
                         const double *ep_t, const double *q_t, double *ep, double *q)
{
    P->nx = nx; P->ny = ny; P->nz = nz; P->c = c; P->nstr = nstr_of(c); P->ngp = ngp;
    P->ve = ve; P->B = B; P->ms = ms; P->nphase = nphase; P->law = law; P->param = param; P->g0 = g0;
    P->ep_t = ep_t; P->q_t = q_t; P->ep = ep; P->q = q;
}

/* r = R(u): Solver::compute_residual (solver.h:272-280, :231-270). */
FO_API void fo_residual(int nx, int ny, int nz, int c, int ngp, double ve, const double *B, const uint16_t *ms,
                        int nphase, const int *law, const double *param, const double *g0, const double *ep_t,
                        const double *q_t, double *ep, double *q, const double *u, double *r)
{
    fo_problem P;
    fill_problem(&P, nx, ny, nz, c, ngp, ve, B, ms, nphase, law, param, g0, ep_t, q_t, ep, q);
    res_ctx rc = {&P, u};
    assemble(nx, ny, nz, c, elem_residual, &rc, r);
}

/* out = K d with per-phase element stiffness (solverCG.h:97-103). */
FO_API void fo_apply_linear(int nx, int ny, int nz, int c, const uint16_t *ms, const double *Kph, const double *d,
                            double *out)
{
    lin_ctx lc = {c, ms, Kph, d};
    assemble(nx, ny, nz, c, elem_linear, &lc, out);
}

/* Element-averaged strain/stress and volume averages: Matmodel::getStrainStress
 * (matmodel.h:203-225) inside Solver::get_homogenized_stress (solver.h:708-737)
 * and Solver::postprocess (solver.h:503-561).  u_e uses absolute nodal values.
 * strain/stress (optional) are [N][nstr]; avg_stress/avg_strain [nstr];
 * phase_* are [nphase][nstr] and phase_count [nphase]. */
FO_API void fo_strain_stress(int nx, int ny, int nz, int c, int ngp, double ve, const double *B, const uint16_t *ms,
                             int nphase, const int *law, const double *param, const double *g0, const double *ep_t,
                             const double *q_t, double *ep, double *q, const double *u, double *strain,
                             double *stress, double *avg_strain, double *avg_stress, double *phase_strain,
                             double *phase_stress, long *phase_count)
{
    fo_problem P;
    fill_problem(&P, nx, ny, nz, c, ngp, ve, B, ms, nphase, law, param, g0, ep_t, q_t, ep, q);
    const int nstr = P.nstr, ncol = 8 * c;
    double   *plane = (double *)calloc((size_t)nx * (2 * nstr + 2 * nstr * nphase), sizeof(double));
    long     *pcnt  = (long *)calloc((size_t)nx * nphase, sizeof(long));
    const int W     = 2 * nstr + 2 * nstr * nphase;
#pragma omp parallel for schedule(dynamic, 1)
    for (int x = 0; x < nx; ++x) {
        double *acc = plane + (size_t)x * W;
        size_t  idx[8];
        double  ue[24], eps[9], sig[9];
        for (int y = 0; y < ny; ++y)
            for (int z = 0; z < nz; ++z) {
                elem_nodes(nx, ny, nz, x, y, z, idx);
                for (int i = 0; i < 8; ++i)
                    for (int j = 0; j < c; ++j)
                        ue[c * i + j] = u[c * idx[i] + j];
                const int phase = ms[idx[0]];
                double    es[9] = {0}, ss[9] = {0};
                for (int gp = 0; gp < ngp; ++gp) {
                    const double *Bp = B + (size_t)gp * nstr * ncol;
                    for (int i = 0; i < nstr; ++i) {
                        double a = 0.0;
                        for (int k = 0; k < ncol; ++k)
                            a += Bp[i * ncol + k] * ue[k];
                        eps[i] = a + g0[i];
                    }
                    law_sigma(&P, phase, idx[0], gp, eps, sig);
                    for (int i = 0; i < nstr; ++i) {
                        es[i] += eps[i] / ngp;
                        ss[i] += sig[i] / ngp;
                    }
                }
                if (strain)
                    for (int i = 0; i < nstr; ++i)
                        strain[idx[0] * nstr + i] = es[i];
                if (stress)
                    for (int i = 0; i < nstr; ++i)
                        stress[idx[0] * nstr + i] = ss[i];
                for (int i = 0; i < nstr; ++i) {
                    acc[i] += ss[i];
                    acc[nstr + i] += es[i];
                    acc[2 * nstr + phase * nstr + i] += ss[i];
                    acc[2 * nstr + nphase * nstr + phase * nstr + i] += es[i];
                }
                pcnt[(size_t)x * nphase + phase]++;
            }
    }
    const double Ninv = 1.0 / ((double)nx * ny * nz);
    for (int i = 0; i < nstr; ++i) {
        double s = 0.0, e = 0.0;
        for (int x = 0; x < nx; ++x) {
            s += plane[(size_t)x * W + i];
            e += plane[(size_t)x * W + nstr + i];
        }
        if (avg_stress) avg_stress[i] = s * Ninv;
        if (avg_strain) avg_strain[i] = e * Ninv;
    }
    for (int ph = 0; ph < nphase; ++ph) {
        long cnt = 0;
        for (int x = 0; x < nx; ++x)
            cnt += pcnt[(size_t)x * nphase + ph];
        if (phase_count) phase_count[ph] = cnt;
        for (int i = 0; i < nstr; ++i) {
            double s = 0.0, e = 0.0;
            for (int x = 0; x < nx; ++x) {
                s += plane[(size_t)x * W + 2 * nstr + ph * nstr + i];
                e += plane[(size_t)x * W + 2 * nstr + nphase * nstr + ph * nstr + i];
            }
            if (phase_stress) phase_stress[ph * nstr + i] = cnt ? s / cnt : 0.0;
            if (phase_strain) phase_strain[ph * nstr + i] = cnt ? e / cnt : 0.0;
        }
    }
    free(plane);
    free(pcnt);
}

/* -------------------------------------------------------------------------- */
/* Vector algebra with thread-count-independent summation order.              */
/* -------------------------------------------------------------------------- */
static double dot(size_t n, const double *a, const double *b, int nblk)
{
    double *part = (double *)calloc(nblk, sizeof(double));
#pragma omp parallel for schedule(static)
    for (int k = 0; k < nblk; ++k) {
        size_t lo = n * k / nblk, hi = n * (k + 1) / nblk;
        double s  = 0.0;
        for (size_t i = lo; i < hi; ++i)
            s += a[i] * b[i];
        part[k] = s;
    }
    double s = 0.0;
    for (int k = 0; k < nblk; ++k)
        s += part[k];
    free(part);
    return s;
}

/* Solver::compute_error norm part (solver.h:415-428). */
FO_API double fo_norm(size_t n, const double *r, int measure)
{
    const int nblk = 256;
    double   *part = (double *)calloc(nblk, sizeof(double));
#pragma omp parallel for schedule(static)
    for (int k = 0; k < nblk; ++k) {
        size_t lo = n * k / nblk, hi = n * (k + 1) / nblk;
        double s  = 0.0;
        for (size_t i = lo; i < hi; ++i) {
            double v = fabs(r[i]);
            if (measure == FO_LINF)
                s = v > s ? v : s;
            else if (measure == FO_L1)
                s += v;
            else
                s += v * v;
        }
        part[k] = s;
    }
    double s = 0.0;
    for (int k = 0; k < nblk; ++k)
        s = (measure == FO_LINF) ? (part[k] > s ? part[k] : s) : s + part[k];
    free(part);
    return (measure == FO_L2) ? sqrt(s) : s;
}

/* -------------------------------------------------------------------------- */
/* Solvers.                                                                    */
/* -------------------------------------------------------------------------- */
typedef struct {
    int    measure, type, n_it;
    double tol;
    int    ls_max_iter;
    double ls_tol;
} fo_solve_opts;

/* Solver::compute_error semantics (solver.h:429-452): err_all[iter] = err,
 * relative = err/err0 with 100 returned at iter 0. */
static double compute_error(size_t n, const double *r, const fo_solve_opts *o, int iter, double *err_all)
{
    double err    = fo_norm(n, r, o->measure);
    err_all[iter] = err;
    double err_rel = (iter == 0) ? 100.0 : err / err_all[0];
    return (o->type == FO_ABS) ? err : err_rel;
}

/* SolverCG::internalSolve (solverCG.h:62-117) and LineSearchSecant
 * (solverCG.h:120-160).  islinear selects the phase_stiffness fast path.
 * u (in/out) [N][c]; r (out) residual; err_all (out, n_it+1); returns iterations. */
FO_API int fo_cg_solve(int nx, int ny, int nz, int c, int ngp, double ve, const double *B, const uint16_t *ms,
                       int nphase, const int *law, const double *param, const double *g0, const double *ep_t,
                       const double *q_t, double *ep, double *q, const double *Kph, const double *G, int islinear,
                       int measure, int type, double tol, int n_it, int ls_max_iter, double ls_tol, double *u,
                       double *r, double *err_all)
{
    const size_t  n = (size_t)nx * ny * nz * c;
    fo_solve_opts o = {measure, type, n_it, tol, ls_max_iter, ls_tol};
    double       *s = (double *)calloc(n, sizeof(double));
    double       *d = (double *)calloc(n, sizeof(double));
    double       *rnew = (double *)calloc(n, sizeof(double));
    const int     nblk = 256;
    double        alpha_warm = 0.1;

    fo_residual(nx, ny, nz, c, ngp, ve, B, ms, nphase, law, param, g0, ep_t, q_t, ep, q, u, r);
    int    iter    = 0;
    double err_rel = compute_error(n, r, &o, iter, err_all);
    double delta = 1.0, delta0, deltamid;

    while (iter < n_it && err_rel > tol) {
        deltamid = dot(n, r, s, nblk);
        fo_convolve(nx, ny, nz, c, G, r, s);
#pragma omp parallel for schedule(static)
        for (size_t i = 0; i < n; ++i)
            s[i] = -s[i];
        delta0 = delta;
        delta  = dot(n, r, s, nblk);
        double beta = (delta - deltamid) / delta0;
        beta        = beta > 0 ? beta : 0; /* fmax(0, .) */
#pragma omp parallel for schedule(static)
        for (size_t i = 0; i < n; ++i)
            d[i] = s[i] + beta * d[i];
        if (islinear) {
            fo_apply_linear(nx, ny, nz, c, ms, Kph, d, rnew);
            double alpha = delta / dot(n, d, rnew, nblk);
#pragma omp parallel for schedule(static)
            for (size_t i = 0; i < n; ++i) {
                r[i] -= alpha * rnew[i];
                u[i] -= alpha * d[i];
            }
        } else {
            /* LineSearchSecant */
            double err = 10.0;
            int    _iter = 0;
            double alpha_prev = 0.0, alpha_curr = alpha_warm;
            double rpd = dot(n, r, d, nblk);
#pragma omp parallel for schedule(static)
            for (size_t i = 0; i < n; ++i)
                u[i] += d[i] * alpha_curr;
            fo_residual(nx, ny, nz, c, ngp, ve, B, ms, nphase, law, param, g0, ep_t, q_t, ep, q, u, rnew);
            double r1pd = dot(n, rnew, d, nblk);
            while (_iter < ls_max_iter && err > ls_tol) {
                double denom = r1pd - rpd;
                if (fabs(denom) < 1e-14 * (fabs(r1pd) + fabs(rpd)))
                    break;
                double alpha_next = alpha_curr - r1pd * (alpha_curr - alpha_prev) / denom;
                if (alpha_next <= 0.0)
                    alpha_next = 0.5 * (alpha_prev + alpha_curr);
                err = fabs(alpha_next - alpha_curr);
                double da = alpha_next - alpha_curr;
#pragma omp parallel for schedule(static)
                for (size_t i = 0; i < n; ++i)
                    u[i] += d[i] * da;
                alpha_prev = alpha_curr;
                rpd        = r1pd;
                alpha_curr = alpha_next;
                _iter++;
                fo_residual(nx, ny, nz, c, ngp, ve, B, ms, nphase, law, param, g0, ep_t, q_t, ep, q, u, rnew);
                r1pd = dot(n, rnew, d, nblk);
            }
            alpha_warm = (_iter == ls_max_iter && err > ls_tol) ? 0.1 : alpha_curr;
            memcpy(r, rnew, sizeof(double) * n);
        }
        iter++;
        err_rel = compute_error(n, r, &o, iter, err_all);
    }
    free(s);
    free(d);
    free(rnew);
    return iter;
}

/* SolverFP::internalSolve (solverFP.h:33-52): u -= G*r; r = R(u). */
FO_API int fo_fp_solve(int nx, int ny, int nz, int c, int ngp, double ve, const double *B, const uint16_t *ms,
                       int nphase, const int *law, const double *param, const double *g0, const double *ep_t,
                       const double *q_t, double *ep, double *q, const double *G, int measure, int type,
                       double tol, int n_it, double *u, double *r, double *err_all)
{
    const size_t  n = (size_t)nx * ny * nz * c;
    fo_solve_opts o = {measure, type, n_it, tol, 5, 1e-2};
    double       *s = (double *)malloc(sizeof(double) * n);
    fo_residual(nx, ny, nz, c, ngp, ve, B, ms, nphase, law, param, g0, ep_t, q_t, ep, q, u, r);
    int    iter    = 0;
    double err_rel = compute_error(n, r, &o, iter, err_all);
    while (iter < n_it && err_rel > tol) {
        fo_convolve(nx, ny, nz, c, G, r, s);
#pragma omp parallel for schedule(static)
        for (size_t i = 0; i < n; ++i)
            u[i] -= s[i];
        fo_residual(nx, ny, nz, c, ngp, ve, B, ms, nphase, law, param, g0, ep_t, q_t, ep, q, u, r);
        iter++;
        err_rel = compute_error(n, r, &o, iter, err_all);
    }
    free(s);
    return iter;
}

FO_API int fo_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

FO_API void fo_set_num_threads(int n)
{
#ifdef _OPENMP
    if (n > 0)
        omp_set_num_threads(n);
#else
    (void)n;
#endif
}
