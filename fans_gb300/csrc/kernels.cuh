// kernels.cuh -- host-side launchers of the GB300 FANS kernels (one declaration
// per fused pass).  Fields on the device are SoA: component planes of N values,
// node (x,y,z) at (x*ny + y)*nz + z.  Reductions accumulate in FP64 and are
// deterministic: per-block partials summed in block order by the last block.
#pragma once
#include "fans_common.cuh"
#include "fft.cuh"

namespace fansgpu {

struct Grid3 {
    int nx, ny, nz;
    __host__ __device__ long long N() const { return (long long)nx * ny * nz; }
};

// ---------------------------------------------------------------- stencil ---
// y = K x (+ F), the CG linear operator (solverCG.h:97-103) and, with F, the
// linear residual R(u) = K u + F(g0) (solver.h:272-280, matmodel.h:191-201).
// Node-centric gather over the 8 elements around each node, with per-phase
// element stiffness K_ph (8C x 8C, node-major rows/cols) and per-phase force
// f_ph (8C).  Optional fusion:
//   fuse_d: x = s + beta*d_old (beta from scal) and x written to d_new;
//   reduction of <x, y> into scal->dAd and alpha = delta/dAd.
struct StencilArgs {
    Grid3          g;
    int            C;
    const void    *x;      // x, or s when fuse_d
    const void    *d_old;  // fuse_d only
    void          *d_new;  // fuse_d only
    void          *y;
    const uint8_t *ms;
    const void    *Kph;    // nph * 64*C*C (device)
    const void    *fph;    // nph * 8C, or null (device)
    const void    *Kph_host; // host copies of the same tables (kernel-parameter path)
    const void    *fph_host;
    int            nph;
    int            fuse_d;
    int            reduce; // 1: <x,y> -> scal (dAd, alpha)
    int            force_only; // y = F only (x known to be zero)
    CgScalars     *scal;
    GridRed        red;
    int            red_site;
    int            wait_limit; // tensor-core operator: polls before a pipeline wait gives up (0: default)
    int            wait_sleep_ns; // basis operator: consumers sleep this long between polls of D (0: spin)
    // several right-hand sides (multi-RHS operator): RHS k's fields at offset k * rhs_stride,
    // its scalars at scal[k]; active[k] == 0 skips it (null: all active)
    int            nrhs;
    long long      rhs_stride;
    const int     *active;
};
template <typename T>
cudaError_t launch_stencil(const StencilArgs &a, cudaStream_t st);

// R(u) = K u + F in double-float (FP32 pairs with error-free transformations):
// x = u (FP64 SoA), y = r (FP64), Kph = FP32 [hi | lo] tables (2 x nph x 64C^2),
// fph = FP64 force table.  FP64-accurate true residual at FP32 issue rates.
cudaError_t launch_residual_df(const StencilArgs &a, cudaStream_t st);

// r = F(g0) for u = 0 with at most two phases: `table` = 256 x C node sums indexed by the 8-bit
// key of the phases (0/1) of the 8 elements around a node (bit p: the element whose node p it is)
cudaError_t launch_force_nodes(const Grid3 &g, int C, const uint8_t *ms, const double *table, double *y,
                               cudaStream_t st);

// Element-averaged strain/stress of linear laws (matmodel.h:203-225,
// solver.h:708-737): eps_e = Bbar u_e + g0 with Bbar (the Gauss-point mean of
// B) = B at the element centre, sig_e = C_ph eps_e.  Sums over the
// elements whose phase matches `phase_filter` (-1: all) land in out_red:
// [0,nstr) sum eps, [nstr,2nstr) sum sig, [2nstr] count.  Optional AoS fields.
struct StrainStressArgs {
    Grid3          g;
    int            C, nstr;
    const double  *u;      // SoA FP64
    const uint8_t *ms;
    double         inv4l[3]; // 1 / (4 l_e) per direction (centre gradient = mean edge difference / l_e)
    const double  *Cph;    // nph x nstr x nstr
    const double  *g0;     // nstr
    int            nph;
    int            phase_filter;
    double        *strain; // [N][nstr] or null
    double        *stress; // [N][nstr] or null
    double        *out_red;
    GridRed        red;
    int            red_site;
};
cudaError_t launch_strain_stress(const StrainStressArgs &a, cudaStream_t st);
// Per-phase strain sums and counts for at most 2 phases: out_red[ph*nstr + i],
// then the two counts at out_red[2*nstr + ph].
cudaError_t launch_strain_sums(const StrainStressArgs &a, cudaStream_t st);

// ---------------------------------------------- tensor-core CG operator ---
// FP32 fused d = s + beta d_old, K d and <d, K d> with the element matvecs on
// tcgen05 (3xTF32); at most 2 phases.
bool        stencil_tc_supported(const Grid3 &g, int C, int nph);
size_t      stencil_tc_weights(int C, int nph); // floats of the packed W (hi + lo)
void        stencil_tc_pack_weights(int C, int nph, const float *K32, float *out);
cudaError_t launch_stencil_tc(const StencilArgs &a, const float *W, int nph, cudaStream_t st);
long long   stencil_tc_blocks(const Grid3 &g);

// Multi-RHS tensor-core CG operator with the element stiffness in an exact basis
// (K_ph = sum_b coef[ph][b] W_b, W_b = K_b / q_b integers exact in tf32; 2 products):
// stencil_tcb_quanta finds q_b (false if a basis matrix is not exact), the packed W
// holds the nb basis blocks, coef is nph x nb FP32 (law coefficient x q_b).  a.nrhs
// right-hand sides (<= kMaxRhs) in one launch, alpha_k per RHS.
bool        stencil_tcb_quanta(int C, const double *Kb, int nb, double *q);
bool        stencil_tcb_supported(const Grid3 &g, int C, int nb, int nph);
size_t      stencil_tcb_weights(int C, int nb);
void        stencil_tcb_pack_weights(int C, int nb, const double *Kb, const double *q, float *out);
cudaError_t launch_stencil_tcb(const StencilArgs &a, const float *W, const float *coef, int nb, cudaStream_t st);

// FP64-accurate y = K x (+ F) on the tensor cores (the exact basis W of the operator above, the
// element rows as three exact fixed-point tf32 slices, double-float epilogue): a.x FP64 (or with
// fuse_d d = s + beta d_old, written to d_new), a.y FP64, optional <x, y> -> scal (dAd, alpha).
// coef_df: nph x nb (hi, lo) FP32 pairs; f_df: [hi | lo] nph x 8C element forces, or null.
bool        stencil_tcx_supported(const Grid3 &g, int C, int nb, int nph);
cudaError_t launch_stencil_tcx(const StencilArgs &a, const float *W, const float *coef_df, const float *f_df, int nb,
                               cudaStream_t st);

// -------------------------------------------------------- element kernels ---
enum ElemMode { ELEM_RESIDUAL = 0, ELEM_AVERAGES = 1 };
struct ElementArgs {
    Grid3          g;
    int            C, nstr, ngp, mode;
    const double  *u;     // SoA FP64
    const uint8_t *ms;
    const double  *B;     // ngp x nstr x 8C
    const double  *Bb;    // ngp x 3 x 8 basic B (dN_q/dx_j), HEX8 / HEX8R mechanics; else null
    const double  *g0;    // nstr
    const int     *law;   // per phase
    const double  *Cph;   // per phase nstr x nstr (linear laws)
    const double  *prm;   // per phase, 8 law parameters (J2, PseudoPlastic)
    const double  *ep_t, *q_t; // committed internal variables [6][ngp][N], [ngp][N]
    double        *ep, *q;     // trial internal variables (written)
    const double  *pb_t;       // committed kinematic hardening psi_bar [6][ngp][N] (J2ViscoPlastic)
    double        *pb;         // trial psi_bar
    double         ve;
    double        *rows;  // RESIDUAL: [8C][N] element rows
    // AVERAGES:
    int            phase_filter;
    double        *strain, *stress; // [N][nstr] or null
    double        *strain_gp, *stress_gp; // [N][ngp][nstr] or null
    double        *flag;                  // [N] element mean of the Gauss-point plastic flags, or null
    const double  *scale;                 // [N] per-voxel stiffness scale (sigma *= scale[e]), or null
    const double  *sy;                    // [N] per-voxel initial yield stress of J2 elements, or null (phase value)
    double        *out_red;         // [0,nstr) sum eps, [nstr,2nstr) sum sig, [2nstr] count
    GridRed        red;
    int            red_site;
};
cudaError_t launch_element(const ElementArgs &a, cudaStream_t st);
// Sensitivity of sum_ij W_ij C_ij to the per-voxel stiffness scale, C_ij the
// energy-form effective stiffness of n stored solutions u_k (load g0_k):
// grad[e] = (1/N) mean_gp sum_ij W_ij eps_i^T C_ph(e) eps_j  (linear laws).
struct SensArgs {
    Grid3          g;
    int            C, nstr, ngp, n;
    const double  *u;     // n stored solutions, each SoA [C][N]
    const double  *g0;    // n x nstr
    const double  *W;     // n x n
    const uint8_t *ms;
    const double  *B, *Cph;
    double        *grad;  // [N]
};
cudaError_t launch_sensitivity(const SensArgs &a, cudaStream_t st);
// Yield-stress adjoint of a strain-controlled J2PlasticityNew load path, one
// kernel over (element, Gauss point) with the state of load step n: u_n, g0_n
// and the committed internal variables alpha_{n-1} before the step.
//   ADJ_OPERATOR: rows = B^T K_alg tau(x), tau = (v_e/n_gp) B x_e      (K_n^T x)
//   ADJ_RESIDUAL: rows = B^T VJP_e(tau(x) + cw, mu_n)                   (K_n^T x + f_n)
//   ADJ_STEP:     mu <- VJP_alpha(tau(x) + cw, mu_n), grad[e] += sum_gp VJP_sy
//   ADJ_REPLAY:   alpha_n = return map(eps_n, alpha_{n-1}) into ep_out/q_out
enum AdjMode { ADJ_OPERATOR = 0, ADJ_RESIDUAL = 1, ADJ_STEP = 2, ADJ_REPLAY = 3 };
struct AdjArgs {
    Grid3          g;
    int            ngp, mode;
    const double  *u, *g0;       // state of step n: u_n [3][N], g0_n (6)
    const double  *x;            // adjoint field [3][N] (lambda or a CG direction)
    const double  *ep_in, *q_in; // alpha_{n-1}: [6][ngp][N], [ngp][N]
    double        *ep_out, *q_out; // ADJ_REPLAY: alpha_n
    double        *mu_ep, *mu_q;   // mu_n, same layout; ADJ_STEP overwrites it with mu_{n-1}
    const double  *cw;           // 6 doubles: w/(N n_gp), the seed of <sigma_N> (last step), or null
    const uint8_t *ms;
    const double  *B;            // ngp x 6 x 24
    const double  *Bb;           // ngp x 3 x 8 basic B, or null (then the dense B)
    const int     *law;
    const double  *Cph;          // per phase 6 x 6 (linear elastic laws)
    const double  *prm;          // per phase, 8 law parameters
    const double  *sy;           // [N] per-voxel initial yield stress, or null
    double         ve;
    double        *rows;         // [24][N]
    double        *grad;         // [N], accumulated
};
cudaError_t launch_adjoint(const AdjArgs &a, cudaStream_t st);
cudaError_t launch_set_alpha(CgScalars *scal, cudaStream_t st); // alpha = delta / dAd
cudaError_t launch_gather(const double *rows, double *r, const Grid3 &g, int C, cudaStream_t st);
cudaError_t launch_dot(const double *a, const double *b, long long n, double *out, GridRed red, int site,
                       cudaStream_t st);
cudaError_t launch_direction(double *d, const double *s, long long n, const CgScalars *scal, cudaStream_t st);
// element means over Gauss points of the committed J2 variables (J2PlasticityNew.h:171-177)
cudaError_t launch_ivar_gp(const double *ep_t, const double *q_t, int ngp, long long N, double *ep_out, double *q_out,
                           cudaStream_t st);
cudaError_t launch_ivar_mean(const double *ep_t, const double *q_t, int ngp, long long N, double *ep_out,
                             double *q_out, cudaStream_t st);

// ----------------------------------------------------------------- layout ---
template <typename TI, typename TO>
cudaError_t launch_aos_to_soa(const TI *aos, TO *soa, long long N, int C, cudaStream_t st);
template <typename TI, typename TO>
cudaError_t launch_soa_to_aos(const TI *soa, TO *aos, long long N, int C, cudaStream_t st);
template <typename TI, typename TO>
cudaError_t launch_convert(const TI *in, TO *out, long long n, cudaStream_t st);

// -------------------------------------------------------------------- fft ---
template <typename T>
struct ConvPlan {
    Grid3          g;
    int            C, M, nzh, nzp; // M = nz/2 complex z-length, nzp = spectrum row stride
    FftDim         dx, dy, dz;     // dz has length M
    const cplx<T> *tw_x, *tw_y, *tw_z, *tw_r2c; // tw_r2c: exp(-2 pi i k/nz), k <= M
    cplx<T>       *spec;           // C * nx * ny * nzp
    const T       *G;              // [nx][ny][gzs][C(C+1)/2], kz < nzh filled
    int            gzs;            // kz row stride of G (nzh for FP64; nzp for FP32, so rows start on 16 bytes)
    int            kc_y, kc_x;     // kz columns per CTA in the y / x passes
    int            use_reg;        // register-resident passes (conv_reg_supported)
    int            var_z, var_y, var_x; // register passes: tile variant (0 default, 1 the alternative)
    int            fuse_zy;        // FP32: the forward z and y passes as one cluster pass (k_zy_fwd)
    // register passes: the fused <r, s> of a reducing convolution is taken in the x pass from the
    // spectra (Parseval) instead of in the z-inverse pass from r and s, which then reads no r
    int            spectral_dot;
    // register passes over several right-hand sides: RHS k's rows follow RHS k-1's (r, s and spec
    // of nrhs consecutive fields; the Green's table is shared); active[k] == 0 skips RHS k
    int            nrhs;
    const int     *active;
    // FP32 x pass fed by the tensor memory accelerator (var_x == 2): host pointer to the
    // TmaMaps of this plan's spectrum and Green's table, or null where none were made
    const void    *tma;
    int            nrhs_alloc; // right-hand sides the spectrum buffer holds (the tensor map's extent)
};

// Tensor maps of the TMA-fed x pass (host side, one per FP32 plan): the spectrum as floats
// [nrhs_alloc * C * nx][ny][2 * nzh] (row stride 2 * nzp) and the Green's table as floats
// [nx][ny][nzh * NT] (row stride nzp * NT), both with boxes of KC = 8 kz columns by all kx.
struct TmaMaps {
    alignas(64) unsigned char spec[128];
    alignas(64) unsigned char green[128];
};
// Encode the maps of an FP32 plan (spec, G, gzs, nrhs_alloc set); false if the driver has no
// tensor-map encoder or the shapes do not fit a tensor map.
bool make_x_tma_maps(const ConvPlan<float> &p, TmaMaps *out);

// s = sign * IFFT(G . FFT(r)); with reduce, <r, s> -> scal (delta0, delta,
// beta) as in solverCG.h:86-94.
struct ConvArgs {
    const void *r;
    void       *s;
    double      sign;
    int         reduce;
    CgScalars  *scal;
    GridRed     red;
    int         red_site;
    cudaEvent_t *ev; // optional: 6 events recorded around the 5 passes
};
template <typename T>
cudaError_t launch_convolution(const ConvPlan<T> &p, const ConvArgs &a, cudaStream_t st);
template <typename T>
size_t conv_smem_bytes(const ConvPlan<T> &p, int pass);
// register-resident passes (line lengths with a two-phase register plan)
bool conv_reg_supported(const Grid3 &g);
// the fused z + y forward cluster pass exists for this grid (FP32, nz == ny)
bool zy_supported(const Grid3 &g);
template <typename T>
cudaError_t launch_convolution_reg(const ConvPlan<T> &p, const ConvArgs &a, cudaStream_t st);
// Times the register passes' tile variants on p's buffers (r in, s out) and
// stores the faster ones in p.var_z / var_y / var_x.
template <typename T>
// times the tile variants as the CG iteration runs them: the z-inverse pass with its fused
// <r, s> reduction (into `scal`, scratch scalars, through `red` at `red_site`)
cudaError_t tune_convolution_reg(ConvPlan<T> &p, const T *r, T *s, CgScalars *scal, GridRed red, int red_site,
                                 cudaStream_t st);

// Green's table (solver.h:145-204) in FP64, optionally also rounded to FP32.
struct GreenArgs {
    Grid3         g;
    int           C;
    const double *K0c;   // 8C x 8C, component-major ("C groups of 8")
    const double *cx, *sx, *cy, *sy, *cz, *sz; // cos/sin(2 pi k / n)
    double       *G64;
    float        *G32;   // optional; kz row stride g32s
    int           g32s;
};
cudaError_t launch_green(const GreenArgs &a, cudaStream_t st);

// ------------------------------------------------------------------ CG vec ---
// r -= alpha*Kd; u -= alpha*d (alpha from scal); err = ||r|| (measure) and
// deltamid = <r, s> -> scal.  T: type of r, Kd, d, s; TU: type of u.
struct UpdateArgs {
    long long  n;
    void      *r;
    const void *Kd;
    void      *u;
    const void *d;
    const void *s;
    int        measure;
    int        do_u;
    CgScalars *scal;
    GridRed    red;
    int        red_site;
    int        nrhs;       // FP32 16-byte update: nrhs consecutive fields of n values (0 or 1: one)
    const int *active;     // active[k] == 0 skips RHS k (null: all active)
};
template <typename T, typename TU>
cudaError_t launch_cg_update(const UpdateArgs &a, cudaStream_t st);

// err = ||r|| (measure) -> scal->err (and err0 if set_err0); optionally also
// writes a copy of r converted to `r_out` (mixed precision re-seed).
template <typename T, typename TO>
cudaError_t launch_norm(const T *r, long long n, int measure, CgScalars *scal, int set_err0, TO *r_out, GridRed red,
                        int red_site, cudaStream_t st);

// Mixed path: ||r|| of the FP64 true residual with FP32 squares / short partial
// sums (FP64 accumulation across them) and the FP32 re-seed copy.
cudaError_t launch_norm_fast(const double *r, long long n, int measure, CgScalars *scal, int set_err0, float *r_out,
                             GridRed red, int site, cudaStream_t st);

// u -= s (fixed-point update, solverFP.h:38).
template <typename T>
cudaError_t launch_axpy(T *y, const T *x, double a, long long n, cudaStream_t st);

// u = u + (u - u_prev); u_prev = u_old (solver.h:303-311).
cudaError_t launch_extrapolate(double *u, double *u_prev, long long n, cudaStream_t st);

// u64 += e32 (mixed precision: fold the FP32 correction into the FP64 solution).
cudaError_t launch_fold(double *u, float *e, long long n, cudaStream_t st);

// uint16 phase ids -> uint8 on the device, atomically folding the maximum id
// into *max_id (caller zeroes it).
cudaError_t launch_ms_convert(const uint16_t *in, uint8_t *out, long long n, unsigned int *max_id, cudaStream_t st);

int grid_blocks_for(long long n);

// number of CTAs of the stencil kernel for grid g
long long stencil_blocks(const Grid3 &g);

} // namespace fansgpu
