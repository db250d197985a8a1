/*
 * fans_gb300.h -- C ABI of the GB300-native FANS solve path.
 *
 * One context = one FANS Solver on one GPU: a periodic voxel grid, its
 * microstructure (phase id per voxel), the per-phase material laws, the
 * reference material, the macroscopic gradient and the solver state.  All
 * device memory is owned by the context; callers pass host buffers and get
 * host results.  Every entry point returns 0 on success or a negative
 * FANSGPU_E* code; fansgpu_last_error() gives a one-line message.
 *
 * Host field layout at this boundary is the reference's: nodal fields
 * [x][y][z][c] with c fastest (solver.h:123-127, without FFTW padding),
 * element fields [x][y][z][n_str], microstructure uint16 [x][y][z]
 * (reader.cpp:380-398).  Strains/stresses use FANS's Mandel ordering
 * (11, 22, 33, sqrt2*12, sqrt2*13, sqrt2*23) (matmodel.h:284-304).
 *
 * Each declaration names the reference interface it replaces
 * (FANS v0.6.2, file:line).
 */
#ifndef FANS_GB300_H
#define FANS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define FANSGPU_OK 0
#define FANSGPU_EINVAL -1      /* bad argument (std::invalid_argument in the reference) */
#define FANSGPU_ENOMEM -2      /* device allocation failed (std::bad_alloc) */
#define FANSGPU_ECUDA -3       /* CUDA runtime error */
#define FANSGPU_ENOTCONV -4    /* n_it reached before the tolerance (reported, not fatal) */
#define FANSGPU_ENAN -5        /* NaN/Inf found in the residual norm */
#define FANSGPU_EUNSUPPORTED -6 /* valid FANS input this build does not handle (named in the message) */
#define FANSGPU_ESTATE -7      /* call order violated (e.g. solve before set_microstructure) */

/* FE_type (reader.cpp:121-128, matmodel.h:82-88) */
#define FANSGPU_HEX8 0
#define FANSGPU_HEX8R 1
#define FANSGPU_BBAR 2

/* material laws (setup.h:22-73); parameter vectors per phase:
 *   THERMAL_ISO  {conductivity}                                   LinearThermal.h:7-50
 *   ELASTIC_ISO  {bulk_modulus, shear_modulus}                    LinearElastic.h:7-75
 *   J2_LINEAR    {bulk, shear, yield_stress, isotropic_hardening} J2PlasticityNew.h:7-152
 *   THERMAL_TRI  {K (3x3 row-major)}                              LinearThermal.h:52-118
 *   ELASTIC_TRI  {C (6x6 row-major, Mandel)}                      LinearElastic.h:77-159
 *   PSEUDO_LINEAR    {bulk, shear, yield_stress, hardening_parameter
 *                     [, index in its material group, phases in the group]}  PseudoPlastic.h:80-122
 *   PSEUDO_NONLINEAR {bulk, shear, yield_stress, hardening_exponent, eps_0
 *                     [, index in its material group, phases in the group]}  PseudoPlastic.h:124-167
 *   (the optional pair sets the plastic_flag values, mat_index / n_mat + mat_index)
 *   J2VISCO_LINEAR    {bulk, shear, yield_stress, isotropic_hardening, kinematic_hardening,
 *                      viscosity, time_step}                        J2Plasticity.h:7-185
 *   J2VISCO_NONLINEAR {... as J2VISCO_LINEAR, saturation_stress, saturation_exponent}
 *                                                                  J2Plasticity.h:187-245 */
#define FANSGPU_LAW_THERMAL_ISO 0
#define FANSGPU_LAW_ELASTIC_ISO 1
#define FANSGPU_LAW_J2_LINEAR 2
#define FANSGPU_LAW_THERMAL_TRI 3
#define FANSGPU_LAW_ELASTIC_TRI 4
#define FANSGPU_LAW_PSEUDO_LINEAR 5
#define FANSGPU_LAW_PSEUDO_NONLINEAR 6
#define FANSGPU_LAW_J2VISCO_LINEAR 7
#define FANSGPU_LAW_J2VISCO_NONLINEAR 8
#define FANSGPU_LAW_SVK 9         /* SaintVenantKirchhoff {bulk, shear} (large strain) */
#define FANSGPU_LAW_NEOHOOKEAN 10 /* CompressibleNeoHookean {bulk, shear} (large strain) */

/* precision of the solve */
#define FANSGPU_FP64 0  /* all FP64: parity path against the FP64 reference */
#define FANSGPU_MIXED 1 /* FP32 stencil + FFT preconditioner inside an FP64 reliable-update loop */

/* method (setup.h:76-85) */
#define FANSGPU_CG 0
#define FANSGPU_FP 1
/* Newton-Krylov (new on the GPU path; FP64, strain control, J2PlasticityNew and
 * linear elastic phases): outer Newton steps on R(u) = 0, each an inexact
 * consistent-tangent solve by the Green's-preconditioned CG (Eisenstat-Walker
 * tolerance) with backtracking.  fansgpu_stats.iterations counts Newton steps,
 * fansgpu_stats.refinements the inner CG iterations. */
#define FANSGPU_NEWTON 2

/* error_parameters (solver.h:415-452) */
#define FANSGPU_L1 0
#define FANSGPU_L2 1
#define FANSGPU_LINF 2
#define FANSGPU_ABSOLUTE 0
#define FANSGPU_RELATIVE 1

/* fields for get/set (solver.h:34-38, :455-705) */
#define FANSGPU_FIELD_U 0        /* displacement/temperature fluctuation v_u, [x][y][z][c] */
#define FANSGPU_FIELD_R 1        /* residual v_r, [x][y][z][c] */
#define FANSGPU_FIELD_STRAIN 2   /* element-averaged strain/gradient, [x][y][z][n_str] */
#define FANSGPU_FIELD_STRESS 3   /* element-averaged stress/flux, [x][y][z][n_str] */
#define FANSGPU_FIELD_U_PREV 4   /* previous step displacement (extrapolation) */
#define FANSGPU_FIELD_PLASTIC_STRAIN 5 /* J2: Gauss-point mean of committed eps_p, [x][y][z][6] (get_field only) */
#define FANSGPU_FIELD_HARDENING 6      /* J2: Gauss-point mean of committed q, [x][y][z] (get_field only) */
#define FANSGPU_FIELD_STRAIN_GP 7          /* strain at every Gauss point, [x][y][z][n_gp][n_str] (get_field only) */
#define FANSGPU_FIELD_STRESS_GP 8          /* stress at every Gauss point, [x][y][z][n_gp][n_str] (get_field only) */
#define FANSGPU_FIELD_PLASTIC_STRAIN_GP 9  /* J2: committed eps_p, [x][y][z][n_gp][6] (get_field only) */
#define FANSGPU_FIELD_HARDENING_GP 10      /* J2: committed q, [x][y][z][n_gp] (get_field only) */
#define FANSGPU_FIELD_PLASTIC_FLAG 11      /* PseudoPlastic: Gauss-point mean of the plastic flag, [x][y][z] */
#define FANSGPU_FIELD_KINEMATIC 12         /* J2ViscoPlastic: Gauss-point mean of committed psi_bar, [x][y][z][6] */
#define FANSGPU_FIELD_KINEMATIC_GP 13      /* J2ViscoPlastic: committed psi_bar, [x][y][z][n_gp][6] */

typedef struct fansgpu_ctx fansgpu_ctx;

/* Grid + discretisation: Reader fields dims/L/FE_type/problem_type
 * (reader.h:24-63) and the Solver template arguments <howmany, n_str>. */
typedef struct {
    int32_t n[3];      /* voxels n_x, n_y, n_z (each even, 4..1024) */
    double  L[3];      /* microstructure box lengths (reader.cpp:83) */
    int32_t howmany;     /* 1: thermal <1,3>; 3: mechanics (main.cpp:67-75) */
    int32_t fe_type;     /* FANSGPU_HEX8 / HEX8R / BBAR */
    int32_t precision;   /* FANSGPU_FP64 / FANSGPU_MIXED */
    int32_t method;      /* FANSGPU_CG / FANSGPU_FP / FANSGPU_NEWTON */
    int32_t strain_type; /* FANSGPU_SMALL_STRAIN <3,6> (0, default) or FANSGPU_LARGE_STRAIN <3,9> */
    int32_t n_rhs;       /* right-hand sides (load cases) held and solved together: 1..FANSGPU_MAX_RHS
                            (0 means 1).  FANS runs its load cases one Solver after another
                            (main.cpp:14-41) and its linear tangent as n_str solves (solver.h:759-776);
                            here they share one solve (see fansgpu_set_gradients) */
} fansgpu_desc;

#define FANSGPU_MAX_RHS 6

#define FANSGPU_SMALL_STRAIN 0
#define FANSGPU_LARGE_STRAIN 1 /* n_str = 9: g0 and strains are the deformation gradient F (row-major),
                                  stresses the first Piola-Kirchhoff stress P (LargeStrainMechModel.h) */

/* error_parameters, n_it and linesearch_parameters (reader.cpp:94-105). */
typedef struct {
    int32_t measure;     /* FANSGPU_L1 / L2 / LINF */
    int32_t type;        /* FANSGPU_ABSOLUTE / RELATIVE */
    double  tolerance;
    int32_t n_it;
    int32_t ls_max_iter; /* default 5 (reader.h:33) */
    double  ls_tol;      /* default 1e-2 (reader.h:34) */
} fansgpu_tol;

typedef struct {
    int32_t iterations;       /* Solver::iter after internalSolve */
    int32_t converged;        /* 1 if the tolerance was met */
    double  err0;             /* err_all[0] */
    double  err;              /* err_all[iter] (absolute, in the configured measure) */
    int32_t refinements;      /* MIXED: FP64 true-residual evaluations after the first */
    double  solve_ms;         /* device time of the solve (CUDA events) */
} fansgpu_stats;

/* Solver ctor (solver.h:105-142, solverCG.h:36-50): allocates all device state.
 * Replaces `createSolver` (setup.h:76-85) + `Solver<h,n>::Solver`. */
int fansgpu_create(const fansgpu_desc *desc, fansgpu_ctx **out);

/* Solver dtor (solver.h:780-805, solverCG.h:162-177). */
int fansgpu_destroy(fansgpu_ctx *ctx);

/* One-line message for the last failing call on this context (NULL ctx: last
 * failure of a call made without a context: fansgpu_create or
 * fansgpu_residual_norm_noalloc). */
const char *fansgpu_last_error(const fansgpu_ctx *ctx);

/* Reader::ReadMS result (reader.cpp:227-411): phase id per voxel, uint16 [x][y][z]. */
int fansgpu_set_microstructure(fansgpu_ctx *ctx, const uint16_t *ms_xyz);

/* MaterialManager phase table (MaterialManager.h:86-103): the law and
 * parameters of one phase (see FANSGPU_LAW_*).  All phases that occur in the
 * microstructure must be assigned before the first solve. */
int fansgpu_set_phase_material(fansgpu_ctx *ctx, int32_t phase, int32_t law, const double *params,
                               int32_t n_params);

/* MaterialManager::compute_reference_stiffness (MaterialManager.h:177-205):
 * kapparef_mat (n_str x n_str, row-major).  Must be set before the first solve;
 * the host mirror computes the reference's default rule.  Small strain and
 * thermal: symmetric positive definite (FANSGPU_EINVAL otherwise); large
 * strain: symmetric (dP/dF at F = I is semidefinite). */
int fansgpu_set_reference(fansgpu_ctx *ctx, const double *kapparef);

/* MaterialManager::set_gradient / Matmodel::setGradient (MaterialManager.h:216-221,
 * matmodel.h:228-236): macroscopic gradient g0 (n_str). */
int fansgpu_set_gradient(fansgpu_ctx *ctx, const double *g0);

/* MixedBCController (mixedBCs.h:149-227, solver.h:71-85): activate mixed
 * stress/strain control for time step `step` of a mixed load case.  idx_e are
 * the strain-controlled Mandel components with this step's values strain_e,
 * idx_f the stress-controlled ones with target stresses stress_f; together they
 * cover each component once.  Step 0 starts from g0 = 0; later steps
 * extrapolate the stress-controlled components linearly.  While active, the CG
 * solve takes the line-search branch (solverCG.h:96) and updates g0 before
 * every residual (solverCG.h:131, :152; solverFP.h:47).  Needs set_reference. */
int fansgpu_enable_mixed_bc(fansgpu_ctx *ctx, int32_t n_e, const int32_t *idx_e, const double *strain_e, int32_t n_f,
                            const int32_t *idx_f, const double *stress_f, int32_t step);
/* Per-voxel material field (new on the GPU path; FANS has one law per phase):
 * FANSGPU_VOXEL_STIFFNESS_SCALE multiplies the stress of voxel element e by
 * values[e] > 0 ([x][y][z] doubles), i.e. K_e = s_e K_phase for linear laws --
 * E(x) = s(x) E_phase at fixed Poisson ratio.  NULL clears it.  With a scale
 * set, solves run the FP64 path with the element kernel as operator. */
#define FANSGPU_VOXEL_STIFFNESS_SCALE 0
/* FANSGPU_VOXEL_YIELD_STRESS replaces the initial yield stress sigma_y of
 * J2PlasticityNew (J2PlasticityNew.h:43-108, a per-phase parameter there) by
 * values[e] > 0 in voxel e; other laws ignore it.  NULL clears it. */
#define FANSGPU_VOXEL_YIELD_STRESS 1
int fansgpu_set_voxel_field(fansgpu_ctx *ctx, int32_t field, const double *values);

/* The tile shapes and operators the context's first setup chose (autotuned
 * unless FANSGPU_TUNE=0 or forced), out[8]: out[0..2] = FP64 z, y, x pass
 * variants, out[3..5] the FP32 ones (0 = default tile, 1 = the smaller one;
 * FP32 x pass only: 2 = the persistent pass fed by tensor-map (TMA) copies;
 * FP32 z entry: + 2 when the forward z and y passes run as one cluster pass),
 * out[6] = the mixed path's CG operator (0 CUDA cores, 1 per-phase tensor-core,
 * 2 exact-basis tensor-core over all right-hand sides, 3 the per-phase tensor-core
 * operator once per right-hand side of the multi-RHS iteration), out[7] = the FP64-accurate operator (the FP64 CG
 * operator, and the mixed path's true residual: 0 FP64 pipe, 1 double-float on
 * the CUDA cores, 2 exact fixed-point slices on the tensor cores).  New on the
 * GPU path (FANS's FFTW plans are chosen by FFTW_MEASURE, solver.h:221-222). */
int fansgpu_tuning(fansgpu_ctx *ctx, int32_t *out);

/* Adjoint of the homogenized stiffness w.r.t. the per-voxel scale.  After
 * solves with g0 = e_k, fansgpu_store_solution(ctx, k) keeps v_u and g0 (slots
 * 0..5).  fansgpu_stiffness_gradient returns grad[e] = d(sum_ij W_ij C_ij)/d s_e
 * for the energy-form C_ij = (1/N) sum_e s_e mean_gp eps_i^T C_ph eps_j of the
 * stored solutions (equal to <sigma_j>_i at equilibrium; no adjoint solve is
 * needed because the displacement fields are stationary).  W is n x n
 * row-major; grad holds n_x*n_y*n_z doubles [x][y][z].  Linear laws only. */
int fansgpu_store_solution(fansgpu_ctx *ctx, int32_t slot);
int fansgpu_stiffness_gradient(fansgpu_ctx *ctx, int32_t n, const double *W, double *grad);

/* Adjoint of the final homogenized stress of a strain-controlled load path
 * w.r.t. the per-voxel initial yield stress (J2PlasticityNew with linear
 * isotropic hardening, linear elastic phases beside it; small strain, CG).
 * Runs the path as runSolver does (main.cpp:23-42): for k = 1..n_steps,
 * g0 = g0_path[k-1] (6 Mandel components), solve (committing the internal
 * variables), extrapolate the displacement; starting from the context's
 * current u and committed state.  It keeps every converged u_k and the
 * committed internal variables every `checkpoint_every` steps, then sweeps
 * backwards: per step one linear CG solve with the consistent tangent
 * (K_k^T lambda_k = -f_k, relative L2 tolerance rel_tol, at most the
 * context's n_it iterations), the states inside a checkpoint segment being
 * recomputed from its checkpoint by the return map alone.
 * Returns stress_final = <sigma> after the last step (n_str doubles, may be
 * NULL), grad[e] = d(w . stress_final)/d sigma_y(e) ([x][y][z] doubles, zero in
 * elastic voxels) and, if iterations is not NULL, the forward CG iterations of
 * each step followed by the adjoint CG iterations of each step (2 n_steps
 * ints).  The context ends in the state after the last step.  The gradient is
 * that of the discrete converged path: the committed state at entry is taken
 * as independent of sigma_y.  Device memory: n_steps displacement fields,
 * ceil(n_steps / checkpoint_every) + checkpoint_every internal-variable sets. */
int fansgpu_yield_stress_adjoint(fansgpu_ctx *ctx, int32_t n_steps, const double *g0_path, int32_t checkpoint_every,
                                 const double *w, double rel_tol, double *stress_final, double *grad,
                                 int32_t *iterations);

/* Solver::disableMixedBC (solver.h:75-78). */
int fansgpu_disable_mixed_bc(fansgpu_ctx *ctx);
/* The current macroscale gradient g0 (n_str values; under mixed BCs the
 * controller's current strain). */
int fansgpu_get_gradient(fansgpu_ctx *ctx, double *g0);

/* Reader error_parameters / n_it / linesearch_parameters (reader.cpp:94-105). */
int fansgpu_set_tolerance(fansgpu_ctx *ctx, const fansgpu_tol *tol);

/* Solver::solve (solver.h:283-300) -> SolverCG::internalSolve (solverCG.h:62-117)
 * or SolverFP::internalSolve (solverFP.h:33-52), then commit of internal
 * variables (solver.h:299).  stats may be NULL.  Returns FANSGPU_ENOTCONV when
 * n_it was reached (the state is still valid, as in the reference). */
int fansgpu_solve(fansgpu_ctx *ctx, fansgpu_stats *stats);

/* Several right-hand sides (fansgpu_desc.n_rhs > 1; new on the GPU path): the
 * context holds one displacement, residual and solver state per RHS.  Each RHS
 * is one FANS load case with its own macroscopic gradient -- the n_str unit
 * gradients of the linear homogenized tangent (solver.h:759-776), or the load
 * cases of an input file (main.cpp:14-41).
 *   fansgpu_set_gradients: g0 of every RHS (n_rhs x n_str, row-major; n must
 *     equal n_rhs).
 *   fansgpu_solve: solves every RHS.  Linear laws only (internal variables are
 *     per solve), strain control, CG or FP.  With MIXED precision on the
 *     tensor-core path all RHS run as one multi-RHS CG: every kernel of an
 *     iteration covers all of them (the Green's table is read once per
 *     iteration for all RHS), each RHS keeps its own CG scalars, reliable
 *     updates and convergence test, and leaves the iteration once converged;
 *     the per-RHS results equal those of separate solves.  Otherwise the RHS are
 *     solved one after another.  stats (may be NULL) gets the aggregate: the
 *     largest iteration count, converged = all converged, err0 / err of the
 *     RHS with the largest relative error, refinements summed.
 *   fansgpu_select_rhs: the RHS that fansgpu_set_gradient, _homogenized_stress,
 *     _homogenized_tangent, _postprocess_averages, _get_field / _set_field,
 *     _get_error_history, _store_solution, _residual, _apply_operator and
 *     _convolve act on (default 0).  fansgpu_reset and
 *     fansgpu_extrapolate_displacement act on every RHS.
 *   fansgpu_rhs_stats: the last solve's statistics of RHS k. */
int fansgpu_set_gradients(fansgpu_ctx *ctx, int32_t n, const double *g0);
int fansgpu_select_rhs(fansgpu_ctx *ctx, int32_t k);
int fansgpu_rhs_stats(fansgpu_ctx *ctx, int32_t k, fansgpu_stats *stats);

/* Independent solves of several contexts at once (batched micro problems, e.g.
 * one per macroscopic integration point): each context's fansgpu_solve runs on
 * its own host thread and CUDA stream, so small problems overlap on the GPU.
 * stats and rc (either may be NULL) receive per-context results; returns 0 or
 * the last hard error (ENOTCONV is reported per context only).  Contexts must
 * be distinct and not used by other threads meanwhile. */
int fansgpu_solve_batch(fansgpu_ctx *const *ctxs, int32_t n, fansgpu_stats *stats, int32_t *rc);

/* Solver::get_homogenized_stress (solver.h:708-737): volume average of the
 * element-averaged stress/flux (n_str doubles). */
int fansgpu_homogenized_stress(fansgpu_ctx *ctx, double *out);

/* Solver::get_homogenized_tangent (solver.h:740-778): n_str x n_str,
 * row-major, symmetrised.  Linear laws: unit-gradient solves; nonlinear: FD
 * with pert_param.  Like the reference it leaves the context's error type
 * relative and the tolerance at max(1e-6, tol), and v_u at the last solve. */
int fansgpu_homogenized_tangent(fansgpu_ctx *ctx, double pert_param, double *out);

/* Solver::postprocess averages (solver.h:469-574): strain/stress averages and
 * per-phase averages (n_phase x n_str, phases in id order) with counts.
 * Any pointer may be NULL. */
int fansgpu_postprocess_averages(fansgpu_ctx *ctx, double *strain_avg, double *stress_avg, double *phase_strain,
                                 double *phase_stress, int64_t *phase_count, int32_t n_phase);

/* Field access (v_u, v_r, postprocess fields).  `host` holds n_x*n_y*n_z*k doubles. */
int fansgpu_get_field(fansgpu_ctx *ctx, int32_t which, double *host);
int fansgpu_set_field(fansgpu_ctx *ctx, int32_t which, const double *host);

/* err_all (solver.h:44, :432): up to max_n entries of the last solve's history. */
int fansgpu_get_error_history(fansgpu_ctx *ctx, double *out, int32_t max_n, int32_t *n_out);

/* Solver::extrapolateDisplacement (solver.h:303-311). */
int fansgpu_extrapolate_displacement(fansgpu_ctx *ctx);

/* MaterialManager::update_internal_variables (MaterialManager.h:207-213). */
int fansgpu_commit_state(fansgpu_ctx *ctx);

/* ---- kernel-level entry points (one hot-path stage each, FP64, host buffers) ---- */

/* Solver::compute_residual (solver.h:272-280): r = R(u) with the current g0.
 * u, r: [x][y][z][c]. */
int fansgpu_residual(fansgpu_ctx *ctx, const double *u, double *r);

/* The CG linear operator (solverCG.h:97-103): y = sum_e A_e^T K_phase(e) x_e. */
int fansgpu_apply_operator(fansgpu_ctx *ctx, const double *x, double *y);

/* Solver::convolution (solver.h:388-412): s = IFFT(G . FFT(r)), unnormalised
 * transforms with 1/N folded into G. */
int fansgpu_convolve(fansgpu_ctx *ctx, const double *r, double *s);

/* Solver::computeFundamentalSolution (solver.h:145-204): the Green's table,
 * [kx][ky][kz] (kz < n_z/2+1) x c(c+1)/2 lower-triangle entries (00,10,11,20,21,22). */
int fansgpu_green_table(fansgpu_ctx *ctx, double *host);

/* Solver ctor state for a new load case (solver.h:133-137, main.cpp:15-16):
 * zero v_u, v_u_prev and v_r without reallocating. */
int fansgpu_reset(fansgpu_ctx *ctx);

/* The CUDA stream (cudaStream_t) all work of this context is ordered on, so a
 * caller can order its own work or CUDA events against it.  No reference
 * counterpart (the reference has no device work). */
int fansgpu_get_stream(fansgpu_ctx *ctx, void **stream);

/* Per-kernel device time.  With timing on, every launch of the solve path is
 * bracketed by CUDA events on the context stream and accumulated per kernel id
 * (FANSGPU_K_*).  The reference prints per-iteration FFT and total CPU times
 * (solver.h:286-298); this is its device-side counterpart. */
#define FANSGPU_K_STENCIL 0   /* fused d = s + beta d; K d; <d, K d> */
#define FANSGPU_K_FFT_Z_FWD 1 /* r2c along z */
#define FANSGPU_K_FFT_Y_FWD 2
#define FANSGPU_K_FFT_X_GREEN 3 /* x FFT, Green multiply, inverse x FFT */
#define FANSGPU_K_FFT_Y_INV 4
#define FANSGPU_K_FFT_Z_INV 5 /* c2r along z, negation, <r, s> */
#define FANSGPU_K_UPDATE 6    /* r -= a Kd, u -= a d, ||r||, <r, s> */
#define FANSGPU_K_RESIDUAL 7  /* FP64 R(u) = K u + F */
#define FANSGPU_K_NORM 8      /* ||r|| (and FP32 re-seed) */
#define FANSGPU_K_GREEN 9     /* Green's table build */
#define FANSGPU_K_STRAIN_STRESS 10 /* element strain/stress + volume averages */
#define FANSGPU_K_COUNT 11
int fansgpu_set_timing(fansgpu_ctx *ctx, int32_t on);
int fansgpu_kernel_times(fansgpu_ctx *ctx, double *ms_total, int64_t *launches, int32_t n);

/* Residual norm (the measure of Solver::compute_error) of a field that already
 * lives in device memory, with no device allocation: no counterpart in the
 * reference.  For callers that cannot call cudaMalloc -- e.g. a process whose
 * device memory is all held by another allocator, or code that must not
 * trigger the device synchronisation cudaMalloc/cudaFree can cause.  Needs no
 * context.  r_dev: n doubles on the current device; *out_dev (device memory)
 * receives ||r|| in `measure` (FANSGPU_L1 / L2 / LINF), ordered on `stream`
 * (a cudaStream_t, NULL = default stream).  The scratch is a static array of
 * 256 KiB + 256 B that every GPU loading the library holds until exit; n is
 * limited to FANSGPU_NOALLOC_MAX_VALUES (FANSGPU_EINVAL beyond).  Each call
 * made outside stream capture looks the array's device address up
 * (cudaGetSymbolAddress); a call made while `stream` is being captured reuses
 * the address the last earlier call on that device found, so the first call on
 * a device must come before any stream capture (FANSGPU_ESTATE otherwise).  All
 * calls on a GPU share the array: calls that overlap on the GPU race and must
 * be serialised.  Errors are reported through fansgpu_last_error(NULL), which
 * is per calling thread. */
#define FANSGPU_NOALLOC_MAX_VALUES 268435456LL
int fansgpu_residual_norm_noalloc(const double *r_dev, int64_t n, int32_t measure, double *out_dev, void *stream);

/* MIXED precision: the factor by which the FP32 residual must fall since the
 * last FP64 true-residual refresh before the next one (default 1e-4; (0, 1)).
 * No reference counterpart (the reference runs in FP64 only). */
int fansgpu_set_refresh(fansgpu_ctx *ctx, double factor);

/* Diagnostics: the bound on each pipeline wait of the tensor-core operator
 * (MIXED precision), in mbarrier polls; 0 restores the default (2^22 polls,
 * far beyond any wait of a healthy launch).  A wait that runs out sets an
 * abort flag that releases every other wait of its CTA; the CTA then waits for
 * its own MMAs in flight, frees its tensor memory and returns, and the solve
 * reports FANSGPU_ECUDA ("... wait timed out") with the context still usable.
 * A small bound lets a test make the waits expire on purpose.  No reference
 * counterpart (the reference has no device work). */
int fansgpu_set_wait_limit(fansgpu_ctx *ctx, int32_t polls);

/* Diagnostics: the device's FP64 FMA rate (FMAs per second), measured by a
 * short kernel of independent FMA chains on every SM of the current device.
 * The FP64 solve path is bound by this rate, not by HBM; bench.py reports the
 * FP64 operator's fraction of it.  No reference counterpart. */
int fansgpu_fp64_fma_rate(double *dfma_per_s);

/* Library version string. */
const char *fansgpu_version(void);

#ifdef __cplusplus
}
#endif
#endif /* FANS_GB300_H */
