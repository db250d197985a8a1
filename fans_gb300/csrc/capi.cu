// capi.cu -- the C ABI (include/fans_gb300.h): context, setup and the solve
// loops of SolverCG / SolverFP (solverCG.h:62-117, solverFP.h:33-52) driving
// the fused sm_103a kernels.  Host code only orchestrates; every per-voxel
// operation runs on the GPU.
#include "../../include/fans_gb300.h"
#include "fe_host.hpp"
#include "kernels.cuh"

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include <thread>
#include <atomic>
#include <array>
#include <map>
#include <mutex>

using namespace fansgpu;

// Message of the last failing call made without a context, per calling thread
// (fansgpu_last_error(NULL) reads the caller's own copy).
static thread_local std::string g_create_error;

// Controls of the device-resident inner loop of the mixed CG.
struct LoopCtl {
    double err0, last_true, tol, reliable;
    int    iter, n_it, relative, cap;
};
// The same for the multi-RHS loop: per right-hand side err0 and the last true residual.
struct LoopCtlR {
    double err0[kMaxRhs], last_true[kMaxRhs], tol, reliable;
    int    iter, n_it, relative, cap, nrhs;
};

struct fansgpu_ctx {
    fansgpu_desc desc{};
    Grid3        g{};
    int          C = 1, nstr = 3, ngp = 8;
    long long    N = 0, n = 0;
    double       le[3]{}, ve = 0;
    std::vector<double> B, Bbar;

    // materials
    int                              nph = 0; // phases in the table: max(1 + max id in ms, assigned)
    int                              ms_max = 0;
    std::vector<int>                 law;
    std::vector<std::vector<double>> prm;
    std::vector<char>                assigned;
    bool have_ms = false, have_ref = false, tables_dirty = true, force_dirty = true, green_dirty = true;
    bool all_linear = true;
    std::vector<double> kapparef, g0;
    fansgpu_tol tol{FANSGPU_L2, FANSGPU_RELATIVE, 1e-10, 100, 5, 1e-2};
    double      reliable_delta = 1e-4; // MIXED: true-residual refresh when the FP32 residual fell by this factor

    cudaStream_t st = nullptr;
    cudaEvent_t  ev0 = nullptr, ev1 = nullptr;
    uint8_t     *d_ms = nullptr;
    double *u = nullptr, *r = nullptr, *s = nullptr, *dd[2] = {nullptr, nullptr}, *Kd = nullptr, *uprev = nullptr;
    float  *r32 = nullptr, *s32 = nullptr, *d32[2] = {nullptr, nullptr}, *Kd32 = nullptr, *e32 = nullptr;
    std::vector<double> K64h, f64h; // host copies of the per-phase tables (kernel-parameter path)
    float              *Kdf = nullptr, *fdf = nullptr; // double-float [hi | lo] tables (mixed refresh)
    size_t              fdf_cap = 0;
    std::vector<float>  K32h;
    bool                u_zero = true; // v_u known to be zero (fresh context / reset): R(u) = F
    double *K64 = nullptr, *f64 = nullptr, *Cph = nullptr, *Bbar_d = nullptr, *g0_d = nullptr, *K0c = nullptr;
    double *fnode = nullptr; // r = F at u = 0 for <= 2 phases: 256 x C node sums by element-phase key
    double *Bgp_d = nullptr; // Gauss-point B matrices, ngp x n_str x 8C
    double *Bb_d  = nullptr; // basic B (dN_q/dx_j) per Gauss point, ngp x 3 x 8: HEX8 / HEX8R mechanics
    float  *K32 = nullptr;
    double *G64 = nullptr;
    float  *G32 = nullptr;
    TmaMaps tmaps{}; // tensor maps of the FP32 spectrum and Green's table (TMA-fed x pass)
    bool    spectral_dot = true; // FP32 convolutions take <r, s> from the spectra in the x pass
    cplx<double> *spec64 = nullptr, *tw64 = nullptr;
    cplx<float>  *spec32 = nullptr, *tw32 = nullptr;
    double       *trig = nullptr; // cos/sin tables for the Green's table
    double       *staging = nullptr;
    CgScalars    *scal = nullptr, *scal_h = nullptr;
    GridRed       red{};
    double       *red_out = nullptr;
    ConvPlan<double> cp64{};
    ConvPlan<float>  cp32{};
    int              cur_d = 0;

    std::vector<double> err_all;
    int                 iter = 0;
    std::string         err_msg;

    // per-kernel CUDA-event timing (fansgpu_set_timing)
    struct Span {
        int id, e0, e1;
    };
    bool                     timing = false;
    std::vector<cudaEvent_t> tpool;
    int                      tused = 0;
    std::vector<Span>        spans;
    double                   ktime[FANSGPU_K_COUNT] = {0};
    int64_t                  kcount[FANSGPU_K_COUNT] = {0};
    unsigned int            *max_id = nullptr;

    // nonlinear laws (J2PlasticityNew): internal variables SoA eps_p [6][ngp][N], q [ngp][N],
    // committed (_t) and trial copies; element-row scratch [8C][N] for the residual gather
    double *ep_t = nullptr, *q_t = nullptr, *ep = nullptr, *q = nullptr, *rows = nullptr;
    double *pb_t = nullptr, *pb = nullptr; // J2ViscoPlastic kinematic hardening [6][ngp][N]
    int    *law_d = nullptr;
    double *prm_d = nullptr;
    double  alpha_warm = 0.1;
    bool    newton_stalled = false; // the last Newton solve stopped without a decrease (u restored)

    // per-voxel stiffness scale and stored solutions for the stiffness sensitivity
    double             *vscale = nullptr, *zero_g0 = nullptr, *stored_u = nullptr;
    double             *vyield = nullptr; // per-voxel initial yield stress of J2PlasticityNew elements
    double             *nwt    = nullptr; // Newton-Krylov scratch: tangent-CG residual, step, saved u: 3 n
    std::vector<double> stored_g0;
    std::vector<char>   stored_ok;

    // mixed stress/strain boundary conditions (MixedBCController, mixedBCs.h:149-227)
    bool                mixed_active = false;
    std::vector<int>    idxE, idxF;
    std::vector<double> PF, Mmix, g0_prev;

    // tensor-core CG operator (mixed path): packed per-phase stiffness, hi/lo tf32 split
    float *Wtc    = nullptr;
    bool   use_tc = false;

    // CUDA graphs of one mixed CG iteration (one per d ping-pong parity)
    bool            use_graphs   = true;
    bool            graphs_valid = false;
    cudaGraphExec_t graph_exec[2] = {nullptr, nullptr}; // device-resident inner loop, by starting d parity
    cudaGraphExec_t iter_exec[2]  = {nullptr, nullptr}; // one iteration, by d parity (host-driven loop)
    bool            loop_on_device = true; // false inside fansgpu_solve_batch: per-iteration graphs interleave
                                           // better across many concurrent streams
    LoopCtl        *ctl = nullptr, *ctl_h = nullptr;    // its controls (device, pinned host copy)
    double         *hist = nullptr;                     // err of every iteration, by iteration number
    int             hist_cap = 0;
    bool   tc_allowed = true; // FANSGPU_STENCIL=simt at create time selects the CUDA-core operator
    bool   tc_slower  = false; // the autotuner measured the CUDA-core operator faster on this grid
    int    tune       = 1;     // FANSGPU_TUNE: 1 FFT tiles (default), 3 + operator, 0 defaults, 2 forced
    int    tune_force[3] = {0, 0, 0}; // forced z / y / x tile variants
    int    tc_wait_limit = 0;         // tensor-core operator's pipeline-wait bound in polls (0: default)
    int    tc_backoff_ns = 0;         // basis operator: consumers' pause between polls (FANSGPU_TC_BACKOFF)
    bool   fp64_df = true;            // FP64 CG: operator in double-float (FANSGPU_FP64_OPERATOR=dfma: FP64 pipe)

    // several right-hand sides (desc.n_rhs): u, r and u_prev are per-RHS slices of u0, r0, up0
    // (n values each) and point at the selected RHS `cur`; the FP32 fields of the mixed path and
    // its spectrum hold nrhs slices (the single-RHS paths use slice 0 as scratch)
    int                              nrhs = 1, cur = 0;
    double                          *u0 = nullptr, *r0 = nullptr, *up0 = nullptr;
    std::vector<std::vector<double>> rhs_g0, rhs_err;
    std::vector<int>                 rhs_iter, rhs_ref;
    std::vector<char>                rhs_uzero;
    double                           rhs_ms = 0; // device time of the last solve (all RHS)
    int                             *act = nullptr, *act_h = nullptr; // active flags of the multi-RHS loop
    LoopCtlR                        *ctlr = nullptr, *ctlr_h = nullptr;
    bool                             graphs_multi = false; // the captured graphs are the multi-RHS iteration

    // basis tensor-core operator (k_stencil_tcb): exact basis blocks and per-phase coefficients
    float *Wtb = nullptr, *coef_tb = nullptr;
    int    tb_nb = 0;
    bool   use_tcb = false;
    // the multi-RHS iteration's operator as one per-phase k_stencil_tc launch per RHS (at most
    // two phases; measured faster per RHS than k_stencil_tcb); FANSGPU_STENCIL=basis keeps tcb
    bool   tcb_via_tc = false, tcb_basis_forced = false;
    // FP64-accurate basis operator on the tensor cores (k_stencil_tcx): double-float coefficients
    float *coef_tx  = nullptr;
    bool   use_tcx  = false;
    bool   exact_tc = true; // FANSGPU_EXACT=df: the CUDA-core double-float kernel instead
    bool   tc_legacy = false; // FANSGPU_STENCIL=tc: the per-phase 3xTF32 operator instead
    bool   tuned      = false;
};

namespace fansgpu {
int fail(fansgpu_ctx *ctx, int code, const char *fmt, ...)
{
    char    buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (ctx)
        ctx->err_msg = buf;
    else
        g_create_error = buf;
    return code;
}
} // namespace fansgpu

namespace {

constexpr int kMaxBlocks = 152 * 16;
constexpr int kRedSites  = 16;
enum { SITE_NORM = 0, SITE_CONV = 1, SITE_STENCIL = 2, SITE_UPDATE = 3, SITE_SS = 4, SITE_DOT = 5, SITE_EL = 6 };

template <typename P>
int dalloc(fansgpu_ctx *ctx, P **p, size_t count)
{
    cudaError_t e = cudaMalloc((void **)p, sizeof(P) * (count ? count : 1));
    if (e != cudaSuccess) {
        *p = nullptr;
        return fail(ctx, FANSGPU_ENOMEM, "cudaMalloc of %zu bytes failed: %s", sizeof(P) * count,
                    cudaGetErrorString(e));
    }
    return 0;
}

int nstr_of(int C) { return C == 1 ? 3 : 6; }

// Largest grid of any kernel that commits reduction partials.
long long max_reduction_blocks(const Grid3 &g, int C)
{
    long long b = std::max<long long>(kMaxBlocks, stencil_blocks(g));
    b           = std::max<long long>(b, (long long)C * g.nx * g.ny); // z passes: at least one row per CTA
    b           = std::max<long long>(b, stencil_tc_blocks(g));
    b           = std::max<long long>(b, (long long)kMaxRhs * kMaxBlocks); // multi-RHS update: one grid per RHS
    return b;
}

// Twiddle tables of one precision: [x: nx][y: ny][z: M][r2c: M+1].
template <typename T>
void make_twiddles(const Grid3 &g, std::vector<cplx<T>> &out)
{
    const int    M   = g.nz / 2;
    const double tpi = 2.0 * std::acos(-1.0);
    out.clear();
    auto push = [&](int n, int count) {
        for (int q = 0; q < count; ++q)
            out.push_back(cplx<T>{(T)std::cos(tpi * q / n), (T)(-std::sin(tpi * q / n))});
    };
    push(g.nx, g.nx);
    push(g.ny, g.ny);
    push(M, M);
    push(g.nz, M + 1);
}

template <typename T>
int make_plan(fansgpu_ctx *ctx, ConvPlan<T> &p, cplx<T> *spec, cplx<T> *tw, T *G)
{
    const Grid3 &g = ctx->g;
    p.g            = g;
    p.C            = ctx->C;
    p.M            = g.nz / 2;
    p.nzh          = g.nz / 2 + 1;
    p.nzp          = ((p.nzh + 15) / 16) * 16;
    p.dx.n         = g.nx;
    p.dy.n         = g.ny;
    p.dz.n         = p.M;
    if (!fe::radix_plan(g.nx, p.dx.rad, &p.dx.nrad, kMaxRadices) ||
        !fe::radix_plan(g.ny, p.dy.rad, &p.dy.nrad, kMaxRadices) ||
        !fe::radix_plan(p.M, p.dz.rad, &p.dz.nrad, kMaxRadices))
        return fail(ctx, FANSGPU_EUNSUPPORTED, "grid %dx%dx%d: FFT lengths need prime factors <= 13", g.nx, g.ny,
                    g.nz);
    p.tw_x   = tw;
    p.tw_y   = tw + g.nx;
    p.tw_z   = tw + g.nx + g.ny;
    p.tw_r2c = tw + g.nx + g.ny + p.M;
    p.spec   = spec;
    p.G      = G;
    p.gzs    = sizeof(T) == 4 ? p.nzp : p.nzh;
    const size_t cs = sizeof(cplx<T>), budget = 100 * 1024;
    int          kc = 16;
    while (kc > 1 && cs * (2 * (size_t)g.ny * kc + g.ny) > budget)
        kc /= 2;
    p.kc_y = kc;
    kc     = 16;
    while (kc > 1 && cs * (2 * (size_t)p.C * g.nx * kc + g.nx) > budget)
        kc /= 2;
    p.kc_x    = kc;
    p.use_reg = conv_reg_supported(g) ? 1 : 0;
    p.nrhs    = 1;
    p.fuse_zy = 0;
    p.spectral_dot = 0;
    p.active  = nullptr;
    p.tma     = nullptr;
    p.nrhs_alloc = ctx->nrhs;
    if (!p.use_reg && cs * (2 * (size_t)p.C * g.nx * p.kc_x + g.nx) > 200 * 1024)
        return fail(ctx, FANSGPU_EUNSUPPORTED, "n_x=%d too large for the shared-memory x pass", g.nx);
    return 0;
}

// -- per-kernel timing: events on the context stream, folded at sync points --
int tk_mark(fansgpu_ctx *ctx)
{
    if (!ctx->timing)
        return -1;
    if (ctx->tused >= (int)ctx->tpool.size())
        return -1;
    cudaEventRecord(ctx->tpool[ctx->tused], ctx->st);
    return ctx->tused++;
}
void tk_span(fansgpu_ctx *ctx, int id, int e0, int e1)
{
    if (e0 >= 0 && e1 >= 0)
        ctx->spans.push_back({id, e0, e1});
}
// reserve k consecutive events (for the convolution passes); null when off
cudaEvent_t *tk_reserve(fansgpu_ctx *ctx, int k, int *first)
{
    *first = -1;
    if (!ctx->timing || ctx->tused + k > (int)ctx->tpool.size())
        return nullptr;
    *first = ctx->tused;
    ctx->tused += k;
    return &ctx->tpool[*first];
}
void tk_flush(fansgpu_ctx *ctx)
{
    if (!ctx->timing)
        return;
    for (const auto &sp : ctx->spans) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, ctx->tpool[sp.e0], ctx->tpool[sp.e1]) == cudaSuccess) {
            ctx->ktime[sp.id] += ms;
            ctx->kcount[sp.id] += 1;
        }
    }
    ctx->spans.clear();
    ctx->tused = 0;
}

int sync_scalars(fansgpu_ctx *ctx)
{
    FANS_CUDA_CHECK(cudaMemcpyAsync(ctx->scal_h, ctx->scal, sizeof(CgScalars), cudaMemcpyDeviceToHost, ctx->st));
    FANS_CUDA_CHECK(cudaStreamSynchronize(ctx->st));
    tk_flush(ctx);
    return 0;
}

// timed convolution: the five passes as FANSGPU_K_FFT_* spans
template <typename T>
cudaError_t run_conv(fansgpu_ctx *ctx, const ConvPlan<T> &p, ConvArgs ca)
{
    int first;
    ca.ev         = tk_reserve(ctx, 6, &first);
    cudaError_t e = launch_convolution<T>(p, ca, ctx->st);
    if (ca.ev)
        for (int k = 0; k < 5; ++k)
            tk_span(ctx, FANSGPU_K_FFT_Z_FWD + k, first + k, first + k + 1);
    return e;
}

// Internal variables (zero: the virgin state of initializeInternalVariables,
// J2PlasticityNew.h:29-35) and the element-row scratch.
int ensure_rows(fansgpu_ctx *ctx)
{
    return ctx->rows ? 0 : dalloc(ctx, &ctx->rows, 8LL * ctx->C * ctx->N);
}

int alloc_nonlinear(fansgpu_ctx *ctx)
{
    const long long N = ctx->N, nep = 6LL * ctx->ngp * N, nq = (long long)ctx->ngp * N;
    int             rc;
    if ((rc = ensure_rows(ctx)))
        return rc;
    bool ivars = false; // laws with internal variables (J2PlasticityNew, J2ViscoPlastic)
    for (int ph = 0; ph < ctx->nph; ++ph)
        ivars |= ctx->law[ph] == FANSGPU_LAW_J2_LINEAR || ctx->law[ph] == FANSGPU_LAW_J2VISCO_LINEAR ||
                 ctx->law[ph] == FANSGPU_LAW_J2VISCO_NONLINEAR;
    if (ivars && !ctx->ep_t) {
        if ((rc = dalloc(ctx, &ctx->ep_t, nep)) || (rc = dalloc(ctx, &ctx->ep, nep)) ||
            (rc = dalloc(ctx, &ctx->q_t, nq)) || (rc = dalloc(ctx, &ctx->q, nq)))
            return rc;
        FANS_CUDA_CHECK(cudaMemsetAsync(ctx->ep_t, 0, sizeof(double) * nep, ctx->st));
        FANS_CUDA_CHECK(cudaMemsetAsync(ctx->ep, 0, sizeof(double) * nep, ctx->st));
        FANS_CUDA_CHECK(cudaMemsetAsync(ctx->q_t, 0, sizeof(double) * nq, ctx->st));
        FANS_CUDA_CHECK(cudaMemsetAsync(ctx->q, 0, sizeof(double) * nq, ctx->st));
    }
    bool visco = false;
    for (int ph = 0; ph < ctx->nph; ++ph)
        visco |= ctx->law[ph] == FANSGPU_LAW_J2VISCO_LINEAR || ctx->law[ph] == FANSGPU_LAW_J2VISCO_NONLINEAR;
    if (visco && !ctx->pb_t) {
        if ((rc = dalloc(ctx, &ctx->pb_t, nep)) || (rc = dalloc(ctx, &ctx->pb, nep)))
            return rc;
        FANS_CUDA_CHECK(cudaMemsetAsync(ctx->pb_t, 0, sizeof(double) * nep, ctx->st));
        FANS_CUDA_CHECK(cudaMemsetAsync(ctx->pb, 0, sizeof(double) * nep, ctx->st));
    }
    return 0;
}

// Per-phase law ids and J2 parameters for the element kernel.
int upload_law_tables(fansgpu_ctx *ctx)
{
    int rc;
    if (ctx->law_d)
        cudaFree(ctx->law_d);
    if (ctx->prm_d)
        cudaFree(ctx->prm_d);
    ctx->law_d = nullptr;
    ctx->prm_d = nullptr;
    constexpr int kPrm = 8;
    if ((rc = dalloc(ctx, &ctx->law_d, ctx->nph)) || (rc = dalloc(ctx, &ctx->prm_d, kPrm * ctx->nph)))
        return rc;
    std::vector<int>    lw(ctx->nph);
    std::vector<double> pr(kPrm * ctx->nph, 0.0);
    for (int ph = 0; ph < ctx->nph; ++ph) {
        lw[ph]                 = ctx->law[ph];
        const auto &p          = ctx->prm[ph];
        double     *o          = &pr[kPrm * ph];
        auto        opt        = [&](size_t i, double d) { return p.size() > i ? p[i] : d; };
        if (lw[ph] == FANSGPU_LAW_PSEUDO_LINEAR) { // PseudoPlastic.h:84-90
            const double G = p[1], sy = p[2], h = p[3];
            const double mi = opt(4, 0.0), nm = opt(5, 1.0);
            const double v[8] = {p[0], G, sy, h, std::sqrt(2. / 3.) * sy / (2. * G), (3. * G) / (3. * G + h), mi, nm + mi};
            std::copy(v, v + 8, o);
        } else if (lw[ph] == FANSGPU_LAW_PSEUDO_NONLINEAR) { // PseudoPlastic.h:133-136
            const double G = p[1], sy = p[2], n = p[3], e0 = p[4];
            const double mi = opt(5, 0.0), nm = opt(6, 1.0);
            const double ec = e0 * std::pow(sy / (3.0 * G * e0), 1.0 / (1.0 - n));
            const double v[8] = {p[0], G, sy, n, e0, ec, mi, nm + mi};
            std::copy(v, v + 8, o);
        } else if (lw[ph] == FANSGPU_LAW_J2VISCO_LINEAR || lw[ph] == FANSGPU_LAW_J2VISCO_NONLINEAR) {
            // {K, G, sigma_y, K_iso, H_kin, eta/dt, sigma_inf, delta} (J2Plasticity.h:12-20, :190-199)
            const double v[8] = {p[0], p[1], p[2], p[3], p[4], p[5] / p[6], opt(7, 0.0), opt(8, 0.0)};
            std::copy(v, v + 8, o);
        } else {
            for (size_t i = 0; i < std::min<size_t>(kPrm, p.size()); ++i)
                o[i] = p[i];
        }
    }
    FANS_CUDA_CHECK(cudaMemcpyAsync(ctx->law_d, lw.data(), sizeof(int) * lw.size(), cudaMemcpyHostToDevice, ctx->st));
    FANS_CUDA_CHECK(cudaMemcpyAsync(ctx->prm_d, pr.data(), sizeof(double) * pr.size(), cudaMemcpyHostToDevice, ctx->st));
    FANS_CUDA_CHECK(cudaStreamSynchronize(ctx->st));
    return 0;
}

int autotune(fansgpu_ctx *ctx);

// Per-phase tables, reference stiffness and Green's operator (lazy).
int setup(fansgpu_ctx *ctx)
{
    if (!ctx->have_ms)
        return fail(ctx, FANSGPU_ESTATE, "set_microstructure must be called before solving");
    const int C = ctx->C, nstr = ctx->nstr, NC = 8 * C;
    if (ctx->tables_dirty) {
        const int nph = std::max(ctx->ms_max + 1, (int)ctx->law.size());
        // per-phase element stiffness tables live in shared memory on the FP64 and
        // double-float paths: 255 phases fit for thermal problems, 32 for mechanics
        const int max_ph = C == 1 ? 255 : 32;
        if (nph > max_ph)
            return fail(ctx, FANSGPU_EUNSUPPORTED, "%d phases: at most %d phases per context for howmany=%d", nph,
                        max_ph, C);
        ctx->law.resize(nph, -1);
        ctx->prm.resize(nph);
        ctx->assigned.resize(nph, 0);
        for (int ph = 0; ph < nph; ++ph)
            if (!ctx->assigned[ph])
                return fail(ctx, FANSGPU_EINVAL, "MaterialManager: Phase %d not assigned", ph);
        if (nph != ctx->nph) {
            void *old[] = {ctx->K64, ctx->K32, ctx->f64, ctx->Cph};
            for (void *p : old)
                if (p)
                    cudaFree(p);
            ctx->K64 = ctx->f64 = ctx->Cph = nullptr;
            ctx->K32                       = nullptr;
            ctx->nph                       = 0;
            int rc;
            if ((rc = dalloc(ctx, &ctx->K64, (size_t)nph * NC * NC)) ||
                (rc = dalloc(ctx, &ctx->K32, (size_t)nph * NC * NC)) || (rc = dalloc(ctx, &ctx->f64, (size_t)nph * NC)) ||
                (rc = dalloc(ctx, &ctx->Cph, (size_t)nph * nstr * nstr)))
                return rc;
            ctx->nph = nph;
        }
        ctx->all_linear = true;
        std::vector<double> K64(ctx->nph * NC * NC), Cph(ctx->nph * nstr * nstr), Ke;
        std::vector<float>  K32(ctx->nph * NC * NC);
        for (int ph = 0; ph < ctx->nph; ++ph) {
            if (ctx->law[ph] == FANSGPU_LAW_J2_LINEAR || ctx->law[ph] == FANSGPU_LAW_PSEUDO_LINEAR ||
                ctx->law[ph] == FANSGPU_LAW_PSEUDO_NONLINEAR || ctx->law[ph] == FANSGPU_LAW_J2VISCO_LINEAR ||
                ctx->law[ph] == FANSGPU_LAW_J2VISCO_NONLINEAR || ctx->law[ph] == FANSGPU_LAW_SVK ||
                ctx->law[ph] == FANSGPU_LAW_NEOHOOKEAN)
                ctx->all_linear = false;
            if (!fe::law_C(ctx->law[ph], ctx->prm[ph], nstr, &Cph[ph * nstr * nstr]))
                return fail(ctx, FANSGPU_EINVAL, "phase %d: law %d does not fit problem with n_str=%d", ph,
                            ctx->law[ph], nstr);
            fe::element_stiffness(C, ctx->ngp, ctx->B, &Cph[ph * nstr * nstr], ctx->ve, Ke);
            for (int i = 0; i < NC * NC; ++i) {
                K64[ph * NC * NC + i] = Ke[i];
                K32[ph * NC * NC + i] = (float)Ke[i];
            }
        }
        {
            int rc3;
            if ((rc3 = upload_law_tables(ctx)) || (!ctx->all_linear && (rc3 = alloc_nonlinear(ctx))))
                return rc3;
        }
        ctx->K64h = K64;
        ctx->K32h = K32;
        ctx->use_tc = false;
        ctx->graphs_valid = false;
        if (ctx->tc_allowed && !ctx->tc_slower && ctx->desc.precision == FANSGPU_MIXED &&
            stencil_tc_supported(ctx->g, C, ctx->nph)) {
            std::vector<float> w(stencil_tc_weights(C, ctx->nph));
            stencil_tc_pack_weights(C, ctx->nph, K32.data(), w.data());
            if (ctx->Wtc)
                cudaFree(ctx->Wtc);
            ctx->Wtc = nullptr;
            int rc4;
            if ((rc4 = dalloc(ctx, &ctx->Wtc, w.size())))
                return rc4;
            FANS_CUDA_CHECK(cudaMemcpyAsync(ctx->Wtc, w.data(), sizeof(float) * w.size(), cudaMemcpyHostToDevice, ctx->st));
            ctx->use_tc = true;
        }
        // the basis operators: every phase an isotropic law of this problem, each basis block exact.
        // k_stencil_tcb (FP32, mixed path) and k_stencil_tcx (FP64-accurate: true residual, FP64 CG)
        ctx->use_tcb    = false;
        ctx->use_tcx    = false;
        ctx->tcb_via_tc = false;
        if (ctx->nstr == (C == 1 ? 3 : 6)) {
            const int iso = C == 1 ? FANSGPU_LAW_THERMAL_ISO : FANSGPU_LAW_ELASTIC_ISO, nb = C == 1 ? 1 : 2;
            bool      ok  = ctx->nph >= 1 && ctx->nph <= 256;
            for (int ph = 0; ph < ctx->nph && ok; ++ph)
                ok = ctx->law[ph] == iso;
            // basis constitutive matrices: conduction I; elasticity 1 1^T (lambda) and 2 I (mu),
            // so that C_ph = lambda 1 1^T + mu 2 I (LinearElastic.h:24-35)
            std::vector<double> Kb((size_t)nb * NC * NC), Cb(nstr * nstr), q(nb);
            for (int b = 0; b < nb && ok; ++b) {
                std::fill(Cb.begin(), Cb.end(), 0.0);
                for (int i = 0; i < nstr; ++i)
                    for (int j = 0; j < nstr; ++j)
                        Cb[i * nstr + j] = C == 1 ? (i == j ? 1.0 : 0.0)
                                         : b == 0 ? (i < 3 && j < 3 ? 1.0 : 0.0)
                                                  : (i == j ? 2.0 : 0.0);
                fe::element_stiffness(C, ctx->ngp, ctx->B, Cb.data(), ctx->ve, Ke);
                std::copy(Ke.begin(), Ke.end(), Kb.begin() + (size_t)b * NC * NC);
            }
            if (ok)
                ok = stencil_tcb_quanta(C, Kb.data(), nb, q.data());
            if (ok) {
                std::vector<float> w(stencil_tcb_weights(C, nb)), cf((size_t)ctx->nph * nb),
                    cfd((size_t)ctx->nph * nb * 2);
                stencil_tcb_pack_weights(C, nb, Kb.data(), q.data(), w.data());
                for (int ph = 0; ph < ctx->nph; ++ph) {
                    const std::vector<double> &pr = ctx->prm[ph];
                    for (int b = 0; b < nb; ++b) {
                        // lambda = K - 2G/3, mu = G (LinearElastic.h:24); conductivity as given
                        const double c = C == 1 ? pr[0] * q[0] : (b == 0 ? (pr[0] - 2.0 * pr[1] / 3.0) * q[0] : pr[1] * q[1]);
                        cf[ph * nb + b]            = (float)c;
                        cfd[(ph * nb + b) * 2]     = (float)c; // double-float pair
                        cfd[(ph * nb + b) * 2 + 1] = (float)(c - (double)(float)c);
                    }
                }
                for (float *p : {ctx->Wtb, ctx->coef_tb, ctx->coef_tx})
                    if (p)
                        cudaFree(p);
                ctx->Wtb = ctx->coef_tb = ctx->coef_tx = nullptr;
                int rc5;
                if ((rc5 = dalloc(ctx, &ctx->Wtb, w.size())) || (rc5 = dalloc(ctx, &ctx->coef_tb, cf.size())) ||
                    (rc5 = dalloc(ctx, &ctx->coef_tx, cfd.size())))
                    return rc5;
                FANS_CUDA_CHECK(cudaMemcpyAsync(ctx->Wtb, w.data(), sizeof(float) * w.size(), cudaMemcpyHostToDevice,
                                                ctx->st));
                FANS_CUDA_CHECK(cudaMemcpyAsync(ctx->coef_tb, cf.data(), sizeof(float) * cf.size(),
                                                cudaMemcpyHostToDevice, ctx->st));
                FANS_CUDA_CHECK(cudaMemcpyAsync(ctx->coef_tx, cfd.data(), sizeof(float) * cfd.size(),
                                                cudaMemcpyHostToDevice, ctx->st));
                FANS_CUDA_CHECK(cudaStreamSynchronize(ctx->st)); // host temporaries
                ctx->tb_nb   = nb;
                ctx->use_tcb = ctx->tc_allowed && !ctx->tc_legacy && !ctx->tc_slower &&
                               ctx->desc.precision == FANSGPU_MIXED && stencil_tcb_supported(ctx->g, C, nb, ctx->nph);
                ctx->use_tcx = ctx->exact_tc && stencil_tcx_supported(ctx->g, C, nb, ctx->nph);
                ctx->tcb_via_tc = ctx->use_tcb && ctx->use_tc && ctx->Wtc && !ctx->tcb_basis_forced;
            }
        }
        {
            std::vector<float> kdf(2 * K64.size());
            for (size_t i = 0; i < K64.size(); ++i) {
                const float hi        = (float)K64[i];
                kdf[i]                = hi;
                kdf[K64.size() + i]   = (float)(K64[i] - (double)hi);
            }
            if (ctx->Kdf)
                cudaFree(ctx->Kdf);
            ctx->Kdf = nullptr;
            int rc2;
            if ((rc2 = dalloc(ctx, &ctx->Kdf, kdf.size())))
                return rc2;
            FANS_CUDA_CHECK(cudaMemcpyAsync(ctx->Kdf, kdf.data(), sizeof(float) * kdf.size(), cudaMemcpyHostToDevice, ctx->st));
        }
        FANS_CUDA_CHECK(cudaMemcpyAsync(ctx->K64, K64.data(), sizeof(double) * K64.size(), cudaMemcpyHostToDevice, ctx->st));
        FANS_CUDA_CHECK(cudaMemcpyAsync(ctx->K32, K32.data(), sizeof(float) * K32.size(), cudaMemcpyHostToDevice, ctx->st));
        FANS_CUDA_CHECK(cudaMemcpyAsync(ctx->Cph, Cph.data(), sizeof(double) * Cph.size(), cudaMemcpyHostToDevice, ctx->st));
        FANS_CUDA_CHECK(cudaStreamSynchronize(ctx->st));
        ctx->tables_dirty = false;
        ctx->force_dirty  = true;
    }
    if (ctx->green_dirty) {
        if (!ctx->have_ref)
            return fail(ctx, FANSGPU_ESTATE, "set_reference (kapparef_mat) must be called before solving");
        std::vector<double> K0n, K0c;
        fe::element_stiffness(C, ctx->ngp, ctx->B, ctx->kapparef.data(), ctx->ve, K0n);
        fe::to_component_major(C, K0n, K0c);
        FANS_CUDA_CHECK(cudaMemcpyAsync(ctx->K0c, K0c.data(), sizeof(double) * K0c.size(), cudaMemcpyHostToDevice, ctx->st));
        const Grid3 &g = ctx->g;
        const int    nzh = g.nz / 2 + 1;
        GreenArgs    ga{};
        ga.g   = g;
        ga.C   = C;
        ga.K0c = ctx->K0c;
        ga.cx  = ctx->trig;
        ga.sx  = ga.cx + g.nx;
        ga.cy  = ga.sx + g.nx;
        ga.sy  = ga.cy + g.ny;
        ga.cz  = ga.sy + g.ny;
        ga.sz  = ga.cz + nzh;
        ga.G64  = ctx->G64;
        ga.G32  = ctx->G32;
        ga.g32s = ((nzh + 15) / 16) * 16; // FP32 rows padded as the spectrum's (16-byte starts)
        int e0 = tk_mark(ctx);
        FANS_CUDA_CHECK(launch_green(ga, ctx->st));
        tk_span(ctx, FANSGPU_K_GREEN, e0, tk_mark(ctx));
        FANS_CUDA_CHECK(cudaStreamSynchronize(ctx->st));
        tk_flush(ctx);
        ctx->green_dirty = false;
    }
    if (ctx->force_dirty) {
        std::vector<double> f(ctx->nph * NC);
        std::vector<double> Cm(nstr * nstr);
        for (int ph = 0; ph < ctx->nph; ++ph) {
            fe::law_C(ctx->law[ph], ctx->prm[ph], nstr, Cm.data());
            fe::element_force(C, ctx->ngp, ctx->B, Cm.data(), ctx->g0.data(), ctx->ve, &f[ph * NC]);
        }
        ctx->f64h = f;
        FANS_CUDA_CHECK(cudaMemcpyAsync(ctx->f64, f.data(), sizeof(double) * f.size(), cudaMemcpyHostToDevice, ctx->st));
        if (ctx->nph <= 2) {
            // node sums of the force rows for every key of the 8 element phases, summed over the
            // local node p = 0..7 in the order the stencil kernels add them (bitwise the same r)
            std::vector<double> tab((size_t)256 * C);
            for (int key = 0; key < 256; ++key)
                for (int cr = 0; cr < C; ++cr) {
                    double acc = 0.0;
                    for (int p = 0; p < 8; ++p)
                        acc += f[(size_t)(std::min((key >> p) & 1, ctx->nph - 1)) * NC + p * C + cr];
                    tab[(size_t)key * C + cr] = acc;
                }
            int rc3;
            if (!ctx->fnode && (rc3 = dalloc(ctx, &ctx->fnode, (size_t)256 * 3)))
                return rc3;
            FANS_CUDA_CHECK(cudaMemcpyAsync(ctx->fnode, tab.data(), sizeof(double) * tab.size(), cudaMemcpyHostToDevice,
                                            ctx->st));
        }
        {
            std::vector<float> fdf(2 * f.size());
            for (size_t i = 0; i < f.size(); ++i) {
                const float hi    = (float)f[i];
                fdf[i]            = hi;
                fdf[f.size() + i] = (float)(f[i] - (double)hi);
            }
            if (ctx->fdf && ctx->fdf_cap < fdf.size()) { // kept across gradients (one RHS after another)
                cudaFree(ctx->fdf);
                ctx->fdf = nullptr;
            }
            int rc2;
            if (!ctx->fdf && (rc2 = dalloc(ctx, &ctx->fdf, fdf.size())))
                return rc2;
            ctx->fdf_cap = std::max(ctx->fdf_cap, fdf.size());
            FANS_CUDA_CHECK(cudaMemcpyAsync(ctx->fdf, fdf.data(), sizeof(float) * fdf.size(), cudaMemcpyHostToDevice, ctx->st));
        }
        FANS_CUDA_CHECK(cudaMemcpyAsync(ctx->g0_d, ctx->g0.data(), sizeof(double) * nstr, cudaMemcpyHostToDevice, ctx->st));
        FANS_CUDA_CHECK(cudaStreamSynchronize(ctx->st));
        ctx->force_dirty = false;
    }
    return autotune(ctx);
}

// y = K x (+F) in FP64 (optionally FP32), no fusion.
template <typename T>
int run_stencil(fansgpu_ctx *ctx, const T *x, T *y, bool with_f)
{
    StencilArgs a{};
    a.g      = ctx->g;
    a.C      = ctx->C;
    a.x      = x;
    a.y      = y;
    a.ms     = ctx->d_ms;
    a.Kph    = std::is_same<T, double>::value ? (const void *)ctx->K64 : (const void *)ctx->K32;
    a.fph    = with_f ? ctx->f64 : nullptr;
    a.Kph_host = std::is_same<T, double>::value ? (const void *)ctx->K64h.data() : (const void *)ctx->K32h.data();
    a.fph_host = with_f ? ctx->f64h.data() : nullptr;
    a.force_only = (with_f && (const void *)x == (const void *)ctx->u && ctx->u_zero) ? 1 : 0;
    a.nph    = ctx->nph;
    if (std::is_same<T, double>::value && a.force_only && ctx->nph <= 2 && ctx->fnode && !ctx->vscale &&
        ctx->all_linear) { // r = F from the node table
        int e0 = tk_mark(ctx);
        FANS_CUDA_CHECK(launch_force_nodes(ctx->g, ctx->C, ctx->d_ms, ctx->fnode, reinterpret_cast<double *>(y), ctx->st));
        tk_span(ctx, FANSGPU_K_RESIDUAL, e0, tk_mark(ctx));
        return 0;
    }
    a.scal   = ctx->scal;
    a.red    = ctx->red;
    a.red_site = SITE_STENCIL;
    int e0     = tk_mark(ctx);
    FANS_CUDA_CHECK(launch_stencil<T>(a, ctx->st));
    tk_span(ctx, with_f ? FANSGPU_K_RESIDUAL : FANSGPU_K_STENCIL, e0, tk_mark(ctx));
    return 0;
}

// r = R(u) = K u + F with FP64 accuracy from FP32 arithmetic (mixed-path refresh).
// A tensor-core wait timeout is reported in scal->converged (-3).
int run_residual_df(fansgpu_ctx *ctx, CgScalars *scal)
{
    if (ctx->u_zero)
        return run_stencil<double>(ctx, ctx->u, ctx->r, true); // r = F, no arithmetic on u
    if (ctx->use_tcx) { // the same, with the products on the tensor cores
        StencilArgs a{};
        a.g          = ctx->g;
        a.C          = ctx->C;
        a.x          = ctx->u;
        a.y          = ctx->r;
        a.ms         = ctx->d_ms;
        a.nph        = ctx->nph;
        a.scal       = scal;
        a.wait_limit = ctx->tc_wait_limit;
        int e0       = tk_mark(ctx);
        FANS_CUDA_CHECK(launch_stencil_tcx(a, ctx->Wtb, ctx->coef_tx, ctx->fdf, ctx->tb_nb, ctx->st));
        tk_span(ctx, FANSGPU_K_RESIDUAL, e0, tk_mark(ctx));
        return 0;
    }
    StencilArgs a{};
    a.g        = ctx->g;
    a.C        = ctx->C;
    a.x        = ctx->u;
    a.y        = ctx->r;
    a.ms       = ctx->d_ms;
    a.Kph      = ctx->Kdf;
    a.fph      = ctx->fdf;
    a.nph      = ctx->nph;
    int e0     = tk_mark(ctx);
    FANS_CUDA_CHECK(launch_residual_df(a, ctx->st));
    tk_span(ctx, FANSGPU_K_RESIDUAL, e0, tk_mark(ctx));
    return 0;
}

ElementArgs element_args(fansgpu_ctx *ctx, const double *u, int mode)
{
    ElementArgs a{};
    a.g     = ctx->g;
    a.C     = ctx->C;
    a.nstr  = ctx->nstr;
    a.ngp   = ctx->ngp;
    a.mode  = mode;
    a.u     = u;
    a.ms    = ctx->d_ms;
    a.B     = ctx->Bgp_d;
    a.Bb    = ctx->Bb_d;
    a.g0    = ctx->g0_d;
    a.law   = ctx->law_d;
    a.Cph   = ctx->Cph;
    a.prm   = ctx->prm_d;
    a.ep_t  = ctx->ep_t;
    a.q_t   = ctx->q_t;
    a.ep    = ctx->ep;
    a.q     = ctx->q;
    a.pb_t  = ctx->pb_t;
    a.pb    = ctx->pb;
    a.ve    = ctx->ve;
    a.rows  = ctx->rows;
    a.red   = ctx->red;
    a.red_site     = SITE_EL;
    a.phase_filter = -1;
    a.scale        = ctx->vscale;
    a.sy           = ctx->vyield;
    return a;
}

// r = R(u) in FP64 (compute_residual, solver.h:231-270).  Linear laws: the
// fused stencil with the g0 force; nonlinear laws: the element kernel (which
// writes the trial internal variables, as get_sigma does) and the node gather.
int run_residual64(fansgpu_ctx *ctx, const double *u, double *r)
{
    if (ctx->all_linear && !ctx->vscale)
        return run_stencil<double>(ctx, u, r, true);
    int e0 = tk_mark(ctx);
    FANS_CUDA_CHECK(launch_element(element_args(ctx, u, ELEM_RESIDUAL), ctx->st));
    FANS_CUDA_CHECK(launch_gather(ctx->rows, r, ctx->g, ctx->C, ctx->st));
    tk_span(ctx, FANSGPU_K_RESIDUAL, e0, tk_mark(ctx));
    return 0;
}

// y = K x through the element kernel with g0 = 0 (linear laws with a per-voxel scale).
int run_operator_elem(fansgpu_ctx *ctx, const double *x, double *y)
{
    ElementArgs a = element_args(ctx, x, ELEM_RESIDUAL);
    a.g0          = ctx->zero_g0;
    a.ep          = nullptr;
    a.q           = nullptr;
    int e0        = tk_mark(ctx);
    FANS_CUDA_CHECK(launch_element(a, ctx->st));
    FANS_CUDA_CHECK(launch_gather(ctx->rows, y, ctx->g, ctx->C, ctx->st));
    tk_span(ctx, FANSGPU_K_STENCIL, e0, tk_mark(ctx));
    return 0;
}

// The selected right-hand side's host state (history, iteration count, u = 0 flag,
// g0) lives in the context's single-RHS members; store_rhs saves it, load_rhs makes
// RHS k the selected one (its field slices, its state; the force tables follow g0).
void store_rhs(fansgpu_ctx *ctx)
{
    const int k       = ctx->cur;
    ctx->rhs_err[k]   = ctx->err_all;
    ctx->rhs_iter[k]  = ctx->iter;
    ctx->rhs_uzero[k] = ctx->u_zero ? 1 : 0;
    ctx->rhs_g0[k]    = ctx->g0;
}

void load_rhs(fansgpu_ctx *ctx, int k)
{
    ctx->cur     = k;
    ctx->u       = ctx->u0 + (long long)k * ctx->n;
    ctx->r       = ctx->r0 + (long long)k * ctx->n;
    ctx->uprev   = ctx->up0 + (long long)k * ctx->n;
    ctx->err_all = ctx->rhs_err[k];
    ctx->iter    = ctx->rhs_iter[k];
    ctx->u_zero  = ctx->rhs_uzero[k] != 0;
    if (ctx->g0 != ctx->rhs_g0[k]) {
        ctx->g0          = ctx->rhs_g0[k];
        ctx->force_dirty = true;
    }
}

int init_scalars(fansgpu_ctx *ctx)
{
    CgScalars s{};
    s.delta    = 1.0; // solverCG.h:82
    s.deltamid = 0.0;
    s.beta     = 0.0;
    *ctx->scal_h = s;
    FANS_CUDA_CHECK(cudaMemcpyAsync(ctx->scal, ctx->scal_h, sizeof(CgScalars), cudaMemcpyHostToDevice, ctx->st));
    return 0;
}

double err_value(fansgpu_ctx *ctx, double err)
{
    // Solver::compute_error return value (solver.h:432-451)
    if (ctx->tol.type == FANSGPU_ABSOLUTE)
        return err;
    return ctx->iter == 0 ? 100.0 : err / ctx->err_all[0];
}

// FP64 flexible CG (SolverCG::internalSolve, linear branch).
int solve_cg64(fansgpu_ctx *ctx)
{
    const long long n = ctx->n;
    int             rc;
    FANS_CUDA_CHECK(cudaMemsetAsync(ctx->s, 0, sizeof(double) * n, ctx->st));
    FANS_CUDA_CHECK(cudaMemsetAsync(ctx->dd[0], 0, sizeof(double) * n, ctx->st));
    ctx->cur_d = 0;
    if ((rc = init_scalars(ctx)))
        return rc;
    // r = R(u) (compute_residual<2>, solverCG.h:76)
    const bool df = ctx->fp64_df && ctx->all_linear && !ctx->vscale; // FP64-accurate operator off the FP64 pipe
    if ((rc = df ? run_residual_df(ctx, ctx->scal) : run_residual64(ctx, ctx->u, ctx->r)))
        return rc;
    { int en = tk_mark(ctx);
    FANS_CUDA_CHECK(launch_norm<double, float>(ctx->r, n, ctx->tol.measure, ctx->scal, 1, nullptr, ctx->red,
                                               SITE_NORM, ctx->st));
    tk_span(ctx, FANSGPU_K_NORM, en, tk_mark(ctx)); }
    if ((rc = sync_scalars(ctx)))
        return rc;
    ctx->iter = 0;
    ctx->err_all.assign(1, ctx->scal_h->err);
    if (ctx->scal_h->converged == -3)
        return fail(ctx, FANSGPU_ECUDA, "tensor-core operator: MMA completion wait timed out (initial residual)");
    if (!std::isfinite(ctx->scal_h->err))
        return fail(ctx, FANSGPU_ENAN, "non-finite initial residual norm (e.g. det F <= 0 in CompressibleNeoHookean)");
    double err_rel = err_value(ctx, ctx->scal_h->err);
    if (ctx->tol.n_it > 0 && err_rel > ctx->tol.tolerance)
        ctx->u_zero = false; // u is updated from here on
    while (ctx->iter < ctx->tol.n_it && err_rel > ctx->tol.tolerance) {
        ConvArgs ca{ctx->r, ctx->s, -1.0, 1, ctx->scal, ctx->red, SITE_CONV};
        FANS_CUDA_CHECK(run_conv<double>(ctx, ctx->cp64, ca));
        StencilArgs sa{};
        sa.g        = ctx->g;
        sa.C        = ctx->C;
        sa.x        = ctx->s;
        sa.d_old    = ctx->dd[ctx->cur_d];
        sa.d_new    = ctx->dd[ctx->cur_d ^ 1];
        sa.y        = ctx->Kd;
        sa.ms       = ctx->d_ms;
        sa.Kph      = ctx->K64;
        sa.Kph_host = ctx->K64h.data();
        sa.nph      = ctx->nph;
        sa.fuse_d   = 1;
        sa.reduce   = 1;
        sa.scal     = ctx->scal;
        sa.red      = ctx->red;
        sa.red_site = SITE_STENCIL;
        if (ctx->vscale) {
            // per-voxel stiffness: d = s + beta d, K d by the element kernel, <d, K d>, alpha
            double *dn = ctx->dd[ctx->cur_d ^ 1];
            FANS_CUDA_CHECK(cudaMemcpyAsync(dn, ctx->dd[ctx->cur_d], sizeof(double) * n, cudaMemcpyDeviceToDevice,
                                            ctx->st));
            FANS_CUDA_CHECK(launch_direction(dn, ctx->s, n, ctx->scal, ctx->st));
            if ((rc = run_operator_elem(ctx, dn, ctx->Kd)))
                return rc;
            FANS_CUDA_CHECK(launch_dot(dn, ctx->Kd, n, &ctx->scal->dAd, ctx->red, SITE_DOT, ctx->st));
            FANS_CUDA_CHECK(launch_set_alpha(ctx->scal, ctx->st));
        } else if (df && ctx->use_tcx) {
            // d = s + beta d_old, K d FP64-accurate with the products on the tensor cores, <d, K d>, alpha
            sa.wait_limit = ctx->tc_wait_limit;
            int e0        = tk_mark(ctx);
            FANS_CUDA_CHECK(launch_stencil_tcx(sa, ctx->Wtb, ctx->coef_tx, nullptr, ctx->tb_nb, ctx->st));
            tk_span(ctx, FANSGPU_K_STENCIL, e0, tk_mark(ctx));
        } else if (df) {
            // d = s + beta d_old, K d in double-float on the FP32 pipes (GB300's FP64 rate is about
            // 1/60 of its FP32 rate), <d, K d> and alpha in FP64
            sa.Kph = ctx->Kdf;
            sa.fph = nullptr;
            int e0 = tk_mark(ctx);
            FANS_CUDA_CHECK(launch_residual_df(sa, ctx->st));
            tk_span(ctx, FANSGPU_K_STENCIL, e0, tk_mark(ctx));
        } else {
            int e0 = tk_mark(ctx);
            FANS_CUDA_CHECK(launch_stencil<double>(sa, ctx->st));
            tk_span(ctx, FANSGPU_K_STENCIL, e0, tk_mark(ctx));
        }
        ctx->cur_d ^= 1;
        UpdateArgs ua{n, ctx->r, ctx->Kd, ctx->u, ctx->dd[ctx->cur_d], ctx->s, ctx->tol.measure, 1, ctx->scal,
                      ctx->red, SITE_UPDATE};
        int e2 = tk_mark(ctx);
        FANS_CUDA_CHECK((launch_cg_update<double, double>(ua, ctx->st)));
        tk_span(ctx, FANSGPU_K_UPDATE, e2, tk_mark(ctx));
        if ((rc = sync_scalars(ctx)))
            return rc;
        ctx->iter++;
        ctx->err_all.push_back(ctx->scal_h->err);
        if (ctx->scal_h->converged == -3)
            return fail(ctx, FANSGPU_ECUDA, "tensor-core operator: MMA completion wait timed out at iteration %d",
                        ctx->iter);
        if (ctx->scal_h->converged < 0)
            return fail(ctx, FANSGPU_ENAN, "non-finite residual norm at iteration %d", ctx->iter);
        err_rel = err_value(ctx, ctx->scal_h->err);
    }
    return 0;
}

// One inner iteration of the mixed CG on the context stream: s = -G*r with
// delta/beta, d = s + beta d_old with K d and alpha, then the FP32 update.
StencilArgs mixed_operator_args(fansgpu_ctx *ctx, int cd)
{
    StencilArgs sa{};
    sa.g        = ctx->g;
    sa.C        = ctx->C;
    sa.x        = ctx->s32;
    sa.d_old    = ctx->d32[cd];
    sa.d_new    = ctx->d32[cd ^ 1];
    sa.y        = ctx->Kd32;
    sa.ms       = ctx->d_ms;
    sa.Kph      = ctx->K32;
    sa.Kph_host = ctx->K32h.data();
    sa.nph      = ctx->nph;
    sa.fuse_d   = 1;
    sa.reduce   = 1;
    sa.scal     = ctx->scal;
    sa.red      = ctx->red;
    sa.red_site = SITE_STENCIL;
    sa.wait_limit = ctx->tc_wait_limit;
    sa.wait_sleep_ns = ctx->tc_backoff_ns;
    return sa;
}

cudaError_t enqueue_mixed_iteration(fansgpu_ctx *ctx, int cd)
{
    const long long n = ctx->n;
    ConvArgs        ca{ctx->r32, ctx->s32, -1.0, 1, ctx->scal, ctx->red, SITE_CONV};
    cudaError_t     e = run_conv<float>(ctx, ctx->cp32, ca);
    if (e != cudaSuccess)
        return e;
    const StencilArgs sa = mixed_operator_args(ctx, cd);
    int               e0 = tk_mark(ctx);
    e = ctx->use_tc ? launch_stencil_tc(sa, ctx->Wtc, ctx->nph, ctx->st) : launch_stencil<float>(sa, ctx->st);
    if (e != cudaSuccess)
        return e;
    tk_span(ctx, FANSGPU_K_STENCIL, e0, tk_mark(ctx));
    UpdateArgs ua{n, ctx->r32, ctx->Kd32, ctx->e32, ctx->d32[cd ^ 1], ctx->s32, ctx->tol.measure, 1, ctx->scal,
                  ctx->red, SITE_UPDATE};
    int e2 = tk_mark(ctx);
    e      = launch_cg_update<float, float>(ua, ctx->st);
    tk_span(ctx, FANSGPU_K_UPDATE, e2, tk_mark(ctx));
    return e;
}

// The mixed path runs as a multi-RHS iteration (every right-hand side in each
// kernel) where the basis tensor-core operator and the register FFT passes apply.
bool multi_rhs_path(const fansgpu_ctx *ctx)
{
    return ctx->desc.precision == FANSGPU_MIXED && ctx->use_tcb && ctx->cp32.use_reg && ctx->all_linear &&
           !ctx->vscale && !ctx->mixed_active;
}

// One inner iteration over all right-hand sides (inactive ones skipped on the
// device): s_k = -G*r_k with delta_k/beta_k, d_k = s_k + beta_k d_k,old with K d_k
// and alpha_k, then the FP32 update of r_k and e_k.
cudaError_t enqueue_mixed_iteration_rhs(fansgpu_ctx *ctx, int cd)
{
    const long long n = ctx->n;
    ConvPlan<float> p = ctx->cp32;
    p.nrhs            = ctx->nrhs;
    p.active          = ctx->act;
    ConvArgs    ca{ctx->r32, ctx->s32, -1.0, 1, ctx->scal, ctx->red, SITE_CONV};
    cudaError_t e = run_conv<float>(ctx, p, ca);
    if (e != cudaSuccess)
        return e;
    StencilArgs sa = mixed_operator_args(ctx, cd);
    sa.nrhs        = ctx->nrhs;
    sa.rhs_stride  = n;
    sa.active      = ctx->act;
    int e0         = tk_mark(ctx);
    if (ctx->tcb_via_tc) {
        // the single-RHS per-phase operator once per RHS (its fields at offset k * n, its scalars
        // at scal[k]); a converged RHS's launch returns at once
        for (int k = 0; k < ctx->nrhs && e == cudaSuccess; ++k) {
            StencilArgs sk = sa;
            sk.x           = ctx->s32 + k * n;
            sk.d_old       = ctx->d32[cd] + k * n;
            sk.d_new       = ctx->d32[cd ^ 1] + k * n;
            sk.y           = ctx->Kd32 + k * n;
            sk.scal        = ctx->scal + k;
            sk.active      = ctx->act + k;
            sk.nrhs        = 1;
            sk.rhs_stride  = 0;
            e              = launch_stencil_tc(sk, ctx->Wtc, ctx->nph, ctx->st);
        }
    } else
        e = launch_stencil_tcb(sa, ctx->Wtb, ctx->coef_tb, ctx->tb_nb, ctx->st);
    if (e != cudaSuccess)
        return e;
    tk_span(ctx, FANSGPU_K_STENCIL, e0, tk_mark(ctx));
    UpdateArgs ua{n, ctx->r32, ctx->Kd32, ctx->e32, ctx->d32[cd ^ 1], ctx->s32, ctx->tol.measure, 1, ctx->scal,
                  ctx->red, SITE_UPDATE, ctx->nrhs, ctx->act};
    int e2 = tk_mark(ctx);
    e      = launch_cg_update<float, float>(ua, ctx->st);
    tk_span(ctx, FANSGPU_K_UPDATE, e2, tk_mark(ctx));
    return e;
}

// ---------------------------------------------------------------------------
// Autotuning: the register FFT passes' tile variants (per precision) and, with
// FANSGPU_TUNE=all, tensor-core against CUDA-core operator on the mixed path.
// Runs once per context on its first setup, timed with CUDA events on the
// context stream on scratch fields (the solve re-initialises them); results
// are cached per grid for the process, so equal grids get equal choices.  The
// operator is left out by default: timed alone on a small grid the CUDA-core
// operator can win (it fills more SMs), while many contexts sharing the GPU
// (fansgpu_solve_batch) run faster on the tensor-core one.
struct TuneChoice {
    int v64[3], v32[3];
    int tc_slower;
};
std::mutex                             g_tune_mu;
std::map<std::array<int, 7>, TuneChoice> g_tune_cache;

float time_mixed_operator(fansgpu_ctx *ctx, bool tc)
{
    const StencilArgs sa = mixed_operator_args(ctx, 0);
    cudaEvent_t       e0 = nullptr, e1 = nullptr;
    float             ms = 1e30f;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
        return ms;
    auto launch = [&] {
        return tc ? launch_stencil_tc(sa, ctx->Wtc, ctx->nph, ctx->st) : launch_stencil<float>(sa, ctx->st);
    };
    if (launch() == cudaSuccess && cudaEventRecord(e0, ctx->st) == cudaSuccess) {
        bool ok = true;
        for (int k = 0; k < 3 && ok; ++k)
            ok = launch() == cudaSuccess;
        if (ok && cudaEventRecord(e1, ctx->st) == cudaSuccess && cudaEventSynchronize(e1) == cudaSuccess)
            cudaEventElapsedTime(&ms, e0, e1);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return ms;
}

int autotune(fansgpu_ctx *ctx)
{
    if (ctx->tuned)
        return 0;
    ctx->tuned       = true;
    const bool mixed = ctx->desc.precision == FANSGPU_MIXED;
    auto apply = [&](const TuneChoice &c) {
        ctx->cp64.var_z = c.v64[0] & 1; // the fused z + y forward pass (bit 1) is FP32 only
        ctx->cp64.var_y = c.v64[1];
        ctx->cp64.var_x = std::min(c.v64[2], 1); // the TMA-fed x pass (2) is FP32 only
        ctx->cp32.var_z = c.v32[0] & 1;
        ctx->cp32.fuse_zy = (c.v32[0] & 2) && zy_supported(ctx->g) ? 1 : 0;
        ctx->cp32.var_y = c.v32[1];
        ctx->cp32.var_x = (c.v32[2] == 2 && !ctx->cp32.tma) ? 0 : c.v32[2];
        if (c.tc_slower && ctx->use_tc) {
            ctx->tc_slower = true;
            ctx->use_tc    = false;
        }
        ctx->graphs_valid = false;
    };
    if (ctx->tune == 0)
        return 0;
    if (ctx->tune == 2) {
        TuneChoice c{};
        for (int k = 0; k < 3; ++k)
            c.v64[k] = c.v32[k] = ctx->tune_force[k];
        apply(c);
        return 0;
    }
    // the multi-RHS iteration runs every FFT pass over all right-hand sides: time the variants so
    const int rhs_tuned = multi_rhs_path(ctx) ? ctx->nrhs : 1;
    const std::array<int, 7> key{ctx->g.nx, ctx->g.ny, ctx->g.nz, ctx->C, ctx->desc.precision,
                                 (ctx->use_tc ? 1 : 0) + 2 * (ctx->tune == 3), rhs_tuned};
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto                        it = g_tune_cache.find(key);
    if (it == g_tune_cache.end()) {
        TuneChoice c{};
        // scratch CG scalars for the z-inverse pass's fused reduction (the context's own are
        // left untouched)
        CgScalars *tscal = nullptr;
        FANS_CUDA_CHECK(cudaMalloc((void **)&tscal, sizeof(CgScalars) * kMaxRhs));
        FANS_CUDA_CHECK(cudaMemsetAsync(tscal, 0, sizeof(CgScalars) * kMaxRhs, ctx->st));
        struct Free {
            CgScalars *p;
            ~Free() { cudaFree(p); }
        } free_tscal{tscal};
        FANS_CUDA_CHECK(tune_convolution_reg<double>(ctx->cp64, ctx->r, ctx->Kd, tscal, ctx->red, SITE_CONV, ctx->st));
        c.v64[0] = ctx->cp64.var_z;
        c.v64[1] = ctx->cp64.var_y;
        c.v64[2] = ctx->cp64.var_x;
        if (mixed) {
            ConvPlan<float> tp = ctx->cp32; // r32, Kd32 and the spectrum hold every RHS
            tp.nrhs            = rhs_tuned;
            tp.active          = nullptr;
            FANS_CUDA_CHECK(tune_convolution_reg<float>(tp, ctx->r32, ctx->Kd32, tscal, ctx->red, SITE_CONV, ctx->st));
            c.v32[0] = tp.var_z + 2 * tp.fuse_zy;
            c.v32[1] = tp.var_y;
            c.v32[2] = tp.var_x;
            if (ctx->use_tc && ctx->tune == 3)
                c.tc_slower = time_mixed_operator(ctx, false) < time_mixed_operator(ctx, true) ? 1 : 0;
        }
        FANS_CUDA_CHECK(cudaStreamSynchronize(ctx->st));
        it = g_tune_cache.emplace(key, c).first;
    }
    apply(it->second);
    return 0;
}

// After one graph-resident iteration (one thread): count it, record its
// residual estimate, and halt the loop wherever the host loop would do more
// than continue -- a reliable update or convergence test (est <= reliable *
// last_true or est_rel <= tol), n_it reached, or an error flag (non-finite
// norm, tensor-core wait timeout).  `first` is the check between the body's two
// iterations: it gates the second through the IF node, and ends the WHILE loop
// when it halts; the second check alone decides whether the loop goes on.
__global__ void k_loop_check(LoopCtl *c, const CgScalars *scal, double *hist, cudaGraphConditionalHandle h_while,
                             cudaGraphConditionalHandle h_if, int first)
{
    if (threadIdx.x != 0 || blockIdx.x != 0)
        return;
    const int    it  = ++c->iter;
    const double err = scal->err;
    if (it < c->cap)
        hist[it] = err;
    const double est_rel = c->relative ? err / c->err0 : err;
    const bool   halt = scal->converged < 0 || !(err == err) || est_rel <= c->tol || err <= c->reliable * c->last_true ||
                      it >= c->n_it || it + 1 >= c->cap;
    if (first) {
        cudaGraphSetConditional(h_if, halt ? 0u : 1u);
        if (halt)
            cudaGraphSetConditional(h_while, 0u);
    } else {
        cudaGraphSetConditional(h_while, halt ? 0u : 1u);
    }
}

// The multi-RHS counterpart of k_loop_check: records every active RHS's residual
// estimate (history row k) and halts where the host would act for any of them.
__global__ void k_loop_check_rhs(LoopCtlR *c, const CgScalars *scal, const int *act, double *hist,
                                 cudaGraphConditionalHandle h_while, cudaGraphConditionalHandle h_if, int first)
{
    if (threadIdx.x != 0 || blockIdx.x != 0)
        return;
    const int it   = ++c->iter;
    bool      halt = it >= c->n_it || it + 1 >= c->cap;
    for (int k = 0; k < c->nrhs; ++k) {
        if (!act[k])
            continue;
        const double err = scal[k].err;
        if (it < c->cap)
            hist[(size_t)k * c->cap + it] = err;
        const double est_rel = c->relative ? err / c->err0[k] : err;
        halt = halt || scal[k].converged < 0 || !(err == err) || est_rel <= c->tol || err <= c->reliable * c->last_true[k];
    }
    if (first) {
        cudaGraphSetConditional(h_if, halt ? 0u : 1u);
        if (halt)
            cudaGraphSetConditional(h_while, 0u);
    } else {
        cudaGraphSetConditional(h_while, halt ? 0u : 1u);
    }
}

// The inner loop as one CUDA graph per starting parity of the d ping-pong:
//   WHILE(h_while) { iteration(p); check; IF(h_if) { iteration(p ^ 1); check } }
// The two iterations are captured once and added as child graphs.
int build_loop_graphs(fansgpu_ctx *ctx, bool multi)
{
    int rc;
    if (!ctx->ctl) {
        if ((rc = dalloc(ctx, &ctx->ctl, 1)))
            return rc;
        FANS_CUDA_CHECK(cudaMallocHost((void **)&ctx->ctl_h, sizeof(LoopCtl)));
    }
    cudaGraph_t it[2] = {nullptr, nullptr};
    cudaError_t e     = cudaSuccess;
    for (int p = 0; p < 2 && e == cudaSuccess; ++p) {
        e = cudaStreamBeginCapture(ctx->st, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess)
            break;
        const cudaError_t ce = multi ? enqueue_mixed_iteration_rhs(ctx, p) : enqueue_mixed_iteration(ctx, p);
        e                    = cudaStreamEndCapture(ctx->st, &it[p]);
        if (ce != cudaSuccess)
            e = ce;
    }
    for (int p = 0; p < 2 && e == cudaSuccess; ++p) {
        if (ctx->iter_exec[p])
            cudaGraphExecDestroy(ctx->iter_exec[p]);
        ctx->iter_exec[p] = nullptr;
        e                 = cudaGraphInstantiate(&ctx->iter_exec[p], it[p], 0);
    }
    for (int p = 0; p < 2 && e == cudaSuccess; ++p) {
        if (ctx->graph_exec[p])
            cudaGraphExecDestroy(ctx->graph_exec[p]);
        ctx->graph_exec[p] = nullptr;
        cudaGraph_t top    = nullptr;
        e                  = cudaGraphCreate(&top, 0);
        cudaGraphConditionalHandle hw = 0, hi = 0;
        cudaGraphNodeParams        wp{}, ip{};
        cudaGraphNode_t            wn, n1, n2, n3, m1, m2;
        cudaGraph_t                body = nullptr, ib = nullptr;
        if (e == cudaSuccess)
            e = cudaGraphConditionalHandleCreate(&hw, top, 1, cudaGraphCondAssignDefault);
        if (e == cudaSuccess) {
            wp.type               = cudaGraphNodeTypeConditional;
            wp.conditional.handle = hw;
            wp.conditional.type   = cudaGraphCondTypeWhile;
            wp.conditional.size   = 1;
            e                     = cudaGraphAddNode(&wn, top, nullptr, nullptr, 0, &wp);
        }
        if (e == cudaSuccess) {
            body = wp.conditional.phGraph_out[0];
            e    = cudaGraphConditionalHandleCreate(&hi, body, 0, cudaGraphCondAssignDefault);
        }
        LoopCtl         *c  = ctx->ctl;
        LoopCtlR        *cr = ctx->ctlr;
        const CgScalars *sc = ctx->scal;
        const int       *ac = ctx->act;
        double          *h  = ctx->hist;
        int              f1 = 1, f0 = 0;
        void            *a1[] = {&c, &sc, &h, &hw, &hi, &f1};
        void            *a0[] = {&c, &sc, &h, &hw, &hi, &f0};
        void            *q1[] = {&cr, &sc, &ac, &h, &hw, &hi, &f1};
        void            *q0[] = {&cr, &sc, &ac, &h, &hw, &hi, &f0};
        cudaKernelNodeParams kp{};
        kp.func     = multi ? (void *)k_loop_check_rhs : (void *)k_loop_check;
        kp.gridDim  = dim3(1);
        kp.blockDim = dim3(32);
        if (e == cudaSuccess)
            e = cudaGraphAddChildGraphNode(&n1, body, nullptr, 0, it[p]);
        if (e == cudaSuccess) {
            kp.kernelParams = multi ? q1 : a1;
            e               = cudaGraphAddKernelNode(&n2, body, &n1, 1, &kp);
        }
        if (e == cudaSuccess) {
            ip.type               = cudaGraphNodeTypeConditional;
            ip.conditional.handle = hi;
            ip.conditional.type   = cudaGraphCondTypeIf;
            ip.conditional.size   = 1;
            e                     = cudaGraphAddNode(&n3, body, &n2, nullptr, 1, &ip);
        }
        if (e == cudaSuccess) {
            ib = ip.conditional.phGraph_out[0];
            e  = cudaGraphAddChildGraphNode(&m1, ib, nullptr, 0, it[p ^ 1]);
        }
        if (e == cudaSuccess) {
            kp.kernelParams = multi ? q0 : a0;
            e               = cudaGraphAddKernelNode(&m2, ib, &m1, 1, &kp);
        }
        if (e == cudaSuccess)
            e = cudaGraphInstantiate(&ctx->graph_exec[p], top, 0);
        if (top)
            cudaGraphDestroy(top);
    }
    for (cudaGraph_t g : it)
        if (g)
            cudaGraphDestroy(g);
    if (e != cudaSuccess)
        return fail(ctx, FANSGPU_ECUDA, "inner-loop graph: %s", cudaGetErrorString(e));
    ctx->graphs_valid = true;
    ctx->graphs_multi = multi;
    return 0;
}

// Mixed precision: FANS's flexible CG run on FP32 fields (stencil, FFT
// preconditioner, recursive residual) with FP64 dot products, an FP64
// solution and reliable updates -- the true residual R(u) recomputed in FP64
// whenever the FP32 residual has dropped by `reliable_delta` since the last
// refresh, and always before convergence is accepted.
int solve_cg_mixed(fansgpu_ctx *ctx, int *refinements)
{
    const long long n = ctx->n;
    int             rc;
    FANS_CUDA_CHECK(cudaMemsetAsync(ctx->s32, 0, sizeof(float) * n, ctx->st));
    FANS_CUDA_CHECK(cudaMemsetAsync(ctx->d32[0], 0, sizeof(float) * n, ctx->st));
    FANS_CUDA_CHECK(cudaMemsetAsync(ctx->e32, 0, sizeof(float) * n, ctx->st));
    ctx->cur_d = 0;
    if ((rc = init_scalars(ctx)))
        return rc;
    if ((rc = run_residual_df(ctx, ctx->scal)))
        return rc;
    { int en = tk_mark(ctx);
    FANS_CUDA_CHECK(launch_norm_fast(ctx->r, n, ctx->tol.measure, ctx->scal, 1, ctx->r32, ctx->red,
                                               SITE_NORM, ctx->st));
    tk_span(ctx, FANSGPU_K_NORM, en, tk_mark(ctx)); }
    if ((rc = sync_scalars(ctx)))
        return rc;
    ctx->iter = 0;
    ctx->err_all.assign(1, ctx->scal_h->err);
    if (ctx->scal_h->converged == -3)
        return fail(ctx, FANSGPU_ECUDA, "tensor-core operator: MMA completion wait timed out (initial residual)");
    if (!std::isfinite(ctx->scal_h->err))
        return fail(ctx, FANSGPU_ENAN, "non-finite initial residual norm (e.g. det F <= 0 in CompressibleNeoHookean)");
    *refinements      = 0;
    double err_rel    = err_value(ctx, ctx->scal_h->err);
    double last_true  = ctx->scal_h->err;
    if (ctx->use_graphs && !ctx->timing && ctx->hist_cap < ctx->tol.n_it + 2) {
        if (ctx->hist)
            cudaFree(ctx->hist);
        ctx->hist = nullptr;
        if ((rc = dalloc(ctx, &ctx->hist, ((size_t)ctx->tol.n_it + 2) * kMaxRhs)))
            return rc;
        ctx->hist_cap     = ctx->tol.n_it + 2;
        ctx->graphs_valid = false; // the graphs hold the history pointer
    }
    while (ctx->iter < ctx->tol.n_it && err_rel > ctx->tol.tolerance) {
        int done = 1; // iterations run by this pass
        if (ctx->use_graphs && !ctx->timing && ctx->iter > 0) { // the first iteration runs uncaptured
            if ((!ctx->graphs_valid || ctx->graphs_multi) && (rc = build_loop_graphs(ctx, false)))
                return rc;
        }
        if (ctx->use_graphs && !ctx->timing && ctx->iter > 0 && !ctx->loop_on_device) {
            FANS_CUDA_CHECK(cudaGraphLaunch(ctx->iter_exec[ctx->cur_d], ctx->st));
            if ((rc = sync_scalars(ctx)))
                return rc;
        } else if (ctx->use_graphs && !ctx->timing && ctx->iter > 0) {
            // iterate on the device until the check kernel halts the loop
            *ctx->ctl_h = LoopCtl{ctx->err_all[0], last_true, ctx->tol.tolerance, ctx->reliable_delta, ctx->iter,
                                  ctx->tol.n_it, ctx->tol.type == FANSGPU_RELATIVE, ctx->hist_cap};
            FANS_CUDA_CHECK(cudaMemcpyAsync(ctx->ctl, ctx->ctl_h, sizeof(LoopCtl), cudaMemcpyHostToDevice, ctx->st));
            FANS_CUDA_CHECK(cudaGraphLaunch(ctx->graph_exec[ctx->cur_d], ctx->st));
            FANS_CUDA_CHECK(cudaMemcpyAsync(ctx->ctl_h, ctx->ctl, sizeof(LoopCtl), cudaMemcpyDeviceToHost, ctx->st));
            if ((rc = sync_scalars(ctx)))
                return rc;
            done = ctx->ctl_h->iter - ctx->iter;
            if (done < 1 || ctx->iter + done > ctx->tol.n_it)
                return fail(ctx, FANSGPU_ECUDA, "inner-loop graph ran %d iterations from %d", done, ctx->iter);
            if (done > 1) { // the iterations it did not halt on only extend the history
                std::vector<double> h(done - 1);
                FANS_CUDA_CHECK(cudaMemcpyAsync(h.data(), ctx->hist + ctx->iter + 1, sizeof(double) * (done - 1),
                                                cudaMemcpyDeviceToHost, ctx->st));
                FANS_CUDA_CHECK(cudaStreamSynchronize(ctx->st));
                ctx->err_all.insert(ctx->err_all.end(), h.begin(), h.end());
                ctx->iter += done - 1;
            }
        } else {
            FANS_CUDA_CHECK(enqueue_mixed_iteration(ctx, ctx->cur_d));
            if ((rc = sync_scalars(ctx)))
                return rc;
        }
        ctx->cur_d ^= done & 1;
        ctx->iter++;
        if (ctx->scal_h->converged == -3)
            return fail(ctx, FANSGPU_ECUDA, "tensor-core operator: MMA completion wait timed out at iteration %d",
                        ctx->iter);
        if (ctx->scal_h->converged < 0)
            return fail(ctx, FANSGPU_ENAN, "non-finite residual norm at iteration %d", ctx->iter);
        double est     = ctx->scal_h->err;
        double est_rel = err_value(ctx, est);
        if (est_rel <= ctx->tol.tolerance || est <= ctx->reliable_delta * last_true) {
            // reliable update: fold the FP32 correction into u, true residual in
            // FP64, re-seed the FP32 residual
            FANS_CUDA_CHECK(launch_fold(ctx->u, ctx->e32, n, ctx->st));
            ctx->u_zero = false;
            if ((rc = run_residual_df(ctx, ctx->scal)))
                return rc;
            { int en = tk_mark(ctx);
    FANS_CUDA_CHECK(launch_norm_fast(ctx->r, n, ctx->tol.measure, ctx->scal, 0, ctx->r32,
                                                       ctx->red, SITE_NORM, ctx->st));
    tk_span(ctx, FANSGPU_K_NORM, en, tk_mark(ctx)); }
            if ((rc = sync_scalars(ctx)))
                return rc;
            if (ctx->scal_h->converged == -3)
                return fail(ctx, FANSGPU_ECUDA, "tensor-core operator: MMA completion wait timed out (true residual)");
            (*refinements)++;
            last_true = ctx->scal_h->err;
            ctx->err_all.push_back(last_true);
            err_rel = err_value(ctx, last_true);
        } else {
            ctx->err_all.push_back(est);
            err_rel = std::max(est_rel, ctx->tol.tolerance * (1.0 + 1e-12)); // never accept an estimate
        }
    }
    // corrections since the last reliable update (n_it reached) belong to u too
    FANS_CUDA_CHECK(launch_fold(ctx->u, ctx->e32, n, ctx->st));
    return 0;
}

// The reliable update of RHS k (the selected one after the call): fold its FP32
// correction into u_k, its true residual R(u_k) in double-float, ||r_k|| into
// scal[k] and the FP32 re-seed of r_k.  Host reads follow at the caller's sync.
// (The per-RHS vectors hold the state here: the members are loaded from them.)
int refresh_rhs(fansgpu_ctx *ctx, int k, bool fold, bool set_err0)
{
    const long long n = ctx->n;
    int             rc;
    load_rhs(ctx, k);
    if ((rc = setup(ctx))) // the force tables of g0_k
        return rc;
    if (fold) {
        FANS_CUDA_CHECK(launch_fold(ctx->u, ctx->e32 + (long long)k * n, n, ctx->st));
        ctx->u_zero       = false;
        ctx->rhs_uzero[k] = 0;
    }
    if ((rc = run_residual_df(ctx, ctx->scal + k)))
        return rc;
    int en = tk_mark(ctx);
    FANS_CUDA_CHECK(launch_norm_fast(ctx->r, n, ctx->tol.measure, ctx->scal + k, set_err0 ? 1 : 0,
                                     ctx->r32 + (long long)k * n, ctx->red, SITE_NORM, ctx->st));
    tk_span(ctx, FANSGPU_K_NORM, en, tk_mark(ctx));
    return 0;
}

int sync_scalars_rhs(fansgpu_ctx *ctx)
{
    FANS_CUDA_CHECK(cudaMemcpyAsync(ctx->scal_h, ctx->scal, sizeof(CgScalars) * ctx->nrhs, cudaMemcpyDeviceToHost,
                                    ctx->st));
    FANS_CUDA_CHECK(cudaStreamSynchronize(ctx->st));
    tk_flush(ctx);
    return 0;
}

// Multi-RHS mixed-precision CG: solve_cg_mixed's recurrences run for every
// right-hand side at once, each RHS with its own CG scalars, reliable updates and
// convergence test (so each takes exactly the iterations and values its own
// solve would).  An RHS leaves the iteration (its active flag drops, so every
// kernel skips it) once its true residual meets the tolerance.  The inner loop
// stays on the device between the points where any RHS needs the host.
int solve_cg_mixed_rhs(fansgpu_ctx *ctx, int only)
{
    const long long n = ctx->n;
    const int       R = ctx->nrhs, home = ctx->cur;
    auto            mine = [&](int k) { return only < 0 || k == only; }; // the RHS this solve covers
    int             rc;
    store_rhs(ctx);
    FANS_CUDA_CHECK(cudaMemsetAsync(ctx->s32, 0, sizeof(float) * n * R, ctx->st));
    FANS_CUDA_CHECK(cudaMemsetAsync(ctx->d32[0], 0, sizeof(float) * n * R, ctx->st));
    FANS_CUDA_CHECK(cudaMemsetAsync(ctx->e32, 0, sizeof(float) * n * R, ctx->st));
    ctx->cur_d = 0;
    for (int k = 0; k < R; ++k) {
        CgScalars s0{};
        s0.delta       = 1.0; // solverCG.h:82
        ctx->scal_h[k] = s0;
        ctx->act_h[k]  = 0;
        if (mine(k))
            ctx->rhs_ref[k] = 0;
    }
    FANS_CUDA_CHECK(cudaMemcpyAsync(ctx->scal, ctx->scal_h, sizeof(CgScalars) * R, cudaMemcpyHostToDevice, ctx->st));
    for (int k = 0; k < R; ++k)
        if (mine(k) && (rc = refresh_rhs(ctx, k, false, true))) // r_k = R(u_k) (compute_residual<2>, solverCG.h:76)
            return rc;
    if ((rc = sync_scalars_rhs(ctx)))
        return rc;
    std::vector<double> last_true(R), err_rel(R);
    std::vector<char>   on(R, 0);
    int                 n_on = 0;
    for (int k = 0; k < R; ++k) {
        if (!mine(k))
            continue;
        if (ctx->scal_h[k].converged == -3)
            return fail(ctx, FANSGPU_ECUDA, "tensor-core operator: MMA completion wait timed out (true residual)");
        const double err = ctx->scal_h[k].err;
        ctx->rhs_err[k].assign(1, err);
        ctx->rhs_iter[k] = 0;
        if (!std::isfinite(err))
            return fail(ctx, FANSGPU_ENAN, "RHS %d: non-finite initial residual norm", k);
        last_true[k] = err;
        err_rel[k]   = ctx->tol.type == FANSGPU_ABSOLUTE ? err : 100.0; // solver.h:432-451 at iteration 0
        on[k]        = ctx->tol.n_it > 0 && err_rel[k] > ctx->tol.tolerance;
        if (on[k]) {
            ctx->rhs_uzero[k] = 0; // u_k is updated from here on
            ++n_on;
        }
        ctx->act_h[k] = on[k];
    }
    const bool graphs = ctx->use_graphs && !ctx->timing;
    if (graphs && ctx->hist_cap < ctx->tol.n_it + 2) {
        if (ctx->hist)
            cudaFree(ctx->hist);
        ctx->hist = nullptr;
        if ((rc = dalloc(ctx, &ctx->hist, ((size_t)ctx->tol.n_it + 2) * kMaxRhs)))
            return rc;
        ctx->hist_cap     = ctx->tol.n_it + 2;
        ctx->graphs_valid = false; // the graphs hold the history pointer
    }
    int it = 0; // iterations of the active right-hand sides (they advance together)
    while (n_on > 0 && it < ctx->tol.n_it) {
        FANS_CUDA_CHECK(cudaMemcpyAsync(ctx->act, ctx->act_h, sizeof(int) * R, cudaMemcpyHostToDevice, ctx->st));
        int done = 1;
        if (graphs && it > 0 && (!ctx->graphs_valid || !ctx->graphs_multi) && (rc = build_loop_graphs(ctx, true)))
            return rc;
        if (graphs && it > 0 && !ctx->loop_on_device) {
            FANS_CUDA_CHECK(cudaGraphLaunch(ctx->iter_exec[ctx->cur_d], ctx->st));
            if ((rc = sync_scalars_rhs(ctx)))
                return rc;
        } else if (graphs && it > 0) {
            LoopCtlR &c = *ctx->ctlr_h;
            for (int k = 0; k < kMaxRhs; ++k) {
                c.err0[k]      = k < R ? ctx->rhs_err[k][0] : 1.0;
                c.last_true[k] = k < R ? last_true[k] : 0.0;
            }
            c.tol      = ctx->tol.tolerance;
            c.reliable = ctx->reliable_delta;
            c.iter     = it;
            c.n_it     = ctx->tol.n_it;
            c.relative = ctx->tol.type == FANSGPU_RELATIVE;
            c.cap      = ctx->hist_cap;
            c.nrhs     = R;
            FANS_CUDA_CHECK(cudaMemcpyAsync(ctx->ctlr, ctx->ctlr_h, sizeof(LoopCtlR), cudaMemcpyHostToDevice, ctx->st));
            FANS_CUDA_CHECK(cudaGraphLaunch(ctx->graph_exec[ctx->cur_d], ctx->st));
            FANS_CUDA_CHECK(cudaMemcpyAsync(ctx->ctlr_h, ctx->ctlr, sizeof(LoopCtlR), cudaMemcpyDeviceToHost, ctx->st));
            if ((rc = sync_scalars_rhs(ctx)))
                return rc;
            done = c.iter - it;
            if (done < 1 || it + done > ctx->tol.n_it)
                return fail(ctx, FANSGPU_ECUDA, "inner-loop graph ran %d iterations from %d", done, it);
            if (done > 1) { // iterations the loop did not halt on only extend the histories
                std::vector<double> h(done - 1);
                for (int k = 0; k < R; ++k) {
                    if (!on[k])
                        continue;
                    FANS_CUDA_CHECK(cudaMemcpyAsync(h.data(), ctx->hist + (size_t)k * ctx->hist_cap + it + 1,
                                                    sizeof(double) * (done - 1), cudaMemcpyDeviceToHost, ctx->st));
                    FANS_CUDA_CHECK(cudaStreamSynchronize(ctx->st));
                    ctx->rhs_err[k].insert(ctx->rhs_err[k].end(), h.begin(), h.end());
                }
            }
        } else {
            FANS_CUDA_CHECK(enqueue_mixed_iteration_rhs(ctx, ctx->cur_d));
            if ((rc = sync_scalars_rhs(ctx)))
                return rc;
        }
        ctx->cur_d ^= done & 1;
        it += done;
        std::vector<int> due;
        for (int k = 0; k < R; ++k) {
            if (!on[k])
                continue;
            ctx->rhs_iter[k] = it;
            const CgScalars &sc = ctx->scal_h[k];
            if (sc.converged == -3)
                return fail(ctx, FANSGPU_ECUDA, "tensor-core operator: MMA completion wait timed out at iteration %d",
                            it);
            if (sc.converged < 0)
                return fail(ctx, FANSGPU_ENAN, "RHS %d: non-finite residual norm at iteration %d", k, it);
            const double est     = sc.err;
            const double est_rel = ctx->tol.type == FANSGPU_ABSOLUTE ? est : est / ctx->rhs_err[k][0];
            if (est_rel <= ctx->tol.tolerance || est <= ctx->reliable_delta * last_true[k])
                due.push_back(k);
            else
                ctx->rhs_err[k].push_back(est);
        }
        // reliable updates of the RHS that asked for one; the others go on from their estimates
        for (int k : due)
            if ((rc = refresh_rhs(ctx, k, true, false)))
                return rc;
        if (!due.empty() && (rc = sync_scalars_rhs(ctx)))
            return rc;
        for (int k : due) {
            if (ctx->scal_h[k].converged == -3)
                return fail(ctx, FANSGPU_ECUDA, "tensor-core operator: MMA completion wait timed out (true residual)");
            ctx->rhs_ref[k]++;
            last_true[k]     = ctx->scal_h[k].err;
            ctx->rhs_err[k].push_back(last_true[k]);
            const double rel = ctx->tol.type == FANSGPU_ABSOLUTE ? last_true[k] : last_true[k] / ctx->rhs_err[k][0];
            if (!(rel > ctx->tol.tolerance)) { // converged (the true residual); NaN was caught by the norm
                on[k]         = 0;
                ctx->act_h[k] = 0;
                --n_on;
            }
        }
    }
    // corrections since the last reliable update (n_it reached) belong to u too
    FANS_CUDA_CHECK(launch_fold(ctx->u0, ctx->e32, n * R, ctx->st));
    for (int k = 0; k < R; ++k)
        if (mine(k) && ctx->rhs_iter[k] > 0)
            ctx->rhs_uzero[k] = 0;
    load_rhs(ctx, home);
    return 0;
}

int mixed_update(fansgpu_ctx *ctx);

// SolverFP::internalSolve: u -= G*r; r = R(u).
int solve_fp64(fansgpu_ctx *ctx)
{
    const long long n = ctx->n;
    int             rc;
    if ((rc = init_scalars(ctx)))
        return rc;
    if ((rc = run_residual64(ctx, ctx->u, ctx->r)))
        return rc;
    { int en = tk_mark(ctx);
    FANS_CUDA_CHECK(launch_norm<double, float>(ctx->r, n, ctx->tol.measure, ctx->scal, 1, nullptr, ctx->red,
                                               SITE_NORM, ctx->st));
    tk_span(ctx, FANSGPU_K_NORM, en, tk_mark(ctx)); }
    if ((rc = sync_scalars(ctx)))
        return rc;
    ctx->iter = 0;
    ctx->err_all.assign(1, ctx->scal_h->err);
    if (!std::isfinite(ctx->scal_h->err))
        return fail(ctx, FANSGPU_ENAN, "non-finite initial residual norm (e.g. det F <= 0 in CompressibleNeoHookean)");
    double err_rel = err_value(ctx, ctx->scal_h->err);
    if (ctx->tol.n_it > 0 && err_rel > ctx->tol.tolerance)
        ctx->u_zero = false; // u is updated from here on
    while (ctx->iter < ctx->tol.n_it && err_rel > ctx->tol.tolerance) {
        ConvArgs ca{ctx->r, ctx->s, 1.0, 0, ctx->scal, ctx->red, SITE_CONV};
        FANS_CUDA_CHECK(run_conv<double>(ctx, ctx->cp64, ca));
        FANS_CUDA_CHECK(launch_axpy<double>(ctx->u, ctx->s, -1.0, n, ctx->st));
        if ((rc = mixed_update(ctx)) || (rc = run_residual64(ctx, ctx->u, ctx->r)))
            return rc;
        { int en = tk_mark(ctx);
    FANS_CUDA_CHECK(launch_norm<double, float>(ctx->r, n, ctx->tol.measure, ctx->scal, 0, nullptr, ctx->red,
                                                   SITE_NORM, ctx->st));
    tk_span(ctx, FANSGPU_K_NORM, en, tk_mark(ctx)); }
        if ((rc = sync_scalars(ctx)))
            return rc;
        ctx->iter++;
        ctx->err_all.push_back(ctx->scal_h->err);
        if (ctx->scal_h->converged < 0)
            return fail(ctx, FANSGPU_ENAN, "non-finite residual norm at iteration %d", ctx->iter);
        err_rel = err_value(ctx, ctx->scal_h->err);
    }
    return 0;
}

int strain_stress(fansgpu_ctx *ctx, int phase_filter, double *strain_f, double *stress_f, double *out,
                  double *strain_gp = nullptr, double *stress_gp = nullptr, double *flag_f = nullptr);

// MixedBCController::update (mixedBCs.h:160-177): g0_F += M (P_F - Q_F^T <sigma>).
int mixed_update(fansgpu_ctx *ctx)
{
    if (!ctx->mixed_active || ctx->idxF.empty())
        return 0;
    int    rc;
    double red[32];
    if ((rc = setup(ctx)) || (rc = strain_stress(ctx, -1, nullptr, nullptr, red, nullptr, nullptr, nullptr)))
        return rc;
    const int nf = (int)ctx->idxF.size();
    std::vector<double> rhs(nf);
    for (int a = 0; a < nf; ++a)
        rhs[a] = ctx->PF[a] - red[ctx->nstr + ctx->idxF[a]] / (double)ctx->N;
    for (int a = 0; a < nf; ++a) {
        double dE = 0.0;
        for (int b = 0; b < nf; ++b)
            dE += ctx->Mmix[a * nf + b] * rhs[b];
        ctx->g0[ctx->idxF[a]] += dE;
    }
    ctx->force_dirty = true;
    return setup(ctx);
}

// <a, b> on the device into *slot (a CgScalars member); read on the next sync.
int dot_to(fansgpu_ctx *ctx, const double *a, const double *b, double *slot)
{
    FANS_CUDA_CHECK(launch_dot(a, b, ctx->n, slot, ctx->red, SITE_DOT, ctx->st));
    return 0;
}

int host_dot(fansgpu_ctx *ctx, const double *a, const double *b, double *out)
{
    int rc;
    if ((rc = dot_to(ctx, a, b, &ctx->scal->aux[0])) || (rc = sync_scalars(ctx)))
        return rc;
    *out = ctx->scal_h->aux[0];
    return 0;
}

// SolverCG::internalSolve with nonlinear laws (solverCG.h:62-117): the flexible
// CG direction, then LineSearchSecant (solverCG.h:120-160) on u along d, with
// r replaced by the last line-search residual.  FP64 throughout; the scalar
// secant logic runs on the host between device dot products.
int solve_cg_nl(fansgpu_ctx *ctx)
{
    const long long n = ctx->n;
    double         *d = ctx->dd[0], *rnew = ctx->Kd;
    int             rc;
    ctx->alpha_warm = 0.1; // solverCG.h:68
    FANS_CUDA_CHECK(cudaMemsetAsync(ctx->s, 0, sizeof(double) * n, ctx->st));
    FANS_CUDA_CHECK(cudaMemsetAsync(d, 0, sizeof(double) * n, ctx->st));
    if ((rc = init_scalars(ctx)))
        return rc;
    if ((rc = run_residual64(ctx, ctx->u, ctx->r)))
        return rc;
    { int en = tk_mark(ctx);
    FANS_CUDA_CHECK(launch_norm<double, float>(ctx->r, n, ctx->tol.measure, ctx->scal, 1, nullptr, ctx->red,
                                               SITE_NORM, ctx->st));
    tk_span(ctx, FANSGPU_K_NORM, en, tk_mark(ctx)); }
    if ((rc = sync_scalars(ctx)))
        return rc;
    ctx->iter = 0;
    ctx->err_all.assign(1, ctx->scal_h->err);
    if (!std::isfinite(ctx->scal_h->err))
        return fail(ctx, FANSGPU_ENAN, "non-finite initial residual norm (e.g. det F <= 0 in CompressibleNeoHookean)");
    double err_rel = err_value(ctx, ctx->scal_h->err);
    if (ctx->tol.n_it > 0 && err_rel > ctx->tol.tolerance)
        ctx->u_zero = false;
    while (ctx->iter < ctx->tol.n_it && err_rel > ctx->tol.tolerance) {
        // deltamid = <r, s>; s = -G*r; delta = <r, s>; beta (solverCG.h:85-94)
        if ((rc = dot_to(ctx, ctx->r, ctx->s, &ctx->scal->deltamid)))
            return rc;
        ConvArgs ca{ctx->r, ctx->s, -1.0, 1, ctx->scal, ctx->red, SITE_CONV};
        FANS_CUDA_CHECK(run_conv<double>(ctx, ctx->cp64, ca));
        FANS_CUDA_CHECK(launch_direction(d, ctx->s, n, ctx->scal, ctx->st));
        // LineSearchSecant
        const int    max_it = ctx->tol.ls_max_iter;
        const double ls_tol = ctx->tol.ls_tol;
        double       err = 10.0, alpha_prev = 0.0, alpha_curr = ctx->alpha_warm, rpd, r1pd;
        int          it  = 0;
        if ((rc = host_dot(ctx, ctx->r, d, &rpd)))
            return rc;
        FANS_CUDA_CHECK(launch_axpy<double>(ctx->u, d, alpha_curr, n, ctx->st));
        if ((rc = mixed_update(ctx)) || (rc = run_residual64(ctx, ctx->u, rnew)) || (rc = host_dot(ctx, rnew, d, &r1pd)))
            return rc;
        while (it < max_it && err > ls_tol) {
            const double denom = r1pd - rpd;
            if (std::fabs(denom) < 1e-14 * (std::fabs(r1pd) + std::fabs(rpd)))
                break;
            double alpha_next = alpha_curr - r1pd * (alpha_curr - alpha_prev) / denom;
            if (alpha_next <= 0.0)
                alpha_next = 0.5 * (alpha_prev + alpha_curr);
            err = std::fabs(alpha_next - alpha_curr);
            FANS_CUDA_CHECK(launch_axpy<double>(ctx->u, d, alpha_next - alpha_curr, n, ctx->st));
            alpha_prev = alpha_curr;
            rpd        = r1pd;
            alpha_curr = alpha_next;
            ++it;
            if ((rc = mixed_update(ctx)) || (rc = run_residual64(ctx, ctx->u, rnew)) ||
                (rc = host_dot(ctx, rnew, d, &r1pd)))
                return rc;
        }
        ctx->alpha_warm = (it == max_it && err > ls_tol) ? 0.1 : alpha_curr;
        FANS_CUDA_CHECK(cudaMemcpyAsync(ctx->r, rnew, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx->st));
        { int en = tk_mark(ctx);
        FANS_CUDA_CHECK(launch_norm<double, float>(ctx->r, n, ctx->tol.measure, ctx->scal, 0, nullptr, ctx->red,
                                                   SITE_NORM, ctx->st));
        tk_span(ctx, FANSGPU_K_NORM, en, tk_mark(ctx)); }
        if ((rc = sync_scalars(ctx)))
            return rc;
        ctx->iter++;
        ctx->err_all.push_back(ctx->scal_h->err);
        if (ctx->scal_h->converged < 0 || !std::isfinite(alpha_curr))
            return fail(ctx, FANSGPU_ENAN, "non-finite residual norm at iteration %d", ctx->iter);
        err_rel = err_value(ctx, ctx->scal_h->err);
    }
    return 0;
}

// MaterialManager::update_internal_variables (MaterialManager.h:207-213).
int commit_ivars(fansgpu_ctx *ctx)
{
    if (ctx->all_linear || !ctx->ep_t)
        return 0;
    const long long nep = 6LL * ctx->ngp * ctx->N, nq = (long long)ctx->ngp * ctx->N;
    FANS_CUDA_CHECK(cudaMemcpyAsync(ctx->ep_t, ctx->ep, sizeof(double) * nep, cudaMemcpyDeviceToDevice, ctx->st));
    FANS_CUDA_CHECK(cudaMemcpyAsync(ctx->q_t, ctx->q, sizeof(double) * nq, cudaMemcpyDeviceToDevice, ctx->st));
    if (ctx->pb_t)
        FANS_CUDA_CHECK(cudaMemcpyAsync(ctx->pb_t, ctx->pb, sizeof(double) * nep, cudaMemcpyDeviceToDevice, ctx->st));
    return 0;
}

int strain_stress(fansgpu_ctx *ctx, int phase_filter, double *strain_f, double *stress_f, double *out,
                  double *strain_gp, double *stress_gp, double *flag_f)
{
    if (ctx->all_linear && !ctx->vscale && !strain_f && !stress_f && !strain_gp && !stress_gp && !flag_f &&
        ctx->nph <= 2) {
        // averages only: per-phase strain sums, stresses by linearity (C_ph times the sums)
        StrainStressArgs a{};
        a.g     = ctx->g;
        a.C     = ctx->C;
        a.nstr  = ctx->nstr;
        a.u     = ctx->u;
        a.ms    = ctx->d_ms;
        for (int d = 0; d < 3; ++d)
            a.inv4l[d] = 0.25 / ctx->le[d];
        a.g0       = ctx->g0_d;
        a.nph      = ctx->nph;
        a.out_red  = ctx->red_out;
        a.red      = ctx->red;
        a.red_site = SITE_SS;
        const int ns = ctx->nstr, nphm = 2;
        int       e0 = tk_mark(ctx);
        FANS_CUDA_CHECK(launch_strain_sums(a, ctx->st));
        tk_span(ctx, FANSGPU_K_STRAIN_STRESS, e0, tk_mark(ctx));
        double sums[4 * 7];
        FANS_CUDA_CHECK(cudaMemcpyAsync(sums, ctx->red_out, sizeof(double) * nphm * (ns + 1), cudaMemcpyDeviceToHost,
                                        ctx->st));
        FANS_CUDA_CHECK(cudaStreamSynchronize(ctx->st));
        tk_flush(ctx);
        std::vector<double> Cm(ns * ns);
        for (int i = 0; i < 2 * ns + 1; ++i)
            out[i] = 0.0;
        for (int ph = 0; ph < ctx->nph; ++ph) {
            if (phase_filter >= 0 && ph != phase_filter)
                continue;
            fe::law_C(ctx->law[ph], ctx->prm[ph], ns, Cm.data());
            for (int i = 0; i < ns; ++i) {
                out[i] += sums[ph * ns + i];
                double acc = 0.0;
                for (int k = 0; k < ns; ++k)
                    acc += Cm[i * ns + k] * sums[ph * ns + k];
                out[ns + i] += acc;
            }
            out[2 * ns] += sums[nphm * ns + ph];
        }
        return 0;
    }
    if (!ctx->all_linear || ctx->vscale || strain_gp || stress_gp || flag_f) {
        // per-Gauss-point law evaluation (Matmodel::getStrainStress, matmodel.h:203-225)
        ElementArgs a  = element_args(ctx, ctx->u, ELEM_AVERAGES);
        a.phase_filter = phase_filter;
        a.strain       = strain_f;
        a.stress       = stress_f;
        a.strain_gp    = strain_gp;
        a.stress_gp    = stress_gp;
        a.flag         = flag_f;
        a.out_red      = ctx->red_out;
        int e0         = tk_mark(ctx);
        FANS_CUDA_CHECK(launch_element(a, ctx->st));
        tk_span(ctx, FANSGPU_K_STRAIN_STRESS, e0, tk_mark(ctx));
        FANS_CUDA_CHECK(cudaMemcpyAsync(out, ctx->red_out, sizeof(double) * (2 * ctx->nstr + 1),
                                        cudaMemcpyDeviceToHost, ctx->st));
        FANS_CUDA_CHECK(cudaStreamSynchronize(ctx->st));
        tk_flush(ctx);
        return 0;
    }
    StrainStressArgs a{};
    a.g            = ctx->g;
    a.C            = ctx->C;
    a.nstr         = ctx->nstr;
    a.u            = ctx->u;
    a.ms           = ctx->d_ms;
    for (int d = 0; d < 3; ++d)
        a.inv4l[d] = 0.25 / ctx->le[d];
    a.Cph          = ctx->Cph;
    a.g0           = ctx->g0_d;
    a.nph          = ctx->nph;
    a.phase_filter = phase_filter;
    a.strain       = strain_f;
    a.stress       = stress_f;
    a.out_red      = ctx->red_out;
    a.red          = ctx->red;
    a.red_site     = SITE_SS;
    int e0 = tk_mark(ctx);
    FANS_CUDA_CHECK(launch_strain_stress(a, ctx->st));
    tk_span(ctx, FANSGPU_K_STRAIN_STRESS, e0, tk_mark(ctx));
    FANS_CUDA_CHECK(cudaMemcpyAsync(out, ctx->red_out, sizeof(double) * (2 * ctx->nstr + 1), cudaMemcpyDeviceToHost,
                                    ctx->st));
    FANS_CUDA_CHECK(cudaStreamSynchronize(ctx->st));
    tk_flush(ctx);
    return 0;
}

} // namespace

extern "C" {

const char *fansgpu_version(void) { return "fans_gb300 0.1 (sm_103a)"; }

const char *fansgpu_last_error(const fansgpu_ctx *ctx)
{
    return ctx ? ctx->err_msg.c_str() : g_create_error.c_str();
}

int fansgpu_create(const fansgpu_desc *desc, fansgpu_ctx **out)
{
    if (!desc || !out)
        return fail(nullptr, FANSGPU_EINVAL, "fansgpu_create: null argument");
    *out = nullptr;
    const int *n = desc->n;
    for (int i = 0; i < 3; ++i)
        if (n[i] < 4 || n[i] > 1024 || (n[i] % 2) != 0)
            return fail(nullptr, FANSGPU_EUNSUPPORTED, "grid dimension %d = %d: need an even size in [4, 1024]", i,
                        n[i]);
    if (desc->howmany != 1 && desc->howmany != 3)
        return fail(nullptr, FANSGPU_EINVAL, "howmany must be 1 (thermal) or 3 (small-strain mechanics)");
    if (desc->fe_type < 0 || desc->fe_type > 2)
        return fail(nullptr, FANSGPU_EINVAL, "FE_type must be one of: 'HEX8', 'HEX8R', or 'BBAR'");
    if (desc->precision != FANSGPU_FP64 && desc->precision != FANSGPU_MIXED)
        return fail(nullptr, FANSGPU_EINVAL, "precision must be FANSGPU_FP64 or FANSGPU_MIXED");
    if (desc->method != FANSGPU_CG && desc->method != FANSGPU_FP && desc->method != FANSGPU_NEWTON)
        return fail(nullptr, FANSGPU_EINVAL, "method must be cg, fp or newton");
    if (desc->precision == FANSGPU_MIXED && desc->method != FANSGPU_CG)
        return fail(nullptr, FANSGPU_EUNSUPPORTED, "mixed precision is implemented for the CG method");
    if (desc->strain_type != FANSGPU_SMALL_STRAIN && desc->strain_type != FANSGPU_LARGE_STRAIN)
        return fail(nullptr, FANSGPU_EINVAL, "strain_type must be either 'small' or 'large'");
    if (desc->strain_type == FANSGPU_LARGE_STRAIN && desc->howmany != 3)
        return fail(nullptr, FANSGPU_EINVAL, "large strain needs a mechanical problem (howmany = 3)");
    for (int i = 0; i < 3; ++i)
        if (!(desc->L[i] > 0))
            return fail(nullptr, FANSGPU_EINVAL, "L must be positive");
    const int nrhs = desc->n_rhs == 0 ? 1 : desc->n_rhs;
    if (nrhs < 1 || nrhs > FANSGPU_MAX_RHS)
        return fail(nullptr, FANSGPU_EINVAL, "n_rhs = %d: 1..%d right-hand sides", desc->n_rhs, FANSGPU_MAX_RHS);
    if (nrhs > 1 && desc->method == FANSGPU_NEWTON)
        return fail(nullptr, FANSGPU_EUNSUPPORTED, "Newton-Krylov solves one right-hand side (n_rhs = 1)");

    fansgpu_ctx *ctx = new fansgpu_ctx();
    ctx->desc        = *desc;
    if (const char *ev = std::getenv("FANSGPU_STENCIL")) { // "simt": CUDA-core operator; "tc": per-phase 3xTF32;
        ctx->tc_allowed       = std::strcmp(ev, "simt") != 0; // "basis": the multi-RHS basis operator
        ctx->tc_legacy        = std::strcmp(ev, "tc") == 0;
        ctx->tcb_basis_forced = std::strcmp(ev, "basis") == 0;
    }
    if (const char *ev = std::getenv("FANSGPU_TUNE")) { // "0": default tiles; "all": + operator; "zyx": forced
        if (std::strcmp(ev, "0") == 0)
            ctx->tune = 0;
        else if (std::strcmp(ev, "all") == 0)
            ctx->tune = 3;
        else if (std::strlen(ev) == 3 && std::strchr("0123", ev[0]) && std::strchr("01", ev[1]) &&
                 std::strchr("012", ev[2])) {
            ctx->tune = 2;
            for (int k = 0; k < 3; ++k)
                ctx->tune_force[k] = ev[k] - '0';
        }
    }
    if (const char *ev = std::getenv("FANSGPU_SPECTRAL_DOT")) // "0": the FP32 <r, s> from r and s in the z pass
        ctx->spectral_dot = std::strcmp(ev, "0") != 0;
    if (const char *ev = std::getenv("FANSGPU_EXACT")) // "df": FP64-accurate products on the CUDA cores
        ctx->exact_tc = std::strcmp(ev, "df") != 0;
    if (const char *ev = std::getenv("FANSGPU_FP64_OPERATOR")) // "dfma": the FP64 CG operator on the FP64 pipe
        ctx->fp64_df = std::strcmp(ev, "dfma") != 0;
    if (const char *ev = std::getenv("FANSGPU_TC_BACKOFF")) // ns between the operator consumers' polls
        ctx->tc_backoff_ns = std::max(0, std::min(100000, std::atoi(ev)));
    if (const char *ev = std::getenv("FANSGPU_GRAPHS")) { // "0": no graphs; "iter": one graph per iteration
        ctx->use_graphs     = std::strcmp(ev, "0") != 0;
        ctx->loop_on_device = std::strcmp(ev, "iter") != 0;
    }
    ctx->g           = Grid3{n[0], n[1], n[2]};
    ctx->C           = desc->howmany;
    ctx->nstr        = desc->strain_type == FANSGPU_LARGE_STRAIN ? 9 : nstr_of(ctx->C);
    ctx->N           = ctx->g.N();
    ctx->n           = ctx->N * ctx->C;
    for (int i = 0; i < 3; ++i)
        ctx->le[i] = desc->L[i] / (double)n[i]; // reader.cpp:293-296
    ctx->ve  = ctx->le[0] * ctx->le[1] * ctx->le[2];
    ctx->ngp = fe::gauss_B(desc->fe_type, ctx->C, ctx->le, ctx->B, ctx->nstr);
    const int NC = 8 * ctx->C, ns = ctx->nstr;
    ctx->Bbar.assign(ns * NC, 0.0);
    for (int gp = 0; gp < ctx->ngp; ++gp)
        for (int i = 0; i < ns * NC; ++i)
            ctx->Bbar[i] += ctx->B[gp * ns * NC + i] / ctx->ngp;
    ctx->g0.assign(ns, 0.0);
    ctx->kapparef.assign(ns * ns, 0.0);
    ctx->nrhs = nrhs;
    ctx->rhs_g0.assign(nrhs, std::vector<double>(ns, 0.0));
    ctx->rhs_err.assign(nrhs, {});
    ctx->rhs_iter.assign(nrhs, 0);
    ctx->rhs_ref.assign(nrhs, 0);
    ctx->rhs_uzero.assign(nrhs, 1);

    int rc = 0;
    auto bail = [&](int code) {
        g_create_error = ctx->err_msg;
        fansgpu_destroy(ctx);
        return code;
    };
    if (cudaStreamCreateWithFlags(&ctx->st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&ctx->ev0) != cudaSuccess || cudaEventCreate(&ctx->ev1) != cudaSuccess) {
        fail(ctx, FANSGPU_ECUDA, "no CUDA device/stream: %s", cudaGetErrorString(cudaGetLastError()));
        return bail(FANSGPU_ECUDA);
    }
    const long long nn = ctx->n, N = ctx->N;
    const int       nzh = ctx->g.nz / 2 + 1, nzp = ((nzh + 15) / 16) * 16, NT = ctx->C * (ctx->C + 1) / 2;
    const long long F = (long long)ctx->g.nx * ctx->g.ny * nzh;
    const long long nspec = (long long)ctx->C * ctx->g.nx * ctx->g.ny * nzp;
    const bool      mixed = desc->precision == FANSGPU_MIXED;
    const long long nr = (long long)nrhs * nn; // per-RHS fields
    if ((rc = dalloc(ctx, &ctx->d_ms, N)) || (rc = dalloc(ctx, &ctx->u0, nr)) || (rc = dalloc(ctx, &ctx->r0, nr)) ||
        (rc = dalloc(ctx, &ctx->s, nn)) || (rc = dalloc(ctx, &ctx->dd[0], nn)) ||
        (rc = dalloc(ctx, &ctx->dd[1], nn)) || (rc = dalloc(ctx, &ctx->Kd, nn)) ||
        (rc = dalloc(ctx, &ctx->up0, nr)) || (rc = dalloc(ctx, &ctx->spec64, nspec)) ||
        (rc = dalloc(ctx, &ctx->G64, F * NT)) || (rc = dalloc(ctx, &ctx->staging, N * std::max(ctx->C, ns))) ||
        (rc = dalloc(ctx, &ctx->scal, kMaxRhs)) || (rc = dalloc(ctx, &ctx->act, kMaxRhs)) ||
        (rc = dalloc(ctx, &ctx->ctlr, 1)) ||
        (rc = dalloc(ctx, &ctx->red.partials, (size_t)max_reduction_blocks(ctx->g, ctx->C) * kMaxRed)) ||
        (rc = dalloc(ctx, &ctx->red.counter, kRedSites)) || (rc = dalloc(ctx, &ctx->red_out, 64)) ||
        (rc = dalloc(ctx, &ctx->K0c, NC * NC)) || (rc = dalloc(ctx, &ctx->Bbar_d, ns * NC)) ||
        (rc = dalloc(ctx, &ctx->Bgp_d, (size_t)ctx->ngp * ns * NC)) ||
        (rc = dalloc(ctx, &ctx->g0_d, ns)) || (rc = dalloc(ctx, &ctx->max_id, 1)) ||
        (rc = dalloc(ctx, &ctx->trig, 2 * (ctx->g.nx + ctx->g.ny + nzh))))
        return bail(rc);
    ctx->u     = ctx->u0;
    ctx->r     = ctx->r0;
    ctx->uprev = ctx->up0;
    if (mixed) {
        if ((rc = dalloc(ctx, &ctx->r32, nr)) || (rc = dalloc(ctx, &ctx->s32, nr)) ||
            (rc = dalloc(ctx, &ctx->d32[0], nr)) || (rc = dalloc(ctx, &ctx->d32[1], nr)) ||
            (rc = dalloc(ctx, &ctx->Kd32, nr)) || (rc = dalloc(ctx, &ctx->e32, nr)) ||
            (rc = dalloc(ctx, &ctx->spec32, nspec * nrhs)) ||
            (rc = dalloc(ctx, &ctx->G32, (long long)ctx->g.nx * ctx->g.ny * nzp * NT)))
            return bail(rc);
    }
    if (cudaMallocHost((void **)&ctx->scal_h, sizeof(CgScalars) * kMaxRhs) != cudaSuccess ||
        cudaMallocHost((void **)&ctx->act_h, sizeof(int) * kMaxRhs) != cudaSuccess ||
        cudaMallocHost((void **)&ctx->ctlr_h, sizeof(LoopCtlR)) != cudaSuccess) {
        fail(ctx, FANSGPU_ENOMEM, "pinned host allocation failed");
        return bail(FANSGPU_ENOMEM);
    }
    cudaMemsetAsync(ctx->red.counter, 0, sizeof(unsigned) * kRedSites, ctx->st);
    cudaMemsetAsync(ctx->u0, 0, sizeof(double) * nr, ctx->st);
    cudaMemsetAsync(ctx->up0, 0, sizeof(double) * nr, ctx->st);
    cudaMemsetAsync(ctx->r0, 0, sizeof(double) * nr, ctx->st);
    cudaMemsetAsync(ctx->scal, 0, sizeof(CgScalars) * kMaxRhs, ctx->st);
    cudaMemcpyAsync(ctx->Bbar_d, ctx->Bbar.data(), sizeof(double) * ns * NC, cudaMemcpyHostToDevice, ctx->st);
    cudaMemcpyAsync(ctx->Bgp_d, ctx->B.data(), sizeof(double) * ctx->B.size(), cudaMemcpyHostToDevice, ctx->st);
    if (ctx->C == 3 && (desc->fe_type == FANSGPU_HEX8 || desc->fe_type == FANSGPU_HEX8R)) {
        // the element kernels' 72-term kinematics, small and large strain (BBAR's volumetric
        // average fills the normal rows, so it keeps the dense B)
        const std::vector<double> bb = fe::gauss_basic_B(desc->fe_type, ctx->le);
        if ((rc = dalloc(ctx, &ctx->Bb_d, bb.size())))
            return bail(rc);
        cudaMemcpyAsync(ctx->Bb_d, bb.data(), sizeof(double) * bb.size(), cudaMemcpyHostToDevice, ctx->st);
        cudaStreamSynchronize(ctx->st); // bb is a host temporary
    }
    // trig tables for the Green's operator (solver.h:156-158)
    {
        std::vector<double> t;
        const double        tpi = 2.0 * std::acos(-1.0);
        auto                add = [&](int nn_, int count, bool sn) {
            for (int k = 0; k < count; ++k)
                t.push_back(sn ? std::sin(tpi * k / nn_) : std::cos(tpi * k / nn_));
        };
        add(ctx->g.nx, ctx->g.nx, false);
        add(ctx->g.nx, ctx->g.nx, true);
        add(ctx->g.ny, ctx->g.ny, false);
        add(ctx->g.ny, ctx->g.ny, true);
        add(ctx->g.nz, nzh, false);
        add(ctx->g.nz, nzh, true);
        cudaMemcpyAsync(ctx->trig, t.data(), sizeof(double) * t.size(), cudaMemcpyHostToDevice, ctx->st);
        std::vector<cplx<double>> tw;
        make_twiddles<double>(ctx->g, tw);
        if ((rc = dalloc(ctx, &ctx->tw64, tw.size())))
            return bail(rc);
        cudaMemcpyAsync(ctx->tw64, tw.data(), sizeof(cplx<double>) * tw.size(), cudaMemcpyHostToDevice, ctx->st);
        if (mixed) {
            std::vector<cplx<float>> tw32;
            make_twiddles<float>(ctx->g, tw32);
            if ((rc = dalloc(ctx, &ctx->tw32, tw32.size())))
                return bail(rc);
            cudaMemcpyAsync(ctx->tw32, tw32.data(), sizeof(cplx<float>) * tw32.size(), cudaMemcpyHostToDevice, ctx->st);
        }
        if (cudaStreamSynchronize(ctx->st) != cudaSuccess) {
            fail(ctx, FANSGPU_ECUDA, "initialisation failed: %s", cudaGetErrorString(cudaGetLastError()));
            return bail(FANSGPU_ECUDA);
        }
    }
    if ((rc = make_plan<double>(ctx, ctx->cp64, ctx->spec64, ctx->tw64, ctx->G64)))
        return bail(rc);
    if (mixed && (rc = make_plan<float>(ctx, ctx->cp32, ctx->spec32, ctx->tw32, ctx->G32)))
        return bail(rc);
    if (mixed && ctx->cp32.use_reg && make_x_tma_maps(ctx->cp32, &ctx->tmaps))
        ctx->cp32.tma = &ctx->tmaps;
    if (mixed && ctx->cp32.use_reg) // the FP32 <r, s> from the spectra (FANSGPU_SPECTRAL_DOT=0: from r and s)
        ctx->cp32.spectral_dot = ctx->spectral_dot ? 1 : 0;
    *out = ctx;
    return 0;
}

int fansgpu_destroy(fansgpu_ctx *ctx)
{
    if (!ctx)
        return 0;
    if (ctx->st)
        cudaStreamSynchronize(ctx->st);
    void *ptrs[] = {ctx->d_ms, ctx->u0,   ctx->r0,     ctx->s,      ctx->dd[0],  ctx->dd[1],      ctx->Kd,
                    ctx->up0,  ctx->act,  ctx->ctlr,   ctx->Wtb,    ctx->coef_tb, ctx->coef_tx, ctx->r32, ctx->s32,   ctx->d32[0], ctx->d32[1], ctx->Kd32, ctx->e32, ctx->Kdf, ctx->fdf,       ctx->K64,
                    ctx->f64,  ctx->fnode, ctx->Cph,  ctx->Bbar_d, ctx->g0_d,  ctx->K0c,    ctx->K32,        ctx->G64,
                    ctx->G32,  ctx->spec64, ctx->tw64, ctx->spec32, ctx->tw32,  ctx->trig,       ctx->staging,
                    ctx->scal, ctx->red.partials, ctx->red.counter, ctx->red_out, ctx->max_id, ctx->Bgp_d, ctx->Bb_d,
                    ctx->ep_t, ctx->q_t, ctx->ep, ctx->q, ctx->rows, ctx->law_d, ctx->prm_d, ctx->Wtc, ctx->pb_t, ctx->pb,
                    ctx->vscale, ctx->zero_g0, ctx->stored_u, ctx->vyield, ctx->ctl, ctx->hist, ctx->nwt};
    for (void *p : ptrs)
        if (p)
            cudaFree(p);
    if (ctx->scal_h)
        cudaFreeHost(ctx->scal_h);
    if (ctx->act_h)
        cudaFreeHost(ctx->act_h);
    if (ctx->ctlr_h)
        cudaFreeHost(ctx->ctlr_h);
    if (ctx->ctl_h)
        cudaFreeHost(ctx->ctl_h);
    if (ctx->ev0)
        cudaEventDestroy(ctx->ev0);
    if (ctx->ev1)
        cudaEventDestroy(ctx->ev1);
    for (auto e : ctx->tpool)
        cudaEventDestroy(e);
    for (auto g : ctx->graph_exec)
        if (g)
            cudaGraphExecDestroy(g);
    for (auto g : ctx->iter_exec)
        if (g)
            cudaGraphExecDestroy(g);
    if (ctx->st)
        cudaStreamDestroy(ctx->st);
    delete ctx;
    return 0;
}

int fansgpu_set_microstructure(fansgpu_ctx *ctx, const uint16_t *ms)
{
    if (!ctx || !ms)
        return ctx ? fail(ctx, FANSGPU_EINVAL, "null microstructure") : FANSGPU_EINVAL;
    // upload as uint16 into the staging buffer, narrow to uint8 on the device
    uint16_t *ms16 = reinterpret_cast<uint16_t *>(ctx->staging);
    FANS_CUDA_CHECK(cudaMemcpyAsync(ms16, ms, sizeof(uint16_t) * ctx->N, cudaMemcpyHostToDevice, ctx->st));
    FANS_CUDA_CHECK(cudaMemsetAsync(ctx->max_id, 0, sizeof(unsigned int), ctx->st));
    FANS_CUDA_CHECK(launch_ms_convert(ms16, ctx->d_ms, ctx->N, ctx->max_id, ctx->st));
    unsigned int mx = 0;
    FANS_CUDA_CHECK(cudaMemcpyAsync(&mx, ctx->max_id, sizeof(unsigned int), cudaMemcpyDeviceToHost, ctx->st));
    FANS_CUDA_CHECK(cudaStreamSynchronize(ctx->st));
    if (mx > 255) {
        ctx->have_ms = false;
        return fail(ctx, FANSGPU_EUNSUPPORTED, "phase id %u > 255: at most 256 phase ids in this build", mx);
    }
    ctx->ms_max       = (int)mx;
    ctx->have_ms      = true;
    ctx->tables_dirty = true;
    return 0;
}

int fansgpu_reset(fansgpu_ctx *ctx)
{
    if (!ctx)
        return FANSGPU_EINVAL;
    const size_t nr = sizeof(double) * ctx->n * ctx->nrhs; // every right-hand side
    FANS_CUDA_CHECK(cudaMemsetAsync(ctx->u0, 0, nr, ctx->st));
    FANS_CUDA_CHECK(cudaMemsetAsync(ctx->up0, 0, nr, ctx->st));
    FANS_CUDA_CHECK(cudaMemsetAsync(ctx->r0, 0, nr, ctx->st));
    for (int k = 0; k < ctx->nrhs; ++k) {
        ctx->rhs_err[k].clear();
        ctx->rhs_iter[k]  = 0;
        ctx->rhs_ref[k]   = 0;
        ctx->rhs_uzero[k] = 1;
    }
    if (ctx->ep_t) {
        const long long nep = 6LL * ctx->ngp * ctx->N, nq = (long long)ctx->ngp * ctx->N;
        FANS_CUDA_CHECK(cudaMemsetAsync(ctx->ep_t, 0, sizeof(double) * nep, ctx->st));
        FANS_CUDA_CHECK(cudaMemsetAsync(ctx->ep, 0, sizeof(double) * nep, ctx->st));
        FANS_CUDA_CHECK(cudaMemsetAsync(ctx->q_t, 0, sizeof(double) * nq, ctx->st));
        FANS_CUDA_CHECK(cudaMemsetAsync(ctx->q, 0, sizeof(double) * nq, ctx->st));
        if (ctx->pb_t) {
            FANS_CUDA_CHECK(cudaMemsetAsync(ctx->pb_t, 0, sizeof(double) * nep, ctx->st));
            FANS_CUDA_CHECK(cudaMemsetAsync(ctx->pb, 0, sizeof(double) * nep, ctx->st));
        }
    }
    ctx->err_all.clear();
    ctx->iter   = 0;
    ctx->u_zero = true;
    return 0;
}

int fansgpu_set_wait_limit(fansgpu_ctx *ctx, int32_t polls)
{
    if (!ctx)
        return FANSGPU_EINVAL;
    if (polls < 0)
        return fail(ctx, FANSGPU_EINVAL, "wait limit: polls >= 0 required (0 restores the default)");
    ctx->tc_wait_limit = polls;
    ctx->graphs_valid  = false; // captured operator launches carry the bound
    return 0;
}

int fansgpu_set_refresh(fansgpu_ctx *ctx, double factor)
{
    if (!ctx)
        return FANSGPU_EINVAL;
    if (!(factor > 0.0 && factor < 1.0))
        return fail(ctx, FANSGPU_EINVAL, "refresh factor must lie in (0, 1)");
    ctx->reliable_delta = factor;
    return 0;
}

int fansgpu_tuning(fansgpu_ctx *ctx, int32_t *out)
{
    if (!ctx || !out)
        return FANSGPU_EINVAL;
    int rc = setup(ctx);
    if (rc)
        return rc;
    const ConvPlan<double> &a = ctx->cp64;
    const ConvPlan<float>  &b = ctx->cp32;
    // the FP64-accurate operator: of the FP64 CG iterations, else of the mixed path's true residual
    const bool fp64_pipe = ctx->desc.precision != FANSGPU_MIXED && !(ctx->fp64_df && ctx->all_linear && !ctx->vscale);
    const int32_t v[8] = {a.var_z, a.var_y, a.var_x, b.var_z + 2 * b.fuse_zy, b.var_y, b.var_x,
                         ctx->use_tcb ? (ctx->tcb_via_tc ? 3 : 2) : ctx->use_tc ? 1 : 0, fp64_pipe ? 0 : ctx->use_tcx ? 2 : 1};
    for (int k = 0; k < 8; ++k)
        out[k] = v[k];
    return 0;
}

int fansgpu_get_stream(fansgpu_ctx *ctx, void **stream)
{
    if (!ctx || !stream)
        return FANSGPU_EINVAL;
    *stream = (void *)ctx->st;
    return 0;
}

int fansgpu_set_timing(fansgpu_ctx *ctx, int32_t on)
{
    if (!ctx)
        return FANSGPU_EINVAL;
    if (on && ctx->tpool.empty()) {
        ctx->tpool.resize(64);
        for (auto &e : ctx->tpool)
            FANS_CUDA_CHECK(cudaEventCreate(&e));
    }
    ctx->timing = on != 0;
    for (int k = 0; k < FANSGPU_K_COUNT; ++k) {
        ctx->ktime[k]  = 0.0;
        ctx->kcount[k] = 0;
    }
    ctx->spans.clear();
    ctx->tused = 0;
    return 0;
}

int fansgpu_kernel_times(fansgpu_ctx *ctx, double *ms_total, int64_t *launches, int32_t n)
{
    if (!ctx)
        return FANSGPU_EINVAL;
    for (int k = 0; k < std::min((int)n, (int)FANSGPU_K_COUNT); ++k) {
        if (ms_total)
            ms_total[k] = ctx->ktime[k];
        if (launches)
            launches[k] = ctx->kcount[k];
    }
    return 0;
}

int fansgpu_set_phase_material(fansgpu_ctx *ctx, int32_t phase, int32_t law, const double *params, int32_t n_params)
{
    if (!ctx)
        return FANSGPU_EINVAL;
    if (phase < 0 || phase > 255)
        return fail(ctx, FANSGPU_EINVAL, "MaterialManager: Invalid or duplicate phase %d", phase);
    if (law < 0 || law > 10 || !params || n_params < 1)
        return fail(ctx, FANSGPU_EINVAL, "invalid material law %d / parameters", law);
    const bool thermal = (law == FANSGPU_LAW_THERMAL_ISO || law == FANSGPU_LAW_THERMAL_TRI);
    if (thermal != (ctx->C == 1))
        return fail(ctx, FANSGPU_EINVAL, "law %d is not valid for a %s problem", law, ctx->C == 1 ? "thermal" : "mechanical");
    const bool large_law = law == FANSGPU_LAW_SVK || law == FANSGPU_LAW_NEOHOOKEAN;
    if (large_law != (ctx->nstr == 9))
        return fail(ctx, FANSGPU_EINVAL, "law %d is not valid for a %s-strain problem", law,
                    ctx->nstr == 9 ? "large" : "small");
    const int need[11] = {1, 2, 4, 9, 36, 4, 5, 7, 9, 2, 2}, most[11] = {1, 2, 4, 9, 36, 6, 7, 7, 9, 2, 2};
    if (n_params < need[law])
        return fail(ctx, FANSGPU_EINVAL, "law %d needs %d parameters, got %d", law, need[law], n_params);
    n_params = std::min(n_params, most[law]);
    for (int i = 0; i < n_params; ++i)
        if (!std::isfinite(params[i]))
            return fail(ctx, FANSGPU_EINVAL, "non-finite material parameter %d of phase %d", i, phase);
    if (phase >= (int)ctx->law.size()) {
        ctx->law.resize(phase + 1, -1);
        ctx->prm.resize(phase + 1);
        ctx->assigned.resize(phase + 1, 0);
    }
    ctx->law[phase]      = law;
    ctx->prm[phase]      = std::vector<double>(params, params + n_params);
    ctx->assigned[phase] = 1;
    ctx->tables_dirty    = true;
    return 0;
}

int fansgpu_set_reference(fansgpu_ctx *ctx, const double *kref)
{
    if (!ctx || !kref)
        return ctx ? fail(ctx, FANSGPU_EINVAL, "null reference material") : FANSGPU_EINVAL;
    const int ns = ctx->nstr;
    for (int i = 0; i < ns * ns; ++i)
        if (!std::isfinite(kref[i]))
            return fail(ctx, FANSGPU_EINVAL, "reference_material has non-finite entries");
    // LLT check as MaterialManager.h:189-192 (symmetric positive definite).  The
    // large-strain reference dP/dF at F = I is only semidefinite (rotations carry
    // no stress, LargeStrainMechModel.h:96-170), so n_str = 9 checks symmetry.
    if (ns == 9) {
        double amax = 0.0;
        for (int i = 0; i < ns * ns; ++i)
            amax = std::max(amax, std::fabs(kref[i]));
        for (int i = 0; i < ns; ++i)
            for (int j = 0; j < i; ++j)
                if (std::fabs(kref[i * ns + j] - kref[j * ns + i]) > 1e-12 * amax)
                    return fail(ctx, FANSGPU_EINVAL, "reference_material must be symmetric");
    }
    std::vector<double> L(ns * ns, 0.0);
    for (int j = 0; j < ns && ns != 9; ++j) {
        double d = kref[j * ns + j];
        for (int k = 0; k < j; ++k)
            d -= L[j * ns + k] * L[j * ns + k];
        if (!(d > 0))
            return fail(ctx, FANSGPU_EINVAL, "reference_material must be symmetric positive definite");
        L[j * ns + j] = std::sqrt(d);
        for (int i = j + 1; i < ns; ++i) {
            double s = kref[i * ns + j];
            for (int k = 0; k < j; ++k)
                s -= L[i * ns + k] * L[j * ns + k];
            L[i * ns + j] = s / L[j * ns + j];
        }
    }
    ctx->kapparef.assign(kref, kref + ns * ns);
    ctx->have_ref    = true;
    ctx->green_dirty = true;
    return 0;
}

int fansgpu_set_gradient(fansgpu_ctx *ctx, const double *g0)
{
    if (!ctx || !g0)
        return ctx ? fail(ctx, FANSGPU_EINVAL, "null gradient") : FANSGPU_EINVAL;
    for (int i = 0; i < ctx->nstr; ++i)
        if (!std::isfinite(g0[i]))
            return fail(ctx, FANSGPU_EINVAL, "non-finite macroscale loading component %d", i);
    ctx->g0.assign(g0, g0 + ctx->nstr);
    ctx->force_dirty = true;
    return 0;
}

int fansgpu_set_gradients(fansgpu_ctx *ctx, int32_t n, const double *g0)
{
    if (!ctx || !g0)
        return ctx ? fail(ctx, FANSGPU_EINVAL, "null gradients") : FANSGPU_EINVAL;
    if (n != ctx->nrhs)
        return fail(ctx, FANSGPU_EINVAL, "set_gradients: %d gradients for %d right-hand sides", n, ctx->nrhs);
    for (int i = 0; i < n * ctx->nstr; ++i)
        if (!std::isfinite(g0[i]))
            return fail(ctx, FANSGPU_EINVAL, "non-finite macroscale loading component %d of RHS %d", i % ctx->nstr,
                        i / ctx->nstr);
    store_rhs(ctx);
    for (int k = 0; k < n; ++k)
        ctx->rhs_g0[k].assign(g0 + (size_t)k * ctx->nstr, g0 + (size_t)(k + 1) * ctx->nstr);
    load_rhs(ctx, ctx->cur);
    return 0;
}

int fansgpu_select_rhs(fansgpu_ctx *ctx, int32_t k)
{
    if (!ctx)
        return FANSGPU_EINVAL;
    if (k < 0 || k >= ctx->nrhs)
        return fail(ctx, FANSGPU_EINVAL, "select_rhs: %d outside 0..%d", k, ctx->nrhs - 1);
    store_rhs(ctx);
    load_rhs(ctx, k);
    return 0;
}

int fansgpu_rhs_stats(fansgpu_ctx *ctx, int32_t k, fansgpu_stats *st)
{
    if (!ctx || !st)
        return FANSGPU_EINVAL;
    if (k < 0 || k >= ctx->nrhs)
        return fail(ctx, FANSGPU_EINVAL, "rhs_stats: %d outside 0..%d", k, ctx->nrhs - 1);
    store_rhs(ctx);
    const std::vector<double> &e = ctx->rhs_err[k];
    if (e.empty())
        return fail(ctx, FANSGPU_ESTATE, "rhs_stats: RHS %d has not been solved", k);
    const double err  = e.back();
    const double rel  = ctx->tol.type == FANSGPU_ABSOLUTE ? err : (ctx->rhs_iter[k] == 0 ? 100.0 : err / e[0]);
    st->iterations    = ctx->rhs_iter[k];
    st->converged     = rel <= ctx->tol.tolerance ? 1 : 0;
    st->err0          = e[0];
    st->err           = err;
    st->refinements   = ctx->rhs_ref[k];
    st->solve_ms      = ctx->rhs_ms;
    return 0;
}

int fansgpu_get_gradient(fansgpu_ctx *ctx, double *g0)
{
    if (!ctx || !g0)
        return FANSGPU_EINVAL;
    for (int i = 0; i < ctx->nstr; ++i)
        g0[i] = ctx->g0[i];
    return 0;
}

int fansgpu_enable_mixed_bc(fansgpu_ctx *ctx, int32_t n_e, const int32_t *idx_e, const double *strain_e, int32_t n_f,
                            const int32_t *idx_f, const double *stress_f, int32_t step)
{
    if (!ctx)
        return FANSGPU_EINVAL;
    const int ns = ctx->nstr;
    if (n_e < 0 || n_f < 0 || (n_e && (!idx_e || !strain_e)) || (n_f && (!idx_f || !stress_f)) || step < 0)
        return fail(ctx, FANSGPU_EINVAL, "mixed BC: bad arguments");
    // MixedBC::from_json checks (mixedBCs.h:69-88)
    std::vector<char> present(ns, 0);
    for (int i = 0; i < n_e; ++i) {
        if (idx_e[i] < 0 || idx_e[i] >= ns)
            return fail(ctx, FANSGPU_EINVAL, "strain index out of range");
        present[idx_e[i]] = 1;
    }
    for (int i = 0; i < n_f; ++i) {
        if (idx_f[i] < 0 || idx_f[i] >= ns)
            return fail(ctx, FANSGPU_EINVAL, "stress index out of range");
        if (present[idx_f[i]])
            return fail(ctx, FANSGPU_EINVAL, "index appears in both strain_indices and stress_indices");
        present[idx_f[i]] = 1;
    }
    for (int k = 0; k < ns; ++k)
        if (!present[k])
            return fail(ctx, FANSGPU_EINVAL, "each component must be either strain- or stress-controlled");
    if (!ctx->have_ref)
        return fail(ctx, FANSGPU_ESTATE, "set_reference must be called before enabling mixed BCs");
    // MixedBC::finalize (mixedBCs.h:30-48): M = pinv(Q_F^T C0 Q_F)
    ctx->idxE.assign(idx_e, idx_e + n_e);
    ctx->idxF.assign(idx_f, idx_f + n_f);
    ctx->PF.assign(stress_f, stress_f + n_f);
    std::vector<double> A(n_f * n_f);
    for (int a = 0; a < n_f; ++a)
        for (int b = 0; b < n_f; ++b)
            A[a * n_f + b] = ctx->kapparef[idx_f[a] * ns + idx_f[b]];
    ctx->Mmix = fe::sym_pinv(A, n_f);
    // MixedBCController::activate (mixedBCs.h:180-226)
    if (step == 0) {
        ctx->g0.assign(ns, 0.0);
        if (ns == 9) // large strain starts from F = I (mixedBCs.h:196-202)
            ctx->g0[0] = ctx->g0[4] = ctx->g0[8] = 1.0;
        ctx->g0_prev = ctx->g0;
    } else {
        if (ctx->g0_prev.size() != (size_t)ns)
            ctx->g0_prev = ctx->g0;
        std::vector<double> delta(ns);
        for (int i = 0; i < ns; ++i)
            delta[i] = ctx->g0[i] - ctx->g0_prev[i];
        ctx->g0_prev = ctx->g0;
        for (int i = 0; i < n_f; ++i)
            ctx->g0[idx_f[i]] += delta[idx_f[i]];
    }
    for (int i = 0; i < n_e; ++i)
        ctx->g0[idx_e[i]] = strain_e[i];
    ctx->force_dirty  = true;
    ctx->mixed_active = true;
    return mixed_update(ctx);
}

int fansgpu_set_voxel_field(fansgpu_ctx *ctx, int32_t field, const double *values)
{
    if (!ctx)
        return FANSGPU_EINVAL;
    if (field != FANSGPU_VOXEL_STIFFNESS_SCALE && field != FANSGPU_VOXEL_YIELD_STRESS)
        return fail(ctx, FANSGPU_EINVAL, "unknown voxel field %d", field);
    const bool yield = field == FANSGPU_VOXEL_YIELD_STRESS;
    double   *&dst   = yield ? ctx->vyield : ctx->vscale;
    if (!values) { // back to the phase table alone
        if (dst)
            cudaFree(dst);
        dst = nullptr;
        return 0;
    }
    for (long long i = 0; i < ctx->N; ++i)
        if (!(values[i] > 0.0) || !std::isfinite(values[i]))
            return fail(ctx, FANSGPU_EINVAL, "%s must be positive and finite (voxel %lld)",
                        yield ? "yield stress" : "stiffness scale", i);
    int rc;
    if ((!dst && (rc = dalloc(ctx, &dst, ctx->N))) || (rc = ensure_rows(ctx)) ||
        (!ctx->zero_g0 && (rc = dalloc(ctx, &ctx->zero_g0, 9))))
        return rc;
    FANS_CUDA_CHECK(cudaMemsetAsync(ctx->zero_g0, 0, sizeof(double) * 9, ctx->st));
    FANS_CUDA_CHECK(cudaMemcpyAsync(ctx->staging, values, sizeof(double) * ctx->N, cudaMemcpyHostToDevice, ctx->st));
    FANS_CUDA_CHECK(cudaMemcpyAsync(dst, ctx->staging, sizeof(double) * ctx->N, cudaMemcpyDeviceToDevice, ctx->st));
    FANS_CUDA_CHECK(cudaStreamSynchronize(ctx->st));
    return 0;
}

int fansgpu_store_solution(fansgpu_ctx *ctx, int32_t slot)
{
    if (!ctx)
        return FANSGPU_EINVAL;
    if (slot < 0 || slot >= 6)
        return fail(ctx, FANSGPU_EINVAL, "solution slot must be in [0, 6)");
    int rc;
    if (!ctx->stored_u && (rc = dalloc(ctx, &ctx->stored_u, 6 * ctx->n)))
        return rc;
    ctx->stored_g0.resize(6 * ctx->nstr, 0.0);
    ctx->stored_ok.resize(6, 0);
    FANS_CUDA_CHECK(cudaMemcpyAsync(ctx->stored_u + slot * ctx->n, ctx->u, sizeof(double) * ctx->n,
                                    cudaMemcpyDeviceToDevice, ctx->st));
    for (int i = 0; i < ctx->nstr; ++i)
        ctx->stored_g0[slot * ctx->nstr + i] = ctx->g0[i];
    ctx->stored_ok[slot] = 1;
    FANS_CUDA_CHECK(cudaStreamSynchronize(ctx->st));
    return 0;
}

int fansgpu_stiffness_gradient(fansgpu_ctx *ctx, int32_t n, const double *W, double *grad)
{
    if (!ctx || !W || !grad)
        return FANSGPU_EINVAL;
    if (n < 1 || n > 6 || (int)ctx->stored_ok.size() < n)
        return fail(ctx, FANSGPU_EINVAL, "stiffness gradient needs solutions stored in slots 0..n-1 (n <= 6)");
    for (int k = 0; k < n; ++k)
        if (!ctx->stored_ok[k])
            return fail(ctx, FANSGPU_EINVAL, "solution slot %d not stored", k);
    int rc = setup(ctx);
    if (rc)
        return rc;
    if (!ctx->all_linear)
        return fail(ctx, FANSGPU_EUNSUPPORTED, "stiffness gradient is defined for linear laws");
    double *g0w = nullptr;
    if ((rc = dalloc(ctx, &g0w, n * ctx->nstr + n * n)))
        return rc;
    std::vector<double> h(ctx->stored_g0.begin(), ctx->stored_g0.begin() + n * ctx->nstr);
    h.insert(h.end(), W, W + n * n);
    SensArgs a{};
    a.g    = ctx->g;
    a.C    = ctx->C;
    a.nstr = ctx->nstr;
    a.ngp  = ctx->ngp;
    a.n    = n;
    a.u    = ctx->stored_u;
    a.g0   = g0w;
    a.W    = g0w + n * ctx->nstr;
    a.ms   = ctx->d_ms;
    a.B    = ctx->Bgp_d;
    a.Cph  = ctx->Cph;
    a.grad = ctx->staging;
    cudaError_t e = cudaMemcpyAsync(g0w, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice, ctx->st);
    if (e == cudaSuccess)
        e = launch_sensitivity(a, ctx->st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(grad, ctx->staging, sizeof(double) * ctx->N, cudaMemcpyDeviceToHost, ctx->st);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(ctx->st);
    cudaFree(g0w);
    return e == cudaSuccess ? 0 : fail(ctx, FANSGPU_ECUDA, "stiffness gradient: %s", cudaGetErrorString(e));
}

// ---------------------------------------------------------------------------
// Yield-stress adjoint of a strain-controlled J2PlasticityNew load path.

// The adjoint kernel's arguments for the state of one load step.
AdjArgs adj_args(fansgpu_ctx *ctx, const double *u_n, const double *g0_n, const double *ep_in, const double *q_in)
{
    AdjArgs a{};
    a.g     = ctx->g;
    a.ngp   = ctx->ngp;
    a.u     = u_n;
    a.g0    = g0_n;
    a.ep_in = ep_in;
    a.q_in  = q_in;
    a.ms    = ctx->d_ms;
    a.B     = ctx->Bgp_d;
    a.Bb    = ctx->Bb_d;
    a.law   = ctx->law_d;
    a.Cph   = ctx->Cph;
    a.prm   = ctx->prm_d;
    a.sy    = ctx->vyield;
    a.ve    = ctx->ve;
    a.rows  = ctx->rows;
    return a;
}

// Linear CG on the consistent tangent (the flexible CG recurrences of
// solverCG.h:62-117 with the Green's operator as preconditioner): x from zero
// until the residual res = K x + f has fallen by rel_tol (L2).  With res_given
// the caller has put f in `res`; otherwise f is the adjoint load of `a`
// (ADJ_RESIDUAL at x = 0: K_n^T lambda + f_n for the yield-stress adjoint).  `a`
// carries the state the tangent is taken at; the context's s, d and Kd vectors
// are the scratch.  Stopped by n_it, it returns ENOTCONV with x as far as it got.
int tangent_cg(fansgpu_ctx *ctx, AdjArgs a, double *x, double *res, bool res_given, double rel_tol, int *iters)
{
    const long long n = ctx->n;
    int             rc;
    *iters = 0;
    FANS_CUDA_CHECK(cudaMemsetAsync(x, 0, sizeof(double) * n, ctx->st));
    FANS_CUDA_CHECK(cudaMemsetAsync(ctx->s, 0, sizeof(double) * n, ctx->st));
    FANS_CUDA_CHECK(cudaMemsetAsync(ctx->dd[0], 0, sizeof(double) * n, ctx->st));
    ctx->cur_d = 0;
    if ((rc = init_scalars(ctx)))
        return rc;
    if (!res_given) {
        a.mode = ADJ_RESIDUAL;
        a.x    = x;
        FANS_CUDA_CHECK(launch_adjoint(a, ctx->st));
        FANS_CUDA_CHECK(launch_gather(ctx->rows, res, ctx->g, ctx->C, ctx->st));
    }
    FANS_CUDA_CHECK(launch_norm<double, float>(res, n, FANSGPU_L2, ctx->scal, 1, nullptr, ctx->red, SITE_NORM,
                                               ctx->st));
    if ((rc = sync_scalars(ctx)))
        return rc;
    const double err0 = ctx->scal_h->err;
    if (!std::isfinite(err0))
        return fail(ctx, FANSGPU_ENAN, "tangent CG: non-finite load");
    double err = err0;
    while (err > rel_tol * err0 && *iters < ctx->tol.n_it) {
        ConvArgs ca{res, ctx->s, -1.0, 1, ctx->scal, ctx->red, SITE_CONV};
        FANS_CUDA_CHECK(run_conv<double>(ctx, ctx->cp64, ca));
        double *dn = ctx->dd[ctx->cur_d ^ 1];
        FANS_CUDA_CHECK(cudaMemcpyAsync(dn, ctx->dd[ctx->cur_d], sizeof(double) * n, cudaMemcpyDeviceToDevice,
                                        ctx->st));
        FANS_CUDA_CHECK(launch_direction(dn, ctx->s, n, ctx->scal, ctx->st));
        a.mode = ADJ_OPERATOR;
        a.x    = dn;
        FANS_CUDA_CHECK(launch_adjoint(a, ctx->st));
        FANS_CUDA_CHECK(launch_gather(ctx->rows, ctx->Kd, ctx->g, ctx->C, ctx->st));
        FANS_CUDA_CHECK(launch_dot(dn, ctx->Kd, n, &ctx->scal->dAd, ctx->red, SITE_DOT, ctx->st));
        FANS_CUDA_CHECK(launch_set_alpha(ctx->scal, ctx->st));
        ctx->cur_d ^= 1;
        UpdateArgs ua{n, res, ctx->Kd, x, dn, ctx->s, FANSGPU_L2, 1, ctx->scal, ctx->red, SITE_UPDATE};
        FANS_CUDA_CHECK((launch_cg_update<double, double>(ua, ctx->st)));
        if ((rc = sync_scalars(ctx)))
            return rc;
        ++*iters;
        err = ctx->scal_h->err;
        if (ctx->scal_h->converged < 0 || !std::isfinite(err))
            return fail(ctx, FANSGPU_ENAN, "tangent CG: non-finite residual at iteration %d", *iters);
    }
    if (err > rel_tol * err0)
        return fail(ctx, FANSGPU_ENOTCONV, "tangent CG: %d iterations reached at relative residual %g", *iters,
                    err / err0);
    return 0;
}

// Device buffers of one adjoint run, freed on every exit path.
struct AdjBuffers {
    double *U = nullptr, *ck = nullptr, *seg = nullptr, *mu = nullptr, *lam = nullptr, *grad = nullptr,
           *path = nullptr, *cw = nullptr, *rsave = nullptr;
    ~AdjBuffers()
    {
        for (double *p : {U, ck, seg, mu, lam, grad, path, cw, rsave})
            if (p)
                cudaFree(p);
    }
};

int fansgpu_yield_stress_adjoint(fansgpu_ctx *ctx, int32_t n_steps, const double *g0_path, int32_t every,
                                 const double *w, double rel_tol, double *stress_final, double *grad,
                                 int32_t *iterations)
{
    if (!ctx || !g0_path || !w || !grad)
        return FANSGPU_EINVAL;
    if (n_steps < 1 || every < 1)
        return fail(ctx, FANSGPU_EINVAL, "yield-stress adjoint: n_steps >= 1 and checkpoint_every >= 1 required");
    if (!(rel_tol > 0.0 && rel_tol < 1.0))
        return fail(ctx, FANSGPU_EINVAL, "yield-stress adjoint: rel_tol must lie in (0, 1)");
    int rc = setup(ctx);
    if (rc)
        return rc;
    if (ctx->C != 3 || ctx->nstr != 6)
        return fail(ctx, FANSGPU_EUNSUPPORTED, "yield-stress adjoint: small-strain mechanics only");
    if (ctx->mixed_active || ctx->vscale || ctx->desc.method == FANSGPU_FP)
        return fail(ctx, FANSGPU_EUNSUPPORTED,
                    "yield-stress adjoint: strain control with the CG or Newton solver, no stiffness scale field");
    bool any_j2 = false;
    for (int ph = 0; ph < ctx->nph; ++ph) {
        const int law = ctx->law[ph];
        if (law == FANSGPU_LAW_J2_LINEAR)
            any_j2 = true;
        else if (law != FANSGPU_LAW_ELASTIC_ISO && law != FANSGPU_LAW_ELASTIC_TRI)
            return fail(ctx, FANSGPU_EUNSUPPORTED,
                        "yield-stress adjoint: phase %d: only J2PlasticityNew and linear elastic laws", ph);
    }
    if (!any_j2 || !ctx->ep_t)
        return fail(ctx, FANSGPU_EUNSUPPORTED, "yield-stress adjoint: no J2PlasticityNew phase");
    const long long N = ctx->N, n = ctx->n, nal = 7LL * ctx->ngp * N, nep = 6LL * ctx->ngp * N;
    const int       nseg = (n_steps + every - 1) / every;
    AdjBuffers      b;
    if ((rc = dalloc(ctx, &b.U, (size_t)n_steps * n)) || (rc = dalloc(ctx, &b.ck, (size_t)nseg * nal)) ||
        (every > 1 && (rc = dalloc(ctx, &b.seg, (size_t)(every - 1) * nal))) || (rc = dalloc(ctx, &b.mu, nal)) ||
        (rc = dalloc(ctx, &b.lam, n)) || (rc = dalloc(ctx, &b.grad, N)) ||
        (rc = dalloc(ctx, &b.path, (size_t)n_steps * 6)) || (rc = dalloc(ctx, &b.cw, 6)) ||
        (rc = dalloc(ctx, &b.rsave, n)))
        return rc;
    auto alpha = [&](int m, int c, int sgi) -> double * { // committed state after step m (c <= m < c + every)
        return m == c ? b.ck + (size_t)sgi * nal : b.seg + (size_t)(m - c - 1) * nal;
    };

    // forward: the load path as runSolver drives it (main.cpp:23-42), keeping
    // every converged u_n and the committed state at every checkpoint
    FANS_CUDA_CHECK(cudaMemcpyAsync(b.ck, ctx->ep_t, sizeof(double) * nep, cudaMemcpyDeviceToDevice, ctx->st));
    FANS_CUDA_CHECK(cudaMemcpyAsync(b.ck + nep, ctx->q_t, sizeof(double) * ctx->ngp * N, cudaMemcpyDeviceToDevice,
                                    ctx->st));
    for (int k = 1; k <= n_steps; ++k) {
        if ((rc = fansgpu_set_gradient(ctx, g0_path + 6 * (k - 1))))
            return rc;
        fansgpu_stats st{};
        if ((rc = fansgpu_solve(ctx, &st)))
            return rc == FANSGPU_ENOTCONV
                       ? fail(ctx, rc, "yield-stress adjoint: load step %d did not converge (%d iterations)", k,
                              st.iterations)
                       : rc;
        if (iterations)
            iterations[k - 1] = st.iterations;
        FANS_CUDA_CHECK(cudaMemcpyAsync(b.U + (size_t)(k - 1) * n, ctx->u, sizeof(double) * n,
                                        cudaMemcpyDeviceToDevice, ctx->st));
        if (k % every == 0 && k < n_steps) {
            double *c = b.ck + (size_t)(k / every) * nal;
            FANS_CUDA_CHECK(cudaMemcpyAsync(c, ctx->ep_t, sizeof(double) * nep, cudaMemcpyDeviceToDevice, ctx->st));
            FANS_CUDA_CHECK(cudaMemcpyAsync(c + nep, ctx->q_t, sizeof(double) * ctx->ngp * N,
                                            cudaMemcpyDeviceToDevice, ctx->st));
        }
        if (k < n_steps && (rc = fansgpu_extrapolate_displacement(ctx)))
            return rc;
    }
    double sig[9];
    if ((rc = fansgpu_homogenized_stress(ctx, sig)))
        return rc;
    if (stress_final)
        for (int i = 0; i < 6; ++i)
            stress_final[i] = sig[i];
    FANS_CUDA_CHECK(cudaMemcpyAsync(b.rsave, ctx->r, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx->st));

    // reverse sweep, one checkpoint segment at a time: replay the segment's
    // committed states from its checkpoint, then run its steps backwards
    double cw[6];
    for (int i = 0; i < 6; ++i)
        cw[i] = w[i] / ((double)N * ctx->ngp);
    FANS_CUDA_CHECK(cudaMemcpyAsync(b.path, g0_path, sizeof(double) * 6 * n_steps, cudaMemcpyHostToDevice, ctx->st));
    FANS_CUDA_CHECK(cudaMemcpyAsync(b.cw, cw, sizeof(cw), cudaMemcpyHostToDevice, ctx->st));
    FANS_CUDA_CHECK(cudaMemsetAsync(b.mu, 0, sizeof(double) * nal, ctx->st));
    FANS_CUDA_CHECK(cudaMemsetAsync(b.grad, 0, sizeof(double) * N, ctx->st));
    for (int sgi = nseg - 1; sgi >= 0; --sgi) {
        const int c = sgi * every, end = std::min(c + every, (int)n_steps);
        for (int m = c + 1; m < end; ++m) {
            const double *ain = alpha(m - 1, c, sgi);
            AdjArgs       a   = adj_args(ctx, b.U + (size_t)(m - 1) * n, b.path + 6 * (m - 1), ain, ain + nep);
            double       *out = alpha(m, c, sgi);
            a.mode            = ADJ_REPLAY;
            a.ep_out          = out;
            a.q_out           = out + nep;
            FANS_CUDA_CHECK(launch_adjoint(a, ctx->st));
        }
        for (int m = end; m > c; --m) {
            const double *ain = alpha(m - 1, c, sgi);
            AdjArgs       a   = adj_args(ctx, b.U + (size_t)(m - 1) * n, b.path + 6 * (m - 1), ain, ain + nep);
            a.mu_ep           = b.mu;
            a.mu_q            = b.mu + nep;
            a.cw              = m == n_steps ? b.cw : nullptr;
            int its           = 0;
            if ((rc = tangent_cg(ctx, a, b.lam, ctx->r, false, rel_tol, &its))) {
                const std::string why = ctx->err_msg;
                return fail(ctx, rc, "yield-stress adjoint, step %d: %s", m, why.c_str());
            }
            if (iterations)
                iterations[n_steps + m - 1] = its;
            a.mode = ADJ_STEP;
            a.x    = b.lam;
            a.grad = b.grad;
            FANS_CUDA_CHECK(launch_adjoint(a, ctx->st));
        }
    }
    FANS_CUDA_CHECK(cudaMemcpyAsync(grad, b.grad, sizeof(double) * N, cudaMemcpyDeviceToHost, ctx->st));
    FANS_CUDA_CHECK(cudaMemcpyAsync(ctx->r, b.rsave, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx->st));
    FANS_CUDA_CHECK(cudaStreamSynchronize(ctx->st));
    return 0;
}

// Newton-Krylov (method FANSGPU_NEWTON, a GPU extension: FANS solves the same
// discrete equations R(u) = 0 by nonlinear CG with LineSearchSecant,
// solverCG.h:62-160).  Each outer step solves the consistent-tangent system
// K(u) du = -R(u), K taken at the current strains and the committed internal
// variables, by the Green's-preconditioned CG to a relative tolerance eta
// (Eisenstat-Walker, choice 2: eta = 0.9 (|R_k| / |R_k-1|)^2 within
// [1e-6, 0.1]), then sets u += lambda du with lambda halved (at most five times)
// while the residual norm does not fall.  Linear elastic phases use their
// stiffness; J2PlasticityNew the vector-Jacobian product of its return map
// (j2_vjp with zero seeds on the internal variables).  The outer steps are the
// solve's iterations and error history; the inner CG iterations go to *inner.
int solve_newton(fansgpu_ctx *ctx, int *inner)
{
    const long long n = ctx->n;
    int             rc;
    *inner = 0;
    if (ctx->C != 3 || ctx->nstr != 6 || ctx->mixed_active || ctx->vscale)
        return fail(ctx, FANSGPU_EUNSUPPORTED,
                    "Newton-Krylov: small-strain mechanics, strain control, no stiffness scale field");
    for (int ph = 0; ph < ctx->nph; ++ph) {
        const int law = ctx->law[ph];
        if (law != FANSGPU_LAW_J2_LINEAR && law != FANSGPU_LAW_ELASTIC_ISO && law != FANSGPU_LAW_ELASTIC_TRI)
            return fail(ctx, FANSGPU_EUNSUPPORTED,
                        "Newton-Krylov: phase %d: only J2PlasticityNew and linear elastic laws have a tangent", ph);
    }
    if (!ctx->nwt && (rc = dalloc(ctx, &ctx->nwt, 3 * (size_t)n)))
        return rc;
    if ((rc = ensure_rows(ctx)))
        return rc;
    double *res = ctx->nwt, *du = ctx->nwt + n, *u_save = ctx->nwt + 2 * n;
    auto residual_norm = [&](int first, double *out) -> int {
        int rr;
        if ((rr = run_residual64(ctx, ctx->u, ctx->r)))
            return rr;
        int en = tk_mark(ctx);
        FANS_CUDA_CHECK(launch_norm<double, float>(ctx->r, n, ctx->tol.measure, ctx->scal, first, nullptr, ctx->red,
                                                   SITE_NORM, ctx->st));
        tk_span(ctx, FANSGPU_K_NORM, en, tk_mark(ctx));
        if ((rr = sync_scalars(ctx)))
            return rr;
        *out = ctx->scal_h->err;
        return 0;
    };
    if ((rc = init_scalars(ctx)))
        return rc;
    double err = 0.0;
    if ((rc = residual_norm(1, &err)))
        return rc;
    ctx->iter = 0;
    ctx->err_all.assign(1, err);
    if (!std::isfinite(err))
        return fail(ctx, FANSGPU_ENAN, "non-finite initial residual norm");
    double err_rel = err_value(ctx, err);
    if (ctx->tol.n_it > 0 && err_rel > ctx->tol.tolerance)
        ctx->u_zero = false;
    double eta = 0.1;
    ctx->newton_stalled = false;
    while (ctx->iter < ctx->tol.n_it && err_rel > ctx->tol.tolerance) {
        // the tangent at the current u and the committed state; its right-hand side is -R(u)
        const AdjArgs a = adj_args(ctx, ctx->u, ctx->g0_d, ctx->ep_t, ctx->q_t);
        FANS_CUDA_CHECK(cudaMemcpyAsync(res, ctx->r, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx->st));
        int its = 0;
        rc      = tangent_cg(ctx, a, du, res, true, eta, &its);
        *inner += its;
        if (rc == FANSGPU_ENAN) {
            // the tangent solve broke down (e.g. a right-hand side at round-off level): no step
            // is taken, u and r stay those of the last accepted step, and the solve reports ENOTCONV
            fail(ctx, FANSGPU_ENOTCONV, "Newton-Krylov: the tangent solve broke down at step %d; u kept",
                 ctx->iter + 1);
            ctx->newton_stalled = true;
            break;
        }
        if (rc && rc != FANSGPU_ENOTCONV) // an inner solve stopped by n_it still gives a usable step
            return rc;
        FANS_CUDA_CHECK(cudaMemcpyAsync(u_save, ctx->u, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx->st));
        FANS_CUDA_CHECK(launch_axpy<double>(ctx->u, du, 1.0, n, ctx->st));
        double err_new = 0.0, lambda = 1.0;
        if ((rc = residual_norm(0, &err_new)))
            return rc;
        for (int ls = 0; ls < 5 && !(err_new < err); ++ls) { // backtracking, NaN included
            lambda *= 0.5;
            FANS_CUDA_CHECK(launch_axpy<double>(ctx->u, du, -lambda, n, ctx->st));
            if ((rc = residual_norm(0, &err_new)))
                return rc;
        }
        if (!(err_new < err)) {
            // no decrease after the last halving: put u back (and with it r and the
            // trial internal variables) and stop; the solve reports ENOTCONV
            FANS_CUDA_CHECK(cudaMemcpyAsync(ctx->u, u_save, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx->st));
            if ((rc = residual_norm(0, &err_new)))
                return rc;
            fail(ctx, FANSGPU_ENOTCONV, "Newton-Krylov: no decrease of the residual after 5 step halvings at step %d",
                 ctx->iter + 1);
            ctx->newton_stalled = true;
            break;
        }
        ctx->iter++;
        ctx->err_all.push_back(err_new);
        if (!std::isfinite(err_new))
            return fail(ctx, FANSGPU_ENAN, "non-finite residual norm at Newton step %d", ctx->iter);
        const double ratio = err_new / err;
        eta = std::min(0.1, std::max(1e-6, 0.9 * ratio * ratio));
        err     = err_new;
        err_rel = err_value(ctx, err);
    }
    return 0;
}

int fansgpu_disable_mixed_bc(fansgpu_ctx *ctx)
{
    if (!ctx)
        return FANSGPU_EINVAL;
    ctx->mixed_active = false;
    return 0;
}

int fansgpu_set_tolerance(fansgpu_ctx *ctx, const fansgpu_tol *t)
{
    if (!ctx || !t)
        return FANSGPU_EINVAL;
    if (t->measure < 0 || t->measure > 2)
        return fail(ctx, FANSGPU_EINVAL, "Unknown measure type");
    if (t->type < 0 || t->type > 1)
        return fail(ctx, FANSGPU_EINVAL, "Unknown error type");
    if (t->n_it < 0 || !(t->tolerance >= 0))
        return fail(ctx, FANSGPU_EINVAL, "n_it >= 0 and tolerance >= 0 required");
    if (t->ls_max_iter < 1 || !(t->ls_tol > 0))
        return fail(ctx, FANSGPU_EINVAL, "linesearch_parameters: max_iter >= 1 and tol > 0 required");
    ctx->tol          = *t;
    ctx->graphs_valid = false; // the update kernel's error measure is a captured argument
    return 0;
}

// Solver::solve of the selected right-hand side (solver.h:283-300).
int solve_one(fansgpu_ctx *ctx, int *refinements)
{
    int rc;
    *refinements = 0;
    if ((rc = setup(ctx))) // the force tables follow this RHS's g0
        return rc;
    if (ctx->desc.method == FANSGPU_FP)
        rc = solve_fp64(ctx);
    else if (ctx->desc.method == FANSGPU_NEWTON)
        rc = solve_newton(ctx, refinements);
    else if (!ctx->all_linear || ctx->mixed_active)
        rc = solve_cg_nl(ctx); // nonlinear laws and mixed BCs run the FP64 line-search path (solverCG.h:96)
    else if (ctx->desc.precision == FANSGPU_MIXED && !ctx->vscale && multi_rhs_path(ctx)) {
        rc = solve_cg_mixed_rhs(ctx, ctx->cur);
        if (!rc)
            *refinements = ctx->rhs_ref[ctx->cur];
    } else if (ctx->desc.precision == FANSGPU_MIXED && !ctx->vscale)
        rc = solve_cg_mixed(ctx, refinements);
    else
        rc = solve_cg64(ctx);
    if (rc)
        return rc;
    // internal variables are committed at the end of every solve (solver.h:299)
    if ((rc = commit_ivars(ctx)))
        return rc;
    ctx->u_zero = ctx->u_zero && ctx->iter == 0;
    ctx->rhs_ref[ctx->cur] = *refinements;
    store_rhs(ctx);
    return 0;
}

int fansgpu_solve(fansgpu_ctx *ctx, fansgpu_stats *stats)
{
    if (!ctx)
        return FANSGPU_EINVAL;
    int rc = setup(ctx);
    if (rc)
        return rc;
    const int R = ctx->nrhs;
    if (R > 1 && (!ctx->all_linear || ctx->mixed_active))
        return fail(ctx, FANSGPU_EUNSUPPORTED,
                    "several right-hand sides need linear laws under strain control (internal variables and mixed "
                    "boundary conditions belong to one load path)");
    FANS_CUDA_CHECK(cudaEventRecord(ctx->ev0, ctx->st));
    int refinements = 0;
    if (R == 1) {
        rc = solve_one(ctx, &refinements);
    } else if (multi_rhs_path(ctx)) {
        rc = solve_cg_mixed_rhs(ctx, -1); // every RHS in each kernel
    } else {
        const int home = ctx->cur; // one after another
        for (int k = 0; k < R && !rc; ++k) {
            store_rhs(ctx);
            load_rhs(ctx, k);
            int rf = 0;
            rc     = solve_one(ctx, &rf);
        }
        store_rhs(ctx);
        load_rhs(ctx, home);
    }
    if (rc)
        return rc;
    FANS_CUDA_CHECK(cudaEventRecord(ctx->ev1, ctx->st));
    FANS_CUDA_CHECK(cudaEventSynchronize(ctx->ev1));
    float ms = 0;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    ctx->rhs_ms = ms;
    // aggregate over the right-hand sides: the worst relative error, all converged
    store_rhs(ctx);
    bool   conv = true;
    int    iters = 0, refs = 0, worst = 0;
    double worst_rel = -1.0;
    for (int k = 0; k < R; ++k) {
        const std::vector<double> &e = ctx->rhs_err[k];
        if (e.empty())
            return fail(ctx, FANSGPU_ECUDA, "RHS %d: no error history after the solve", k);
        const double rel = ctx->tol.type == FANSGPU_ABSOLUTE ? e.back() : (ctx->rhs_iter[k] == 0 ? 100.0 : e.back() / e[0]);
        conv             = conv && rel <= ctx->tol.tolerance;
        iters            = std::max(iters, ctx->rhs_iter[k]);
        refs += ctx->rhs_ref[k];
        if (!(rel <= worst_rel)) {
            worst_rel = rel;
            worst     = k;
        }
    }
    if (stats) {
        stats->iterations  = iters;
        stats->converged   = conv ? 1 : 0;
        stats->err0        = ctx->rhs_err[worst][0];
        stats->err         = ctx->rhs_err[worst].back();
        stats->refinements = refs;
        stats->solve_ms    = ms;
    }
    return conv ? 0 : FANSGPU_ENOTCONV;
}

int fansgpu_solve_batch(fansgpu_ctx *const *ctxs, int32_t n, fansgpu_stats *stats, int32_t *rcs)
{
    if (!ctxs || n < 0)
        return fail(nullptr, FANSGPU_EINVAL, "fansgpu_solve_batch: bad arguments");
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < i; ++j)
            if (!ctxs[i] || ctxs[i] == ctxs[j])
                return fail(nullptr, FANSGPU_EINVAL, "fansgpu_solve_batch: null or repeated context");
    std::vector<int>         rc(n, 0);
    std::vector<std::thread> pool;
    const int                nt = std::min<int>(n, std::max(1u, std::thread::hardware_concurrency()) * 2);
    std::atomic<int>         next{0};
    for (int t = 0; t < nt; ++t)
        pool.emplace_back([&]() {
            for (int i = next++; i < n; i = next++) {
                const bool keep         = ctxs[i]->loop_on_device;
                ctxs[i]->loop_on_device = false;
                rc[i]                   = fansgpu_solve(ctxs[i], stats ? &stats[i] : nullptr);
                ctxs[i]->loop_on_device = keep;
            }
        });
    for (auto &th : pool)
        th.join();
    int worst = 0;
    for (int i = 0; i < n; ++i) {
        if (rcs)
            rcs[i] = rc[i];
        if (rc[i] != 0 && rc[i] != FANSGPU_ENOTCONV) {
            worst          = rc[i];
            g_create_error = "context " + std::to_string(i) + ": " + ctxs[i]->err_msg;
        }
    }
    return worst;
}

int fansgpu_homogenized_stress(fansgpu_ctx *ctx, double *out)
{
    if (!ctx || !out)
        return FANSGPU_EINVAL;
    int rc = setup(ctx);
    if (rc)
        return rc;
    double red[32];
    if ((rc = strain_stress(ctx, -1, nullptr, nullptr, red)))
        return rc;
    for (int i = 0; i < ctx->nstr; ++i)
        out[i] = red[ctx->nstr + i] / (double)ctx->N;
    return 0;
}

int fansgpu_postprocess_averages(fansgpu_ctx *ctx, double *strain_avg, double *stress_avg, double *phase_strain,
                                 double *phase_stress, int64_t *phase_count, int32_t n_phase)
{
    if (!ctx)
        return FANSGPU_EINVAL;
    int rc = setup(ctx);
    if (rc)
        return rc;
    const int ns = ctx->nstr;
    double    red[32];
    if ((rc = strain_stress(ctx, -1, nullptr, nullptr, red)))
        return rc;
    for (int i = 0; i < ns; ++i) {
        if (strain_avg)
            strain_avg[i] = red[i] / (double)ctx->N;
        if (stress_avg)
            stress_avg[i] = red[ns + i] / (double)ctx->N;
    }
    for (int ph = 0; ph < n_phase; ++ph) {
        if (ph >= ctx->nph) {
            for (int i = 0; i < ns; ++i) {
                if (phase_strain) phase_strain[ph * ns + i] = 0.0;
                if (phase_stress) phase_stress[ph * ns + i] = 0.0;
            }
            if (phase_count) phase_count[ph] = 0;
            continue;
        }
        if ((rc = strain_stress(ctx, ph, nullptr, nullptr, red)))
            return rc;
        const double cnt = red[2 * ns];
        for (int i = 0; i < ns; ++i) {
            if (phase_strain) phase_strain[ph * ns + i] = cnt > 0 ? red[i] / cnt : 0.0;
            if (phase_stress) phase_stress[ph * ns + i] = cnt > 0 ? red[ns + i] / cnt : 0.0;
        }
        if (phase_count)
            phase_count[ph] = (int64_t)cnt;
    }
    return 0;
}

int fansgpu_homogenized_tangent(fansgpu_ctx *ctx, double pert, double *out)
{
    if (!ctx || !out)
        return FANSGPU_EINVAL;
    int rc = setup(ctx);
    if (rc)
        return rc;
    const int  ns     = ctx->nstr;
    const bool linear = ctx->all_linear;
    if (!linear && !(pert != 0.0 && std::isfinite(pert)))
        return fail(ctx, FANSGPU_EINVAL, "nonlinear tangent needs a finite, non-zero perturbation");
    std::vector<double> g_save = ctx->g0, T(ns * ns), sig(ns), sig0(ns);
    if (!linear && (rc = fansgpu_homogenized_stress(ctx, sig0.data()))) // unperturbed stress (solver.h:743)
        return rc;
    // solver.h:749-750: relative error type and TOL >= 1e-6 for the rest of the run
    ctx->tol.type      = FANSGPU_RELATIVE;
    ctx->tol.tolerance = std::max(1e-6, ctx->tol.tolerance);
    for (int i = 0; i < ns; ++i) {
        // linear: unit gradients; nonlinear: g0 + pert e_i (solver.h:758-765).  Each solve
        // commits internal variables, as the reference's does.
        std::vector<double> g = linear ? std::vector<double>(ns, 0.0) : g_save;
        g[i] += linear ? 1.0 : pert;
        if ((rc = fansgpu_set_gradient(ctx, g.data())))
            return rc;
        ctx->mixed_active = false; // solver.h:769
        int rf            = 0;
        if ((rc = solve_one(ctx, &rf))) // the selected right-hand side only
            return rc;
        if ((rc = fansgpu_homogenized_stress(ctx, sig.data())))
            return rc;
        for (int k = 0; k < ns; ++k)
            T[k * ns + i] = linear ? sig[k] : (sig[k] - sig0[k]) / pert;
    }
    for (int i = 0; i < ns; ++i)
        for (int j = 0; j < ns; ++j)
            out[i * ns + j] = 0.5 * (T[i * ns + j] + T[j * ns + i]);
    return 0;
}

int fansgpu_get_field(fansgpu_ctx *ctx, int32_t which, double *host)
{
    if (!ctx || !host)
        return FANSGPU_EINVAL;
    const long long N = ctx->N;
    if (which == FANSGPU_FIELD_U || which == FANSGPU_FIELD_R || which == FANSGPU_FIELD_U_PREV) {
        const double *src = which == FANSGPU_FIELD_U ? ctx->u : which == FANSGPU_FIELD_R ? ctx->r : ctx->uprev;
        FANS_CUDA_CHECK((launch_soa_to_aos<double, double>(src, ctx->staging, N, ctx->C, ctx->st)));
        FANS_CUDA_CHECK(cudaMemcpyAsync(host, ctx->staging, sizeof(double) * N * ctx->C, cudaMemcpyDeviceToHost, ctx->st));
        FANS_CUDA_CHECK(cudaStreamSynchronize(ctx->st));
        return 0;
    }
    if (which == FANSGPU_FIELD_STRAIN || which == FANSGPU_FIELD_STRESS) {
        int rc = setup(ctx);
        if (rc)
            return rc;
        double red[32];
        if ((rc = strain_stress(ctx, -1, which == FANSGPU_FIELD_STRAIN ? ctx->staging : nullptr,
                                which == FANSGPU_FIELD_STRESS ? ctx->staging : nullptr, red)))
            return rc;
        FANS_CUDA_CHECK(cudaMemcpyAsync(host, ctx->staging, sizeof(double) * N * ctx->nstr, cudaMemcpyDeviceToHost, ctx->st));
        FANS_CUDA_CHECK(cudaStreamSynchronize(ctx->st));
        return 0;
    }
    if (which == FANSGPU_FIELD_PLASTIC_STRAIN || which == FANSGPU_FIELD_HARDENING) {
        int rc = setup(ctx);
        if (rc)
            return rc;
        if (ctx->all_linear || !ctx->ep_t)
            return fail(ctx, FANSGPU_EINVAL, "field %d: no material with internal variables", which);
        // J2PlasticityNew::postprocess (J2PlasticityNew.h:171-177): Gauss-point means of the committed state
        const bool ps = which == FANSGPU_FIELD_PLASTIC_STRAIN;
        FANS_CUDA_CHECK(launch_ivar_mean(ctx->ep_t, ctx->q_t, ctx->ngp, N, ps ? ctx->staging : nullptr,
                                         ps ? nullptr : ctx->staging, ctx->st));
        FANS_CUDA_CHECK(cudaMemcpyAsync(host, ctx->staging, sizeof(double) * N * (ps ? 6 : 1), cudaMemcpyDeviceToHost,
                                        ctx->st));
        FANS_CUDA_CHECK(cudaStreamSynchronize(ctx->st));
        return 0;
    }
    if (which == FANSGPU_FIELD_KINEMATIC || which == FANSGPU_FIELD_KINEMATIC_GP) {
        int rc = setup(ctx);
        if (rc)
            return rc;
        if (!ctx->pb_t)
            return fail(ctx, FANSGPU_EINVAL, "field %d: no J2ViscoPlastic material", which);
        const bool gpf = which == FANSGPU_FIELD_KINEMATIC_GP;
        double    *tmp = nullptr;
        if (gpf && (rc = dalloc(ctx, &tmp, N * ctx->ngp * 6)))
            return rc;
        cudaError_t e = gpf ? launch_ivar_gp(ctx->pb_t, nullptr, ctx->ngp, N, tmp, nullptr, ctx->st)
                            : launch_ivar_mean(ctx->pb_t, nullptr, ctx->ngp, N, ctx->staging, nullptr, ctx->st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(host, gpf ? tmp : ctx->staging, sizeof(double) * N * (gpf ? ctx->ngp : 1) * 6,
                                cudaMemcpyDeviceToHost, ctx->st);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(ctx->st);
        if (tmp)
            cudaFree(tmp);
        return e == cudaSuccess ? 0 : fail(ctx, FANSGPU_ECUDA, "kinematic field: %s", cudaGetErrorString(e));
    }
    if (which == FANSGPU_FIELD_PLASTIC_FLAG) {
        int rc = setup(ctx);
        if (rc)
            return rc;
        double red[32];
        if ((rc = strain_stress(ctx, -1, nullptr, nullptr, red, nullptr, nullptr, ctx->staging)))
            return rc;
        FANS_CUDA_CHECK(cudaMemcpyAsync(host, ctx->staging, sizeof(double) * N, cudaMemcpyDeviceToHost, ctx->st));
        FANS_CUDA_CHECK(cudaStreamSynchronize(ctx->st));
        return 0;
    }
    if (which >= FANSGPU_FIELD_STRAIN_GP && which <= FANSGPU_FIELD_HARDENING_GP) {
        int rc = setup(ctx);
        if (rc)
            return rc;
        const bool ivar = which >= FANSGPU_FIELD_PLASTIC_STRAIN_GP;
        if (ivar && (ctx->all_linear || !ctx->ep_t))
            return fail(ctx, FANSGPU_EINVAL, "field %d: no material with internal variables", which);
        const long long per = which == FANSGPU_FIELD_HARDENING_GP ? 1 : which == FANSGPU_FIELD_PLASTIC_STRAIN_GP ? 6 : ctx->nstr;
        const long long cnt = N * ctx->ngp * per;
        double         *tmp = nullptr; // postprocess only: a temporary of n_gp x the staging size
        if ((rc = dalloc(ctx, &tmp, cnt)))
            return rc;
        double red[32];
        if (!ivar) {
            rc = strain_stress(ctx, -1, nullptr, nullptr, red, which == FANSGPU_FIELD_STRAIN_GP ? tmp : nullptr,
                               which == FANSGPU_FIELD_STRESS_GP ? tmp : nullptr);
        } else {
            const cudaError_t e = launch_ivar_gp(ctx->ep_t, ctx->q_t, ctx->ngp, N,
                                                 which == FANSGPU_FIELD_PLASTIC_STRAIN_GP ? tmp : nullptr,
                                                 which == FANSGPU_FIELD_HARDENING_GP ? tmp : nullptr, ctx->st);
            rc = e == cudaSuccess ? 0 : fail(ctx, FANSGPU_ECUDA, "ivar gather: %s", cudaGetErrorString(e));
        }
        if (!rc) {
            const cudaError_t e1 = cudaMemcpyAsync(host, tmp, sizeof(double) * cnt, cudaMemcpyDeviceToHost, ctx->st);
            const cudaError_t e2 = cudaStreamSynchronize(ctx->st);
            if (e1 != cudaSuccess || e2 != cudaSuccess)
                rc = fail(ctx, FANSGPU_ECUDA, "field copy: %s", cudaGetErrorString(e1 != cudaSuccess ? e1 : e2));
        }
        cudaFree(tmp);
        return rc;
    }
    return fail(ctx, FANSGPU_EINVAL, "unknown field %d", which);
}

int fansgpu_set_field(fansgpu_ctx *ctx, int32_t which, const double *host)
{
    if (!ctx || !host)
        return FANSGPU_EINVAL;
    double *dst = which == FANSGPU_FIELD_U ? ctx->u : which == FANSGPU_FIELD_R ? ctx->r : which == FANSGPU_FIELD_U_PREV ? ctx->uprev : nullptr;
    if (!dst)
        return fail(ctx, FANSGPU_EINVAL, "field %d cannot be set", which);
    FANS_CUDA_CHECK(cudaMemcpyAsync(ctx->staging, host, sizeof(double) * ctx->n, cudaMemcpyHostToDevice, ctx->st));
    FANS_CUDA_CHECK((launch_aos_to_soa<double, double>(ctx->staging, dst, ctx->N, ctx->C, ctx->st)));
    if (which == FANSGPU_FIELD_U)
        ctx->u_zero = false;
    FANS_CUDA_CHECK(cudaStreamSynchronize(ctx->st));
    return 0;
}

int fansgpu_get_error_history(fansgpu_ctx *ctx, double *out, int32_t max_n, int32_t *n_out)
{
    if (!ctx)
        return FANSGPU_EINVAL;
    int n = (int)ctx->err_all.size();
    if (n_out)
        *n_out = n;
    if (out)
        for (int i = 0; i < std::min(n, (int)max_n); ++i)
            out[i] = ctx->err_all[i];
    return 0;
}

int fansgpu_extrapolate_displacement(fansgpu_ctx *ctx)
{
    if (!ctx)
        return FANSGPU_EINVAL;
    // every right-hand side (their slices are contiguous)
    FANS_CUDA_CHECK(launch_extrapolate(ctx->u0, ctx->up0, ctx->n * ctx->nrhs, ctx->st));
    ctx->u_zero = false;
    for (int k = 0; k < ctx->nrhs; ++k)
        ctx->rhs_uzero[k] = 0;
    FANS_CUDA_CHECK(cudaStreamSynchronize(ctx->st));
    return 0;
}

int fansgpu_commit_state(fansgpu_ctx *ctx)
{
    if (!ctx)
        return FANSGPU_EINVAL;
    int rc = commit_ivars(ctx);
    if (rc)
        return rc;
    FANS_CUDA_CHECK(cudaStreamSynchronize(ctx->st));
    return 0;
}

int fansgpu_residual(fansgpu_ctx *ctx, const double *u, double *r)
{
    if (!ctx || !u || !r)
        return FANSGPU_EINVAL;
    int rc = setup(ctx);
    if (rc)
        return rc;
    const long long N = ctx->N;
    FANS_CUDA_CHECK(cudaMemcpyAsync(ctx->staging, u, sizeof(double) * ctx->n, cudaMemcpyHostToDevice, ctx->st));
    FANS_CUDA_CHECK((launch_aos_to_soa<double, double>(ctx->staging, ctx->Kd, N, ctx->C, ctx->st)));
    if ((rc = run_residual64(ctx, ctx->Kd, ctx->s)))
        return rc;
    FANS_CUDA_CHECK((launch_soa_to_aos<double, double>(ctx->s, ctx->staging, N, ctx->C, ctx->st)));
    FANS_CUDA_CHECK(cudaMemcpyAsync(r, ctx->staging, sizeof(double) * ctx->n, cudaMemcpyDeviceToHost, ctx->st));
    FANS_CUDA_CHECK(cudaStreamSynchronize(ctx->st));
    return 0;
}

int fansgpu_apply_operator(fansgpu_ctx *ctx, const double *x, double *y)
{
    if (!ctx || !x || !y)
        return FANSGPU_EINVAL;
    int rc = setup(ctx);
    if (rc)
        return rc;
    const long long N = ctx->N;
    FANS_CUDA_CHECK(cudaMemcpyAsync(ctx->staging, x, sizeof(double) * ctx->n, cudaMemcpyHostToDevice, ctx->st));
    FANS_CUDA_CHECK((launch_aos_to_soa<double, double>(ctx->staging, ctx->Kd, N, ctx->C, ctx->st)));
    if ((rc = ctx->vscale ? run_operator_elem(ctx, ctx->Kd, ctx->s) : run_stencil<double>(ctx, ctx->Kd, ctx->s, false)))
        return rc;
    FANS_CUDA_CHECK((launch_soa_to_aos<double, double>(ctx->s, ctx->staging, N, ctx->C, ctx->st)));
    FANS_CUDA_CHECK(cudaMemcpyAsync(y, ctx->staging, sizeof(double) * ctx->n, cudaMemcpyDeviceToHost, ctx->st));
    FANS_CUDA_CHECK(cudaStreamSynchronize(ctx->st));
    return 0;
}

int fansgpu_convolve(fansgpu_ctx *ctx, const double *rin, double *sout)
{
    if (!ctx || !rin || !sout)
        return FANSGPU_EINVAL;
    int rc = setup(ctx);
    if (rc)
        return rc;
    const long long N = ctx->N;
    FANS_CUDA_CHECK(cudaMemcpyAsync(ctx->staging, rin, sizeof(double) * ctx->n, cudaMemcpyHostToDevice, ctx->st));
    FANS_CUDA_CHECK((launch_aos_to_soa<double, double>(ctx->staging, ctx->Kd, N, ctx->C, ctx->st)));
    ConvArgs ca{ctx->Kd, ctx->s, 1.0, 0, ctx->scal, ctx->red, SITE_CONV};
    FANS_CUDA_CHECK(launch_convolution<double>(ctx->cp64, ca, ctx->st));
    FANS_CUDA_CHECK((launch_soa_to_aos<double, double>(ctx->s, ctx->staging, N, ctx->C, ctx->st)));
    FANS_CUDA_CHECK(cudaMemcpyAsync(sout, ctx->staging, sizeof(double) * ctx->n, cudaMemcpyDeviceToHost, ctx->st));
    FANS_CUDA_CHECK(cudaStreamSynchronize(ctx->st));
    return 0;
}

int fansgpu_green_table(fansgpu_ctx *ctx, double *host)
{
    if (!ctx || !host)
        return FANSGPU_EINVAL;
    int rc = setup(ctx);
    if (rc)
        return rc;
    const long long F = (long long)ctx->g.nx * ctx->g.ny * (ctx->g.nz / 2 + 1);
    const int       NT = ctx->C * (ctx->C + 1) / 2;
    FANS_CUDA_CHECK(cudaMemcpyAsync(host, ctx->G64, sizeof(double) * F * NT, cudaMemcpyDeviceToHost, ctx->st));
    FANS_CUDA_CHECK(cudaStreamSynchronize(ctx->st));
    return 0;
}

} // extern "C"
