/*
 * fans_gb300_solver.hpp -- header-only C++17 binding of the C ABI
 * (fans_gb300.h) with the public surface of FANS's Solver<howmany, n_str>
 * (include/solver.h:11-103): solve(), extrapolateDisplacement(),
 * get_homogenized_stress(), get_homogenized_tangent(pert_param),
 * enableMixedBC / disableMixedBC / isMixedBCActive, and the members n_x, n_y,
 * n_z, n_it, TOL, v_u, v_r, err_all, iter.
 *
 * It uses standard containers instead of Eigen and takes the Reader /
 * MaterialManager settings as plain structs, so it compiles without FANS's
 * dependencies; a FANS build wraps it in its createSolver branch
 * (include/setup.h:76-85) by filling SolverGPUConfig from its Reader and the
 * phase table from its MaterialManager.  Errors are thrown as the reference
 * throws them: FANSGPU_EINVAL as std::invalid_argument, every other failing
 * status as std::runtime_error; FANSGPU_ENOTCONV is not an error (the reference
 * stops at n_it silently).
 */
#ifndef FANS_GB300_SOLVER_HPP
#define FANS_GB300_SOLVER_HPP

#include "fans_gb300.h"

#include <array>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

namespace fansgpu {

/* The Reader fields a Solver reads (reader.cpp:62-187). */
struct SolverGPUConfig {
    int                  dims[3]       = {0, 0, 0};
    double               L[3]          = {1.0, 1.0, 1.0};
    std::string          FE_type       = "HEX8";  /* HEX8 / HEX8R / BBAR */
    std::string          method        = "cg";    /* cg / fp / newton */
    std::string          precision     = "fp64";  /* fp64 / mixed */
    std::string          strain_type   = "small"; /* small / large */
    std::string          measure       = "Linfinity"; /* error_parameters.measure */
    std::string          type          = "absolute";  /* error_parameters.type */
    double               TOL           = 1e-10;
    int                  n_it          = 100;
    int                  ls_max_iter   = 5;
    double               ls_tol        = 1e-2;
    std::vector<uint16_t> ms;                         /* phase id per voxel, [x][y][z] */
};

/* One row of MaterialManager's phase table (MaterialManager.h:86-103). */
struct PhaseMaterial {
    int                 law;    /* FANSGPU_LAW_* */
    std::vector<double> params; /* see fans_gb300.h */
};

inline void throw_status(const fansgpu_ctx *ctx, int rc)
{
    const char       *m   = fansgpu_last_error(ctx);
    const std::string msg = m ? m : "fans_gb300 error";
    if (rc == FANSGPU_EINVAL)
        throw std::invalid_argument(msg);
    throw std::runtime_error(msg);
}

template <int howmany, int n_str>
class SolverGPU {
    static_assert(howmany == 1 || howmany == 3, "howmany is 1 (thermal) or 3 (mechanics)");
    static_assert((howmany == 1 && n_str == 3) || (howmany == 3 && (n_str == 6 || n_str == 9)),
                  "the template instances of main.cpp:67-75: <1,3>, <3,6>, <3,9>");

  public:
    const long n_x, n_y, n_z;
    const int  n_it;
    double     TOL;

    std::vector<double> v_u;     /* [x][y][z][howmany], refreshed after every solve() */
    std::vector<double> v_r;     /* residual, same layout */
    std::vector<double> err_all; /* absolute error history of the last solve */
    size_t              iter = 0;

    /* Solver ctor (solver.h:105-142) + createSolver (setup.h:76-85). */
    SolverGPU(const SolverGPUConfig &cfg, const std::vector<PhaseMaterial> &phases, const std::vector<double> &kapparef)
        : n_x(cfg.dims[0]), n_y(cfg.dims[1]), n_z(cfg.dims[2]), n_it(cfg.n_it), TOL(cfg.TOL)
    {
        fansgpu_desc d{};
        for (int i = 0; i < 3; ++i) {
            d.n[i] = cfg.dims[i];
            d.L[i] = cfg.L[i];
        }
        d.howmany     = howmany;
        d.fe_type     = pick(cfg.FE_type, {"HEX8", "HEX8R", "BBAR"}, "FE_type");
        d.precision   = pick(cfg.precision, {"fp64", "mixed"}, "precision");
        d.method      = pick(cfg.method, {"cg", "fp", "newton"}, "method");
        d.strain_type = n_str == 9 ? FANSGPU_LARGE_STRAIN : FANSGPU_SMALL_STRAIN;
        const fansgpu_tol t{pick(cfg.measure, {"L1", "L2", "Linfinity"}, "measure"),
                            pick(cfg.type, {"absolute", "relative"}, "type"), cfg.TOL, cfg.n_it, cfg.ls_max_iter,
                            cfg.ls_tol};
        const size_t nvox = (size_t)n_x * n_y * n_z;
        if (cfg.ms.size() != nvox)
            throw std::invalid_argument("microstructure size does not match dims");
        if (kapparef.size() != (size_t)n_str * n_str)
            throw std::invalid_argument("kapparef must hold n_str x n_str values");
        const int rc = fansgpu_create(&d, &ctx_);
        if (rc)
            throw_status(nullptr, rc);
        try {
            check(fansgpu_set_microstructure(ctx_, cfg.ms.data()));
            for (size_t p = 0; p < phases.size(); ++p)
                check(fansgpu_set_phase_material(ctx_, (int32_t)p, phases[p].law, phases[p].params.data(),
                                                 (int32_t)phases[p].params.size()));
            check(fansgpu_set_reference(ctx_, kapparef.data()));
            check(fansgpu_set_tolerance(ctx_, &t));
        } catch (...) {
            fansgpu_destroy(ctx_); // the destructor does not run for a half-built object
            ctx_ = nullptr;
            throw;
        }
        v_u.assign(nvox * howmany, 0.0);
        v_r.assign(nvox * howmany, 0.0);
    }
    SolverGPU(const SolverGPU &)            = delete;
    SolverGPU &operator=(const SolverGPU &) = delete;
    ~SolverGPU()
    {
        if (ctx_)
            fansgpu_destroy(ctx_);
    }

    /* MaterialManager::set_gradient (MaterialManager.h:216-221). */
    void set_gradient(const std::array<double, n_str> &g0) { check(fansgpu_set_gradient(ctx_, g0.data())); }

    /* Solver::solve (solver.h:283-300): internalSolve, then the commit of internal variables. */
    void solve()
    {
        fansgpu_stats st{};
        const int     rc = fansgpu_solve(ctx_, &st);
        if (rc != FANSGPU_OK && rc != FANSGPU_ENOTCONV)
            throw_status(ctx_, rc);
        iter = (size_t)st.iterations;
        err_all.assign((size_t)st.iterations + 1, 0.0);
        int32_t n = 0;
        check(fansgpu_get_error_history(ctx_, err_all.data(), (int32_t)err_all.size(), &n));
        err_all.resize((size_t)n);
        check(fansgpu_get_field(ctx_, FANSGPU_FIELD_U, v_u.data()));
        check(fansgpu_get_field(ctx_, FANSGPU_FIELD_R, v_r.data()));
    }

    /* Solver::extrapolateDisplacement (solver.h:303-311). */
    void extrapolateDisplacement() { check(fansgpu_extrapolate_displacement(ctx_)); }

    /* Solver::get_homogenized_stress (solver.h:708-737). */
    std::array<double, n_str> get_homogenized_stress()
    {
        std::array<double, n_str> s{};
        check(fansgpu_homogenized_stress(ctx_, s.data()));
        return s;
    }

    /* Solver::get_homogenized_tangent (solver.h:740-778): n_str x n_str, row-major. */
    std::vector<double> get_homogenized_tangent(double pert_param)
    {
        std::vector<double> C((size_t)n_str * n_str);
        check(fansgpu_homogenized_tangent(ctx_, pert_param, C.data()));
        return C;
    }

    /* Solver::enableMixedBC / disableMixedBC / isMixedBCActive (solver.h:71-82). */
    void enableMixedBC(const std::vector<int32_t> &idx_E, const std::vector<double> &strain_E,
                       const std::vector<int32_t> &idx_F, const std::vector<double> &stress_F, size_t step)
    {
        check(fansgpu_enable_mixed_bc(ctx_, (int32_t)idx_E.size(), idx_E.data(), strain_E.data(),
                                      (int32_t)idx_F.size(), idx_F.data(), stress_F.data(), (int32_t)step));
        mixed_ = true;
    }
    void disableMixedBC()
    {
        check(fansgpu_disable_mixed_bc(ctx_));
        mixed_ = false;
    }
    bool isMixedBCActive() const { return mixed_; }

    fansgpu_ctx *handle() { return ctx_; }

  private:
    fansgpu_ctx *ctx_  = nullptr;
    bool         mixed_ = false;

    void check(int rc)
    {
        if (rc)
            throw_status(ctx_, rc);
    }
    static int32_t pick(const std::string &v, std::initializer_list<const char *> names, const char *what)
    {
        int32_t i = 0;
        for (const char *n : names) {
            if (v == n)
                return i;
            ++i;
        }
        throw std::invalid_argument(std::string(what) + ": unknown value '" + v + "'");
    }
};

} // namespace fansgpu

#endif /* FANS_GB300_SOLVER_HPP */
