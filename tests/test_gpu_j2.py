"""J2PlasticityNew (linear isotropic hardening) on the GPU against the oracle.

The element kernel evaluates the radial return of J2PlasticityNew.h:43-108 at
every Gauss point and writes trial internal variables; the nonlinear CG runs
LineSearchSecant (solverCG.h:120-160); every solve commits the internal
variables (solver.h:299).  The load path is strain-controlled uniaxial strain,
eps_11 = 0.004 k, k = 1..4, with the matrix yielding from step 2 on.

Tolerances: a single residual evaluation is compared at 1e-12 (FP64, only the
summation order differs).  Solves are compared through their converged results
(tolerance 1e-10 relative L2): the secant line search takes discrete decisions
(`err > ls_tol`, the `alpha_next <= 0` bisection) on values that differ by
round-off between the two implementations, so iterates can differ while both
converge to the same solution; the stress averages agree to 1e-7 relative, the
committed plastic strains to 1e-6 of their maximum.
"""
import numpy as np
import pytest

import oracle as O
from helpers import gpu_context, oracle_problem, random_ms, rel

pytestmark = pytest.mark.gpu

J2 = [(O.LAW_J2, [0], [[68.6275, 26.3158, 0.25, 2.0]]), (O.LAW_ELASTIC_ISO, [1], [[222.222, 166.667]])]


@pytest.mark.parametrize("fe", ["HEX8", "HEX8R", "BBAR"])
def test_j2_residual_matches_oracle(fe):
    ms = random_ms((12, 10, 8), vf=0.25, seed=5)
    P = oracle_problem(ms, 3, J2, fe)
    ctx = gpu_context(P)
    g0 = np.array([0.02, -0.004, 0.001, 0.003, 0.0, -0.002])  # beyond first yield in the matrix
    P.set_gradient(g0)
    ctx.set_gradient(g0)
    rng = np.random.default_rng(7)
    u = 1e-3 * rng.standard_normal(P.u.shape)
    r_ref = P.residual(u)
    assert np.abs(P.ep).max() > 0  # the trial state is plastic somewhere
    r_gpu = ctx.residual(u)
    assert rel(r_gpu, r_ref) < 1e-12
    ctx.close()


def test_j2_stress_average_matches_oracle():
    ms = random_ms((10, 12, 8), vf=0.3, seed=2)
    P = oracle_problem(ms, 3, J2, "HEX8")
    ctx = gpu_context(P)
    g0 = np.array([0.015, 0.0, 0.0, 0.0, 0.004, 0.0])
    P.set_gradient(g0)
    ctx.set_gradient(g0)
    rng = np.random.default_rng(3)
    u = 1e-3 * rng.standard_normal(P.u.shape)
    ctx.set_field(0, u)
    ref = P.strain_stress(u, fields=True)
    assert rel(ctx.homogenized_stress(), ref["stress_average"]) < 1e-12
    sig = ctx.get_field(3).reshape(-1, 6)
    assert rel(sig, ref["stress"]) < 1e-12
    avg = ctx.postprocess_averages(2)
    assert rel(avg["phase_stress"], ref["phase_stress"]) < 1e-12
    ctx.close()


@pytest.mark.parametrize("fe,method", [("HEX8", "cg"), ("HEX8R", "cg"), ("HEX8", "fp")])
def test_j2_load_path_matches_oracle(fe, method):
    ms = random_ms((12, 10, 8), vf=0.25, seed=5)
    P = oracle_problem(ms, 3, J2, fe)
    ctx = gpu_context(P, method=method)
    tol, n_it = (1e-10, 300) if method == "cg" else (1e-6, 3000)
    ctx.set_tolerance("L2", "relative", tol, n_it)
    for k in range(1, 5):
        g0 = np.zeros(6)
        g0[0] = 0.004 * k
        P.set_gradient(g0)
        ctx.set_gradient(g0)
        it = P.solve(method=method, tol=tol, n_it=n_it)
        st = ctx.solve()
        assert st["converged"], (k, st)
        # the fixed-point scheme has no line search: same iterates up to round-off
        assert abs(st["iterations"] - it) <= (max(3, it // 5) if method == "cg" else 1), (k, st["iterations"], it)
        s_ref = P.homogenized_stress()
        assert rel(ctx.homogenized_stress(), s_ref) < (1e-7 if method == "cg" else 1e-9), k
    ep = ctx.get_field(5).reshape(-1, 6)
    ep_ref = P.ep_t.mean(axis=1)
    assert np.abs(ep_ref).max() > 1e-3  # plastic flow happened
    assert rel(ep, ep_ref) < 1e-6
    q = ctx.get_field(6).reshape(-1)
    assert rel(q, P.q_t.mean(axis=1)) < 1e-6
    ctx.close()


def test_j2_reset_clears_internal_variables():
    ms = random_ms((8, 8, 8), vf=0.25, seed=1)
    P = oracle_problem(ms, 3, J2, "HEX8")
    ctx = gpu_context(P)
    ctx.set_tolerance("L2", "relative", 1e-10, 300)
    g0 = np.zeros(6)
    g0[0] = 0.012
    ctx.set_gradient(g0)
    ctx.solve()
    assert np.abs(ctx.get_field(5)).max() > 0
    ctx.reset()
    assert np.abs(ctx.get_field(5)).max() == 0
    assert np.abs(ctx.get_field(6)).max() == 0
    # same load from the virgin state reproduces the first solve
    s1 = ctx.solve()
    P.set_gradient(g0)
    P.solve(tol=1e-10, n_it=300)
    assert s1["converged"]
    assert rel(ctx.homogenized_stress(), P.homogenized_stress()) < 1e-7
    ctx.close()


def test_j2_nonlinear_tangent_is_finite_difference():
    """get_homogenized_tangent, nonlinear branch (solver.h:758-772): columns are
    (sigma(g0 + pert e_i) - sigma(g0)) / pert after each perturbed solve, then
    symmetrised; each solve commits, as in the reference."""
    ms = random_ms((8, 8, 8), vf=0.25, seed=4)
    P = oracle_problem(ms, 3, J2, "HEX8")
    ctx = gpu_context(P)
    ctx.set_tolerance("L2", "relative", 1e-10, 300)
    g0 = np.zeros(6)
    g0[0] = 0.002  # elastic range: the FD tangent equals the elastic C_eff
    ctx.set_gradient(g0)
    ctx.solve()
    T = ctx.homogenized_tangent(1e-6)
    assert np.allclose(T, T.T)
    # elastic reference: the same microstructure with the matrix kept elastic
    E = [(O.LAW_ELASTIC_ISO, [0, 1], [[68.6275, 26.3158], [222.222, 166.667]])]
    Pe = oracle_problem(ms, 3, E, "HEX8", kapparef=P.kapparef)
    Ce = Pe.homogenized_tangent_unit(tol=1e-10, n_it=300)
    assert rel(T, Ce) < 1e-4
    ctx.close()
