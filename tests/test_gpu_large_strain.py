"""Large-strain mechanics <3,9> (LargeStrainMechModel.h, SaintVenantKirchhoff.h,
CompressibleNeoHookean.h) on the GPU against the oracle.

Tolerances: single residual / average evaluations 1e-12 (FP64, summation order
only).  Solves run the secant line search, whose discrete decisions can follow
round-off, so converged stresses and gradients are compared at 1e-7."""
import numpy as np
import pytest

import oracle as O
from helpers import gpu_context, oracle_problem, random_ms, rel

pytestmark = pytest.mark.gpu

SVK = [(O.LAW_SVK, [0, 1], [[62.5, 28.8462], [222.222, 166.6667]])]
NH = [(O.LAW_NEOHOOKEAN, [0, 1], [[62.5, 28.8462], [222.222, 166.6667]])]
MIXED_LAWS = [(O.LAW_NEOHOOKEAN, [0], [[62.5, 28.8462]]), (O.LAW_SVK, [1], [[222.222, 166.6667]])]


def _F(t):
    H = np.array([[0.02, 0.01, 0.0], [0.0, -0.005, 0.004], [0.003, 0.0, -0.006]])
    return (np.eye(3) + t * H).ravel()


@pytest.mark.parametrize("groups,fe", [(SVK, "HEX8"), (NH, "HEX8"), (MIXED_LAWS, "HEX8R"), (NH, "BBAR")])
def test_large_strain_residual_and_averages_match_oracle(groups, fe):
    ms = random_ms((12, 10, 8), vf=0.3, seed=21)
    P = oracle_problem(ms, 3, groups, fe, strain_type="large")
    ctx = gpu_context(P)
    assert ctx.n_str == 9
    g0 = _F(2.0)
    P.set_gradient(g0)
    ctx.set_gradient(g0)
    u = 1e-3 * np.random.default_rng(3).standard_normal(P.u.shape)
    assert rel(ctx.residual(u), P.residual(u)) < 1e-12
    ctx.set_field(0, u)
    ref = P.strain_stress(u, fields=True)
    avg = ctx.postprocess_averages(P.nphase)
    assert rel(avg["stress_average"], ref["stress_average"]) < 1e-12
    assert rel(avg["strain_average"], ref["strain_average"]) < 1e-12
    assert rel(ctx.get_field(3).reshape(-1, 9), ref["stress"]) < 1e-12
    ctx.close()


@pytest.mark.parametrize("groups,method", [(SVK, "cg"), (NH, "cg"), (MIXED_LAWS, "cg")])
def test_large_strain_load_path_matches_oracle(groups, method):
    ms = random_ms((10, 8, 8), vf=0.3, seed=22)
    P = oracle_problem(ms, 3, groups, "HEX8", strain_type="large")
    ctx = gpu_context(P, method=method)
    tol = 1e-10 if method == "cg" else 1e-8
    ctx.set_tolerance("L2", "relative", tol, 2000)
    for t in (1.0, 2.0, 3.0):
        g0 = _F(t)
        P.set_gradient(g0)
        ctx.set_gradient(g0)
        P.solve(method=method, tol=tol, n_it=2000)
        st = ctx.solve()
        assert st["converged"], st
        assert rel(ctx.homogenized_stress(), P.homogenized_stress()) < 1e-7
        P.extrapolate_displacement()
        ctx.extrapolate_displacement()
    ctx.close()


def test_large_strain_fixed_point_diverges_as_the_oracle_does():
    """SolverFP with the reference's large-strain reference stiffness (shear
    entries halved, LargeStrainMechModel.h:120-160) over-corrects and diverges;
    the GPU reports the non-finite residual at the iteration the oracle does."""
    from fans_gb300 import FansGpuError

    ms = random_ms((10, 8, 8), vf=0.3, seed=22)
    P = oracle_problem(ms, 3, MIXED_LAWS, "HEX8", strain_type="large")
    ctx = gpu_context(P, method="fp")
    ctx.set_tolerance("L2", "relative", 1e-8, 2000)
    P.set_gradient(_F(1.0))
    ctx.set_gradient(_F(1.0))
    it = P.solve(method="fp", tol=1e-8, n_it=2000)
    assert not np.isfinite(P.homogenized_stress()).all()
    with pytest.raises(FansGpuError) as e:
        ctx.solve()
    assert e.value.code == -5 and f"iteration {it}" in str(e.value)
    ctx.close()


def test_large_strain_homogeneous_known_answer():
    """One phase: u~ = 0 solves the problem and P = F S(F) everywhere."""
    K, G = 62.5, 28.8462
    ms = np.zeros((8, 8, 8), np.uint16)
    P = oracle_problem(ms, 3, [(O.LAW_SVK, [0], [[K, G]])], "HEX8", strain_type="large")
    ctx = gpu_context(P)
    F = _F(3.0).reshape(3, 3)
    ctx.set_gradient(F.ravel())
    ctx.set_tolerance("Linfinity", "absolute", 1e-10, 100)  # the residual is round-off from the start
    st = ctx.solve()
    assert st["converged"]
    lam, mu = K - 2.0 / 3.0 * G, G
    E = 0.5 * (F.T @ F - np.eye(3))
    S = lam * np.trace(E) * np.eye(3) + 2 * mu * E
    assert np.allclose(ctx.homogenized_stress(), (F @ S).ravel(), rtol=1e-12, atol=1e-12)
    ctx.close()


def test_large_strain_mixed_bc_uniaxial_stress():
    """F11 prescribed, the other eight components stress-free (uniaxial stress),
    starting from F = I (mixedBCs.h:192-201)."""
    ms = random_ms((8, 8, 8), vf=0.27, seed=23)
    P = oracle_problem(ms, 3, MIXED_LAWS, "HEX8", strain_type="large")
    ctx = gpu_context(P)
    ctx.set_tolerance("Linfinity", "absolute", 1e-10, 2000)
    idx_F = [1, 2, 3, 4, 5, 6, 7, 8]
    for step in range(2):
        F11 = 1.0 + 0.01 * (step + 1)
        P.enable_mixed_bc([0], [F11], idx_F, np.zeros(8), step)
        ctx.enable_mixed_bc([0], [F11], idx_F, np.zeros(8), step)
        P.solve(measure="Linfinity", type="absolute", tol=1e-10, n_it=2000)
        st = ctx.solve()
        assert st["converged"], st
        Pk = ctx.homogenized_stress()
        assert rel(Pk, P.homogenized_stress()) < 1e-7
        assert rel(ctx.gradient(), P.g0) < 1e-7
        assert np.abs(Pk[1:]).max() < 1e-4 * abs(Pk[0])
        g = ctx.gradient()
        assert g[0] == pytest.approx(F11) and g[4] < 1.0 and g[8] < 1.0  # lateral contraction
        P.extrapolate_displacement()
        ctx.extrapolate_displacement()
    ctx.close()


def test_neo_hookean_inverted_element_reports_non_finite():
    from fans_gb300 import FansGpuError

    ms = random_ms((6, 6, 6), vf=0.3, seed=24)
    P = oracle_problem(ms, 3, NH, "HEX8", strain_type="large")
    ctx = gpu_context(P)
    ctx.set_gradient(np.diag([-1.0, 1.0, 1.0]).ravel())
    with pytest.raises(FansGpuError) as e:
        ctx.solve()
    assert e.value.code == -5  # FANSGPU_ENAN
    ctx.close()
