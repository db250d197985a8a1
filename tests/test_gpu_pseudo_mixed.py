"""PseudoPlastic laws (PseudoPlastic.h) and mixed stress/strain boundary
conditions (mixedBCs.h, solverCG.h:96-160) on the GPU against the oracle.

Tolerances: single residual / average evaluations 1e-12 (FP64, summation order
only).  Solves: the secant line search makes discrete decisions on values that
differ by round-off, so iterates may differ while both converge; converged
stresses and macroscopic strains agree to 1e-7, and the stress-controlled
components meet their targets to the solver tolerance scale."""
import numpy as np
import pytest

import oracle as O
from helpers import gpu_context, oracle_problem, random_ms, rel

pytestmark = pytest.mark.gpu

PS_LIN = [(O.LAW_PSEUDO_LIN, [0], [[62.5, 28.8462, 0.1, 0.5]]), (O.LAW_ELASTIC_ISO, [1], [[222.222, 166.6667]])]
PS_NL = [(O.LAW_PSEUDO_NL, [0], [[62.5, 28.8462, 0.1, 0.2, 0.001]]), (O.LAW_ELASTIC_ISO, [1], [[222.222, 166.6667]])]


def _ctx(P, method="cg"):
    ctx = gpu_context(P, method=method)
    return ctx


@pytest.mark.parametrize("groups", [PS_LIN, PS_NL])
def test_pseudo_plastic_residual_matches_oracle(groups):
    ms = random_ms((12, 10, 8), vf=0.3, seed=6)
    P = oracle_problem(ms, 3, groups, "HEX8")
    ctx = _ctx(P)
    g0 = np.array([0.01, -0.002, 0.001, 0.003, 0.0, -0.002])
    P.set_gradient(g0)
    ctx.set_gradient(g0)
    u = 1e-3 * np.random.default_rng(2).standard_normal(P.u.shape)
    assert rel(ctx.residual(u), P.residual(u)) < 1e-12
    ctx.set_field(0, u)
    assert rel(ctx.homogenized_stress(), P.strain_stress(u)["stress_average"]) < 1e-12
    ctx.close()


@pytest.mark.parametrize("groups", [PS_LIN, PS_NL])
def test_pseudo_plastic_load_path_matches_oracle(groups):
    ms = random_ms((10, 8, 8), vf=0.3, seed=7)
    P = oracle_problem(ms, 3, groups, "HEX8")
    ctx = _ctx(P)
    ctx.set_tolerance("L2", "relative", 1e-10, 300)
    for k in (1, 2, 3):
        g0 = np.array([0.002 * k, 0, 0, 0.0005 * k, 0, 0])
        P.set_gradient(g0)
        ctx.set_gradient(g0)
        P.solve(tol=1e-10, n_it=300)
        st = ctx.solve()
        assert st["converged"]
        assert rel(ctx.homogenized_stress(), P.homogenized_stress()) < 1e-7
    # plastic_flag: Gauss-point mean of mat_index / n_mat + mat_index (PseudoPlastic.h:103-108)
    flag = ctx.get_field(11).reshape(-1)
    eps = ctx.get_field(7).reshape(-1, 8, 6)
    law, prm = groups[0][0], groups[0][2][0]
    G, sy = prm[1], prm[2]
    tr = eps[..., :3].sum(axis=-1, keepdims=True)
    dev = np.concatenate([eps[..., :3] - tr / 3.0, eps[..., 3:]], axis=-1)
    nrm = np.linalg.norm(dev, axis=-1)
    if law == O.LAW_PSEUDO_LIN:
        plastic = nrm > np.sqrt(2 / 3) * sy / (2 * G)
    else:
        n, e0 = prm[3], prm[4]
        plastic = np.sqrt(2 / 3) * nrm > e0 * (sy / (3 * G * e0)) ** (1 / (1 - n))
    matrix = (P.ms.reshape(-1) == 0)
    # matrix (group index 0 of a one-phase group): 0 elastic, 1 plastic; elastic inclusions keep 0
    expect = np.where(matrix[:, None], np.where(plastic, 1.0, 0.0), 0.0).mean(axis=1)
    assert plastic[matrix].any() and not plastic[matrix].all()
    assert np.allclose(flag, expect)
    ctx.close()


@pytest.mark.parametrize("groups,method", [(PS_LIN, "cg"), ([(O.LAW_ELASTIC_ISO, [0, 1], [[62.5, 28.8462],
                                                                                          [222.222, 166.6667]])],
                                                          "cg"),
                                           ([(O.LAW_ELASTIC_ISO, [0, 1], [[62.5, 28.8462], [222.222, 166.6667]])],
                                            "fp")])
def test_mixed_bc_path_matches_oracle(groups, method):
    ms = random_ms((10, 8, 8), vf=0.27, seed=5)
    P = oracle_problem(ms, 3, groups, "HEX8")
    ctx = _ctx(P, method)
    tol = 1e-10 if method == "cg" else 1e-8
    ctx.set_tolerance("Linfinity", "absolute", tol, 3000)
    for step in range(3):
        e_vals, s_vals = [0.002 * (step + 1), 0.0, 0.0, 0.0], [0.0, 0.0]
        P.enable_mixed_bc([2, 3, 4, 5], e_vals, [0, 1], s_vals, step)
        ctx.enable_mixed_bc([2, 3, 4, 5], e_vals, [0, 1], s_vals, step)
        P.solve(method=method, measure="Linfinity", type="absolute", tol=tol, n_it=3000)
        st = ctx.solve()
        assert st["converged"], (step, st)
        sig = ctx.homogenized_stress()
        assert rel(sig, P.homogenized_stress()) < 1e-7
        assert rel(ctx.gradient(), P.g0) < 1e-7
        assert np.abs(sig[:2]).max() < 1e-4 * np.abs(sig).max()  # stress-controlled components ~ 0
        P.extrapolate_displacement()
        ctx.extrapolate_displacement()
    ctx.disable_mixed_bc()
    ctx.close()


def test_mixed_bc_pure_stress_control():
    """All six components stress-controlled (the second load case of the
    reference's test_MixedBCs.json): hydrostatic compression of a linear
    composite reaches the prescribed stress and a negative volumetric strain."""
    ms = random_ms((8, 8, 8), vf=0.27, seed=9)
    E = [(O.LAW_ELASTIC_ISO, [0, 1], [[62.5, 28.8462], [222.222, 166.6667]])]
    P = oracle_problem(ms, 3, E, "HEX8")
    ctx = _ctx(P)
    ctx.set_tolerance("Linfinity", "absolute", 1e-10, 2000)
    target = np.array([-0.05, -0.05, -0.05, 0.0, 0.0, 0.0])
    ctx.enable_mixed_bc([], [], list(range(6)), target, 0)
    P.enable_mixed_bc([], [], list(range(6)), target, 0)
    st = ctx.solve()
    P.solve(measure="Linfinity", type="absolute", tol=1e-10, n_it=2000)
    assert st["converged"]
    sig = ctx.homogenized_stress()
    assert np.allclose(sig, target, atol=1e-6)
    assert ctx.gradient()[:3].max() < 0
    assert rel(ctx.gradient(), P.g0) < 1e-6
    ctx.close()
