"""J2ViscoPlastic (J2Plasticity.h, linear and saturation isotropic hardening
with kinematic hardening and viscosity) on the GPU against the oracle.

As in the reference, the trial hardening variables psi and psi_bar accumulate
over every law evaluation of a time step (psi += sqrt(2/3) gamma, psi_bar -=
gamma n) and are committed at the end of the solve; the nonlinear law's Newton
iteration keeps the reference's zero derivative term ((2 / 3) is integer
division in J2Plasticity.h:209).  Residual evaluations compare at 1e-12; load
paths through the secant line search at 1e-7 (stress) and 1e-6 (committed
variables), since round-off-level differences can change the line search's
discrete decisions and so the number of evaluations that feed psi."""
import numpy as np
import pytest

import oracle as O
from helpers import gpu_context, oracle_problem, random_ms, rel

pytestmark = pytest.mark.gpu

VL = [(O.LAW_J2VISCO_LIN, [0], [[62.5, 28.8462, 0.1, 0.5, 0.3, 1.0, 0.01]]),
      (O.LAW_ELASTIC_ISO, [1], [[222.222, 166.6667]])]
VN = [(O.LAW_J2VISCO_NL, [0], [[62.5, 28.8462, 0.1, 0.0, 0.2, 1.0, 0.01, 0.15, 1000.0]]),
      (O.LAW_ELASTIC_ISO, [1], [[222.222, 166.6667]])]


@pytest.mark.parametrize("groups", [VL, VN])
def test_j2visco_residual_matches_oracle(groups):
    ms = random_ms((12, 10, 8), vf=0.3, seed=6)
    P = oracle_problem(ms, 3, groups, "HEX8")
    ctx = gpu_context(P)
    g0 = np.array([0.004, -0.001, 0.0005, 0.002, 0.0, -0.001])
    P.set_gradient(g0)
    ctx.set_gradient(g0)
    u = 1e-4 * np.random.default_rng(2).standard_normal(P.u.shape)
    r_ref = P.residual(u)
    assert np.abs(P.ep).max() > 0
    assert rel(ctx.residual(u), r_ref) < 1e-12
    ctx.close()


@pytest.mark.parametrize("groups", [VL, VN])
def test_j2visco_load_path_matches_oracle(groups):
    ms = random_ms((10, 8, 8), vf=0.3, seed=7)
    P = oracle_problem(ms, 3, groups, "HEX8")
    ctx = gpu_context(P)
    ctx.set_tolerance("L2", "relative", 1e-10, 300)
    for k in (1, 2, 3):
        g0 = np.array([0.001 * k, 0, 0, 0.0003 * k, 0, 0])
        P.set_gradient(g0)
        ctx.set_gradient(g0)
        P.solve(tol=1e-10, n_it=300)
        st = ctx.solve()
        assert st["converged"]
        assert rel(ctx.homogenized_stress(), P.homogenized_stress()) < 1e-7
    ep = ctx.get_field(5).reshape(-1, 6)
    assert np.abs(P.ep_t).max() > 1e-5
    assert rel(ep, P.ep_t.mean(axis=1)) < 1e-6
    kin = ctx.get_field(12).reshape(-1, 6)
    assert rel(kin, P.pb_t.mean(axis=1)) < 1e-6
    ctx.close()
