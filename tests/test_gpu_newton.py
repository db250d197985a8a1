"""Newton-Krylov (FANSGPU_NEWTON) on J2PlasticityNew load paths: it solves the
same discrete equations R(u) = 0 as FANS's nonlinear CG with LineSearchSecant
(solverCG.h:62-160), so both converge to the same states.

* Down-sampled J2 workload (32^3, six steps of eps_11 = 0.001): per step the
  Newton stresses agree with nonlinear CG's and with the oracle's to 1e-7 (the
  solves stop at Linfinity 1e-10 absolute, so the two solvers' states differ at
  about 2e-9); the committed plastic strains agree to 1e-6 of their maximum.
* J2 workload at 128^3 (eight steps of 0.001): Newton against nonlinear CG,
  stresses to 1e-7, both timed.
* Laws without a tangent are refused."""
import time

import numpy as np
import pytest

import oracle as O
from helpers import gpu_context, oracle_problem, random_ms, rel

pytestmark = pytest.mark.gpu

J2 = [(O.LAW_J2, [0], [[68.6275, 26.3158, 0.25, 2.0]]), (O.LAW_ELASTIC_ISO, [1], [[222.222, 166.667]])]
TOL = ("Linfinity", "absolute", 1e-10, 2000)


def _ms(n):
    from fans_gb300.microstructure import spheres

    ms, _ = spheres(128, 8, 0.25, 4)
    step = 128 // n
    return np.ascontiguousarray(ms[::step, ::step, ::step]).astype(np.uint16)


def test_newton_matches_nonlinear_cg_and_oracle():
    P = oracle_problem(_ms(32), 3, J2, "HEX8")
    cg = gpu_context(P, method="cg")
    nt = gpu_context(P, method="newton")
    for c in (cg, nt):
        c.set_tolerance(*TOL)
    for k in range(1, 7):
        g = np.zeros(6)
        g[0] = 0.001 * k
        for c in (cg, nt):
            c.set_gradient(g)
        s_cg, s_nt = cg.solve(), nt.solve()
        assert s_cg["converged"] and s_nt["converged"], (k, s_cg, s_nt)
        assert s_nt["iterations"] <= 12, s_nt
        P.set_gradient(g)
        P.solve(measure="Linfinity", type="absolute", tol=1e-10, n_it=2000)
        sig_cg, sig_nt = cg.homogenized_stress(), nt.homogenized_stress()
        assert rel(sig_nt, sig_cg) < 1e-7, k
        assert rel(sig_nt, P.homogenized_stress()) < 1e-7, k
        for c in (cg, nt):
            c.extrapolate_displacement()
        P.extrapolate_displacement()
    ep_cg = cg.get_field(5)
    ep_nt = nt.get_field(5)
    assert np.abs(ep_cg).max() > 0
    assert np.abs(ep_nt - ep_cg).max() <= 1e-6 * np.abs(ep_cg).max()
    cg.close()
    nt.close()


def test_newton_j2_workload_128():
    P = oracle_problem(_ms(128)[:4, :4, :4], 3, J2, "HEX8")
    from fans_gb300 import Context

    ms = _ms(128)
    out = {}
    for method in ("cg", "newton"):
        ctx = Context(ms.shape, (1.0, 1.0, 1.0), 3, "HEX8", "fp64", method)
        ctx.set_microstructure(ms)
        ctx.set_phase_material(0, O.LAW_J2, [68.6275, 26.3158, 0.25, 2.0])
        ctx.set_phase_material(1, O.LAW_ELASTIC_ISO, [222.222, 166.667])
        ctx.set_reference(P.kapparef)
        ctx.set_tolerance(*TOL)
        t0, curve, its = time.time(), [], []
        for k in range(1, 9):
            g = np.zeros(6)
            g[0] = 0.001 * k
            ctx.set_gradient(g)
            st = ctx.solve()
            assert st["converged"], (method, k, st)
            its.append((st["iterations"], st["refinements"]))
            curve.append(ctx.homogenized_stress())
            ctx.extrapolate_displacement()
        out[method] = (time.time() - t0, np.array(curve), its)
        ctx.close()
    assert rel(out["newton"][1], out["cg"][1]) < 1e-7
    print(f"J2 128^3, 8 steps: nonlinear CG {out['cg'][0]:.1f} s {out['cg'][2]}, "
          f"Newton-Krylov {out['newton'][0]:.1f} s (outer, inner) {out['newton'][2]}")


def test_newton_refuses_laws_without_tangent():
    from fans_gb300 import FansGpuError

    ms = random_ms((8, 8, 8), vf=0.3, seed=2)
    P = oracle_problem(ms, 3, [(O.LAW_PSEUDO_LIN, [0, 1], [[68.6, 26.3, 0.25, 2.0], [68.6, 26.3, 0.3, 2.0]])],
                       "HEX8")
    ctx = gpu_context(P, method="newton")
    ctx.set_gradient(np.array([0.001, 0, 0, 0, 0, 0]))
    with pytest.raises(FansGpuError, match="tangent"):
        ctx.solve()
    ctx.close()


def test_newton_stall_restores_u_and_reports_not_converged():
    """A Newton step that does not lower the residual after five halvings is
    undone: u (and with it r and the trial internal variables) goes back to the
    state before the step and the solve stops with ENOTCONV instead of running
    to n_it; so does a step whose tangent solve breaks down.  Forced by asking
    for an absolute Linfinity tolerance of 0 from a state already converged to
    round-off, where no step can keep lowering the residual."""
    from fans_gb300 import _lib

    P = oracle_problem(_ms(16), 3, J2, "HEX8")
    nt = gpu_context(P, method="newton")
    nt.set_tolerance("Linfinity", "absolute", 1e-12, 200)
    g = np.zeros(6)
    g[0] = 0.004
    nt.set_gradient(g)
    assert nt.solve()["converged"]
    sig0 = nt.homogenized_stress()
    nt.set_tolerance("Linfinity", "absolute", 0.0, 200)
    st = nt.solve()
    assert not st["converged"] and st["iterations"] < 200, st
    hist = nt.error_history()
    assert len(hist) == st["iterations"] + 1 and hist[-1] == st["err"] and st["err"] <= hist[0]
    msg = _lib.load().fansgpu_last_error(nt.ctx).decode()
    assert "no decrease" in msg or "broke down" in msg, msg
    # the state is the last accepted one: its residual norm is the reported error
    r = nt.get_field(_lib.FIELD_R)
    assert np.abs(r).max() == pytest.approx(st["err"], rel=1e-12, abs=0)
    assert rel(nt.homogenized_stress(), sig0) < 1e-9
    nt.close()
