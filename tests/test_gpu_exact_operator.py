"""The FP64-accurate operator on the tensor cores (k_stencil_tcx): FANS's residual
R(u) = K u + F (solver.h:231-270 with phase_stiffness, solverCG.h:97-103) from
exact fixed-point tf32 slices of the element rows, exact integer basis blocks
and a double-float epilogue.  It computes the true residual of the mixed path's
reliable updates and the operator of the FP64 CG path.

* The residual of a random and of a smooth displacement field equals the FP64
  oracle's (fo_residual) to 1e-10 relative, and so does the CUDA-core
  double-float kernel it replaces (FANSGPU_EXACT=df).
* FP64 CG solves with it match the oracle (iterations +-1, stress 1e-10) and the
  same solve with the operator on the FP64 pipe (FANSGPU_FP64_OPERATOR=dfma) to
  1e-11; mixed solves take the same iterations and refreshes as with the
  CUDA-core double-float refresh, stresses to 1e-12.
* Its bounded pipeline waits expire on request (fansgpu_set_wait_limit) with
  ECUDA and the context recovers."""
import os

import numpy as np
import pytest

from helpers import ELASTIC, THERMAL, gpu_context, oracle_problem, random_ms, rel

pytestmark = pytest.mark.gpu


def _with_env(env, fn):
    old = {k: os.environ.get(k) for k in env}
    os.environ.update(env)
    try:
        return fn()
    finally:
        for k, v in old.items():
            if v is None:
                del os.environ[k]
            else:
                os.environ[k] = v


def _residual(P, u, g0, env):
    from fans_gb300 import _lib

    def run():
        ctx = gpu_context(P, precision="fp64")
        ctx.set_field(_lib.FIELD_U, u)
        ctx.set_gradient(g0)
        ctx.set_tolerance("L2", "absolute", 0.0, 0)  # n_it = 0: r = R(u) only
        ctx.solve()
        r = ctx.get_field(_lib.FIELD_R)
        ctx.close()
        return r

    return _with_env(env, run)


@pytest.mark.parametrize("c,groups,shape", [(3, ELASTIC, (32, 32, 32)), (3, ELASTIC, (40, 16, 48)),
                                            (1, THERMAL, (24, 32, 32))])
def test_exact_operator_residual_matches_oracle(c, groups, shape):
    P = oracle_problem(random_ms(shape, vf=0.3, seed=61), c, groups, "HEX8")
    rng = np.random.default_rng(62)
    g0 = np.linspace(0.5, -0.2, P.nstr)
    x = np.arange(shape[0])[:, None, None, None] / shape[0]
    smooth = np.sin(2 * np.pi * x) * np.ones(shape + (c,)) * 3.0 + 1e3  # long wave on a large offset
    for u in (rng.standard_normal(shape + (c,)), smooth):
        P.set_gradient(g0)
        ref = P.residual(u)
        for env in ({"FANSGPU_EXACT": ""}, {"FANSGPU_EXACT": "df"}):
            r = _residual(P, u, g0, env)
            assert rel(r, ref) < 1e-10, (env, rel(r, ref))


def _solve(P, g0, precision, env, tol=1e-10):
    def run():
        ctx = gpu_context(P, precision=precision)
        ctx.set_tolerance("L2", "relative", tol, 2000)
        ctx.set_gradient(g0)
        st = ctx.solve()
        out = (st, ctx.homogenized_stress())
        ctx.close()
        return out

    return _with_env(env, run)


def test_exact_operator_in_fp64_and_mixed_solves():
    P = oracle_problem(random_ms((32, 32, 32), vf=0.3, seed=63), 3, ELASTIC, "HEX8")
    g0 = np.array([1.0, -0.3, 0.2, 0.1, 0.0, 0.05])
    st, sig = _solve(P, g0, "fp64", {"FANSGPU_EXACT": "", "FANSGPU_FP64_OPERATOR": ""})
    st_f, sig_f = _solve(P, g0, "fp64", {"FANSGPU_EXACT": "", "FANSGPU_FP64_OPERATOR": "dfma"})
    P.set_gradient(g0)
    it = P.solve(measure="L2", type="relative", tol=1e-10, n_it=2000)
    assert st["converged"] and abs(st["iterations"] - it) <= 1 and abs(st_f["iterations"] - it) <= 1
    assert rel(sig, P.homogenized_stress()) < 1e-10
    assert rel(sig, sig_f) < 1e-11
    m, sig_m = _solve(P, g0, "mixed", {"FANSGPU_EXACT": ""}, 1e-8)
    d, sig_d = _solve(P, g0, "mixed", {"FANSGPU_EXACT": "df"}, 1e-8)
    assert m["iterations"] == d["iterations"] and m["refinements"] == d["refinements"]
    assert rel(sig_m, sig_d) < 1e-12


def test_exact_operator_wait_timeout_is_reported_and_recovered():
    from fans_gb300 import _lib

    P = oracle_problem(random_ms((32, 32, 32), vf=0.3, seed=64), 3, ELASTIC, "HEX8")
    g0 = np.linspace(1.0, 0.4, 6)
    ref_st, ref = _solve(P, g0, "fp64", {"FANSGPU_EXACT": ""})
    ctx = gpu_context(P, precision="fp64")
    ctx.set_tolerance("L2", "relative", 1e-10, 2000)
    ctx.set_gradient(g0)
    ctx.set_wait_limit(2)
    with pytest.raises(_lib.FansGpuError) as ei:
        ctx.solve()
    assert ei.value.code == _lib.ECUDA and "timed out" in str(ei.value)
    ctx.set_wait_limit(0)
    ctx.reset()
    st = ctx.solve()
    assert st["iterations"] == ref_st["iterations"] and rel(ctx.homogenized_stress(), ref) < 1e-12
    ctx.close()
