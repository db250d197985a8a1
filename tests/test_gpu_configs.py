"""The thermal 32^3 and elastic 128^3 workloads at their stated sizes, GPU
against the FP64 oracle (FANS's SolverCG, solverCG.h:62-117, restated in C).

* Thermal 32^3: spheres seed 0, r = 4, vf 0.20; conductivities 1 and 10; load
  cases e1, e2, e3; CG, L2 relative 1e-10, FP64.  kappa_eff within 1e-10,
  iterations within +-1, per-voxel flux within 1e-8.
* Elastic 128^3: spheres seed 1, r = 6, vf 0.30; E/nu 3/0.35 and 70/0.22; six
  unit Mandel load cases; CG, L2 relative 1e-8.  FP64 C_eff within 1e-10 and
  iterations within +-1; mixed-precision C_eff within 1e-6."""
import numpy as np
import pytest

import oracle as O
from helpers import ELASTIC, THERMAL, gpu_context, oracle_problem, rel

pytestmark = pytest.mark.gpu


def effective(ctx, P, nstr, tol, check_fields=False):
    K_gpu, K_ref = np.zeros((nstr, nstr)), np.zeros((nstr, nstr))
    for i in range(nstr):
        g = np.zeros(nstr)
        g[i] = 1.0
        ctx.reset()
        ctx.set_gradient(g)
        st = ctx.solve()
        assert st["converged"], i
        K_gpu[:, i] = ctx.homogenized_stress()
        if P is None:
            continue
        P.u[...] = 0.0
        P.set_gradient(g)
        it = P.solve(measure="L2", type="relative", tol=tol, n_it=2000)
        K_ref[:, i] = P.homogenized_stress()
        assert abs(st["iterations"] - it) <= 1, (i, st["iterations"], it)
        if check_fields:
            flux = ctx.get_field(3).reshape(-1, nstr)
            ref = P.strain_stress(fields=True)["stress"]
            assert rel(flux, ref) < 1e-8
    return K_gpu, K_ref


def test_thermal_32_fp64_matches_oracle():
    from fans_gb300.microstructure import spheres

    ms, _ = spheres(32, 4, 0.20, 0)
    P = oracle_problem(ms.astype(np.uint16), 1, THERMAL, "HEX8")
    ctx = gpu_context(P, precision="fp64")
    ctx.set_tolerance("L2", "relative", 1e-10, 2000)
    K_gpu, K_ref = effective(ctx, P, 3, 1e-10, check_fields=True)
    assert rel(K_gpu, K_ref) < 1e-10
    ctx.close()


def test_elastic_128_fp64_and_mixed_match_oracle():
    from fans_gb300.microstructure import spheres

    ms, _ = spheres(128, 6, 0.30, 1)
    P = oracle_problem(ms.astype(np.uint16), 3, ELASTIC, "HEX8")
    ctx = gpu_context(P, precision="fp64")
    ctx.set_tolerance("L2", "relative", 1e-8, 2000)
    C64, C_ref = effective(ctx, P, 6, 1e-8)
    ctx.close()
    assert rel(C64, C_ref) < 1e-10
    mix = gpu_context(P, precision="mixed")
    mix.set_tolerance("L2", "relative", 1e-8, 2000)
    C_mix, _ = effective(mix, None, 6, 1e-8)
    mix.close()
    C_mix, C_ref = 0.5 * (C_mix + C_mix.T), 0.5 * (C_ref + C_ref.T)
    assert np.linalg.norm(C_mix - C_ref) / np.linalg.norm(C_ref) < 1e-6
    print(f"elastic 128^3: |C_fp64 - C_oracle| {rel(C64, C_ref):.2e}, "
          f"|C_mixed - C_oracle| / |C_oracle| {np.linalg.norm(C_mix - C_ref) / np.linalg.norm(C_ref):.2e}")


def test_elastic_256_multi_rhs_matches_oracle_fixture():
    """The headline workload (256^3, seed 0, r 6, vf 0.30, six unit loads, rel. L2
    1e-8) as one multi-RHS mixed-precision solve: C_eff within 1e-6 of the FP64
    oracle's complete solve (tests/golden/elastic256_ceff.json, made by
    tests/golden/make_workload_fixtures.py), each load case within +-1 of the
    oracle's iteration count."""
    import json
    import os

    from fans_gb300 import Context
    from fans_gb300.microstructure import spheres

    fx = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "elastic256_ceff.json")))
    ms, _ = spheres(256, 6, 0.30, 0)
    assert abs(ms.mean() - fx["vf"]) < 1e-12
    P = oracle_problem(ms[:4, :4, :4].astype(np.uint16), 3, ELASTIC, "HEX8")  # the reference-stiffness rule only
    ctx = Context((256, 256, 256), (1.0, 1.0, 1.0), 3, "HEX8", "mixed", "cg", n_rhs=6)
    ctx.set_microstructure(ms)
    for ph in range(2):
        ctx.set_phase_material(ph, int(P.law[ph]), P.param[ph, :2])
    ctx.set_reference(P.kapparef)
    ctx.set_tolerance("L2", "relative", 1e-8, 2000)
    ctx.set_gradients(np.eye(6))
    assert ctx.solve()["converged"]
    its = [ctx.rhs_stats(k)["iterations"] for k in range(6)]
    C = ctx.homogenized_stresses().T
    ctx.close()
    Cf = np.array(fx["C_eff_columns"])
    C, Cf = 0.5 * (C + C.T), 0.5 * (Cf + Cf.T)
    err = np.linalg.norm(C - Cf) / np.linalg.norm(Cf)
    assert err < 1e-6, err
    assert all(abs(a - b) <= 1 for a, b in zip(its, fx["iterations"])), (its, fx["iterations"])
    print(f"elastic 256^3 multi-RHS: |C - C_oracle| / |C_oracle| = {err:.2e}, iterations {its}")
