"""The tensor-core CG operator (tcgen05 kind::tf32, 3xTF32 split) against the
CUDA-core FP32 operator and the FP64 oracle.

Mixed-precision solves are run twice on the same context settings, once with
the tensor-core operator (the default for at most two phases, any grid) and
once with FANSGPU_STENCIL=simt, which selects the CUDA-core operator at
context creation.  The shapes include ragged tiles in every direction (the
operator's CTAs own 64 x 3 x 31 nodes) and grids whose FFT lengths have no
register plan.  Both are FP32-accurate
operators inside the same reliable-update CG, so they take the same number of
iterations (within 1) and give the same solution to the accuracy the FP64
refreshes pin (1e-9 relative on the stress average); both meet the oracle's
C_eff to 1e-6, the bar of the mixed-precision parity test."""
import os

import numpy as np
import pytest

from helpers import ELASTIC, THERMAL, gpu_context, oracle_problem, random_ms, rel

pytestmark = pytest.mark.gpu


def _solve(P, g0, simt, mode=None):
    """mode: "tcb" (the exact-basis tensor-core operator where it applies), "default" (the
    default choice: for at most two phases the per-phase operator once per RHS), "tc" (per-phase
    3xTF32 tensor-core operator) or "simt" (CUDA cores)."""
    mode = mode or ("simt" if simt else "tc")
    old = os.environ.get("FANSGPU_STENCIL")
    os.environ["FANSGPU_STENCIL"] = {"tcb": "basis", "default": ""}.get(mode, mode)
    try:
        ctx = gpu_context(P, precision="mixed")
    finally:
        if old is None:
            del os.environ["FANSGPU_STENCIL"]
        else:
            os.environ["FANSGPU_STENCIL"] = old
    ctx.set_tolerance("L2", "relative", 1e-8, 500)
    ctx.set_gradient(g0)
    ctx.set_timing(True)
    st = ctx.solve()
    out = dict(st=st, stress=ctx.homogenized_stress(), u=ctx.get_field(0), times=ctx.kernel_times())
    ctx.close()
    return out


@pytest.mark.parametrize("c,groups,shape", [(3, ELASTIC, (32, 32, 32)), (3, ELASTIC, (16, 8, 64)),
                                            (1, THERMAL, (32, 16, 32)), (3, ELASTIC, (20, 24, 32)),
                                            (3, ELASTIC, (12, 14, 18)), (3, ELASTIC, (70, 4, 66)),
                                            (1, THERMAL, (6, 10, 36))])
def test_tensor_operator_matches_cuda_core_operator(c, groups, shape):
    ms = random_ms(shape, vf=0.3, seed=21)
    P = oracle_problem(ms, c, groups, "HEX8")
    g0 = np.linspace(1.0, 0.4, P.nstr)
    a = _solve(P, g0, simt=False)
    b = _solve(P, g0, simt=True)
    assert a["st"]["converged"] and b["st"]["converged"]
    assert abs(a["st"]["iterations"] - b["st"]["iterations"]) <= 1
    assert rel(a["stress"], b["stress"]) < 1e-9
    assert rel(a["u"], b["u"]) < 1e-6
    P.set_gradient(g0)
    P.solve(measure="L2", type="relative", tol=1e-8, n_it=500)
    assert rel(a["stress"], P.homogenized_stress()) < 1e-7


@pytest.mark.parametrize("c,groups,shape", [(3, ELASTIC, (32, 32, 32)), (3, ELASTIC, (40, 16, 48)),
                                            (3, ELASTIC, (80, 40, 64)), (1, THERMAL, (24, 32, 32)),
                                            (1, THERMAL, (16, 48, 32))])
def test_basis_operator_matches_cuda_core_and_per_phase_operators(c, groups, shape):
    """The exact-basis tensor-core operator (the default where every phase is an
    isotropic law and the register FFT applies; ragged tiles in x, y and z here)
    against the CUDA-core and the per-phase 3xTF32 operators: same iterations
    (within 1), stresses to 1e-9, the oracle to 1e-7."""
    ms = random_ms(shape, vf=0.3, seed=22)
    P = oracle_problem(ms, c, groups, "HEX8")
    g0 = np.linspace(0.7, -0.3, P.nstr)
    a = _solve(P, g0, False, "tcb")
    b = _solve(P, g0, True)
    t = _solve(P, g0, False, "tc")
    d = _solve(P, g0, False, "default")
    for o in (a, b, t, d):
        assert o["st"]["converged"]
    for o in (b, t, d):
        assert abs(a["st"]["iterations"] - o["st"]["iterations"]) <= 1
        assert rel(a["stress"], o["stress"]) < 1e-9
    assert rel(a["u"], b["u"]) < 1e-6 and rel(a["u"], d["u"]) < 1e-6
    P.set_gradient(g0)
    P.solve(measure="L2", type="relative", tol=1e-8, n_it=500)
    assert rel(a["stress"], P.homogenized_stress()) < 1e-7


def test_tensor_operator_single_phase_and_hex8r():
    ms = np.zeros((16, 16, 32), dtype=np.uint16)
    ms[4:9, 3:12, 10:20] = 1
    for fe in ("HEX8R", "BBAR"):
        P = oracle_problem(ms, 3, ELASTIC, fe)
        g0 = np.array([0.3, -0.1, 0.2, 0.05, 0.0, 0.1])
        a = _solve(P, g0, simt=False)
        b = _solve(P, g0, simt=True)
        assert abs(a["st"]["iterations"] - b["st"]["iterations"]) <= 1
        assert rel(a["stress"], b["stress"]) < 1e-9


def test_tensor_operator_wait_timeout_is_reported_and_recovered():
    """Failure detection of the tensor-core pipeline without a GPU fault: with
    the pipeline-wait bound cut to two polls (fansgpu_set_wait_limit), the
    waits run out, every CTA sets its abort flag, waits for its own MMAs in
    flight, frees its tensor memory and returns; the solve reports ECUDA with
    "timed out" and the context stays usable.  With the default bound restored,
    the same context (and a fresh one) solve to the same answer as before."""
    from fans_gb300 import _lib

    ms = random_ms((32, 32, 32), vf=0.3, seed=31)
    P = oracle_problem(ms, 3, ELASTIC, "HEX8")
    g0 = np.linspace(1.0, 0.4, 6)
    ref = _solve(P, g0, simt=False)
    ctx = gpu_context(P, precision="mixed")
    ctx.set_tolerance("L2", "relative", 1e-8, 500)
    ctx.set_gradient(g0)
    assert ctx.tuning()["tensor_core"]
    ctx.set_wait_limit(2)
    with pytest.raises(_lib.FansGpuError) as ei:
        ctx.solve()
    assert ei.value.code == _lib.ECUDA and "timed out" in str(ei.value)
    ctx.set_wait_limit(0)
    ctx.reset()
    st = ctx.solve()
    assert st["converged"] and st["iterations"] == ref["st"]["iterations"]
    assert rel(ctx.homogenized_stress(), ref["stress"]) < 1e-12
    ctx.close()
    again = _solve(P, g0, simt=False)
    assert rel(again["stress"], ref["stress"]) < 1e-12
