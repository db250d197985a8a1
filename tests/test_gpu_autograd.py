"""torch.autograd.Function front ends on the pyfans binding (fans_gb300.autograd):
gradients through loss.backward() equal the adjoint entry points and the oracle.

* EffectiveStiffness: C(s) from the unit load cases; the gradient of
  1/2 ||C - T||^2 equals fansgpu_stiffness_gradient with W = C - T and a central
  finite difference of the loss at one voxel.
* YieldPathStress: <sigma_N>(sigma_y) of a J2 path; the gradient of w . sigma
  equals the oracle's dense discrete adjoint."""
import numpy as np
import pytest

import j2_adjoint as A
import oracle as O
from helpers import ELASTIC, gpu_context, oracle_problem, random_ms, rel

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def test_effective_stiffness_backward():
    from fans_gb300.pyfans import EffectiveStiffness

    n = 8
    ms = random_ms((n, n, n), vf=0.3, seed=12)
    ctx = gpu_context(oracle_problem(ms, 3, ELASTIC, "HEX8"))
    ctx.set_tolerance("L2", "relative", 1e-12, 2000)
    rng = np.random.default_rng(1)
    s = torch.tensor(np.exp(0.3 * rng.standard_normal(ms.shape)), dtype=torch.float64, requires_grad=True)
    C = EffectiveStiffness.apply(s, ctx)
    T = C.detach() + 0.01 * C.detach().abs().max() * torch.tensor(rng.standard_normal((6, 6)))
    loss = 0.5 * ((C - T) ** 2).sum()
    loss.backward()
    ref = ctx.stiffness_gradient((C - T).detach().numpy())
    assert np.abs(s.grad.numpy() - ref).max() <= 1e-14 * np.abs(ref).max()
    v, h = (3, 4, 5), 1e-4
    Ls = []
    for sgn in (1, -1):
        s2 = s.detach().clone()
        s2[v] += sgn * h * s2[v]
        with torch.no_grad():
            Ls.append(float(0.5 * ((EffectiveStiffness.apply(s2, ctx) - T) ** 2).sum()))
    fd = (Ls[0] - Ls[1]) / (2 * h * float(s[v]))
    assert abs(fd - float(s.grad[v])) <= 1e-4 * float(s.grad.abs().max())
    ctx.close()


def test_yield_path_stress_backward_matches_oracle_adjoint():
    from fans_gb300 import Context
    from fans_gb300.pyfans import YieldPathStress

    J2P, ELP = (68.6275, 26.3158, 0.25, 2.0), (222.222, 166.667)
    ms = random_ms((4, 4, 4), vf=0.3, seed=7)
    sy = 0.25 * (1.0 + 0.3 * np.random.default_rng(2).random(ms.shape))
    path = np.array([[0.002 * k, 0.0005 * k, 0, 0.0007 * k, 0, 0] for k in (1, 2, 3)])
    w = np.array([1.0, 0.3, -0.2, 0.5, 0.1, 0.0])
    Y = A.YieldPathProblem(ms, J2P, ELP, sy)
    st_o, g_o = Y.adjoint(path, w)
    ctx = Context(ms.shape, (1.0, 1.0, 1.0), 3, "HEX8", "fp64", "cg")
    ctx.set_microstructure(ms)
    ctx.set_phase_material(0, O.LAW_J2, list(J2P))
    ctx.set_phase_material(1, O.LAW_ELASTIC_ISO, list(ELP))
    ctx.set_reference(Y.kapparef)
    ctx.set_tolerance("L2", "absolute", 1e-12, 5000)
    t = torch.tensor(sy, requires_grad=True)
    sig = YieldPathStress.apply(t, ctx, path, 2, 1e-12)
    assert rel(sig.detach().numpy(), st_o) < 1e-9
    (sig * torch.tensor(w)).sum().backward()
    assert np.abs(t.grad.numpy() - g_o).max() <= 1e-7 * np.abs(g_o).max()
    ctx.close()
