"""Yield-stress adjoint of a strain-controlled J2PlasticityNew load path on the
GPU (fansgpu_yield_stress_adjoint through the C ABI).

1. The per-voxel yield-stress field equals the oracle with one J2 phase per
   voxel, and the GPU gradient equals the oracle's dense discrete adjoint
   (complex-step Gauss-point Jacobians, lstsq tangent solves) on the same path.
   The forward path may run nonlinear CG or Newton-Krylov.
2. The checkpoint interval changes nothing: every interval recomputes the same
   committed states from its checkpoints.
3. At 16^3 the gradient equals central finite differences of the GPU forward
   path, voxel by voxel.
4. The J2 workload (128^3 spheres, 20 steps of eps_11 = 0.0005, checkpoint
   every 5 steps): zero gradient in the inclusions, and the gradient's sum (the
   derivative for a uniform shift of sigma_y) equals a central finite
   difference of two more forward paths."""
import time

import numpy as np
import pytest

import j2_adjoint as A
import oracle as O
from helpers import random_ms, rel

pytestmark = pytest.mark.gpu

J2P = (68.6275, 26.3158, 0.25, 2.0)
ELP = (222.222, 166.667)


def yield_context(ms, sy, kapparef, tol=("Linfinity", "absolute", 1e-14, 20000), method="cg"):
    from fans_gb300 import Context

    ctx = Context(ms.shape, (1.0, 1.0, 1.0), 3, "HEX8", "fp64", method)
    ctx.set_microstructure(np.asarray(ms, dtype=np.uint16))
    ctx.set_phase_material(0, O.LAW_J2, list(J2P))
    ctx.set_phase_material(1, O.LAW_ELASTIC_ISO, list(ELP))
    ctx.set_reference(kapparef)
    ctx.set_tolerance(*tol)
    ctx.set_voxel_yield_stress(sy)
    return ctx


def forward(ctx, path):
    ctx.reset()
    for k, g in enumerate(path):
        ctx.set_gradient(g)
        assert ctx.solve()["converged"], k
        if k + 1 < len(path):
            ctx.extrapolate_displacement()
    return ctx.homogenized_stress()


KREF = 0.5 * (O.iso_elastic_C(*J2P[:2]) + O.iso_elastic_C(*ELP))


@pytest.mark.parametrize("method", ["cg", "newton"])
def test_voxel_yield_field_and_adjoint_match_oracle(method):
    """The forward path by nonlinear CG or by Newton-Krylov: the same converged
    states, so the same gradient."""
    ms = random_ms((4, 4, 4), vf=0.3, seed=7)
    rng = np.random.default_rng(2)
    sy = 0.25 * (1.0 + 0.3 * rng.random(ms.shape))
    path = [np.array([0.002 * k, 0.0005 * k, 0, 0.0007 * k, 0, 0]) for k in (1, 2, 3)]
    w = np.array([1.0, 0.3, -0.2, 0.5, 0.1, 0.0])
    Y = A.YieldPathProblem(ms, J2P, ELP, sy)
    st_o, g_o = Y.adjoint(path, w)
    ctx = yield_context(ms, sy, Y.kapparef, ("L2", "absolute", 1e-12, 5000), method)
    out = ctx.yield_stress_adjoint(path, w, checkpoint_every=2, rel_tol=1e-12)
    assert rel(out["stress"], st_o) < 1e-9
    assert np.all(out["grad"][ms != 0] == 0.0)
    assert np.abs(out["grad"] - g_o).max() <= 1e-7 * np.abs(g_o).max()
    # step 1 is elastic: its committed state does not depend on the strain, so its adjoint load is zero
    assert (out["forward_iterations"] > 0).all() and out["adjoint_iterations"][-1] > 0
    ctx.close()


def test_checkpoint_interval_does_not_change_the_gradient():
    ms = random_ms((6, 6, 4), vf=0.3, seed=11)
    sy = 0.25 * (1.0 + 0.3 * np.random.default_rng(4).random(ms.shape))
    path = [np.array([0.0015 * k, 0, 0, 0, 0.0005 * k, 0]) for k in range(1, 6)]
    w = np.array([0.0, 0.0, 0.0, 0.0, 1.0, 0.0])
    ctx = yield_context(ms, sy, KREF)
    grads = []
    for every in (1, 2, 5, 8):
        ctx.reset()
        grads.append(ctx.yield_stress_adjoint(path, w, checkpoint_every=every, rel_tol=1e-12)["grad"])
    for g in grads[1:]:
        assert np.abs(g - grads[0]).max() <= 1e-14 * np.abs(grads[0]).max()
    ctx.close()


def test_adjoint_matches_gpu_finite_differences_16():
    from fans_gb300.microstructure import spheres

    ms, _ = spheres(16, 3, 0.25, 5)
    ms = ms.astype(np.uint16)
    rng = np.random.default_rng(6)
    sy = 0.25 * (1.0 + 0.2 * rng.random(ms.shape))
    path = [np.array([0.001 * k, -0.0003 * k, 0, 0.0004 * k, 0, 0]) for k in range(1, 7)]
    w = np.array([1.0, 0.0, 0.5, 0.0, 0.0, 0.2])
    ctx = yield_context(ms, sy, KREF)
    out = ctx.yield_stress_adjoint(path, w, checkpoint_every=4, rel_tol=1e-12)
    g = out["grad"]
    assert rel(forward(ctx, path), out["stress"]) < 1e-12
    # voxels with the largest gradients: far inside the plastic zone, no branch flips under +-h
    order = np.argsort(-np.abs(g).ravel())
    h = 2e-5
    for flat in order[:3].tolist() + order[200:202].tolist():
        v = np.unravel_index(flat, ms.shape)
        L = []
        for sgn in (1, -1):
            s2 = sy.copy()
            s2[v] += sgn * h
            ctx.set_voxel_yield_stress(s2)
            L.append(w @ forward(ctx, path))
        fd = (L[0] - L[1]) / (2 * h)
        assert abs(fd - g[v]) <= 2e-4 * np.abs(g).max(), (v, fd, g[v])
    ctx.close()


def test_j2_workload_128_yield_adjoint():
    from fans_gb300.microstructure import spheres

    ms, _ = spheres(128, 8, 0.25, 4)
    ms = ms.astype(np.uint16)
    sy = np.full(ms.shape, J2P[2])
    path = [np.array([0.0005 * k, 0, 0, 0, 0, 0]) for k in range(1, 21)]
    w = np.array([1.0, 0, 0, 0, 0, 0])
    tol = ("Linfinity", "absolute", 1e-12, 5000)
    ctx = yield_context(ms, sy, KREF, tol)
    t0 = time.time()
    out = ctx.yield_stress_adjoint(path, w, checkpoint_every=5, rel_tol=1e-8)
    t_adj = time.time() - t0
    g = out["grad"]
    assert np.all(g[ms != 0] == 0.0) and np.abs(g).max() > 0
    # the strain-stress curve rises and the matrix has yielded (sigma_11 below the elastic line)
    assert out["stress"][0] > 0
    D = g.sum()  # derivative for a uniform shift of sigma_y
    h = 1e-4
    L = []
    for sgn in (1, -1):
        ctx.set_voxel_yield_stress(sy + sgn * h)
        L.append(w @ forward(ctx, path))
    fd = (L[0] - L[1]) / (2 * h)
    print(f"128^3 J2 yield adjoint: forward+adjoint {t_adj:.1f} s, sigma_11 {out['stress'][0]:.6f}, "
          f"d sigma_11/d sigma_y (uniform) adjoint {D:.8f} fd {fd:.8f}, forward its "
          f"{out['forward_iterations'].tolist()}, adjoint its {out['adjoint_iterations'].tolist()}")
    assert D > 0
    assert abs(D - fd) <= 1e-3 * abs(fd)
    ctx.close()
