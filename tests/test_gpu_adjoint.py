"""Per-voxel stiffness field and the stiffness sensitivity (adjoint) on the GPU.

E(x) = s(x) E_phase at fixed Poisson ratio.  The homogenized stiffness of the
six unit-strain solutions is C_ij; for the loss L = 1/2 ||C - T||_F^2 the
gradient w.r.t. s is sum_ij (C - T)_ij dC_ij/ds_e, with dC_ij/ds_e =
(1/N) mean_gp eps_i^T C_ph eps_j from the stored solutions (no adjoint solve:
the displacement fields are stationary points of the energy).

Checks: (1) with s = 1 everywhere the voxel-field solve equals the phase-table
solve (1e-10); (2) the voxel-field residual matches the oracle with the stress
scaled per voxel (oracle: one phase per voxel class, 1e-12); (3) Euler's
theorem: C is homogeneous of degree one in s, so sum_e s_e dC_ij/ds_e = C_ij
(1e-8, the solve tolerance scale); (4) central finite differences of the loss
at 6 voxels with h = 1e-4 s_e (solves at relative tolerance 1e-12; the FD
difference is O(h^2) accurate, agreement 1e-4 relative).  The spec's
96^3 / h = 1e-6 E check needs C differences of 1e-12 relative, below what an
FP64 solve resolves; the size-independent check (3) covers it at full size in
the bench-sized test below."""
import numpy as np
import pytest

import oracle as O
from helpers import ELASTIC, gpu_context, oracle_problem, random_ms, rel

pytestmark = pytest.mark.gpu


def smooth_log_field(n, seed, ell, std=0.5):
    """Seeded N(0,1) white noise filtered by exp(-1/2 |k|^2 ell^2) (k in radians per
    voxel), rescaled to mean 0 and the given std (the 96^3 adjoint workload's field)."""
    rng = np.random.default_rng(seed)
    w = rng.standard_normal((n, n, n))
    k = 2 * np.pi * np.fft.fftfreq(n)
    kx, ky, kz = np.meshgrid(k, k, k, indexing="ij")
    g = np.real(np.fft.ifftn(np.fft.fftn(w) * np.exp(-0.5 * (kx ** 2 + ky ** 2 + kz ** 2) * ell ** 2)))
    g = (g - g.mean()) / g.std() * std
    return g


def ceff(ctx, store=False):
    C = np.zeros((6, 6))
    for i in range(6):
        g = np.zeros(6)
        g[i] = 1.0
        ctx.reset()
        ctx.set_gradient(g)
        st = ctx.solve()
        assert st["converged"]
        C[:, i] = ctx.homogenized_stress()
        if store:
            ctx.store_solution(i)
    return C


def test_unit_scale_equals_phase_table_and_residual_parity():
    ms = random_ms((12, 8, 10), vf=0.3, seed=3)
    P = oracle_problem(ms, 3, ELASTIC, "HEX8")
    a = gpu_context(P)
    a.set_tolerance("L2", "relative", 1e-10, 500)
    b = gpu_context(P)
    b.set_tolerance("L2", "relative", 1e-10, 500)
    b.set_voxel_scale(np.ones(ms.shape))
    assert rel(ceff(b), ceff(a)) < 1e-8  # element-kernel vs stencil operator, both at tol 1e-10
    # residual with a two-valued scale = oracle with four phases (phase x scale class)
    s = np.where(random_ms(ms.shape, vf=0.5, seed=4) > 0, 2.5, 1.0)
    b.set_voxel_scale(s)
    ms4 = ms + 2 * (s > 1)
    (K0, G0), (K1, G1) = ELASTIC[0][2]
    P4 = oracle_problem(ms4.astype(np.uint16), 3, [(O.LAW_ELASTIC_ISO, [0, 1, 2, 3],
                                                    [[K0, G0], [K1, G1], [2.5 * K0, 2.5 * G0], [2.5 * K1, 2.5 * G1]])],
                        "HEX8", kapparef=P.kapparef)
    g0 = np.array([0.3, 0.1, -0.2, 0.05, 0.0, 0.1])
    P4.set_gradient(g0)
    b.set_gradient(g0)
    u = 1e-2 * np.random.default_rng(1).standard_normal(P.u.shape)
    assert rel(b.residual(u), P4.residual(u)) < 1e-12
    b.reset()
    b.set_gradient(g0)
    b.solve()
    P4.set_gradient(g0)
    P4.solve(tol=1e-10, n_it=500)
    assert rel(b.homogenized_stress(), P4.homogenized_stress()) < 1e-8
    a.close()
    b.close()


def test_stiffness_gradient_euler_and_finite_differences():
    n = 16
    ms = random_ms((n, n, n), vf=0.25, seed=8)
    P = oracle_problem(ms, 3, ELASTIC, "HEX8")
    ctx = gpu_context(P)
    ctx.set_tolerance("L2", "relative", 1e-12, 2000)
    s = np.exp(smooth_log_field(n, 2, 3.0, 0.5))
    ctx.set_voxel_scale(s)
    C = ceff(ctx, store=True)
    rng = np.random.default_rng(3)
    T = C + 0.01 * np.abs(C).max() * (lambda M: M + M.T)(rng.standard_normal((6, 6)))
    W = C - T  # dL/dC for L = 1/2 ||C - T||^2
    grad = ctx.stiffness_gradient(W)
    # Euler: sum_e s_e dC_ij/ds_e = C_ij, tested through W = unit matrices
    for (i, j) in [(0, 0), (0, 1), (3, 3), (2, 5)]:
        E = np.zeros((6, 6))
        E[i, j] = 1.0
        gij = ctx.stiffness_gradient(E)
        assert abs((s * gij).sum() - C[i, j]) <= 1e-8 * abs(C).max()
    loss = lambda Cm: 0.5 * ((Cm - T) ** 2).sum()
    vox = [tuple(v) for v in rng.integers(0, n, size=(6, 3))]
    for v in vox:
        h = 1e-4 * s[v]
        sp, sm = s.copy(), s.copy()
        sp[v] += h
        sm[v] -= h
        ctx.set_voxel_scale(sp)
        Lp = loss(ceff(ctx))
        ctx.set_voxel_scale(sm)
        Lm = loss(ceff(ctx))
        fd = (Lp - Lm) / (2 * h)
        assert abs(fd - grad[v]) <= 1e-4 * abs(grad).max(), (v, fd, grad[v])
    ctx.close()


def test_adjoint_workload_96_euler_property():
    """The 96^3 adjoint workload: E = 10 exp(g), g filtered noise (seed 2, ell = 8
    voxels, std 0.5), nu = 0.3, one phase.  Euler's theorem holds for the full
    gradient at the solve tolerance."""
    n = 96
    ms = np.zeros((n, n, n), dtype=np.uint16)
    K, G = 10.0 / (3 * (1 - 0.6)), 10.0 / (2 * 1.3)
    P = oracle_problem(ms[:4, :4, :4], 3, [(O.LAW_ELASTIC_ISO, [0], [[K, G]])], "HEX8")
    from fans_gb300 import Context

    ctx = Context((n, n, n), (1.0, 1.0, 1.0), 3, "HEX8", "fp64", "cg")
    ctx.set_microstructure(ms)
    ctx.set_phase_material(0, O.LAW_ELASTIC_ISO, [K, G])
    ctx.set_reference(P.kapparef)
    ctx.set_tolerance("L2", "relative", 1e-8, 1000)
    s = np.exp(smooth_log_field(n, 2, 8.0, 0.5))
    ctx.set_voxel_scale(s)
    C = ceff(ctx, store=True)
    assert np.allclose(C, C.T, rtol=1e-6, atol=1e-8 * abs(C).max())
    for (i, j) in [(0, 0), (0, 1), (3, 3)]:
        E = np.zeros((6, 6))
        E[i, j] = 1.0
        gij = ctx.stiffness_gradient(E)
        assert abs((s * gij).sum() - C[i, j]) <= 1e-6 * abs(C).max()
    ctx.close()
