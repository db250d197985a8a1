"""The yield-stress adjoint's checker on the CPU (no GPU).

1. The numpy return map of oracle/j2_adjoint.py equals the C oracle's
   J2PlasticityNew::get_sigma (J2PlasticityNew.h:43-108) on a solved step.
2. The closed-form vector-Jacobian product that the CUDA kernels use
   (fans_gb300/csrc/j2_law.cuh, restated below in numpy) equals J^T seed with J
   from complex-step differentiation, at elastic and plastic Gauss points.
3. The oracle's dense discrete adjoint equals central finite differences of the
   C oracle's forward load path, voxel by voxel."""
import numpy as np
import pytest

import j2_adjoint as A
from helpers import random_ms

J2P = (68.6275, 26.3158, 0.25, 2.0)  # K, G, sigma_y, h of the J2 128^3 workload's matrix
ELP = (222.222, 166.667)


def closed_form_vjp(K, G, h, sy0, e, ep, q, tau, mep, mq):
    """The VJP of j2_law.cuh (j2_vjp), per Gauss point."""
    lam = K - 2.0 / 3.0 * G
    s = 2.0 * G * (e - ep)
    s[:3] += lam * e[:3].sum()
    st = s.copy()
    st[:3] -= s[:3].sum() / 3.0
    s_t = np.sqrt(st @ st)
    a = 2.0 * G + 2.0 / 3.0 * h
    phi = s_t - A.C23 * (sy0 + q * h)
    ge = 2.0 * G * tau
    ge[:3] += lam * tau[:3].sum()
    gep = mep - 2.0 * G * tau
    gq, gsy = mq, 0.0
    if phi > 0 and s_t > 1e-12:
        dg = phi / a
        n = st / s_t
        v = dg * (mep - 2.0 * G * tau)
        ka = (-2.0 * G * (tau @ n) + mep @ n + A.C23 * mq) / a
        w = ka * n + (v - (v @ n) * n) / s_t
        pw = 2.0 * G * (w - np.r_[np.full(3, w[:3].mean()), np.zeros(3)])
        ge, gep = ge + pw, gep - pw
        gq -= A.C23 * h * ka
        gsy = -A.C23 * ka
    return ge, gep, gq, gsy


def test_return_map_matches_c_oracle():
    ms = random_ms((4, 4, 4), vf=0.3, seed=5)
    rng = np.random.default_rng(0)
    sy = 0.25 * (1.0 + 0.2 * rng.random(ms.shape))
    Y = A.YieldPathProblem(ms, J2P, ELP, sy)
    path = [np.array([0.004 * k, 0, 0, 0, 0, 0]) for k in (1, 2)]
    stress, states = Y.run(path)
    P = Y.P
    u, g0, ep0, q0 = states[-1]
    dofs = A.element_dofs(*ms.shape)
    e = A.gp_strain(P, u, g0, dofs)
    nel = ms.size
    j2 = ms.ravel() == 0
    sig, ep1, q1 = A.j2_return_map(np.full((nel, 8), J2P[0]), np.full((nel, 8), J2P[1]), J2P[3],
                                    np.repeat(sy.ravel()[:, None], 8, 1), e, ep0, q0)
    assert (q1[j2] > 0).any() and (q1[j2] == 0).any()  # plastic and elastic Gauss points
    assert np.abs(ep1[j2] - P.ep_t[j2]).max() <= 1e-12 * np.abs(P.ep_t).max()
    assert np.abs(q1[j2] - P.q_t[j2]).max() <= 1e-12 * np.abs(P.q_t).max()
    from oracle import iso_elastic_C

    sig[~j2] = e[~j2] @ iso_elastic_C(*ELP)
    assert np.abs(sig.mean(axis=(0, 1)) - stress).max() <= 1e-12 * np.abs(stress).max()


@pytest.mark.parametrize("plastic", [False, True])
def test_closed_form_vjp_matches_complex_step(plastic):
    rng = np.random.default_rng(1 + plastic)
    K, G, sy, h = J2P
    for _ in range(20):
        e = rng.standard_normal(6) * (0.01 if plastic else 0.0002)
        ep = rng.standard_normal(6) * (0.001 if plastic else 0.0001)
        ep[:3] -= ep[:3].mean()
        q = abs(rng.standard_normal()) * 0.001
        tau, mep, mq = rng.standard_normal(6), rng.standard_normal(6), rng.standard_normal()
        J = A.j2_jacobian(np.array(K), np.array(G), h, np.array(sy), e[None], ep[None], np.array([q]))[0]
        _, _, q1 = A.j2_return_map(np.array([K]), np.array([G]), h, np.array([sy]), e[None], ep[None], np.array([q]))
        assert (q1[0] > q) == plastic
        seed = np.r_[tau, mep, mq]
        ref = seed @ J  # (14,): d/de, d/dep, d/dq, d/dsy
        ge, gep, gq, gsy = closed_form_vjp(K, G, h, sy, e, ep, q, tau, mep, mq)
        got = np.r_[ge, gep, gq, gsy]
        assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max(), (got, ref)


def test_oracle_adjoint_matches_finite_differences():
    ms = random_ms((4, 4, 4), vf=0.3, seed=7)
    rng = np.random.default_rng(2)
    sy = 0.25 * (1.0 + 0.3 * rng.random(ms.shape))
    path = [np.array([0.002 * k, 0.0005 * k, 0, 0.0007 * k, 0, 0]) for k in (1, 2, 3)]
    w = np.array([1.0, 0.3, -0.2, 0.5, 0.1, 0.0])
    stress, grad = A.YieldPathProblem(ms, J2P, ELP, sy).adjoint(path, w)
    assert np.all(grad[ms != 0] == 0.0)
    j2_vox = [tuple(v) for v in np.argwhere(ms == 0)]
    pick = [j2_vox[i] for i in rng.choice(len(j2_vox), 6, replace=False)]
    hstep = 1e-6
    for v in pick:
        Ls = []
        for sgn in (1, -1):
            s2 = sy.copy()
            s2[v] += sgn * hstep
            st, _ = A.YieldPathProblem(ms, J2P, ELP, s2).run(path)
            Ls.append(w @ st)
        fd = (Ls[0] - Ls[1]) / (2 * hstep)
        assert abs(fd - grad[v]) <= 1e-5 * np.abs(grad).max() + 1e-9, (v, fd, grad[v])
    assert np.abs(grad).max() > 0
