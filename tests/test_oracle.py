"""CPU tests of the oracle (fans_oracle.c): pinned against an independent numpy
restatement, known answers and the reference tests' invariants.

The reference ships no golden numbers (its tests check invariants of its HDF5
output), and it cannot be built here, so these pins are the oracle's anchor:
  * numpy restatement (numpy.fft + LAPACK eigh, vectorised stencil) agrees to
    round-off on B, element stiffness, operator, residual, Green's table,
    convolution and the CG iteration history;
  * homogeneous medium: C_eff = C exactly; thermal and elastic laminates:
    harmonic / arithmetic means, the FE solution is exact there;
  * invariants of test/pytest (mean fluctuation 0, <eps> = loading,
    C_eff symmetric positive definite, <sigma> = C_eff <eps>).
"""
import numpy as np
import pytest

import numpy_ref as R
import oracle as O
from helpers import ELASTIC, THERMAL, random_ms, rel


@pytest.fixture(scope="module", autouse=True)
def _build():
    O.build()


def test_fft_matches_numpy():
    rng = np.random.default_rng(0)
    for shape in [(12, 10, 16), (8, 6, 10), (5, 7, 9)]:
        f = rng.standard_normal(shape)
        assert rel(O.rfft3(f), np.fft.rfftn(f)) < 1e-13
        back = O.irfft3(np.fft.rfftn(f), shape[2]) / f.size
        assert np.abs(back - f).max() < 1e-13


@pytest.mark.parametrize("fe", ["HEX8", "HEX8R", "BBAR"])
@pytest.mark.parametrize("c,groups", [(1, THERMAL), (3, ELASTIC)])
def test_oracle_vs_numpy(c, groups, fe):
    shape = (8, 6, 10)
    rng = np.random.default_rng(1)
    ms = random_ms(shape, seed=2)
    P = O.OracleProblem(ms, [1, 1, 1], c, groups, fe)
    Bs = R.gauss_B(c, fe, P.le)
    assert np.allclose(Bs.ravel(), P.B, rtol=0, atol=1e-14 * np.abs(Bs).max())
    Cph = np.array([O.law_C(P.law[i], P.param[i]) for i in range(P.nphase)])
    Kph = np.array([R.element_stiffness(Bs, Cm, P.ve) for Cm in Cph])
    assert rel(P.Kph, Kph) < 1e-14
    d = rng.standard_normal(shape + (c,))
    assert rel(P.apply_linear(d), R.apply_linear(ms.astype(int), Kph, d)) < 1e-13
    g0 = rng.standard_normal(P.nstr)
    P.set_gradient(g0)
    assert rel(P.residual(d), R.linear_residual(ms.astype(int), Bs, Cph, P.ve, g0, d)) < 1e-13
    K0 = R.element_stiffness(Bs, P.kapparef, P.ve)
    Gn = R.green(shape, c, K0)
    tri = np.tril_indices(c)
    assert rel(P.G, Gn[..., tri[0], tri[1]]) < 1e-12
    assert rel(P.convolve(d), R.convolve(Gn, d)) < 1e-12


@pytest.mark.parametrize("c,groups", [(1, THERMAL), (3, ELASTIC)])
def test_cg_history_matches_numpy(c, groups):
    shape = (10, 8, 12)
    ms = random_ms(shape, seed=3)
    P = O.OracleProblem(ms, [1, 1, 1], c, groups, "HEX8")
    g0 = np.zeros(P.nstr)
    g0[0] = 1.0
    P.set_gradient(g0)
    it = P.solve(tol=1e-10, n_it=300)
    Bs = R.gauss_B(c, "HEX8", P.le)
    Cph = np.array([O.law_C(P.law[i], P.param[i]) for i in range(P.nphase)])
    u, r, it2, err = R.cg_linear(ms.astype(int), Bs, Cph, P.Kph, P.ve, R.green(shape, c, P.K0), g0,
                                 np.zeros(shape + (c,)), 1e-10, 300)
    assert it == it2
    assert rel(P.u, u) < 1e-10
    assert np.abs(P.err_all - err).max() / err[0] < 1e-12


def test_homogeneous_known_answer():
    ms = np.zeros((8, 8, 8), np.uint16)
    P = O.OracleProblem(ms, [1, 1, 1], 3, [(O.LAW_ELASTIC_ISO, [0], [[3.0, 1.5]])], "HEX8")
    C = P.homogenized_tangent_unit(tol=1e-12, type="absolute")
    assert np.abs(C - O.iso_elastic_C(3.0, 1.5)).max() < 1e-13


@pytest.mark.parametrize("fe", ["HEX8", "HEX8R"])
def test_laminate_known_answers(fe):
    ms = np.zeros((16, 4, 6), np.uint16)
    ms[8:] = 1
    T = O.OracleProblem(ms, [1, 1, 1], 1, THERMAL, fe)
    K = T.homogenized_tangent_unit(tol=1e-12, n_it=500, type="absolute")
    assert abs(K[0, 0] - 2 / (1 + 0.1)) < 1e-10
    assert abs(K[1, 1] - 5.5) < 1e-10 and abs(K[2, 2] - 5.5) < 1e-10
    E = O.OracleProblem(ms, [1, 1, 1], 3, ELASTIC, fe)
    Ce = E.homogenized_tangent_unit(tol=1e-12, n_it=500, type="absolute")
    mu = [ELASTIC[0][2][0][1], ELASTIC[0][2][1][1]]
    # Mandel shear 12 and 13 (normal to the layers): harmonic mean of 2 mu; 23: arithmetic mean
    assert abs(Ce[3, 3] - 2 * 2 / (1 / mu[0] + 1 / mu[1])) < 1e-9
    assert abs(Ce[4, 4] - 2 * 2 / (1 / mu[0] + 1 / mu[1])) < 1e-9
    assert abs(Ce[5, 5] - (mu[0] + mu[1])) < 1e-9


def test_reference_invariants_on_random_microstructure():
    """Invariants of the reference's test/pytest checks, on the oracle."""
    ms = random_ms((12, 12, 12), vf=0.3, seed=4)
    P = O.OracleProblem(ms, [1, 1, 1], 3, ELASTIC, "HEX8")
    g0 = np.array([0.001, -0.002, 0.003, 0.0015, -0.0025, 0.001])
    P.set_gradient(g0)
    P.solve(tol=1e-10, n_it=300)
    ss = P.strain_stress(fields=True)
    # test_loading_to_strain_average.py:81 and test_displacement_averaging.py:84-85
    assert np.allclose(ss["strain_average"], g0, rtol=0, atol=1e-12)
    assert np.abs(P.u.reshape(-1, 3).mean(0)).max() < 1e-12
    # test_strain_stress_averaging.py:94-95
    assert np.allclose(ss["stress"].mean(0), ss["stress_average"], rtol=1e-12, atol=1e-14)
    C = P.homogenized_tangent_unit(tol=1e-10, n_it=300)
    # test_homogenized_tangent_spd.py:79-83
    assert np.allclose(C, C.T, rtol=1e-5)
    assert np.linalg.eigvalsh(C).min() > 0
    # test_homogenization_consistency.py:94-95
    assert np.allclose(C @ g0, ss["stress_average"], rtol=1e-4, atol=1e-8)


def test_fp_solver_converges_to_cg_solution():
    ms = random_ms((10, 10, 10), vf=0.2, seed=8)
    A = O.OracleProblem(ms, [1, 1, 1], 1, THERMAL, "HEX8")
    B = O.OracleProblem(ms, [1, 1, 1], 1, THERMAL, "HEX8")
    A.set_gradient([1.0, 0, 0])
    B.set_gradient([1.0, 0, 0])
    A.solve(method="cg", tol=1e-12, n_it=500)
    B.solve(method="fp", tol=1e-12, n_it=2000)
    assert rel(A.homogenized_stress(), B.homogenized_stress()) < 1e-9
