"""Large-strain host rules (no GPU): the oracle's SaintVenantKirchhoff and
CompressibleNeoHookean stresses against the derivative of their strain
energies, and the reference stiffness of MaterialManager against the oracle's
restatement of LargeStrainMechModel::compute_spatial_tangent
(LargeStrainMechModel.h:96-170)."""
import numpy as np
import pytest

import oracle as O
from helpers import oracle_problem


def _energy(law, lam, mu, F):
    C = F.T @ F
    E = 0.5 * (C - np.eye(3))
    J = np.linalg.det(F)
    if law == O.LAW_SVK:
        return 0.5 * lam * np.trace(E) ** 2 + mu * np.trace(E @ E)
    return 0.5 * mu * (np.trace(C) - 3.0) - mu * np.log(J) + 0.5 * lam * np.log(J) ** 2


@pytest.mark.parametrize("law", [O.LAW_SVK, O.LAW_NEOHOOKEAN])
def test_oracle_first_piola_is_the_energy_derivative(law):
    K, G = 2.5, 1.2
    lam, mu = K - 2.0 / 3.0 * G, G
    F = np.eye(3) + 0.08 * np.random.default_rng(1).standard_normal((3, 3))
    P = oracle_problem(np.zeros((2, 2, 2), np.uint16), 3, [(law, [0], [[K, G]])], strain_type="large")
    P.set_gradient(F.ravel())
    Pk = P.strain_stress()["stress_average"].reshape(3, 3)
    h, D = 1e-6, np.zeros((3, 3))
    for i in range(3):
        for j in range(3):
            d = np.zeros((3, 3))
            d[i, j] = h
            D[i, j] = (_energy(law, lam, mu, F + d) - _energy(law, lam, mu, F - d)) / (2 * h)
    assert np.abs(Pk - D).max() < 1e-8 * np.abs(D).max() + 1e-9


def test_neo_hookean_negative_jacobian_is_not_finite():
    P = oracle_problem(np.zeros((2, 2, 2), np.uint16), 3, [(O.LAW_NEOHOOKEAN, [0], [[2.0, 1.0]])],
                       strain_type="large")
    P.set_gradient(np.diag([-1.0, 1.0, 1.0]).ravel())
    assert not np.isfinite(P.strain_stress()["stress_average"]).all()


def test_reference_stiffness_matches_spatial_tangent_restatement():
    from fans_gb300.materials import MaterialManager

    props = {"bulk_modulus": [62.5, 222.222], "shear_modulus": [28.8462, 166.6667]}
    for name, law in (("SaintVenantKirchhoff", O.LAW_SVK), ("CompressibleNeoHookean", O.LAW_NEOHOOKEAN)):
        mm = MaterialManager({"materials": [{"phases": [0, 1], "matmodel": name, "material_properties": props}]},
                             "mechanical", strain_type="large")
        assert mm.law == [law, law] and mm.kapparef_mat.shape == (9, 9)
        ref = O.model_reference_stiffness(law, [[62.5, 28.8462], [222.222, 166.6667]])
        assert np.allclose(mm.kapparef_mat, ref, rtol=1e-14, atol=1e-12)
        assert np.allclose(mm.kapparef_mat, mm.kapparef_mat.T)
    with pytest.raises(ValueError, match="not a valid small strain material model"):
        MaterialManager({"materials": [{"phases": [0], "matmodel": "SaintVenantKirchhoff",
                                        "material_properties": props}]}, "mechanical")
    with pytest.raises(ValueError, match="not a valid large strain material model"):
        MaterialManager({"materials": [{"phases": [0], "matmodel": "LinearElasticIsotropic",
                                        "material_properties": props}]}, "mechanical", strain_type="large")


def test_large_strain_b_matrix_layout():
    P = oracle_problem(np.zeros((4, 4, 4), np.uint16), 3, [(O.LAW_SVK, [0], [[2.0, 1.0]])], strain_type="large")
    B = P.B.reshape(P.ngp, 9, 24)
    # a homogeneous displacement gradient H (u_i = H_iJ X_J at the nodes) gives F - I = H at every Gauss point
    H = np.arange(9.0).reshape(3, 3) / 10.0
    le = P.le
    X = np.array([[(q & 1) * le[0], ((q >> 1) & 1) * le[1], ((q >> 2) & 1) * le[2]] for q in range(8)])
    ue = (X @ H.T).ravel()
    for gp in range(P.ngp):
        assert np.allclose(B[gp] @ ue, H.ravel())
