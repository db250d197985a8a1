"""The oracle against numbers the reference itself computed (no GPU).

The reference's test/input_files/test_MixedBCs.json and
test_MixedBCs_LargeStrain.json load their later load cases with the
macroscopic state their first load case reached on sphere32 -- reference
outputs written into its own inputs (extracted to tests/golden by
make_fixtures.py):
  * small strain (PseudoPlasticLinearHardening matrix, elastic sphere, HEX8):
    hydrostatic stress -0.05 / -0.1 gives strain -2.01177817616389e-4 /
    -4.0235563523281944e-4 on each normal component, and that strain gives the
    stress back;
  * large strain (CompressibleNeoHookean, HEX8): F = diag(0.832542244829,
    0.832542244829, 2.000000000001) carries P33 = 74.757449712464 with the
    other components zero.
The reference solved with Linfinity absolute 1e-10 and printed 12 (large) or
17 (small) significant digits; the tolerances below are those digits plus the
solver tolerance."""
import json
import os

import numpy as np
import pytest

import oracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _inputs(name):
    return json.load(open(os.path.join(GOLDEN, "reference_inputs.json")))[name]


def _groups(j):
    out = []
    for mg in j["materials"]:
        p = mg["material_properties"]
        name = mg["matmodel"]
        if name == "PseudoPlasticLinearHardening":
            law, prm = O.LAW_PSEUDO_LIN, [[p["bulk_modulus"][i], p["shear_modulus"][i], p["yield_stress"][i],
                                          p["hardening_parameter"][i]] for i in range(len(mg["phases"]))]
        elif name == "LinearElasticIsotropic":
            law, prm = O.LAW_ELASTIC_ISO, [[p["bulk_modulus"][i], p["shear_modulus"][i]] for i in range(len(mg["phases"]))]
        elif name == "CompressibleNeoHookean":
            law, prm = O.LAW_NEOHOOKEAN, [[p["bulk_modulus"][i], p["shear_modulus"][i]] for i in range(len(mg["phases"]))]
        else:
            raise AssertionError(name)
        out.append((law, mg["phases"], prm))
    return out


@pytest.fixture(scope="module")
def sphere32():
    return np.load(os.path.join(GOLDEN, "sphere32_ms.npy"))


def test_small_strain_mixed_bc_hydrostatic_matches_reference(sphere32):
    j = _inputs("test_MixedBCs")
    stress_lc, strain_lc = j["macroscale_loading"][1], j["macroscale_loading"][2]
    P = O.OracleProblem(sphere32, (1.0, 1.0, 1.0), 3, _groups(j), j["FE_type"])
    for step, target in enumerate(stress_lc["stress"]):
        P.enable_mixed_bc(stress_lc["strain_indices"], [], stress_lc["stress_indices"], target, step)
        P.solve(measure="Linfinity", type="absolute", tol=1e-10, n_it=j["n_it"])
        eps = P.strain_stress()["strain_average"]
        gold = np.asarray(strain_lc[step])
        assert np.allclose(eps, gold, rtol=1e-8, atol=1e-15), (step, eps, gold)
        P.extrapolate_displacement()
    # and the golden strain, prescribed, gives the stress back (load case 3 of the same file)
    Q = O.OracleProblem(sphere32, (1.0, 1.0, 1.0), 3, _groups(j), j["FE_type"])
    for step, g in enumerate(strain_lc):
        Q.set_gradient(g)
        Q.solve(measure="Linfinity", type="absolute", tol=1e-10, n_it=j["n_it"])
        assert np.allclose(Q.homogenized_stress(), stress_lc["stress"][step], rtol=0, atol=1e-9)
        Q.extrapolate_displacement()


def test_large_strain_neo_hookean_matches_reference(sphere32):
    j = _inputs("test_MixedBCs_LargeStrain")
    stress_lc, strain_lc = j["macroscale_loading"][1], j["macroscale_loading"][2]
    P = O.OracleProblem(sphere32, (1.0, 1.0, 1.0), 3, _groups(j), j["FE_type"], strain_type="large")
    P.set_gradient(strain_lc[0])
    P.solve(measure="Linfinity", type="absolute", tol=1e-10, n_it=j["n_it"])
    Pk = P.homogenized_stress()
    gold = np.asarray(stress_lc["stress"][0])
    assert abs(Pk[8] - gold[8]) < 2e-9  # 74.757449712464 printed to 12 decimals
    assert np.abs(Pk[:8] - gold[:8]).max() < 2e-9
