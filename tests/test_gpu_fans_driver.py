"""The FANS driver on the GPU path, end to end: input JSON -> Reader -> one
Solver per load case -> postprocess -> HDF5 results file, on the reference's
own test problems (sphere32, test_LinearElastic / test_LinearThermal settings).

The checks are the reference's pytest suite (test/pytest/*.py) applied to our
results file with its tolerances:
  strain_average == loading               (test_loading_to_strain_average, np.allclose defaults)
  mean(strain|stress field) == average    (test_strain_stress_averaging, rtol 1e-5, atol 1e-8)
  mean(displacement_fluctuation) == 0     (test_displacement_averaging, rtol 1e-5, atol 1e-8)
  tangent symmetric and SPD               (test_homogenized_tangent_spd, rtol 1e-5, atol 1e-8)
  Reuss <= tangent <= Voigt               (test_homogenized_tangent_within_VRbounds)
  stress_average == tangent strain_average (test_homogenization_consistency, rtol 1e-4, atol 1e-1)
plus parity of the stress average with the oracle on the same problem (1e-9:
both solves stop at the same absolute L-infinity tolerance 1e-10)."""
import copy
import json
import os

import numpy as np
import pytest

import oracle as O
from fans_gb300 import h5
from fans_gb300.reader import Reader
from fans_gb300.run import ResultsFile, run_solver
from helpers import rel

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _phase_tensors(j):
    out = []
    for mg in j["materials"]:
        p = mg["material_properties"]
        for i, _ in enumerate(mg["phases"]):
            if "conductivity" in p:
                out.append(p["conductivity"][i] * np.eye(3))
            else:
                out.append(O.iso_elastic_C(p["bulk_modulus"][i], p["shear_modulus"][i]))
    return out


@pytest.mark.parametrize("case", ["test_LinearElastic", "test_LinearThermal"])
def test_reference_problem_results_file(case, tmp_path):
    j = copy.deepcopy(json.load(open(os.path.join(GOLDEN, "reference_inputs.json")))[case])
    j["results"] = sorted(set(j["results"]) | {"strain", "stress", "displacement_fluctuation", "residual"})
    reader = Reader().ReadInputFile(j)
    ms = np.load(os.path.join(GOLDEN, "sphere32_ms.npy"))
    reader.set_microstructure(ms)
    out = str(tmp_path / "results.h5")
    res = ResultsFile(reader, out)
    logs = []
    run_solver(reader, res, "fp64", log=logs.append)
    res.close()

    f = h5.H5File(out)
    base = f"{reader.dataset_name}/load0/time_step0"
    load = np.asarray(j["macroscale_loading"][0][0])
    strain_avg, stress_avg = f.read(base + "/strain_average"), f.read(base + "/stress_average")
    assert np.allclose(strain_avg, load)
    strain = np.swapaxes(f.read(base + "/strain"), 0, 2)
    stress = np.swapaxes(f.read(base + "/stress"), 0, 2)
    assert np.allclose(strain.mean(axis=(0, 1, 2)), strain_avg, rtol=1e-5, atol=1e-8)
    assert np.allclose(stress.mean(axis=(0, 1, 2)), stress_avg, rtol=1e-5, atol=1e-8)
    u = np.swapaxes(f.read(base + "/displacement_fluctuation"), 0, 2)
    assert np.allclose(u.mean(axis=(0, 1, 2)), 0.0, rtol=1e-5, atol=1e-8)
    T = f.read(base + "/homogenized_tangent")
    assert np.allclose(T, T.T, rtol=1e-5, atol=1e-8)
    assert np.linalg.eigvalsh(T).min() > 0
    vf = np.array([np.mean(ms == k) for k in range(2)])
    Cs = _phase_tensors(j)
    voigt = sum(v * C for v, C in zip(vf, Cs))
    reuss = np.linalg.inv(sum(v * np.linalg.inv(C) for v, C in zip(vf, Cs)))
    assert np.linalg.eigvalsh(voigt - T).min() > 0
    assert np.linalg.eigvalsh(T - reuss).min() > 0
    assert np.allclose(T @ strain_avg, stress_avg, rtol=1e-4, atol=1e-1)
    err = f.read(base + "/absolute_error")
    assert err[-1] <= 1e-10 < err[0]
    assert f.attrs(base + "/stress")["permute_order"] == b"zyx"

    # parity with the oracle on the same problem and tolerance
    c = 1 if j["problem_type"] == "thermal" else 3
    law = O.LAW_THERMAL_ISO if c == 1 else O.LAW_ELASTIC_ISO
    mp = j["materials"][0]["material_properties"]
    params = [[k] for k in mp["conductivity"]] if c == 1 else [[K, G] for K, G in zip(mp["bulk_modulus"],
                                                                                          mp["shear_modulus"])]
    P = O.OracleProblem(ms, [1.0, 1.0, 1.0], c, [(law, [0, 1], params)], j["FE_type"])
    P.set_gradient(load)
    P.solve(measure="Linfinity", type="absolute", tol=1e-10, n_it=100)
    assert rel(stress_avg, P.homogenized_stress()) < 1e-9


def test_j2_load_path_results_file(tmp_path):
    """A J2PlasticityNew load path through the driver: internal variables are
    committed per step and written as plastic_strain / isotropic_hardening_variable."""
    ms = np.load(os.path.join(GOLDEN, "sphere32_ms.npy"))[::2, ::2, ::2].copy()
    j = {"microstructure": {"filepath": "unused.h5", "datasetname": "/ms", "L": [1.0, 1.0, 1.0]},
         "problem_type": "mechanical", "method": "cg", "FE_type": "HEX8", "n_it": 300,
         "error_parameters": {"measure": "L2", "type": "relative", "tolerance": 1e-10},
         "materials": [{"phases": [0], "matmodel": "J2PlasticityNew_LinearIsotropicHardening",
                        "material_properties": {"bulk_modulus": [68.6275], "shear_modulus": [26.3158],
                                                "yield_stress": [0.25], "isotropic_hardening_parameter": [2.0]}},
                       {"phases": [1], "matmodel": "LinearElasticIsotropic",
                        "material_properties": {"bulk_modulus": [222.222], "shear_modulus": [166.667]}}],
         "macroscale_loading": [[[0.004 * k, 0, 0, 0, 0, 0] for k in range(1, 4)]],
         "results": ["stress_average", "strain_average", "plastic_strain", "isotropic_hardening_variable",
                     "plastic_strain_gp", "stress_gp", "absolute_error"]}
    reader = Reader().ReadInputFile(j)
    reader.set_microstructure(ms)
    out = str(tmp_path / "j2.h5")
    res = ResultsFile(reader, out)
    steps = run_solver(reader, res, "fp64", log=lambda *a: None)
    res.close()
    f = h5.H5File(out)
    # oracle on the same path (extrapolate_displacement defaults to true, as in main.cpp:36-37)
    P = O.OracleProblem(ms.astype(np.uint16), [1.0, 1.0, 1.0], 3,
                        [(O.LAW_J2, [0], [[68.6275, 26.3158, 0.25, 2.0]]),
                         (O.LAW_ELASTIC_ISO, [1], [[222.222, 166.667]])], "HEX8")
    for t in range(3):
        g = np.zeros(6)
        g[0] = 0.004 * (t + 1)
        P.set_gradient(g)
        P.solve(tol=1e-10, n_it=300)
        base = f"{reader.dataset_name}/load0/time_step{t}"
        assert rel(f.read(base + "/stress_average"), P.homogenized_stress()) < 1e-7
        P.extrapolate_displacement()
    ep = np.swapaxes(f.read(f"{reader.dataset_name}/load0/time_step2/plastic_strain"), 0, 2).reshape(-1, 6)
    assert rel(ep, P.ep_t.mean(axis=1)) < 1e-6
    epg = np.swapaxes(f.read(f"{reader.dataset_name}/load0/time_step2/plastic_strain_gp"), 0, 2)
    assert epg.shape == ms.shape + (8, 6)
    assert rel(epg.reshape(-1, 8, 6), P.ep_t) < 1e-6
    sg = np.swapaxes(f.read(f"{reader.dataset_name}/load0/time_step2/stress_gp"), 0, 2)
    assert np.allclose(sg.mean(axis=3).mean(axis=(0, 1, 2)), steps[-1]["stress"], rtol=1e-10, atol=1e-12)
