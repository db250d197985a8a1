"""PyFANS.MicroSimulation mirror (pyfans/micro.cpp:27-85) on the GPU path: the
dict keys, the 21-entry cmat1..cmat7 packing of the tangent's upper triangle,
and the values against the oracle, with the microstructure read from an HDF5
file written by fans_gb300.h5 (ZYX on disk, as FANS expects by default)."""
import copy
import json
import os

import numpy as np
import pytest

import oracle as O
from fans_gb300 import h5
from fans_gb300.pyfans import CMAT_ENTRIES, MicroSimulation
from helpers import rel

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_micro_simulation_solve(tmp_path):
    ms = np.load(os.path.join(GOLDEN, "sphere32_ms.npy"))
    with h5.H5Writer(str(tmp_path / "ms.h5")) as w:
        w.dataset("/sphere/32x32x32/ms", np.ascontiguousarray(ms.transpose(2, 1, 0)))
    j = copy.deepcopy(json.load(open(os.path.join(GOLDEN, "reference_inputs.json")))["test_LinearElastic"])
    j["microstructure"]["filepath"] = str(tmp_path / "ms.h5")
    j["error_parameters"] = {"measure": "L2", "type": "relative", "tolerance": 1e-8}
    inp = tmp_path / "input.json"
    inp.write_text(json.dumps(j))
    sim = MicroSimulation(0, str(inp))
    e13, e46 = np.array([0.005, 0.005, 0.005]), np.array([0.0005, 0.0005, 0.0005])
    out = sim.solve({"strains1to3": e13, "strains4to6": e46}, 1.0)
    sim.close()
    assert sorted(out) == sorted(["stresses1to3", "stresses4to6"] + [f"cmat{k}" for k in range(1, 8)])
    C = np.zeros((6, 6))
    for k in range(7):
        for (r, c), v in zip(CMAT_ENTRIES[3 * k:3 * k + 3], out[f"cmat{k + 1}"]):
            C[r, c] = C[c, r] = v
    sig = np.concatenate([out["stresses1to3"], out["stresses4to6"]])
    eps = np.concatenate([e13, e46])
    assert np.allclose(C @ eps, sig, rtol=1e-4)  # linear material: sigma = C eps
    mp = j["materials"][0]["material_properties"]
    P = O.OracleProblem(ms, [1.0, 1.0, 1.0], 3, [(O.LAW_ELASTIC_ISO, [0, 1],
                                                  [[K, G] for K, G in zip(mp["bulk_modulus"], mp["shear_modulus"])])],
                        j["FE_type"])
    P.set_gradient(eps)
    P.solve(measure="L2", type="relative", tol=1e-8, n_it=200)
    assert rel(sig, P.homogenized_stress()) < 1e-7
