"""The GPU path, through the FANS driver (Reader -> run_solver -> results
file), on the reference's own mixed-BC test inputs, against the numbers the
reference computed and wrote into those inputs (see make_fixtures.py):

test_MixedBCs.json (small strain, PseudoPlasticLinearHardening + elastic
sphere, HEX8): load case 2 (pure stress control, hydrostatic -0.05 / -0.1)
reaches the strains that load case 3 prescribes (-2.01177817616389e-4 /
-4.0235563523281944e-4), and load case 3 gives the stresses back.

test_MixedBCs_LargeStrain.json (CompressibleNeoHookean, HEX8): load case 1
(F33 to 2 in ten steps, P11 = P22 = 0) ends at F11 = F22 = 0.832542244829 with
P33 = 74.757449712464; load case 2 (those stresses prescribed) and load case 3
(that F prescribed) reach the same state.

Tolerances: the reference solved to Linfinity 1e-10 (absolute) and printed
12 decimals (large strain); both solves stop somewhere inside that tolerance,
so strains agree to 1e-8 relative and stresses to 1e-8 absolute."""
import copy
import json
import os

import numpy as np
import pytest

from fans_gb300.reader import Reader
from fans_gb300.run import ResultsFile, run_solver

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _run(name, tmp_path):
    j = copy.deepcopy(json.load(open(os.path.join(GOLDEN, "reference_inputs.json")))[name])
    j["results"] = ["stress_average", "strain_average", "absolute_error"]
    reader = Reader().ReadInputFile(j)
    reader.set_microstructure(np.load(os.path.join(GOLDEN, "sphere32_ms.npy")))
    res = ResultsFile(reader, str(tmp_path / (name + ".h5")))
    steps = run_solver(reader, res, "fp64", log=lambda *a: None)
    res.close()
    return j, steps


def _last(steps, load):
    return [s for s in steps if s["load"] == load]


def test_small_strain_mixed_bcs_reproduce_reference(tmp_path):
    j, steps = _run("test_MixedBCs", tmp_path)
    stress_lc, strain_lc = j["macroscale_loading"][1], j["macroscale_loading"][2]
    lc1 = _last(steps, 0)
    assert len(lc1) == len(j["macroscale_loading"][0]["strain"])
    for s in lc1:  # stress-controlled components 0, 1 stay at zero
        assert np.abs(s["stress"][:2]).max() < 1e-8
    for k, s in enumerate(_last(steps, 1)):
        assert np.allclose(s["strain"], strain_lc[k], rtol=1e-8, atol=1e-15), (k, s["strain"], strain_lc[k])
        assert np.allclose(s["stress"], stress_lc["stress"][k], rtol=0, atol=1e-9)
    for k, s in enumerate(_last(steps, 2)):
        assert np.allclose(s["stress"], stress_lc["stress"][k], rtol=0, atol=1e-9)


def test_large_strain_mixed_bcs_reproduce_reference(tmp_path):
    j, steps = _run("test_MixedBCs_LargeStrain", tmp_path)
    stress_lc, strain_lc = j["macroscale_loading"][1], j["macroscale_loading"][2]
    F_gold, P_gold = np.asarray(strain_lc[0]), np.asarray(stress_lc["stress"][0])
    lc1 = _last(steps, 0)
    assert len(lc1) == 10
    end = lc1[-1]
    assert np.allclose(end["strain"], F_gold, rtol=0, atol=2e-9), end["strain"]
    assert np.allclose(end["stress"], P_gold, rtol=0, atol=1e-8), end["stress"]
    (lc2,) = _last(steps, 1)
    assert np.allclose(lc2["strain"], F_gold, rtol=0, atol=2e-9)
    assert np.allclose(lc2["stress"], P_gold, rtol=0, atol=1e-8)
    (lc3,) = _last(steps, 2)
    assert np.allclose(lc3["stress"], P_gold, rtol=0, atol=1e-8)
