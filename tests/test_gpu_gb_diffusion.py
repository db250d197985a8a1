"""GBDiffusion (GBDiffusion.h) through the driver: a synthetic polycrystal (4
crystals, 3 grain-boundary tags) in an HDF5 file whose dataset carries
num_crystals, num_GB and the GBVoxelInfo JSON as attributes; the solve must
match the oracle with the same per-phase conductivity tensors (1e-9), and the
GBnormals field must hold each GB voxel's normal."""
import json
import os

import numpy as np
import pytest

import oracle as O
from fans_gb300 import h5
from fans_gb300.materials import gb_diffusion_tensors
from fans_gb300.reader import Reader
from fans_gb300.run import ResultsFile, run_solver
from helpers import rel

pytestmark = pytest.mark.gpu


def polycrystal(n, seed=0):
    rng = np.random.default_rng(seed)
    seeds = rng.uniform(0, n, size=(4, 3))
    X = np.stack(np.meshgrid(*[np.arange(n) + 0.5] * 3, indexing="ij"), -1)
    d = np.linalg.norm(((X[..., None, :] - seeds) + n / 2) % n - n / 2, axis=-1)
    grain = d.argmin(-1)
    ms = grain.copy()
    gb = np.zeros_like(grain, dtype=bool)
    for ax in range(3):
        gb |= grain != np.roll(grain, 1, axis=ax)
    ms[gb] = 4 + (grain[gb] % 3)  # three GB tags
    return ms.astype(np.uint8)


def test_gb_diffusion_driver_matches_oracle(tmp_path):
    n = 16
    ms = polycrystal(n)
    info = {f"gb{t}": {"GB_tag": t, "GB_normal": nrm} for t, nrm in
            zip((4, 5, 6), ([1.0, 0.0, 0.0], [0.0, 0.6, 0.8], [0.3, 0.4, 0.0]))}
    with h5.H5Writer(str(tmp_path / "poly.h5")) as w:
        w.dataset("/poly/ms", np.ascontiguousarray(ms.transpose(2, 1, 0)),
                  {"num_crystals": np.int64(4), "num_GB": np.int64(3), "GBVoxelInfo": h5.VlenStr(json.dumps(info))})
    props = {"GB_unformity": True, "D_bulk": 1.0, "D_par": 5.0, "D_perp": 0.2}
    j = {"microstructure": {"filepath": str(tmp_path / "poly.h5"), "datasetname": "/poly/ms", "L": [1, 1, 1]},
         "problem_type": "thermal", "method": "cg", "FE_type": "HEX8", "n_it": 500,
         "error_parameters": {"measure": "L2", "type": "relative", "tolerance": 1e-10},
         "materials": [{"phases": list(range(7)), "matmodel": "GBDiffusion", "material_properties": props}],
         "macroscale_loading": [[[1.0, 0.5, 0.0]]], "results": ["stress_average", "GBnormals"]}
    reader = Reader().ReadInputFile(j)
    out = str(tmp_path / "res.h5")
    res = ResultsFile(reader, out)
    run_solver(reader, res, "fp64", log=lambda *a: None)
    res.close()
    f = h5.H5File(out)
    base = "/poly/ms_results/load0/time_step0"
    sig = f.read(base + "/stress_average")
    K, normals = gb_diffusion_tensors(props, {"num_crystals": 4, "num_GB": 3, "GBVoxelInfo": json.dumps(info)})
    P = O.OracleProblem(ms, [1.0, 1.0, 1.0], 1, [(O.LAW_THERMAL_TRI, list(range(7)), K)], "HEX8")
    P.set_gradient(np.array([1.0, 0.5, 0.0]))
    P.solve(tol=1e-10, n_it=500)
    assert rel(sig, P.homogenized_stress()) < 1e-9
    gbn = np.swapaxes(f.read(base + "/GBnormals"), 0, 2)
    assert np.allclose(gbn[ms == 5], [0.0, 0.6, 0.8])
    assert np.allclose(gbn[ms < 4], 0.0)
