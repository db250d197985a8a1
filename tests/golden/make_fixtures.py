"""Builds the committed fixtures of this folder from the reference's own test data.

* sphere32_ms.npy -- the microstructure /sphere/32x32x32/ms of the reference's
  test/microstructures/sphere32.h5, decoded by fans_gb300.h5 (chunked, deflate)
  and put in [x][y][z] order as Reader::ReadMS does (ZYX on disk, reader.h:54);
  sphere32.json records the source file's SHA-256, shape and volume fraction.
* reference_inputs.json -- the solver, material and loading settings of the
  reference's test/input_files/*.json (the problem definitions its pytest suite
  runs on sphere32).  test_MixedBCs.json and test_MixedBCs_LargeStrain.json
  carry reference outputs inside their loading: their later load cases are
  loaded with the macroscopic strain / stress the first load case reached
  (hydrostatic strain -2.01177817616389e-4 at stress -0.05; F11 = F22 =
  0.832542244829 and P33 = 74.757449712464 at F33 = 2 on CompressibleNeoHookean),
  which pins the oracle and the GPU path to numbers the reference computed.

Run from the repository root with a FANS checkout given as the argument or in
the FANS_REFERENCE environment variable:  python tests/golden/make_fixtures.py REF
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from fans_gb300 import h5  # noqa: E402

REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("FANS_REFERENCE", "")
KEEP = ("microstructure", "problem_type", "strain_type", "materials", "FE_type", "method", "error_parameters",
        "n_it", "macroscale_loading", "results")


def main():
    if not REF or not os.path.isdir(REF):
        sys.exit("usage: make_fixtures.py REF  (or set FANS_REFERENCE): REF is a FANS checkout")
    src = os.path.join(REF, "test", "microstructures", "sphere32.h5")
    raw = open(src, "rb").read()
    ms = h5.read_microstructure(src, "/sphere/32x32x32/ms").astype(np.uint8)
    np.save(os.path.join(HERE, "sphere32_ms.npy"), ms)
    meta = {"source": "test/microstructures/sphere32.h5", "dataset": "/sphere/32x32x32/ms",
            "sha256": hashlib.sha256(raw).hexdigest(), "shape": list(ms.shape),
            "volume_fraction_phase1": float(ms.mean()), "order": "xyz (transposed from the file's zyx)"}
    with open(os.path.join(HERE, "sphere32.json"), "w") as f:
        json.dump(meta, f, indent=1)
    inputs = {}
    for name in ("test_LinearElastic", "test_LinearThermal", "test_MixedBCs", "test_MixedBCs_LargeStrain",
                 "test_CompressibleNeoHookean", "test_J2Plasticity", "test_PseudoPlastic"):
        with open(os.path.join(REF, "test", "input_files", name + ".json")) as f:
            j = json.load(f)
        inputs[name] = {k: j[k] for k in KEEP if k in j}
    with open(os.path.join(HERE, "reference_inputs.json"), "w") as f:
        json.dump(inputs, f, indent=1)
    print(meta)


if __name__ == "__main__":
    main()
