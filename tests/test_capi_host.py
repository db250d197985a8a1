"""CPU tests of the C ABI library and the host mirror (no GPU compute calls).

* libfans_gb300.so loads and exports every symbol include/fans_gb300.h declares;
* fansgpu_create fails cleanly (status + message, no crash) without a device;
* MaterialManager mirror: phase table, legacy JSON format, reference
  stiffness rule, SPD check, error paths -- against the oracle's restatement.
"""
import ctypes
import os
import re

import numpy as np
import pytest

import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    src = open(os.path.join(ROOT, "include", "fans_gb300.h")).read()
    return sorted(set(re.findall(r"\b(fansgpu_[a-z_0-9]+)\s*\(", src)))


def test_library_exports_every_header_symbol():
    from fans_gb300 import _lib

    L = _lib.load()
    syms = header_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(L, s), s
    assert set(syms) == set(_lib.EXPORTS)
    assert b"sm_103a" in L.fansgpu_version()


def test_header_constants_match_the_binding():
    """Every #define FANSGPU_<NAME> value the ctypes binding also names (as <NAME>)
    is the same number on both sides."""
    from fans_gb300 import _lib

    src = open(os.path.join(ROOT, "include", "fans_gb300.h")).read()
    defs = {m.group(1): int(m.group(2)) for m in re.finditer(r"#define FANSGPU_([A-Z0-9_]+)\s+(-?\d+)", src)}
    shared = [k for k in defs if hasattr(_lib, k)]
    assert {"NEWTON", "VOXEL_YIELD_STRESS", "LAW_J2_LINEAR", "FIELD_U", "MIXED", "LARGE_STRAIN"} <= set(shared)
    for k in shared:
        assert getattr(_lib, k) == defs[k], k


def test_create_without_device_fails_cleanly():
    from conftest import have_gpu

    if have_gpu():
        pytest.skip("device present")
    from fans_gb300 import Context, FansGpuError

    with pytest.raises(FansGpuError) as ei:
        Context((8, 8, 8), (1, 1, 1), 3)
    assert ei.value.code == -3


def test_create_argument_validation():
    from fans_gb300 import Context, FansGpuError

    for kw, code in [(dict(n=(7, 8, 8)), -6), (dict(n=(8, 8, 8), howmany=2), -1), (dict(n=(8, 8, 8), fe_type=5), -1),
                     (dict(n=(8, 8, 8), precision="mixed", method="fp"), -6),
                     (dict(n=(8, 8, 8), precision="mixed", method="newton"), -6), (dict(n=(8, 8, 8), method=3), -1)]:
        n = kw.pop("n")
        with pytest.raises(FansGpuError) as ei:
            Context(n, (1, 1, 1), **({"howmany": 3} | kw))
        assert ei.value.code == code


def _mm_json(materials, **extra):
    return {"materials": materials, **extra}


def test_material_manager_reference_rule_matches_oracle():
    from fans_gb300.materials import MaterialManager

    j = _mm_json([
        {"phases": [0, 2], "matmodel": "LinearElasticIsotropic",
         "material_properties": {"bulk_modulus": [3.0, 40.0], "shear_modulus": [1.0, 30.0]}},
        {"phases": [1], "matmodel": "J2PlasticityNew_LinearIsotropicHardening",
         "material_properties": {"bulk_modulus": [68.6], "shear_modulus": [26.3], "yield_stress": [0.25],
                                 "isotropic_hardening_parameter": [2.0]}},
    ])
    mm = MaterialManager(j)
    assert mm.n_phases == 3 and not mm.all_linear
    groups = [(O.LAW_ELASTIC_ISO, [0, 2], [[3.0, 1.0], [40.0, 30.0]]),
              (O.LAW_J2, [1], [[68.6, 26.3, 0.25, 2.0]])]
    P = O.OracleProblem(np.zeros((4, 4, 4), np.uint16), [1, 1, 1], 3, groups, "HEX8")
    assert np.allclose(mm.kapparef_mat, P.kapparef, rtol=1e-15)
    assert mm.params[2] == [40.0, 30.0] and mm.params[1] == [68.6, 26.3, 0.25, 2.0]


def test_material_manager_legacy_and_errors():
    from fans_gb300.materials import MaterialManager

    legacy = {"matmodel": "LinearThermalIsotropic", "material_properties": {"conductivity": [1.0, 10.0]}}
    mm = MaterialManager(legacy)
    assert mm.n_phases == 2 and np.allclose(mm.kapparef_mat, 5.5 * np.eye(3))
    with pytest.raises(RuntimeError, match="not assigned"):
        MaterialManager(_mm_json([{"phases": [0, 2], "matmodel": "LinearThermalIsotropic",
                                   "material_properties": {"conductivity": [1.0, 2.0]}}]))
    with pytest.raises(RuntimeError, match="duplicate"):
        MaterialManager(_mm_json([{"phases": [0, 0], "matmodel": "LinearThermalIsotropic",
                                   "material_properties": {"conductivity": [1.0, 2.0]}}]))
    with pytest.raises(ValueError, match="positive definite"):
        MaterialManager(_mm_json([{"phases": [0], "matmodel": "LinearThermalIsotropic",
                                   "material_properties": {"conductivity": [1.0]}}],
                                 reference_material=[[1, 0, 0], [0, -1, 0], [0, 0, 1]]))
    with pytest.raises(RuntimeError, match="Missing material properties"):
        MaterialManager(_mm_json([{"phases": [0], "matmodel": "LinearElasticIsotropic",
                                   "material_properties": {"bulk_modulus": [1.0]}}]))
    with pytest.raises(ValueError, match="not a valid matmodel"):
        MaterialManager(_mm_json([{"phases": [0], "matmodel": "Nope", "material_properties": {}}]))


def test_triclinic_parameters_symmetric():
    from fans_gb300.materials import MaterialManager

    keys = ["K_11", "K_12", "K_13", "K_22", "K_23", "K_33"]
    props = {k: [float(i + 1)] for i, k in enumerate(keys)}
    mm = MaterialManager(_mm_json([{"phases": [0], "matmodel": "LinearThermalTriclinic",
                                    "material_properties": props}]))
    K = np.array(mm.params[0]).reshape(3, 3)
    assert np.allclose(K, K.T) and K[0, 1] == 2.0 and K[2, 2] == 6.0


def test_sphere_generator_counts():
    from fans_gb300.microstructure import spheres

    ms, c = spheres(32, 4, 0.2, seed=0)
    assert len(c) == 24 and ms.dtype == np.uint8
    ms2, c2 = spheres(32, 4, 0.2, seed=0)
    assert np.array_equal(ms, ms2)
    assert 0.17 < ms.mean() < 0.23


def test_struct_layouts_match_a_c_compiler(tmp_path):
    """fansgpu_desc / fansgpu_tol / fansgpu_stats as gcc lays them out from
    include/fans_gb300.h (sizes and every field offset) equal the ctypes mirror
    the Python binding passes."""
    import shutil
    import subprocess

    from fans_gb300 import _lib

    cc = shutil.which("gcc")
    if cc is None:
        pytest.skip("gcc not available")
    structs = {"fansgpu_desc": _lib.Desc, "fansgpu_tol": _lib.Tol, "fansgpu_stats": _lib.Stats}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "fans_gb300.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {}
    for ln in out:
        if ln:
            parts = ln.split()
            got[tuple(parts[:-1])] = int(parts[-1])
    for cname, py in structs.items():
        assert got[(cname, "size")] == ctypes.sizeof(py), cname
        for fname, _ in py._fields_:
            assert got[(cname, fname)] == getattr(py, fname).offset, (cname, fname)
