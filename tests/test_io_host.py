"""Host-side I/O of the FANS driver (no GPU): the HDF5 reader and writer in
fans_gb300/h5.py, the input-file Reader (reader.cpp:62-187) and the results-file
layout of Reader::writeData / writeSlab (reader.h:170-351)."""
import json
import os

import numpy as np
import pytest

from fans_gb300 import h5
from fans_gb300.reader import MixedBC, Reader

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
# a FANS checkout named by the FANS_REFERENCE environment variable (optional): its
# test/microstructures/sphere32.h5 is the file the committed fixture was decoded from
REF_H5 = os.path.join(os.environ.get("FANS_REFERENCE", ""), "test", "microstructures", "sphere32.h5")


def test_sphere32_fixture_metadata():
    ms = np.load(os.path.join(GOLDEN, "sphere32_ms.npy"))
    meta = json.load(open(os.path.join(GOLDEN, "sphere32.json")))
    assert ms.shape == (32, 32, 32) and ms.dtype == np.uint8
    assert set(np.unique(ms)) == {0, 1}
    assert ms.mean() == pytest.approx(meta["volume_fraction_phase1"])
    assert ms.mean() == pytest.approx(0.2668, abs=1e-4)  # 26.7 % inclusion


@pytest.mark.skipif(not os.environ.get("FANS_REFERENCE") or not os.path.exists(REF_H5),
                    reason="FANS_REFERENCE does not name a FANS checkout")
def test_reader_decodes_chunked_deflate_fixture():
    f = h5.H5File(REF_H5)
    assert f.keys("/") == ["sphere"]
    raw = f.read("/sphere/32x32x32/ms")
    assert raw.dtype == np.uint8 and raw.shape == (32, 32, 32)
    ms = h5.read_microstructure(REF_H5, "/sphere/32x32x32/ms")
    assert np.array_equal(ms, np.transpose(raw, (2, 1, 0)))
    assert np.array_equal(ms, np.load(os.path.join(GOLDEN, "sphere32_ms.npy")))


def test_writer_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    a = rng.random((5, 4, 3))
    b = rng.integers(0, 255, (6, 7, 8), dtype=np.uint8)
    c = rng.integers(-5, 5, (3, 2), dtype=np.int32)
    p = tmp_path / "t.h5"
    with h5.H5Writer(str(p)) as w:
        w.dataset("/g/h/a", a, {"permute_order": "zyx"})
        w.dataset("/g/b", b)
        w.dataset("/g//c", c)  # empty path element, as "<ds>_results//load0" has
        for i in range(40):  # several symbol-table nodes in one group
            w.dataset(f"/many/load{i}/v", np.arange(i + 1, dtype=np.float64))
        w.dataset("/g/b", b + 1)  # replace, as WriteData does
        w.dataset("/f32", np.float32([1.5, -2.0]))
    f = h5.H5File(str(p))
    assert f.keys("/") == ["f32", "g", "many"]
    assert f.keys("/g") == ["b", "c", "h"]
    assert np.array_equal(f.read("/g/h/a"), a)
    assert np.array_equal(f.read("/g/b"), b + 1)
    assert np.array_equal(f.read("/g/c"), c)
    assert f.read("/f32").dtype == np.float32
    assert f.attrs("/g/h/a")["permute_order"] == b"zyx"
    for i in range(40):
        assert np.array_equal(f.read(f"/many/load{i}/v"), np.arange(i + 1.0))
    # a file our writer made is also a valid microstructure source
    q = tmp_path / "ms.h5"
    ms = rng.integers(0, 3, (6, 5, 4)).astype(np.uint8)
    with h5.H5Writer(str(q)) as w:
        w.dataset("/m/ms", np.ascontiguousarray(ms.transpose(2, 1, 0)))  # zyx on disk, no attribute
        w.dataset("/m/ms_xyz", ms, {"permute_order": "xyz"})
    assert np.array_equal(h5.read_microstructure(str(q), "/m/ms"), ms)
    assert np.array_equal(h5.read_microstructure(str(q), "/m/ms_xyz"), ms)


def test_writer_output_read_by_h5py(tmp_path):
    """An independent HDF5 implementation (h5py over libhdf5) reads what
    fans_gb300.h5 writes: groups, the empty path element FANS's result paths
    have, float64 / float32 / uint8 / int32 datasets, a replaced dataset and the
    permute_order string attribute of Reader::WriteSlab (reader.h:314-329).
    Skipped where h5py is not installed."""
    h5py = pytest.importorskip("h5py")
    rng = np.random.default_rng(1)
    a = rng.random((5, 4, 3))
    b = rng.integers(0, 255, (6, 7, 8), dtype=np.uint8)
    c = rng.integers(-5, 5, (3, 2), dtype=np.int32)
    p = tmp_path / "t.h5"
    with h5.H5Writer(str(p)) as w:
        w.dataset("/ms_results//load0/time_step0/stress", a, {"permute_order": "zyx"})
        w.dataset("/g/b", b)
        w.dataset("/g/b", b + 1)
        w.dataset("/g/c", c)
        w.dataset("/f32", np.float32([1.5, -2.0]))
        for i in range(40):
            w.dataset(f"/many/load{i}/v", np.arange(i + 1, dtype=np.float64))
    with h5py.File(str(p), "r") as f:
        d = f["/ms_results//load0/time_step0/stress"]
        assert np.array_equal(d[...], a)
        pa = d.attrs["permute_order"]
        assert (pa.decode() if isinstance(pa, bytes) else str(pa)) == "zyx"
        assert np.array_equal(f["/g/b"][...], b + 1) and f["/g/b"].dtype == np.uint8
        assert np.array_equal(f["/g/c"][...], c)
        assert f["/f32"].dtype == np.float32
        assert sorted(f["/many"].keys()) == sorted(f"load{i}" for i in range(40))
        assert np.array_equal(f["/many/load39/v"][...], np.arange(40.0))


def test_reader_parses_reference_inputs():
    inputs = json.load(open(os.path.join(GOLDEN, "reference_inputs.json")))
    r = Reader().ReadInputFile(inputs["test_LinearElastic"])
    assert r.problemType == "mechanical" and r.FE_type == "HEX8R" and r.method == "cg"
    assert r.ms_datasetname == "/sphere/32x32x32/ms"
    assert r.dataset_name == "/sphere/32x32x32/ms_results/"
    assert r.TOL == 1e-10 and r.n_it == 100 and r.errorParameters["measure"] == "Linfinity"
    assert r.extrapolate_displacement is True and r.ls_max_iter == 5 and r.ls_tol == 1e-2
    assert len(r.load_cases) == 1 and r.load_cases[0].n_steps == 1
    assert "homogenized_tangent" in r.resultsToWrite
    r.set_microstructure(np.load(os.path.join(GOLDEN, "sphere32_ms.npy")))
    assert r.dims == [32, 32, 32] and r.n_mat == 2 and r.l_e == [1 / 32] * 3
    t = Reader().ReadInputFile(inputs["test_LinearThermal"])
    assert t.problemType == "thermal" and len(t.load_cases[0].g0_path[0]) == 3


def test_reader_errors_match_reference_messages():
    base = json.load(open(os.path.join(GOLDEN, "reference_inputs.json")))["test_LinearElastic"]
    j = json.loads(json.dumps(base))
    j["FE_type"] = "HEX20"
    with pytest.raises(ValueError, match="FE_type must be one of"):
        Reader().ReadInputFile(j)
    j = json.loads(json.dumps(base))
    j["macroscale_loading"] = [[[1.0, 0.0, 0.0]]]
    with pytest.raises(ValueError, match="expected 6 components but got 3"):
        Reader().ReadInputFile(j)
    j = json.loads(json.dumps(base))
    j["microstructure"]["datasetname"] = ""
    with pytest.raises(ValueError, match="datasetname must not be empty"):
        Reader().ReadInputFile(j)
    j = json.loads(json.dumps(base))
    j["linesearch_parameters"] = {"max_iter": 0}
    with pytest.raises(ValueError, match="max_iter >= 1"):
        Reader().ReadInputFile(j)


def test_mixed_bc_parsing():
    mbc = MixedBC.from_json({"strain_indices": [0, 1, 2, 3, 4], "stress_indices": [5],
                             "strain": [[0.0] * 5, [0.001] * 5], "stress": [[0.0], [0.0]]}, 6)
    assert mbc.F_E_path.shape == (2, 5) and mbc.P_F_path.shape == (2, 1)
    with pytest.raises(RuntimeError, match="both strain_indices and stress_indices"):
        MixedBC.from_json({"strain_indices": [0, 1, 2, 3, 4, 5], "stress_indices": [5], "strain": [[0] * 6],
                           "stress": [[0]]}, 6)
    with pytest.raises(RuntimeError, match="either strain"):
        MixedBC.from_json({"strain_indices": [0, 1], "stress_indices": [5], "strain": [[0, 0]], "stress": [[0]]}, 6)


def test_results_file_layout(tmp_path):
    from fans_gb300.run import ResultsFile

    r = Reader().ReadInputFile(json.load(open(os.path.join(GOLDEN, "reference_inputs.json")))["test_LinearElastic"])
    r.set_microstructure(np.zeros((4, 3, 2), dtype=np.uint8))
    p = str(tmp_path / "out.h5")
    res = ResultsFile(r, p)
    field = np.arange(4 * 3 * 2 * 6, dtype=np.float64).reshape(4, 3, 2, 6)
    res.writeSlab("stress", 0, 0, field, (6,))
    res.writeSlab("not_requested", 0, 0, field, (6,))
    res.writeData("stress_average", 0, 0, np.ones(6))
    res.close()
    f = h5.H5File(p)
    base = "/sphere/32x32x32/ms_results/load0/time_step0"
    assert f.keys(base) == ["stress", "stress_average"]
    s = f.read(base + "/stress")
    assert s.shape == (2, 3, 4, 6)  # Z Y X n_str on disk
    assert np.array_equal(np.swapaxes(s, 0, 2), field)
    assert f.attrs(base + "/stress")["permute_order"] == b"zyx"


def test_cli_usage_and_bad_input(tmp_path, capsys):
    from fans_gb300.run import main

    assert main([]) == 10
    bad = tmp_path / "bad.json"
    bad.write_text("{}")
    assert main([str(bad), str(tmp_path / "o.h5")]) == 10
    assert "ERROR trying to read input file" in capsys.readouterr().err


def test_pyfans_cmat_packing_is_the_upper_triangle_row_by_row():
    from fans_gb300.pyfans import CMAT_ENTRIES

    assert len(CMAT_ENTRIES) == 21 and len(set(CMAT_ENTRIES)) == 21
    assert CMAT_ENTRIES == [(r, c) for r in range(6) for c in range(r, 6)]


def test_vlen_string_attribute_round_trip(tmp_path):
    info = {"g0": {"GB_tag": 5, "GB_normal": [0.0, 0.6, 0.8]}}
    p = str(tmp_path / "gb.h5")
    with h5.H5Writer(p) as w:
        w.dataset("/poly/ms", np.zeros((4, 4, 4), np.uint8),
                  {"num_crystals": np.int64(5), "num_GB": np.int64(1), "GBVoxelInfo": h5.VlenStr(json.dumps(info))})
    a = h5.H5File(p).attrs("/poly/ms")
    assert int(a["num_crystals"]) == 5 and int(a["num_GB"]) == 1
    assert json.loads(a["GBVoxelInfo"]) == info


def test_gb_diffusion_tensors():
    from fans_gb300.materials import MaterialManager, gb_diffusion_tensors

    info = {"num_crystals": 2, "num_GB": 2,
            "GBVoxelInfo": json.dumps({"a": {"GB_tag": 2, "GB_normal": [0, 0, 2.0]},
                                       "b": {"GB_tag": 3, "GB_normal": [1.0, 1.0, 0]}})}
    props = {"GB_unformity": True, "D_bulk": 1.5, "D_par": 4.0, "D_perp": 0.5}
    K, normals = gb_diffusion_tensors(props, info)
    assert np.allclose(np.reshape(K[0], (3, 3)), 1.5 * np.eye(3))
    assert np.allclose(np.reshape(K[2], (3, 3)), np.diag([4.0, 4.0, 0.5]))  # normal z, normalised
    n = np.array([1.0, 1.0, 0]) / np.sqrt(2)
    assert np.allclose(np.reshape(K[3], (3, 3)) @ n, 0.5 * n)
    mm = MaterialManager({"materials": [{"phases": [0, 1, 2, 3], "matmodel": "GBDiffusion",
                                         "material_properties": props}]}, "thermal", info)
    assert mm.law == [3, 3, 3, 3]
    assert np.allclose(mm.kapparef_mat, np.mean([np.reshape(k, (3, 3)) for k in K], axis=0))
    with pytest.raises(ValueError):
        MaterialManager({"materials": [{"phases": [0], "matmodel": "GBDiffusion", "material_properties": props}]},
                        "mechanical", info)
