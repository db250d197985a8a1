"""Reader: the FANS input file and microstructure (reader.h, reader.cpp).

`Reader.ReadInputFile` follows Reader::ReadInputFile (reader.cpp:62-187): the
same keys, defaults and validation messages; `Reader.ReadMS` follows
Reader::ReadMS (reader.cpp:227-411) through the HDF5 reader in h5.py, and
`ComputeVolumeFractions` reader.cpp:12-60.  Errors raise the exception types
the reference throws (the reference's catch-all turns them into exit(10),
which the command-line driver in __main__.py mirrors).
"""
from __future__ import annotations

import json
import os
from dataclasses import dataclass, field

import numpy as np

from . import h5


@dataclass
class MixedBC:
    """MixedBC (mixedBCs.h:15-131): strain- and stress-controlled component
    index sets and their per-step paths."""

    idx_E: list
    idx_F: list
    F_E_path: np.ndarray  # n_steps x |E|
    P_F_path: np.ndarray  # n_steps x |F|

    @staticmethod
    def from_json(jc, n_str):
        """MixedBC::from_json (mixedBCs.h:51-131), same checks and messages."""
        if "strain_indices" not in jc or "stress_indices" not in jc:
            raise RuntimeError("mixed BC: strain_indices or stress_indices missing")
        idx_E = [int(v) for v in jc["strain_indices"]]
        idx_F = [int(v) for v in jc["stress_indices"]]
        present = [False] * n_str
        for k in idx_E:
            if k < 0 or k >= n_str:
                raise RuntimeError("strain index out of range")
            present[k] = True
        for k in idx_F:
            if k < 0 or k >= n_str:
                raise RuntimeError("stress index out of range")
            if present[k]:
                raise RuntimeError("index appears in both strain_indices and stress_indices")
            present[k] = True
        if not all(present):
            raise RuntimeError("each component must be either strain\u2011 or stress\u2011controlled")
        strain_raw, stress_raw, n_steps = [], [], 0
        if idx_E:
            if "strain" not in jc:
                raise RuntimeError("strain array missing")
            strain_raw = jc["strain"]
            n_steps = len(strain_raw)
        if idx_F:
            if "stress" not in jc:
                raise RuntimeError("stress array missing")
            stress_raw = jc["stress"]
            n_steps = max(n_steps, len(stress_raw))
        if n_steps == 0:
            raise RuntimeError("mixed BC: at least one of strain/stress must have timesteps")
        strain_raw = strain_raw or [[] for _ in range(n_steps)]
        stress_raw = stress_raw or [[] for _ in range(n_steps)]
        FE, PF = np.zeros((n_steps, len(idx_E))), np.zeros((n_steps, len(idx_F)))
        for t in range(n_steps):
            if t >= len(strain_raw) or len(strain_raw[t]) != len(idx_E):
                raise RuntimeError("strain row length mismatch")
            FE[t] = strain_raw[t]
            if t >= len(stress_raw) or len(stress_raw[t]) != len(idx_F):
                raise RuntimeError("stress row length mismatch")
            PF[t] = stress_raw[t]
        return MixedBC(idx_E, idx_F, FE, PF)


@dataclass
class LoadCase:
    """One entry of macroscale_loading (mixedBCs.h:137-142)."""

    mixed: bool = False
    g0_path: list = field(default_factory=list)  # n_steps x n_str (pure strain / gradient control)
    mbc: MixedBC | None = None
    n_steps: int = 0


class Reader:
    def __init__(self):
        self.inputJson = {}
        self.ms_filename = ""
        self.ms_datasetname = ""
        self.L = [1.0, 1.0, 1.0]
        self.results_prefix = ""
        self.dataset_name = ""
        self.errorParameters = {}
        self.TOL = 0.0
        self.n_it = 0
        self.extrapolate_displacement = True  # reader.h:35
        self.ls_max_iter = 5                  # reader.h:33
        self.ls_tol = 1e-2                    # reader.h:34
        self.problemType = ""
        self.method = ""
        self.strain_type = "small"
        self.FE_type = "HEX8"
        self.resultsToWrite = []
        self.load_cases: list[LoadCase] = []
        self.dims = None
        self.l_e = None
        self.ms = None
        self.n_mat = 0
        self.is_zyx = True
        self.base_dir = "."

    # -- reader.cpp:62-187 --
    def ReadInputFile(self, input_fn):
        if isinstance(input_fn, dict):
            j = input_fn
        else:
            with open(input_fn) as f:
                j = json.load(f)
            self.base_dir = os.path.dirname(os.path.abspath(input_fn))
        self.inputJson = j
        micro = j["microstructure"]
        self.ms_filename = micro["filepath"]
        ds = micro["datasetname"]
        if not ds:
            raise ValueError("datasetname must not be empty and must refer to a valid HDF5 path")
        self.ms_datasetname = ds if ds.startswith("/") else "/" + ds
        self.L = [float(v) for v in micro["L"]]
        self.results_prefix = j.get("results_prefix", "")
        self.dataset_name = f"{self.ms_datasetname}_results/{self.results_prefix}"
        self.errorParameters = dict(j["error_parameters"])
        self.TOL = float(self.errorParameters["tolerance"])
        self.n_it = int(j["n_it"])
        self.extrapolate_displacement = bool(j.get("extrapolate_displacement", self.extrapolate_displacement))
        if "linesearch_parameters" in j:
            lp = j["linesearch_parameters"]
            self.ls_max_iter = int(lp.get("max_iter", self.ls_max_iter))
            self.ls_tol = float(lp.get("tol", self.ls_tol))
            if self.ls_max_iter < 1 or self.ls_tol <= 0.0:
                raise ValueError("linesearch_parameters: max_iter >= 1 and tol > 0 required")
        self.problemType = j["problem_type"]
        self.method = j["method"]
        self.strain_type = j.get("strain_type", "small")
        if self.strain_type not in ("small", "large"):
            raise ValueError("strain_type must be either 'small' or 'large'")
        self.FE_type = j.get("FE_type", "HEX8")
        if self.FE_type not in ("HEX8", "HEX8R", "BBAR"):
            raise ValueError("FE_type must be one of: 'HEX8', 'HEX8R', or 'BBAR'")
        self.resultsToWrite = list(j["results"])
        ml = j["macroscale_loading"]
        if not isinstance(ml, list):
            raise RuntimeError("macroscale_loading must be an array")
        if self.problemType == "thermal":
            n_str = 3
        elif self.strain_type == "large":
            n_str = 9
        else:
            n_str = 6
        self.load_cases = []
        for entry in ml:
            if isinstance(entry, list):
                path = [[float(v) for v in step] for step in entry]
                if len(path[0]) != n_str:
                    raise ValueError(f"Invalid length of loading vector: expected {n_str} components but got "
                                     f"{len(path[0])}")
                self.load_cases.append(LoadCase(False, path, None, len(path)))
            else:
                mbc = MixedBC.from_json(entry, n_str)
                self.load_cases.append(LoadCase(True, [], mbc, mbc.F_E_path.shape[0]))
        return self

    # -- reader.cpp:227-411 --
    def ReadMS(self, hm=None):
        path = self.ms_filename
        if not os.path.isabs(path):
            cand = os.path.join(self.base_dir, path)
            path = cand if os.path.exists(cand) else path
        f = h5.H5File(path)
        ms = f.read(self.ms_datasetname)
        if ms.ndim != 3:
            raise RuntimeError(f"[ReadMS] dataset {self.ms_datasetname} is not 3-D")
        attrs = f.attrs(self.ms_datasetname)
        self.is_zyx = True
        if "permute_order" in attrs:
            o = attrs["permute_order"]
            o = o.decode() if isinstance(o, (bytes, np.bytes_)) else str(o)
            self.is_zyx = o[:1] in ("z", "Z")
        if self.is_zyx:
            ms = np.transpose(ms, (2, 1, 0))
        self.set_microstructure(ms)
        return self

    def gb_info(self):
        """num_crystals, num_GB and GBVoxelInfo of the microstructure dataset (the
        attributes GBDiffusion reads, GBDiffusion.h:50-60), or None."""
        if getattr(self, "_gb_info", None) is not None:
            return self._gb_info
        path = self.ms_filename
        if not os.path.isabs(path) and os.path.exists(os.path.join(self.base_dir, path)):
            path = os.path.join(self.base_dir, path)
        if not os.path.exists(path):
            return None
        attrs = h5.H5File(path).attrs(self.ms_datasetname)
        if "num_crystals" not in attrs:
            return None
        self._gb_info = {k: attrs[k] for k in ("num_crystals", "num_GB", "GBVoxelInfo")}
        return self._gb_info

    def set_microstructure(self, ms):
        """Install an [x][y][z] phase array directly (the ReadMS result)."""
        ms = np.ascontiguousarray(ms).astype(np.uint16)  # H5T_NATIVE_USHORT (reader.cpp:259)
        self.ms = ms
        self.dims = list(ms.shape)
        self.l_e = [self.L[i] / float(self.dims[i]) for i in range(3)]  # reader.cpp:293-296
        self.ComputeVolumeFractions()
        return self

    def ComputeVolumeFractions(self):
        lo, hi = int(self.ms.min()), int(self.ms.max())
        self.n_mat = hi - lo + 1
        counts = np.bincount(self.ms.ravel().astype(np.int64) - lo, minlength=self.n_mat)
        self.volume_fractions = {lo + i: counts[i] / self.ms.size for i in range(self.n_mat)}
        return self.volume_fractions
