"""PyFANS.MicroSimulation on the GPU path (pyfans/micro.cpp:27-85, micro.hpp:20-32).

The Micro Manager calls `MicroSimulation(sim_id)` once per micro problem and then
`solve(macro_data, dt)` per coupling step with the macro strain split as
"strains1to3" / "strains4to6"; it gets back the homogenized stress as
"stresses1to3" / "stresses4to6" and the upper triangle of the homogenized
tangent packed row by row into "cmat1" .. "cmat7" (three entries each,
micro.cpp:64-83).  As in the reference, the solver is created once from the
input file (mechanical, small strain), every solve commits internal variables,
and the tangent is the solver's get_homogenized_tangent(1e-6) with its side
effects on the error type and tolerance.
"""
from __future__ import annotations

import numpy as np

from .materials import MaterialManager
from .reader import Reader
from .solver import create_solver

# (row, col) of the 21 upper-triangle entries in cmat1..cmat7 order (micro.cpp:66-82)
CMAT_ENTRIES = [(0, 0), (0, 1), (0, 2), (0, 3), (0, 4), (0, 5), (1, 1), (1, 2), (1, 3), (1, 4), (1, 5), (2, 2),
                (2, 3), (2, 4), (2, 5), (3, 3), (3, 4), (3, 5), (4, 4), (4, 5), (5, 5)]


class MicroSimulation:
    pert_param = 1e-6  # micro.hpp:31

    def __init__(self, sim_id: int, input_file="input.json", precision="fp64"):
        self._sim_id = sim_id
        self.reader = Reader().ReadInputFile(input_file)
        self.reader.ReadMS(3)
        self.matmanager = MaterialManager(self.reader.inputJson, "mechanical")
        self.solver = create_solver(self.reader, self.matmanager, precision)

    def solve(self, macro_data: dict, dt: float = 0.0) -> dict:
        """One coupling step: g0 from the macro strains, solve, stress and tangent."""
        strain = np.concatenate([np.asarray(macro_data["strains1to3"], dtype=float).ravel(),
                                 np.asarray(macro_data["strains4to6"], dtype=float).ravel()])
        self.solver.set_gradient(strain)
        self.solver.solve()
        stress = self.solver.get_homogenized_stress()
        C = self.solver.get_homogenized_tangent(self.pert_param)
        out = {"stresses1to3": [float(v) for v in stress[0:3]], "stresses4to6": [float(v) for v in stress[3:6]]}
        for k in range(7):
            out[f"cmat{k + 1}"] = [float(C[r, c]) for r, c in CMAT_ENTRIES[3 * k:3 * k + 3]]
        return out

    def close(self):
        self.solver.close()


def __getattr__(name):
    """The torch.autograd.Function front ends of the adjoints (fans_gb300.autograd),
    importable from the binding without importing torch for MicroSimulation alone."""
    if name in ("EffectiveStiffness", "YieldPathStress"):
        from . import autograd

        return getattr(autograd, name)
    raise AttributeError(name)
