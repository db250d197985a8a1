"""The FANS driver on the GPU path: runSolver (main.cpp:10-46), the results
file (Reader::writeData / writeSlab, reader.h:88-351) and
Solver::postprocess (solver.h:455-705) with the J2 additions of
J2PlasticityNew::postprocess (J2PlasticityNew.h:160-200).

Every quantity comes from the GPU context through the C ABI; this module only
orders the calls and writes the HDF5 results file.
"""
from __future__ import annotations

import numpy as np

from . import _lib as C
from . import h5
from .materials import MaterialManager
from .reader import Reader
from .solver import create_solver

VERSION = "0.1"


class ResultsFile:
    """Reader::OpenResultsFile / writeData / writeSlab / CloseResultsFile."""

    def __init__(self, reader: Reader, path: str):
        self.reader = reader
        self.w = h5.H5Writer(path)

    def _name(self, field, load_idx, time_idx):
        return f"{self.reader.dataset_name}/load{load_idx}/time_step{time_idx}/{field}"

    def wanted(self, field):
        return field in self.reader.resultsToWrite

    def writeData(self, field, load_idx, time_idx, data):
        """A plain array as given (reader.h:332-340)."""
        if self.wanted(field):
            self.w.dataset(self._name(field, load_idx, time_idx), np.asarray(data))

    def writeSlab(self, field, load_idx, time_idx, data, extra_dims):
        """An [x][y][z][extra...] field stored Z Y X extra... with permute_order
        "zyx" (reader.h:170-253, :343-351)."""
        if not self.wanted(field):
            return
        dims = self.reader.dims
        a = np.asarray(data).reshape(tuple(dims) + tuple(extra_dims))
        a = np.ascontiguousarray(np.swapaxes(a, 0, 2))
        self.w.dataset(self._name(field, load_idx, time_idx), a, {"permute_order": "zyx"})

    def close(self):
        self.w.close()


def postprocess(solver, reader: Reader, results: ResultsFile, load_idx: int, time_idx: int, log=print):
    """Solver::postprocess (solver.h:455-705)."""
    ctx = solver.ctx
    n_str, howmany, n_mat = solver.n_str, solver.howmany, reader.n_mat
    want = results.wanted
    avg = ctx.postprocess_averages(n_mat)
    stress_average, strain_average = avg["stress_average"], avg["strain_average"]
    log("# Effective Stress .. (" + " ".join(f"{v:+.12f}" for v in stress_average) + ") ")
    log("# Effective Strain .. (" + " ".join(f"{v:+.12f}" for v in strain_average) + ") \n")

    # u_total = g0 . X + u~ with X measured from the box centre (solver.h:567-640)
    v_u = ctx.get_field(C.FIELD_U)
    nx, ny, nz = reader.dims
    dx, dy, dz = reader.l_e
    x = np.arange(nx) * dx - reader.L[0] / 2.0
    y = np.arange(ny) * dy - reader.L[1] / 2.0
    z = np.arange(nz) * dz - reader.L[2] / 2.0
    X, Y, Z = np.meshgrid(x, y, z, indexing="ij")
    u_total = v_u.copy()
    if n_str == 9:  # large strain: u = (F - I) X (solver.h:622-640)
        Fm = np.reshape(strain_average, (3, 3)) - np.eye(3)
        for i in range(3):
            u_total[..., i] += Fm[i, 0] * X + Fm[i, 1] * Y + Fm[i, 2] * Z
    elif howmany == 3:
        rs2 = 0.7071067811865475
        g11, g22, g33 = strain_average[0], strain_average[1], strain_average[2]
        g12, g13, g23 = strain_average[3] * rs2, strain_average[4] * rs2, strain_average[5] * rs2
        u_total[..., 0] += g11 * X + g12 * Y + g13 * Z
        u_total[..., 1] += g12 * X + g22 * Y + g23 * Z
        u_total[..., 2] += g13 * X + g23 * Y + g33 * Z
    else:
        u_total[..., 0] += strain_average[0] * X + strain_average[1] * Y + strain_average[2] * Z

    results.writeData("stress_average", load_idx, time_idx, stress_average)
    results.writeData("strain_average", load_idx, time_idx, strain_average)
    for m in range(n_mat):
        results.writeData(f"phase_stress_average_phase{m}", load_idx, time_idx, avg["phase_stress"][m])
        results.writeData(f"phase_strain_average_phase{m}", load_idx, time_idx, avg["phase_strain"][m])
    results.writeData("absolute_error", load_idx, time_idx, ctx.error_history())

    results.writeSlab("mpi_rank", load_idx, time_idx, np.zeros(reader.dims, dtype=np.int32), (1,))
    results.writeSlab("microstructure", load_idx, time_idx, reader.ms.astype(np.uint16), (1,))
    results.writeSlab("displacement_fluctuation", load_idx, time_idx, v_u, (howmany,))
    results.writeSlab("displacement", load_idx, time_idx, u_total, (howmany,))
    if want("residual"):
        results.writeSlab("residual", load_idx, time_idx, ctx.get_field(C.FIELD_R), (howmany,))
    if want("strain"):
        results.writeSlab("strain", load_idx, time_idx, ctx.get_field(C.FIELD_STRAIN), (n_str,))
    if want("stress"):
        results.writeSlab("stress", load_idx, time_idx, ctx.get_field(C.FIELD_STRESS), (n_str,))
    if want("strain_gp"):
        results.writeSlab("strain_gp", load_idx, time_idx, ctx.get_field(C.FIELD_STRAIN_GP), (ctx.n_gp, n_str))
    if want("stress_gp"):
        results.writeSlab("stress_gp", load_idx, time_idx, ctx.get_field(C.FIELD_STRESS_GP), (ctx.n_gp, n_str))

    # MaterialManager::postprocess -> J2PlasticityNew::postprocess (J2PlasticityNew.h:160-200) and
    # J2Plasticity::postprocess (J2Plasticity.h:248-322)
    ivar_laws = (C.LAW_J2_LINEAR, C.LAW_J2VISCO_LINEAR, C.LAW_J2VISCO_NONLINEAR)
    if any(law in ivar_laws for law in solver.matmanager.law):
        if want("plastic_strain"):
            results.writeSlab("plastic_strain", load_idx, time_idx, ctx.get_field(C.FIELD_PLASTIC_STRAIN), (6,))
        if want("plastic_strain_gp"):
            results.writeSlab("plastic_strain_gp", load_idx, time_idx, ctx.get_field(C.FIELD_PLASTIC_STRAIN_GP),
                              (ctx.n_gp, 6))
        if want("isotropic_hardening_variable"):
            results.writeSlab("isotropic_hardening_variable", load_idx, time_idx,
                              ctx.get_field(C.FIELD_HARDENING), (1,))
        if want("isotropic_hardening_variable_gp"):
            results.writeSlab("isotropic_hardening_variable_gp", load_idx, time_idx,
                              ctx.get_field(C.FIELD_HARDENING_GP), (ctx.n_gp,))
        visco = any(law in (C.LAW_J2VISCO_LINEAR, C.LAW_J2VISCO_NONLINEAR) for law in solver.matmanager.law)
        if visco and want("kinematic_hardening_variable"):  # J2Plasticity.h:283-288
            results.writeSlab("kinematic_hardening_variable", load_idx, time_idx, ctx.get_field(C.FIELD_KINEMATIC),
                              (6,))
        if visco and want("kinematic_hardening_variable_gp"):
            results.writeSlab("kinematic_hardening_variable_gp", load_idx, time_idx,
                              ctx.get_field(C.FIELD_KINEMATIC_GP), (ctx.n_gp, 6))

    # PseudoPlastic::postprocess (PseudoPlastic.h:55-63): element mean of the plastic flags, float32
    if want("plastic_flag") and any(law in (C.LAW_PSEUDO_LINEAR, C.LAW_PSEUDO_NONLINEAR)
                                    for law in solver.matmanager.law):
        results.writeSlab("plastic_flag", load_idx, time_idx,
                          ctx.get_field(C.FIELD_PLASTIC_FLAG).astype(np.float32), (1,))

    # GBDiffusion::postprocess (GBDiffusion.h:171-187): the GB normal of each GB voxel
    if want("GBnormals") and solver.matmanager.gb_normals is not None:
        nc = int(reader.gb_info()["num_crystals"])
        normals = np.where((reader.ms >= nc)[..., None], solver.matmanager.gb_normals[reader.ms], 0.0)
        results.writeSlab("GBnormals", load_idx, time_idx, normals, (3,))

    if want("homogenized_tangent"):
        T = solver.get_homogenized_tangent(1e-6)
        log("# Homogenized tangent: \n" + np.array2string(T, precision=12) + "\n")
        results.writeData("homogenized_tangent", load_idx, time_idx, T)
    return avg


def run_solver(reader: Reader, results: ResultsFile, precision="fp64", log=print):
    """runSolver (main.cpp:10-46): one MaterialManager + Solver per load case,
    then per time step set_gradient, solve, postprocess, extrapolate."""
    if reader.ms is None:
        reader.ReadMS()
    out = []
    for li, lc in enumerate(reader.load_cases):
        mm = MaterialManager(reader.inputJson, reader.problemType, reader.gb_info(), reader.strain_type)
        solver = create_solver(reader, mm, precision)
        try:
            log(f"# Load case {li + 1}/{len(reader.load_cases)}: {lc.n_steps} time steps")
            for ti in range(lc.n_steps):
                log(f"#   Time step {ti + 1}/{lc.n_steps} (load case {li + 1}/{len(reader.load_cases)})")
                if lc.mixed:  # main.cpp:29-34
                    solver.enableMixedBC(lc.mbc, ti)
                else:
                    solver.set_gradient(lc.g0_path[ti])
                st = solver.solve()
                avg = postprocess(solver, reader, results, li, ti, log)
                out.append(dict(load=li, step=ti, iterations=st["iterations"], stress=avg["stress_average"].copy(),
                                strain=avg["strain_average"].copy()))
                if reader.extrapolate_displacement:
                    solver.extrapolateDisplacement()
        finally:
            solver.close()
    return out


def main(argv=None, log=print):
    """FANS command line (main.cpp:48-80): `<input.json> <output.h5>`; exit 10 on
    bad usage or an unreadable input file, as the reference does."""
    import sys

    argv = list(sys.argv[1:] if argv is None else argv)
    precision = "fp64"
    if "--precision" in argv:
        i = argv.index("--precision")
        precision = argv[i + 1]
        del argv[i:i + 2]
    if argv and argv[0] == "--version":
        log(f"FANS version {VERSION} (fans_gb300)")
        return 0
    if len(argv) != 2:
        sys.stderr.write("USAGE: fans_gb300 [input file basename] [output file basename] [--precision fp64|mixed]\n")
        return 10
    reader = Reader()
    try:
        reader.ReadInputFile(argv[0])
    except Exception as e:  # reader.cpp:179-182
        sys.stderr.write(f"ERROR trying to read input file '{argv[0]}' for FANS: {e}\n")
        return 10
    if reader.problemType not in ("thermal", "mechanical"):  # main.cpp:64-77
        raise ValueError(f"Invalid problem type: {reader.problemType}")
    results = ResultsFile(reader, argv[1])
    try:
        run_solver(reader, results, precision, log)
    finally:
        results.close()
    return 0
