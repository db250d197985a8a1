"""The drop-in boundary from C++: tests/cpp/solver_gpu_demo.cpp, a consumer of
include/fans_gb300_solver.hpp (the SolverGPU class a FANS build selects in
createSolver, include/setup.h:76-85, with the Solver surface of
include/solver.h:11-103), is compiled with g++ against include/fans_gb300.h,
linked to libfans_gb300.so and run on a 16^3 two-phase elastic problem.

Its load cases (solve, get_homogenized_stress, extrapolateDisplacement, as
runSolver does, src/main.cpp:22-39) match the FP64 oracle's <sigma> to 1e-10
relative, its get_homogenized_tangent (unit-gradient solves at relative 1e-6,
solver.h:740-778) matches the oracle's unit-load tangent to 1e-5, and a bad
FE_type is rejected as std::invalid_argument."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from helpers import ELASTIC, oracle_problem, random_ms, rel

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "solver_gpu_demo.cpp")


def _compile(out, link):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not available")
    cmd = [cxx, "-std=c++17", "-O1", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), SRC]
    if link:
        libdir = os.path.join(ROOT, "fans_gb300")
        cmd += ["-o", out, "-L", libdir, "-lfans_gb300", f"-Wl,-rpath,{libdir}"]
    else:
        cmd += ["-fsyntax-only"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)


def test_cpp_binding_compiles(tmp_path):
    """No GPU needed: the header and its consumer compile warning-free."""
    _compile(str(tmp_path / "demo"), link=False)


@pytest.mark.gpu
def test_cpp_binding_solves_like_the_oracle(tmp_path):
    from fans_gb300 import _lib

    _lib.load()  # builds the library if it is missing
    exe = str(tmp_path / "demo")
    _compile(exe, link=True)
    shape = (16, 16, 16)
    ms = random_ms(shape, vf=0.3, seed=41)
    P = oracle_problem(ms, 3, ELASTIC, "HEX8")
    loads = [np.array([1.0, 0, 0, 0, 0, 0]), np.array([0.3, -0.2, 0.1, 0.05, -0.04, 0.02])]
    lines = ["16 16 16", "HEX8 fp64 cg L2 relative 1e-12 2000", str(P.nphase)]
    for ph in range(P.nphase):
        lines.append(f"{int(P.law[ph])} 2 {float(P.param[ph, 0])!r} {float(P.param[ph, 1])!r}")
    lines.append(" ".join(repr(float(v)) for v in np.asarray(P.kapparef).ravel()))
    lines.append(str(len(loads)))
    lines += [" ".join(repr(float(v)) for v in g) for g in loads]
    lines.append(" ".join(str(int(v)) for v in ms.ravel()))
    inp = tmp_path / "in.txt"
    inp.write_text("\n".join(lines) + "\n")
    res = subprocess.run([exe, str(inp)], capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stderr
    out = {}
    for ln in res.stdout.splitlines():
        parts = ln.split()
        if parts[0] == "stress":
            out[("stress", int(parts[1]))] = np.array([float(v) for v in parts[2:]])
        elif parts[0] == "tangent":
            out["tangent"] = np.array([float(v) for v in parts[1:]]).reshape(6, 6)
    assert "invalid_argument ok" in res.stdout
    for k, g in enumerate(loads):
        P.set_gradient(g)
        P.solve(measure="L2", type="relative", tol=1e-12, n_it=2000)
        assert rel(out[("stress", k)], P.homogenized_stress()) < 1e-10, k
        P.extrapolate_displacement()
    P.u[...] = 0.0
    C_ref = P.homogenized_tangent_unit(measure="L2", type="relative", tol=1e-10, n_it=2000)
    assert rel(out["tangent"], C_ref) < 1e-5
