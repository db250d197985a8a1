"""Builds the oracle fixtures of the two workloads too large to run the oracle
inside a test: the elastic 256^3 effective stiffness and the J2 128^3 load path.

TEST INFRASTRUCTURE ONLY: runs the FP64 C oracle (oracle/fans_oracle.c, the
restatement of FANS's SolverCG, solverCG.h:62-160, and its laws) on the host
cores and writes small JSON fixtures that the GPU tests compare against.

* elastic256 -> elastic256_ceff.json: 256^3 periodic spheres (seed 0, r 6,
  vf 0.30), E/nu 3/0.35 and 70/0.22 (K, G as below), HEX8, the six unit Mandel
  load cases of Solver::get_homogenized_tangent's linear branch
  (solver.h:759-776) solved one by one with CG to L2 relative 1e-8 from u = 0.
  Records the 6x6 C_eff (unsymmetrised columns), the iteration count and the
  wall time of each load case, the thread count and the CPU model.
* j2_128 -> j2_128_curve.json: 128^3 spheres (seed 4, r 8, vf 0.25), matrix
  J2PlasticityNew with linear isotropic hardening (K 68.6275, G 26.3158, yield
  0.25, hardening 2), elastic inclusions (K 222.222, G 166.667), eps_11 =
  0.0005 k for k = 1..20, nonlinear CG with LineSearchSecant to Linfinity 1e-10
  absolute, extrapolateDisplacement between steps (src/main.cpp:22-39).
  Records <sigma> after every step and the iteration counts.

Usage, from the repository root:  python tests/golden/make_workload_fixtures.py
elastic256|j2_128 [--threads N]
"""
import argparse
import json
import os
import platform
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle as O  # noqa: E402
from fans_gb300.microstructure import spheres  # noqa: E402

ELASTIC = [(O.LAW_ELASTIC_ISO, [0, 1], [[3.3333333333333335, 1.1111111111111112],
                                        [41.666666666666664, 28.688524590163933]])]
J2 = [(O.LAW_J2, [0], [[68.6275, 26.3158, 0.25, 2.0]]), (O.LAW_ELASTIC_ISO, [1], [[222.222, 166.667]])]


def cpu_model():
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return platform.processor() or platform.machine()


def elastic256(out):
    ms, centres = spheres(256, 6, 0.30, 0)
    P = O.OracleProblem(ms.astype(np.uint16), (1.0, 1.0, 1.0), 3, ELASTIC, "HEX8")
    t0 = time.time()
    _ = P.G  # Green's table, built once (the reference builds it per Solver)
    t_green = time.time() - t0
    C = np.zeros((6, 6))
    iters, secs = [], []
    for i in range(6):
        g = np.zeros(6)
        g[i] = 1.0
        P.u[...] = 0.0
        P.set_gradient(g)
        t0 = time.time()
        it = P.solve(measure="L2", type="relative", tol=1e-8, n_it=2000)
        secs.append(time.time() - t0)
        C[:, i] = P.homogenized_stress()
        iters.append(int(it))
        print(f"load case {i}: {it} iterations, {secs[-1]:.1f} s", flush=True)
    res = {"workload": "256^3 two-phase elastic HEX8, 6 unit load cases, CG rel L2 1e-08",
           "seed": 0, "radius": 6, "vf_target": 0.30, "vf": float(ms.mean()), "spheres": int(len(centres)),
           "C_eff_columns": C.tolist(), "iterations": iters, "solve_seconds": secs, "green_seconds": t_green,
           "threads": O.num_threads(), "cpu": cpu_model(), "machine": platform.machine()}
    with open(out, "w") as f:
        json.dump(res, f, indent=1)
    print(json.dumps({k: res[k] for k in ("iterations", "solve_seconds", "threads", "cpu")}))


def j2_128(out):
    ms, centres = spheres(128, 8, 0.25, 4)
    P = O.OracleProblem(ms.astype(np.uint16), (1.0, 1.0, 1.0), 3, J2, "HEX8")
    sig, iters, secs = [], [], []
    for k in range(1, 21):
        g = np.zeros(6)
        g[0] = 0.0005 * k
        P.set_gradient(g)
        t0 = time.time()
        it = P.solve(measure="Linfinity", type="absolute", tol=1e-10, n_it=2000)
        secs.append(time.time() - t0)
        sig.append(P.homogenized_stress().tolist())
        iters.append(int(it))
        P.extrapolate_displacement()
        print(f"step {k}: {it} iterations, {secs[-1]:.1f} s, sigma_11 {sig[-1][0]:.10f}", flush=True)
    res = {"workload": "J2 128^3, eps_11 = 0.0005 k, k = 1..20, nonlinear CG, Linfinity 1e-10 absolute",
           "seed": 4, "radius": 8, "vf_target": 0.25, "vf": float(ms.mean()), "spheres": int(len(centres)),
           "strain_11": [0.0005 * k for k in range(1, 21)], "stress": sig, "iterations": iters,
           "solve_seconds": secs, "threads": O.num_threads(), "cpu": cpu_model(), "machine": platform.machine()}
    with open(out, "w") as f:
        json.dump(res, f, indent=1)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("which", choices=["elastic256", "j2_128"])
    ap.add_argument("--threads", type=int, default=0)
    ap.add_argument("--out", default=None)
    a = ap.parse_args()
    if a.threads:
        O.set_threads(a.threads)
    name = {"elastic256": "elastic256_ceff.json", "j2_128": "j2_128_curve.json"}[a.which]
    out = a.out or os.path.join(HERE, name)
    (elastic256 if a.which == "elastic256" else j2_128)(out)


if __name__ == "__main__":
    main()
