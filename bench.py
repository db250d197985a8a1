"""Benchmark of the GB300 FANS solve path on its headline workload.

Workload (one step): 256^3 two-phase linear-elastic homogenization -- periodic
non-overlapping spheres (seed 0, radius 6 voxels, 30 % volume fraction;
matrix E=3 GPa nu=0.35, inclusions E=70 GPa nu=0.22), HEX8 elements, six unit
Mandel strain load cases, flexible CG with the FFT Green's preconditioner to
relative L2 residual 1e-8 -> the 6x6 effective stiffness.  A step rebuilds the
Green's operator (as FANS does per Solver) and runs the six solves.

The six load cases run as one multi-RHS solve (a context with n_rhs = 6;
--rhs 1 solves them one after another in a single-RHS context instead).

  value : ms per step, mixed precision, inputs resident in HBM, CUDA events on
          the solver's stream (fields are ~0.2-0.4 GB each: inputs larger than L2)
  e2e   : the same through the C ABI from pinned host buffers (microstructure
          upload + parameters in, 6x6 stiffness and per-iteration scalars out)
  fp64  : the all-FP64 GPU path on the same step
  cpu_baseline: the oracle (FP64 C restatement of the reference's algorithm,
          OpenMP, all host cores): setup + a bounded number of CG iterations of
          one load case, per-iteration time x the oracle's own iteration counts
          of the full 256^3 solve (tests/golden/elastic256_ceff.json) -- an
          estimate, labelled so;
  --impl reference: the oracle's complete solve of all six load cases on the
          host cores, timed once (one step, iteration counts from that run).

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference] [--n 256] [--rhs 6]
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "256^3 elastic solve ms to 1e-8: mixed vs FP64 GPU vs CPU; kernel HBM GB/s"
MAT = [[3.3333333333333335, 1.1111111111111112], [41.666666666666664, 28.688524590163933]]  # (K, G) from (E, nu)
HBM_FALLBACK_GBS = 6800.0
ORACLE_256 = os.path.join(ROOT, "tests", "golden", "elastic256_ceff.json")  # the oracle's full 256^3 solve


def oracle_256():
    try:
        with open(ORACLE_256) as f:
            return json.load(f)
    except Exception:
        return None


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--tol", type=float, default=1e-8)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 GPU path")
    ap.add_argument("--cpu-iters", type=int, default=8)
    ap.add_argument("--rhs", type=int, default=6, choices=[1, 6],
                    help="6: the load cases as one multi-RHS solve; 1: one after another")
    ap.add_argument("--workload", default="headline", choices=["headline", "batch64"],
                    help="batch64: 64 independent micro problems, sequential vs fansgpu_solve_batch (own JSON line)")
    return ap.parse_args()


def kapparef():
    """LinearElasticIsotropic reference: (max+min)/2 of lambda and mu (LinearElastic.h:55-70)."""
    from fans_gb300.materials import group_reference_stiffness

    return group_reference_stiffness(1, MAT)


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return HBM_FALLBACK_GBS, "fallback"


def traffic_table():
    """Per-launch DRAM bytes from committed ncu summaries: lines
    'TRAFFIC <kernel> <n> <rhs per launch> <bytes>' (key (kernel, n, rhs))."""
    out = {}
    pdir = os.path.join(ROOT, "profiles")
    if not os.path.isdir(pdir):
        return out
    for fn in os.listdir(pdir):
        if not fn.endswith((".md", ".txt")):
            continue
        for line in open(os.path.join(pdir, fn)):
            parts = line.strip().strip("`").split()
            if len(parts) == 5 and parts[0] == "TRAFFIC":
                out[(parts[1], int(parts[2]), int(parts[3]))] = float(parts[4])
    return out


def algo_bytes(kernel, n, C=3, w=4, r=1.0):
    """Algorithmic (compulsory) DRAM bytes of one launch of `kernel` on an n^3 grid
    with C components of w-byte values (w=4: mixed precision inner loop) covering
    r right-hand sides on average (the iteration kernels of the multi-RHS solve;
    the refresh kernels run per RHS).  Per voxel and RHS the operator reads s,
    d_old and writes d, K d (4 C w) and reads the phase id (1 byte, once per
    launch); the x pass reads the Green's table once per launch."""
    N = n ** 3
    nzh = n // 2 + 1
    spec = C * n * n * nzh * 2 * w  # half spectrum, complex, one RHS
    nt = C * (C + 1) // 2
    return {
        "stencil": r * 4 * C * w * N + N,               # read s, d_old; write d, Kd; phases once
        "fft_z_fwd": r * (C * w * N + spec),            # read r, write spectrum
        "fft_y_fwd": r * 2 * spec,
        "fft_x_green": r * 2 * spec + nt * n * n * nzh * w,  # + Green's table, once
        "fft_y_inv": r * 2 * spec,
        # read spectrum (+ r where <r, s> is taken from r and s), write s; on the FP32 path
        # <r, s> comes from the spectra in the x pass unless FANSGPU_SPECTRAL_DOT=0
        "fft_z_inv": r * (spec + (1 if w == 4 and SPECTRAL_DOT else 2) * C * w * N),
        "cg_update": r * 7 * C * w * N,                 # read r, Kd, e, d, s; write r, e (FP32)
        "residual64": (2 * 8 * C + 1) * N,
        "norm": (8 * C + 4 * C) * N,
        "strain_stress": (8 * C + 1) * N,
    }.get(kernel)


SPECTRAL_DOT = os.environ.get("FANSGPU_SPECTRAL_DOT", "1") != "0"

ITER_KERNELS = ("stencil", "fft_z_fwd", "fft_y_fwd", "fft_x_green", "fft_y_inv", "fft_z_inv", "cg_update")


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.f = tempfile.NamedTemporaryFile("w+", delete=False, suffix=".csv")
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.flush()
        rows = []
        with open(self.f.name) as fh:
            for line in fh:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.f.name)
        if not rows:
            return None
        dev0 = rows[0][0]
        rows = [r for r in rows if r[0] == dev0]
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for k, name in enumerate(names):
                if r[5 + k].lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def max_over_ranks(value, dist=None, device="cpu"):
    """The job's figure for a time-like per-rank value: N independent replicas
    (one process per GPU) finish when the slowest rank does, so the max over
    ranks.  `dist` is torch.distributed when the process group is up, else None."""
    if dist is None:
        return float(value)
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def fp64_rate():
    import ctypes

    from fans_gb300 import _lib

    v = ctypes.c_double(0.0)
    rc = _lib.load().fansgpu_fp64_fma_rate(ctypes.byref(v))
    return v.value if rc == 0 else None


def cpu_model():
    """The host CPU as /proc/cpuinfo names it (model name, or the Arm implementer/part ids)."""
    try:
        info = open("/proc/cpuinfo").read()
    except OSError:
        return platform.machine()
    for key in ("model name", "Model"):
        for line in info.splitlines():
            if line.startswith(key) and ":" in line:
                return line.split(":", 1)[1].strip()
    ids = [line.split(":", 1)[1].strip() for line in info.splitlines()
           if line.startswith(("CPU implementer", "CPU part")) and ":" in line][:2]
    return f"{platform.machine()} (implementer/part {'/'.join(ids)})" if ids else platform.machine()


def build_problem(n, seed=0):
    from fans_gb300.microstructure import spheres

    ms, centres = spheres(n, 6, 0.30, seed)
    return ms, len(centres)


def make_ctx(ms, n, precision, tol, n_rhs=1):
    from fans_gb300 import Context

    ctx = Context((n, n, n), (1.0, 1.0, 1.0), 3, "HEX8", precision, "cg", n_rhs=n_rhs)
    ctx.set_microstructure(ms)
    for ph in range(2):
        ctx.set_phase_material(ph, 1, MAT[ph])
    ctx.set_reference(kapparef())
    ctx.set_tolerance("L2", "relative", tol, 2000)
    return ctx


def homogenize(ctx, kref, stats=None):
    """One step: Green's operator rebuild + six unit-strain solves -> C_eff (6x6).
    A context with six right-hand sides solves them as one multi-RHS solve."""
    ctx.set_reference(kref)
    if ctx.n_rhs == 6:
        ctx.reset()
        ctx.set_gradients(np.eye(6))
        st = ctx.solve()
        if not st["converged"]:
            raise RuntimeError(f"multi-RHS solve did not converge: {st}")
        if stats is not None:
            stats.extend(ctx.rhs_stats(k) for k in range(6))
        Ceff = ctx.homogenized_stresses().T  # column i: <sigma> of load case i
        return 0.5 * (Ceff + Ceff.T)
    Ceff = np.zeros((6, 6))
    for i in range(6):
        ctx.reset()
        g = np.zeros(6)
        g[i] = 1.0
        ctx.set_gradient(g)
        st = ctx.solve()
        if not st["converged"]:
            raise RuntimeError(f"load case {i} did not converge: {st}")
        if stats is not None:
            stats.append(st)
        Ceff[:, i] = ctx.homogenized_stress()
    return 0.5 * (Ceff + Ceff.T)


def timed_steps(ctx, steps, fn):
    import torch

    s = torch.cuda.ExternalStream(ctx.stream())
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(s)
    out = None
    for _ in range(steps):
        out = fn()
    e1.record(s)
    e1.synchronize()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1), out


def cpu_baseline(ms, n, iters, threads=None):
    """Oracle (FP64 C restatement, OpenMP) on a bounded sample of the workload:
    setup (B, K, Green's table) + `iters` CG iterations of load case 0."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    O.build()
    if threads:
        O.set_threads(threads)
    cores = O.num_threads()
    t0 = time.perf_counter()
    P = O.OracleProblem(ms.astype(np.uint16), (1, 1, 1), 3, [(O.LAW_ELASTIC_ISO, [0, 1], MAT)], "HEX8")
    _ = P.G
    t_setup = time.perf_counter() - t0
    P.set_gradient(np.eye(6)[0])
    t1 = time.perf_counter()
    P.solve(measure="L2", type="relative", tol=1e-30, n_it=iters)
    t_solve = time.perf_counter() - t1
    # the solve sample = initial residual + `iters` iterations; charge it all to iterations
    return {"setup_s": t_setup, "per_iter_s": t_solve / max(1, iters), "cores": cores,
            "sample_s": t_setup + t_solve}


def oracle_solve_all(ms, n, tol, cases=6):
    """The oracle's complete solve of the workload as FANS runs it (src/main.cpp:14-41):
    per load case a new Solver -- Green's table built again -- and CG from u = 0 to
    relative L2 `tol`.  Returns wall seconds, iterations, C_eff columns, cores."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    O.build()
    cores = O.num_threads()
    t0 = time.perf_counter()
    P = O.OracleProblem(ms.astype(np.uint16), (1, 1, 1), 3, [(O.LAW_ELASTIC_ISO, [0, 1], MAT)], "HEX8")
    iters, C = [], np.zeros((6, 6))
    for i in range(cases):
        P._G = None  # the Solver constructor's computeFundamentalSolution (solver.h:145-204)
        P.u[...] = 0.0
        P.set_gradient(np.eye(6)[i])
        iters.append(int(P.solve(measure="L2", type="relative", tol=tol, n_it=2000)))
        C[:, i] = P.homogenized_stress()
    return {"seconds": time.perf_counter() - t0, "iterations": iters, "C": C, "cores": cores}


def run_reference(args):
    """The reference arm: the oracle's complete solve of all six load cases, timed
    once on all host cores.  One step is the whole workload (about ten minutes of
    CPU time at 256^3), so the arm runs it once whatever --steps / --warmup ask and
    reports steps = 1, warmup = 0."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    n = args.n
    ms, nsph = build_problem(n)
    res = oracle_solve_all(ms, n, args.tol)
    value_ms = 1e3 * res["seconds"]
    C = 0.5 * (res["C"] + res["C"].T)
    fx = oracle_256() if n == 256 else None
    check = None
    if fx is not None:
        Cf = np.array(fx["C_eff_columns"])
        Cf = 0.5 * (Cf + Cf.T)
        check = float(np.linalg.norm(C - Cf) / np.linalg.norm(Cf))
    sample = (f"complete FP64 solve of the six load cases at {n}^3 to rel L2 {args.tol} (one Green's table per "
              f"load case, as FANS builds one Solver per load case), {res['cores']} threads, iterations "
              f"{res['iterations']} from this run")
    line = {"impl": "reference", "metric": METRIC, "value": round(value_ms, 1), "unit": "ms", "n_gpus": 0,
            "steps": 1, "warmup": 0, "requested_steps": args.steps, "requested_warmup": args.warmup,
            "ms_per_step": round(value_ms, 1), "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": f"synthetic: seeded spheres ({nsph}), seed 0, r=6, vf=0.30",
            "config": {"workload": f"{n}^3 two-phase elastic HEX8, 6 unit load cases, CG rel L2 {args.tol}",
                       "parallelism": "cpu-openmp", "iterations": res["iterations"]},
            "cpu_baseline": {"value": round(value_ms, 1), "unit": "ms", "cores": res["cores"], "cpu": cpu_model(),
                             "kind": "port",
                             "sample": sample},
            "e2e": {"value": round(value_ms, 1), "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "ceff_rel_diff_vs_committed_oracle_run": check}
    print(json.dumps(line), flush=True)
    return 0


def run_batch64(args):
    """The batched workload: 64 instances (edges 32..96, thermal 3 load cases /
    elastic 6, mixed precision, rel. L2 tol), contexts created and Green's tables
    built beforehand.  Each instance's load cases are one multi-RHS solve (a
    context with n_rhs = 3 or 6); the 64 solves run one after another, then as
    one fansgpu_solve_batch call (one host thread and stream per context).  With
    --rhs 1 every load case is a solve of its own (288 solves; six batch calls)."""
    import torch

    from fans_gb300 import Context, solve_batch
    from fans_gb300.microstructure import batch_workload

    torch.cuda.set_device(0)
    work = batch_workload(64)
    multi = args.rhs == 6
    ctxs = []
    for w in work:
        n = w["n"]
        nl = 3 if w["thermal"] else 6
        if w["thermal"]:
            c = Context((n, n, n), (1.0, 1.0, 1.0), 1, "HEX8", "mixed", "cg", n_rhs=nl if multi else 1)
            c.set_microstructure(w["ms"])
            c.set_phase_material(0, 0, [1.0])
            c.set_phase_material(1, 0, [10.0])
            c.set_reference(5.5 * np.eye(3))
        else:
            c = Context((n, n, n), (1.0, 1.0, 1.0), 3, "HEX8", "mixed", "cg", n_rhs=nl if multi else 1)
            c.set_microstructure(w["ms"])
            for ph in range(2):
                c.set_phase_material(ph, 1, MAT[ph])
            c.set_reference(kapparef())
        c.set_tolerance("L2", "relative", args.tol, 2000)
        ctxs.append(c)

    def prepare(c, l=None):
        c.reset()
        if multi:
            c.set_gradients(np.eye(c.n_str))
        else:
            g = np.zeros(c.n_str)
            g[l] = 1.0
            c.set_gradient(g)

    def stresses(c):
        return c.homogenized_stresses() if multi else c.homogenized_stress()

    for c in ctxs:  # warm-up: tables, Green's operator, graphs
        prepare(c, 0)
        c.solve()
    torch.cuda.synchronize()
    seq, t0 = {}, time.perf_counter()
    for i, c in enumerate(ctxs):
        for l in ([None] if multi else range(c.n_str)):
            prepare(c, l)
            c.solve()
            seq[(i, l)] = stresses(c)
    seq_ms = (time.perf_counter() - t0) * 1e3
    bat, t0 = {}, time.perf_counter()
    for l in ([None] if multi else range(6)):
        group = [(i, c) for i, c in enumerate(ctxs) if multi or l < c.n_str]
        for _, c in group:
            prepare(c, l)
        sts = solve_batch([c for _, c in group])
        assert all(st["converged"] for st in sts)
        for i, c in group:
            bat[(i, l)] = stresses(c)
    bat_ms = (time.perf_counter() - t0) * 1e3
    diff = max(float(np.abs(bat[k] - v).max()) for k, v in seq.items())
    voxel_rhs = sum(w["n"] ** 3 * (3 if w["thermal"] else 6) for w in work)
    print(json.dumps({"workload": "batch64: 64 micro problems (edges 32-96; thermal 3 RHS / elastic 6 RHS), "
                                  f"mixed precision, rel L2 {args.tol}",
                      "rhs": "one multi-RHS solve per instance" if multi else "one solve per load case",
                      "solves": len(seq), "voxel_rhs": voxel_rhs,
                      "sequential_ms": round(seq_ms, 1), "batched_ms": round(bat_ms, 1),
                      "speedup": round(seq_ms / bat_ms, 2), "max_stress_diff_batched_vs_sequential": diff,
                      "graphs": os.environ.get("FANSGPU_GRAPHS", "1") != "0"}))
    for c in ctxs:
        c.close()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "batch64":
        return run_batch64(args)
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if dist:
            dist.barrier()
        torch.cuda.synchronize()

    n = args.n
    ms, nsph = build_problem(n)
    kref = kapparef()
    ctx = make_ctx(ms, n, "mixed", args.tol, n_rhs=args.rhs)

    # warm-up (W full steps)
    for _ in range(args.warmup):
        homogenize(ctx, kref)

    # timed region: K steps as a user runs them (the device-resident CG loop in
    # CUDA graphs), CUDA events on the solver stream
    stats: list = []
    clocks = ClockSampler()
    barrier()
    ms_total, Ceff = timed_steps(ctx, args.steps, lambda: homogenize(ctx, kref, stats))
    barrier()
    ms_step = max_over_ranks(ms_total / args.steps, dist, "cuda")
    iters = [s["iterations"] for s in stats[:6]]
    refinements = [s["refinements"] for s in stats[:6]]
    # kernel-timed region: the same K steps again with a CUDA event pair around
    # every launch on the solver stream (graphs off) -> per-kernel breakdown and
    # the roofline's average launch duration
    ctx.set_timing(True)
    barrier()
    timed_steps(ctx, args.steps, lambda: homogenize(ctx, kref))
    barrier()
    clk = clocks.stop()
    ktimes = ctx.kernel_times()
    ctx.set_timing(False)
    # launches in the timed region: the timed kernels, plus the folds (one per
    # refresh and one at the end of a solve) and one loop-check kernel per
    # graph-resident iteration (every iteration but the first)
    if args.rhs == 6:
        steps_stats = [stats[i:i + 6] for i in range(0, len(stats), 6)]
        launches = sum(c for _, c in ktimes.values()) + sum(
            sum(s["refinements"] for s in g) + 1 + max(max(s["iterations"] for s in g) - 1, 0) for g in steps_stats)
    else:
        launches = sum(c for _, c in ktimes.values()) + sum(
            (s["refinements"] + 1) + max(s["iterations"] - 1, 0) for s in stats)
    # the operator either covers every RHS still iterating in one launch (k_stencil_tcb) or runs
    # once per RHS (k_stencil_tc, "tc_per_rhs": a converged RHS's launch returns at once); its
    # timing span covers the iteration's operator launches either way
    op_per_rhs = ctx.tuning()["operator"] == "tc_per_rhs" and args.rhs > 1
    if op_per_rhs:
        launches += (args.rhs - 1) * ktimes.get("stencil", (0, 0))[1]
    # right-hand sides per iteration-kernel launch (the multi-RHS solve's launches
    # cover every RHS still iterating)
    rhs_iters_step = sum(iters)
    stencil_launches = ktimes.get("stencil", (0, 0))[1] / args.steps
    r_avg = rhs_iters_step / stencil_launches if stencil_launches else 1.0

    # e2e through the C ABI from pinned host buffers
    pinned = torch.empty(n ** 3, dtype=torch.int16, pin_memory=True)
    ms_host = pinned.numpy().view(np.uint16).reshape(n, n, n)
    ms_host[...] = ms

    def e2e_step():
        ctx.set_microstructure(ms_host)
        for ph in range(2):
            ctx.set_phase_material(ph, 1, MAT[ph])
        return homogenize(ctx, kref)

    e2e_step()
    barrier()
    t0 = time.perf_counter()
    e2e_ms_dev, _ = timed_steps(ctx, args.steps, e2e_step)
    e2e_wall = (time.perf_counter() - t0) * 1e3 / args.steps
    e2e_ms = max_over_ranks(max(e2e_ms_dev / args.steps, 0.0), dist, "cuda")
    scal_bytes = 144
    h2d = 2 * n ** 3 + 2 * 2 * 8 + 36 * 8 + 6 * 6 * 8
    d2h = 6 * 6 * 8 + scal_bytes * (sum(iters) + sum(refinements) + 6) + 4

    # roofline of the dominant kernel (by device time in the kernel-timed region)
    hbm, peak_kind = peaks()
    def abytes(k):
        return algo_bytes(k, n, r=r_avg if k in ITER_KERNELS else 1.0)

    dom = max((k for k in ktimes if ktimes[k][1] > 0 and abytes(k) is not None), key=lambda k: ktimes[k][0])
    if dom == "stencil" and op_per_rhs:
        # one launch per RHS: the launch's bytes are one RHS's, its time the span per active RHS
        dom_bytes, avg_ms, r_dom = algo_bytes(dom, n, r=1.0), ktimes[dom][0] / (rhs_iters_step * args.steps), 1
        traffic = traffic_table().get((dom, n, 1))
        kname = "k_stencil_tc (one launch per RHS)"
    else:
        dom_bytes, avg_ms, r_dom = abytes(dom), ktimes[dom][0] / ktimes[dom][1], args.rhs
        traffic = traffic_table().get((dom, n, args.rhs))  # ncu bytes of a launch with every RHS active
        if traffic is not None and dom in ITER_KERNELS:
            traffic = round(traffic * r_avg / args.rhs)     # the average launch of the step
        kname = {"stencil": "k_stencil_tcb"}.get(dom, dom)
    achieved = dom_bytes / (avg_ms * 1e-3) / 1e9
    roofline = {"bound": "hbm", "kernel": dom, "kernel_name": kname, "achieved": round(achieved, 1), "peak": hbm,
                "unit": "GB/s", "frac": round(achieved / hbm, 3), "peak_kind": peak_kind, "traffic": traffic,
                "algorithmic_bytes_per_launch": int(dom_bytes), "avg_launch_ms": round(avg_ms, 4),
                "rhs_per_launch": (round(r_avg, 3) if r_dom != 1 else 1.0) if dom in ITER_KERNELS else 1.0}
    per_kernel = {k: {"ms": round(v[0] / args.steps, 3), "launches": v[1] // args.steps,
                      "GBps": (round(abytes(k) * v[1] / (v[0] * 1e-3) / 1e9, 1) if v[1] and abytes(k) else None)}
                  for k, v in ktimes.items() if v[1]}

    # FP64 GPU path, same step, once
    fp64 = None
    if not args.no_fp64 and rank == 0:
        ctx64 = make_ctx(ms, n, "fp64", args.tol)
        ctx64.set_tolerance("L2", "relative", args.tol, 3)
        ctx64.set_gradient(np.eye(6)[0])
        ctx64.solve()  # builds the Green's table; 3 iterations as warm-up
        ctx64.set_tolerance("L2", "relative", args.tol, 2000)
        st64: list = []
        ctx64.set_timing(True)  # per-launch events: the FP64 path runs no graphs, so the step time is unchanged
        t64, C64 = timed_steps(ctx64, 1, lambda: homogenize(ctx64, kref, st64))
        k64 = ctx64.kernel_times()
        fp64 = {"ms_per_step": round(t64, 1), "iterations": [s["iterations"] for s in st64],
                "ceff_rel_diff_mixed_vs_fp64": float(np.linalg.norm(Ceff - C64) / np.linalg.norm(C64)),
                "speedup_mixed_vs_fp64": round(t64 / ms_step, 2),
                "kernels_ms": {k: round(v[0], 1) for k, v in k64.items() if v[1]}}
        # the FP64 CG operator: FP64-accurate, computed off the FP64 pipe (exact fixed-point
        # slices on the tensor cores, or double-float on the CUDA cores), so its roofline is
        # the HBM one of an FP64 field sweep; the FP64 pipe's measured FMA rate is reported
        # beside it as the rate an FP64-pipe operator could not exceed
        rate = fp64_rate()
        sl = k64.get("stencil", (0.0, 0))
        if sl[1]:
            t_launch = sl[0] * 1e-3 / sl[1]
            ab = algo_bytes("stencil", n, 3, 8)
            dfma = 64 * 3 * 3 * n ** 3  # 8 elements x (8 nodes x 3 comps) x 3 rows per node
            fp64["operator_roofline"] = {
                "kernel": {"tc_slices": "k_stencil_tcx", "df": "k_residual_df", "fp64": "k_stencil<double>"}[
                    ctx64.tuning()["exact_operator"]],
                "bound": "hbm", "achieved": round(ab / t_launch / 1e9, 1), "peak": hbm, "unit": "GB/s",
                "frac": round(ab / t_launch / 1e9 / hbm, 3), "avg_launch_ms": round(t_launch * 1e3, 3),
                "fp64_pipe_dfma_per_s": rate,
                "fp64_pipe_time_ms": round(dfma / rate * 1e3, 3) if rate else None}
        ctx64.close()

    cpu = None
    fx = oracle_256() if n == 256 else None
    if not args.no_cpu and rank == 0:
        # the oracle's own iteration counts of the complete solve (committed run), else this run's FP64 GPU ones
        if fx is not None:
            it_cpu, it_src = fx["iterations"], "the oracle's complete 256^3 solve (tests/golden/elastic256_ceff.json)"
        else:
            it_cpu, it_src = (fp64["iterations"] if fp64 else iters), "this run's GPU iteration counts"
        cb = cpu_baseline(ms, n, args.cpu_iters)
        cpu_ms = 1e3 * (6 * cb["setup_s"] + cb["per_iter_s"] * sum(it_cpu))
        cpu = {"value": round(cpu_ms, 1), "unit": "ms", "cores": cb["cores"], "cpu": cpu_model(), "kind": "port",
               "estimate": True,
               "sample": (f"oracle (FP64 C restatement, OpenMP) on {n}^3: solver setup + {args.cpu_iters} CG "
                          f"iterations of load case 0 ({cb['sample_s']:.1f} s, {cb['per_iter_s'] * 1e3:.0f} ms per "
                          f"iteration), times 6 setups and the iteration counts {it_cpu} of {it_src}; the measured "
                          f"complete solve is the reference arm (bench.py --impl reference)")}
    ceff_err = None
    if fx is not None:
        Cf = np.array(fx["C_eff_columns"])
        Cf = 0.5 * (Cf + Cf.T)
        ceff_err = float(np.linalg.norm(Ceff - Cf) / np.linalg.norm(Cf))

    if rank == 0:
        line = {"metric": METRIC, "value": round(ms_step, 2), "unit": "ms", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": round(ms_step, 2), "higher_is_better": False,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
                "data": f"synthetic: seeded periodic spheres ({nsph}), seed 0, r=6, vf=0.30",
                "config": {"workload": f"{n}^3 two-phase elastic HEX8, 6 unit load cases, CG rel L2 {args.tol}",
                           "precision": "mixed: FP32 stencil+FFT inner, FP64 residual/dots/solution",
                           "rhs": "one multi-RHS solve of the 6 load cases" if args.rhs == 6 else "6 solves in turn",
                           "l2": "inputs larger than L2 (fields 0.2-0.4 GB each)",
                           "parallelism": f"replicas{world}" if world > 1 else "single-gpu",
                           "iterations": iters, "refinements": refinements,
                           "fft_tiles_zyx": list(ctx.tuning()["fp32"])},
                "ceff_rel_err_vs_oracle": ceff_err,
                "e2e": {"value": round(e2e_ms, 2), "unit": "ms", "h2d_bytes_per_step": h2d,
                        "d2h_bytes_per_step": d2h, "wall_ms": round(e2e_wall, 2)},
                "gpu_launches": int(launches),
                "roofline": roofline, "kernels": per_kernel, "fp64_gpu": fp64, "cpu_baseline": cpu,
                "clocks": clk}
        print(json.dumps(line), flush=True)
    ctx.close()
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
