"""Host mirror of FANS's Solver / SolverCG / SolverFP API over the C ABI.

`Context` is a thin owner of one `fansgpu_ctx` (one GPU solver state).
`Solver`, `SolverCG` and `SolverFP` keep the reference's public surface
(solver.h:11-103): solve(), get_homogenized_stress(), get_homogenized_tangent(),
extrapolateDisplacement(), fields v_u / v_r, iter and err_all.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib as C
from .materials import MaterialManager

_dp = ctypes.POINTER(ctypes.c_double)


def _ptr(a):
    return a.ctypes.data_as(_dp)


class Context:
    """One GPU solver context (fansgpu_create .. fansgpu_destroy)."""

    def __init__(self, n, L=(1.0, 1.0, 1.0), howmany=3, fe_type="HEX8", precision="fp64", method="cg",
                 strain_type="small", n_rhs=1):
        self.lib = C.load()
        d = C.Desc()
        d.n[:] = [int(v) for v in n]
        d.L[:] = [float(v) for v in L]
        d.howmany = int(howmany)
        d.fe_type = C.FE_TYPES[fe_type] if isinstance(fe_type, str) else int(fe_type)
        d.precision = {"fp64": C.FP64, "mixed": C.MIXED}[precision] if isinstance(precision, str) else int(precision)
        d.method = {"cg": C.CG, "fp": C.FP, "newton": C.NEWTON}[method] if isinstance(method, str) else int(method)
        d.strain_type = C.STRAIN_TYPES[strain_type] if isinstance(strain_type, str) else int(strain_type)
        d.n_rhs = int(n_rhs)
        ptr = ctypes.c_void_p()
        rc = self.lib.fansgpu_create(ctypes.byref(d), ctypes.byref(ptr))
        if rc != C.OK:
            raise C.FansGpuError(rc, self.lib.fansgpu_last_error(None).decode())
        self.ctx = ptr
        self.n = tuple(int(v) for v in n)
        self.howmany = int(howmany)
        self.large_strain = d.strain_type == C.LARGE_STRAIN
        self.n_str = 9 if self.large_strain else (3 if howmany == 1 else 6)
        self.n_gp = 1 if d.fe_type == C.FE_TYPES["HEX8R"] else 8
        self.N = self.n[0] * self.n[1] * self.n[2]
        self.n_rhs = max(1, int(n_rhs))

    def close(self):
        if getattr(self, "ctx", None):
            self.lib.fansgpu_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _chk(self, rc, allow=()):
        return C.check(self.ctx, rc, allow)

    # -- state ---------------------------------------------------------------
    def set_microstructure(self, ms):
        ms = np.ascontiguousarray(ms, dtype=np.uint16)
        assert ms.shape == self.n, (ms.shape, self.n)
        self._chk(self.lib.fansgpu_set_microstructure(self.ctx, ms.ctypes.data_as(ctypes.POINTER(ctypes.c_uint16))))

    def set_phase_material(self, phase, law, params):
        p = np.ascontiguousarray(params, dtype=float).ravel()
        self._chk(self.lib.fansgpu_set_phase_material(self.ctx, int(phase), int(law), _ptr(p), p.size))

    def set_reference(self, kapparef):
        k = np.ascontiguousarray(kapparef, dtype=float)
        self._chk(self.lib.fansgpu_set_reference(self.ctx, _ptr(k)))

    def set_gradient(self, g0):
        g = np.ascontiguousarray(g0, dtype=float)
        assert g.size == self.n_str
        self._chk(self.lib.fansgpu_set_gradient(self.ctx, _ptr(g)))

    def set_tolerance(self, measure="L2", type="relative", tolerance=1e-10, n_it=100, ls_max_iter=5, ls_tol=1e-2):
        t = C.Tol(C.MEASURES[measure], C.ERROR_TYPES[type], float(tolerance), int(n_it), int(ls_max_iter),
                  float(ls_tol))
        self._chk(self.lib.fansgpu_set_tolerance(self.ctx, ctypes.byref(t)))

    # -- solve ---------------------------------------------------------------
    def solve(self):
        st = C.Stats()
        self._chk(self.lib.fansgpu_solve(self.ctx, ctypes.byref(st)), allow=(C.ENOTCONV,))
        return {"iterations": st.iterations, "converged": bool(st.converged), "err0": st.err0, "err": st.err,
                "refinements": st.refinements, "solve_ms": st.solve_ms}

    # -- several right-hand sides (fansgpu_set_gradients / select_rhs / rhs_stats) ----
    def set_gradients(self, g0s):
        g = np.ascontiguousarray(g0s, dtype=float).reshape(-1, self.n_str)
        self._chk(self.lib.fansgpu_set_gradients(self.ctx, g.shape[0], _ptr(g)))

    def select_rhs(self, k):
        self._chk(self.lib.fansgpu_select_rhs(self.ctx, int(k)))

    def rhs_stats(self, k):
        st = C.Stats()
        self._chk(self.lib.fansgpu_rhs_stats(self.ctx, int(k), ctypes.byref(st)))
        return {"iterations": st.iterations, "converged": bool(st.converged), "err0": st.err0, "err": st.err,
                "refinements": st.refinements, "solve_ms": st.solve_ms}

    def homogenized_stresses(self):
        """<sigma> of every right-hand side (n_rhs x n_str); RHS 0 is selected afterwards."""
        out = np.zeros((self.n_rhs, self.n_str))
        for k in range(self.n_rhs):
            self.select_rhs(k)
            out[k] = self.homogenized_stress()
        self.select_rhs(0)
        return out

    def homogenized_stress(self):
        out = np.zeros(self.n_str)
        self._chk(self.lib.fansgpu_homogenized_stress(self.ctx, _ptr(out)))
        return out

    def homogenized_tangent(self, pert=1e-6):
        out = np.zeros((self.n_str, self.n_str))
        self._chk(self.lib.fansgpu_homogenized_tangent(self.ctx, float(pert), _ptr(out)))
        return out

    def postprocess_averages(self, n_phase):
        ns = self.n_str
        se, ss = np.zeros(ns), np.zeros(ns)
        pe, ps = np.zeros((n_phase, ns)), np.zeros((n_phase, ns))
        cnt = np.zeros(n_phase, dtype=np.int64)
        self._chk(self.lib.fansgpu_postprocess_averages(self.ctx, _ptr(se), _ptr(ss), _ptr(pe), _ptr(ps),
                                                        cnt.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                                        int(n_phase)))
        return dict(strain_average=se, stress_average=ss, phase_strain=pe, phase_stress=ps, phase_count=cnt)

    def get_field(self, which):
        if which in (C.FIELD_U, C.FIELD_R, C.FIELD_U_PREV):
            shape = (self.howmany,)
        elif which in (C.FIELD_PLASTIC_STRAIN, C.FIELD_KINEMATIC):
            shape = (6,)
        elif which == C.FIELD_KINEMATIC_GP:
            shape = (self.n_gp, 6)
        elif which in (C.FIELD_HARDENING, C.FIELD_PLASTIC_FLAG):
            shape = (1,)
        elif which in (C.FIELD_STRAIN_GP, C.FIELD_STRESS_GP):
            shape = (self.n_gp, self.n_str)
        elif which == C.FIELD_PLASTIC_STRAIN_GP:
            shape = (self.n_gp, 6)
        elif which == C.FIELD_HARDENING_GP:
            shape = (self.n_gp,)
        else:
            shape = (self.n_str,)
        out = np.zeros(self.n + shape)
        self._chk(self.lib.fansgpu_get_field(self.ctx, int(which), _ptr(out)))
        return out

    def set_field(self, which, arr):
        a = np.ascontiguousarray(arr, dtype=float)
        assert a.shape == self.n + (self.howmany,)
        self._chk(self.lib.fansgpu_set_field(self.ctx, int(which), _ptr(a)))

    def error_history(self):
        n = ctypes.c_int32()
        self._chk(self.lib.fansgpu_get_error_history(self.ctx, None, 0, ctypes.byref(n)))
        out = np.zeros(max(n.value, 1))
        self._chk(self.lib.fansgpu_get_error_history(self.ctx, _ptr(out), n.value, ctypes.byref(n)))
        return out[: n.value]

    def extrapolate_displacement(self):
        self._chk(self.lib.fansgpu_extrapolate_displacement(self.ctx))

    def reset(self):
        """Solver ctor state for a new load case: v_u = v_u_prev = v_r = 0."""
        self._chk(self.lib.fansgpu_reset(self.ctx))

    def stream(self):
        """cudaStream_t (as int) of this context."""
        p = ctypes.c_void_p()
        self._chk(self.lib.fansgpu_get_stream(self.ctx, ctypes.byref(p)))
        return p.value or 0

    def set_refresh(self, factor):
        """Mixed precision: FP32-residual reduction that triggers an FP64 refresh."""
        self._chk(self.lib.fansgpu_set_refresh(self.ctx, float(factor)))

    def set_wait_limit(self, polls):
        """Diagnostics: polls before a tensor-core pipeline wait gives up (0: default)."""
        self._chk(self.lib.fansgpu_set_wait_limit(self.ctx, int(polls)))

    def tuning(self):
        """fansgpu_tuning: {"fp64": (z, y, x), "fp32": (z, y, x), "tensor_core": bool,
        "operator": "cuda" | "tc" | "tc_basis" | "tc_per_rhs", "exact_operator": "fp64" | "df" | "tc_slices"}."""
        out = np.zeros(8, dtype=np.int32)
        self._chk(self.lib.fansgpu_tuning(self.ctx, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))))
        return {"fp64": tuple(int(v) for v in out[:3]), "fp32": tuple(int(v) for v in out[3:6]),
                "tensor_core": bool(out[6]), "operator": ("cuda", "tc", "tc_basis", "tc_per_rhs")[int(out[6])],
                "exact_operator": ("fp64", "df", "tc_slices")[int(out[7])]}

    def set_timing(self, on=True):
        self._chk(self.lib.fansgpu_set_timing(self.ctx, int(bool(on))))

    def kernel_times(self):
        """{kernel name: (total ms, launches)} since set_timing(True)."""
        n = len(C.KERNEL_NAMES)
        ms = np.zeros(n)
        cnt = np.zeros(n, dtype=np.int64)
        self._chk(self.lib.fansgpu_kernel_times(self.ctx, _ptr(ms), cnt.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                                n))
        return {k: (float(ms[i]), int(cnt[i])) for i, k in enumerate(C.KERNEL_NAMES)}

    def enable_mixed_bc(self, idx_e, strain_e, idx_f, stress_f, step):
        """MixedBCController::activate (mixedBCs.h:180-226) for one time step."""
        ie = np.ascontiguousarray(idx_e, dtype=np.int32)
        jf = np.ascontiguousarray(idx_f, dtype=np.int32)
        se = np.ascontiguousarray(strain_e, dtype=float)
        sf = np.ascontiguousarray(stress_f, dtype=float)
        i32 = ctypes.POINTER(ctypes.c_int32)
        self._chk(self.lib.fansgpu_enable_mixed_bc(self.ctx, len(ie), ie.ctypes.data_as(i32), _ptr(se), len(jf),
                                                   jf.ctypes.data_as(i32), _ptr(sf), int(step)))

    def disable_mixed_bc(self):
        self._chk(self.lib.fansgpu_disable_mixed_bc(self.ctx))

    def gradient(self):
        g = np.zeros(self.n_str)
        self._chk(self.lib.fansgpu_get_gradient(self.ctx, _ptr(g)))
        return g

    def set_voxel_scale(self, scale):
        """Per-voxel stiffness scale s(x) ([x][y][z]); None clears it."""
        if scale is None:
            self._chk(self.lib.fansgpu_set_voxel_field(self.ctx, C.VOXEL_STIFFNESS_SCALE, None))
            return
        a = np.ascontiguousarray(scale, dtype=float)
        assert a.shape == self.n
        self._chk(self.lib.fansgpu_set_voxel_field(self.ctx, C.VOXEL_STIFFNESS_SCALE, _ptr(a)))

    def set_voxel_yield_stress(self, sy):
        """Per-voxel initial yield stress of J2PlasticityNew voxels ([x][y][z]); None clears it."""
        if sy is None:
            self._chk(self.lib.fansgpu_set_voxel_field(self.ctx, C.VOXEL_YIELD_STRESS, None))
            return
        a = np.ascontiguousarray(sy, dtype=float)
        assert a.shape == self.n
        self._chk(self.lib.fansgpu_set_voxel_field(self.ctx, C.VOXEL_YIELD_STRESS, _ptr(a)))

    def yield_stress_adjoint(self, g0_path, w, checkpoint_every=5, rel_tol=1e-10):
        """fansgpu_yield_stress_adjoint: run the strain-controlled path g0_path
        (n_steps x 6) and return the final <sigma>, d(w . <sigma>)/d sigma_y per
        voxel ([x][y][z]) and the forward / adjoint CG iterations per step."""
        path = np.ascontiguousarray(g0_path, dtype=float).reshape(-1, 6)
        w = np.ascontiguousarray(w, dtype=float).ravel()
        assert w.size == 6
        stress, grad = np.zeros(6), np.zeros(self.n)
        its = np.zeros(2 * len(path), dtype=np.int32)
        self._chk(self.lib.fansgpu_yield_stress_adjoint(
            self.ctx, len(path), _ptr(path), int(checkpoint_every), _ptr(w), float(rel_tol), _ptr(stress), _ptr(grad),
            its.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))))
        return {"stress": stress, "grad": grad, "forward_iterations": its[: len(path)],
                "adjoint_iterations": its[len(path):]}

    def store_solution(self, slot):
        self._chk(self.lib.fansgpu_store_solution(self.ctx, int(slot)))

    def stiffness_gradient(self, W):
        W = np.ascontiguousarray(W, dtype=float)
        out = np.zeros(self.n)
        self._chk(self.lib.fansgpu_stiffness_gradient(self.ctx, W.shape[0], _ptr(W), _ptr(out)))
        return out

    def commit_state(self):
        self._chk(self.lib.fansgpu_commit_state(self.ctx))

    # -- kernel-level --------------------------------------------------------
    def _map(self, fn, x):
        x = np.ascontiguousarray(x, dtype=float)
        assert x.shape == self.n + (self.howmany,)
        y = np.zeros_like(x)
        self._chk(fn(self.ctx, _ptr(x), _ptr(y)))
        return y

    def residual(self, u):
        return self._map(self.lib.fansgpu_residual, u)

    def apply_operator(self, x):
        return self._map(self.lib.fansgpu_apply_operator, x)

    def convolve(self, r):
        return self._map(self.lib.fansgpu_convolve, r)

    def green_table(self):
        nt = self.howmany * (self.howmany + 1) // 2
        out = np.zeros((self.n[0], self.n[1], self.n[2] // 2 + 1, nt))
        self._chk(self.lib.fansgpu_green_table(self.ctx, _ptr(out)))
        return out


def solve_batch(contexts):
    """fansgpu_solve_batch: solve several independent contexts concurrently.
    Returns one stats dict per context (as Context.solve) plus its status code."""
    lib = C.load()
    n = len(contexts)
    arr = (ctypes.c_void_p * n)(*[c.ctx for c in contexts])
    st = (C.Stats * n)()
    rcs = (ctypes.c_int32 * n)()
    rc = lib.fansgpu_solve_batch(arr, n, st, rcs)
    if rc not in (C.OK, C.ENOTCONV):
        raise C.FansGpuError(rc, lib.fansgpu_last_error(None).decode())
    return [{"iterations": s.iterations, "converged": bool(s.converged), "err0": s.err0, "err": s.err,
             "refinements": s.refinements, "solve_ms": s.solve_ms, "rc": int(r)} for s, r in zip(st, rcs)]


class Solver:
    """Solver<howmany, n_str> (solver.h:11-103) on the GPU.

    `reader` is a fans_gb300.reader.Reader (or any object with the same
    attributes: dims, L, problemType, FE_type, method, errorParameters, TOL,
    n_it, ls_max_iter, ls_tol, ms, inputJson)."""

    method = "cg"

    def __init__(self, reader, matmanager: MaterialManager, precision="fp64"):
        self.reader = reader
        self.matmanager = matmanager
        self.howmany = 1 if reader.problemType == "thermal" else 3
        strain_type = getattr(reader, "strain_type", "small") if self.howmany == 3 else "small"
        self.ctx = Context(reader.dims, reader.L, self.howmany, reader.FE_type, precision, self.method, strain_type)
        self.n_str = self.ctx.n_str
        self.ctx.set_microstructure(reader.ms)
        matmanager.apply(self.ctx)
        self._push_tolerance()
        self.iter = 0
        self.err_all = np.zeros(0)
        self.last_stats = None

    def _push_tolerance(self):
        ep = self.reader.errorParameters
        self.ctx.set_tolerance(ep["measure"], ep["type"], self.reader.TOL, self.reader.n_it, self.reader.ls_max_iter,
                               self.reader.ls_tol)

    def set_gradient(self, g0):
        """MaterialManager::set_gradient (MaterialManager.h:216-221)."""
        self.ctx.set_gradient(g0)

    def solve(self):
        """Solver::solve (solver.h:283-300)."""
        st = self.ctx.solve()
        self.iter = st["iterations"]
        self.err_all = self.ctx.error_history()
        self.last_stats = st
        return st

    @property
    def v_u(self):
        return self.ctx.get_field(C.FIELD_U)

    @property
    def v_r(self):
        return self.ctx.get_field(C.FIELD_R)

    def get_homogenized_stress(self):
        return self.ctx.homogenized_stress()

    def get_homogenized_tangent(self, pert_param=1e-6):
        """solver.h:740-778, including its side effects on the error type and tolerance."""
        C_ = self.ctx.homogenized_tangent(pert_param)
        self.reader.errorParameters["type"] = "relative"
        self.reader.TOL = max(1e-6, self.reader.TOL)
        return C_

    def extrapolateDisplacement(self):
        self.ctx.extrapolate_displacement()

    def enableMixedBC(self, mbc, step):
        """Solver::enableMixedBC (solver.h:71-74) with a reader.MixedBC."""
        self.ctx.enable_mixed_bc(mbc.idx_E, mbc.F_E_path[step], mbc.idx_F, mbc.P_F_path[step], step)

    def disableMixedBC(self):
        self.ctx.disable_mixed_bc()

    def close(self):
        self.ctx.close()


class SolverCG(Solver):
    method = "cg"


class SolverFP(Solver):
    method = "fp"


def create_solver(reader, matmanager, precision="fp64"):
    """createSolver (setup.h:76-85)."""
    if reader.method == "fp":
        return SolverFP(reader, matmanager, precision)
    if reader.method == "cg":
        return SolverCG(reader, matmanager, precision)
    raise ValueError(f"{reader.method} is not a valid method")
