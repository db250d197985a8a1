"""ctypes binding of libfans_gb300.so (the C ABI declared in include/fans_gb300.h).

The library is the only compute path: if it is missing or fails to load, every
call raises -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libfans_gb300.so")

OK = 0
EINVAL, ENOMEM, ECUDA, ENOTCONV, ENAN, EUNSUPPORTED, ESTATE = -1, -2, -3, -4, -5, -6, -7
HEX8, HEX8R, BBAR = 0, 1, 2
LAW_THERMAL_ISO, LAW_ELASTIC_ISO, LAW_J2_LINEAR, LAW_THERMAL_TRI, LAW_ELASTIC_TRI = 0, 1, 2, 3, 4
LAW_PSEUDO_LINEAR, LAW_PSEUDO_NONLINEAR = 5, 6
LAW_J2VISCO_LINEAR, LAW_J2VISCO_NONLINEAR = 7, 8
LAW_SVK, LAW_NEOHOOKEAN = 9, 10
SMALL_STRAIN, LARGE_STRAIN = 0, 1
STRAIN_TYPES = {"small": SMALL_STRAIN, "large": LARGE_STRAIN}
FP64, MIXED = 0, 1
CG, FP, NEWTON = 0, 1, 2
L1, L2, LINF = 0, 1, 2
ABSOLUTE, RELATIVE = 0, 1
FIELD_U, FIELD_R, FIELD_STRAIN, FIELD_STRESS, FIELD_U_PREV = 0, 1, 2, 3, 4
FIELD_PLASTIC_STRAIN, FIELD_HARDENING = 5, 6
FIELD_STRAIN_GP, FIELD_STRESS_GP, FIELD_PLASTIC_STRAIN_GP, FIELD_HARDENING_GP = 7, 8, 9, 10
FIELD_PLASTIC_FLAG = 11
FIELD_KINEMATIC, FIELD_KINEMATIC_GP = 12, 13
VOXEL_STIFFNESS_SCALE, VOXEL_YIELD_STRESS = 0, 1

FE_TYPES = {"HEX8": HEX8, "HEX8R": HEX8R, "BBAR": BBAR}
MEASURES = {"L1": L1, "L2": L2, "Linfinity": LINF}
ERROR_TYPES = {"absolute": ABSOLUTE, "relative": RELATIVE}

#: every exported symbol of include/fans_gb300.h
EXPORTS = [
    "fansgpu_create", "fansgpu_destroy", "fansgpu_last_error", "fansgpu_set_microstructure",
    "fansgpu_set_phase_material", "fansgpu_set_reference", "fansgpu_set_gradient", "fansgpu_set_tolerance",
    "fansgpu_solve", "fansgpu_homogenized_stress", "fansgpu_homogenized_tangent", "fansgpu_postprocess_averages",
    "fansgpu_get_field", "fansgpu_set_field", "fansgpu_get_error_history", "fansgpu_extrapolate_displacement",
    "fansgpu_commit_state", "fansgpu_residual", "fansgpu_apply_operator", "fansgpu_convolve",
    "fansgpu_green_table", "fansgpu_version", "fansgpu_reset", "fansgpu_get_stream", "fansgpu_set_timing",
    "fansgpu_kernel_times", "fansgpu_residual_norm_noalloc", "fansgpu_set_refresh",
    "fansgpu_enable_mixed_bc", "fansgpu_disable_mixed_bc", "fansgpu_get_gradient", "fansgpu_set_voxel_field",
    "fansgpu_store_solution", "fansgpu_stiffness_gradient", "fansgpu_solve_batch", "fansgpu_yield_stress_adjoint",
    "fansgpu_tuning", "fansgpu_set_wait_limit", "fansgpu_set_gradients", "fansgpu_select_rhs", "fansgpu_rhs_stats",
    "fansgpu_fp64_fma_rate",
]
MAX_RHS = 6
KERNEL_NAMES = ["stencil", "fft_z_fwd", "fft_y_fwd", "fft_x_green", "fft_y_inv", "fft_z_inv", "cg_update",
                "residual64", "norm", "green_table", "strain_stress"]


class Desc(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int32 * 3), ("L", ctypes.c_double * 3), ("howmany", ctypes.c_int32),
                ("fe_type", ctypes.c_int32), ("precision", ctypes.c_int32), ("method", ctypes.c_int32),
                ("strain_type", ctypes.c_int32), ("n_rhs", ctypes.c_int32)]


class Tol(ctypes.Structure):
    _fields_ = [("measure", ctypes.c_int32), ("type", ctypes.c_int32), ("tolerance", ctypes.c_double),
                ("n_it", ctypes.c_int32), ("ls_max_iter", ctypes.c_int32), ("ls_tol", ctypes.c_double)]


class Stats(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int32), ("converged", ctypes.c_int32), ("err0", ctypes.c_double),
                ("err", ctypes.c_double), ("refinements", ctypes.c_int32), ("solve_ms", ctypes.c_double)]


class FansGpuError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"[{code}] {msg}")
        self.code = code


_lib = None


def load(build_if_missing: bool = True):
    """Load the library (building it first if absent and nvcc is available)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if not build_if_missing:
            raise FansGpuError(ECUDA, f"{LIB_PATH} not built")
        from . import build as _build

        _build.build()
    L = ctypes.CDLL(LIB_PATH)
    _declare(L)
    _lib = L
    return L


def _declare(L):
    vp, dp, ip = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.c_int32
    L.fansgpu_create.argtypes = [ctypes.POINTER(Desc), ctypes.POINTER(vp)]
    L.fansgpu_destroy.argtypes = [vp]
    L.fansgpu_last_error.argtypes = [vp]
    L.fansgpu_last_error.restype = ctypes.c_char_p
    L.fansgpu_version.restype = ctypes.c_char_p
    L.fansgpu_set_microstructure.argtypes = [vp, ctypes.POINTER(ctypes.c_uint16)]
    L.fansgpu_set_phase_material.argtypes = [vp, ip, ip, dp, ip]
    L.fansgpu_set_reference.argtypes = [vp, dp]
    L.fansgpu_set_gradient.argtypes = [vp, dp]
    L.fansgpu_set_tolerance.argtypes = [vp, ctypes.POINTER(Tol)]
    L.fansgpu_solve.argtypes = [vp, ctypes.POINTER(Stats)]
    L.fansgpu_homogenized_stress.argtypes = [vp, dp]
    L.fansgpu_homogenized_tangent.argtypes = [vp, ctypes.c_double, dp]
    L.fansgpu_postprocess_averages.argtypes = [vp, dp, dp, dp, dp, ctypes.POINTER(ctypes.c_int64), ip]
    L.fansgpu_get_field.argtypes = [vp, ip, dp]
    L.fansgpu_set_field.argtypes = [vp, ip, dp]
    L.fansgpu_get_error_history.argtypes = [vp, dp, ip, ctypes.POINTER(ctypes.c_int32)]
    L.fansgpu_extrapolate_displacement.argtypes = [vp]
    L.fansgpu_commit_state.argtypes = [vp]
    L.fansgpu_residual.argtypes = [vp, dp, dp]
    L.fansgpu_apply_operator.argtypes = [vp, dp, dp]
    L.fansgpu_convolve.argtypes = [vp, dp, dp]
    L.fansgpu_green_table.argtypes = [vp, dp]
    L.fansgpu_reset.argtypes = [vp]
    L.fansgpu_get_stream.argtypes = [vp, ctypes.POINTER(vp)]
    L.fansgpu_set_timing.argtypes = [vp, ip]
    L.fansgpu_kernel_times.argtypes = [vp, dp, ctypes.POINTER(ctypes.c_int64), ip]
    L.fansgpu_residual_norm_noalloc.argtypes = [vp, ctypes.c_int64, ip, vp, vp]
    L.fansgpu_set_refresh.argtypes = [vp, ctypes.c_double]
    i32p = ctypes.POINTER(ctypes.c_int32)
    L.fansgpu_enable_mixed_bc.argtypes = [vp, ip, i32p, dp, ip, i32p, dp, ip]
    L.fansgpu_disable_mixed_bc.argtypes = [vp]
    L.fansgpu_get_gradient.argtypes = [vp, dp]
    L.fansgpu_set_voxel_field.argtypes = [vp, ip, dp]
    L.fansgpu_store_solution.argtypes = [vp, ip]
    L.fansgpu_stiffness_gradient.argtypes = [vp, ip, dp, dp]
    L.fansgpu_solve_batch.argtypes = [ctypes.POINTER(vp), ip, ctypes.POINTER(Stats), i32p]
    L.fansgpu_yield_stress_adjoint.argtypes = [vp, ip, dp, ip, dp, ctypes.c_double, dp, dp, i32p]
    L.fansgpu_tuning.argtypes = [vp, i32p]
    L.fansgpu_set_wait_limit.argtypes = [vp, ip]
    L.fansgpu_set_gradients.argtypes = [vp, ip, dp]
    L.fansgpu_select_rhs.argtypes = [vp, ip]
    L.fansgpu_rhs_stats.argtypes = [vp, ip, ctypes.POINTER(Stats)]
    L.fansgpu_fp64_fma_rate.argtypes = [dp]
    for name in EXPORTS:
        if name not in ("fansgpu_last_error", "fansgpu_version"):
            getattr(L, name).restype = ctypes.c_int


def check(ctx, rc, allow=()):
    if rc == OK or rc in allow:
        return rc
    msg = load().fansgpu_last_error(ctx)
    raise FansGpuError(rc, msg.decode() if msg else "")
