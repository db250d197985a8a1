"""torch.autograd.Function front ends of the GPU adjoints.

* `EffectiveStiffness`: per-voxel stiffness scale s(x) -> homogenized stiffness
  (n_str x n_str) of a linear problem, columns from the unit load cases
  (Solver::get_homogenized_tangent's linear branch, solver.h:759-776); its
  backward is fansgpu_stiffness_gradient (no adjoint solve: the unit-load
  displacement fields are stationary points of the energy).
* `YieldPathStress`: per-voxel initial yield stress -> <sigma> after a
  strain-controlled J2PlasticityNew load path; its backward is
  fansgpu_yield_stress_adjoint with grad_output as the seed w (a reverse sweep
  over the load steps with checkpointed internal variables).  The adjoint call
  runs the path again from the context's reset state, so forward + backward
  cost two forward paths and one reverse sweep.

The Context does the work on its GPU; tensors cross the C ABI as host float64
arrays and come back on the input's device and dtype.
"""
from __future__ import annotations

import numpy as np
import torch


def _host(t: torch.Tensor) -> np.ndarray:
    return np.ascontiguousarray(t.detach().to("cpu", torch.float64).numpy())


def _like(a: np.ndarray, t: torch.Tensor) -> torch.Tensor:
    return torch.from_numpy(np.ascontiguousarray(a)).to(device=t.device, dtype=t.dtype)


class EffectiveStiffness(torch.autograd.Function):
    """C = EffectiveStiffness.apply(scale, context): scale is [x][y][z]; the
    context holds the microstructure, the linear phase laws and the tolerance."""

    @staticmethod
    def forward(fctx, scale, context):
        context.set_voxel_scale(_host(scale))
        n = context.n_str
        C = np.zeros((n, n))
        for i in range(n):
            g = np.zeros(n)
            g[i] = 1.0
            context.reset()
            context.set_gradient(g)
            if not context.solve()["converged"]:
                raise RuntimeError(f"EffectiveStiffness: unit load case {i} did not converge")
            C[:, i] = context.homogenized_stress()
            context.store_solution(i)
        fctx.context = context
        fctx.save_for_backward(scale)
        return _like(C, scale)

    @staticmethod
    def backward(fctx, grad_C):
        (scale,) = fctx.saved_tensors
        g = fctx.context.stiffness_gradient(_host(grad_C))
        return _like(g, scale), None


class YieldPathStress(torch.autograd.Function):
    """sigma = YieldPathStress.apply(sigma_y, context, path, checkpoint_every=5,
    rel_tol=1e-10): sigma_y is [x][y][z], path is n_steps x 6 macroscopic strains."""

    @staticmethod
    def forward(fctx, sigma_y, context, path, checkpoint_every=5, rel_tol=1e-10):
        path = np.ascontiguousarray(path, dtype=float).reshape(-1, 6)
        context.set_voxel_yield_stress(_host(sigma_y))
        context.reset()
        for k, g in enumerate(path):
            context.set_gradient(g)
            if not context.solve()["converged"]:
                raise RuntimeError(f"YieldPathStress: load step {k + 1} did not converge")
            if k + 1 < len(path):
                context.extrapolate_displacement()
        stress = context.homogenized_stress()
        fctx.context, fctx.path, fctx.every, fctx.rel_tol = context, path, checkpoint_every, rel_tol
        fctx.save_for_backward(sigma_y)
        return _like(stress, sigma_y)

    @staticmethod
    def backward(fctx, grad_stress):
        (sigma_y,) = fctx.saved_tensors
        c = fctx.context
        c.reset()
        out = c.yield_stress_adjoint(fctx.path, _host(grad_stress), fctx.every, fctx.rel_tol)
        return _like(out["grad"], sigma_y), None, None, None, None
