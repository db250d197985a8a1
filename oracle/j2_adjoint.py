"""Yield-stress adjoint of a strain-controlled J2PlasticityNew load path, restated
densely in numpy for tiny grids.

TEST INFRASTRUCTURE ONLY.  This module is a checker for the CUDA product; only
tests/ may import it.

Forward: the C oracle (OracleProblem) runs the load path as runSolver does
(main.cpp:23-42: set the macroscopic strain, solve, commit, extrapolate), with
one J2 phase per voxel so that every voxel carries its own initial yield
stress.  Reverse: for L = w . <sigma_N> the discrete adjoint of the converged
path, n = N..1 with mu_N = 0,
    K_n lambda_n = -sum_gp B^T (J_e^T (cw [n = N]) + A_e^T mu_n)
    tau_n        = (v_e/n_gp) B lambda_n + cw [n = N]
    mu_{n-1}     = S_a^T tau_n + A_a^T mu_n
    dL/dsy(e)   += sum_gp S_y^T tau_n + A_y^T mu_n
with S = d sigma and A = d(eps_p, q) of the Gauss-point return map
(J2PlasticityNew.h:43-108) w.r.t. strain (e), the committed state (a) and the
initial yield stress (y), and cw = w/(N n_gp).  Those Jacobians come from
complex-step differentiation of `j2_return_map` -- exact to round-off and
independent of the closed-form vector-Jacobian product the CUDA kernels use.
K_n = sum (v_e/n_gp) B^T (dsigma/de) B is assembled densely and solved with
lstsq (the rigid translations are its null space; the load is orthogonal to
them, and tau does not see them).
"""
from __future__ import annotations

import numpy as np

import oracle as O

C23 = np.sqrt(2.0 / 3.0)


def j2_return_map(K, G, h, sy0, e, ep, q):
    """J2PlasticityNew::get_sigma (J2PlasticityNew.h:43-108) on arrays of Gauss
    points (last axis = Mandel components); complex inputs carry a complex-step
    perturbation, every branch is taken on real parts."""
    e, ep = np.asarray(e), np.asarray(ep)
    s = 2.0 * G[..., None] * (e - ep)
    lam = K - 2.0 / 3.0 * G
    tr = e[..., 0] + e[..., 1] + e[..., 2]
    s[..., :3] += (lam * tr)[..., None]
    st = s.copy()
    st[..., :3] -= (s[..., 0] + s[..., 1] + s[..., 2])[..., None] / 3.0
    s_t = np.sqrt((st * st).sum(-1))
    phi = s_t - C23 * (sy0 + q * h)
    dgamma = phi / (2.0 * G + 2.0 / 3.0 * h)
    dgamma = np.where(dgamma.real < 0.0, 0.0, dgamma)
    on = (s_t.real > 1e-12)[..., None]
    n = st / np.where(on[..., 0], s_t, 1.0)[..., None]
    ep_out = np.where(on, ep + dgamma[..., None] * n, ep)
    sig = np.where(on, s - (dgamma * 2.0 * G)[..., None] * n, s)
    return sig, ep_out, q + C23 * dgamma


def j2_jacobian(K, G, h, sy0, e, ep, q, step=1e-30):
    """d(sigma, eps_p', q') / d(e, eps_p, q, sy0) per Gauss point: shape (..., 13, 14),
    by complex step."""
    shape = e.shape[:-1]
    J = np.zeros(shape + (13, 14))
    for k in range(14):
        ec, epc = e.astype(complex), ep.astype(complex)
        qc, syc = np.asarray(q, dtype=complex), np.asarray(sy0, dtype=complex) * np.ones(shape)
        if k < 6:
            ec[..., k] += 1j * step
        elif k < 12:
            epc[..., k - 6] += 1j * step
        elif k == 12:
            qc = qc + 1j * step
        else:
            syc = syc + 1j * step
        sig, epo, qo = j2_return_map(K, G, h, syc, ec, epc, qc)
        J[..., :6, k] = sig.imag / step
        J[..., 6:12, k] = epo.imag / step
        J[..., 12, k] = qo.imag / step
    return J


def element_dofs(nx, ny, nz):
    """(N_el, 24) global dof indices (node-major u[x][y][z][c]) in the element's
    local order p = bx + 2 by + 4 bz (solver.h:318-385)."""
    x, y, z = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    x, y, z = x.ravel(), y.ravel(), z.ravel()
    dofs = np.zeros((x.size, 24), dtype=np.int64)
    for p in range(8):
        bx, by, bz = p & 1, (p >> 1) & 1, (p >> 2) & 1
        node = (((x + bx) % nx) * ny + (y + by) % ny) * nz + (z + bz) % nz
        for c in range(3):
            dofs[:, 3 * p + c] = 3 * node + c
    return dofs


def gp_strain(P, u, g0, dofs):
    """(N_el, n_gp, 6): B_gp u_e + g0 with u_e relative to node 0 (solver.h:252)."""
    ue = u.ravel()[dofs]
    ue = ue - np.tile(ue[:, :3], 8)
    B = P.B.reshape(P.ngp, 6, 24)
    return np.einsum("gik,ek->egi", B, ue) + g0


class YieldPathProblem:
    """A two-material J2 problem (matrix phase 0: J2 with per-voxel yield stress;
    phase 1: linear elastic) as the C oracle runs it, one J2 phase per matrix voxel."""

    def __init__(self, ms, j2_params, elastic_params, sy, L=(1.0, 1.0, 1.0)):
        self.ms = np.asarray(ms, dtype=np.uint16)
        self.K, self.G, _, self.h = j2_params
        self.sy = np.asarray(sy, dtype=float)
        nel = self.ms.size
        flat = self.ms.ravel()
        j2_vox = np.flatnonzero(flat == 0)
        ph = np.full(nel, 0, dtype=np.uint16)
        ph[j2_vox] = np.arange(j2_vox.size)
        ph[flat != 0] = j2_vox.size
        self.j2_vox = j2_vox
        self.elastic_params = tuple(elastic_params)
        groups = [(O.LAW_J2, list(range(j2_vox.size)),
                   [[self.K, self.G, float(self.sy.ravel()[v]), self.h] for v in j2_vox]),
                  (O.LAW_ELASTIC_ISO, [j2_vox.size], [list(elastic_params)])]
        # the reference stiffness of the two-material problem (mean of the two models' isotropic C)
        ref = 0.5 * (O.iso_elastic_C(self.K, self.G) + O.iso_elastic_C(*elastic_params))
        self.P = O.OracleProblem(ph.reshape(self.ms.shape), L, 3, groups, "HEX8", kapparef=ref)
        self.kapparef = ref

    def run(self, path, tol=1e-12, n_it=5000):
        """The forward path; returns the final <sigma> and the per-step states."""
        P = self.P
        states = []
        for g in path:
            ep0, q0 = P.ep_t.copy(), P.q_t.copy()
            P.set_gradient(np.asarray(g, dtype=float))
            P.solve(measure="L2", type="absolute", tol=tol, n_it=n_it)
            states.append((P.u.copy(), np.asarray(g, dtype=float), ep0, q0))
            P.extrapolate_displacement()
        # undo the last extrapolation so that P.u is the converged final field
        P.u[...] = P.u_prev
        return P.homogenized_stress(), states

    def adjoint(self, path, w, tol=1e-12):
        """(final <sigma>, dL/dsy per voxel [x][y][z]) for L = w . <sigma_N>."""
        P = self.P
        stress, states = self.run(path, tol)
        nx, ny, nz = P.nx, P.ny, P.nz
        nel, ngp = nx * ny * nz, P.ngp
        dofs = element_dofs(nx, ny, nz)
        B = P.B.reshape(ngp, 6, 24)
        flat = self.ms.ravel()
        j2 = flat == 0
        Cel = O.iso_elastic_C(*self.elastic_params)
        sy_el = np.where(j2, self.sy.ravel(), 0.0)
        cw = np.asarray(w, dtype=float) / (nel * ngp)
        mu = np.zeros((nel, ngp, 7))
        grad = np.zeros(nel)
        Nst = len(states)
        for n in range(Nst, 0, -1):
            u, g0, ep0, q0 = states[n - 1]
            e = gp_strain(P, u, g0, dofs)
            Kb = np.full((nel, ngp), self.K)
            Gb = np.full((nel, ngp), self.G)
            J = j2_jacobian(Kb, Gb, self.h, np.repeat(sy_el[:, None], ngp, 1), e, ep0, q0)
            # elastic voxels: sigma = C e, no internal variables
            J[~j2] = 0.0
            J[~j2, :, :6, :6] = Cel
            Se, Sa, Sy = J[..., :6, :6], J[..., :6, 6:13], J[..., :6, 13]
            Ae, Aa, Ay = J[..., 6:, :6], J[..., 6:, 6:13], J[..., 6:, 13]
            seed = cw if n == Nst else np.zeros(6)
            h_gp = np.einsum("egij,i->egj", Se, seed) + np.einsum("egij,egi->egj", Ae, mu)
            f = np.zeros(3 * nel)
            np.add.at(f, dofs, np.einsum("gik,egi->ek", B, h_gp))
            Kd = np.zeros((3 * nel, 3 * nel))
            ke = np.einsum("gia,egji,gjb->eab", B, Se, B) * (P.ve / ngp)  # K_n^T
            np.add.at(Kd, (dofs[:, :, None], dofs[:, None, :]), ke)
            lam = np.linalg.lstsq(Kd, -f, rcond=None)[0]
            le = lam[dofs]
            tau = (P.ve / ngp) * np.einsum("gik,ek->egi", B, le) + seed
            grad += (np.einsum("egi,egi->eg", Sy, tau) + np.einsum("egi,egi->eg", Ay, mu)).sum(1)
            mu = np.einsum("egij,egi->egj", Sa, tau) + np.einsum("egij,egi->egj", Aa, mu)
        return stress, grad.reshape(self.ms.shape)
