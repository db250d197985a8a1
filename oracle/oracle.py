"""Python side of the oracle: ctypes binding of fans_oracle.c plus the
reference's host-side rules the oracle needs (reference stiffness, phase
parameter packing).

TEST INFRASTRUCTURE ONLY.  This module is the checker for the CUDA product.
Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline / reference
arm may import it; the product package never does.

Parity pinning: the reference (FANS v0.6.2) cannot be built in this image (MPI,
FFTW3-MPI, parallel HDF5, Eigen and nlohmann_json are absent).  Its test inputs
test/input_files/test_MixedBCs.json and test_MixedBCs_LargeStrain.json carry
macroscopic states the reference computed on test/microstructures/sphere32.h5
(the loading of their later load cases), and the oracle reproduces them
(tests/test_oracle_reference_pins.py): small-strain mixed BCs with
PseudoPlasticLinearHardening + linear elasticity, and CompressibleNeoHookean
at large strain.  Everything else is anchored by (1) an independent numpy
restatement (numpy.fft / LAPACK eigh) of the same reference lines, (2) known
answers (homogeneous media, laminates, strain-energy derivatives), and (3) the
reference tests' invariants on sphere32 -- for the laws the two files do not
exercise, parity is unpinned.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libfans_oracle.so")

HEX8, HEX8R, BBAR = 0, 1, 2
FE_TYPES = {"HEX8": HEX8, "HEX8R": HEX8R, "BBAR": BBAR}
LAW_THERMAL_ISO, LAW_ELASTIC_ISO, LAW_J2, LAW_THERMAL_TRI, LAW_ELASTIC_TRI = 0, 1, 2, 3, 4
LAW_PSEUDO_LIN, LAW_PSEUDO_NL = 5, 6
LAW_J2VISCO_LIN, LAW_J2VISCO_NL = 7, 8
LAW_SVK, LAW_NEOHOOKEAN = 9, 10
LARGE_STRAIN_LAWS = (LAW_SVK, LAW_NEOHOOKEAN)
NONLINEAR_LAWS = (LAW_J2, LAW_PSEUDO_LIN, LAW_PSEUDO_NL, LAW_J2VISCO_LIN, LAW_J2VISCO_NL) + LARGE_STRAIN_LAWS
L1, L2, LINF = 0, 1, 2
ABS, REL = 0, 1
MEASURES = {"L1": L1, "L2": L2, "Linfinity": LINF}
TYPES = {"absolute": ABS, "relative": REL}
PARAM_STRIDE = 36


def build(force: bool = False) -> str:
    """Compile fans_oracle.c into libfans_oracle.so (gcc, OpenMP)."""
    src = os.path.join(HERE, "fans_oracle.c")
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= os.path.getmtime(src):
        return LIB_PATH
    cmd = ["gcc", "-O3", "-fopenmp", "-fPIC", "-shared", "-std=c11", "-o", LIB_PATH, src, "-lm"]
    subprocess.check_call(cmd)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(LIB_PATH)
        _declare(_lib)
    return _lib


_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_u16p = ctypes.POINTER(ctypes.c_uint16)
_lp = ctypes.POINTER(ctypes.c_long)


def _declare(L):
    L.fo_bind_kinematic.argtypes = [ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
    L.fo_bind_kinematic.restype = None
    L.fo_set_large_strain.argtypes = [ctypes.c_int]
    L.fo_set_large_strain.restype = None
    i, d, sz = ctypes.c_int, ctypes.c_double, ctypes.c_size_t
    L.fo_build_B.argtypes = [i, i, _dp, _dp]
    L.fo_build_B.restype = i
    L.fo_element_stiffness.argtypes = [i, i, _dp, _dp, d, _dp]
    L.fo_green.argtypes = [i, i, i, i, _dp, _dp]
    L.fo_rfft3.argtypes = [i, i, i, _dp, i, _dp, _dp]
    L.fo_irfft3.argtypes = [i, i, i, _dp, _dp, _dp, i]
    L.fo_convolve.argtypes = [i, i, i, i, _dp, _dp, _dp]
    common = [i, i, i, i, i, d, _dp, _u16p, i, _ip, _dp, _dp, _dp, _dp, _dp, _dp]
    L.fo_residual.argtypes = common + [_dp, _dp]
    L.fo_apply_linear.argtypes = [i, i, i, i, _u16p, _dp, _dp, _dp]
    L.fo_strain_stress.argtypes = common + [_dp, _dp, _dp, _dp, _dp, _dp, _dp, _lp]
    L.fo_norm.argtypes = [sz, _dp, i]
    L.fo_norm.restype = d
    L.fo_cg_solve.argtypes = common + [_dp, _dp, i, i, i, d, i, i, d, _dp, _dp, _dp]
    L.fo_cg_solve.restype = i
    L.fo_fp_solve.argtypes = common + [_dp, i, i, d, i, _dp, _dp, _dp]
    L.fo_fp_solve.restype = i
    L.fo_num_threads.restype = i
    L.fo_set_num_threads.argtypes = [i]


def _p(a, t=_dp):
    if a is None:
        return ctypes.cast(None, t)
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(t)


# ---------------------------------------------------------------------------
# Reference host rules restated for the oracle
# ---------------------------------------------------------------------------

def iso_elastic_C(K, G):
    """6x6 Mandel stiffness: topLeft(3,3)=lambda, + 2 mu I (LinearElastic.h:28-35)."""
    lam = K - 2.0 / 3.0 * G
    C = np.zeros((6, 6))
    C[:3, :3] = lam
    C += 2.0 * G * np.eye(6)
    return C


_MANDEL_PAIRS = [(0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2)]


def spatial_tangent(F, S, Cm):
    """LargeStrainMechModel::compute_spatial_tangent (LargeStrainMechModel.h:96-170):
    A[3i+J, 3k+L] = d_ik S_LJ + sum_M F_iM sum_{P<=Q} C_MJPQ (F_kP d_QL + F_kQ d_PL)/2,
    C_MJPQ read from the 6x6 Mandel tangent with its sqrt(2) shear factors divided out."""
    def mandel(a, b):
        return next(i for i, (x, y) in enumerate(_MANDEL_PAIRS) if (x, y) in ((a, b), (b, a)))

    A = np.zeros((9, 9))
    for i in range(3):
        for J in range(3):
            for k in range(3):
                for L in range(3):
                    v = S[L, J] if i == k else 0.0
                    for M in range(3):
                        mj = mandel(M, J)
                        for P in range(3):
                            for Q in range(P, 3):
                                pq = mandel(P, Q)
                                c = Cm[mj, pq] / (np.sqrt(2.0) if mj >= 3 else 1.0) / (np.sqrt(2.0) if pq >= 3 else 1.0)
                                dE = (0.5 * F[k, P] if Q == L else 0.0) + (0.5 * F[k, Q] if P == L else 0.0)
                                v += F[i, M] * c * dE
                    A[3 * i + J, 3 * k + L] = v
    return A


def large_strain_tangent_at_identity(law, params):
    """get_reference_stiffness of one phase of SaintVenantKirchhoff
    (SaintVenantKirchhoff.h:61-80) or CompressibleNeoHookean
    (CompressibleNeoHookean.h:108-121): both have S = 0 and the Mandel tangent
    lambda 1 1^T + 2 mu I at F = I (CompressibleNeoHookean.h:52-104 with C^-1 = I)."""
    K, G = float(params[0]), float(params[1])
    lam, mu = K - 2.0 / 3.0 * G, G
    Cm = np.zeros((6, 6))
    Cm[:3, :3] = lam
    Cm += 2.0 * mu * np.eye(6)
    return spatial_tangent(np.eye(3), np.zeros((3, 3)), Cm)


def law_C(law, params):
    if law in LARGE_STRAIN_LAWS:
        return large_strain_tangent_at_identity(law, params)
    if law == LAW_THERMAL_ISO:
        return params[0] * np.eye(3)
    if law in (LAW_ELASTIC_ISO,) + NONLINEAR_LAWS:
        return iso_elastic_C(params[0], params[1])
    if law == LAW_THERMAL_TRI:
        return np.asarray(params[:9], dtype=float).reshape(3, 3)
    if law == LAW_ELASTIC_TRI:
        return np.asarray(params[:36], dtype=float).reshape(6, 6)
    raise ValueError(law)


def model_reference_stiffness(law, phase_params):
    """Matmodel::get_reference_stiffness of one material group.

    LinearThermalIsotropic: mean conductivity (LinearThermal.h:21-31, :49-52);
    LinearElasticIsotropic: (max+min)/2 of lambda and mu (LinearElastic.h:55-70);
    J2PlasticityNew: mean K and G (J2PlasticityNew.h:111-121);
    triclinic: mean C (LinearElastic.h:146-154, LinearThermal.h:103-110)."""
    pp = [np.asarray(p, dtype=float) for p in phase_params]
    if law == LAW_THERMAL_ISO:
        return np.mean([p[0] for p in pp]) * np.eye(3)
    if law == LAW_ELASTIC_ISO:
        lam = [p[0] - 2.0 / 3.0 * p[1] for p in pp]
        mu = [p[1] for p in pp]
        lr = (max(lam) + min(lam)) / 2
        mr = (max(mu) + min(mu)) / 2
        C = np.zeros((6, 6))
        C[:3, :3] = lr
        C += 2 * mr * np.eye(6)
        return C
    if law in LARGE_STRAIN_LAWS:
        return np.mean([large_strain_tangent_at_identity(law, p) for p in pp], axis=0)
    if law in NONLINEAR_LAWS:  # J2PlasticityNew.h:111-121, PseudoPlastic.h:41-51
        Kb = np.mean([p[0] for p in pp])
        Gb = np.mean([p[1] for p in pp])
        C = np.zeros((6, 6))
        C[:3, :3] = Kb - 2.0 * Gb / 3.0
        C[np.diag_indices(6)] += 2.0 * Gb
        return C
    return np.mean([law_C(law, p) for p in pp], axis=0)


class OracleProblem:
    """A FANS problem as the oracle sees it (one MaterialManager + Solver).

    groups: list of (law, [phase ids], [per-phase parameter vectors]) in the
    order of the JSON 'materials' array."""

    def __init__(self, ms, L, c, groups, fe_type="HEX8", kapparef=None, strain_type="small"):
        self.ms = np.ascontiguousarray(ms, dtype=np.uint16)
        self.nx, self.ny, self.nz = self.ms.shape
        self.c = c
        self.large = c == 3 and strain_type == "large"
        self.nstr = 3 if c == 1 else (9 if self.large else 6)
        lib().fo_set_large_strain(int(self.large))
        self.fe = FE_TYPES[fe_type] if isinstance(fe_type, str) else fe_type
        self.L = np.asarray(L, dtype=float)
        self.le = np.array([self.L[0] / self.nx, self.L[1] / self.ny, self.L[2] / self.nz])
        self.ve = float(self.le[0] * self.le[1] * self.le[2])
        B = np.zeros(8 * 9 * 24)
        self.ngp = lib().fo_build_B(self.fe, c, _p(self.le), _p(B))
        self.B = np.ascontiguousarray(B[: self.ngp * self.nstr * 8 * c])
        nphase = 1 + max(max(ph) for _, ph, _ in groups)
        self.nphase = nphase
        self.law = np.zeros(nphase, dtype=np.int32)
        self.param = np.zeros((nphase, PARAM_STRIDE))
        self.linear = True
        refs = []
        for law, phases, params in groups:
            for ph, pr in zip(phases, params):
                self.law[ph] = law
                pr = np.asarray(pr, dtype=float).ravel()
                self.param[ph, : pr.size] = pr
            if law in NONLINEAR_LAWS:
                self.linear = False
            refs.append(model_reference_stiffness(law, params))
        # MaterialManager::compute_reference_stiffness (MaterialManager.h:177-205)
        self.kapparef = np.mean(refs, axis=0) if kapparef is None else np.asarray(kapparef, dtype=float)
        self.Kph = np.zeros((nphase, 8 * c, 8 * c))
        for ph in range(nphase):
            C = np.ascontiguousarray(law_C(self.law[ph], self.param[ph]))
            lib().fo_element_stiffness(c, self.ngp, _p(self.B), _p(C), self.ve, _p(self.Kph[ph]))
        self.K0 = np.zeros((8 * c, 8 * c))
        lib().fo_element_stiffness(c, self.ngp, _p(self.B), _p(np.ascontiguousarray(self.kapparef)), self.ve,
                                   _p(self.K0))
        nel = self.nx * self.ny * self.nz
        self.ep_t = np.zeros((nel, self.ngp, 6)) if not self.linear else np.zeros(6)
        self.q_t = np.zeros((nel, self.ngp)) if not self.linear else np.zeros(1)
        self.ep = self.ep_t.copy()
        self.q = self.q_t.copy()
        # J2ViscoPlastic kinematic hardening psi_bar [N][ngp][6] (committed, trial)
        self.pb_t = np.zeros((nel, self.ngp, 6)) if not self.linear else np.zeros(6)
        self.pb = self.pb_t.copy()
        self.g0 = np.zeros(self.nstr)
        self.u = np.zeros((self.nx, self.ny, self.nz, c))
        self.u_prev = np.zeros_like(self.u)
        self._G = None

    # -- pieces --------------------------------------------------------------
    @property
    def G(self):
        if self._G is None:
            nzh = self.nz // 2 + 1
            nt = self.c * (self.c + 1) // 2
            G = np.zeros((self.nx, self.ny, nzh, nt))
            lib().fo_green(self.nx, self.ny, self.nz, self.c, _p(self.K0), _p(G))
            self._G = G
        return self._G

    def _common(self):
        lib().fo_bind_kinematic(_p(self.pb_t), _p(self.pb))
        lib().fo_set_large_strain(int(self.large))
        return (self.nx, self.ny, self.nz, self.c, self.ngp, self.ve, _p(self.B), _p(self.ms, _u16p), self.nphase,
                _p(self.law, _ip), _p(self.param), _p(self.g0), _p(self.ep_t), _p(self.q_t), _p(self.ep),
                _p(self.q))

    def set_gradient(self, g0):
        self.g0 = np.ascontiguousarray(g0, dtype=float)

    def residual(self, u=None):
        u = self.u if u is None else np.ascontiguousarray(u, dtype=float)
        r = np.zeros_like(u)
        lib().fo_residual(*self._common(), _p(u), _p(r))
        return r

    def apply_linear(self, d):
        d = np.ascontiguousarray(d, dtype=float)
        out = np.zeros_like(d)
        lib().fo_apply_linear(self.nx, self.ny, self.nz, self.c, _p(self.ms, _u16p), _p(self.Kph), _p(d), _p(out))
        return out

    def convolve(self, r):
        r = np.ascontiguousarray(r, dtype=float)
        s = np.zeros_like(r)
        lib().fo_convolve(self.nx, self.ny, self.nz, self.c, _p(self.G), _p(r), _p(s))
        return s

    def strain_stress(self, u=None, fields=False):
        u = self.u if u is None else np.ascontiguousarray(u, dtype=float)
        N = self.nx * self.ny * self.nz
        strain = np.zeros((N, self.nstr)) if fields else None
        stress = np.zeros((N, self.nstr)) if fields else None
        a_e, a_s = np.zeros(self.nstr), np.zeros(self.nstr)
        p_e, p_s = np.zeros((self.nphase, self.nstr)), np.zeros((self.nphase, self.nstr))
        cnt = np.zeros(self.nphase, dtype=np.int64)
        lib().fo_strain_stress(*self._common(), _p(u), _p(strain), _p(stress), _p(a_e), _p(a_s), _p(p_e), _p(p_s),
                               _p(cnt, _lp))
        return dict(strain=strain, stress=stress, strain_average=a_e, stress_average=a_s, phase_strain=p_e,
                    phase_stress=p_s, phase_count=cnt)

    def homogenized_stress(self):
        return self.strain_stress()["stress_average"]

    # -- mixed stress/strain boundary conditions (mixedBCs.h:149-227) ----------
    mixed_active = False

    def enable_mixed_bc(self, idx_E, strain_E, idx_F, stress_F, step):
        """MixedBCController::activate (mixedBCs.h:180-226) with MixedBC::finalize
        (mixedBCs.h:30-48): M = pinv(Q_F^T C0 Q_F); step 0 starts from g0 = 0, later
        steps extrapolate the stress-controlled components; then one update."""
        self.idx_E, self.idx_F = list(idx_E), list(idx_F)
        self.mbc_PF = np.asarray(stress_F, dtype=float)
        C0 = np.asarray(self.kapparef, dtype=float)
        self.mbc_M = np.linalg.pinv(C0[np.ix_(self.idx_F, self.idx_F)]) if self.idx_F else np.zeros((0, 0))
        g0 = np.asarray(self.g0, dtype=float).copy()
        if step == 0:  # large strain starts from F = I (mixedBCs.h:192-201)
            g0 = np.eye(3).ravel() if self.nstr == 9 else np.zeros(self.nstr)
            self.g0_prev = g0.copy()
        else:
            delta = g0 - self.g0_prev
            self.g0_prev = g0.copy()
            g0[self.idx_F] += delta[self.idx_F]
        g0[self.idx_E] = np.asarray(strain_E, dtype=float)
        self.g0 = g0
        self.mixed_active = True
        self._mixed_update()

    def disable_mixed_bc(self):
        self.mixed_active = False

    def _mixed_update(self):
        """MixedBCController::update (mixedBCs.h:160-177)."""
        if not self.mixed_active or not self.idx_F:
            return
        Pbar = self.strain_stress()["stress_average"]
        g0 = self.g0.copy()
        g0[self.idx_F] += self.mbc_M @ (self.mbc_PF - Pbar[self.idx_F])
        self.g0 = g0

    def _solve_mixed(self, method, measure, type, tol, n_it, ls_max_iter, ls_tol):
        """SolverCG::internalSolve with mixed BCs active: the line-search branch
        (solverCG.h:96-105, LineSearchSecant :120-160) with an update before every
        residual (:131, :152); SolverFP likewise (solverFP.h:44-48).  Vector algebra
        in numpy; residual, convolution and averages from the C oracle."""
        m = MEASURES[measure]

        def norm(r):
            return np.abs(r).sum() if m == 0 else (np.sqrt((r * r).sum()) if m == 1 else np.abs(r).max())

        err_all = []

        def err(it, r):
            e = norm(r)
            err_all.append(e)
            if type == "absolute":
                return e
            return 100.0 if it == 0 else e / err_all[0]

        u = self.u
        r = self.residual(u)
        it = 0
        err_rel = err(0, r)
        if method == "fp":
            while it < n_it and err_rel > tol:
                u -= self.convolve(r)
                self._mixed_update()
                r = self.residual(u)
                it += 1
                err_rel = err(it, r)
        else:
            s = np.zeros_like(u)
            d = np.zeros_like(u)
            delta, alpha_warm = 1.0, 0.1
            while it < n_it and err_rel > tol:
                deltamid = float((r * s).sum())
                s = -self.convolve(r)
                delta0, delta = delta, float((r * s).sum())
                d = s + max(0.0, (delta - deltamid) / delta0) * d
                e_ls, k, a_prev, a_cur = 10.0, 0, 0.0, alpha_warm
                rpd = float((r * d).sum())
                u += d * a_cur
                self._mixed_update()
                rnew = self.residual(u)
                r1pd = float((rnew * d).sum())
                while k < ls_max_iter and e_ls > ls_tol:
                    denom = r1pd - rpd
                    if abs(denom) < 1e-14 * (abs(r1pd) + abs(rpd)):
                        break
                    a_next = a_cur - r1pd * (a_cur - a_prev) / denom
                    if a_next <= 0.0:
                        a_next = 0.5 * (a_prev + a_cur)
                    e_ls = abs(a_next - a_cur)
                    u += d * (a_next - a_cur)
                    a_prev, rpd, a_cur = a_cur, r1pd, a_next
                    k += 1
                    self._mixed_update()
                    rnew = self.residual(u)
                    r1pd = float((rnew * d).sum())
                alpha_warm = 0.1 if (k == ls_max_iter and e_ls > ls_tol) else a_cur
                r = rnew
                it += 1
                err_rel = err(it, r)
        self.r = r
        self.err_all = np.array(err_all)
        self.iterations = it
        if not self.linear:
            self.ep_t[...] = self.ep
            self.q_t[...] = self.q
            self.pb_t[...] = self.pb
        return it

    def solve(self, method="cg", measure="L2", type="relative", tol=1e-10, n_it=100, ls_max_iter=5, ls_tol=1e-2):
        """Solver::solve (solver.h:283-300): internalSolve then commit internal variables."""
        if self.mixed_active:
            return self._solve_mixed(method, measure, type, tol, n_it, ls_max_iter, ls_tol)
        r = np.zeros_like(self.u)
        err = np.zeros(n_it + 1)
        m, t = MEASURES[measure], TYPES[type]
        if method == "cg":
            it = lib().fo_cg_solve(*self._common(), _p(self.Kph), _p(self.G), int(self.linear), m, t, tol, n_it,
                                   ls_max_iter, ls_tol, _p(self.u), _p(r), _p(err))
        else:
            it = lib().fo_fp_solve(*self._common(), _p(self.G), m, t, tol, n_it, _p(self.u), _p(r), _p(err))
        self.r = r
        self.err_all = err[: it + 1]
        self.iterations = it
        if not self.linear:
            self.ep_t[...] = self.ep
            self.q_t[...] = self.q
            self.pb_t[...] = self.pb
        return it

    def extrapolate_displacement(self):
        """Solver::extrapolateDisplacement (solver.h:303-311)."""
        delta = self.u - self.u_prev
        self.u_prev[...] = self.u
        self.u += delta

    def homogenized_tangent_unit(self, **solve_kw):
        """C_eff from explicit unit-load solves, one per column (the linear branch of
        Solver::get_homogenized_tangent, solver.h:759-776, at the configured tolerance)."""
        C = np.zeros((self.nstr, self.nstr))
        for i in range(self.nstr):
            g = np.zeros(self.nstr)
            g[i] = 1.0
            self.set_gradient(g)
            self.solve(**solve_kw)
            C[:, i] = self.homogenized_stress()
        return 0.5 * (C + C.T)


def rfft3(f):
    """FFTW-convention r2c of a real [x][y][z] array via the C oracle FFT."""
    f = np.ascontiguousarray(f, dtype=float)
    nx, ny, nz = f.shape
    re = np.zeros((nx, ny, nz // 2 + 1))
    im = np.zeros_like(re)
    lib().fo_rfft3(nx, ny, nz, _p(f), 1, _p(re), _p(im))
    return re + 1j * im


def irfft3(spec, nz):
    spec = np.asarray(spec)
    nx, ny, _ = spec.shape
    re = np.ascontiguousarray(spec.real, dtype=float)
    im = np.ascontiguousarray(spec.imag, dtype=float)
    f = np.zeros((nx, ny, nz))
    lib().fo_irfft3(nx, ny, nz, _p(re), _p(im), _p(f), 1)
    return f


def set_threads(n):
    lib().fo_set_num_threads(int(n))


def num_threads():
    return lib().fo_num_threads()
