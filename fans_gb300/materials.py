"""Host mirror of FANS's MaterialManager and Matmodel parameter handling.

Parses the JSON `materials` array (or the legacy top-level `matmodel` +
`material_properties`, MaterialManager.h:38-65) into a phase table and
computes the reference stiffness `kapparef_mat` by the reference's rule
(MaterialManager.h:177-205): the user's `reference_material` if given (checked
symmetric positive definite), else the mean over material groups of each
model's get_reference_stiffness().
"""
from __future__ import annotations

import json

import numpy as np

from . import _lib as C

# matmodel name -> (law id, problem kind, parameter builder)
#   parameter builders take the group's material_properties and the phase's
#   position in the group (local_mat_id) and return the per-phase vector.


def _iso_thermal(props, i):
    return [float(props["conductivity"][i])]


def _iso_elastic(props, i):
    return [float(props["bulk_modulus"][i]), float(props["shear_modulus"][i])]


def _pseudo_lin(props, i):
    # plastic_flag values: index in the group and group size (PseudoPlastic.h:103-108)
    return [float(props["bulk_modulus"][i]), float(props["shear_modulus"][i]), float(props["yield_stress"][i]),
            float(props["hardening_parameter"][i]), float(i), float(len(props["bulk_modulus"]))]


def _pseudo_nl(props, i):
    return [float(props["bulk_modulus"][i]), float(props["shear_modulus"][i]), float(props["yield_stress"][i]),
            float(props["hardening_exponent"][i]), float(props["eps_0"][i]), float(i),
            float(len(props["bulk_modulus"]))]


def _j2visco(nonlinear):
    def build(props, i):  # J2Plasticity.h:12-20, :190-199
        p = [float(props["bulk_modulus"][i]), float(props["shear_modulus"][i]), float(props["yield_stress"][i]),
             float(props["isotropic_hardening_parameter"][i]), float(props["kinematic_hardening_parameter"][i]),
             float(props["viscosity"][i]), float(props["time_step"])]
        if nonlinear:
            p += [float(props["saturation_stress"][i]), float(props["saturation_exponent"][i])]
        return p

    return build


def _large(props, i):  # SaintVenantKirchhoff.h:17-31, CompressibleNeoHookean.h:19-33
    return [float(props["bulk_modulus"][i]), float(props["shear_modulus"][i])]


def _j2(props, i):
    return [float(props["bulk_modulus"][i]), float(props["shear_modulus"][i]), float(props["yield_stress"][i]),
            float(props["isotropic_hardening_parameter"][i])]


_TRI_T = ["K_11", "K_12", "K_13", "K_22", "K_23", "K_33"]
_TRI_E = ["C_11", "C_12", "C_13", "C_14", "C_15", "C_16", "C_22", "C_23", "C_24", "C_25", "C_26", "C_33", "C_34",
          "C_35", "C_36", "C_44", "C_45", "C_46", "C_55", "C_56", "C_66"]


def _tri(keys, n):
    def build(props, i):
        M = np.zeros((n, n))
        k = 0
        for r in range(n):
            for c in range(r, n):
                M[r, c] = M[c, r] = float(props[keys[k]][i])
                k += 1
        return list(M.ravel())

    return build


MODELS = {
    "LinearThermalIsotropic": (C.LAW_THERMAL_ISO, "thermal", _iso_thermal),
    "LinearThermalTriclinic": (C.LAW_THERMAL_TRI, "thermal", _tri(_TRI_T, 3)),
    "LinearElasticIsotropic": (C.LAW_ELASTIC_ISO, "mechanical", _iso_elastic),
    "LinearElasticTriclinic": (C.LAW_ELASTIC_TRI, "mechanical", _tri(_TRI_E, 6)),
    "J2PlasticityNew_LinearIsotropicHardening": (C.LAW_J2_LINEAR, "mechanical", _j2),
    "PseudoPlasticLinearHardening": (C.LAW_PSEUDO_LINEAR, "mechanical", _pseudo_lin),
    "PseudoPlasticNonLinearHardening": (C.LAW_PSEUDO_NONLINEAR, "mechanical", _pseudo_nl),
    "J2ViscoPlastic_LinearIsotropicHardening": (C.LAW_J2VISCO_LINEAR, "mechanical", _j2visco(False)),
    "J2ViscoPlastic_NonLinearIsotropicHardening": (C.LAW_J2VISCO_NONLINEAR, "mechanical", _j2visco(True)),
    "SaintVenantKirchhoff": (C.LAW_SVK, "mechanical_large", _large),
    "CompressibleNeoHookean": (C.LAW_NEOHOOKEAN, "mechanical_large", _large),
}


NONLINEAR_LAWS = (C.LAW_J2_LINEAR, C.LAW_PSEUDO_LINEAR, C.LAW_PSEUDO_NONLINEAR, C.LAW_J2VISCO_LINEAR,
                  C.LAW_J2VISCO_NONLINEAR, C.LAW_SVK, C.LAW_NEOHOOKEAN)
LARGE_STRAIN_LAWS = (C.LAW_SVK, C.LAW_NEOHOOKEAN)


def large_strain_tangent(K, G):
    """dP/dF at F = I (row 3i + J, column 3k + L) as
    LargeStrainMechModel::compute_spatial_tangent (LargeStrainMechModel.h:96-170)
    assembles it from the Mandel tangent lambda 1 1^T + 2 mu I that both
    SaintVenantKirchhoff and CompressibleNeoHookean have at F = I (S = 0).  That
    loop visits each symmetric pair (P, Q) once with dE_PQ/dF_kL =
    (F_kP d_QL + F_kQ d_PL)/2, so entries with k != L carry half of
    lambda d_iJ d_kL + mu (d_ik d_JL + d_iL d_Jk)."""
    lam, mu = K - 2.0 / 3.0 * G, G
    A = np.zeros((9, 9))
    d = np.eye(3)
    for i in range(3):
        for J in range(3):
            for k in range(3):
                for L in range(3):
                    v = lam * d[i, J] * d[k, L] + mu * (d[i, k] * d[J, L] + d[i, L] * d[J, k])
                    A[3 * i + J, 3 * k + L] = v if k == L else 0.5 * v
    return A


def iso_elastic_C(K, G):
    lam = K - 2.0 / 3.0 * G
    M = np.zeros((6, 6))
    M[:3, :3] = lam
    M += 2.0 * G * np.eye(6)
    return M


def group_reference_stiffness(law, params):
    """Matmodel::get_reference_stiffness for one material group."""
    if law == C.LAW_THERMAL_ISO:  # LinearThermal.h:21-31, :49-52 (kappa_average)
        return np.mean([p[0] for p in params]) * np.eye(3)
    if law == C.LAW_ELASTIC_ISO:  # LinearElastic.h:55-70 ((max+min)/2 of lambda, mu)
        lam = [p[0] - 2.0 / 3.0 * p[1] for p in params]
        mu = [p[1] for p in params]
        lr, mr = (max(lam) + min(lam)) / 2, (max(mu) + min(mu)) / 2
        M = np.zeros((6, 6))
        M[:3, :3] = lr
        return M + 2 * mr * np.eye(6)
    if law in LARGE_STRAIN_LAWS:  # SaintVenantKirchhoff.h:61-80, CompressibleNeoHookean.h:108-121
        return np.mean([large_strain_tangent(p[0], p[1]) for p in params], axis=0)
    if law in NONLINEAR_LAWS:
        # J2PlasticityNew.h:111-121, PseudoPlastic.h:41-51, J2Plasticity.h:113-124 (mean K, G)
        Kb, Gb = np.mean([p[0] for p in params]), np.mean([p[1] for p in params])
        M = np.zeros((6, 6))
        M[:3, :3] = Kb - 2.0 * Gb / 3.0
        M[np.diag_indices(6)] += 2.0 * Gb
        return M
    n = 3 if law == C.LAW_THERMAL_TRI else 6  # triclinic: mean C (LinearElastic.h:146-154)
    return np.mean([np.asarray(p).reshape(n, n) for p in params], axis=0)


def gb_diffusion_tensors(props, gb_info):
    """GBDiffusion phase conductivities (GBDiffusion.h:45-118): crystals (tags below
    num_crystals) D_bulk I, grain boundaries D_par (I - n n^T) + D_perp n n^T with the
    normalised GB normal of the tag.  `gb_info` holds num_crystals, num_GB and the
    GBVoxelInfo JSON of the microstructure dataset's attributes."""
    nc, ngb = int(gb_info["num_crystals"]), int(gb_info["num_GB"])
    n_mat = nc + ngb
    info = gb_info["GBVoxelInfo"]
    info = json.loads(info) if isinstance(info, (str, bytes)) else info
    normals = np.zeros((n_mat, 3))
    for v in info.values():
        normals[int(v["GB_tag"])] = np.asarray(v["GB_normal"], dtype=float)
    if props["GB_unformity"]:
        Db, Dpa, Dpe = np.zeros(n_mat), np.zeros(n_mat), np.zeros(n_mat)
        Db[:nc] = float(props["D_bulk"])
        Dpa[nc:] = float(props["D_par"])
        Dpe[nc:] = float(props["D_perp"])
    else:
        Db, Dpa, Dpe = (np.asarray(props[k][:n_mat], dtype=float) for k in ("D_bulk", "D_par", "D_perp"))
    out = []
    for i in range(n_mat):
        if i < nc:
            K = Db[i] * np.eye(3)
        else:
            n = normals[i] / np.linalg.norm(normals[i])
            K = Dpa[i] * (np.eye(3) - np.outer(n, n)) + Dpe[i] * np.outer(n, n)
        out.append(list(K.ravel()))
    return out, normals


class MaterialManager:
    """Phase id -> (law, parameters) table plus the reference stiffness.

    `gb_info` supplies the microstructure attributes a GBDiffusion group needs
    (num_crystals, num_GB, GBVoxelInfo); the driver reads them from the HDF5
    dataset as GBDiffusion.h:50-60 does."""

    def __init__(self, input_json: dict, problem_type: str | None = None, gb_info: dict | None = None,
                 strain_type: str = "small"):
        if "matmodel" in input_json and "material_properties" in input_json:
            props = input_json["material_properties"]
            n = next(len(v) for v in props.values() if isinstance(v, list))
            mats = [{"matmodel": input_json["matmodel"], "material_properties": props, "phases": list(range(n))}]
        else:
            mats = input_json.get("materials")
        if not isinstance(mats, list) or not mats:
            raise RuntimeError("MaterialManager: 'materials' must be non-empty array")
        for mg in mats:
            if not all(k in mg for k in ("phases", "matmodel", "material_properties")):
                raise RuntimeError("MaterialManager: material group missing required fields")
        n_phases = 1 + max(max(mg["phases"]) for mg in mats)
        self.n_phases = n_phases
        self.law = [None] * n_phases
        self.params = [None] * n_phases
        self.groups = []
        self.all_linear = True
        refs = []
        self.gb_normals = None
        for mg in mats:
            name = mg["matmodel"]
            if name == "GBDiffusion":
                if problem_type is not None and problem_type != "thermal":
                    raise ValueError(f"{name} is not a valid matmodel for {problem_type} problem")
                if gb_info is None:
                    raise RuntimeError("Error in GBDiffusion initialization: microstructure attributes missing")
                tensors, self.gb_normals = gb_diffusion_tensors(mg["material_properties"], gb_info)
                gparams = []
                for i, ph in enumerate(mg["phases"]):
                    if ph < 0 or ph >= n_phases or self.law[ph] is not None:
                        raise RuntimeError(f"MaterialManager: Invalid or duplicate phase {ph}")
                    self.law[ph] = C.LAW_THERMAL_TRI
                    self.params[ph] = tensors[i]
                    gparams.append(tensors[i])
                self.groups.append((name, C.LAW_THERMAL_TRI, list(mg["phases"]), gparams))
                refs.append(np.mean([np.asarray(p).reshape(3, 3) for p in tensors], axis=0))  # kappa_average
                continue
            if name not in MODELS:
                raise ValueError(f"{name} is not a valid matmodel")
            law, kind, builder = MODELS[name]
            want = problem_type
            if problem_type == "mechanical" and strain_type == "large":
                want = "mechanical_large"
            if problem_type is not None and kind != want:  # setup.h:22-73
                what = {"thermal": "matmodel for thermal problem", "mechanical": "small strain material model",
                        "mechanical_large": "large strain material model"}[want]
                raise ValueError(f"{name} is not a valid {what}")
            gparams = []
            for i, ph in enumerate(mg["phases"]):
                if ph < 0 or ph >= n_phases or self.law[ph] is not None:
                    raise RuntimeError(f"MaterialManager: Invalid or duplicate phase {ph}")
                try:
                    prm = builder(mg["material_properties"], i)
                except (KeyError, IndexError) as e:
                    raise RuntimeError("Missing material properties for the requested material model.") from e
                self.law[ph] = law
                self.params[ph] = prm
                gparams.append(prm)
            if law in NONLINEAR_LAWS:
                self.all_linear = False
            self.groups.append((name, law, list(mg["phases"]), gparams))
            refs.append(group_reference_stiffness(law, gparams))
        for ph in range(n_phases):
            if self.law[ph] is None:
                raise RuntimeError(f"MaterialManager: Phase {ph} not assigned")
        self.n_str = refs[0].shape[0]
        if "reference_material" in input_json:
            ref = np.asarray(input_json["reference_material"], dtype=float)
            if ref.shape != (self.n_str, self.n_str):
                raise ValueError(f"reference_material must be {self.n_str}x{self.n_str}")
            try:
                np.linalg.cholesky(ref)
            except np.linalg.LinAlgError as e:
                raise ValueError("reference_material must be symmetric positive definite") from e
            self.kapparef_mat = ref
        else:
            self.kapparef_mat = np.mean(refs, axis=0)

    def apply(self, solver):
        """Push the phase table and reference stiffness into a GPU context."""
        for ph in range(self.n_phases):
            solver.set_phase_material(ph, self.law[ph], self.params[ph])
        solver.set_reference(self.kapparef_mat)
