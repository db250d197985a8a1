"""Shared builders for parity tests: the same problem as an oracle instance and
as a GPU context (through the C ABI)."""
from __future__ import annotations

import numpy as np

import oracle as O

# material groups used across tests (law ids match fans_gb300._lib)
THERMAL = [(O.LAW_THERMAL_ISO, [0, 1], [[1.0], [10.0]])]
ELASTIC = [(O.LAW_ELASTIC_ISO, [0, 1], [[3.3333333333333335, 1.1111111111111112], [41.666666666666664, 28.688524590163933]])]
ELASTIC_FIXTURE = [(O.LAW_ELASTIC_ISO, [0, 1], [[62.5, 28.8462], [222.222, 166.6667]])]


def random_ms(shape, vf=0.3, seed=0, nphase=2):
    rng = np.random.default_rng(seed)
    if nphase == 2:
        return (rng.random(shape) < vf).astype(np.uint16)
    return rng.integers(0, nphase, size=shape).astype(np.uint16)


def oracle_problem(ms, c, groups, fe="HEX8", L=(1.0, 1.0, 1.0), kapparef=None, strain_type="small"):
    return O.OracleProblem(ms, L, c, groups, fe, kapparef=kapparef, strain_type=strain_type)


def gpu_context(P, precision="fp64", method="cg"):
    """GPU context mirroring oracle problem P (same phases, reference, FE type)."""
    from fans_gb300 import Context

    fe = {O.HEX8: "HEX8", O.HEX8R: "HEX8R", O.BBAR: "BBAR"}[P.fe]
    ctx = Context((P.nx, P.ny, P.nz), tuple(P.L), P.c, fe, precision, method, "large" if P.large else "small")
    ctx.set_microstructure(P.ms)
    nparams = {O.LAW_THERMAL_ISO: 1, O.LAW_ELASTIC_ISO: 2, O.LAW_J2: 4, O.LAW_THERMAL_TRI: 9, O.LAW_ELASTIC_TRI: 36,
               O.LAW_PSEUDO_LIN: 4, O.LAW_PSEUDO_NL: 5, O.LAW_J2VISCO_LIN: 7, O.LAW_J2VISCO_NL: 9,
               O.LAW_SVK: 2, O.LAW_NEOHOOKEAN: 2}
    for ph in range(P.nphase):
        law = int(P.law[ph])
        ctx.set_phase_material(ph, law, P.param[ph, : nparams[law]])
    ctx.set_reference(P.kapparef)
    return ctx


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))
