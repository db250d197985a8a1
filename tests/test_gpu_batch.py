"""fansgpu_solve_batch: independent contexts solved concurrently (one host
thread and CUDA stream each) give the same results as solving them one after
another -- the kernels and reductions are deterministic, so the stresses are
bit-identical -- for a mix of thermal and elastic, FP64 and mixed contexts."""
import numpy as np
import pytest

from fans_gb300 import Context, solve_batch
from fans_gb300.microstructure import spheres

pytestmark = pytest.mark.gpu


def _ctx(n, thermal, precision, seed):
    ms, _ = spheres(n, 3, 0.25, seed)
    if thermal:
        c = Context((n, n, n), (1.0, 1.0, 1.0), 1, "HEX8", precision, "cg")
        c.set_microstructure(ms)
        c.set_phase_material(0, 0, [1.0])
        c.set_phase_material(1, 0, [10.0])
        c.set_reference(5.5 * np.eye(3))
    else:
        from helpers import ELASTIC
        import oracle as O

        c = Context((n, n, n), (1.0, 1.0, 1.0), 3, "HEX8", precision, "cg")
        c.set_microstructure(ms)
        for ph, prm in enumerate(ELASTIC[0][2]):
            c.set_phase_material(ph, 1, prm)
        lam = [p[0] - 2 / 3 * p[1] for p in ELASTIC[0][2]]
        mu = [p[1] for p in ELASTIC[0][2]]
        C0 = np.zeros((6, 6))
        C0[:3, :3] = sum(lam) / 2
        C0 += sum(mu) * np.eye(6)
        c.set_reference(C0)
    c.set_tolerance("L2", "relative", 1e-8, 1000)
    return c


def test_batch_equals_sequential():
    specs = [(16, True, "fp64"), (24, False, "mixed"), (32, True, "mixed"), (16, False, "fp64"),
             (32, False, "mixed"), (24, True, "fp64")]
    ctxs = [_ctx(n, t, p, 10 + i) for i, (n, t, p) in enumerate(specs)]
    for c in ctxs:
        g = np.zeros(c.n_str)
        g[0] = 1.0
        c.set_gradient(g)
    seq = []
    for c in ctxs:
        c.reset()
        st = c.solve()
        seq.append((st["iterations"], c.homogenized_stress()))
    for c in ctxs:
        c.reset()
    sts = solve_batch(ctxs)
    for (it, sig), st, c in zip(seq, sts, ctxs):
        assert st["converged"] and st["rc"] == 0
        assert st["iterations"] == it
        assert np.array_equal(c.homogenized_stress(), sig)
    for c in ctxs:
        c.close()


def test_batch_rejects_repeated_context():
    c = _ctx(16, True, "fp64", 1)
    with pytest.raises(Exception):
        solve_batch([c, c])
    c.close()
