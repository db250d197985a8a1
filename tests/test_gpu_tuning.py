"""Autotuned tile shapes (FANSGPU_TUNE; the tuner runs on a context's first
setup).  Every forced combination of the register FFT passes' variants (z, y, x)
gives the bitwise-same FP64 convolution and the same mixed-precision solve; the
default (tuned) context agrees with the oracle."""
import numpy as np
import pytest

import oracle as O
from helpers import ELASTIC, gpu_context, oracle_problem, random_ms, rel

pytestmark = pytest.mark.gpu

_ref = {}


def _problem():
    ms = random_ms((32, 32, 64), vf=0.3, seed=21)
    return oracle_problem(ms, 3, ELASTIC, "HEX8")


@pytest.mark.parametrize("tiles", ["000", "100", "010", "001", "111"])
def test_forced_tile_variants_agree(tiles, monkeypatch):
    monkeypatch.setenv("FANSGPU_TUNE", tiles)
    P = _problem()
    r = np.random.default_rng(3).standard_normal(P.u.shape)
    ctx = gpu_context(P, precision="fp64")
    s = ctx.convolve(r)
    assert ctx.tuning()["fp64"] == tuple(int(c) for c in tiles)
    ctx.close()
    mix = gpu_context(P, precision="mixed")
    mix.set_tolerance("L2", "relative", 1e-8, 500)
    mix.set_gradient(np.array([0.0, 0.0, 1.0, 0.0, 0.5, 0.0]))
    st = mix.solve()
    assert mix.tuning()["fp32"] == tuple(int(c) for c in tiles)
    sig = mix.homogenized_stress()
    mix.close()
    if "000" not in _ref:
        assert tiles == "000"
        _ref["000"] = (s, st["iterations"], sig)
        assert rel(s, P.convolve(r)) < 1e-12
        return
    s0, it0, sig0 = _ref["000"]
    assert np.array_equal(s, s0)
    assert st["iterations"] == it0
    assert rel(sig, sig0) < 1e-12


def test_tuned_context_matches_oracle():
    P = _problem()
    ctx = gpu_context(P, precision="mixed")
    ctx.set_tolerance("L2", "relative", 1e-10, 500)
    g = np.array([1.0, 0.0, 0.0, 0.0, 0.0, 0.3])
    ctx.set_gradient(g)
    assert ctx.solve()["converged"]
    P.set_gradient(g)
    P.solve(tol=1e-10, n_it=500)
    assert rel(ctx.homogenized_stress(), P.homogenized_stress()) < 1e-8
    ctx.close()


def _mixed_run(monkeypatch, graphs, n_it=500):
    monkeypatch.setenv("FANSGPU_GRAPHS", graphs)
    P = _problem()
    ctx = gpu_context(P, precision="mixed")
    ctx.set_tolerance("L2", "relative", 1e-9, n_it)
    out = []
    for g in (np.array([1.0, 0, 0, 0, 0, 0]), np.array([0, 0.5, 0, 0.3, 0, 0])):
        ctx.reset()
        ctx.set_gradient(g)
        st = ctx.solve()
        out.append((st["iterations"], st["refinements"], st["converged"], ctx.error_history(),
                    ctx.homogenized_stress()))
    ctx.close()
    return out


@pytest.mark.parametrize("n_it", [500, 17])
def test_graph_modes_take_the_same_decisions(monkeypatch, n_it):
    """The device-resident loop (WHILE/IF graph nodes and the check kernel), one
    graph per iteration and plain launches run the same kernels: iteration counts,
    refreshes, the whole error history and the stresses agree bitwise, also when
    n_it stops the solve before convergence."""
    ref = _mixed_run(monkeypatch, "0", n_it)
    for mode in ("iter", "1"):
        got = _mixed_run(monkeypatch, mode, n_it)
        for (i0, r0, c0, h0, s0), (i1, r1, c1, h1, s1) in zip(ref, got):
            assert (i0, r0, c0) == (i1, r1, c1), mode
            assert np.array_equal(h0, h1), mode
            assert np.array_equal(s0, s1), mode
    assert ref[0][2] == (n_it == 500)
