"""Autotuned tile shapes (FANSGPU_TUNE; the tuner runs on a context's first
setup).  Every forced combination of the register FFT passes' variants (z, y, x)
gives the bitwise-same FP64 convolution and the same mixed-precision solve; the
FP32-only variants (z + 2:
fused z + y forward cluster pass, x = 2: TMA-fed x pass) follow the register
passes to FP32 rounding; the default (tuned) context agrees with the oracle."""
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


def _multi_solve(P, n_rhs):
    from fans_gb300 import Context

    ctx = Context((P.nx, P.ny, P.nz), tuple(P.L), P.c, "HEX8", "mixed", "cg", n_rhs=n_rhs)
    ctx.set_microstructure(P.ms)
    for ph in range(P.nphase):
        ctx.set_phase_material(ph, int(P.law[ph]), P.param[ph, : (1 if P.c == 1 else 2)])
    ctx.set_reference(P.kapparef)
    ctx.set_tolerance("L2", "relative", 1e-8, 1000)
    loads = np.eye(P.nstr)[:n_rhs] if n_rhs > 1 else np.eye(P.nstr)[:1] * 0.7
    ctx.set_gradients(loads)
    agg = ctx.solve()
    out = {"tuning": ctx.tuning()["fp32"], "agg": (agg["iterations"], agg["converged"])}
    for k in range(n_rhs):
        ctx.select_rhs(k)
        st = ctx.rhs_stats(k)
        out[k] = (st["iterations"], st["refinements"], ctx.error_history(), ctx.homogenized_stress(),
                  ctx.get_field(0))
    ctx.close()
    return out


@pytest.mark.parametrize("tiles,c,shape,n_rhs", [
    ("002", 3, (32, 32, 64), 6),   # elastic, six RHS, N1 = N2 x line, ragged last kz tile (nz/2+1 = 33)
    ("002", 3, (48, 16, 32), 3),   # N1 != N2 (48 = 8 x 6), three RHS
    ("002", 1, (64, 32, 48), 3),   # thermal (one component, one Green's entry per frequency)
    ("002", 3, (128, 16, 32), 1),  # one RHS: every job starts a new tile (a Green's slice per job)
    # the fused z + y forward cluster pass (z entry + 2)
    ("200", 3, (32, 32, 32), 6),   # one CTA per plane
    ("200", 3, (48, 64, 64), 3),
    ("200", 1, (40, 48, 48), 3),   # thermal, 48 = 8 x 6 lines in y, 24 = 8 x 3 in z
    ("200", 3, (16, 256, 256), 1), # four CTAs per plane (rows shared through distributed shared memory)
    ("302", 1, (16, 256, 256), 2), # with the other z-inverse tile and the TMA-fed x pass
])
def test_fft_pass_variants_equal_register_passes(monkeypatch, tiles, c, shape, n_rhs):
    """The FP32 x pass fed by tensor-map copies (x variant 2: persistent CTAs, two job
    buffers in flight, Green's multiply fused into the inverse transform's load) and
    the fused z + y forward cluster pass (z entry + 2: a plane's rows transformed
    along z in shared memory, then along y through distributed shared memory) run
    the register passes' operations per value; only FP32 roundings may differ (the
    compiler may fuse products and sums differently).  A mixed multi-RHS solve
    forced onto them must therefore follow the register passes
    residual history to FP32 accuracy in its first iterations (a wrong tile, Green's
    entry or stale buffer moves it at once by far more), take the same refreshes and
    the same iterations within one (the mixed path's bar against the oracle), and
    reach the same stresses and displacements within the FP64 true residual
    tolerance."""
    from helpers import THERMAL

    ms = random_ms(shape, vf=0.3, seed=61)
    P = oracle_problem(ms, c, ELASTIC if c == 3 else THERMAL, "HEX8")
    monkeypatch.setenv("FANSGPU_TUNE", "000")
    ref = _multi_solve(P, n_rhs)
    monkeypatch.setenv("FANSGPU_TUNE", tiles)
    got = _multi_solve(P, n_rhs)
    assert ref["tuning"] == (0, 0, 0) and got["tuning"] == tuple(int(v) for v in tiles)
    assert ref["agg"][1] and got["agg"][1] and abs(got["agg"][0] - ref["agg"][0]) <= 1
    for k in range(n_rhs):
        i0, r0, h0, s0, u0 = ref[k]
        i1, r1, h1, s1, u1 = got[k]
        assert abs(i0 - i1) <= 1 and r0 == r1, (k, i0, i1, r0, r1)
        assert h0[0] == h1[0], k
        assert np.abs(h1[:4] / h0[:4] - 1).max() < 2e-6, (k, h0[:4], h1[:4])
        assert rel(s1, s0) < 1e-8, k
        assert rel(u1, u0) < 1e-6, k


@pytest.mark.parametrize("c,shape,n_rhs", [(3, (32, 32, 64), 6), (1, (48, 32, 32), 3)])
def test_spectral_dot_equals_spatial_dot(monkeypatch, c, shape, n_rhs):
    """<r, s> of the mixed path's convolution taken from the spectra in the x pass (Parseval,
    the default) or from r and s in the z-inverse pass (FANSGPU_SPECTRAL_DOT=0): the two differ
    by the FP32 rounding of the inverse transform, so the solves follow the same residual
    history to FP32 accuracy, take the same refreshes and the same iterations within one, and
    meet the same stresses to the FP64 tolerance."""
    from helpers import THERMAL

    ms = random_ms(shape, vf=0.3, seed=62)
    P = oracle_problem(ms, c, ELASTIC if c == 3 else THERMAL, "HEX8")
    monkeypatch.setenv("FANSGPU_TUNE", "000")
    monkeypatch.setenv("FANSGPU_SPECTRAL_DOT", "0")
    ref = _multi_solve(P, n_rhs)
    monkeypatch.setenv("FANSGPU_SPECTRAL_DOT", "1")
    got = _multi_solve(P, n_rhs)
    assert ref["agg"][1] and got["agg"][1] and abs(got["agg"][0] - ref["agg"][0]) <= 1
    for k in range(n_rhs):
        i0, r0, h0, s0, u0 = ref[k]
        i1, r1, h1, s1, u1 = got[k]
        assert abs(i0 - i1) <= 1 and r0 == r1, (k, i0, i1, r0, r1)
        assert h0[0] == h1[0], k
        assert np.abs(h1[:4] / h0[:4] - 1).max() < 2e-6, (k, h0[:4], h1[:4])
        assert rel(s1, s0) < 1e-8, k
        assert rel(u1, u0) < 1e-6, k
