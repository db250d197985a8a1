"""fansgpu_residual_norm_noalloc: the residual norm for callers that cannot
allocate device memory (their device memory is held by another allocator, or
they must not trigger cudaMalloc's device synchronisation).

Its result, through the C ABI on a caller-owned device buffer, must equal the
norm the solver itself computes (err_all[0] of a solve with n_it = 0, i.e.
||R(u)|| from the context's norm kernel and its allocated scratch) to 1e-12
relative, on two calls in a row (the second sees the first's leftover scratch).
This file is collected last so that a run stopping at the first failure has
already run every other test.
"""
import ctypes

import numpy as np
import pytest

from helpers import ELASTIC, gpu_context, oracle_problem, random_ms

pytestmark = pytest.mark.gpu


def _call(lib, ptr, n, measure, out_ptr, stream):
    return lib.fansgpu_residual_norm_noalloc(ctypes.c_void_p(ptr), n, measure, ctypes.c_void_p(out_ptr),
                                             ctypes.c_void_p(stream))


@pytest.mark.parametrize("measure", ["L1", "L2", "Linfinity"])
def test_noalloc_norm_matches_solver_norm(measure):
    import torch

    from fans_gb300 import _lib

    shape = (16, 12, 20)
    P = oracle_problem(random_ms(shape, seed=21), 3, ELASTIC, "HEX8")
    ctx = gpu_context(P)
    rng = np.random.default_rng(22)
    ctx.set_field(_lib.FIELD_U, rng.standard_normal(shape + (3,)))
    ctx.set_gradient(rng.standard_normal(6))
    ctx.set_tolerance(measure, "absolute", 0.0, 0)  # n_it = 0: r = R(u) and err_all[0] only
    ctx.solve()
    ref = float(ctx.error_history()[0])
    r = ctx.get_field(_lib.FIELD_R)
    ctx.close()
    assert ref > 0

    lib = _lib.load()
    r_dev = torch.from_numpy(np.ascontiguousarray(r).ravel()).cuda()
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    results = []
    for _ in range(2):
        out.fill_(-1.0)
        rc = _call(lib, r_dev.data_ptr(), r_dev.numel(), _lib.MEASURES[measure], out.data_ptr(), stream)
        assert rc == 0, lib.fansgpu_last_error(None)
        torch.cuda.synchronize()
        results.append(out.item())
    for v in results:
        assert abs(v - ref) <= 1e-12 * ref, (v, ref)
    assert results[0] == results[1]


def test_noalloc_norm_limits():
    import torch

    from fans_gb300 import _lib

    lib = _lib.load()
    x = torch.ones(8, dtype=torch.float64, device="cuda")
    out = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    too_big = _lib_max(lib) + 1
    assert _call(lib, x.data_ptr(), too_big, _lib.L2, out.data_ptr(), stream) == _lib.EINVAL
    assert b"outside" in lib.fansgpu_last_error(None)
    assert _call(lib, x.data_ptr(), 8, 7, out.data_ptr(), stream) == _lib.EINVAL
    assert _call(lib, x.data_ptr(), 0, _lib.L2, out.data_ptr(), stream) == 0
    torch.cuda.synchronize()
    assert out.item() == 0.0
    assert _call(lib, x.data_ptr(), 8, _lib.L2, out.data_ptr(), stream) == 0
    torch.cuda.synchronize()
    assert abs(out.item() - np.sqrt(8.0)) < 1e-15


def _lib_max(lib):
    import os
    import re

    hdr = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "fans_gb300.h")
    return int(re.search(r"FANSGPU_NOALLOC_MAX_VALUES\s+(\d+)LL", open(hdr).read()).group(1))


def test_noalloc_norm_many_blocks_and_nan():
    """A field of 8192 * 300 + 17 values spans 301 blocks (the last one ragged),
    so the last block folds 301 partials in block order: L1, L2 and Linfinity
    equal torch's FP64 norms to 1e-12, twice in a row; one NaN makes every
    measure NaN (the maximum keeps NaN, as the solver's Linfinity does)."""
    import torch

    from fans_gb300 import _lib

    lib = _lib.load()
    n = 8192 * 300 + 17
    g = torch.Generator(device="cpu").manual_seed(23)
    x = torch.randn(n, dtype=torch.float64, generator=g).cuda()
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    refs = {"L1": x.abs().sum().item(), "L2": x.norm().item(), "Linfinity": x.abs().max().item()}
    for measure, ref in refs.items():
        vals = []
        for _ in range(2):
            out.fill_(-1.0)
            assert _call(lib, x.data_ptr(), n, _lib.MEASURES[measure], out.data_ptr(), stream) == 0
            torch.cuda.synchronize()
            vals.append(out.item())
        assert vals[0] == vals[1]
        assert abs(vals[0] - ref) <= 1e-12 * ref, (measure, vals[0], ref)
    x[n // 2] = float("nan")
    for measure in refs:
        out.fill_(-1.0)
        assert _call(lib, x.data_ptr(), n, _lib.MEASURES[measure], out.data_ptr(), stream) == 0
        torch.cuda.synchronize()
        assert np.isnan(out.item()), measure
