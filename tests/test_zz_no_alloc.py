"""The allocation-free histogram entry point, checked against the allocating one.

Callers that cannot allocate device memory (a framework owning the device pool, a
plugin or callback limited to the buffers it is handed, a call sequence to be replayed
from a captured stream) use mlc_histogram_f64_noalloc, whose counters live in a fixed
array inside the library.  This file is collected last so that a failure here leaves
every other test already run.
"""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _noalloc(ctx, v, nbins, lo, hi, log):
    out = np.zeros(nbins, np.uint64)
    st = ctx.L.mlc_histogram_f64_noalloc(ctx.h, v.numel(), C.c_void_p(v.data_ptr()), nbins, lo, hi, int(log),
                                         out.ctypes.data_as(C.c_void_p))
    ctx.check(st)
    return out


def test_noalloc_histogram_matches_allocating_entry(lib_built):
    import microsn_gb300 as mlc
    ctx = mlc.Context(0)  # own context: the entry point must not touch any workspace
    rng = np.random.default_rng(42)
    a = torch.as_tensor(np.exp(rng.normal(0, 2.5, 400_000)), device="cuda:0")
    b = torch.as_tensor(rng.random(123_457) * 80.0, device="cuda:0")
    torch.cuda.synchronize()
    mem0 = torch.cuda.memory_allocated(0)
    # two calls in a row, different sizes and data: the second must not see the first's counts
    got_a = _noalloc(ctx, a, 1000, -5.0, 5.0, True)
    got_b = _noalloc(ctx, b, 97, 0.0, 100.0, False)
    assert ctx.workspace_bytes() == 0
    assert torch.cuda.memory_allocated(0) == mem0
    ref_a = mlc.histogram_f64(ctx, a, 1000, -5.0, 5.0, log=True)
    ref_b = mlc.histogram_f64(ctx, b, 97, 0.0, 100.0, log=False)
    np.testing.assert_array_equal(got_a, ref_a)
    np.testing.assert_array_equal(got_b, ref_b)
    assert int(got_a.sum()) > 0 and int(got_b.sum()) == b.numel()
    # same call again after the allocating entry ran: still identical
    np.testing.assert_array_equal(_noalloc(ctx, a, 1000, -5.0, 5.0, True), ref_a)
    ctx.close()


def test_noalloc_histogram_rejects_too_many_bins(lib_built):
    import microsn_gb300 as mlc
    ctx = mlc.Context(0)
    v = torch.ones(10, dtype=torch.float64, device="cuda:0")
    out = np.zeros(12001, np.uint64)
    st = ctx.L.mlc_histogram_f64_noalloc(ctx.h, 10, C.c_void_p(v.data_ptr()), 12001, 0.0, 1.0, 0,
                                         out.ctypes.data_as(C.c_void_p))
    assert st == 6  # MLC_ERR_LIMIT
    assert b"12000" in ctx.L.mlc_ctx_last_error(ctx.h)
    ctx.close()
