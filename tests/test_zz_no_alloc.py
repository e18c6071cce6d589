"""The allocation-free histogram entry point, checked against the allocating one and the
CPU oracle.

Some callers cannot allocate device memory: code running inside a framework that has
reserved the whole device pool for its own allocator, and plugins or callbacks that may
only use the buffers they are handed.  They use mlc_histogram_f64_noalloc, whose
counters live in a fixed array inside the library.  This file is collected last so that
a failure here leaves every other test already run; it passes alone in a fresh process
as well as after the others.
"""
import ctypes as C

import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu

MAX_BINS = 12000


def _noalloc(ctx, v, nbins, lo, hi, log):
    out = np.full(nbins, 7, np.uint64)  # not zero: the call must overwrite every bin
    st = ctx.L.mlc_histogram_f64_noalloc(ctx.h, v.numel(), C.c_void_p(v.data_ptr()), nbins, lo, hi, int(log),
                                         out.ctypes.data_as(C.c_void_p))
    ctx.check(st)
    return out


def _agrees_with_oracle(got, v_host, nbins, lo, hi, log):
    """Counts equal to the oracle's, except values within 1e-14 relative of a bin edge,
    each of which may land on either side."""
    ref, near = oracle.histogram(v_host, nbins, lo, hi, log, rel_tol=1e-14)
    return int(np.abs(got.astype(np.int64) - ref.astype(np.int64)).sum()) <= 2 * near


def test_noalloc_histogram_matches_allocating_entry_and_oracle(lib_built):
    import microsn_gb300 as mlc
    ctx = mlc.Context(0)  # own context: the entry point must not touch any workspace
    rng = np.random.default_rng(42)
    ha = np.exp(rng.normal(0, 2.5, 400_000))
    hb = rng.random(123_457) * 80.0
    a = torch.as_tensor(ha, device="cuda:0")
    b = torch.as_tensor(hb, device="cuda:0")
    tiny = torch.as_tensor(ha[:3], device="cuda:0")
    # a first call loads the kernel module and resolves the counter array's address
    _noalloc(ctx, tiny, 4, -1.0, 1.0, True)
    torch.cuda.synchronize()
    mem0 = torch.cuda.memory_allocated(0)
    free0, _ = torch.cuda.mem_get_info(0)  # sees raw cudaMalloc / cudaMallocAsync too
    # two calls in a row, different sizes and data: the second must not see the first's counts
    got_a = _noalloc(ctx, a, 1000, -5.0, 5.0, True)
    got_b = _noalloc(ctx, b, 97, 0.0, 100.0, False)
    # the largest bin count the fixed array holds (48000 B of shared-memory counters)
    got_max = _noalloc(ctx, a, MAX_BINS, -5.0, 5.0, True)
    # n = 0 after calls that filled the array: every bin must read zero
    got_empty = _noalloc(ctx, a[:0], MAX_BINS, -5.0, 5.0, True)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info(0)
    assert ctx.workspace_bytes() == 0
    assert torch.cuda.memory_allocated(0) == mem0
    assert free1 == free0, f"device free memory changed by {free0 - free1} bytes"

    ref_a = mlc.histogram_f64(ctx, a, 1000, -5.0, 5.0, log=True)
    ref_b = mlc.histogram_f64(ctx, b, 97, 0.0, 100.0, log=False)
    ref_max = mlc.histogram_f64(ctx, a, MAX_BINS, -5.0, 5.0, log=True)
    np.testing.assert_array_equal(got_a, ref_a)
    np.testing.assert_array_equal(got_b, ref_b)
    np.testing.assert_array_equal(got_max, ref_max)
    assert _agrees_with_oracle(got_a, ha, 1000, -5.0, 5.0, True)
    assert _agrees_with_oracle(got_b, hb, 97, 0.0, 100.0, False)
    assert _agrees_with_oracle(got_max, ha, MAX_BINS, -5.0, 5.0, True)
    assert int(got_a.sum()) > 0 and int(got_b.sum()) == b.numel()
    assert not got_empty.any()
    # the same call again after the allocating entry ran: still identical
    np.testing.assert_array_equal(_noalloc(ctx, a, 1000, -5.0, 5.0, True), ref_a)
    ctx.close()


def test_noalloc_histogram_rejects_too_many_bins(lib_built):
    import microsn_gb300 as mlc
    ctx = mlc.Context(0)
    v = torch.ones(10, dtype=torch.float64, device="cuda:0")
    out = np.zeros(MAX_BINS + 1, np.uint64)
    st = ctx.L.mlc_histogram_f64_noalloc(ctx.h, 10, C.c_void_p(v.data_ptr()), MAX_BINS + 1, 0.0, 1.0, 0,
                                         out.ctypes.data_as(C.c_void_p))
    assert st == 6  # MLC_ERR_LIMIT
    assert b"12000" in ctx.L.mlc_ctx_last_error(ctx.h)
    ctx.close()
