"""Multi-filter flux-ratio likelihood (getChi2GPU's job) on the GPU vs the FP64 oracle.

Tolerance: chi2 per pair and the likelihood within 1e-5 relative of the FP64 oracle
(FP32 terms, FP64 likelihood accumulation)."""
import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu


def _inputs(N, F, T, seed, spread=0.5):
    rng = np.random.default_rng(seed)
    fo = rng.uniform(0.6, 1.4, (F, T)).astype(np.float32)
    dfo = rng.uniform(0.2, 0.6, (F, T)).astype(np.float32)
    m1 = rng.uniform(1 - spread, 1 + spread, (N, F, T)).astype(np.float32)
    m2 = rng.uniform(1 - spread, 1 + spread, (N, F, T)).astype(np.float32)
    return fo, dfo, m1, m2


@pytest.mark.parametrize("N,F,T", [(1, 1, 1), (63, 7, 10), (130, 3, 11), (257, 1, 33), (700, 7, 10)])
def test_flux_ratio_matches_oracle(ctx, N, F, T):
    import microsn_gb300 as mlc
    fo, dfo, m1, m2 = _inputs(N, F, T, seed=N + F)
    like, chi2 = mlc.flux_ratio_chi2(ctx, fo, dfo, torch.as_tensor(m1, device="cuda:0"),
                                     torch.as_tensor(m2, device="cuda:0"), want_chi2=True)
    ref_like, ref_chi2 = oracle.flux_ratio(fo, dfo, m1, m2, want_chi2=True)
    got = chi2.cpu().numpy().astype(np.float64)
    assert np.max(np.abs(got - ref_chi2) / np.abs(ref_chi2)) < 1e-5
    assert abs(like - ref_like) <= 1e-5 * abs(ref_like)
    like2 = mlc.flux_ratio_chi2(ctx, fo, dfo, torch.as_tensor(m1, device="cuda:0"),
                                torch.as_tensor(m2, device="cuda:0"))
    assert like2 == like  # deterministic, and the same without the chi2 matrix


def test_flux_ratio_reference_workload_size(ctx):
    """The reference driver's size (N = 10^4, F = 7, T = 10) against the oracle on a subset:
    the likelihood of a 2000-location slice of both images."""
    import microsn_gb300 as mlc
    fo, dfo, m1, m2 = _inputs(10_000, 7, 10, seed=5, spread=0.2)
    d1 = torch.as_tensor(m1, device="cuda:0"); d2 = torch.as_tensor(m2, device="cuda:0")
    like_full, chi2 = mlc.flux_ratio_chi2(ctx, fo, dfo, d1, d2, want_chi2=True)
    n = 2000
    sub = mlc.flux_ratio_chi2(ctx, fo, dfo, d1[:n].contiguous(), d2[:n].contiguous())
    ref = oracle.flux_ratio(fo, dfo, m1[:n], m2[:n])
    assert abs(sub - ref) <= 1e-5 * abs(ref)
    # the full matrix: its sum of exp(-chi2) equals the likelihood
    s = torch.exp(-chi2.double()).sum().item()
    assert abs(s - like_full) <= 1e-6 * abs(like_full)


def test_flux_ratio_large_chi2_keeps_fp64_range(ctx):
    """Every chi2 above the FP32 exp range (min chi2 ~ 125): the likelihood stays non-zero."""
    import microsn_gb300 as mlc
    fo, dfo, m1, m2 = _inputs(150, 7, 10, seed=8, spread=0.2)
    dfo = (dfo * 0.3).astype(np.float32)
    like, chi2 = mlc.flux_ratio_chi2(ctx, fo, dfo, torch.as_tensor(m1, device="cuda:0"),
                                     torch.as_tensor(m2, device="cuda:0"), want_chi2=True)
    ref, ref_chi2 = oracle.flux_ratio(fo, dfo, m1, m2, want_chi2=True)
    assert ref_chi2.min() > 110 and ref > 0 and like > 0
    assert np.max(np.abs(chi2.cpu().numpy() - ref_chi2) / ref_chi2) < 1e-5
    # exp(-chi2) turns the FP32 chi2 rounding (<= 1e-5 relative, i.e. ~1e-3 absolute at
    # chi2 ~ 125) into a relative error of the same absolute size
    assert abs(like - ref) <= 2e-3 * ref
