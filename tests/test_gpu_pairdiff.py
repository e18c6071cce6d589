"""Magnitude-difference pair chi2 (plain FP64 and tensor-core forms) vs the FP64 oracle:
the chi2 matrix within 1e-5 relative, the log10-chi2 histogram exact except values
within 1e-5 of a bin edge, and the top-k pairs."""
import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def _curves(NA, NB, T, seed, close=0):
    rng = np.random.default_rng(seed)
    A = np.cumsum(rng.normal(0, 0.05, (NA, T)), axis=1) + rng.normal(0, 0.3, (NA, 1))
    B = np.cumsum(rng.normal(0, 0.05, (NB, T)), axis=1) + rng.normal(0, 0.3, (NB, 1))
    d = rng.normal(0, 0.02, T)
    sig = rng.uniform(0.02, 0.1, T)
    for c in range(close):  # near-identical pairs: B_j = A_i + d + tiny noise
        B[c] = A[c] - d + rng.normal(0, 1e-4, T)
    return A.astype(np.float32), B.astype(np.float32), 1.0 / sig ** 2, d


@pytest.mark.parametrize("method", ["tensor", "plain"])
@pytest.mark.parametrize("offset", [False, True])
@pytest.mark.parametrize("NA,NB,T", [(300, 200, 50), (129, 65, 128), (64, 300, 7)])
def test_matrix_matches_oracle(ctx, method, offset, NA, NB, T):
    import microsn_gb300 as mlc
    A, B, w, d = _curves(NA, NB, T, NA + NB + T, close=5)
    r = mlc.pair_chi2_magdiff(ctx, torch.as_tensor(A, device=DEV), torch.as_tensor(B, device=DEV), w, d, offset,
                              method=method, nbins=200, lo=-6, hi=8, k=20, want_matrix=True)
    got = r["matrix"].cpu().numpy().astype(np.float64).ravel()
    ref = oracle.pair_chi2_magdiff(A, B, w, d, offset)
    rel = np.abs(got - ref) / np.maximum(ref, 1e-300)
    assert rel.max() < 1e-5, (rel.max(), r["stats"])
    if method == "tensor":
        assert r["stats"]["refined"] >= 5  # the near-identical pairs went through the FP64 refinement
        assert r["stats"]["refined"] < 0.5 * NA * NB  # most values come from the tensor-core path
    counts, near = oracle.histogram(ref, 200, -6, 8, log=True, rel_tol=1e-5)
    assert np.abs(r["hist"].astype(np.int64) - counts.astype(np.int64)).sum() <= 2 * near
    # every pair is counted once: in a bin, below 10^lo or at/above 10^hi
    st = r["stats"]
    assert int(r["hist"].sum()) + st["below"] + st["above"] == NA * NB
    below = int((ref < 10.0 ** -6).sum()); above = int((ref >= 1e8).sum())
    assert abs(st["below"] - below) <= near and abs(st["above"] - above) <= near
    idx = oracle.topk_smallest(ref, 20)
    np.testing.assert_allclose(r["topk_val"], ref[idx], rtol=1e-5)
    got_pairs = r["topk_i"] * NB + r["topk_j"]
    assert np.array_equal(np.sort(got_pairs[:15]), np.sort(idx[:15])) or np.allclose(ref[got_pairs], ref[idx],
                                                                                      rtol=1e-5)


@pytest.mark.parametrize("offset", [False, True])
def test_tensor_large_with_sampled_threshold(ctx, offset):
    """3e6 pairs: several work items per CTA, both TMEM buffers, the sampled top-k threshold."""
    import microsn_gb300 as mlc
    NA, NB, T = 1000, 3000, 128
    A, B, w, d = _curves(NA, NB, T, 99, close=40)
    tA = torch.as_tensor(A, device=DEV); tB = torch.as_tensor(B, device=DEV)
    k = 100
    r = mlc.pair_chi2_magdiff(ctx, tA, tB, w, d, offset, method="tensor", nbins=1000, lo=-4, hi=8, k=k)
    ref = oracle.pair_chi2_magdiff(A, B, w, d, offset)
    counts, near = oracle.histogram(ref, 1000, -4, 8, log=True, rel_tol=1e-5)
    assert int(r["hist"].sum()) == int(counts.sum())
    assert int(r["hist"].sum()) + r["stats"]["below"] + r["stats"]["above"] == NA * NB
    assert np.abs(r["hist"].astype(np.int64) - counts.astype(np.int64)).sum() <= 2 * near
    idx = oracle.topk_smallest(ref, k)
    np.testing.assert_allclose(r["topk_val"], ref[idx], rtol=1e-5)
    assert r["stats"]["candidates"] >= k
    # a fixed subset through the FP64 list entry point
    rng = np.random.default_rng(1)
    ia = rng.integers(0, NA, 5000); ib = rng.integers(0, NB, 5000)
    sub = mlc.pair_chi2_magdiff_list(ctx, tA, tB, w, ia, ib, d, offset).cpu().numpy()
    np.testing.assert_allclose(sub, ref[ia * NB + ib], rtol=1e-12)


def test_plain_and_tensor_agree(ctx):
    import microsn_gb300 as mlc
    A, B, w, d = _curves(700, 900, 100, 5)
    tA = torch.as_tensor(A, device=DEV); tB = torch.as_tensor(B, device=DEV)
    a = mlc.pair_chi2_magdiff(ctx, tA, tB, w, d, True, method="tensor", nbins=500, lo=-2, hi=7, k=50,
                              want_matrix=True)
    b = mlc.pair_chi2_magdiff(ctx, tA, tB, w, d, True, method="plain", nbins=500, lo=-2, hi=7, k=50,
                              want_matrix=True)
    ma, mb = a["matrix"].cpu().numpy().astype(np.float64), b["matrix"].cpu().numpy().astype(np.float64)
    assert (np.abs(ma - mb) / mb).max() < 1e-5
    assert np.array_equal(a["topk_i"] * 900 + a["topk_j"], b["topk_i"] * 900 + b["topk_j"]) or \
        np.allclose(a["topk_val"], b["topk_val"], rtol=1e-5)
