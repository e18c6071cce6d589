"""Pair stage (reference ratio form), radix sort and histograms on the GPU vs the
oracle and the reference's golden vectors."""
import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def _vars(golden):
    import microsn_gb300 as mlc
    d, s, sizes, Dfac = golden["setup_d"], golden["setup_s"], golden["setup_sizes"], float(golden["setup_Dfac"])
    return mlc.setup_chi2_calculation((0.4, 0.5), (1.0,), Dfac, d, golden["setup0_t"], s, sizes)


def test_pair_stage_matches_reference_golden(ctx, golden):
    import microsn_gb300 as mlc
    LCA, LCB = golden["pair_LCA"], golden["pair_LCB"]
    tA = torch.as_tensor(LCA, device=DEV); tB = torch.as_tensor(LCB, device=DEV)
    dA = torch.as_tensor(np.diff(LCA, axis=1).copy(), device=DEV); dB = torch.as_tensor(np.diff(LCB, axis=1).copy(), device=DEV)
    rank, lower, nper = mlc.setup_integral(ctx, tA, tB, golden["pair_edges"])
    assert np.array_equal(rank.cpu().numpy().view(np.uint32), golden["pair_rank"])
    assert np.array_equal(lower, golden["pair_lower"]) and np.array_equal(nper, golden["pair_nper"])
    v = _vars(golden)
    chi2 = mlc.calculate_chi2(ctx, v, tA, dA, tB, dB, rank)
    np.testing.assert_allclose(chi2.cpu().numpy(), golden["pair_chi2"], rtol=1e-12)
    bc, be = mlc.bin_chi2(ctx, lower, nper, chi2)
    full = nper > 0
    np.testing.assert_allclose(bc[full], golden["pair_bchi2"][full], rtol=1e-12)
    np.testing.assert_allclose(be[full], golden["pair_bexp"][full], rtol=1e-12)
    assert np.all(bc[~full] == 2000.0)
    fb, fe, fn = mlc.pair_bin_fused(ctx, v, tA, dA, tB, dB, golden["pair_edges"])
    assert np.array_equal(fn, nper)
    np.testing.assert_allclose(fb, bc, rtol=1e-12)
    np.testing.assert_allclose(fe, be, rtol=1e-12)


@pytest.mark.parametrize("Nloc", [1, 37, 600, 2100])
def test_pair_stage_random_vs_oracle(ctx, golden, Nloc):
    import microsn_gb300 as mlc
    rng = np.random.default_rng(Nloc)
    Nprof = 5
    LCA = np.exp(rng.normal(0, 0.6, (Nloc, Nprof))); LCB = np.exp(rng.normal(0, 0.6, (Nloc, Nprof)))
    LCA[: Nloc // 4, 0] = 1.25; LCB[: Nloc // 4, 0] = 1.25  # ties
    edges = mlc.bin_edges(300, 1e-4, 300, True)
    tA = torch.as_tensor(LCA, device=DEV); tB = torch.as_tensor(LCB, device=DEV)
    dA = torch.as_tensor(np.diff(LCA, axis=1).copy(), device=DEV); dB = torch.as_tensor(np.diff(LCB, axis=1).copy(), device=DEV)
    rank, lower, nper = mlc.setup_integral(ctx, tA, tB, edges)
    if Nloc <= 600:
        r_o, l_o, n_o = oracle.pair_rank(LCA, LCB, edges)
        assert np.array_equal(rank.cpu().numpy().view(np.uint32), r_o)
        assert np.array_equal(lower, l_o) and np.array_equal(nper, n_o)
    v = _vars(golden)
    chi2 = mlc.calculate_chi2(ctx, v, tA, dA, tB, dB, rank)
    if Nloc <= 600:
        ov = dict(Njp=v.Njp, indA=v.indA, indB=v.indB, facA=v.facA, facB=v.facB, d=v.d, s=v.s)
        ref = oracle.pair_chi2_ratio(ov, LCA, np.diff(LCA, axis=1), LCB, np.diff(LCB, axis=1), r_o)
        np.testing.assert_allclose(chi2.cpu().numpy(), ref, rtol=1e-12)
    bc, be = mlc.bin_chi2(ctx, lower, nper, chi2)
    fb, fe, fn = mlc.pair_bin_fused(ctx, v, tA, dA, tB, dB, edges)
    assert np.array_equal(fn, nper)
    full = nper > 0
    np.testing.assert_allclose(fb[full], bc[full], rtol=1e-10)
    np.testing.assert_allclose(fe[full], be[full], rtol=1e-10)


@pytest.mark.parametrize("n", [0, 1, 1000, 4097, 300_000])
def test_radix_sort_stable(ctx, n):
    import microsn_gb300 as mlc
    rng = np.random.default_rng(n)
    k = rng.normal(0, 1, n)
    if n > 10:
        k[::7] = 0.5; k[1::11] = -0.0; k[2::13] = -3.25  # ties and negative zero
    keys = torch.as_tensor(k, device=DEV)
    vals = torch.arange(n, dtype=torch.int32, device=DEV)
    mlc.sort_f64_u32(ctx, keys, vals)
    order = np.lexsort((np.arange(n), np.where(k == 0, np.copysign(1, k) * 1e-300, k)))
    got_v = vals.cpu().numpy()
    assert np.array_equal(keys.cpu().numpy(), k[order])
    assert np.array_equal(got_v, order.astype(np.int32))


def test_histogram_matches_oracle(ctx):
    import microsn_gb300 as mlc
    rng = np.random.default_rng(9)
    v = np.exp(rng.normal(0, 3, 200_000))
    for log, lo, hi in [(True, -4, 4), (False, 0.0, 50.0)]:
        got = mlc.histogram_f64(ctx, torch.as_tensor(v, device=DEV), 100, lo, hi, log)
        ref, near = oracle.histogram(v, 100, lo, hi, log, rel_tol=1e-14)
        assert np.abs(got.astype(np.int64) - ref.astype(np.int64)).sum() <= 2 * near


def test_fused_bins_exact_at_edges(ctx, golden):
    """z exactly on a bin edge, one ulp either side, zero, infinite and NaN quotients: the
    fused kernel's float pre-search must give the rank path's counts exactly."""
    import microsn_gb300 as mlc
    edges = mlc.bin_edges(300, 1e-4, 300, True)
    k = np.arange(0, 300, 7)
    za = np.concatenate([edges[k], np.nextafter(edges[k], 0), np.nextafter(edges[k], np.inf),
                         [0.0, 1e-300, 1e300, edges[-1] * 1.0000001, 5e-5]])
    Nloc, Nprof = za.size, 5
    rng = np.random.default_rng(3)
    LCA = np.exp(rng.normal(0, 0.3, (Nloc, Nprof))); LCB = np.exp(rng.normal(0, 0.3, (Nloc, Nprof)))
    LCA[:, 0] = za
    LCB[:, 0] = 1.0          # z = LCA / 1 exactly for these columns
    LCB[-5:, 0] = [0.0, 2.0, 0.5, 1.0, 1e-300]  # 0 -> inf / NaN quotients, tiny -> huge
    tA = torch.as_tensor(LCA, device=DEV); tB = torch.as_tensor(LCB, device=DEV)
    dA = torch.as_tensor(np.diff(LCA, axis=1).copy(), device=DEV); dB = torch.as_tensor(np.diff(LCB, axis=1).copy(), device=DEV)
    _, lower, nper = mlc.setup_integral(ctx, tA, tB, edges)
    v = _vars(golden)
    fb, fe, fn = mlc.pair_bin_fused(ctx, v, tA, dA, tB, dB, edges)
    assert np.array_equal(fn, nper)
    fin = np.isfinite(LCA[:, 0][:, None] / np.where(LCB[:, 0] == 0, np.nan, LCB[:, 0])[None, :]).all()
    assert not fin  # the case includes quotients outside the finite range
