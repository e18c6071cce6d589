"""Map MPDs on the GPU: getBinnedMpd (one-pass histogram) and Mpd::divide_by, bit-exact
against the reference's outputs (golden vectors) and the oracle."""
import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu


def test_binned_mpd_matches_golden(ctx, golden):
    import microsn_gb300 as mlc
    m = mlc.Map(ctx, golden["mpd_map"], "f64")
    b, c = mlc.map_binned_mpd(ctx, m, 50, 0.02, 200.0)
    assert np.array_equal(b, golden["mpd_bins"])
    assert np.array_equal(c, golden["mpd_counts"])
    assert np.array_equal(mlc.mpd_normalize(b, c), golden["mpd_counts_norm"])
    m.close()


@pytest.mark.parametrize("n,nb,seed", [(720, 300, 1), (1000, 12000, 2), (64, 1, 3), (2048, 16000, 4)])
def test_binned_mpd_f64_matches_oracle(ctx, n, nb, seed):
    import microsn_gb300 as mlc
    rng = np.random.default_rng(seed)
    # integer ray counts times a factor: many exact ties, values on and around edges
    mp = rng.poisson(rng.lognormal(1.0, 1.3, (n, n))).astype(np.float64) * 0.173
    lo, hi = 10 ** rng.uniform(-3, -1), 10 ** rng.uniform(1, 3)
    e = oracle.mpd_edges(nb, lo, hi, True)
    flat = mp.ravel()
    k = min(nb, 50)
    flat[:k] = e[rng.integers(0, nb, k)]
    flat[k:k + 4] = [lo, hi, np.nextafter(hi, 0), np.nextafter(lo, 0)]
    m = mlc.Map(ctx, mp, "f64")
    b, c = mlc.map_binned_mpd(ctx, m, nb, lo, hi)
    bo, co = oracle.binned_mpd(mp, nb, lo, hi)
    assert np.array_equal(b, bo)
    assert np.array_equal(c, co)
    m.close()


def test_binned_mpd_f32_bins_the_fp32_values(ctx):
    """An FP32 map is binned exactly by its FP32 values."""
    import microsn_gb300 as mlc
    rng = np.random.default_rng(9)
    mp = rng.lognormal(0.0, 1.5, (900, 900)).astype(np.float32)
    e = oracle.mpd_edges(500, 0.02, 200.0, True)
    flat = mp.ravel()
    flat[:40] = e[rng.integers(0, 500, 40)].astype(np.float32)  # rounded edges: both sides
    m = mlc.Map(ctx, torch.as_tensor(mp, device="cuda:0"), "f32")
    b, c = mlc.map_binned_mpd(ctx, m, 500, 0.02, 200.0)
    bo, co = oracle.binned_mpd(mp.astype(np.float64), 500, 0.02, 200.0)
    assert np.array_equal(b, bo)
    assert np.array_equal(c, co)
    m.close()


def test_mpd_divide_matches_golden_and_oracle(ctx, golden):
    import microsn_gb300 as mlc
    cR = mlc.mpd_divide(ctx, golden["mpd_bins"], golden["mpd_counts_norm"], golden["mpd_binsB"],
                        golden["mpd_countsB_norm"], golden["mpd_ratio_bins"])
    assert np.array_equal(cR, golden["mpd_ratio_counts"])
    rng = np.random.default_rng(5)
    for NA, NB, NR in [(300, 500, 300), (17, 1000, 5), (2000, 40, 700)]:
        bA = np.sort(10 ** rng.uniform(-2, 2, NA)); cA = rng.random(NA)
        bB = np.sort(10 ** rng.uniform(-2, 2, NB)); cB = rng.random(NB)
        bR = oracle.mpd_edges(NR, 0.01, 100.0, True)
        bR[: min(NR, 3)] = bA[1] / bB[: min(NR, 3)]  # products landing on A's edges
        got = mlc.mpd_divide(ctx, bA, cA, bB, cB, bR)
        assert np.array_equal(got, oracle.mpd_divide(bA, cA, bB, cB, bR))


def test_binned_mpd_rejects_bad_ranges(ctx):
    import microsn_gb300 as mlc
    m = mlc.Map(ctx, np.ones((16, 16)), "f64")
    with pytest.raises(mlc.MlcError):
        mlc.map_binned_mpd(ctx, m, 16001, 0.02, 200.0)
    with pytest.raises(mlc.MlcError):
        mlc.map_binned_mpd(ctx, m, 10, 0.0, 200.0)
    m.close()
