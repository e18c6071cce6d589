"""Pair sides: curves prepared once per image and paired by the tensor-core kernel give the
results of the two-stage path (pair_chi2_magdiff, tensor form) exactly -- histogram,
out-of-range counts, top-k and the chi2 matrix -- whether a side is built from stored FP32
curves or straight from an expanding source's convolved maps (sample -> magnitude ->
centre in one pass, no light curve stored).  Also: one side paired with several others,
and the refusals for sides that do not fit together."""
import numpy as np
import pytest
import torch

import oracle
from microsn_gb300 import synth

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def _curves(NA, NB, T, seed):
    rng = np.random.default_rng(seed)
    A = np.cumsum(rng.normal(0, 0.05, (NA, T)), axis=1) + rng.normal(0, 0.3, (NA, 1))
    B = np.cumsum(rng.normal(0, 0.05, (NB, T)), axis=1) + rng.normal(0, 0.3, (NB, 1))
    d = rng.normal(0, 0.02, T)
    sig = rng.uniform(0.02, 0.1, T)
    for c in range(5):  # near-identical pairs go through the FP64 refinement
        B[c] = A[c] - d + rng.normal(0, 1e-4, T)
    return A.astype(np.float32), B.astype(np.float32), 1.0 / sig ** 2, d


def _same(r1, r2):
    assert np.array_equal(r1["hist"], r2["hist"])
    for key in ("delta", "below", "above", "refined", "candidates", "threshold"):
        assert r1["stats"][key] == r2["stats"][key], key
    assert np.array_equal(r1["topk_val"], r2["topk_val"])
    assert np.array_equal(r1["topk_i"], r2["topk_i"]) and np.array_equal(r1["topk_j"], r2["topk_j"])
    if r1["matrix"] is not None:
        assert torch.equal(r1["matrix"], r2["matrix"])


@pytest.mark.parametrize("offset", [False, True])
@pytest.mark.parametrize("NA,NB,T", [(300, 200, 50), (129, 65, 128), (700, 390, 7)])
def test_sides_from_curves_equal_two_stage(ctx, offset, NA, NB, T):
    import microsn_gb300 as mlc
    A, B, w, d = _curves(NA, NB, T, NA + 3 * NB + T)
    tA, tB = torch.as_tensor(A, device=DEV), torch.as_tensor(B, device=DEV)
    kw = dict(nbins=200, lo=-6, hi=8, k=20, want_matrix=True)
    two = mlc.pair_chi2_magdiff(ctx, tA, tB, w, d, offset, method="tensor", **kw)
    sA = mlc.PairSide.curves(ctx, tA, w, None, offset)
    sB = mlc.PairSide.curves(ctx, tB, w, d, offset)
    one = mlc.pair_chi2_sides(ctx, sA, sB, **kw)
    _same(one, two)
    # and both against the FP64 oracle
    ref = oracle.pair_chi2_magdiff(A, B, w, d, offset)
    got = one["matrix"].cpu().numpy().astype(np.float64).ravel()
    assert (np.abs(got - ref) / np.maximum(ref, 1e-300)).max() < 1e-5
    st = one["stats"]
    assert int(one["hist"].sum()) + st["below"] + st["above"] == NA * NB
    sA.close(); sB.close()


def test_one_side_paired_with_several(ctx):
    import microsn_gb300 as mlc
    A, B, w, d = _curves(400, 300, 40, 5)
    _, B2, _, _ = _curves(400, 250, 40, 6)
    tA = torch.as_tensor(A, device=DEV)
    sA = mlc.PairSide.curves(ctx, tA, w, None, True)
    for Bx in (B, B2, B):
        tB = torch.as_tensor(Bx, device=DEV)
        sB = mlc.PairSide.curves(ctx, tB, w, d, True)
        one = mlc.pair_chi2_sides(ctx, sA, sB, nbins=100, lo=-4, hi=6, k=10)
        two = mlc.pair_chi2_magdiff(ctx, tA, tB, w, d, True, method="tensor", nbins=100, lo=-4, hi=6, k=10)
        _same(one, two)
        sB.close()
    sA.close()


def _sn_profiles(nep, bands, rmax):
    import microsn_gb300 as mlc
    R = np.linspace(1.0, rmax, nep)
    return [mlc.profile("limb_darkened", r / np.sqrt(2.0), 1.0, ref_compat=False, u=u) for r in R for u in bands]


@pytest.mark.parametrize("offset", [False, True])
def test_sides_from_expanding_maps_equal_two_stage(ctx, offset):
    """Expanding source, 10 epochs x 3 bands (T = 30) on a 400^2 FP32 map: image A's and
    image B's tracks sampled straight into their sides equal sampling the light curves and
    pairing them."""
    import microsn_gb300 as mlc
    N, nep, nb = 400, 10, 3
    mp = synth.lognormal_map(N, seed=11).astype(np.float32)
    m = mlc.Map(ctx, mp, "f32")
    maps = mlc.convolve_many(ctx, m, _sn_profiles(nep, (0.7, 0.5, 0.3), 20.0))
    rng = np.random.default_rng(4)
    t = np.sort(rng.uniform(0, 80, nep)).astype(np.float32)
    F = lambda a: torch.as_tensor(np.asarray(a, np.float32), device=DEV)

    def tracks(n):
        # start within [130, 270] px, at most 0.8 px per day for 80 days: inside the map
        return [F(rng.uniform(130, 270, n)), F(rng.uniform(130, 270, n)), F(rng.uniform(0, 2 * np.pi, n)),
                F(rng.uniform(0.1, 0.8, n))]

    trA, trB = tracks(500), tracks(333)
    T = nep * nb
    w = 1.0 / rng.uniform(0.02, 0.1, T) ** 2
    d = rng.normal(0, 0.05, T)
    LA = mlc.sample_expanding(ctx, maps, nb, *trA, F(t))
    LB = mlc.sample_expanding(ctx, maps, nb, *trB, F(t))
    kw = dict(nbins=300, lo=-3, hi=7, k=25, want_matrix=True)
    two = mlc.pair_chi2_magdiff(ctx, LA, LB, w, d, offset, method="tensor", **kw)
    sA = mlc.PairSide.expanding(ctx, maps, nep, nb, *trA, F(t), w, None, offset)
    sB = mlc.PairSide.expanding(ctx, maps, nep, nb, *trB, F(t), w, d, offset)
    one = mlc.pair_chi2_sides(ctx, sA, sB, **kw)
    _same(one, two)
    # a side from the stored curves is the same side
    cB = mlc.PairSide.curves(ctx, LB, w, d, offset)
    _same(mlc.pair_chi2_sides(ctx, sA, cB, **kw), one)
    for s in (sA, sB, cB):
        s.close()
    m.close()


def test_side_refusals(ctx):
    import microsn_gb300 as mlc
    A, B, w, d = _curves(100, 80, 20, 1)
    tA, tB = torch.as_tensor(A, device=DEV), torch.as_tensor(B, device=DEV)
    sA = mlc.PairSide.curves(ctx, tA, w, None, False)
    with pytest.raises(mlc.MlcError):  # other weights
        mlc.pair_chi2_sides(ctx, sA, mlc.PairSide.curves(ctx, tB, 2 * w, d, False))
    with pytest.raises(mlc.MlcError):  # other offset form
        mlc.pair_chi2_sides(ctx, sA, mlc.PairSide.curves(ctx, tB, w, d, True))
    with pytest.raises(mlc.MlcError):  # other T
        mlc.pair_chi2_sides(ctx, sA, mlc.PairSide.curves(ctx, tB[:, :10].contiguous(), w[:10], d[:10], False))
    with pytest.raises(mlc.MlcError):  # side A built with d
        sd = mlc.PairSide.curves(ctx, tA, w, d, False)
        mlc.pair_chi2_sides(ctx, sd, mlc.PairSide.curves(ctx, tB, w, d, False))
    with pytest.raises(mlc.MlcError):  # T > 128
        big = torch.zeros((4, 129), dtype=torch.float32, device=DEV)
        mlc.PairSide.curves(ctx, big, np.ones(129))
    bad = tA.clone()
    bad[3, 4] = float("inf")
    with pytest.raises(mlc.MlcError):  # non-finite curve values
        mlc.PairSide.curves(ctx, bad, w)
    sA.close()
