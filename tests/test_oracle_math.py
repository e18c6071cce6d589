"""Self-consistency of the oracle's restatements that have no reference pin."""
import numpy as np

import oracle
from microsn_gb300 import synth


def test_conv_fft_equals_direct():
    rng = np.random.default_rng(0)
    for (Ny, Nx, shape, rhalf, pix) in [(32, 40, "gaussian", 0.05, 0.01), (48, 48, "uniform", 0.04, 0.01),
                                       (30, 24, "exponential", 0.02, 0.01)]:
        mp = rng.random((Ny, Nx)) + 0.1
        prof = oracle.profile(shape, rhalf, pix)
        a = oracle.conv_fft(mp, prof)
        b = oracle.conv_direct(mp, prof)
        np.testing.assert_allclose(a, b, rtol=1e-12, atol=1e-13)


def test_bilinear_degenerate_is_nearest():
    rng = np.random.default_rng(1)
    mp = rng.random((20, 30))
    for i in range(20):
        for j in range(30):
            assert oracle.bilinear(mp, j + 0.5, i + 0.5) == mp[i, j]


def test_bilinear_linear_field_exact():
    yy, xx = np.mgrid[0:16, 0:16].astype(np.float64)
    mp = 2.0 * (xx + 0.5) - 3.0 * (yy + 0.5) + 7.0
    for x, y in [(3.3, 4.9), (0.5, 0.5), (15.5, 15.5), (7.0, 2.25)]:
        assert abs(oracle.bilinear(mp, x, y) - (2 * x - 3 * y + 7)) < 1e-12
    assert oracle.bilinear(mp, 0.49, 3.0) == 0.0 and oracle.bilinear(mp, 3.0, 15.51) == 0.0


def test_chi2_offset_matches_numpy():
    rng = np.random.default_rng(2)
    m = rng.normal(0, 1, (50, 33)); o = rng.normal(0, 1, 33); w = rng.random(33) + 0.5
    chi2, dm = oracle.chi2_offset(m, o, w)
    r = o[None, :] - m
    dmn = (w * r).sum(1) / w.sum()
    c = (w * (r - dmn[:, None]) ** 2).sum(1)
    np.testing.assert_allclose(dm, dmn, rtol=1e-12)
    np.testing.assert_allclose(chi2, c, rtol=1e-12)


def test_magdiff_pair_matches_numpy():
    rng = np.random.default_rng(3)
    A = rng.normal(0, 1, (7, 16)).astype(np.float32); B = rng.normal(0, 1, (9, 16)).astype(np.float32)
    w = rng.random(16) + 0.1; d = rng.normal(0, 0.1, 16)
    for off in (False, True):
        c = oracle.pair_chi2_magdiff(A, B, w, d, off).reshape(7, 9)
        r = d[None, None, :] - (A[:, None, :].astype(np.float64) - B[None, :, :].astype(np.float64))
        if off:
            r = r - ((w * r).sum(-1) / w.sum())[..., None]
        np.testing.assert_allclose(c, (w * r * r).sum(-1), rtol=1e-12)


def test_histogram_and_topk():
    rng = np.random.default_rng(4)
    v = np.exp(rng.normal(0, 2, 5000))
    counts, _ = oracle.histogram(v, 40, -3, 3, log=True)
    ref, _ = np.histogram(np.log10(v), bins=40, range=(-3, 3))
    assert np.array_equal(counts, ref)
    idx = oracle.topk_smallest(v, 17)
    assert np.array_equal(idx, np.argsort(v, kind="stable")[:17])


def test_synthetic_map_statistics():
    mp, counts, meta = synth.rayshoot_numpy(64, 4.0, 0.4, 0.4, seed=0, rays_per_pixel=16)
    assert mp.shape == (64, 64) and counts.dtype == np.int32
    assert 0.7 < mp.mean() < 1.3 and (mp >= 0).all()


def test_fit_raster_derivatives():
    """The smooth thin-disc raster's derivative rasters equal central differences of the
    same law evaluated at shifted offsets (x, y) and radii (library and oracle agree)."""
    import microsn_gb300 as mlc
    N, pix = 64, 1.0

    def law(x, y, R):
        sig = 0.4106 * R
        core = 10.0 / (np.exp((1 / 0.4106) ** 0.75) - 1.0)
        u = np.hypot(x, y) / sig
        with np.errstate(divide="ignore"):
            v = 1.0 / (np.exp(u ** 0.75) - 1.0)
        return np.minimum(v, core)

    for R in (3.3, 9.0, 14.5):
        P, Px, Py, PR = mlc.fit_raster(R, pix, N)
        for a, b in zip((P, Px, Py, PR), oracle.fit_raster(R, pix, N)):
            assert np.max(np.abs(a - b)) <= 1e-15 * np.max(np.abs(a))
        c = (np.arange(N) - N // 2) * pix + pix / 2.0
        X, Y = np.meshgrid(c, c)
        S = law(X, Y, R).sum()
        h = 1e-5
        fx = (law(X + h, Y, R) - law(X - h, Y, R)) / (2 * h) / S
        fy = (law(X, Y + h, R) - law(X, Y - h, R)) / (2 * h) / S
        assert np.max(np.abs(fx - Px)) <= 1e-6 * np.max(np.abs(Px))
        assert np.max(np.abs(fy - Py)) <= 1e-6 * np.max(np.abs(Py))
        Pp = mlc.fit_raster(R * (1 + 1e-6), pix, N)[0]
        Pm = mlc.fit_raster(R * (1 - 1e-6), pix, N)[0]
        assert np.max(np.abs((Pp - Pm) / (2e-6 * R) - PR)) <= 1e-6 * np.max(np.abs(PR))
