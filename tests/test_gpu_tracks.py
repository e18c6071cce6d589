"""Bilinear track sampling and offset-minimised chi2 on the GPU vs the oracle."""
import numpy as np
import pytest
import torch

import oracle
from microsn_gb300 import synth

pytestmark = pytest.mark.gpu


def _tracks(n, N, seed, dtype):
    x0, y0, phi, v, off, t = synth.tracks(n, N, 3.0, seed, epochs=(5, 60), v_range=(0.01, 0.2))
    dev = "cuda:0"
    T = lambda a: torch.as_tensor(np.asarray(a, dtype), device=dev)
    return (x0, y0, phi, v, off, t), (T(x0), T(y0), T(phi), T(v), torch.as_tensor(off, device=dev), T(t))


def test_tracks_f64_match_oracle(ctx):
    import microsn_gb300 as mlc
    N = 160
    maps = [synth.lognormal_map(N, seed=s) for s in (1, 2, 3)]
    host, dev = _tracks(500, N, 4, np.float64)
    tmaps = [torch.as_tensor(m, device="cuda:0") for m in maps]
    for mag in (True, False):
        out = mlc.sample_tracks(ctx, tmaps, N, N, *dev, mag=mag).cpu().numpy()
        for q, m in enumerate(maps):
            ref = oracle.sample_tracks(m, *host, mag=mag)
            if mag:
                assert np.max(np.abs(out[q] - ref)) < 1e-9
            else:
                assert np.max(np.abs(out[q] - ref) / np.abs(ref)) < 1e-9


def test_tracks_degenerate_equals_nearest(ctx):
    import microsn_gb300 as mlc
    N = 64
    mp = synth.lognormal_map(N, seed=7)
    rng = np.random.default_rng(0)
    lx = rng.integers(0, N, 200); ly = rng.integers(0, N, 200)
    dev = "cuda:0"
    x0 = torch.as_tensor(lx + 0.5, dtype=torch.float64, device=dev)
    y0 = torch.as_tensor(ly + 0.5, dtype=torch.float64, device=dev)
    z = torch.zeros(200, dtype=torch.float64, device=dev)
    off = torch.arange(0, 201, dtype=torch.int64, device=dev)
    t = torch.ones(200, dtype=torch.float64, device=dev)
    out = mlc.sample_tracks(ctx, [torch.as_tensor(mp, device=dev)], N, N, x0, y0, z, z, off, t, mag=False)
    assert np.array_equal(out.cpu().numpy()[0], mp[ly, lx])


def test_tracks_f32_tolerance(ctx):
    import microsn_gb300 as mlc
    N = 2000
    mp = synth.lognormal_map(N, seed=11)
    host, dev = _tracks(2000, N, 5, np.float32)
    host64 = tuple(np.asarray(a, np.float64) if i != 4 else a for i, a in enumerate(host))
    out = mlc.sample_tracks(ctx, [torch.as_tensor(mp.astype(np.float32), device="cuda:0")], N, N, *dev,
                            mag=True).cpu().numpy()[0]
    ref = oracle.sample_tracks(mp.astype(np.float32).astype(np.float64), *host64, mag=True)
    # FP32 positions and bilinear weights: 2e-4 mag
    assert np.max(np.abs(out - ref)) < 2e-4, np.max(np.abs(out - ref))


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_chi2_offset(ctx, prec):
    import microsn_gb300 as mlc
    rng = np.random.default_rng(3)
    m = rng.normal(0, 1, (1000, 50))
    o = rng.normal(0, 1, 50); w = 1 / (rng.random(50) * 0.1 + 0.02) ** 2
    dt = torch.float64 if prec == "f64" else torch.float32
    mt = torch.as_tensor(m, dtype=dt, device="cuda:0")
    chi2, dm = mlc.chi2_offset(ctx, mt, o, w)
    ref, dmr = oracle.chi2_offset(mt.double().cpu().numpy(), o, w)
    np.testing.assert_allclose(chi2.cpu().numpy(), ref, rtol=1e-12)
    np.testing.assert_allclose(dm.cpu().numpy(), dmr, rtol=1e-12, atol=1e-14)


@pytest.mark.parametrize("dtype,nm,stride", [(np.float32, 16, 16), (np.float64, 3, 4), (np.float32, 5, 8),
                                            (np.float32, 1, 1)])
def test_interleaved_sampling_equals_planar(ctx, dtype, nm, stride):
    import microsn_gb300 as mlc
    N = 300
    tdt = torch.float32 if dtype == np.float32 else torch.float64
    maps = [torch.as_tensor(synth.lognormal_map(N, seed=20 + q), dtype=tdt, device="cuda:0") for q in range(nm)]
    host, dev = _tracks(3000, N, 8, dtype)
    il = mlc.interleave_maps(ctx, maps, N, N, stride)
    ref_il = torch.zeros((N, N, stride), dtype=tdt, device="cuda:0")
    for q in range(nm):
        ref_il[:, :, q] = maps[q]
    assert torch.equal(il, ref_il)
    for mag in (True, False):
        a = mlc.sample_tracks(ctx, maps, N, N, *dev, mag=mag)
        b = mlc.sample_tracks_interleaved(ctx, il, nm, *dev, mag=mag)
        assert torch.equal(a, b)


@pytest.mark.parametrize("prec,nm,stride", [("f64", 1, 1), ("f64", 3, 4), ("f32", 16, 16), ("f32", 5, 8)])
def test_fused_track_chi2_offset_matches_two_step(ctx, prec, nm, stride):
    """Fused sample -> magnitude -> offset chi2 (no light curve in memory) equals sampling
    the light curves and then running the offset chi2: FP64 1e-10, FP32 1e-5 relative."""
    import microsn_gb300 as mlc
    N, n, T = 240, 700, 50
    dt = torch.float64 if prec == "f64" else torch.float32
    maps = [torch.as_tensor(synth.lognormal_map(N, seed=40 + q), dtype=dt, device="cuda:0") for q in range(nm)]
    imap = mlc.interleave_maps(ctx, maps, N, N, stride) if stride > 1 else maps[0]
    rng = np.random.default_rng(9)
    x0 = rng.uniform(30, 60, n); y0 = rng.uniform(30, 60, n); phi = rng.uniform(0, 2 * np.pi, n)
    v = rng.uniform(0.5, 3.0, n)
    t = np.arange(T, dtype=np.float64)
    D = lambda a: torch.as_tensor(a, dtype=dt, device="cuda:0")
    off = torch.arange(0, (n + 1) * T, T, dtype=torch.int64, device="cuda:0")
    lc = mlc.sample_tracks(ctx, maps, N, N, D(x0), D(y0), D(phi), D(v), off, D(np.tile(t, n)), mag=True)
    obs = lc[0, :T].double().cpu().numpy() + rng.normal(0, 0.05, T)
    w = np.full(T, 1 / 0.05 ** 2)
    c2, dm = mlc.track_chi2_offset(ctx, imap, nm, D(x0), D(y0), D(phi), D(v), D(t),
                                   torch.as_tensor(obs, device="cuda:0"), torch.as_tensor(w, device="cuda:0"))
    for q in range(nm):
        ref, dref = oracle.chi2_offset(lc[q].double().cpu().numpy().reshape(n, T), obs, w)
        tol = 1e-10 if prec == "f64" else 1e-5
        np.testing.assert_allclose(c2[q].cpu().numpy(), ref, rtol=tol)
        np.testing.assert_allclose(dm[q].cpu().numpy(), dref, rtol=tol, atol=tol)


def test_fp64_magnitudes_log10_accuracy(ctx):
    """FP64 magnitudes use a float-float log10 (GB300's FP64 rate): against numpy's log10 of
    the same fluxes over values from 1e-300 to 1e300, subnormal and zero pixels included,
    within 1e-13 mag (1e-14 relative in log10 near 0, 1e-16 relative near +-300)."""
    import microsn_gb300 as mlc
    rng = np.random.default_rng(9)
    N = 256
    mp = np.exp(rng.uniform(-690.0, 690.0, (N, N)))
    mp[rng.random((N, N)) < 0.01] = 4e-320  # subnormal
    mp[rng.random((N, N)) < 0.01] = 0.0
    mp[:, :8] = 10.0 ** rng.uniform(-3, 3, (N, 8))  # ordinary magnifications
    DEV = "cuda:0"
    maps = [torch.as_tensor(mp, device=DEV)]
    ntr, T = 2000, 64
    x0 = rng.uniform(-10, N + 10, ntr); y0 = rng.uniform(-10, N + 10, ntr)
    phi = rng.uniform(0, 2 * np.pi, ntr); v = rng.uniform(0.0, 2.0, ntr)
    off = np.arange(ntr + 1, dtype=np.int64) * T
    t = np.tile(np.arange(T, dtype=np.float64), ntr)
    D = lambda a: torch.as_tensor(a, device=DEV)
    args = (maps, N, N, D(x0), D(y0), D(phi), D(v), D(off), D(t))
    mu = mlc.sample_tracks(ctx, *args, mag=False).cpu().numpy()[0]
    mag = mlc.sample_tracks(ctx, *args, mag=True).cpu().numpy()[0]
    with np.errstate(divide="ignore"):
        ref = -2.5 * np.log10(mu)
    assert np.array_equal(np.isfinite(ref), np.isfinite(mag)) and np.array_equal(ref == np.inf, mag == np.inf)
    fin = np.isfinite(ref)
    assert fin.sum() > 0.5 * ref.size and np.abs(ref[fin]).max() > 700
    err = np.abs(mag[fin] - ref[fin])
    assert np.max(err / np.maximum(1.0, np.abs(ref[fin]))) < 1e-13, np.max(err)
