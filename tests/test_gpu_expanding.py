"""Many profiles per map (mlc_convolve_many, eager and CUDA-graph replay) and the
expanding-source sampler (supernova case: one profile per epoch and band)."""
import numpy as np
import pytest
import torch

import oracle
from microsn_gb300 import synth

pytestmark = pytest.mark.gpu


def _sn_profiles(nep, bands, rmax, pix=1.0):
    import microsn_gb300 as mlc
    R = np.linspace(1.0, rmax, nep)
    return [mlc.profile("limb_darkened", r / np.sqrt(2.0) * pix, pix, ref_compat=False, u=u) for r in R for u in bands]


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_convolve_many_equals_single_convolutions_and_graph_replays(ctx, prec):
    import microsn_gb300 as mlc
    N = 240
    dt = torch.float64 if prec == "f64" else torch.float32
    m = mlc.Map(ctx, synth.lognormal_map(N, seed=3).astype(np.float64 if prec == "f64" else np.float32), prec)
    profs = _sn_profiles(6, (0.6, 0.3), 20.0)
    got = mlc.convolve_many(ctx, m, profs)
    for k, p in enumerate(profs):
        assert torch.equal(got[k], mlc.convolve(ctx, m, p, "fused")), k
    # graph: first call captures, second replays; new profile values of the same raster
    # sizes replay the same graph
    out = torch.empty_like(got)
    l0 = ctx.launch_count()
    mlc.convolve_many(ctx, m, profs)
    per_call = ctx.launch_count() - l0  # FFT and (autotuned) direct-form kernels of one call
    l0 = ctx.launch_count()
    mlc.convolve_many(ctx, m, profs, out=out, graph=True)
    assert torch.equal(out, got)
    out.zero_()
    mlc.convolve_many(ctx, m, profs, out=out, graph=True)
    assert torch.equal(out, got)
    assert ctx.launch_count() - l0 == 2 * per_call  # the replay counts the graph's kernels
    profs2 = _sn_profiles(6, (0.5, 0.2), 20.0)  # other limb darkening, same radii and sizes
    mlc.convolve_many(ctx, m, profs2, out=out, graph=True)
    ref2 = mlc.convolve_many(ctx, m, profs2)
    assert torch.equal(out, ref2)
    m.close()


def test_sample_expanding_matches_oracle(ctx):
    import microsn_gb300 as mlc
    N, nep, nb, n = 200, 8, 3, 300
    mp = synth.lognormal_map(N, seed=5)
    m = mlc.Map(ctx, mp, "f64")
    profs = _sn_profiles(nep, (0.7, 0.5, 0.3), 15.0)
    maps = mlc.convolve_many(ctx, m, profs)
    rng = np.random.default_rng(2)
    x0 = rng.uniform(40, 160, n); y0 = rng.uniform(40, 160, n); phi = rng.uniform(0, 2 * np.pi, n)
    v = rng.uniform(0.1, 0.5, n); t = np.sort(rng.uniform(0, 60, nep))
    D = lambda a: torch.as_tensor(a, dtype=torch.float64, device="cuda:0")
    out = mlc.sample_expanding(ctx, maps, nb, D(x0), D(y0), D(phi), D(v), D(t)).cpu().numpy()
    for k, p in enumerate(profs):
        e, b = divmod(k, nb)
        conv = oracle.conv_fft(mp, mlc.profile_raster(p))
        ref = oracle.sample_tracks(conv, x0, y0, phi, v, np.arange(n + 1, dtype=np.int64), np.full(n, t[e]), mag=True)
        assert np.max(np.abs(out[:, e * nb + b] - ref)) < 1e-9, k
    m.close()
