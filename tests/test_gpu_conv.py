"""FFT convolution and expanding_source on the GPU vs the FP64 oracle."""
import numpy as np
import pytest
import torch

import oracle
from microsn_gb300 import synth

pytestmark = pytest.mark.gpu


def rel_err(a, b, floor):
    return np.max(np.abs(a - b) / np.maximum(np.abs(b), floor))


@pytest.mark.parametrize("Ny,Nx", [(64, 64), (48, 80), (250, 200), (128, 96), (30, 36)])
@pytest.mark.parametrize("mode", ["fused", "plain"])
def test_convolve_f64(ctx, Ny, Nx, mode):
    import microsn_gb300 as mlc
    mp = synth.lognormal_map(max(Ny, Nx), seed=Ny + Nx)[:Ny, :Nx].copy()
    m = mlc.Map(ctx, mp, "f64")
    for shape, rhalf in [("gaussian", 0.03), ("uniform", 0.05), ("exponential", 0.02)]:
        p = mlc.profile(shape, rhalf, 0.01)
        prof = mlc.profile_raster(p)
        if prof.shape[0] > min(Ny, Nx):
            continue
        got = mlc.convolve(ctx, m, p, mode).cpu().numpy()
        ref = oracle.conv_fft(mp, prof)
        # FP64 maps within 1e-9 relative (pixel floor 1e-3 of the mean)
        assert rel_err(got, ref, 1e-3 * ref.mean()) < 1e-9, (shape, mode)


@pytest.mark.parametrize("N", [100, 2000])
def test_convolve_f32(ctx, N):
    import microsn_gb300 as mlc
    mp = synth.lognormal_map(N, seed=5)
    m = mlc.Map(ctx, mp, "f32")
    p = mlc.profile("gaussian", 0.1, 0.01)
    got = mlc.convolve(ctx, m, p, "fused").cpu().numpy().astype(np.float64)
    ref = oracle.conv_fft(mp.astype(np.float32).astype(np.float64), mlc.profile_raster(p))
    # FP32 FFT: errors scale with the map's rms, not per pixel
    assert np.max(np.abs(got - ref)) < 2e-5 * np.sqrt((ref ** 2).mean()) * np.log2(N), np.max(np.abs(got - ref))


def test_convolve_rayshoot_map_f64(ctx):
    import microsn_gb300 as mlc
    mp, counts, meta = synth.rayshoot_numpy(128, 4.0, 0.4, 0.4, seed=0, rays_per_pixel=8)
    m = mlc.Map(ctx, mp, "f64")
    for mode in ("fused", "plain"):
        p = mlc.profile("gaussian", 0.1, 4.0 / 128)
        got = mlc.convolve(ctx, m, p, mode).cpu().numpy()
        ref = oracle.conv_fft(mp, mlc.profile_raster(p))
        assert rel_err(got, ref, 1e-3) < 1e-9


@pytest.mark.parametrize("mode", ["fused", "plain"])
def test_expanding_source_matches_oracle(ctx, mode):
    import microsn_gb300 as mlc
    N, width = 200, 25.0 * 200 / 10000 * 50  # 25 R_E over 10000 px scaled: pixel 0.0125 R_E
    mp = synth.lognormal_map(N, seed=9)
    sizes = [0, 0.05, 0.1, 0.2, 0.3]
    pix = width / N  # Rein = 1
    Noff = int(np.ceil((N / width) * sizes[-1]))
    lx, ly = mlc.locations_random(300, N, Noff, 5)
    m = mlc.Map(ctx, mp, "f64")
    base = mlc.profile("gaussian", 0.0, pix)
    LC, DLC = mlc.expanding_source(ctx, m, sizes, base, width, lx, ly, mode)
    LCo, DLCo = oracle.expanding_source(mp, sizes, "gaussian", lx, ly, pix, width)
    LC = LC.cpu().numpy(); DLC = DLC.cpu().numpy()
    assert np.array_equal(LC[:, 0], LCo[:, 0])  # point source: exact pixel reads
    assert rel_err(LC, LCo, 1e-3) < 1e-9
    assert np.max(np.abs(DLC - DLCo)) < 1e-9 * np.abs(LCo).max()


# Every map side with a specialised transform kernel: rows of Nx/2 = 5000, 4096, 2000 and
# 1000 complex points (three-level register kernels), columns of N1, N2 in {100, 64, 128,
# 80, 50, 40} (two-level register kernels); the short sides keep the oracle cheap.
@pytest.mark.parametrize("Ny,Nx", [(100, 10000), (128, 8192), (80, 4000), (50, 2000), (6400, 64), (4000, 80)])
@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_convolve_specialised_sizes(ctx, Ny, Nx, prec):
    import microsn_gb300 as mlc
    rng = np.random.default_rng(Ny + Nx)
    mp = np.exp(rng.normal(0, 0.5, (Ny, Nx)))
    prof = mlc.profile("exponential", 7.0, 1.0, ref_compat=False)
    P = mlc.profile_raster(prof)
    ref = oracle.conv_fft(mp, P)
    if prec == "f64":
        m = mlc.Map(ctx, mp, "f64")
        for mode in ("fused", "plain"):
            got = mlc.convolve(ctx, m, prof, mode).cpu().numpy()
            assert rel_err(got, ref, 1e-3 * ref.mean()) < 1e-9, mode
    else:
        m = mlc.Map(ctx, mp.astype(np.float32), "f32")
        got = mlc.convolve(ctx, m, prof, "fused").cpu().numpy().astype(np.float64)
        rms = np.sqrt(np.mean(ref ** 2))
        assert np.max(np.abs(got - ref)) < 2e-5 * rms * np.log2(max(Nx, Ny))
    m.close()
