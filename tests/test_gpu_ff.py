"""Float-float transforms (mlc_map_set_fft(map, MLC_FFT_F32X2)) on the GPU, of FP64 maps and
of FP32 maps.

The forward transform and the fused convolutions of an FP64 map run in pairs of FP32
values (about 48 significant bits) while pixels and every output stay FP64.  Checked
against the FP64 oracle: convolved maps within 1e-11 relative (pixel floor 1e-3 of the
mean; the FP64 bar is 1e-9), expanding_source light curves within 1e-9, and the batched
step's magnitudes against native FP64 transforms, through the cluster last pass (2000²:
1000-point rows) and the generic one (360²).
"""
import numpy as np
import pytest
import torch

import oracle
from microsn_gb300 import synth

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def _rel(a, b, floor):
    return np.max(np.abs(a - b) / np.maximum(np.abs(b), floor))


@pytest.mark.parametrize("Ny,Nx", [(200, 250), (360, 480), (2000, 2000), (128, 96)])
def test_ff_convolution_matches_oracle(ctx, Ny, Nx):
    import microsn_gb300 as mlc
    mp = synth.lognormal_map(max(Ny, Nx), seed=Ny + 3 * Nx)[:Ny, :Nx].copy()
    m = mlc.Map(ctx, mp, "f64")
    m.set_fft("f32x2")
    for shape, rhalf in [("gaussian", 0.03), ("uniform", 0.05), ("exponential", 0.02), ("gaussian", 0.15)]:
        p = mlc.profile(shape, rhalf, 0.01)
        prof = mlc.profile_raster(p)
        if prof.shape[0] > min(Ny, Nx):
            continue
        got = mlc.convolve(ctx, m, p, "fused").cpu().numpy()
        ref = oracle.conv_fft(mp, prof)
        assert _rel(got, ref, 1e-3 * ref.mean()) < 1e-11, (shape, rhalf)


def test_ff_expanding_source_matches_oracle(ctx):
    import microsn_gb300 as mlc
    N, width = 360, 12.0
    mp = synth.lognormal_map(N, seed=17)
    m = mlc.Map(ctx, mp, "f64")
    m.set_fft("f32x2")
    sizes = [0.0, 0.05, 0.1, 0.2, 0.3]
    Noff = int(np.ceil((N / width) * sizes[-1]))
    lx, ly = mlc.locations_random(500, N, Noff, 3)
    pix = width / N
    LC, DLC = mlc.expanding_source(ctx, m, sizes, mlc.profile("gaussian", 0.0, pix), width, lx, ly)
    LCo, DLCo = oracle.expanding_source(mp, sizes, "gaussian", lx, ly, pix, width)
    assert _rel(LC.cpu().numpy(), LCo, 1e-3) < 1e-9


@pytest.mark.parametrize("N,nprof", [(2000, 12), (360, 5)])
def test_ff_batched_step_matches_native_fp64(ctx, N, nprof):
    import microsn_gb300 as mlc
    mp = synth.lognormal_map(N, seed=N + nprof)
    shapes = ["uniform", "exponential", "gaussian"]
    profs = [mlc.profile(shapes[i % 3], 1.5 + 2.0 * i, 1.0, ref_compat=False) for i in range(nprof)]
    x0, y0, phi, v, off, t = synth.tracks(400, N, 3.0, 5, epochs=(0, 40), v_range=(0.01, 0.3))
    tr = {k: torch.as_tensor(np.ascontiguousarray(a, np.int64 if k == "off" else np.float64), device=DEV)
          for k, a in zip(("x0", "y0", "phi", "v", "off", "t"), (x0, y0, phi, v, off, t))}
    m = mlc.Map(ctx, mp, "f64")
    ref = mlc.convolve_sample_tracks(ctx, m, profs, tr, mag=True)
    m.set_fft("f32x2")
    got = mlc.convolve_sample_tracks(ctx, m, profs, tr, mag=True)
    fin = torch.isfinite(ref)
    assert torch.equal(fin, torch.isfinite(got))
    # magnitudes: 1e-11 in flux is about 1e-11 mag
    assert float((got[fin] - ref[fin]).abs().max()) < 1e-10


def test_ff_mode_refusals(ctx):
    import microsn_gb300 as mlc
    mp = synth.lognormal_map(64, seed=2)
    for m in (mlc.Map(ctx, mp, "f64"), mlc.Map(ctx, mp.astype(np.float32), "f32")):
        m.set_fft("f32x2")
        with pytest.raises(mlc.MlcError):
            mlc.convolve(ctx, m, mlc.profile("gaussian", 0.03, 0.01), "plain")  # the plain form: own precision
        m.set_fft("native")
        mlc.convolve(ctx, m, mlc.profile("gaussian", 0.03, 0.01), "plain")


# FP32 maps with float-float transforms: the only error left is the FP32 rounding of the
# inputs (exact: FP32 pixels) and of the convolved pixels, so the bound is a few FP32 ulp
# relative in every pixel -- where FP32 transforms are off by up to ~1e-5 in faint pixels.
FF32_REL = 4e-7


@pytest.mark.parametrize("Ny,Nx", [(200, 250), (2000, 2000), (128, 96)])
def test_ff_fp32_map_convolution_matches_oracle(ctx, Ny, Nx):
    import microsn_gb300 as mlc
    mp = synth.lognormal_map(max(Ny, Nx), seed=Ny + 5 * Nx)[:Ny, :Nx].astype(np.float32)
    m = mlc.Map(ctx, mp, "f32")
    m.set_fft("f32x2")
    for shape, rhalf in [("gaussian", 0.03), ("uniform", 0.05), ("exponential", 0.02)]:
        p = mlc.profile(shape, rhalf, 0.01)
        prof = mlc.profile_raster(p)
        if prof.shape[0] > min(Ny, Nx):
            continue
        got = mlc.convolve(ctx, m, p, "fused")
        assert got.dtype == torch.float32
        ref = oracle.conv_fft(mp.astype(np.float64), prof)
        assert _rel(got.cpu().numpy().astype(np.float64), ref, 1e-3 * ref.mean()) < FF32_REL, (shape, rhalf)


@pytest.mark.parametrize("N,nprof", [(2000, 12), (360, 5), (10000, 2)])
def test_ff_fp32_map_batched_step_matches_fp64(ctx, N, nprof):
    """The batched step of an FP32 map in float-float mode against the FP64 step on the same
    pixels: FP32 magnitudes within a few FP32 ulp of the FP64 ones."""
    import microsn_gb300 as mlc
    mp = synth.lognormal_map(N, seed=N + 7 * nprof).astype(np.float32)
    shapes = ["uniform", "exponential", "gaussian"]
    profs = [mlc.profile(shapes[i % 3], 1.5 + 2.0 * i, 1.0, ref_compat=False) for i in range(nprof)]
    x0, y0, phi, v, off, t = synth.tracks(400, N, 3.0, 6, epochs=(0, 40), v_range=(0.01, 0.3))
    arrs = dict(zip(("x0", "y0", "phi", "v", "off", "t"), (x0, y0, phi, v, off, t)))
    tr32 = {k: torch.as_tensor(np.ascontiguousarray(a, np.int64 if k == "off" else np.float32), device=DEV)
            for k, a in arrs.items()}
    tr64 = {k: (a.double() if a.is_floating_point() else a) for k, a in tr32.items()}
    ref = mlc.convolve_sample_tracks(ctx, mlc.Map(ctx, mp.astype(np.float64), "f64"), profs, tr64, mag=True)
    m = mlc.Map(ctx, mp, "f32")
    m.set_fft("f32x2")
    got = mlc.convolve_sample_tracks(ctx, m, profs, tr32, mag=True)
    assert got.dtype == torch.float32
    fin = torch.isfinite(ref)
    assert torch.equal(fin, torch.isfinite(got))
    # FP32 magnitudes: the flux within FP32_REL (1.0857 FP32_REL in magnitude), then the FP32
    # logarithm and its rounding (|m| < 8: an ulp is at most 9.5e-7)
    assert float((got.double()[fin] - ref[fin]).abs().max()) < 1.0857 * FF32_REL + 2e-6


@pytest.mark.parametrize("prec,key", [("f32", "conv P1 f32x2->f32 10000x10000"), ("f64", "conv P1 f32x2 10000x10000")])
def test_p1_staged_and_prefetched_forms_agree(lib_built, prec, key):
    """The fused convolution's P1 in float-float arithmetic at 10000^2 (N2 = 100), with the map
    spectrum prefetched into L2 or staged in shared memory (the autotuner's two candidates,
    pinned here): the same arithmetic, so the same pixels bit for bit."""
    import microsn_gb300 as mlc
    N = 10000
    dt = np.float32 if prec == "f32" else np.float64
    mp = synth.lognormal_map(N, seed=17).astype(dt)
    p = mlc.profile("exponential", 12.0, 1.0, ref_compat=False)
    out = []
    for choice in (0, 1):
        c = mlc.Context(0)
        c.tune_set(key, choice)
        m = mlc.Map(c, mp, prec)
        m.set_fft("f32x2")
        out.append(mlc.convolve(c, m, p, "fused").cpu())
        assert c.autotune_report()[key][0] == f"pinned {choice}"
        m.close()
        c.close()
    assert torch.equal(out[0], out[1])
