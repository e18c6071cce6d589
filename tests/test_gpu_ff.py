"""Float-float transforms of FP64 maps (mlc_map_set_fft(map, MLC_FFT_F32X2)) on the GPU.

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
    m32 = mlc.Map(ctx, mp.astype(np.float32), "f32")
    with pytest.raises(mlc.MlcError):
        m32.set_fft("f32x2")
    m64 = mlc.Map(ctx, mp, "f64")
    m64.set_fft("f32x2")
    with pytest.raises(mlc.MlcError):
        mlc.convolve(ctx, m64, mlc.profile("gaussian", 0.03, 0.01), "plain")  # the plain form is native FP64
    m64.set_fft("native")
    mlc.convolve(ctx, m64, mlc.profile("gaussian", 0.03, 0.01), "plain")
